// mdg_api.cu -- host implementation of the C ABI declared in include/mdg.h.
//
// Owns the device state of one context (one or more systems), restates the
// reference's setup computations on the host (neighbor_setup/compute_bin_grid,
// MaterialTable::build_pair_tables, LJPairCoeffs::from_params,
// setup_nose_hoover) and drives the per-step kernel sequence, eagerly or as
// captured CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <new>
#include <vector>

#include "../../include/mdg.h"
#include "mdg_internal.cuh"

using namespace mdg;

namespace {

constexpr double kPi = 3.14159265358979323846;

template <class T>
T* dalloc(size_t n, int& err) {
    if (err) return nullptr;
    if (n == 0) n = 1;
    void* p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        err = MDG_ERR_OOM;
        return nullptr;
    }
    cudaMemset(p, 0, n * sizeof(T));
    return static_cast<T*>(p);
}

inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

// MaterialTable::build_pair_tables (crates/dem_atom/src/lib.rs:389-515):
// packed [table][i][j] for one system.
void material_tables(const mdg_material* m, int n, std::vector<double>& out) {
    const size_t nn = (size_t)n * n;
    out.assign(nn * NTAB, 0.0);
    auto at = [&](int t, int i, int j) -> double& { return out[(size_t)t * nn + (size_t)i * n + j]; };
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const double e_ij = std::sqrt(m[i].restitution * m[j].restitution);
            const double log_e = std::log(e_ij);
            at(T_BETA, i, j) = -log_e / std::sqrt(kPi * kPi + log_e * log_e);
            at(T_FRICTION, i, j) = std::sqrt(m[i].friction * m[j].friction);
            at(T_ROLL_FRICTION, i, j) = std::sqrt(m[i].rolling_friction * m[j].rolling_friction);
            at(T_COHESION, i, j) = std::sqrt(m[i].cohesion_energy * m[j].cohesion_energy);
            at(T_SURFACE, i, j) = std::sqrt(m[i].surface_energy * m[j].surface_energy);
            at(T_TWIST_FRICTION, i, j) =
                std::sqrt(std::fmax(m[i].twisting_friction, 0.0) * std::fmax(m[j].twisting_friction, 0.0));
            const double nu_i = m[i].poisson_ratio, nu_j = m[j].poisson_ratio;
            at(T_EEFF, i, j) = 1.0 / ((1.0 - nu_i * nu_i) / m[i].youngs_mod + (1.0 - nu_j * nu_j) / m[j].youngs_mod);
            at(T_GEFF, i, j) = 1.0 / (2.0 * (2.0 - nu_i) * (1.0 + nu_i) / m[i].youngs_mod +
                                      2.0 * (2.0 - nu_j) * (1.0 + nu_j) / m[j].youngs_mod);
            const double ki = m[i].kn, kj = m[j].kn;
            at(T_KN, i, j) = (ki > 0.0 && kj > 0.0) ? 2.0 * ki * kj / (ki + kj) : 0.0;
            const double kti = m[i].kt, ktj = m[j].kt;
            at(T_KT, i, j) = (kti > 0.0 && ktj > 0.0) ? 2.0 * kti * ktj / (kti + ktj) : 0.0;
            const double kri = m[i].rolling_stiffness, krj = m[j].rolling_stiffness;
            at(T_KROLL, i, j) = (kri > 0.0 && krj > 0.0) ? 2.0 * kri * krj / (kri + krj) : (kri > 0.0 ? kri : krj);
            at(T_GROLL, i, j) = std::sqrt(std::fmax(m[i].rolling_damping, 0.0) * std::fmax(m[j].rolling_damping, 0.0));
            const double kwi = m[i].twisting_stiffness, kwj = m[j].twisting_stiffness;
            at(T_KTWIST, i, j) = (kwi > 0.0 && kwj > 0.0) ? 2.0 * kwi * kwj / (kwi + kwj) : (kwi > 0.0 ? kwi : kwj);
            at(T_GTWIST, i, j) =
                std::sqrt(std::fmax(m[i].twisting_damping, 0.0) * std::fmax(m[j].twisting_damping, 0.0));
        }
}

int validate_config(const mdg_config& c) {
    if (c.kind != MDG_KIND_DEM && c.kind != MDG_KIND_LJ) return MDG_ERR_CONFIG;
    if (c.precision != MDG_FP64 && c.precision != MDG_MIXED) return MDG_ERR_CONFIG;
    if (!(c.dt > 0.0) || !std::isfinite(c.dt)) return MDG_ERR_CONFIG;
    for (int d = 0; d < 3; d++)
        if (!(c.box_hi[d] > c.box_lo[d])) return MDG_ERR_CONFIG;
    if (!(c.skin_fraction >= 1.0) || !(c.bin_size > 0.0)) return MDG_ERR_CONFIG;
    if (c.every < 0 || c.sort_every < 0) return MDG_ERR_CONFIG;
    if (c.kind == MDG_KIND_DEM) {
        if (c.n_materials < 1 || !c.materials) return MDG_ERR_CONFIG;
        for (int k = 0; k < c.n_materials; k++) {
            const mdg_material& m = c.materials[k];
            if (!(m.youngs_mod > 0.0) || !(m.restitution > 0.0) || m.restitution > 1.0) return MDG_ERR_CONFIG;
            if (m.poisson_ratio < 0.0 || m.poisson_ratio >= 0.5) return MDG_ERR_CONFIG;
        }
        if (c.contact_model == MDG_CONTACT_HOOKE) {
            for (int k = 0; k < c.n_materials; k++)
                if (!(c.materials[k].kn > 0.0)) return MDG_ERR_CONFIG;
        }
    } else if (c.n_lj_types > 1) {
        // the pair table replaces the single type; it must be symmetric, as
        // PairCoeffTable::set makes it (mddem_core/src/pair_coeff.rs:37-41)
        if (!c.lj_pairs) return MDG_ERR_CONFIG;
        const int nt = c.n_lj_types;
        for (int a = 0; a < nt; a++)
            for (int b = 0; b < nt; b++) {
                const mdg_lj_pair& q = c.lj_pairs[a * nt + b];
                const mdg_lj_pair& r = c.lj_pairs[b * nt + a];
                if (!(q.epsilon >= 0.0) || !(q.sigma > 0.0) || !(q.cutoff > 0.0) || !std::isfinite(q.epsilon) ||
                    !std::isfinite(q.sigma) || !std::isfinite(q.cutoff))
                    return MDG_ERR_CONFIG;
                if (q.epsilon != r.epsilon || q.sigma != r.sigma || q.cutoff != r.cutoff) return MDG_ERR_CONFIG;
            }
    } else {
        if (c.n_lj_types < 0) return MDG_ERR_CONFIG;
        if (!(c.lj_epsilon > 0.0) || !(c.lj_sigma > 0.0) || !(c.lj_cutoff > 0.0)) return MDG_ERR_CONFIG;
    }
    if (c.nose_hoover && (!(c.nh_temperature > 0.0) || !(c.nh_coupling > 0.0))) return MDG_ERR_CONFIG;
    if (c.langevin && (c.nose_hoover || !(c.lv_temperature >= 0.0) || !(c.lv_damping >= 0.0))) return MDG_ERR_CONFIG;
    if (c.n_walls < 0 || c.n_walls > MDG_MAX_WALLS || (c.n_walls > 0 && (!c.walls || c.kind != MDG_KIND_DEM)))
        return MDG_ERR_CONFIG;
    for (int w = 0; w < c.n_walls; w++) {
        const mdg_wall& q = c.walls[w];
        const double mag = sqrt(q.normal[0] * q.normal[0] + q.normal[1] * q.normal[1] + q.normal[2] * q.normal[2]);
        if (!(mag > 1e-15) || q.material < 0 || q.material >= c.n_materials) return MDG_ERR_CONFIG;
    }
    const int t = c.threads_per_particle;
    if (!(t == 0 || t == 1 || t == 2 || t == 4 || t == 8)) return MDG_ERR_CONFIG;
    if (c.neighbor_capacity < 0 || c.history_capacity < 0) return MDG_ERR_CONFIG;
    return MDG_OK;
}

}  // namespace

struct mdg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // captures the conditional rebuild branch
    int nsys = 0;
    std::vector<mdg_config> cfg;
    std::vector<std::vector<mdg_material>> mats;
    std::vector<std::vector<mdg_wall>> wls;     // per system: its plane walls
    std::vector<std::vector<mdg_lj_pair>> ljp;  // per system: the LJ pair table (1 x 1 for one type)
    std::vector<int> ljn;                       // its number of types
    std::vector<SysParams> sp;
    std::vector<size_t> capacity;
    std::vector<int> uploaded;
    std::vector<int> ncap_sys;  // current list capacity per system
    // step budget of each system as the device counts it (-1 unlimited):
    // every running system advances every step until its budget reaches 0
    std::vector<long long> rem_host;
    std::vector<int> run_sys;      // systems in the current run maps
    bool maps_dirty = true;
    std::vector<int> cblk0_host, cseg_blocks;  // cell segment of each system
    int* d_blk_run = nullptr;
    int* d_blk_run_kind[2] = {nullptr, nullptr};
    int* d_cblk_run = nullptr;
    int* d_run_sys = nullptr;
    Dev d{};
    bool has_lj = false, has_dem = false, has_mixed = false, any_virial = false;
    int tpp_lj = 1;
    int build_mode = -1;  // list-build mode of every system; -1 = chosen per system
    long long cells_alloc = 0, lst_alloc = 0;
    int* d_blk_sys = nullptr;
    int* d_cblk_sys = nullptr;
    int* d_cblk0 = nullptr;
    SysParams* d_sp = nullptr;
    double* d_mat = nullptr;
    float* d_matf = nullptr;
    double* d_thermo = nullptr;
    std::vector<long long> mat_off;
    int graph_mode = 1;
    cudaGraphExec_t wgraph = nullptr;                 // multi-step WHILE graph
    cudaGraphExec_t tgraph = nullptr;                 // timed single-step graph
    long long* d_loop = nullptr;  // {iterations left, iterations of the launch} of the WHILE graph
    bool run_nh = false;          // some running system is thermostatted
    bool has_walls = false;       // some system has plane walls (once set, stays)
    // measurement scratch (allocated on first use, grown when needed)
    float4* rdf_posf = nullptr;
    long long rdf_posf_n = 0;
    unsigned long long* rdf_counts = nullptr;
    int rdf_counts_n = 0;
    std::vector<double*> msd_ref;       // per system: unwrapped positions by tag
    std::vector<long long> msd_ntag;    // per system: tags covered (max tag + 1)
    double* msd_part = nullptr;
    long long msd_part_n = 0;
    cudaEvent_t tev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    int tkernels = 0;
    void* flush_buf = nullptr;
    size_t flush_bytes = 0;
    long long launches = 0;
    // mdg_step_async / mdg_step_wait: the launched step count (0 = none in
    // flight) and pinned copies of the rebuild-branch counter before and
    // after the launch
    int64_t pending_steps = 0;
    unsigned long long* h_stat = nullptr;
    std::vector<void*> allocs;

    ~mdg_ctx() {
        if (wgraph) cudaGraphExecDestroy(wgraph);
        if (tgraph) cudaGraphExecDestroy(tgraph);
        for (auto& e : tev)
            if (e) cudaEventDestroy(e);
        if (flush_buf) cudaFree(flush_buf);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
        if (stream2) cudaStreamDestroy(stream2);
        if (h_stat) cudaFreeHost(h_stat);
    }
    template <class T>
    T* alloc(size_t n, int& err) {
        T* p = dalloc<T>(n, err);
        if (p) allocs.push_back(p);
        return p;
    }
    void free_ptr(void* p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
    }
    void drop_graphs() {
        if (wgraph) {
            cudaGraphExecDestroy(wgraph);
            wgraph = nullptr;
        }
        if (tgraph) {
            cudaGraphExecDestroy(tgraph);
            tgraph = nullptr;
        }
    }
};

namespace {

// The per-system physics a config sets: contact laws, materials (pair tables
// into `tabs`), LJ coefficients, timestep and [neighbor] rebuild settings.
// The slot's memory layout is left alone.
void apply_physics(mdg_ctx* c, int s, const mdg_config& k, std::vector<double>& tabs) {
    SysParams& p = c->sp[s];
    c->cfg[s] = k;
    // the context keeps its own copies of the arrays the config points at;
    // each is built aside and swapped in, so a config read back by
    // mdg_get_config (pointing at the current copies) stays readable here:
    // the previous copies live in these locals until the function returns
    std::vector<mdg_wall> wl;
    std::vector<mdg_material> ml;
    std::vector<mdg_lj_pair> lp;
    if (k.walls && k.n_walls > 0) wl.assign(k.walls, k.walls + k.n_walls);
    c->wls[s].swap(wl);
    c->cfg[s].walls = c->wls[s].empty() ? nullptr : c->wls[s].data();
    if (k.kind == MDG_KIND_DEM && k.materials) ml.assign(k.materials, k.materials + k.n_materials);
    c->mats[s].swap(ml);
    c->cfg[s].materials = k.kind == MDG_KIND_DEM ? c->mats[s].data() : nullptr;
    if (k.kind != MDG_KIND_DEM) c->cfg[s].n_materials = 0;
    if (k.kind == MDG_KIND_LJ && k.n_lj_types > 1 && k.lj_pairs)
        lp.assign(k.lj_pairs, k.lj_pairs + (size_t)k.n_lj_types * k.n_lj_types);
    else if (k.kind == MDG_KIND_LJ)
        lp.assign(1, mdg_lj_pair{k.lj_epsilon, k.lj_sigma, k.lj_cutoff});
    c->ljp[s].swap(lp);
    c->cfg[s].lj_pairs = (k.kind == MDG_KIND_LJ && k.n_lj_types > 1) ? c->ljp[s].data() : nullptr;
    p.contact_model = k.contact_model;
    p.adhesion_model = k.adhesion_model;
    p.rolling_model = k.rolling_model;
    p.twisting_model = k.twisting_model;
    p.dt = k.dt;
    p.policy = k.rebuild_policy;
    p.every = k.every;
    p.check = k.check;
    p.sort_every = k.sort_every;
    p.newton = k.newton;
    p.virial = k.virial;
    for (int d = 0; d < 3; d++) p.per[d] = k.fixed[d] ? 0 : 1;
    p.nwall = k.n_walls;
    if (k.n_walls > 0) {
        if (!c->has_walls) c->drop_graphs();
        c->has_walls = true;
    }
    for (int w = 0; w < k.n_walls; w++) {
        // WallPlugin's plane set-up (dem_wall/src/lib.rs:675-685): unit normal
        const mdg_wall& q = c->wls[s][w];
        WallP& o = p.walls[w];
        const double mag = sqrt(q.normal[0] * q.normal[0] + q.normal[1] * q.normal[1] + q.normal[2] * q.normal[2]);
        for (int d = 0; d < 3; d++) {
            o.p[d] = q.point[d];
            o.nrm[d] = q.normal[d] / mag;
            o.lo[d] = q.bound_lo[d];
            o.hi[d] = q.bound_hi[d];
            o.vel[d] = q.velocity[d];
        }
        o.mat = q.material;
    }
    p.lv = k.langevin && k.lv_damping > 0.0;  // gamma = 0: no forces (langevin_force's early return)
    p.lv_gamma = k.lv_damping;
    p.lv_kT = k.lv_temperature;
    p.lv_seed = (unsigned long long)k.lv_seed;
    p.tpp = k.threads_per_particle ? k.threads_per_particle : 1;
    tabs.clear();
    if (k.kind == MDG_KIND_DEM) {
        material_tables(c->mats[s].data(), k.n_materials, tabs);
        p.nmat = k.n_materials;
        // no JKR pull-off range: a pair interacts only when the spheres touch
        bool pull = false;
        for (int m = 0; m < k.n_materials; m++) pull = pull || c->mats[s][m].surface_energy > 0.0;
        p.touch_only = (k.contact_model == 1 || k.adhesion_model == 1 || !pull) ? 1 : 0;
    } else {
        // the pair table (build_lj_pair_table, crates/md_lj/src/lib.rs:334-384):
        // n x n from the config, or 1 x 1 from the single type
        const int nt = k.n_lj_types > 1 ? k.n_lj_types : 1;
        c->ljn[s] = nt;
        // LJPairCoeffs::from_params (crates/md_lj/src/lib.rs:230-239), plus
        // 4 eps sigma^12 and 4 eps sigma^6 for the energy
        auto coeffs = [](const mdg_lj_pair& q, double* o) {
            const double s2 = q.sigma * q.sigma;
            const double sigma6 = s2 * s2 * s2;
            o[TL_LJ1] = 48.0 * q.epsilon * sigma6 * sigma6;
            o[TL_LJ2] = 24.0 * q.epsilon * sigma6;
            o[TL_LJ3] = 4.0 * q.epsilon * sigma6 * sigma6;
            o[TL_LJ4] = 4.0 * q.epsilon * sigma6;
            const double rc = q.cutoff * q.sigma;
            o[TL_CUT2] = rc * rc;
        };
        double o[NTAB_LJ];
        coeffs(c->ljp[s][0], o);
        p.lj1 = o[TL_LJ1];
        p.lj2 = o[TL_LJ2];
        p.lj3 = o[TL_LJ3];
        p.lj4 = o[TL_LJ4];
        p.lj_cut2 = o[TL_CUT2];
        p.lj1f = (float)p.lj1;
        p.lj2f = (float)p.lj2;
        p.lj3f = (float)p.lj3;
        p.lj4f = (float)p.lj4;
        p.lj_cut2f = (float)p.lj_cut2;
        p.nmat = nt;
        if (nt > 1) {
            tabs.assign((size_t)NTAB_LJ * nt * nt, 0.0);
            for (int a = 0; a < nt; a++)
                for (int b = 0; b < nt; b++) {
                    coeffs(c->ljp[s][(size_t)a * nt + b], o);
                    for (int t = 0; t < NTAB_LJ; t++) tabs[((size_t)t * nt + a) * nt + b] = o[t];
                }
            if (!c->d.lj_multi) c->drop_graphs();  // the force launch changes instantiation
            c->d.lj_multi = 1;
        }
    }
}

int cuda_err(cudaError_t e) {
    if (e == cudaSuccess) return MDG_OK;
    if (e == cudaErrorMemoryAllocation) return MDG_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MDG_ERR_NODEVICE;
    return MDG_ERR_CUDA;
}

// neighbor_setup + compute_bin_grid (crates/mddem_core/src/neighbor.rs:480-541,
// 290-371) for one rank, from the uploaded cutoff radii.
// List build mode (all give the same rows): under about 6 particles per bin
// a thread per particle; a warp per bin from 512 bins on in a single-system
// context, from 64 in a batch (and no more bins than particles, as bins take
// particle slots); else a warp per particle.  Measured on GB300 (LJ melts,
// rho 0.85), one system alone: a warp per particle is faster up to about
// 7000 atoms (343 bins: 59 against 75 us: a few hundred warps leave the GPU
// idle), a warp per bin from about 1300 bins on (27436 atoms: 99 against
// 203 us).  In a batch several systems rebuild in the same launch and fill
// the GPU together, and a warp per bin does about half the work per atom:
// the served stream runs 3.06 G particle-steps/s with the threshold at 512
// bins, 3.15 G at 216, 3.16 G at 64.
int auto_build_mode(const SysParams& p, size_t n, bool batch) {
    const double nbins = (double)p.nc[0] * (double)p.nc[1] * (double)p.nc[2];
    if ((double)n < 6.0 * nbins) return 2;
    if (nbins >= (batch ? 64.0 : 512.0) && (size_t)p.ncell <= n) return 0;
    return 1;
}

int setup_grid(const mdg_config& c, double min_skin, double max_skin, size_t n, SysParams& p) {
    const double sf = c.skin_fraction;
    double bin_min = c.bin_size;
    const double max_cutoff = max_skin > 0.0 ? 2.0 * max_skin * sf : bin_min;
    const double disp_buf = (min_skin < std::numeric_limits<double>::max() * 0.5) ? (sf - 1.0) * min_skin : 0.0;
    const double ghost_cutoff = std::fmax(max_cutoff + 2.0 * disp_buf, 0.0);
    if (bin_min < max_cutoff) bin_min = max_cutoff;
    const double min_bin = std::fmax(bin_min, max_cutoff);
    const double ghost_cut = ghost_cutoff > max_cutoff ? ghost_cutoff : max_cutoff;
    long long ncell = 1;
    for (int d = 0; d < 3; d++) {
        p.lo[d] = c.box_lo[d];
        p.hi[d] = c.box_hi[d];
        p.L[d] = c.box_hi[d] - c.box_lo[d];
        const int xi = (int)std::fmax(std::floor(p.L[d] / min_bin), 1.0);
        p.nc[d] = xi;
        p.bin[d] = p.L[d] / (double)xi;
        p.inv_bin[d] = 1.0 / p.bin[d];
        const int sr = (int)std::ceil(max_cutoff / p.bin[d]);
        p.sl[d] = (int)std::ceil(ghost_cut / p.bin[d]) + sr;
        p.ext[d] = xi + 2 * p.sl[d];
        p.origin[d] = p.lo[d] - p.bin[d] * (double)p.sl[d];
        p.win[d] = sr;
        ncell *= p.ext[d];
        // one periodic image per neighbour: the box must exceed twice the list cutoff
        if (!c.fixed[d] && !(p.L[d] > 2.0 * max_cutoff)) return MDG_ERR_CONFIG;
        if (p.win[d] > xi) return MDG_ERR_CONFIG;
    }
    if (ncell > (1LL << 30)) return MDG_ERR_CONFIG;
    p.ncell = (int)ncell;
    p.build_mode = auto_build_mode(p, n, false);
    p.max_cutoff = max_cutoff;
    p.stencil_cut_sq = max_cutoff * max_cutoff;
    // stencil membership of every offset (compute_bin_grid's distance test,
    // neighbor.rs:341-361), as a bit table indexed by the offset
    const int wx = 2 * p.sl[0] + 1, wy = 2 * p.sl[1] + 1, wz = 2 * p.sl[2] + 1;
    if ((long long)wx * wy * wz > 32 * 32) return MDG_ERR_CONFIG;
    std::memset(p.stencil_bits, 0, sizeof(p.stencil_bits));
    for (int dx = -p.sl[0]; dx <= p.sl[0]; dx++)
        for (int dy = -p.sl[1]; dy <= p.sl[1]; dy++)
            for (int dz = -p.sl[2]; dz <= p.sl[2]; dz++) {
                const double mdx = (double)std::max(std::abs(dx) - 1, 0) * p.bin[0];
                const double mdy = (double)std::max(std::abs(dy) - 1, 0) * p.bin[1];
                const double mdz = (double)std::max(std::abs(dz) - 1, 0) * p.bin[2];
                if (mdx * mdx + mdy * mdy + mdz * mdz < p.stencil_cut_sq) {
                    const int b = ((dx + p.sl[0]) * wy + (dy + p.sl[1])) * wz + (dz + p.sl[2]);
                    p.stencil_bits[b >> 5] |= 1u << (b & 31);
                }
            }
    p.skin_fraction = sf;
    p.sf2 = sf * sf;
    p.min_skin = min_skin;
    p.uniform = std::fabs(max_skin - min_skin) < 1e-15;
    const double uc = 2.0 * min_skin * sf;
    p.uniform_cutoff_sq = uc * uc;
    p.ucut2f = (float)p.uniform_cutoff_sq;
    p.sf2f = (float)p.sf2;
    for (int d = 0; d < 3; d++) {
        p.Lh[d] = (float)p.L[d];
        p.Ll[d] = (float)(p.L[d] - (double)p.Lh[d]);
        p.uinv[d] = std::ldexp(1.0, 32) / p.L[d];
        p.uscale[d] = (float)std::ldexp(p.L[d], -32);
        // mixed LJ: the wrapped fixed-point difference is the separation only
        // below L / 2, on fixed axes too
        if (c.kind == MDG_KIND_LJ && c.precision == MDG_MIXED && !(p.L[d] > 2.0 * max_cutoff)) return MDG_ERR_CONFIG;
    }
    const double per_atom_skin = (sf - 1.0) * min_skin;
    p.disp_thr_sq = per_atom_skin * per_atom_skin;
    p.disp_thr2f = (float)(p.disp_thr_sq * (1.0 - 1e-5));
    // fp32 prefilter: bound the error of (x_j_hi + s L_f) - x_i_hi per axis
    double xmax = 0.0;
    for (int d = 0; d < 3; d++) xmax = std::fmax(xmax, std::fmax(std::fabs(p.lo[d]), std::fabs(p.hi[d])) + 2.0 * p.L[d]);
    const double E = 8.0 * std::ldexp(1.0, -24) * xmax;
    const double rpre = max_cutoff + 2.0 * std::sqrt(3.0) * E;
    p.pre_cut2 = std::nextafter((float)(rpre * rpre * (1.0 + 1e-5)), std::numeric_limits<float>::infinity());
    // |r2_hi - r2| <= (2 r + 2 sqrt(3) E) 2 sqrt(3) E + fp32 rounding; relative to the
    // smallest pair cutoff of the system
    const double rmin_cut = std::fmax(2.0 * min_skin * sf, 1e-300);
    const double eabs = (2.0 * rpre + 2.0 * std::sqrt(3.0) * E) * 2.0 * std::sqrt(3.0) * E;
    p.band_rel = (float)(2.0 * eabs / (rmin_cut * rmin_cut) + 1e-5);
    return MDG_OK;
}

int auto_ncap(const mdg_config& c, const SysParams& p, size_t n) {
    if (c.neighbor_capacity > 0) return c.neighbor_capacity;
    const double vol = p.L[0] * p.L[1] * p.L[2];
    const double rho = (double)n / vol;
    const double rc = p.max_cutoff;
    const double expect = rho * 4.0 / 3.0 * kPi * rc * rc * rc;
    int cap;
    if (c.kind == MDG_KIND_LJ) cap = (int)std::ceil(expect * 1.4) + 24;
    else cap = std::max(32, (int)std::ceil(expect * 3.0) + 24);
    return std::min(cap, 1024);
}

int sys_status_to_err(int st) {
    if (st & ST_OVERLAP) return MDG_ERR_OVERLAP_LIMIT;
    if (st & ST_NAN) return MDG_ERR_NAN;
    if (st & (ST_NBR_OVF | ST_HIST_OVF)) return MDG_ERR_LIST_OVERFLOW;
    if (st & ST_TIMEOUT) return MDG_ERR_TIMEOUT;
    if (st & ST_LOST) return MDG_ERR_LOST;
    return MDG_OK;
}

// (Re)compute cell and list segment offsets; (re)allocate when they grow.
// Cell arrays only live within one rebuild, so they are simply reallocated.
// Neighbour-list blocks of systems other than `fresh` (whose list is rebuilt
// on its next step anyway) are copied to their new offsets, so a system
// uploaded into a running batch does not disturb the others.
int ensure_layout(mdg_ctx* c, int fresh = -1) {
    int err = 0;
    long long cells = 0;
    std::vector<int> cblk_sys, cblk0(c->nsys);
    std::vector<long long> old_lst0(c->nsys);
    long long lst = 0;
    for (int s = 0; s < c->nsys; s++) {
        SysParams& p = c->sp[s];
        p.c0 = (int)cells;
        const long long seg = round_up((long long)p.ncell + 1, BLK);
        cblk0[s] = (int)(cells / BLK);
        c->cseg_blocks[s] = (int)(seg / BLK);
        p.ncb = (int)(seg / BLK);
        for (long long b = 0; b < seg / BLK; b++) cblk_sys.push_back(s);
        cells += seg;
        old_lst0[s] = p.lst0;
        p.lst0 = lst;
        lst += (long long)p.ncap * p.npad;
    }
    bool realloc_cells = cells > c->cells_alloc;
    bool moved = false;
    for (int s = 0; s < c->nsys; s++)
        if (s != fresh && c->uploaded[s] && old_lst0[s] != c->sp[s].lst0) moved = true;
    bool realloc_lst = lst > c->lst_alloc || moved;
    if (realloc_cells) {
        c->free_ptr(c->d.cnt);
        c->free_ptr(c->d.cstart);
        c->free_ptr(c->d.csum);
        c->free_ptr(c->d.cbase);
        c->free_ptr(c->d_cblk_sys);
        c->free_ptr(c->d_cblk_run);
        c->d.cnt = c->alloc<int>(cells, err);
        c->d.cstart = c->alloc<int>(cells, err);
        c->d.csum = c->alloc<int>(cells / BLK, err);
        c->d.cbase = c->alloc<int>(cells / BLK, err);
        c->d_cblk_sys = c->alloc<int>(cells / BLK, err);
        c->d_cblk_run = c->alloc<int>(cells / BLK, err);
        if (err) return err;
        c->cells_alloc = cells;
        c->drop_graphs();
    }
    if (realloc_lst) {
        const long long cap = std::max(lst, c->lst_alloc);
        uint32_t* nl = c->alloc<uint32_t>(cap, err);
        if (err) return err;
        if (c->d.nlist) {
            for (int s = 0; s < c->nsys; s++) {
                if (s == fresh || !c->uploaded[s]) continue;
                const SysParams& p = c->sp[s];
                cudaMemcpy(nl + p.lst0, c->d.nlist + old_lst0[s], (size_t)p.ncap * p.npad * sizeof(uint32_t),
                           cudaMemcpyDeviceToDevice);
            }
        }
        c->free_ptr(c->d.nlist);
        c->d.nlist = nl;
        c->lst_alloc = cap;
        c->drop_graphs();
    }
    // the per-cell kernels run over every allocated cell block, so captured
    // graphs stay valid while the systems' cell grids change inside the
    // allocation; blocks past the systems' cells find -1 and return
    cblk_sys.resize((size_t)(c->cells_alloc / BLK), -1);
    cudaMemcpy(c->d_cblk_sys, cblk_sys.data(), cblk_sys.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_cblk0, cblk0.data(), cblk0.size() * sizeof(int), cudaMemcpyHostToDevice);
    c->d.cblk_sys = c->d_cblk_sys;
    c->d.cblk0 = c->d_cblk0;
    c->cblk0_host = cblk0;
    c->maps_dirty = true;
    c->d.ncblocks = (int)(c->cells_alloc / BLK);
    cudaMemcpy(c->d_sp, c->sp.data(), c->nsys * sizeof(SysParams), cudaMemcpyHostToDevice);
    return cuda_err(cudaGetLastError());
}

// Run maps for the next launch: the particle and cell blocks of the systems
// that will advance (uploaded, budget not exhausted).  Captured graphs carry
// the maps' lengths as grid sizes, so they are dropped when the set changes.
// Returns the number of running systems, or -MDG_ERR_CUDA.
int update_run_maps(mdg_ctx* c) {
    std::vector<int> run;
    for (int s = 0; s < c->nsys; s++)
        if (c->uploaded[s] && c->rem_host[s] != 0) run.push_back(s);
    if (!c->maps_dirty && run == c->run_sys) return (int)run.size();
    std::vector<int> pb, cb, pk[2];
    for (int s : run) {
        const SysParams& p = c->sp[s];
        for (int b = 0; b < p.nb; b++) {
            pb.push_back(p.b0 + b);
            pk[p.kind == 1 ? 1 : 0].push_back(p.b0 + b);
        }
        for (int b = 0; b < c->cseg_blocks[s]; b++) cb.push_back(c->cblk0_host[s] + b);
    }
    if (!pb.empty() &&
        (cudaMemcpyAsync(c->d_blk_run, pb.data(), pb.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream) !=
             cudaSuccess ||
         cudaMemcpyAsync(c->d_cblk_run, cb.data(), cb.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream) !=
             cudaSuccess ||
         cudaMemcpyAsync(c->d_run_sys, run.data(), run.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream) !=
             cudaSuccess))
        return -MDG_ERR_CUDA;
    for (int q = 0; q < 2; q++) {
        if (!pk[q].empty() && cudaMemcpyAsync(c->d_blk_run_kind[q], pk[q].data(), pk[q].size() * sizeof(int),
                                              cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return -MDG_ERR_CUDA;
        c->d.blk_run_kind[q] = c->d_blk_run_kind[q];
        c->d.nrun_kind[q] = (int)pk[q].size();
    }
    c->drop_graphs();  // grid sizes follow the maps
    c->d.blk_run = c->d_blk_run;
    c->d.cblk_run = c->d_cblk_run;
    c->d.nrun = (int)pb.size();
    c->d.ncrun = (int)cb.size();
    c->d.run_sys = c->d_run_sys;
    c->d.nrun_sys = (int)run.size();
    c->run_sys = run;
    c->run_nh = false;
    for (int s : run) c->run_nh = c->run_nh || c->sp[s].nh;
    c->maps_dirty = false;
    return (int)run.size();
}

// Budgets after n more steps of the running systems.
void advance_budgets(mdg_ctx* c, int64_t n) {
    for (int s : c->run_sys)
        if (c->rem_host[s] > 0) c->rem_host[s] = c->rem_host[s] > n ? c->rem_host[s] - n : 0;
}

// Rebuild pipeline (+ the mixed DEM worklist) and final kernel of the
// context's precision.
int launch_rb(mdg_ctx* c, const Dev& d, cudaStream_t st) {
    return launch_rebuild(d, st) + (c->has_mixed ? launch_rebuild_tail_mixed(d, c->has_dem, st) : 0);
}
int rb_kernels(const mdg_ctx* c) { return 9 + (c->has_mixed && c->has_dem ? 1 : 0); }
int launch_fin(mdg_ctx* c, const Dev& d, cudaStream_t st, int integrate) {
    return c->has_mixed ? launch_final_mixed(d, st, integrate) : launch_final(d, st, integrate);
}

int launch_force(mdg_ctx* c, const Dev& d, cudaStream_t st, int integrating = 1) {
    int n = c->has_mixed ? launch_force_mixed(d, c->has_lj, c->has_dem, c->tpp_lj, st)
                         : launch_force_fp64(d, c->has_lj, c->has_dem, c->tpp_lj, st);
    if (c->has_walls) n += launch_walls(d, integrating, st);  // added after the pair forces
    return n;
}

int enqueue_step(mdg_ctx* c, cudaStream_t st) {
    int n = 0;
    n += c->has_mixed ? launch_initial_mixed(c->d, st) : launch_initial(c->d, st);
    n += launch_rb(c, c->d, st);
    n += launch_force(c, c->d, st);
    n += launch_fin(c, c->d, st, 1);
    return n;
}

// Capture one step into the graph being captured on c->stream: the rebuild
// pipeline sits in the body of an IF conditional node whose condition
// k_initial sets on the device.  ev (optional) = 5 events bracketing the
// phases.  Returns kernels in the step (rebuild kernels counted when run).
int capture_step(mdg_ctx* c, cudaEvent_t* ev, int* nk) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraphConditionalHandle hd;
    e = cudaGraphConditionalHandleCreate(&hd, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return cuda_err(e);
    Dev d = c->d;
    d.cond = (unsigned long long)hd;
    d.use_cond = 1;
    int n = 0;
    if (ev) cudaEventRecordWithFlags(ev[0], c->stream, cudaEventRecordExternal);
    n += c->has_mixed ? launch_initial_mixed(d, c->stream) : launch_initial(d, c->stream);
    if (ev) cudaEventRecordWithFlags(ev[1], c->stream, cudaEventRecordExternal);
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hd;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaStreamBeginCaptureToGraph(c->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(e);
    n += launch_rb(c, d, c->stream2);
    cudaGraph_t body_out = nullptr;
    e = cudaStreamEndCapture(c->stream2, &body_out);
    if (e != cudaSuccess) return cuda_err(e);
    if (ev) cudaEventRecordWithFlags(ev[2], c->stream, cudaEventRecordExternal);
    n += launch_force(c, d, c->stream);
    if (ev) cudaEventRecordWithFlags(ev[3], c->stream, cudaEventRecordExternal);
    n += launch_fin(c, d, c->stream, 1);
    if (ev) cudaEventRecordWithFlags(ev[4], c->stream, cudaEventRecordExternal);
    if (nk) *nk = n;
    return MDG_OK;
}

// The WHILE body of a mixed-precision context: the fused step kernel (final
// half of the previous step + initial half of this one), the thermostatted
// systems' initial half, the rebuild IF node, the force kernels.
int capture_body_mixed(mdg_ctx* c, int* nk) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraphConditionalHandle hd;
    e = cudaGraphConditionalHandleCreate(&hd, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return cuda_err(e);
    Dev d = c->d;
    d.cond = (unsigned long long)hd;
    d.use_cond = 1;
    int n = launch_step_mixed(d, c->d_loop, c->stream);
    if (c->run_nh) n += launch_initial_mixed(d, c->stream, 1, c->d_loop);
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hd;
    np.conditional.type = cudaGraphCondTypeIf;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
    if (e != cudaSuccess) return cuda_err(e);
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaStreamBeginCaptureToGraph(c->stream2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(e);
    n += launch_rb(c, d, c->stream2);
    cudaGraph_t body_out = nullptr;
    e = cudaStreamEndCapture(c->stream2, &body_out);
    if (e != cudaSuccess) return cuda_err(e);
    n += launch_force(c, d, c->stream);
    if (nk) *nk = n;
    return MDG_OK;
}

// Multi-step graph: a WHILE conditional node whose body is one step (with the
// rebuild IF node inside) followed by the loop-control kernel, which counts
// down d_loop and closes the loop when it reaches zero or no system is active.
// One launch runs any number of steps without returning to the host.  Mixed
// contexts loop over the fused body and finish the last step after the loop.
int build_while_graph(mdg_ctx* c) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(e);
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    int r = MDG_OK;
    cudaGraphConditionalHandle wh;
    cudaGraphNode_t node;
    cudaGraphNodeParams np{};
    e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &cg, nullptr, nullptr, nullptr);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&wh, cg, 1, cudaGraphCondAssignDefault);
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &cg, &deps, nullptr, &nd);
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = wh;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np);
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    // mixed path: the loop's fused kernels leave the last step's final half,
    // done once after the loop
    if (e == cudaSuccess && c->has_mixed) launch_fin(c, c->d, c->stream, 1);
    cudaGraph_t g_end = nullptr;
    e = e == cudaSuccess ? cudaStreamEndCapture(c->stream, &g) : (cudaStreamEndCapture(c->stream, &g_end), e);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (g_end) cudaGraphDestroy(g_end);
        return cuda_err(e);
    }
    // body: capture on c->stream into the WHILE body graph
    cudaGraph_t body = np.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        r = c->has_mixed ? capture_body_mixed(c, nullptr) : capture_step(c, nullptr, nullptr);
        if (!r) launch_loop_ctl(c->d, c->d_loop, (unsigned long long)wh, c->stream);
        cudaGraph_t bo = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &bo);
        if (!r && e2 != cudaSuccess) r = cuda_err(e2);
    } else {
        r = cuda_err(e);
    }
    if (!r) {
        e = cudaGraphInstantiate(&c->wgraph, g, 0);
        if (e != cudaSuccess) r = cuda_err(e);
    }
    cudaGraphDestroy(g);
    return r;
}

// One step captured with event records between its phases.
int build_timed_graph(mdg_ctx* c) {
    for (auto& e : c->tev)
        if (!e && cudaEventCreate(&e) != cudaSuccess) return MDG_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(e);
    int n = 0;
    int r = capture_step(c, c->tev, &n);
    e = cudaStreamEndCapture(c->stream, &g);
    if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaGraphInstantiate(&c->tgraph, g, 0);
    cudaGraphDestroy(g);
    c->tkernels = n;
    return cuda_err(e);
}

int sys_hcur(mdg_ctx* c, int sys) {
    SysState ss;
    cudaMemcpy(&ss, c->d.ss + sys, sizeof(SysState), cudaMemcpyDeviceToHost);
    return ss.hcur & 1;
}

int check_status(mdg_ctx* c) {
    std::vector<SysState> ss(c->nsys);
    cudaError_t e = cudaMemcpy(ss.data(), c->d.ss, c->nsys * sizeof(SysState), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e);
    for (int s = 0; s < c->nsys; s++) {
        int r = sys_status_to_err(ss[s].status);
        if (r) return r;
    }
    return MDG_OK;
}

}  // namespace

extern "C" {

int mdg_abi_version(void) { return MDG_ABI_VERSION; }

const char* mdg_status_string(int s) {
    switch (s) {
        case MDG_OK: return "ok";
        case MDG_ERR_CONFIG: return "invalid configuration";
        case MDG_ERR_CUDA: return "CUDA runtime error";
        case MDG_ERR_OOM: return "device allocation failed";
        case MDG_ERR_BUDGET: return "request exceeds the HBM budget";
        case MDG_ERR_OVERLAP_LIMIT: return "more than 500 large overlaps in one step";
        case MDG_ERR_NAN: return "non-finite value in the particle state";
        case MDG_ERR_LIST_OVERFLOW: return "neighbor or contact-history capacity exceeded";
        case MDG_ERR_TIMEOUT: return "bounded device wait gave up";
        case MDG_ERR_ARG: return "bad argument";
        case MDG_ERR_STATE: return "call out of order";
        case MDG_ERR_NODEVICE: return "no CUDA device";
        case MDG_ERR_LOST: return "a particle left the box across a fixed boundary";
        default: return "unknown status";
    }
}

int mdg_device_count(int* count) {
    if (!count) return MDG_ERR_ARG;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
        return MDG_ERR_NODEVICE;
    }
    *count = n;
    return MDG_OK;
}

int mdg_batch_create(const mdg_config* cfgs, const size_t* capacity, int nsys, mdg_ctx** out) {
    if (!cfgs || !capacity || nsys < 1 || !out) return MDG_ERR_ARG;
    *out = nullptr;
    for (int s = 0; s < nsys; s++) {
        int r = validate_config(cfgs[s]);
        if (r) return r;
        if (capacity[s] < 1 || capacity[s] > (size_t)IDX_MASK) return MDG_ERR_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MDG_ERR_NODEVICE;
    }
    mdg_ctx* c = new (std::nothrow) mdg_ctx();
    if (!c) return MDG_ERR_OOM;
    cudaGetDevice(&c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&c->h_stat, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return MDG_ERR_CUDA;
    }
    c->nsys = nsys;
    c->cfg.assign(cfgs, cfgs + nsys);
    c->mats.resize(nsys);
    c->ljp.resize(nsys);
    c->wls.resize(nsys);
    c->ljn.assign(nsys, 1);
    c->sp.assign(nsys, SysParams{});
    c->capacity.assign(capacity, capacity + nsys);
    c->uploaded.assign(nsys, 0);
    c->rem_host.assign(nsys, 0);
    c->cseg_blocks.assign(nsys, 0);
    long long P = 0;
    int nblocks = 0;
    long long hist_entries = 0;
    std::vector<int> blk_sys;
    std::vector<double> mat_all;
    int has_mixed = -1;
    for (int s = 0; s < nsys; s++) {
        const mdg_config& k = cfgs[s];
        SysParams& p = c->sp[s];
        p.kind = k.kind;
        p.precision = k.precision;
        if (has_mixed < 0) has_mixed = k.precision;
        else if (has_mixed != k.precision) {
            delete c;
            return MDG_ERR_CONFIG;  // one precision per context
        }
        // memory layout of the slot (fixed for the context's lifetime)
        p.npad = (int)round_up((long long)capacity[s], BLK);
        p.p0 = (int)P;
        p.n = 0;
        p.b0 = nblocks;
        p.nb = 0;  // blocks in use: set by each upload
        for (int b = 0; b < p.npad / BLK; b++) blk_sys.push_back(s);
        nblocks += p.npad / BLK;
        P += p.npad;
        p.ncap = 0;
        if (k.kind == MDG_KIND_DEM) {
            c->has_dem = true;
            p.matcap = std::max(k.n_materials, 4);
            p.mat0 = (long long)mat_all.size();
            mat_all.resize(mat_all.size() + (size_t)NTAB * p.matcap * p.matcap, 0.0);
            p.hcap = k.history_capacity ? k.history_capacity : 24;
            p.h0 = hist_entries;
            hist_entries += (long long)p.hcap * p.npad;
        } else {
            c->has_lj = true;
            // pair-table slots: the config's types, at least 4 (a reconfigured
            // or served system may bring more types than its first config)
            p.matcap = std::max(k.n_lj_types, 4);
            p.mat0 = (long long)mat_all.size();
            mat_all.resize(mat_all.size() + (size_t)NTAB_LJ * p.matcap * p.matcap, 0.0);
            p.hcap = 0;
        }
        if (k.virial) c->any_virial = true;
        // threads per particle of the LJ force kernel: explicit, or 2 for the
        // mixed path and 1 for fp64 (measured on GB300 with ~76-entry rows:
        // the served stream 3.47 G particle-steps/s at 2 against 3.40 G at 4
        // and 3.03 G at 8; LJ 256k alone 0.068 against 0.074 ms per force)
        if (k.threads_per_particle > 0) c->tpp_lj = k.threads_per_particle;
        else if (k.kind == MDG_KIND_LJ && k.precision == MDG_MIXED) c->tpp_lj = 2;
        // the physics of the slot (replaceable by mdg_configure_system)
        std::vector<double> tabs;
        apply_physics(c, s, k, tabs);
        if (!tabs.empty()) std::copy(tabs.begin(), tabs.end(), mat_all.begin() + p.mat0);
    }
    if (P > (long long)IDX_MASK * 8) {
        delete c;
        return MDG_ERR_ARG;
    }
    c->has_mixed = has_mixed == MDG_MIXED;
    int err = 0;
    Dev& d = c->d;
    d.P = P;
    d.nsys = nsys;
    d.nblocks = nblocks;
    d.pos = c->alloc<double4>(P, err);
    d.vel = c->alloc<double4>(P, err);
    d.frc = c->alloc<double4>(P, err);
    d.lbp = c->alloc<double4>(P, err);
    d.mass = c->alloc<double>(P, err);
    d.cutr = c->alloc<double>(P, err);
    d.tag = c->alloc<uint32_t>(P, err);
    d.type = c->alloc<uint32_t>(P, err);
    d.img = c->alloc<int4>(P, err);
    d.nnum = c->alloc<int>(P, err);
    d.cell = c->alloc<int>(P, err);
    d.perm = c->alloc<int>(P, err);
    d.s_pos = c->alloc<double4>(P, err);
    d.s_vel = c->alloc<double4>(P, err);
    d.s_mass = c->alloc<double>(P, err);
    d.s_cutr = c->alloc<double>(P, err);
    d.s_tag = c->alloc<uint32_t>(P, err);
    d.s_type = c->alloc<uint32_t>(P, err);
    d.s_img = c->alloc<int4>(P, err);
    d.pos2 = c->alloc<float4>(2 * P, err);
    if (c->has_mixed) {
        d.lbp2 = c->alloc<float4>(2 * P, err);
        d.posu = c->alloc<uint4>(P, err);
        d.lbpu = c->alloc<uint4>(P, err);
    }
    if (c->has_dem) {
        d.omg = c->alloc<double4>(P, err);
        d.trq = c->alloc<double4>(P, err);
        d.quat = c->alloc<double4>(P, err);
        d.s_omg = c->alloc<double4>(P, err);
        d.s_quat = c->alloc<double4>(P, err);
        d.hist_any = 1;
        for (int b = 0; b < 2; b++) {
            d.hcnt[b] = c->alloc<int>(P, err);
            d.htag[b] = c->alloc<uint32_t>(hist_entries, err);
            d.hval[b] = c->alloc<double>(hist_entries * 7, err);
        }
        d.s_hcnt = c->alloc<int>(P, err);
        d.s_htag = c->alloc<uint32_t>(hist_entries, err);
        d.s_hval = c->alloc<double>(hist_entries * 7, err);
    }
    if (c->any_virial) d.vir = c->alloc<double>(6 * P, err);
    d.blkpart = c->alloc<double>((size_t)nblocks * 8, err);
    c->d_blk_sys = c->alloc<int>(nblocks, err);
    c->d_blk_run = c->alloc<int>(nblocks, err);
    for (int q = 0; q < 2; q++) c->d_blk_run_kind[q] = c->alloc<int>(nblocks, err);
    c->d_run_sys = c->alloc<int>(nsys, err);
    d.rb_sys = c->alloc<int>(nsys + 1, err);
    d.rb_poff = c->alloc<int>(nsys + 1, err);
    d.rb_coff = c->alloc<int>(nsys + 1, err);
    d.rb_n = c->alloc<int>(1, err);
    if (c->has_mixed && c->has_dem) {
        d.dem_wl = c->alloc<int>(P, err);
        d.dem_wl_n = c->alloc<int>(nsys, err);
        d.dem_cl = c->alloc<int>(P, err);
        d.dem_cl_n = c->alloc<int>(2, err);
    }
    c->d_cblk0 = c->alloc<int>(nsys, err);
    c->d_sp = c->alloc<SysParams>(nsys, err);
    d.ss = c->alloc<SysState>(nsys, err);
    c->d_mat = c->alloc<double>(std::max<size_t>(mat_all.size(), 1), err);
    c->d_matf = c->alloc<float>(std::max<size_t>(mat_all.size(), 1), err);
    c->d_thermo = c->alloc<double>((size_t)nsys * THERMO_W, err);
    d.grid_ctr = c->alloc<unsigned int>(1, err);
    d.stat_ctr = c->alloc<unsigned long long>(4, err);
    c->d_loop = c->alloc<long long>(2, err);
    if (err) {
        delete c;
        return err;
    }
    cudaMemcpy(c->d_blk_sys, blk_sys.data(), blk_sys.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (!mat_all.empty()) {
        cudaMemcpy(c->d_mat, mat_all.data(), mat_all.size() * sizeof(double), cudaMemcpyHostToDevice);
        std::vector<float> mf(mat_all.begin(), mat_all.end());
        cudaMemcpy(c->d_matf, mf.data(), mf.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    d.matf = c->d_matf;
    d.blk_sys = c->d_blk_sys;
    d.sp = c->d_sp;
    d.mat = c->d_mat;
    for (int s = 0; s < nsys; s++) {
        // a placeholder grid until the first upload
        SysParams& p = c->sp[s];
        p.ncell = 1;
        p.ncap = 1;
    }
    int r = ensure_layout(c);
    if (r) {
        delete c;
        return r;
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        delete c;
        return cuda_err(e);
    }
    *out = c;
    return MDG_OK;
}

int mdg_configure_system(mdg_ctx* c, int sys, const mdg_config* cfg) {
    if (!c || !cfg || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    int r = validate_config(*cfg);
    if (r) return r;
    SysParams& p = c->sp[sys];
    if (cfg->kind != p.kind || cfg->precision != p.precision) return MDG_ERR_CONFIG;
    if (cfg->kind == MDG_KIND_DEM && cfg->n_materials > p.matcap) return MDG_ERR_CONFIG;
    if (cfg->kind == MDG_KIND_LJ && cfg->n_lj_types > p.matcap) return MDG_ERR_CONFIG;
    if (cfg->virial && !c->d.vir) return MDG_ERR_CONFIG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<double> tabs;
    apply_physics(c, sys, *cfg, tabs);
    if (!tabs.empty()) {
        std::vector<float> tf(tabs.begin(), tabs.end());
        cudaMemcpy(c->d_mat + p.mat0, tabs.data(), tabs.size() * sizeof(double), cudaMemcpyHostToDevice);
        cudaMemcpy(c->d_matf + p.mat0, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    // freeze the slot until its next upload
    long long zero = 0;
    cudaMemcpy(&c->d.ss[sys].remaining, &zero, sizeof(zero), cudaMemcpyHostToDevice);
    c->uploaded[sys] = 0;
    c->rem_host[sys] = 0;
    e = cudaMemcpy(c->d_sp + sys, &p, sizeof(SysParams), cudaMemcpyHostToDevice);
    return cuda_err(e);
}

int mdg_create(const mdg_config* cfg, size_t capacity, mdg_ctx** out) {
    return mdg_batch_create(cfg, &capacity, 1, out);
}

void mdg_destroy(mdg_ctx* c) { delete c; }

int mdg_num_systems(const mdg_ctx* c) { return c ? c->nsys : 0; }

// Grid, list capacity and thermostat of system `sys` for n particles whose
// list cutoff radii span [min_cut, max_cut], then the context's layout; the
// particle arrays are written next (from the host or by a generator) and
// finish_upload arms the first step.
static int prepare_system(mdg_ctx* c, int sys, size_t n, double min_cut, double max_cut) {
    const mdg_config& k = c->cfg[sys];
    SysParams& p = c->sp[sys];
    int r = setup_grid(k, min_cut, max_cut, n, p);
    if (r) return r;
    if (c->nsys > 1) p.build_mode = auto_build_mode(p, n, true);
    if (c->build_mode >= 0) p.build_mode = c->build_mode;
    p.n = (int)n;
    p.nb = (int)((n + BLK - 1) / BLK);
    c->maps_dirty = true;
    p.ncap = auto_ncap(k, p, n);
    if (k.nose_hoover) {
        // setup_nose_hoover (crates/md_thermostat/src/lib.rs:195-243)
        p.nh = 1;
        p.nh_ndof = 3.0 * (double)n - 3.0;
        p.nh_T = k.nh_temperature;
        p.nh_Q = p.nh_ndof * p.nh_T * k.nh_coupling * k.nh_coupling;
    } else {
        p.nh = 0;
    }
    return ensure_layout(c, sys);
}

// The first step of a freshly written system performs a full rebuild
// (CommState::FullRebuild); the kinetic energies of every system are
// refreshed.
static int finish_upload(mdg_ctx* c, int sys) {
    Dev& d = c->d;
    cudaStream_t s0 = c->stream;
    SysState ss{};
    ss.rebuild = 1;
    ss.remaining = -1;
    cudaMemcpyAsync(d.ss + sys, &ss, sizeof(SysState), cudaMemcpyHostToDevice, s0);
    cudaError_t e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) return cuda_err(e);
    c->launches += launch_ke_init(d, s0);
    e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e);
    c->uploaded[sys] = 1;
    c->rem_host[sys] = -1;
    return MDG_OK;
}

int mdg_upload_state(mdg_ctx* c, int sys, const mdg_state_view* st) {
    if (!c || !st || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    const mdg_config& k = c->cfg[sys];
    const size_t n = st->n;
    if (n < 1 || n > c->capacity[sys]) return MDG_ERR_ARG;
    if (!st->tag || !st->pos || !st->vel || !st->mass || !st->cutoff_radius) return MDG_ERR_ARG;
    if (k.kind == MDG_KIND_DEM && (!st->radius || !st->inv_inertia)) return MDG_ERR_ARG;
    SysParams& p = c->sp[sys];
    for (size_t i = 0; i < n; i++) {
        for (int q = 0; q < 3; q++)
            if (!std::isfinite(st->pos[3 * i + q]) || !std::isfinite(st->vel[3 * i + q])) return MDG_ERR_NAN;
        if (!(st->mass[i] > 0.0) || !(st->cutoff_radius[i] > 0.0)) return MDG_ERR_ARG;
        if (st->type && k.kind == MDG_KIND_DEM && (int)st->type[i] >= k.n_materials) return MDG_ERR_ARG;
        // multi-type LJ: the type indexes the pair table
        if (k.kind == MDG_KIND_LJ && c->ljn[sys] > 1 && (!st->type || st->type[i] >= (uint32_t)c->ljn[sys]))
            return MDG_ERR_ARG;
    }
    double min_cut = std::numeric_limits<double>::max(), max_cut = 0.0;
    for (size_t i = 0; i < n; i++) {
        max_cut = std::fmax(max_cut, st->cutoff_radius[i]);
        min_cut = std::fmin(min_cut, st->cutoff_radius[i]);
    }
    int r = prepare_system(c, sys, n, min_cut, max_cut);
    if (r) return r;
    const size_t np = (size_t)p.npad;
    std::vector<double4> pos(np), vel(np), zero4(np), frc(np), trq, omg, quat;
    std::vector<double> mass(np, 1.0), cutr(np, 0.0);
    std::vector<uint32_t> tag(np, 0xffffffffu), type(np, 0);
    std::vector<int4> img(np);
    std::vector<int> zi(np, 0);
    for (size_t i = 0; i < np; i++) {
        zero4[i] = make_double4(0, 0, 0, 0);
        img[i] = make_int4(0, 0, 0, 0);
        pos[i] = zero4[i];
        vel[i] = zero4[i];
        frc[i] = zero4[i];
    }
    const bool dem = k.kind == MDG_KIND_DEM;
    if (dem) {
        omg.assign(np, zero4[0]);
        trq.assign(np, zero4[0]);
        quat.assign(np, make_double4(1, 0, 0, 0));
    }
    for (size_t i = 0; i < n; i++) {
        pos[i] = make_double4(st->pos[3 * i], st->pos[3 * i + 1], st->pos[3 * i + 2], dem ? st->radius[i] : 0.0);
        vel[i] = make_double4(st->vel[3 * i], st->vel[3 * i + 1], st->vel[3 * i + 2], 1.0 / st->mass[i]);
        mass[i] = st->mass[i];
        cutr[i] = st->cutoff_radius[i];
        tag[i] = st->tag[i];
        type[i] = st->type ? st->type[i] : 0;
        if (st->image) img[i] = make_int4(st->image[3 * i], st->image[3 * i + 1], st->image[3 * i + 2], 0);
        if (st->force) frc[i] = make_double4(st->force[3 * i], st->force[3 * i + 1], st->force[3 * i + 2], 0.0);
        if (dem && st->torque) trq[i] = make_double4(st->torque[3 * i], st->torque[3 * i + 1], st->torque[3 * i + 2], 0.0);
        if (dem) {
            const double* w = st->omega;
            omg[i] = make_double4(w ? w[3 * i] : 0.0, w ? w[3 * i + 1] : 0.0, w ? w[3 * i + 2] : 0.0, st->inv_inertia[i]);
            if (st->quat)
                quat[i] = make_double4(st->quat[4 * i], st->quat[4 * i + 1], st->quat[4 * i + 2], st->quat[4 * i + 3]);
        }
    }
    const size_t o = (size_t)p.p0;
    Dev& d = c->d;
    cudaStream_t s0 = c->stream;
    cudaMemcpyAsync(d.pos + o, pos.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.lbp + o, pos.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.vel + o, vel.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.frc + o, frc.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.mass + o, mass.data(), np * sizeof(double), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.cutr + o, cutr.data(), np * sizeof(double), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.tag + o, tag.data(), np * sizeof(uint32_t), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.type + o, type.data(), np * sizeof(uint32_t), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.img + o, img.data(), np * sizeof(int4), cudaMemcpyHostToDevice, s0);
    cudaMemcpyAsync(d.nnum + o, zi.data(), np * sizeof(int), cudaMemcpyHostToDevice, s0);
    if (dem) {
        cudaMemcpyAsync(d.omg + o, omg.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
        cudaMemcpyAsync(d.trq + o, trq.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
        cudaMemcpyAsync(d.quat + o, quat.data(), np * sizeof(double4), cudaMemcpyHostToDevice, s0);
        for (int b = 0; b < 2; b++) cudaMemcpyAsync(d.hcnt[b] + o, zi.data(), np * sizeof(int), cudaMemcpyHostToDevice, s0);
    }
    return finish_upload(c, sys);
}

int mdg_generate_fcc(mdg_ctx* c, int sys, const mdg_fcc_spec* f, size_t* n_out) {
    if (!c || !f || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (n_out) *n_out = 0;
    const mdg_config& k = c->cfg[sys];
    if (k.kind != MDG_KIND_LJ) return MDG_ERR_CONFIG;
    // fcc_insert's checks (md_lattice/src/lib.rs:257-269, 395-405)
    if (!(f->density > 0.0) || !std::isfinite(f->density) || !(f->temperature >= 0.0) ||
        !std::isfinite(f->temperature) || !(f->mass > 0.0) || !(f->skin > 0.0) || f->n_types < 0 ||
        f->n_types > MDG_GEN_MAX_TYPES)
        return MDG_ERR_CONFIG;
    FccArgs a{};
    const double a_ideal = std::cbrt(4.0 / f->density);
    long long n = 4;
    for (int d = 0; d < 3; d++) {
        const double L = k.box_hi[d] - k.box_lo[d];
        const double cells = std::floor(L / a_ideal);
        if (!(cells >= 1.0) || cells > 4096.0) return MDG_ERR_CONFIG;
        a.nc[d] = (int)cells;
        a.a[d] = L / cells;
        a.lo[d] = k.box_lo[d];
        n *= a.nc[d];
    }
    if ((size_t)n > c->capacity[sys]) return MDG_ERR_ARG;
    a.temperature = f->temperature;
    a.skin = f->skin;
    a.seed = f->seed;
    a.ntypes = f->n_types > 1 ? f->n_types : 1;
    for (int t = 0; t < a.ntypes; t++) {
        a.frac[t] = f->n_types > 1 ? f->type_fractions[t] : 1.0;
        a.tmass[t] = f->type_masses[t] > 0.0 && f->n_types > 1 ? f->type_masses[t] : f->mass;
    }
    // multi-type LJ: the type indexes the pair table
    if (c->ljn[sys] > 1 ? a.ntypes > c->ljn[sys] : a.ntypes > 1) return MDG_ERR_ARG;
    int r = prepare_system(c, sys, (size_t)n, f->skin, f->skin);
    if (r) return r;
    r = gen_fcc(c->d, c->sp[sys], a, c->stream, &c->launches);
    if (r) return r;
    if (n_out) *n_out = (size_t)n;
    return finish_upload(c, sys);
}

int mdg_generate_gas(mdg_ctx* c, int sys, const mdg_gas_spec* g, size_t* placed) {
    if (!c || !g || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (placed) *placed = 0;
    const mdg_config& k = c->cfg[sys];
    if (k.kind != MDG_KIND_DEM) return MDG_ERR_CONFIG;
    if (g->n < 1 || g->n > c->capacity[sys]) return MDG_ERR_ARG;
    if (!(g->rmin > 0.0) || !(g->rmax >= g->rmin) || !std::isfinite(g->rmax) || !(g->sep_factor > 0.0) ||
        !(g->density > 0.0) || !(g->speed >= 0.0) || !std::isfinite(g->speed) ||
        g->velocity_mode < MDG_VEL_SPEED || g->velocity_mode > MDG_VEL_GAUSSIAN ||
        (int)g->material >= k.n_materials)
        return MDG_ERR_ARG;
    GasArgs a{};
    a.n = (long long)g->n;
    a.rmin = g->rmin;
    a.rmax = g->rmax;
    a.density = g->density;
    a.sep = g->sep_factor;
    a.inset = g->inset ? 1 : 0;
    a.vel_mode = g->velocity_mode;
    a.speed = g->speed;
    a.material = g->material;
    a.seed = g->seed;
    a.max_proposals = g->max_proposals;
    GasPlacement gp;
    int r = gen_gas_place(a, k.box_lo, k.box_hi, c->stream, &gp, &c->launches);
    if (placed) *placed = gp.count;
    if (r) {
        gp.release(c->stream);
        cudaStreamSynchronize(c->stream);
        return r;
    }
    r = prepare_system(c, sys, g->n, gp.rmin, gp.rmax);
    if (!r) r = gen_gas_write(c->d, c->sp[sys], a, gp, c->stream, &c->launches);
    gp.release(c->stream);
    if (r) return r;
    return finish_upload(c, sys);
}

int mdg_download_state(mdg_ctx* c, int sys, mdg_state_view* st) {
    if (!c || !st || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const SysParams& p = c->sp[sys];
    const size_t n = (size_t)p.n;
    if (st->n < n) return MDG_ERR_ARG;
    st->n = n;
    const size_t o = (size_t)p.p0;
    Dev& d = c->d;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<double4> pos(n), vel(n), frc(n);
    std::vector<double> mass(n), cutr(n);
    std::vector<uint32_t> tag(n), type(n);
    std::vector<int4> img(n);
    cudaMemcpy(pos.data(), d.pos + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
    cudaMemcpy(vel.data(), d.vel + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
    cudaMemcpy(frc.data(), d.frc + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
    cudaMemcpy(mass.data(), d.mass + o, n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(cutr.data(), d.cutr + o, n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaMemcpy(tag.data(), d.tag + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(type.data(), d.type + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(img.data(), d.img + o, n * sizeof(int4), cudaMemcpyDeviceToHost);
    const bool dem = p.kind == MDG_KIND_DEM;
    std::vector<double4> omg, trq, quat;
    if (dem) {
        omg.resize(n);
        trq.resize(n);
        quat.resize(n);
        cudaMemcpy(omg.data(), d.omg + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
        cudaMemcpy(trq.data(), d.trq + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
        cudaMemcpy(quat.data(), d.quat + o, n * sizeof(double4), cudaMemcpyDeviceToHost);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e);
    for (size_t i = 0; i < n; i++) {
        if (st->tag) st->tag[i] = tag[i];
        if (st->type) st->type[i] = type[i];
        if (st->pos) { st->pos[3 * i] = pos[i].x; st->pos[3 * i + 1] = pos[i].y; st->pos[3 * i + 2] = pos[i].z; }
        if (st->vel) { st->vel[3 * i] = vel[i].x; st->vel[3 * i + 1] = vel[i].y; st->vel[3 * i + 2] = vel[i].z; }
        if (st->force) { st->force[3 * i] = frc[i].x; st->force[3 * i + 1] = frc[i].y; st->force[3 * i + 2] = frc[i].z; }
        if (st->mass) st->mass[i] = mass[i];
        if (st->cutoff_radius) st->cutoff_radius[i] = cutr[i];
        if (st->image) { st->image[3 * i] = img[i].x; st->image[3 * i + 1] = img[i].y; st->image[3 * i + 2] = img[i].z; }
        if (dem) {
            if (st->radius) st->radius[i] = pos[i].w;
            if (st->inv_inertia) st->inv_inertia[i] = omg[i].w;
            if (st->omega) { st->omega[3 * i] = omg[i].x; st->omega[3 * i + 1] = omg[i].y; st->omega[3 * i + 2] = omg[i].z; }
            if (st->torque) { st->torque[3 * i] = trq[i].x; st->torque[3 * i + 1] = trq[i].y; st->torque[3 * i + 2] = trq[i].z; }
            if (st->quat) {
                st->quat[4 * i] = quat[i].x; st->quat[4 * i + 1] = quat[i].y;
                st->quat[4 * i + 2] = quat[i].z; st->quat[4 * i + 3] = quat[i].w;
            }
        }
    }
    return MDG_OK;
}

int mdg_set_history(mdg_ctx* c, int sys, size_t nent, const uint32_t* keys, const double* vals) {
    if (!c || sys < 0 || sys >= c->nsys || (nent && (!keys || !vals))) return MDG_ERR_ARG;
    const SysParams& p = c->sp[sys];
    if (p.kind != MDG_KIND_DEM) return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const size_t n = (size_t)p.n, np = (size_t)p.npad, o = (size_t)p.p0;
    Dev& d = c->d;
    cudaStreamSynchronize(c->stream);
    std::vector<uint32_t> tag(n);
    cudaMemcpy(tag.data(), d.tag + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    std::map<uint32_t, size_t> idx;
    for (size_t i = 0; i < n; i++) idx[tag[i]] = i;
    std::vector<int> cnt(np, 0);
    std::vector<uint32_t> ht((size_t)p.hcap * np, 0);
    std::vector<double> hv((size_t)p.hcap * 7 * np, 0.0);
    for (size_t k = 0; k < nent; k++) {
        auto it = idx.find(keys[2 * k]);
        if (it == idx.end()) return MDG_ERR_ARG;
        const size_t i = it->second;
        const int cc = cnt[i];
        if (cc >= p.hcap) return MDG_ERR_LIST_OVERFLOW;
        ht[(size_t)cc * np + i] = keys[2 * k + 1];
        for (int q = 0; q < 7; q++) hv[(size_t)(cc * 7 + q) * np + i] = vals[7 * k + q];
        cnt[i] = cc + 1;
    }
    const int h = sys_hcur(c, sys);
    cudaMemcpy(d.hcnt[h] + o, cnt.data(), np * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d.htag[h] + p.h0, ht.data(), ht.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    cudaMemcpy(d.hval[h] + p.h0 * 7, hv.data(), hv.size() * sizeof(double), cudaMemcpyHostToDevice);
    return cuda_err(cudaGetLastError());
}

int mdg_get_history(mdg_ctx* c, int sys, uint32_t* keys, double* vals, size_t cap, size_t* nout) {
    if (!c || sys < 0 || sys >= c->nsys || !nout) return MDG_ERR_ARG;
    const SysParams& p = c->sp[sys];
    *nout = 0;
    if (p.kind != MDG_KIND_DEM) return MDG_OK;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const size_t n = (size_t)p.n, np = (size_t)p.npad, o = (size_t)p.p0;
    Dev& d = c->d;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<uint32_t> tag(n);
    std::vector<int> cnt(n);
    std::vector<uint32_t> ht((size_t)p.hcap * np);
    std::vector<double> hv((size_t)p.hcap * 7 * np);
    const int h = sys_hcur(c, sys);
    cudaMemcpy(tag.data(), d.tag + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(cnt.data(), d.hcnt[h] + o, n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(ht.data(), d.htag[h] + p.h0, ht.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(hv.data(), d.hval[h] + p.h0 * 7, hv.size() * sizeof(double), cudaMemcpyDeviceToHost);
    size_t m = 0;
    for (size_t i = 0; i < n; i++)
        for (int cc = 0; cc < cnt[i]; cc++) {
            if (m < cap && keys && vals) {
                keys[2 * m] = tag[i];
                keys[2 * m + 1] = ht[(size_t)cc * np + i];
                for (int q = 0; q < 7; q++) vals[7 * m + q] = hv[(size_t)(cc * 7 + q) * np + i];
            }
            m++;
        }
    *nout = m;
    return cuda_err(cudaGetLastError());
}

// Systems never uploaded (or reconfigured and not yet uploaded) hold a step
// budget of zero -- set at creation and by mdg_configure_system, and
// mdg_set_remaining refuses to lift it -- so every kernel skips them and a
// batch may run with free slots.
static bool any_uploaded(const mdg_ctx* c) {
    for (int s = 0; s < c->nsys; s++)
        if (c->uploaded[s]) return true;
    return false;
}

int mdg_step_async(mdg_ctx* c, int64_t nsteps) {
    if (!c || nsteps < 0) return MDG_ERR_ARG;
    if (!any_uploaded(c)) return MDG_ERR_STATE;
    if (c->pending_steps) return MDG_ERR_STATE;  // the previous launch was not waited for
    if (nsteps == 0) return MDG_OK;
    const int nrun = update_run_maps(c);
    if (nrun < 0) return -nrun;
    if (nrun == 0) return MDG_OK;  // every system's budget is spent
    cudaMemcpyAsync(c->h_stat, c->d.stat_ctr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
    if (c->graph_mode) {
        // one launch: the WHILE graph counts the steps down on the device
        if (!c->wgraph) {
            int r = build_while_graph(c);
            if (r) return r;
        }
        long long n = nsteps;
        const long long nn[2] = {n, n};
        cudaMemcpyAsync(c->d_loop, nn, sizeof(nn), cudaMemcpyHostToDevice, c->stream);
        cudaError_t e = cudaGraphLaunch(c->wgraph, c->stream);
        if (e != cudaSuccess) return cuda_err(e);
    } else {
        for (int64_t k = 0; k < nsteps; k++) enqueue_step(c, c->stream);
    }
    cudaMemcpyAsync(c->h_stat + 1, c->d.stat_ctr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
    c->pending_steps = nsteps;
    return cuda_err(cudaGetLastError());
}

int mdg_step_wait(mdg_ctx* c) {
    if (!c) return MDG_ERR_ARG;
    const int64_t nsteps = c->pending_steps;
    if (!nsteps) return MDG_OK;  // nothing in flight
    c->pending_steps = 0;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e);
    const unsigned long long rb0 = c->h_stat[0], rb1 = c->h_stat[1];
    advance_budgets(c, nsteps);
    // kernels that ran: per step initial + force + final (+ loop control),
    // plus the rebuild kernels on the steps whose rebuild branch opened
    // (the mixed DEM force is two kernels: screen and contact; each kind's
    // force kernels launch only while some system of that kind runs)
    const long long nforce = (c->d.nrun_kind[1] ? 1 : 0) + (c->d.nrun_kind[0] ? (c->has_mixed ? 2 : 1) : 0) +
                             (c->has_walls ? 1 : 0);
    long long base = 2 + nforce + (c->graph_mode ? 1 : 0);
    if (c->graph_mode && c->has_mixed) {
        // fused step kernel (+ thermostatted initial) per iteration, the
        // epilogue final once per launch
        base = 1 + (c->run_nh ? 1 : 0) + nforce + 1;
        c->launches += 1;
    }
    c->launches += nsteps * base + (long long)rb_kernels(c) * (long long)(c->graph_mode ? (rb1 - rb0) : nsteps);
    return check_status(c);
}

int mdg_step(mdg_ctx* c, int64_t nsteps) {
    const int r = mdg_step_async(c, nsteps);
    if (r) return r;
    return mdg_step_wait(c);
}

int mdg_force_only(mdg_ctx* c) {
    if (!c) return MDG_ERR_ARG;
    if (!any_uploaded(c)) return MDG_ERR_STATE;
    const int nrun = update_run_maps(c);
    if (nrun < 0) return -nrun;
    if (nrun == 0) return MDG_OK;
    std::vector<SysState> ss(c->nsys);
    cudaMemcpy(ss.data(), c->d.ss, c->nsys * sizeof(SysState), cudaMemcpyDeviceToHost);
    for (auto& x : ss) x.rebuild = 1;
    cudaMemcpy(c->d.ss, ss.data(), c->nsys * sizeof(SysState), cudaMemcpyHostToDevice);
    cudaStream_t st = c->stream;
    c->launches += launch_rb(c, c->d, st);
    c->launches += launch_force(c, c->d, st, 0);
    c->launches += launch_fin(c, c->d, st, 0);  // reductions + bookkeeping, no integration
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_err(e);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e);
    return check_status(c);
}

int mdg_get_status(mdg_ctx* c, int sys, int32_t* status) {
    if (!c || sys < 0 || sys >= c->nsys || !status) return MDG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    int v = 0;
    e = cudaMemcpy(&v, &c->d.ss[sys].status, sizeof(int), cudaMemcpyDeviceToHost);
    *status = v;
    return cuda_err(e);
}

int mdg_set_remaining(mdg_ctx* c, int sys, int64_t steps) {
    if (!c || sys < 0 || sys >= c->nsys || steps < -1) return MDG_ERR_ARG;
    if (steps != 0 && !c->uploaded[sys]) return MDG_ERR_STATE;  // nothing to run
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    long long v = steps;
    e = cudaMemcpy(&c->d.ss[sys].remaining, &v, sizeof(v), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) c->rem_host[sys] = steps;
    return cuda_err(e);
}

int mdg_get_config(mdg_ctx* c, int sys, mdg_config* out) {
    if (!c || !out || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    *out = c->cfg[sys];
    return MDG_OK;
}

int mdg_set_threads_per_particle(mdg_ctx* c, int tpp) {
    if (!c || !(tpp == 1 || tpp == 2 || tpp == 4 || tpp == 8)) return MDG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    if (c->tpp_lj != tpp) c->drop_graphs();
    c->tpp_lj = tpp;
    return MDG_OK;
}

int mdg_get_threads_per_particle(const mdg_ctx* c) { return c ? c->tpp_lj : 0; }

int mdg_set_build_mode(mdg_ctx* c, int mode) {
    if (!c || mode < -1 || mode > 2) return MDG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    c->build_mode = mode;
    // systems uploaded so far take the mode now; -1 restores the automatic choice
    for (int s = 0; s < c->nsys; s++) {
        if (!c->uploaded[s]) continue;
        SysParams& p = c->sp[s];
        p.build_mode = mode >= 0 ? mode : auto_build_mode(p, (size_t)p.n, c->nsys > 1);
        e = cudaMemcpy(c->d_sp + s, &p, sizeof(SysParams), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_err(e);
    }
    return MDG_OK;
}

int mdg_rdf(mdg_ctx* c, int sys, double r_max, int nbins, uint64_t* counts) {
    if (!c || !counts || sys < 0 || sys >= c->nsys || nbins < 1 || nbins > rdf_max_bins() || !(r_max > 0.0))
        return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const SysParams& p = c->sp[sys];
    int err = 0;
    if (c->rdf_posf_n < p.n) {
        c->free_ptr(c->rdf_posf);
        c->rdf_posf = c->alloc<float4>(p.n, err);
        if (err) return err;
        c->rdf_posf_n = p.n;
    }
    if (c->rdf_counts_n < nbins) {
        c->free_ptr(c->rdf_counts);
        c->rdf_counts = c->alloc<unsigned long long>(nbins, err);
        if (err) return err;
        c->rdf_counts_n = nbins;
    }
    cudaMemsetAsync(c->rdf_counts, 0, nbins * sizeof(unsigned long long), c->stream);
    c->launches += launch_rdf(c->d, sys, p, c->rdf_posf, r_max, nbins, c->rdf_counts, c->stream);
    cudaError_t e = cudaMemcpyAsync(counts, c->rdf_counts, nbins * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_err(e == cudaSuccess ? cudaGetLastError() : e);
}

int mdg_msd_reset(mdg_ctx* c, int sys) {
    if (!c || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const SysParams& p = c->sp[sys];
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<uint32_t> tag(p.n);
    e = cudaMemcpy(tag.data(), c->d.tag + p.p0, p.n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e);
    long long ntag = 0;
    for (uint32_t t : tag) ntag = std::max(ntag, (long long)t + 1);
    if (c->msd_ref.empty()) {
        c->msd_ref.assign(c->nsys, nullptr);
        c->msd_ntag.assign(c->nsys, 0);
    }
    int err = 0;
    if (c->msd_ntag[sys] < ntag) {
        c->free_ptr(c->msd_ref[sys]);
        c->msd_ref[sys] = c->alloc<double>(3 * ntag, err);
        if (err) return err;
        c->msd_ntag[sys] = ntag;
    }
    c->launches += launch_msd_ref(c->d, sys, p.n, c->msd_ref[sys], c->stream);
    return cuda_err(cudaStreamSynchronize(c->stream));
}

int mdg_msd(mdg_ctx* c, int sys, double* msd) {
    if (!c || !msd || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (!c->uploaded[sys] || c->msd_ref.empty() || !c->msd_ref[sys]) return MDG_ERR_STATE;
    const SysParams& p = c->sp[sys];
    const long long nb = (p.n + BLK - 1) / BLK;
    int err = 0;
    if (c->msd_part_n < nb) {
        c->free_ptr(c->msd_part);
        c->msd_part = c->alloc<double>(nb, err);
        if (err) return err;
        c->msd_part_n = nb;
    }
    c->launches += launch_msd(c->d, sys, p.n, c->msd_ref[sys], c->msd_part, c->stream);
    std::vector<double> part(nb);
    cudaError_t e = cudaMemcpyAsync(part.data(), c->msd_part, nb * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    double sum = 0.0;
    for (double x : part) sum += x;
    *msd = sum / (double)p.n;
    return cuda_err(cudaGetLastError());
}

int mdg_get_stream(mdg_ctx* c, void** stream) {
    if (!c || !stream) return MDG_ERR_ARG;
    *stream = (void*)c->stream;
    return MDG_OK;
}

int mdg_set_stream_priority(mdg_ctx* c, int priority) {
    if (!c) return MDG_ERR_ARG;
    if (c->pending_steps) return MDG_ERR_STATE;  // a launch is in flight on the old stream
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return cuda_err(e);
    const int p = std::min(least, std::max(greatest, priority));
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    cudaStream_t s = nullptr;
    e = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, p);
    if (e != cudaSuccess) return cuda_err(e);
    cudaStreamDestroy(c->stream);
    c->stream = s;
    return MDG_OK;
}

int mdg_get_progress(mdg_ctx* c, int64_t* remaining, int32_t* status, int64_t* steps) {
    if (!c) return MDG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<SysState> ss(c->nsys);
    e = cudaMemcpy(ss.data(), c->d.ss, c->nsys * sizeof(SysState), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e);
    for (int s = 0; s < c->nsys; s++) {
        if (remaining) remaining[s] = ss[s].remaining;
        if (status) status[s] = ss[s].status;
        if (steps) steps[s] = ss[s].step;
    }
    return MDG_OK;
}

int mdg_get_remaining(mdg_ctx* c, int sys, int64_t* steps) {
    if (!c || sys < 0 || sys >= c->nsys || !steps) return MDG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    long long v = 0;
    e = cudaMemcpy(&v, &c->d.ss[sys].remaining, sizeof(v), cudaMemcpyDeviceToHost);
    *steps = v;
    return cuda_err(e);
}

int mdg_get_pairs(mdg_ctx* c, int sys, uint32_t* pairs, size_t cap, size_t* nout) {
    if (!c || sys < 0 || sys >= c->nsys || !nout) return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    const SysParams& p = c->sp[sys];
    const size_t n = (size_t)p.n, np = (size_t)p.npad, o = (size_t)p.p0;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    std::vector<int> nn(n);
    std::vector<uint32_t> tag(n), lst((size_t)p.ncap * np);
    cudaMemcpy(nn.data(), c->d.nnum + o, n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(tag.data(), c->d.tag + o, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(lst.data(), c->d.nlist + p.lst0, lst.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    size_t m = 0;
    for (size_t i = 0; i < n; i++)
        for (int k = 0; k < nn[i]; k++) {
            const uint32_t e2 = lst[(size_t)k * np + i];
            if ((e2 >> IDX_BITS) < 27u) continue;
            if (pairs && m < cap) {
                pairs[2 * m] = tag[i];
                pairs[2 * m + 1] = tag[e2 & IDX_MASK];
            }
            m++;
        }
    *nout = m;
    return cuda_err(cudaGetLastError());
}

int mdg_thermo(mdg_ctx* c, int sys, mdg_thermo_t* out) {
    if (!c || !out || sys < 0 || sys >= c->nsys) return MDG_ERR_ARG;
    if (!c->uploaded[sys]) return MDG_ERR_STATE;
    c->launches += launch_thermo(c->d, c->d_thermo, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(e);
    double t[THERMO_W];
    SysState ss;
    cudaMemcpy(t, c->d_thermo + (size_t)sys * THERMO_W, sizeof(t), cudaMemcpyDeviceToHost);
    cudaMemcpy(&ss, c->d.ss + sys, sizeof(SysState), cudaMemcpyDeviceToHost);
    const SysParams& p = c->sp[sys];
    const double ndof = 3.0 * (double)p.n - 3.0;
    out->ke = t[0];
    out->pe = t[1];
    out->temp = ndof > 0 ? 2.0 * t[0] / ndof : 0.0;
    out->p_xi = ss.p_xi_post;
    out->granular_temp = t[4];
    out->momentum = t[5];
    // mixed systems: the virial of the last force evaluation, summed here
    for (int k = 0; k < 6; k++) out->virial[k] = (p.precision == MDG_MIXED && p.virial) ? t[16 + k] : ss.vir[k];
    out->step = ss.step;
    out->nbuilds = ss.nbuilds;
    out->n = p.n;
    out->status = ss.status;
    out->max_neighbors = ss.max_nbr;
    out->rot_temp = t[6];
    out->e_tail = out->p_tail = 0.0;
    if (p.kind == MDG_KIND_LJ) {
        // setup_lj_tails (md_lj/src/lib.rs:397-445): rho = N / V, V = the
        // product of the box sides; per type pair rc = sqrt((cutoff sigma)^2),
        // weighted by (1 / ntypes)^2 (an equimolar mixture), in table order
        const int nt = c->ljn[sys];
        const double n = (double)p.n;
        const double rho = n / (p.L[0] * p.L[1] * p.L[2]);
        const double frac = 1.0 / (double)nt;
        const double w = frac * frac;
        const double pi = 3.141592653589793;
        double e_tail = 0.0, p_tail = 0.0;
        for (int a = 0; a < nt; a++)
            for (int b = 0; b < nt; b++) {
                const mdg_lj_pair& q = c->ljp[sys][(size_t)a * nt + b];
                const double cs = q.cutoff * q.sigma;
                const double rc = std::sqrt(cs * cs);
                const double sigma3 = (q.sigma * q.sigma) * q.sigma;
                const double rc3 = (rc * rc) * rc, rc9 = (rc3 * rc3) * rc3;
                const double sigma9 = (sigma3 * sigma3) * sigma3;
                e_tail += w * (8.0 / 3.0) * pi * n * rho * q.epsilon * sigma3 * (sigma9 / (3.0 * rc9) - sigma3 / rc3);
                p_tail += w * (16.0 / 3.0) * pi * rho * rho * q.epsilon * sigma3 *
                          (2.0 * sigma9 / (3.0 * rc9) - sigma3 / rc3);
            }
        out->e_tail = e_tail;
        out->p_tail = p_tail;
    }
    {
        // compute_pressure (md_measure/src/lib.rs:605-652): rho T - tr(W) / (3V) + P_tail
        const double v = p.L[0] * p.L[1] * p.L[2];
        const double trace = out->virial[0] + out->virial[1] + out->virial[2];
        out->pressure = (double)p.n / v * out->temp - trace / (3.0 * v) + out->p_tail;
    }
    return cuda_err(cudaGetLastError());
}

int mdg_synchronize(mdg_ctx* c) {
    if (!c) return MDG_ERR_ARG;
    return cuda_err(cudaStreamSynchronize(c->stream));
}

int64_t mdg_kernel_launches(const mdg_ctx* c) { return c ? c->launches : 0; }

int mdg_timed_steps(mdg_ctx* c, int64_t nsteps, size_t l2_flush_bytes, mdg_step_timing* out) {
    if (!c || nsteps < 0 || (nsteps && !out)) return MDG_ERR_ARG;
    if (!any_uploaded(c)) return MDG_ERR_STATE;
    const int nrun = update_run_maps(c);
    if (nrun < 0) return -nrun;
    if (nrun == 0) {  // every system's budget is spent: nothing runs
        for (int64_t k = 0; k < nsteps; k++) out[k] = mdg_step_timing{};
        return MDG_OK;
    }
    if (l2_flush_bytes > c->flush_bytes) {
        if (c->flush_buf) cudaFree(c->flush_buf);
        c->flush_buf = nullptr;
        c->flush_bytes = 0;
        if (cudaMalloc(&c->flush_buf, l2_flush_bytes) != cudaSuccess) {
            cudaGetLastError();
            return MDG_ERR_OOM;
        }
        c->flush_bytes = l2_flush_bytes;
    }
    std::vector<SysState> ss(c->nsys);
    for (auto& ev : c->tev)
        if (!ev && cudaEventCreate(&ev) != cudaSuccess) return MDG_ERR_CUDA;
    for (int64_t k = 0; k < nsteps; k++) {
        if (c->graph_mode && !c->tgraph) {
            int r = build_timed_graph(c);
            if (r) return r;
        }
        if (l2_flush_bytes) cudaMemsetAsync(c->flush_buf, (int)(k & 0xff), l2_flush_bytes, c->stream);
        cudaError_t e = cudaSuccess;
        if (c->graph_mode) {
            e = cudaGraphLaunch(c->tgraph, c->stream);
        } else {
            // eager launches (profilers see every kernel); rebuild kernels always run
            cudaStream_t st = c->stream;
            int n = 0;
            cudaEventRecord(c->tev[0], st);
            n += c->has_mixed ? launch_initial_mixed(c->d, st) : launch_initial(c->d, st);
            cudaEventRecord(c->tev[1], st);
            n += launch_rb(c, c->d, st);
            cudaEventRecord(c->tev[2], st);
            n += launch_force(c, c->d, st);
            cudaEventRecord(c->tev[3], st);
            n += launch_fin(c, c->d, st, 1);
            cudaEventRecord(c->tev[4], st);
            c->tkernels = n;
        }
        if (e != cudaSuccess) return cuda_err(e);
        e = cudaEventSynchronize(c->tev[4]);
        if (e != cudaSuccess) return cuda_err(e);
        float ms[5];
        cudaEventElapsedTime(&ms[0], c->tev[0], c->tev[4]);
        for (int q = 0; q < 4; q++) cudaEventElapsedTime(&ms[1 + q], c->tev[q], c->tev[q + 1]);
        out[k].step_ms = ms[0];
        for (int q = 0; q < 4; q++) out[k].phase_ms[q] = ms[1 + q];
        cudaMemcpy(ss.data(), c->d.ss, c->nsys * sizeof(SysState), cudaMemcpyDeviceToHost);
        int rb = 0;
        for (int s : c->run_sys) rb |= (ss[s].steps_since_build == 0);
        out[k].rebuilt = rb;
        // the rebuild-pipeline kernels run only when the conditional opened
        out[k].kernels = c->tkernels - ((rb || !c->graph_mode) ? 0 : rb_kernels(c));
        c->launches += out[k].kernels;
    }
    advance_budgets(c, nsteps);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e);
    return check_status(c);
}

int mdg_set_graph_mode(mdg_ctx* c, int enabled) {
    if (!c) return MDG_ERR_ARG;
    c->graph_mode = enabled ? 1 : 0;
    return MDG_OK;
}

}  // extern "C"
