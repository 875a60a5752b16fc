// mdg_oracle.cpp -- CPU FP64 restatement of MDDEM's single-rank particle hot path.
//
// TEST INFRASTRUCTURE ONLY (the checker for the CUDA path, and the timed CPU
// baseline); never linked into the product library.
//
// Every function below restates the reference's algorithm in the reference's
// loop order and operation order (crate paths are relative to the reference
// repository).  Floating-point rules: compiled with -ffp-contract=off, plain
// IEEE operations everywhere, std::fma exactly where the Rust source uses
// f64::mul_add.  Documented deviations from the reference:
//   * sort_atoms_by_bin uses a stable sort by bin (the reference uses
//     sort_unstable_by_key, crates/mddem_core/src/neighbor.rs:740, whose
//     within-bin order is unspecified);
//   * inputs come from a seeded generator instead of rand::rng();
//   * an LJ potential-energy sum is added (the reference computes none).
// Scope: one rank, fully periodic box, single LJ type, DEM with any number
// of materials.

#include "mdg_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

namespace {

using V3 = std::array<double, 3>;
using Q4 = std::array<double, 4>;
using I3 = std::array<int, 3>;

constexpr double kPi = 3.14159265358979323846;
// crates/dem_atom/src/lib.rs:63
constexpr double SQRT_5_3 = 0.9128709291752768;
// crates/dem_granular/src/lib.rs:93,101,108
constexpr double TANGENTIAL_EPSILON = 1e-30;
constexpr double LARGE_OVERLAP_WARN_THRESHOLD = 0.90;
constexpr long MAX_OVERLAP_WARNINGS = 500;

struct Contact {
    uint32_t tag;
    double s[7];
    bool active;
};

enum CommState { FullRebuild = 0, CommunicateOnly = 1 };

struct Swap {
    std::vector<int> send;
    int recv_start = 0, recv_count = 0;
    V3 off{0, 0, 0};
};

// MaterialTable pair tables, crates/dem_atom/src/lib.rs:389-515
struct MatTables {
    int n = 0;
    std::vector<double> E, nu;
    std::vector<double> beta, friction, rolling_friction, cohesion, surface, e_eff, g_eff,
        twisting_friction, kn, kt, k_roll, g_roll, k_twist, g_twist;
    double at(const std::vector<double>& t, int i, int j) const { return t[(size_t)i * n + j]; }
};

MatTables build_pair_tables(const orc_material* m, int n) {
    MatTables t;
    t.n = n;
    auto sz = (size_t)n * n;
    for (auto* v : {&t.beta, &t.friction, &t.rolling_friction, &t.cohesion, &t.surface, &t.e_eff,
                    &t.g_eff, &t.twisting_friction, &t.kn, &t.kt, &t.k_roll, &t.g_roll, &t.k_twist,
                    &t.g_twist})
        v->assign(sz, 0.0);
    for (int i = 0; i < n; i++) {
        t.E.push_back(m[i].youngs_mod);
        t.nu.push_back(m[i].poisson_ratio);
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            size_t k = (size_t)i * n + j;
            double e_ij = std::sqrt(m[i].restitution * m[j].restitution);
            double log_e = std::log(e_ij);
            t.beta[k] = -log_e / std::sqrt(kPi * kPi + log_e * log_e);
            t.friction[k] = std::sqrt(m[i].friction * m[j].friction);
            t.rolling_friction[k] = std::sqrt(m[i].rolling_friction * m[j].rolling_friction);
            t.cohesion[k] = std::sqrt(m[i].cohesion_energy * m[j].cohesion_energy);
            t.surface[k] = std::sqrt(m[i].surface_energy * m[j].surface_energy);
            t.twisting_friction[k] = std::sqrt(std::fmax(m[i].twisting_friction, 0.0) *
                                               std::fmax(m[j].twisting_friction, 0.0));
            double nu_i = m[i].poisson_ratio, nu_j = m[j].poisson_ratio;
            t.e_eff[k] = 1.0 / ((1.0 - nu_i * nu_i) / m[i].youngs_mod +
                                (1.0 - nu_j * nu_j) / m[j].youngs_mod);
            t.g_eff[k] = 1.0 / (2.0 * (2.0 - nu_i) * (1.0 + nu_i) / m[i].youngs_mod +
                                2.0 * (2.0 - nu_j) * (1.0 + nu_j) / m[j].youngs_mod);
            double ki = m[i].kn, kj = m[j].kn;
            t.kn[k] = (ki > 0.0 && kj > 0.0) ? 2.0 * ki * kj / (ki + kj) : 0.0;
            double kti = m[i].kt, ktj = m[j].kt;
            t.kt[k] = (kti > 0.0 && ktj > 0.0) ? 2.0 * kti * ktj / (kti + ktj) : 0.0;
            double kri = m[i].rolling_stiffness, krj = m[j].rolling_stiffness;
            t.k_roll[k] = (kri > 0.0 && krj > 0.0) ? 2.0 * kri * krj / (kri + krj)
                          : (kri > 0.0 ? kri : krj);
            t.g_roll[k] = std::sqrt(std::fmax(m[i].rolling_damping, 0.0) *
                                    std::fmax(m[j].rolling_damping, 0.0));
            double kwi = m[i].twisting_stiffness, kwj = m[j].twisting_stiffness;
            t.k_twist[k] = (kwi > 0.0 && kwj > 0.0) ? 2.0 * kwi * kwj / (kwi + kwj)
                           : (kwi > 0.0 ? kwi : kwj);
            t.g_twist[k] = std::sqrt(std::fmax(m[i].twisting_damping, 0.0) *
                                     std::fmax(m[j].twisting_damping, 0.0));
        }
    return t;
}

inline double signum(double x) { return std::copysign(1.0, x); }

struct Sim {
    orc_config cfg{};
    std::vector<orc_material> mats;
    MatTables mt;
    bool dem = true;
    double lo[3], hi[3], size[3];
    double dt = 0;

    // Atom SoA (locals then ghosts), crates/mddem_core/src/atom.rs:310-335
    std::vector<uint32_t> tag, type;
    std::vector<int> origin_index;
    std::vector<char> is_ghost;
    std::vector<V3> pos, vel, force;
    std::vector<double> mass, inv_mass, cutoff_radius;
    std::vector<I3> image;
    // DemAtom, crates/dem_atom/src/lib.rs:530-557
    std::vector<double> radius, density, inv_inertia, body_id;
    std::vector<Q4> quat;
    std::vector<V3> omega, ang_mom, torque;
    // ContactHistoryStore, crates/dem_granular/src/tangential.rs:54-75
    std::vector<std::vector<Contact>> contacts;
    // Checker only (no counterpart in the reference): per atom the sums of the
    // pair force magnitudes |f_pair| and pair torque magnitudes |tau_pair| of
    // the last force evaluation, folded onto owners like the reverse
    // communication; the normaliser of the per-particle force-error metric
    // max(|F|, sum_pairs |f_pair|).
    std::vector<double> fscale, tscale;
    int nlocal = 0, nghost = 0;

    std::vector<Swap> swaps;
    CommState state = FullRebuild;

    // Neighbor, crates/mddem_core/src/neighbor.rs:87-159
    double skin_fraction = 1, bin_min_size = 1;
    int every = 0, check = 1, sort_every = 1000, newton = 1;
    std::vector<uint32_t> nb_off, nb_idx;
    double bin_size[3]{}, bin_origin[3]{};
    int bin_count[3]{};
    int total_cells = 0;
    std::vector<int> stencil, stencil_fwd;
    bool stencil_self = false;
    std::vector<V3> last_build_pos;
    long steps_since_build = 0, sort_counter = 0;
    double ghost_cutoff = 0, cached_min_skin = 0, cached_max_cutoff = 0;
    bool uniform = false;
    double uniform_cutoff_sq = 0;

    // LJ, crates/md_lj/src/lib.rs:230-239: the pair table (1 x 1 for one type)
    struct LJC {
        double lj1, lj2, cut2, lj3, lj4;
        orc_lj_pair p;
    };
    std::vector<LJC> ljt;
    int ljn = 1;
    // Nose-Hoover, crates/md_thermostat/src/lib.rs:128-139
    bool nh = false;
    double p_xi = 0, q_mass = 1, target_temp = 0.85, ndof = 3;
    // VirialStress, crates/mddem_core/src/virial.rs
    bool virial = false;
    double vir[6]{};
    double pe = 0;
    long step_count = 0, nbuilds = 0, overlap_total = 0;
    int error = 0;
    bool periodic[3] = {true, true, true};  // Domain::periodic_flags
    std::vector<orc_wall> walls;            // plane walls, unit normals

    size_t len() const { return pos.size(); }

    // ---- setup ------------------------------------------------------------
    void configure(const orc_config* c) {
        cfg = *c;
        dem = (c->kind == 0);
        for (int d = 0; d < 3; d++) {
            lo[d] = c->lo[d];
            hi[d] = c->hi[d];
            size[d] = hi[d] - lo[d];
            periodic[d] = !c->fixed[d];
        }
        walls.clear();
        for (int w = 0; dem && w < c->n_walls; w++) {
            orc_wall q = c->walls[w];
            // WallPlane normalisation, dem_wall/src/lib.rs:1259-1262
            double mag = std::sqrt(q.normal[0] * q.normal[0] + q.normal[1] * q.normal[1] + q.normal[2] * q.normal[2]);
            for (int d = 0; d < 3; d++) q.normal[d] /= mag;
            walls.push_back(q);
        }
        cfg.walls = nullptr;
        dt = c->dt;
        skin_fraction = c->skin_fraction;
        bin_min_size = c->bin_size;
        every = c->every;
        check = c->check;
        sort_every = c->sort_every;
        newton = c->newton;
        if (dem && c->n_materials > 0) {
            mats.assign(c->materials, c->materials + c->n_materials);
            mt = build_pair_tables(mats.data(), c->n_materials);
        }
        if (!dem) {
            // build_lj_pair_table, crates/md_lj/src/lib.rs:334-384: the config's
            // n x n table, or the single type's 1 x 1
            ljn = (c->n_lj_types > 1 && c->lj_pairs) ? c->n_lj_types : 1;
            std::vector<orc_lj_pair> tab;
            if (ljn > 1)
                tab.assign(c->lj_pairs, c->lj_pairs + (size_t)ljn * ljn);
            else
                tab.push_back(orc_lj_pair{c->lj_epsilon, c->lj_sigma, c->lj_cutoff});
            ljt.clear();
            for (const orc_lj_pair& q : tab) {
                // LJPairCoeffs::from_params, crates/md_lj/src/lib.rs:230-239
                double s2 = q.sigma * q.sigma;
                double sigma6 = s2 * s2 * s2;
                double rc = q.cutoff * q.sigma;
                ljt.push_back(LJC{48.0 * q.epsilon * sigma6 * sigma6, 24.0 * q.epsilon * sigma6, rc * rc,
                                  4.0 * q.epsilon * sigma6 * sigma6, 4.0 * q.epsilon * sigma6, q});
            }
            cfg.lj_pairs = nullptr;
        }
        nh = c->nose_hoover != 0;
        virial = c->virial != 0;
    }

    // neighbor_setup + compute_bin_grid, crates/mddem_core/src/neighbor.rs:480-541, 290-371
    void neighbor_setup() {
        double max_skin = 0.0;
        double min_skin = 1.7976931348623157e308;
        for (int i = 0; i < nlocal; i++) {
            max_skin = std::fmax(max_skin, cutoff_radius[i]);
            min_skin = std::fmin(min_skin, cutoff_radius[i]);
        }
        double max_cutoff = max_skin > 0.0 ? 2.0 * max_skin * skin_fraction : bin_min_size;
        double disp_buf = (min_skin < 1.7976931348623157e308 * 0.5) ? (skin_fraction - 1.0) * min_skin : 0.0;
        double gc = std::fmax(max_cutoff + 2.0 * disp_buf, 0.0);
        ghost_cutoff = gc;
        cached_max_cutoff = max_cutoff;
        if (bin_min_size < max_cutoff) bin_min_size = max_cutoff;
        double min_bin = std::fmax(bin_min_size, max_cutoff);
        int xi[3];
        for (int d = 0; d < 3; d++) {
            xi[d] = (int)std::fmax(std::floor(size[d] / min_bin), 1.0);
            bin_size[d] = size[d] / (double)xi[d];
        }
        double ghost_cut = ghost_cutoff > max_cutoff ? ghost_cutoff : max_cutoff;
        int s[3];
        for (int d = 0; d < 3; d++) {
            int sr = (int)std::ceil(max_cutoff / bin_size[d]);
            s[d] = (int)std::ceil(ghost_cut / bin_size[d]) + sr;
            bin_count[d] = xi[d] + 2 * s[d];
            bin_origin[d] = lo[d] - bin_size[d] * (double)s[d];
        }
        total_cells = bin_count[0] * bin_count[1] * bin_count[2];
        double cutoff_sq = max_cutoff * max_cutoff;
        stencil.clear();
        stencil_fwd.clear();
        stencil_self = false;
        int ny = bin_count[1], nz = bin_count[2];
        for (int dx = -s[0]; dx <= s[0]; dx++)
            for (int dy = -s[1]; dy <= s[1]; dy++)
                for (int dz = -s[2]; dz <= s[2]; dz++) {
                    double mdx = (double)std::max(std::abs(dx) - 1, 0) * bin_size[0];
                    double mdy = (double)std::max(std::abs(dy) - 1, 0) * bin_size[1];
                    double mdz = (double)std::max(std::abs(dz) - 1, 0) * bin_size[2];
                    if (mdx * mdx + mdy * mdy + mdz * mdz < cutoff_sq) {
                        int off = dx * ny * nz + dy * nz + dz;
                        stencil.push_back(off);
                        if (off > 0) stencil_fwd.push_back(off);
                        else if (off == 0) stencil_self = true;
                    }
                }
    }

    // setup_nose_hoover, crates/md_thermostat/src/lib.rs:195-243
    void setup_nose_hoover() {
        double n = (double)nlocal;
        ndof = 3.0 * n - 3.0;
        double tau = cfg.nh_coupling;
        target_temp = cfg.nh_temperature;
        q_mass = ndof * target_temp * tau * tau;
        p_xi = 0.0;
    }

    // ---- per-atom array helpers ----------------------------------------------
    void truncate_to_nlocal() {
        size_t n = nlocal;
        tag.resize(n); type.resize(n); origin_index.resize(n); is_ghost.resize(n);
        pos.resize(n); vel.resize(n); force.resize(n); mass.resize(n); inv_mass.resize(n);
        cutoff_radius.resize(n); image.resize(n);
        if (dem) {
            radius.resize(n); density.resize(n); inv_inertia.resize(n); body_id.resize(n);
            quat.resize(n); omega.resize(n); ang_mom.resize(n); torque.resize(n);
            contacts.resize(n);
        }
        nghost = 0;
    }

    // Atom::pack_border + DemAtom/ContactHistoryStore pack/unpack as one copy
    void push_ghost(int i, const V3& change) {
        tag.push_back(tag[i]);
        origin_index.push_back(i);
        cutoff_radius.push_back(cutoff_radius[i]);
        type.push_back(type[i]);
        V3 p = pos[i];
        for (int d = 0; d < 3; d++) p[d] = p[d] + change[d];
        pos.push_back(p);
        vel.push_back(vel[i]);
        force.push_back(force[i]);
        mass.push_back(mass[i]);
        inv_mass.push_back(1.0 / mass[i]);
        image.push_back(image[i]);
        is_ghost.push_back(1);
        if (dem) {
            radius.push_back(radius[i]);
            density.push_back(density[i]);
            inv_inertia.push_back(inv_inertia[i]);
            quat.push_back(quat[i]);
            omega.push_back(omega[i]);
            ang_mom.push_back(ang_mom[i]);
            torque.push_back(torque[i]);
            body_id.push_back(body_id[i]);
            std::vector<Contact> c = contacts[i];
            for (auto& e : c) e.active = false;
            contacts.push_back(c);
        }
        nghost++;
    }

    template <class T>
    static void permute(std::vector<T>& v, const std::vector<int>& perm, int n) {
        std::vector<T> nv(n);
        for (int k = 0; k < n; k++) nv[k] = v[perm[k]];
        std::copy(nv.begin(), nv.end(), v.begin());
    }

    void apply_permutation(const std::vector<int>& perm) {
        int n = nlocal;
        permute(tag, perm, n); permute(type, perm, n); permute(origin_index, perm, n);
        permute(is_ghost, perm, n); permute(pos, perm, n); permute(vel, perm, n);
        permute(force, perm, n); permute(mass, perm, n); permute(inv_mass, perm, n);
        permute(cutoff_radius, perm, n); permute(image, perm, n);
        if (dem) {
            permute(radius, perm, n); permute(density, perm, n); permute(inv_inertia, perm, n);
            permute(body_id, perm, n); permute(quat, perm, n); permute(omega, perm, n);
            permute(ang_mom, perm, n); permute(torque, perm, n); permute(contacts, perm, n);
        }
    }

    // ---- schedule systems ----------------------------------------------------
    // initial_integration, crates/mddem_verlet/src/lib.rs:97-123
    void initial_integration() {
        for (int i = 0; i < nlocal; i++) {
            double h = 0.5 * dt * inv_mass[i];
            V3& v = vel[i];
            const V3& f = force[i];
            v[0] += h * f[0];
            v[1] += h * f[1];
            v[2] += h * f[2];
            V3& p = pos[i];
            p[0] += v[0] * dt;
            p[1] += v[1] * dt;
            p[2] += v[2] * dt;
        }
    }
    // final_integration, crates/mddem_verlet/src/lib.rs:136-154
    void final_integration() {
        for (int i = 0; i < nlocal; i++) {
            double h = 0.5 * dt * inv_mass[i];
            V3& v = vel[i];
            const V3& f = force[i];
            v[0] += h * f[0];
            v[1] += h * f[1];
            v[2] += h * f[2];
        }
    }
    // quat_mul, crates/dem_granular/src/rotational.rs:34-41
    static Q4 quat_mul(const Q4& a, const Q4& b) {
        return {a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3],
                a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2],
                a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1],
                a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0]};
    }
    // initial_rotation, crates/dem_granular/src/rotational.rs:59-84
    void initial_rotation() {
        for (int i = 0; i < nlocal; i++) {
            double ii = inv_inertia[i];
            if (ii == 0.0) continue;
            for (int d = 0; d < 3; d++) omega[i][d] += 0.5 * dt * torque[i][d] * ii;
            double ox = omega[i][0], oy = omega[i][1], oz = omega[i][2];
            double om = std::sqrt(ox * ox + oy * oy + oz * oz);
            double angle = om * dt;
            if (angle > 1e-14) {
                double inv = 1.0 / om;
                double half = angle * 0.5;
                double s = std::sin(half);
                Q4 dq = {std::cos(half), ox * inv * s, oy * inv * s, oz * inv * s};
                quat[i] = quat_mul(dq, quat[i]);
            }
        }
    }
    // final_rotation, crates/dem_granular/src/rotational.rs:87-100
    void final_rotation() {
        for (int i = 0; i < nlocal; i++) {
            double ii = inv_inertia[i];
            if (ii == 0.0) continue;
            for (int d = 0; d < 3; d++) omega[i][d] += 0.5 * dt * torque[i][d] * ii;
        }
    }

    // compute_ke, crates/mddem_core/src/atom.rs:489-502
    double compute_ke() const {
        double ke = 0.0;
        for (int i = 0; i < nlocal; i++) {
            const V3& v = vel[i];
            ke += mass[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        }
        return 0.5 * ke;
    }

    // nh_pre_initial, crates/md_thermostat/src/lib.rs:254-301
    void nh_pre_initial() {
        double ke = compute_ke();
        p_xi += (dt / 2.0) * (2.0 * ke - ndof * target_temp);
        double scale = std::exp(-dt / 2.0 * p_xi / q_mass);
        for (int i = 0; i < nlocal; i++) {
            V3& v = vel[i];
            v[0] *= scale;
            v[1] *= scale;
            v[2] *= scale;
            double h = 0.5 * dt * inv_mass[i];
            const V3& f = force[i];
            v[0] += h * f[0];
            v[1] += h * f[1];
            v[2] += h * f[2];
            V3& p = pos[i];
            p[0] += v[0] * dt;
            p[1] += v[1] * dt;
            p[2] += v[2] * dt;
        }
    }
    // nh_post_final, crates/md_thermostat/src/lib.rs:313-353
    void nh_post_final() {
        double scale = std::exp(-dt / 2.0 * p_xi / q_mass);
        for (int i = 0; i < nlocal; i++) {
            V3& v = vel[i];
            double h = 0.5 * dt * inv_mass[i];
            const V3& f = force[i];
            v[0] += h * f[0];
            v[1] += h * f[1];
            v[2] += h * f[2];
            v[0] *= scale;
            v[1] *= scale;
            v[2] *= scale;
        }
        double ke = compute_ke();
        p_xi += (dt / 2.0) * (2.0 * ke - ndof * target_temp);
    }

    // displacement_exceeded, crates/mddem_core/src/neighbor.rs:564-601
    bool displacement_exceeded() const {
        double per_atom_skin = (skin_fraction - 1.0) * cached_min_skin;
        double thr = per_atom_skin * per_atom_skin;
        double bx = size[0], by = size[1], bz = size[2];
        double hbx = bx * 0.5, hby = by * 0.5, hbz = bz * 0.5;
        for (size_t i = 0; i < last_build_pos.size(); i++) {
            double dx = pos[i][0] - last_build_pos[i][0];
            double dy = pos[i][1] - last_build_pos[i][1];
            double dz = pos[i][2] - last_build_pos[i][2];
            if (periodic[0]) { if (dx > hbx) dx -= bx; else if (dx < -hbx) dx += bx; }
            if (periodic[1]) { if (dy > hby) dy -= by; else if (dy < -hby) dy += by; }
            if (periodic[2]) { if (dz > hbz) dz -= bz; else if (dz < -hbz) dz += bz; }
            if (dx * dx + dy * dy + dz * dz > thr) return true;
        }
        return false;
    }
    // needs_rebuild, crates/mddem_core/src/neighbor.rs:605-627
    bool needs_rebuild() const {
        if ((int)last_build_pos.size() != nlocal || nlocal == 0) return true;
        if (state == FullRebuild) return true;
        if (every == 0) return displacement_exceeded();
        if (check) return steps_since_build >= every || displacement_exceeded();
        return steps_since_build >= every;
    }
    // decide_rebuild, crates/mddem_core/src/neighbor.rs:639-674
    void decide_rebuild() {
        bool need = needs_rebuild();
        if (!need) {
            for (int i = 0; i < nlocal && !need; i++)
                for (int d = 0; d < 3; d++)
                    if (periodic[d] && (pos[i][d] < lo[d] || pos[i][d] >= hi[d])) { need = true; break; }
        }
        if (need) state = FullRebuild;
        else steps_since_build += 1;
    }

    // zero_all_forces, crates/mddem_core/src/atom.rs:529-533
    void zero_all_forces() {
        for (auto& f : force) f = {0, 0, 0};
        if (dem) for (auto& t : torque) t = {0, 0, 0};
    }

    // pbc + wrap_periodic, crates/mddem_core/src/domain.rs:396-459.  On a
    // fixed axis the reference removes a particle outside [lo, hi); the
    // oracle, like the GPU path, reports it as an error (12) instead.
    void pbc() {
        for (int i = 0; i < nlocal; i++)
            for (int d = 0; d < 3; d++) {
                double p = pos[i][d];
                double high = lo[d] + size[d];
                if (!periodic[d]) {
                    if (p < lo[d] || p >= hi[d]) error = 12;
                    continue;
                }
                if (p < lo[d]) { p += size[d]; image[i][d] -= 1; }
                else if (p >= high) { p -= size[d]; image[i][d] += 1; }
                pos[i][d] = p;
            }
    }

    // compute_per_atom_offset, crates/mddem_core/src/comm.rs:318-353
    V3 per_atom_offset(const V3& p, const V3& stored) const {
        V3 off{0, 0, 0};
        for (int d = 0; d < 3; d++) {
            if (stored[d] != 0.0) {
                double sg = signum(stored[d]);
                double gp = p[d] + sg * size[d];
                if (gp > lo[d] && gp < hi[d]) off[d] = -sg * size[d];
                else off[d] = sg * size[d];
            }
        }
        return off;
    }
    // forward_comm, crates/mddem_core/src/comm.rs:367-424 (self-sends)
    void forward_comm() {
        for (auto& sw : swaps) {
            struct Pk { V3 p, v, w; double b; };
            std::vector<Pk> buf;
            buf.reserve(sw.send.size());
            for (int idx : sw.send) {
                V3 off = per_atom_offset(pos[idx], sw.off);
                Pk k;
                k.p = {pos[idx][0] + off[0], pos[idx][1] + off[1], pos[idx][2] + off[2]};
                k.v = vel[idx];
                if (dem) { k.w = omega[idx]; k.b = body_id[idx]; }
                buf.push_back(k);
            }
            for (int k = 0; k < sw.recv_count; k++) {
                int g = sw.recv_start + k;
                pos[g] = buf[k].p;
                vel[g] = buf[k].v;
                if (dem) { omega[g] = buf[k].w; body_id[g] = buf[k].b; }
            }
        }
    }
    // borders, crates/mddem_core/src/comm.rs:449-570 (one rank: all swaps are self-sends)
    void borders() {
        if (nghost > 0) truncate_to_nlocal();
        swaps.clear();
        int scan_end = nlocal;
        for (int dim = 0; dim < 3; dim++) {
            int dim_scan_end = scan_end;
            // a fixed axis has no neighbor in either direction on one rank
            // (comm_setup, comm.rs:226-250): no ghosts, no swaps
            if (!periodic[dim]) continue;
            for (int sw = 0; sw < 2; sw++) {
                double periodic_offset = (sw == 0) ? 1.0 : -1.0;
                Swap s;
                s.off[dim] = periodic_offset * size[dim];
                V3 change{0, 0, 0};
                change[dim] = periodic_offset * size[dim];
                std::vector<int> packed;
                for (int i = 0; i < dim_scan_end; i++) {
                    double pd = pos[i][dim];
                    bool in_skin = (sw == 0) ? (pd < lo[dim] + ghost_cutoff) : (pd >= hi[dim] - ghost_cutoff);
                    if (in_skin) packed.push_back(i);
                }
                s.recv_start = (int)len();
                s.recv_count = (int)packed.size();
                for (int i : packed) push_ghost(i, change);
                s.send = packed;
                swaps.push_back(s);
            }
            scan_end = nlocal + nghost;
        }
    }
    // reverse_send_force, crates/mddem_core/src/comm.rs:579-656 (self-sends)
    void reverse_send_force() {
        for (auto it = swaps.rbegin(); it != swaps.rend(); ++it) {
            for (int k = 0; k < it->recv_count; k++) {
                int g = it->recv_start + k;
                int o = origin_index[g];
                if ((int)fscale.size() > g) {
                    fscale[o] += fscale[g];
                    tscale[o] += tscale[g];
                }
                force[o][0] += force[g][0];
                force[o][1] += force[g][1];
                force[o][2] += force[g][2];
                if (dem) {
                    torque[o][0] += torque[g][0];
                    torque[o][1] += torque[g][1];
                    torque[o][2] += torque[g][2];
                }
            }
        }
    }

    int cell_of(const V3& p) const {
        int c[3];
        for (int d = 0; d < 3; d++) {
            int cc = (int)std::floor((p[d] - bin_origin[d]) * (1.0 / bin_size[d]));
            c[d] = std::min(std::max(cc, 0), bin_count[d] - 1);
        }
        return c[0] * bin_count[1] * bin_count[2] + c[1] * bin_count[2] + c[2];
    }

    // sort_atoms_by_bin, crates/mddem_core/src/neighbor.rs:686-794 (stable sort: documented deviation)
    void sort_atoms_by_bin() {
        sort_counter += 1;
        bool periodic_sort = sort_every > 0 && sort_counter >= sort_every;
        if (periodic_sort) sort_counter = 0;
        if (nlocal == 0 || total_cells == 0) {
            return;
        }
        bool rebuild_needed = needs_rebuild();
        if (!periodic_sort && !rebuild_needed) return;
        std::vector<std::pair<uint32_t, int>> idx(nlocal);
        for (int i = 0; i < nlocal; i++) idx[i] = {(uint32_t)cell_of(pos[i]), i};
        std::stable_sort(idx.begin(), idx.end(),
                         [](const auto& a, const auto& b) { return a.first < b.first; });
        std::vector<int> perm(nlocal);
        bool already = true;
        for (int i = 0; i < nlocal; i++) {
            perm[i] = idx[i].second;
            if (perm[i] != i) already = false;
        }
        if (!already) {
            apply_permutation(perm);
            if ((int)last_build_pos.size() >= nlocal) {
                std::vector<V3> old = last_build_pos;
                for (int k = 0; k < nlocal; k++) last_build_pos[k] = old[perm[k]];
            }
            if (nghost > 0) {
                std::vector<int> inv(nlocal);
                for (int k = 0; k < nlocal; k++) inv[perm[k]] = k;
                for (int g = nlocal; g < nlocal + nghost; g++)
                    if (origin_index[g] < nlocal) origin_index[g] = inv[origin_index[g]];
            }
        }
        if (periodic_sort && !already) {
            last_build_pos.clear();
            state = FullRebuild;
        }
    }

    // save_build_positions, crates/mddem_core/src/neighbor.rs:545-561
    void save_build_positions() {
        last_build_pos.assign(pos.begin(), pos.begin() + nlocal);
        steps_since_build = 0;
        double mn = 1.7976931348623157e308, mx = -1.7976931348623157e308;
        for (int i = 0; i < nlocal; i++) {
            mn = std::fmin(mn, cutoff_radius[i]);
            mx = std::fmax(mx, cutoff_radius[i]);
        }
        cached_min_skin = mn;
        if (std::fabs(mx - mn) < 1e-15) {
            double c = 2.0 * mn * skin_fraction;
            uniform = true;
            uniform_cutoff_sq = c * c;
        } else {
            uniform = false;
        }
    }

    // bin_neighbor_list, crates/mddem_core/src/neighbor.rs:810-1080
    void bin_neighbor_list() {
        int total = (int)len();
        state = CommunicateOnly;
        save_build_positions();
        nbuilds++;
        std::vector<uint32_t> atom_cell(total), bin_cnt(total_cells, 0);
        for (int i = 0; i < total; i++) {
            uint32_t c = (uint32_t)cell_of(pos[i]);
            atom_cell[i] = c;
            bin_cnt[c]++;
        }
        std::vector<uint32_t> bin_start(total_cells + 1, 0);
        for (int c = 0; c < total_cells; c++) bin_start[c + 1] = bin_start[c] + bin_cnt[c];
        std::vector<uint32_t> sorted(total), sorted_idx(total);
        for (int c = 0; c < total_cells; c++) bin_cnt[c] = bin_start[c];
        for (int i = 0; i < total; i++) {
            uint32_t c = atom_cell[i];
            uint32_t p = bin_cnt[c];
            sorted[p] = i;
            sorted_idx[i] = p;
            bin_cnt[c] = p + 1;
        }
        std::vector<V3> spos(total);
        for (int m = 0; m < total; m++) spos[m] = pos[sorted[m]];
        const std::vector<int>& st = newton ? stencil_fwd : stencil;
        double sf2 = skin_fraction * skin_fraction;
        nb_off.clear();
        nb_idx.clear();
        for (int i = 0; i < nlocal; i++) {
            nb_off.push_back((uint32_t)nb_idx.size());
            int my = (int)atom_cell[i];
            V3 pi = pos[i];
            double si = cutoff_radius[i];
            auto accept = [&](int m) {
                const V3& pj = spos[m];
                double dx = pj[0] - pi[0], dy = pj[1] - pi[1], dz = pj[2] - pi[2];
                double r2 = std::fma(dx, dx, std::fma(dy, dy, dz * dz));
                if (uniform) return r2 < uniform_cutoff_sq;
                double ss = si + cutoff_radius[sorted[m]];
                return r2 < ss * ss * sf2;
            };
            if (stencil_self) {
                uint32_t cs = bin_start[my], ce = bin_start[my + 1];
                if (newton) {
                    for (uint32_t m = sorted_idx[i] + 1; m < ce; m++)
                        if (accept((int)m)) nb_idx.push_back(sorted[m]);
                } else {
                    for (uint32_t m = cs; m < ce; m++) {
                        if ((int)sorted[m] == i) continue;
                        if (accept((int)m)) nb_idx.push_back(sorted[m]);
                    }
                }
            }
            for (int off : st) {
                if (!newton && off == 0) continue;
                int c = my + off;
                for (uint32_t m = bin_start[c]; m < bin_start[c + 1]; m++)
                    if (accept((int)m)) nb_idx.push_back(sorted[m]);
            }
        }
        nb_off.push_back((uint32_t)nb_idx.size());
    }

    // lj_force, crates/md_lj/src/lib.rs:488-633 (+ PE sum): pair_table.get(ti, tj)
    // when the table has several types, else the one entry
    void lj_force() {
        pe = 0.0;
        double vxx = 0, vyy = 0, vzz = 0, vxy = 0, vxz = 0, vyz = 0;
        double vs = newton ? 1.0 : 0.5;
        const bool multi = ljn > 1;
        for (int i = 0; i < nlocal; i++) {
            V3 pi = pos[i];
            V3 fi = force[i];
            const uint32_t ti = type[i];
            for (uint32_t k = nb_off[i]; k < nb_off[i + 1]; k++) {
                int j = (int)nb_idx[k];
                const V3& pj = pos[j];
                double dx = pj[0] - pi[0], dy = pj[1] - pi[1], dz = pj[2] - pi[2];
                double r2 = std::fma(dx, dx, std::fma(dy, dy, dz * dz));
                const LJC& c = multi ? ljt[(size_t)ti * ljn + type[j]] : ljt[0];
                const double lj1 = c.lj1, lj2 = c.lj2, lj3 = c.lj3, lj4 = c.lj4;
                if (r2 >= c.cut2) continue;
                double r2inv = 1.0 / r2;
                double r6inv = r2inv * r2inv * r2inv;
                double fpair = r2inv * r6inv * std::fma(lj1, r6inv, -lj2);
                add_scale(i, fpair * dx, fpair * dy, fpair * dz, fscale);
                add_scale(j, fpair * dx, fpair * dy, fpair * dz, fscale);
                pe += r6inv * (lj3 * r6inv - lj4) * (newton ? 1.0 : 0.5);
                if (virial) {
                    double fx = -fpair * dx, fy = -fpair * dy, fz = -fpair * dz;
                    vxx += dx * fx * vs; vyy += dy * fy * vs; vzz += dz * fz * vs;
                    vxy += dx * fy * vs; vxz += dx * fz * vs; vyz += dy * fz * vs;
                    fi[0] += fx; fi[1] += fy; fi[2] += fz;
                    if (newton) { force[j][0] -= fx; force[j][1] -= fy; force[j][2] -= fz; }
                } else {
                    fi[0] = std::fma(-fpair, dx, fi[0]);
                    fi[1] = std::fma(-fpair, dy, fi[1]);
                    fi[2] = std::fma(-fpair, dz, fi[2]);
                    if (newton) {
                        force[j][0] = std::fma(fpair, dx, force[j][0]);
                        force[j][1] = std::fma(fpair, dy, force[j][1]);
                        force[j][2] = std::fma(fpair, dz, force[j][2]);
                    }
                }
            }
            force[i] = fi;
        }
        if (virial) {
            vir[0] += vxx; vir[1] += vyy; vir[2] += vzz;
            vir[3] += vxy; vir[4] += vxz; vir[5] += vyz;
        }
    }

    void add_virial(double dx, double dy, double dz, double fx, double fy, double fz) {
        vir[0] += dx * fx; vir[1] += dy * fy; vir[2] += dz * fz;
        vir[3] += dx * fy; vir[4] += dx * fz; vir[5] += dy * fz;
    }

    Contact* find_contact(int i, uint32_t tj) {
        for (auto& e : contacts[i])
            if (e.tag == tj) return &e;
        return nullptr;
    }

    // hertz_mindlin_contact_force (contact_model 0), crates/dem_granular/src/contact.rs:103-615
    // hooke_contact_force (contact_model 1), crates/dem_granular/src/contact.rs:622-990
    void contact_force() {
        bool hooke = cfg.contact_model == 1;
        bool use_dmt = cfg.adhesion_model == 1;
        bool sds_roll = cfg.rolling_model == 1, sds_twist = cfg.twisting_model == 1;
        if ((int)contacts.size() < (int)len()) contacts.resize(len());
        long overlap_warnings = 0;
        for (int i = 0; i < nlocal; i++)
            for (auto& e : contacts[i]) e.active = false;
        double vs = newton ? 1.0 : 0.5;
        for (int i = 0; i < nlocal; i++) {
            for (uint32_t kk = nb_off[i]; kk < nb_off[i + 1]; kk++) {
                int j = (int)nb_idx[kk];
                // same_body, crates/dem_atom/src/lib.rs:583-587
                if (body_id[i] > 0.0 && body_id[j] > 0.0 && std::fabs(body_id[i] - body_id[j]) < 0.5) continue;
                double r1 = radius[i], r2 = radius[j];
                double dx = pos[j][0] - pos[i][0];
                double dy = pos[j][1] - pos[i][1];
                double dz = pos[j][2] - pos[i][2];
                double dist_sq = dx * dx + dy * dy + dz * dz;
                double sum_r = r1 + r2;
                int mi = (int)type[i], mj = (int)type[j];
                double surface_energy = hooke ? 0.0 : mt.at(mt.surface, mi, mj);
                double r_eff = (r1 * r2) / sum_r;
                double e_eff = mt.at(mt.e_eff, mi, mj);
                double delta_pulloff = 0.0;
                if (!hooke && surface_energy > 0.0 && !use_dmt) {
                    double g = surface_energy;
                    delta_pulloff = std::cbrt(kPi * kPi * g * g * r_eff / (4.0 * e_eff * e_eff));
                }
                double interaction_r = sum_r + delta_pulloff;
                if (dist_sq >= interaction_r * interaction_r) continue;
                double distance = std::sqrt(dist_sq);
                if (distance == 0.0) continue;
                double r_min = std::fmin(r1, r2);
                double delta = std::fmin(sum_r - distance, 0.5 * r_min);
                if (hooke && delta <= 0.0) continue;
                if (delta > 0.0 && distance / sum_r < LARGE_OVERLAP_WARN_THRESHOLD) {
                    overlap_warnings++;
                    overlap_total++;
                    if (overlap_warnings > MAX_OVERLAP_WARNINGS) { error = 5; return; }
                }
                if (!hooke && delta <= 0.0 && surface_energy <= 0.0) continue;
                double inv_dist = 1.0 / distance;
                double nx = dx * inv_dist, ny = dy * inv_dist, nz = dz * inv_dist;
                double g_eff = mt.at(mt.g_eff, mi, mj);
                double inv_m_i = inv_mass[i] > 0.0 ? inv_mass[i] : 1.0 / mass[i];
                double inv_m_j = inv_mass[j] > 0.0 ? inv_mass[j] : 1.0 / mass[j];
                double m_r = 1.0 / (inv_m_i + inv_m_j);
                double beta = mt.at(mt.beta, mi, mj);
                double mu = mt.at(mt.friction, mi, mj);
                double mu_r = mt.at(mt.rolling_friction, mi, mj);
                double mu_tw = mt.at(mt.twisting_friction, mi, mj);
                double cohesion_energy = mt.at(mt.cohesion, mi, mj);
                bool jkr_adhesion_only = !hooke && surface_energy > 0.0 && !use_dmt && delta <= 0.0;
                double s_n = 0, k_n = 0, k_t = 0, kn = 0, kt = 0, gamma_n = 0;
                if (hooke) {
                    kn = mt.at(mt.kn, mi, mj);
                    kt = mt.at(mt.kt, mi, mj);
                    gamma_n = 2.0 * beta * std::sqrt(kn * m_r);
                } else if (delta > 0.0) {
                    double sdr = std::sqrt(delta * r_eff);
                    s_n = 2.0 * e_eff * sdr;
                    k_n = 4.0 / 3.0 * e_eff * sdr;
                    k_t = 8.0 * g_eff * sdr;
                }
                double oix = omega[i][0], oiy = omega[i][1], oiz = omega[i][2];
                double ojx = omega[j][0], ojy = omega[j][1], ojz = omega[j][2];
                double r1nx = r1 * nx, r1ny = r1 * ny, r1nz = r1 * nz;
                double vcix = vel[i][0] + (oiy * r1nz - oiz * r1ny);
                double vciy = vel[i][1] + (oiz * r1nx - oix * r1nz);
                double vciz = vel[i][2] + (oix * r1ny - oiy * r1nx);
                double r2nx = r2 * nx, r2ny = r2 * ny, r2nz = r2 * nz;
                double vcjx = vel[j][0] + (-ojy * r2nz + ojz * r2ny);
                double vcjy = vel[j][1] + (-ojz * r2nx + ojx * r2nz);
                double vcjz = vel[j][2] + (-ojx * r2ny + ojy * r2nx);
                double vrx = vcjx - vcix, vry = vcjy - vciy, vrz = vcjz - vciz;
                double v_n = vrx * nx + vry * ny + vrz * nz;
                double f_n_mag;
                if (hooke) {
                    if (cohesion_energy > 0.0) {
                        double f_coh = cohesion_energy * kPi * delta * r_eff;
                        f_n_mag = kn * delta - gamma_n * v_n - f_coh;
                    } else {
                        f_n_mag = std::fmax(kn * delta - gamma_n * v_n, 0.0);
                    }
                } else if (surface_energy > 0.0 && use_dmt) {
                    double f_dmt = 2.0 * kPi * surface_energy * r_eff;
                    double f_diss = 2.0 * beta * SQRT_5_3 * std::sqrt(s_n * m_r) * v_n;
                    f_n_mag = k_n * delta - f_diss - f_dmt;
                } else if (surface_energy > 0.0) {
                    double f_adh = 1.5 * kPi * surface_energy * r_eff;
                    if (jkr_adhesion_only) {
                        f_n_mag = -f_adh;
                    } else {
                        double f_diss = 2.0 * beta * SQRT_5_3 * std::sqrt(s_n * m_r) * v_n;
                        f_n_mag = k_n * delta - f_diss - f_adh;
                    }
                } else if (cohesion_energy > 0.0) {
                    double f_diss = 2.0 * beta * SQRT_5_3 * std::sqrt(s_n * m_r) * v_n;
                    double f_coh = cohesion_energy * kPi * delta * r_eff;
                    f_n_mag = k_n * delta - f_diss - f_coh;
                } else {
                    double f_diss = 2.0 * beta * SQRT_5_3 * std::sqrt(s_n * m_r) * v_n;
                    f_n_mag = std::fmax(k_n * delta - f_diss, 0.0);
                }
                double fnx = f_n_mag * nx, fny = f_n_mag * ny, fnz = f_n_mag * nz;
                force[i][0] -= fnx; force[i][1] -= fny; force[i][2] -= fnz;
                if (newton) { force[j][0] += fnx; force[j][1] += fny; force[j][2] += fnz; }
                if (jkr_adhesion_only) {
                    add_scale(i, fnx, fny, fnz, fscale);
                    add_scale(j, fnx, fny, fnz, fscale);
                    if (virial) add_virial(dx, dy, dz, -fnx * vs, -fny * vs, -fnz * vs);
                    continue;
                }
                double vtx = vrx - v_n * nx, vty = vry - v_n * ny, vtz = vrz - v_n * nz;
                uint32_t tag_i = tag[i], tag_j = tag[j];
                double sign = tag_i < tag_j ? 1.0 : -1.0;
                Contact* entry = find_contact(i, tag_j);
                double stored[7] = {0, 0, 0, 0, 0, 0, 0};
                if (entry) std::memcpy(stored, entry->s, sizeof(stored));
                double sx = sign * stored[0], sy = sign * stored[1], sz = sign * stored[2];
                double sdn = sx * nx + sy * ny + sz * nz;
                sx -= sdn * nx; sy -= sdn * ny; sz -= sdn * nz;
                sx += vtx * dt; sy += vty * dt; sz += vtz * dt;
                double ktt = hooke ? kt : k_t;
                double s_mag = std::sqrt(sx * sx + sy * sy + sz * sz);
                double fts = ktt * s_mag;
                double ft_max = mu * std::fabs(f_n_mag);
                if (fts > ft_max && fts > TANGENTIAL_EPSILON) {
                    double sc = ft_max / fts;
                    sx *= sc; sy *= sc; sz *= sc;
                }
                double gamma_t = 2.0 * SQRT_5_3 * beta * std::sqrt(ktt * m_r);
                double ftx = ktt * sx - gamma_t * vtx;
                double fty = ktt * sy - gamma_t * vty;
                double ftz = ktt * sz - gamma_t * vtz;
                double ftm = std::sqrt(ftx * ftx + fty * fty + ftz * ftz);
                if (ftm > ft_max && ftm > TANGENTIAL_EPSILON) {
                    double sc = ft_max / ftm;
                    ftx *= sc; fty *= sc; ftz *= sc;
                }
                double tix = r1ny * ftz - r1nz * fty, tiy = r1nz * ftx - r1nx * ftz, tiz = r1nx * fty - r1ny * ftx;
                double tjx = r2ny * ftz - r2nz * fty, tjy = r2nz * ftx - r2nx * ftz, tjz = r2nx * fty - r2ny * ftx;
                force[i][0] += ftx; force[i][1] += fty; force[i][2] += ftz;
                if (newton) { force[j][0] -= ftx; force[j][1] -= fty; force[j][2] -= ftz; }
                torque[i][0] += tix; torque[i][1] += tiy; torque[i][2] += tiz;
                if (newton) { torque[j][0] += tjx; torque[j][1] += tjy; torque[j][2] += tjz; }
                add_scale(i, ftx - fnx, fty - fny, ftz - fnz, fscale);
                add_scale(j, ftx - fnx, fty - fny, ftz - fnz, fscale);
                add_scale(i, tix, tiy, tiz, tscale);
                add_scale(j, tjx, tjy, tjz, tscale);
                double orx = oix - ojx, ory = oiy - ojy, orz = oiz - ojz;
                double odn = orx * nx + ory * ny + orz * nz;
                double rollx = orx - odn * nx, rolly = ory - odn * ny, rollz = orz - odn * nz;
                double rdx = sign * stored[3], rdy = sign * stored[4], rdz = sign * stored[5];
                double twd = sign * stored[6];
                if (mu_r > 0.0) {
                    double roll_mag = std::sqrt(rollx * rollx + rolly * rolly + rollz * rollz);
                    if (sds_roll) {
                        double k_roll = mt.at(mt.k_roll, mi, mj);
                        double g_roll = mt.at(mt.g_roll, mi, mj);
                        double rdn = rdx * nx + rdy * ny + rdz * nz;
                        rdx -= rdn * nx; rdy -= rdn * ny; rdz -= rdn * nz;
                        rdx += rollx * dt; rdy += rolly * dt; rdz += rollz * dt;
                        double trx = -k_roll * rdx - g_roll * rollx;
                        double try_ = -k_roll * rdy - g_roll * rolly;
                        double trz = -k_roll * rdz - g_roll * rollz;
                        double trm = std::sqrt(trx * trx + try_ * try_ + trz * trz);
                        double tau_max = mu_r * std::fabs(f_n_mag) * r_eff;
                        if (trm > tau_max && trm > TANGENTIAL_EPSILON) {
                            double sc = tau_max / trm;
                            trx *= sc; try_ *= sc; trz *= sc;
                            if (k_roll > TANGENTIAL_EPSILON) {
                                rdx = (trx + g_roll * rollx) / (-k_roll);
                                rdy = (try_ + g_roll * rolly) / (-k_roll);
                                rdz = (trz + g_roll * rollz) / (-k_roll);
                            }
                        }
                        torque[i][0] += trx; torque[i][1] += try_; torque[i][2] += trz;
                        if (newton) { torque[j][0] -= trx; torque[j][1] -= try_; torque[j][2] -= trz; }
                        add_scale(i, trx, try_, trz, tscale);
                        add_scale(j, trx, try_, trz, tscale);
                    } else if (roll_mag > 1e-30) {
                        double tau_mag = mu_r * std::fabs(f_n_mag) * r_eff;
                        double inv_roll = tau_mag / roll_mag;
                        double trx = -inv_roll * rollx, try_ = -inv_roll * rolly, trz = -inv_roll * rollz;
                        torque[i][0] += trx; torque[i][1] += try_; torque[i][2] += trz;
                        if (newton) { torque[j][0] -= trx; torque[j][1] -= try_; torque[j][2] -= trz; }
                        add_scale(i, trx, try_, trz, tscale);
                        add_scale(j, trx, try_, trz, tscale);
                    }
                }
                if (mu_tw > 0.0) {
                    double twist_vel = odn;
                    if (sds_twist) {
                        double k_tw = mt.at(mt.k_twist, mi, mj);
                        double g_tw = mt.at(mt.g_twist, mi, mj);
                        twd += twist_vel * dt;
                        double tau_tw = -k_tw * twd - g_tw * twist_vel;
                        double tau_max = mu_tw * std::fabs(f_n_mag) * r_eff;
                        if (std::fabs(tau_tw) > tau_max) {
                            tau_tw = signum(tau_tw) * tau_max;
                            if (k_tw > TANGENTIAL_EPSILON) twd = (tau_tw + g_tw * twist_vel) / (-k_tw);
                        }
                        double ttx = tau_tw * nx, tty = tau_tw * ny, ttz = tau_tw * nz;
                        torque[i][0] += ttx; torque[i][1] += tty; torque[i][2] += ttz;
                        if (newton) { torque[j][0] -= ttx; torque[j][1] -= tty; torque[j][2] -= ttz; }
                        add_scale(i, ttx, tty, ttz, tscale);
                        add_scale(j, ttx, tty, ttz, tscale);
                    } else if (std::fabs(twist_vel) > 1e-30) {
                        double tau = mu_tw * std::fabs(f_n_mag) * r_eff;
                        double sg = twist_vel > 0.0 ? -1.0 : 1.0;
                        double ttx = sg * tau * nx, tty = sg * tau * ny, ttz = sg * tau * nz;
                        torque[i][0] += ttx; torque[i][1] += tty; torque[i][2] += ttz;
                        if (newton) { torque[j][0] -= ttx; torque[j][1] -= tty; torque[j][2] -= ttz; }
                        add_scale(i, ttx, tty, ttz, tscale);
                        add_scale(j, ttx, tty, ttz, tscale);
                    }
                }
                if (virial) {
                    double vfx = (-fnx + ftx) * vs, vfy = (-fny + fty) * vs, vfz = (-fnz + ftz) * vs;
                    add_virial(dx, dy, dz, vfx, vfy, vfz);
                }
                double ns[7] = {sign * sx, sign * sy, sign * sz, sign * rdx, sign * rdy, sign * rdz, sign * twd};
                if (entry) {
                    std::memcpy(entry->s, ns, sizeof(ns));
                    entry->active = true;
                } else {
                    Contact c;
                    c.tag = tag_j;
                    std::memcpy(c.s, ns, sizeof(ns));
                    c.active = true;
                    contacts[i].push_back(c);
                }
            }
        }
        for (int i = 0; i < nlocal; i++) {
            auto& v = contacts[i];
            v.erase(std::remove_if(v.begin(), v.end(), [](const Contact& c) { return !c.active; }), v.end());
        }
    }

    // wall_contact_force (plane walls), crates/dem_wall/src/lib.rs:848-985:
    // Hertz normal force against a half-space of infinite radius and mass,
    // damping, JKR / DMT / SJKR adhesion, twisting friction torque.
    void wall_force() {
        bool use_dmt = cfg.adhesion_model == 1;
        for (const orc_wall& W : walls) {
            int wm = W.material;
            for (int i = 0; i < nlocal; i++) {
                const V3& p = pos[i];
                if (!(p[0] >= W.bound_lo[0] && p[0] <= W.bound_hi[0] && p[1] >= W.bound_lo[1] &&
                      p[1] <= W.bound_hi[1] && p[2] >= W.bound_lo[2] && p[2] <= W.bound_hi[2]))
                    continue;
                double distance = (p[0] - W.point[0]) * W.normal[0] + (p[1] - W.point[1]) * W.normal[1] +
                                  (p[2] - W.point[2]) * W.normal[2];
                if (distance <= 0.0) continue;
                double r = radius[i];
                int mi = (int)type[i];
                double e_eff = mt.at(mt.e_eff, mi, wm);
                double gam = mt.at(mt.surface, mi, wm);
                double pull = (gam > 0.0 && !use_dmt) ? std::cbrt(kPi * kPi * gam * gam * r / (4.0 * e_eff * e_eff)) : 0.0;
                double delta = std::fmin(r - distance, 0.5 * r);
                if (delta <= 0.0 && gam <= 0.0) continue;
                if (delta < -pull) continue;
                bool adhesion_only = gam > 0.0 && !use_dmt && delta <= 0.0;
                double s_n = 0.0, k_n = 0.0;
                if (delta > 0.0) {
                    double sdr = std::sqrt(delta * r);
                    s_n = 2.0 * e_eff * sdr;
                    k_n = 4.0 / 3.0 * e_eff * sdr;
                }
                double v_n = (vel[i][0] - W.velocity[0]) * W.normal[0] + (vel[i][1] - W.velocity[1]) * W.normal[1] +
                             (vel[i][2] - W.velocity[2]) * W.normal[2];
                double beta = mt.at(mt.beta, mi, wm);
                double coh = mt.at(mt.cohesion, mi, wm);
                double f_diss = 2.0 * beta * SQRT_5_3 * std::sqrt(s_n * mass[i]) * v_n;
                double fn;
                if (gam > 0.0 && use_dmt) fn = k_n * delta - f_diss - 2.0 * kPi * gam * r;
                else if (gam > 0.0) fn = adhesion_only ? -(1.5 * kPi * gam * r) : k_n * delta - f_diss - 1.5 * kPi * gam * r;
                else if (coh > 0.0) fn = k_n * delta - f_diss - coh * kPi * delta * r;
                else fn = std::fmax(k_n * delta - f_diss, 0.0);
                for (int d = 0; d < 3; d++) force[i][d] += fn * W.normal[d];
                if (i < (int)fscale.size()) fscale[i] += std::fabs(fn);
                if (delta > 0.0) {
                    double mu = mt.at(mt.twisting_friction, mi, wm);
                    if (mu > 0.0) {
                        double tw = omega[i][0] * W.normal[0] + omega[i][1] * W.normal[1] + omega[i][2] * W.normal[2];
                        if (std::fabs(tw) > 1e-30) {
                            double tau = mu * std::fabs(fn) * r;
                            double sg = tw > 0.0 ? -1.0 : 1.0;
                            for (int d = 0; d < 3; d++) torque[i][d] += sg * tau * W.normal[d];
                            if (i < (int)tscale.size()) tscale[i] += std::fabs(tau);
                        }
                    }
                }
            }
        }
    }

    // Counter-based N(0,1): SplitMix64 finaliser over (seed, step, tag, draw),
    // 53-bit uniforms, Box-Muller cosine branch with the reference's
    // max(u1, 1e-300) clamp (normal_sample, md_thermostat/src/lib.rs:565-581).
    static uint64_t lv_mix(uint64_t z) {
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    static double lv_uniform(uint64_t seed, long step, uint32_t tag, int draw) {
        const uint64_t h = lv_mix(seed + lv_mix((uint64_t)step * 0x9e3779b97f4a7c15ull +
                                                lv_mix(((uint64_t)tag << 3) + (uint64_t)draw)));
        return (double)(h >> 11) * 0x1.0p-53;
    }
    static double lv_normal(uint64_t seed, long step, uint32_t tag, int k) {
        const double u1 = lv_uniform(seed, step, tag, 2 * k), u2 = lv_uniform(seed, step, tag, 2 * k + 1);
        return std::sqrt(-2.0 * std::log(std::fmax(u1, 1e-300))) * std::cos(6.283185307179586 * u2);
    }
    // langevin_force, md_thermostat/src/lib.rs:529-563 (PostForce)
    void langevin_force() {
        const double gamma = cfg.lv_damping, kt = cfg.lv_temperature;
        if (gamma == 0.0) return;
        for (int i = 0; i < nlocal; i++) {
            const double drag = gamma * mass[i];
            const double rc = std::sqrt(2.0 * drag * kt / dt);
            for (int d = 0; d < 3; d++) force[i][d] -= drag * vel[i][d];
            for (int d = 0; d < 3; d++) force[i][d] += rc * lv_normal(cfg.lv_seed, step_count, tag[i], d);
        }
    }

    void add_scale(int a, double fx, double fy, double fz, std::vector<double>& sc) {
        sc[a] += std::sqrt(fx * fx + fy * fy + fz * fz);
    }

    void compute_forces() {
        fscale.assign(len(), 0.0);
        tscale.assign(len(), 0.0);
        if (virial) for (double& v : vir) v = 0.0;  // zero_virial_stress
        if (dem) contact_force();
        else lj_force();
    }

    // One timestep in the compiled schedule order (schedule.dot:45-153).
    void step() {
        // wall_move, crates/dem_wall/src/lib.rs:766-790 (PreInitialIntegration)
        for (orc_wall& W : walls)
            for (int d = 0; d < 3; d++) W.point[d] += W.velocity[d] * dt;
        if (nh) nh_pre_initial();
        else {
            initial_integration();
            if (dem) initial_rotation();
        }
        if (state == CommunicateOnly) decide_rebuild();
        zero_all_forces();
        if (state == FullRebuild) {
            truncate_to_nlocal();  // remove_ghost_atoms
            pbc();
        } else {
            forward_comm();
        }
        sort_atoms_by_bin();
        if (state == FullRebuild) {
            borders();
            bin_neighbor_list();
        }
        compute_forces();
        reverse_send_force();
        if (!walls.empty()) wall_force();
        if (cfg.langevin) langevin_force();
        if (nh) nh_post_final();
        else {
            final_integration();
            if (dem) final_rotation();
        }
        step_count++;
    }

    void force_only() {
        zero_all_forces();
        truncate_to_nlocal();
        state = FullRebuild;
        pbc();
        sort_atoms_by_bin();
        borders();
        bin_neighbor_list();
        compute_forces();
        reverse_send_force();
        if (!walls.empty()) wall_force();
    }

    // print_granular_temperature, crates/dem_granular/src/granular_temp.rs:44-134
    void granular(double& tg, double& ke, double& mom) const {
        double mvx = 0, mvy = 0, mvz = 0, m = 0;
        for (int i = 0; i < nlocal; i++) {
            mvx += mass[i] * vel[i][0];
            mvy += mass[i] * vel[i][1];
            mvz += mass[i] * vel[i][2];
            m += mass[i];
        }
        double ax = mvx / m, ay = mvy / m, az = mvz / m;
        double vd = 0;
        for (int i = 0; i < nlocal; i++) {
            double dx = vel[i][0] - ax, dy = vel[i][1] - ay, dz = vel[i][2] - az;
            vd += mass[i] * (dx * dx) + mass[i] * (dy * dy) + mass[i] * (dz * dz);
        }
        tg = vd / (3.0 * m);
        ke = 0;
        for (int i = 0; i < nlocal; i++)
            ke += 0.5 * mass[i] * (vel[i][0] * vel[i][0] + vel[i][1] * vel[i][1] + vel[i][2] * vel[i][2]);
        mom = std::sqrt(mvx * mvx + mvy * mvy + mvz * mvz);
    }
};

}  // namespace

extern "C" {

void* orc_create(const orc_config* cfg) {
    if (!cfg) return nullptr;
    Sim* s = new Sim();
    s->configure(cfg);
    return s;
}

void orc_destroy(void* h) { delete static_cast<Sim*>(h); }

int orc_load(void* h, size_t n, const uint32_t* tag, const uint32_t* type, const double* pos,
             const double* vel, const double* mass, const double* cutoff_radius, const double* radius,
             const double* density, const double* inv_inertia, const double* omega, const double* quat) {
    Sim* s = static_cast<Sim*>(h);
    s->nlocal = (int)n;
    s->nghost = 0;
    s->tag.assign(tag, tag + n);
    s->type.assign(n, 0);
    if (type) s->type.assign(type, type + n);
    s->origin_index.assign(n, 0);
    s->is_ghost.assign(n, 0);
    s->pos.resize(n); s->vel.resize(n); s->force.assign(n, {0, 0, 0});
    s->mass.assign(mass, mass + n);
    s->inv_mass.resize(n);
    s->cutoff_radius.assign(cutoff_radius, cutoff_radius + n);
    s->image.assign(n, {0, 0, 0});
    for (size_t i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            s->pos[i][d] = pos[3 * i + d];
            s->vel[i][d] = vel[3 * i + d];
        }
        s->inv_mass[i] = 1.0 / mass[i];
    }
    if (s->dem) {
        s->radius.assign(radius, radius + n);
        s->density.assign(n, 2500.0);
        if (density) s->density.assign(density, density + n);
        s->inv_inertia.assign(inv_inertia, inv_inertia + n);
        s->body_id.assign(n, 0.0);
        s->quat.resize(n);
        s->omega.resize(n);
        s->ang_mom.assign(n, {0, 0, 0});
        s->torque.assign(n, {0, 0, 0});
        s->contacts.assign(n, {});
        for (size_t i = 0; i < n; i++) {
            for (int d = 0; d < 3; d++) s->omega[i][d] = omega ? omega[3 * i + d] : 0.0;
            for (int d = 0; d < 4; d++) s->quat[i][d] = quat ? quat[4 * i + d] : (d == 0 ? 1.0 : 0.0);
        }
    }
    s->neighbor_setup();
    if (s->nh) s->setup_nose_hoover();
    s->state = FullRebuild;
    return 0;
}

int orc_set_force(void* h, size_t i, const double* f3, const double* t3) {
    Sim* s = static_cast<Sim*>(h);
    if (i >= (size_t)s->nlocal) return 9;
    for (int d = 0; d < 3; d++) {
        if (f3) s->force[i][d] = f3[d];
        if (t3 && s->dem) s->torque[i][d] = t3[d];
    }
    return 0;
}

int orc_step(void* h, long nsteps) {
    Sim* s = static_cast<Sim*>(h);
    for (long k = 0; k < nsteps && !s->error; k++) s->step();
    return s->error;
}

int orc_force_only(void* h) {
    Sim* s = static_cast<Sim*>(h);
    s->force_only();
    return s->error;
}

size_t orc_nlocal(void* h) { return (size_t) static_cast<Sim*>(h)->nlocal; }

int orc_get_field(void* h, int field, double* out) {
    Sim* s = static_cast<Sim*>(h);
    int n = s->nlocal;
    switch (field) {
        case ORC_F_POS: for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->pos[i][d]; break;
        case ORC_F_VEL: for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->vel[i][d]; break;
        case ORC_F_FORCE: for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->force[i][d]; break;
        case ORC_F_OMEGA: for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->dem ? s->omega[i][d] : 0.0; break;
        case ORC_F_TORQUE: for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->dem ? s->torque[i][d] : 0.0; break;
        case ORC_F_QUAT: for (int i = 0; i < n; i++) for (int d = 0; d < 4; d++) out[4 * i + d] = s->dem ? s->quat[i][d] : (d == 0); break;
        case ORC_F_MASS: for (int i = 0; i < n; i++) out[i] = s->mass[i]; break;
        case ORC_F_RADIUS: for (int i = 0; i < n; i++) out[i] = s->dem ? s->radius[i] : s->cutoff_radius[i]; break;
        case ORC_F_LAST_BUILD_POS:
            for (int i = 0; i < n; i++) for (int d = 0; d < 3; d++)
                out[3 * i + d] = i < (int)s->last_build_pos.size() ? s->last_build_pos[i][d] : 0.0;
            break;
        default: return 9;
    }
    return 0;
}

int orc_get_tags(void* h, uint32_t* out) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < s->nlocal; i++) out[i] = s->tag[i];
    return 0;
}

int orc_get_scale(void* h, double* fs, double* ts) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < s->nlocal; i++) {
        const bool have = i < (int)s->fscale.size();
        if (fs) fs[i] = have ? s->fscale[i] : 0.0;
        if (ts) ts[i] = have ? s->tscale[i] : 0.0;
    }
    return 0;
}

int orc_get_types(void* h, uint32_t* out) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < s->nlocal; i++) out[i] = s->type[i];
    return 0;
}

int orc_get_image(void* h, int32_t* out) {
    Sim* s = static_cast<Sim*>(h);
    for (int i = 0; i < s->nlocal; i++) for (int d = 0; d < 3; d++) out[3 * i + d] = s->image[i][d];
    return 0;
}

size_t orc_get_pairs(void* h, uint32_t* out, size_t cap) {
    Sim* s = static_cast<Sim*>(h);
    size_t n = 0;
    for (int i = 0; i < s->nlocal; i++)
        for (uint32_t k = s->nb_off[i]; k < s->nb_off[i + 1]; k++) {
            if (n < cap) {
                out[2 * n] = s->tag[i];
                out[2 * n + 1] = s->tag[s->nb_idx[k]];
            }
            n++;
        }
    return n;
}

size_t orc_get_history(void* h, uint32_t* keys, double* vals, size_t cap) {
    Sim* s = static_cast<Sim*>(h);
    size_t n = 0;
    if (!s->dem) return 0;
    for (int i = 0; i < s->nlocal; i++)
        for (auto& c : s->contacts[i]) {
            if (n < cap) {
                keys[2 * n] = s->tag[i];
                keys[2 * n + 1] = c.tag;
                for (int d = 0; d < 7; d++) vals[7 * n + d] = c.s[d];
            }
            n++;
        }
    return n;
}

int orc_set_history(void* h, size_t n, const uint32_t* keys, const double* vals) {
    Sim* s = static_cast<Sim*>(h);
    if (!s->dem) return 9;
    std::map<uint32_t, int> idx;
    for (int i = 0; i < s->nlocal; i++) idx[s->tag[i]] = i;
    for (int i = 0; i < s->nlocal; i++) s->contacts[i].clear();
    for (size_t k = 0; k < n; k++) {
        auto it = idx.find(keys[2 * k]);
        if (it == idx.end()) return 9;
        Contact c;
        c.tag = keys[2 * k + 1];
        for (int d = 0; d < 7; d++) c.s[d] = vals[7 * k + d];
        c.active = false;
        s->contacts[it->second].push_back(c);
    }
    return 0;
}

int orc_thermo(void* h, double* out) {
    Sim* s = static_cast<Sim*>(h);
    double ke = s->compute_ke();
    double ndof = 3.0 * (double)s->nlocal - 3.0;
    double tg = 0, ke2 = 0, mom = 0;
    s->granular(tg, ke2, mom);
    out[0] = ke;
    out[1] = s->pe;
    out[2] = ndof > 0 ? 2.0 * ke / ndof : 0.0;
    out[3] = s->p_xi;
    out[4] = tg;
    out[5] = mom;
    for (int k = 0; k < 6; k++) out[6 + k] = s->vir[k];
    out[12] = (double)s->nbuilds;
    out[13] = (double)s->step_count;
    out[14] = s->ndof;
    out[15] = s->q_mass;
    return 0;
}

long orc_overlap_count(void* h) { return static_cast<Sim*>(h)->overlap_total; }

// setup_lj_tails (md_lj/src/lib.rs:397-445): rho = N / V with V = size_x
// size_y size_z (domain.rs:153); per type pair, in table order, rc =
// sqrt((cutoff sigma)^2) and the weight (1 / ntypes)^2 of an equimolar
// mixture; powi(3) as (x x) x.
int orc_lj_tails(void* h, double* e_tail, double* p_tail) {
    Sim* s = static_cast<Sim*>(h);
    const double n = (double)s->nlocal;
    const double v = s->size[0] * s->size[1] * s->size[2];
    const double rho = n / v;
    const double frac = 1.0 / (double)s->ljn;
    const double PI = 3.141592653589793;
    double e = 0.0, p = 0.0;
    for (const Sim::LJC& c : s->ljt) {
        const double eps = c.p.epsilon, sig = c.p.sigma;
        const double cs = c.p.cutoff * sig;
        const double rc = std::sqrt(cs * cs);
        const double sigma3 = (sig * sig) * sig;
        const double rc3 = (rc * rc) * rc;
        const double rc9 = (rc3 * rc3) * rc3;
        const double sigma6 = sigma3 * sigma3;
        const double sigma9 = sigma6 * sigma3;
        const double w = frac * frac;
        e += w * (8.0 / 3.0) * PI * n * rho * eps * sigma3 * (sigma9 / (3.0 * rc9) - sigma3 / rc3);
        p += w * (16.0 / 3.0) * PI * rho * rho * eps * sigma3 * (2.0 * sigma9 / (3.0 * rc9) - sigma3 / rc3);
    }
    *e_tail = e;
    *p_tail = p;
    return 0;
}

}  // extern "C"

// ---- seeded random sequential addition (input generation for the CPU arm) --
// The same stream and acceptance rule as the library's mdg_rsa_spheres:
// candidate centres uniform in the box (inset by rmax when asked), radius
// uniform in [rmin, rmax], rejected when a placed sphere lies within
// sep_factor (r_i + r_j) under the minimum image (insert.rs:523-571), with
// xoshiro256** (Blackman & Vigna 2018) seeded through splitmix64 and a
// cell grid of side >= sep_factor 2 rmax.  Same seed, same spheres.
namespace {
struct OrcRng {
    uint64_t s[4];
    explicit OrcRng(uint64_t seed) {
        for (auto& v : s) {
            uint64_t z = (seed += 0x9e3779b97f4a7c15ull);
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            v = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    double uniform() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return (double)(r >> 11) * 0x1.0p-53;
    }
};
}  // namespace

extern "C" int orc_rsa_spheres(size_t n, const double* box_lo, const double* box_hi, double rmin, double rmax,
                               double sep_factor, int inset, uint64_t seed, uint64_t max_attempts, double* pos,
                               double* rad, size_t* placed) {
    *placed = 0;
    if (!(rmin > 0.0) || !(rmax >= rmin) || !(sep_factor > 0.0)) return 9;
    double L[3], lo[3], hi[3], cell[3];
    int nc[3];
    const double reach = sep_factor * 2.0 * rmax;
    for (int d = 0; d < 3; d++) {
        L[d] = box_hi[d] - box_lo[d];
        lo[d] = box_lo[d] + (inset ? rmax : 0.0);
        hi[d] = box_hi[d] - (inset ? rmax : 0.0);
        if (!(L[d] > 0.0) || !(hi[d] > lo[d])) return 9;
        const double c = std::floor(L[d] / reach);
        nc[d] = c < 1.0 ? 1 : (c > 1024.0 ? 1024 : (int)c);
        cell[d] = L[d] / nc[d];
    }
    std::vector<int64_t> head((size_t)nc[0] * nc[1] * nc[2], -1), link;
    link.reserve(n);
    const uint64_t limit = max_attempts ? max_attempts : (uint64_t)n * 20000ull;
    const bool poly = rmax > rmin;
    OrcRng rng(seed);
    auto cell_of = [&](double x, int d) {
        int c = (int)std::floor((x - box_lo[d]) / cell[d]) % nc[d];
        return c < 0 ? c + nc[d] : c;
    };
    // the cells around a candidate: all of an axis with fewer than 3 cells
    auto nb = [&](int ci, int d, int k) { return nc[d] >= 3 ? (ci + k - 1 + nc[d]) % nc[d] : k; };
    size_t count = 0;
    for (uint64_t att = 0; att < limit && count < n; att++) {
        double c[3];
        for (int d = 0; d < 3; d++) c[d] = lo[d] + (hi[d] - lo[d]) * rng.uniform();
        const double r = poly ? rmin + (rmax - rmin) * rng.uniform() : rmin;
        const int ci[3] = {cell_of(c[0], 0), cell_of(c[1], 1), cell_of(c[2], 2)};
        const int m[3] = {nc[0] >= 3 ? 3 : nc[0], nc[1] >= 3 ? 3 : nc[1], nc[2] >= 3 ? 3 : nc[2]};
        bool ok = true;
        for (int a = 0; a < m[0] && ok; a++)
            for (int b = 0; b < m[1] && ok; b++)
                for (int e = 0; e < m[2] && ok; e++) {
                    const size_t k = ((size_t)nb(ci[0], 0, a) * nc[1] + nb(ci[1], 1, b)) * nc[2] + nb(ci[2], 2, e);
                    for (int64_t j = head[k]; j >= 0 && ok; j = link[j]) {
                        double r2 = 0.0;
                        for (int d = 0; d < 3; d++) {
                            double dx = pos[3 * j + d] - c[d];
                            dx -= L[d] * std::nearbyint(dx / L[d]);
                            r2 += dx * dx;
                        }
                        const double md = sep_factor * (r + rad[j]);
                        ok = !(r2 <= md * md);
                    }
                }
        if (!ok) continue;
        for (int d = 0; d < 3; d++) pos[3 * count + d] = c[d];
        rad[count] = r;
        const size_t k = ((size_t)ci[0] * nc[1] + ci[1]) * nc[2] + ci[2];
        link.push_back(head[k]);
        head[k] = (int64_t)count;
        count++;
    }
    *placed = count;
    return count == n ? 0 : 9;
}
