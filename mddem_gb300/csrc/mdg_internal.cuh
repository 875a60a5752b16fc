// mdg_internal.cuh -- device data layout shared by the kernels and the C ABI.
//
// Layout in HBM (one context = one or more independent systems):
//   * Particles of all systems live in one SoA address space.  System s owns
//     [p0, p0 + n) padded to npad (a multiple of BLK) so that every block of a
//     per-particle kernel belongs to exactly one system (blk_sys[b]).
//   * 32-byte rows for everything a pair kernel gathers: pos = (x,y,z,radius),
//     vel = (vx,vy,vz,1/m), omg = (wx,wy,wz,1/I).  One sector per neighbour.
//   * Neighbour list: per-system ELL block [ncap][npad] of u32 entries
//     (j | code << 26), code = owner*27 + periodic-image shift (base 3).
//   * Contact history: per particle up to hcap (partner tag, 7 doubles),
//     layout [c][npad] / [c*7+k][npad] per system, double-buffered per step.
//   * Bin grid: per system the reference's extended grid (interior + ghost
//     layers), counts/starts over ext cells, particles sorted by ext cell.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mdg {

constexpr int BLK = 128;               // particles per block (segment padding unit)
constexpr int IDX_BITS = 26;
constexpr uint32_t IDX_MASK = (1u << IDX_BITS) - 1u;
constexpr int NTAB = 14;               // material pair tables

// device status bits (sticky per system)
enum : int {
    ST_OVERLAP = 1,
    ST_NAN = 2,
    ST_NBR_OVF = 4,
    ST_HIST_OVF = 8,
    ST_TIMEOUT = 16,
};

// material pair table ids (MaterialTable::build_pair_tables order)
enum : int {
    T_BETA = 0, T_FRICTION, T_ROLL_FRICTION, T_COHESION, T_SURFACE, T_EEFF, T_GEFF,
    T_TWIST_FRICTION, T_KN, T_KT, T_KROLL, T_GROLL, T_KTWIST, T_GTWIST
};

struct SysParams {
    int kind;            // 0 DEM, 1 LJ
    int precision;       // 0 fp64, 1 mixed
    int contact_model, adhesion_model, rolling_model, twisting_model;
    int p0, n, npad;     // particle segment
    int b0, nb;          // first particle block; blocks holding the n particles
    int ncb;             // cell blocks of the system's cell segment
    int c0, ncell;       // ext-cell segment
    int nc[3];           // interior cells per axis
    int ext[3];          // extended grid (interior + 2*layers)
    int sl[3];           // ghost layers per side
    int win[3];          // enumeration half-width in interior cells
    double lo[3], hi[3], L[3];
    double bin[3], inv_bin[3], origin[3];
    double max_cutoff, stencil_cut_sq;
    unsigned int stencil_bits[32];  // offsets in [-sl, sl]^3 that pass the stencil distance test
    float pre_cut2;      // fp32 prefilter radius^2 for the list build (conservative)
    float band_rel;      // relative error bound of the hi-only fp32 r^2 in the list build
    float ucut2f;        // fp32 copy of uniform_cutoff_sq
    float sf2f;          // fp32 copy of sf2
    float Lh[3], Ll[3];  // two-float split of the box lengths
    double skin_fraction, sf2;
    int uniform;         // all cutoff radii equal
    double uniform_cutoff_sq;
    double min_skin;
    double disp_thr_sq;
    double dt;
    int policy, every, check, sort_every, newton;
    int nmat;
    int matcap;          // material slots reserved in the packed tables
    long long mat0;      // offset into the packed material tables
    double lj1, lj2, lj3, lj4, lj_cut2;
    float lj1f, lj2f, lj3f, lj4f, lj_cut2f;
    float disp_thr2f;    // fp32 rebuild threshold of the mixed path, 1e-5 on the safe side
    int nh;
    double nh_T, nh_Q, nh_ndof;
    int virial;
    int ncap;            // neighbour-list capacity per particle
    long long lst0;      // offset of this system's ELL block
    int hcap;            // contact-history capacity per particle
    long long h0;        // offset of this system's history block (entries)
    int tpp;             // threads per particle in force kernels
};

struct SysState {
    int rebuild;         // 1: rebuild this step (FullRebuild)
    int periodic_sort;   // 1: periodic spatial sort this step
    int nonid;           // periodic sort produced a non-identity permutation
    int status;          // sticky error bits
    int steps_since_build;
    int sort_counter;
    int nbuilds;
    int max_nbr;
    int overlap;         // large-overlap count this step
    unsigned int red_count;
    double ke;           // KE after the last post-final (NH)
    double p_xi_pre;     // p_xi after the pre-initial half step
    double p_xi_post;    // p_xi after the post-final half step
    double nh_scale;     // exp(-dt/2 p_xi_pre / Q) for the current step (pre and post)
    double vir[6];
    double pe;
    long long step;
    long long remaining; // steps left before the system freezes; -1 = unlimited
    int hcur;            // contact-history buffer holding the current springs
    int pad_;
};

__device__ __forceinline__ bool sys_active(const SysState* st) {
    return *((volatile const long long*)&st->remaining) != 0;
}

struct Dev {
    // per particle
    double4* pos;   // x y z radius
    double4* vel;   // vx vy vz inv_mass
    double4* frc;   // fx fy fz pe_i
    double4* omg;   // wx wy wz inv_inertia
    double4* trq;   // tx ty tz 0
    double4* quat;  // w x y z
    double4* lbp;   // last build position
    double* mass;
    double* cutr;
    uint32_t* tag;
    uint32_t* type;
    int4* img;
    // contact history, buffer [cur] read and [cur^1] written each step
    int* hcnt[2];
    uint32_t* htag[2];
    double* hval[2];
    // neighbour list
    int* nnum;
    uint32_t* nlist;
    // rebuild scratch
    int* cell;       // ext flat cell of each particle (system-relative); after the
                     // permutation bit 31 flags a bin coordinate within 1e-9 of a bin edge
    int* cnt;        // per ext cell count / cursor
    int* cstart;     // per ext cell start (absolute particle index), +1 sentinel per system
    int* perm;       // new -> old (absolute)
    // gather scratch (same shapes as the primaries)
    double4 *s_pos, *s_vel, *s_omg, *s_quat;
    double *s_mass, *s_cutr;
    uint32_t *s_tag, *s_type;
    int4* s_img;
    int* s_hcnt;
    uint32_t* s_htag;
    double* s_hval;
    // two-float geometry copy relative to the box corner, interleaved so one
    // particle is one 32-byte sector: pos2[2i] = (x_hi, y_hi, z_hi, cutoff
    // radius), pos2[2i+1] = (x_lo, y_lo, z_lo, 0).  lbp2: same at the last build.
    float4* pos2;
    float4* lbp2;
    // per-particle virial (6 x P) when any system accumulates it
    double* vir;
    // reductions
    double* blkpart;   // [nblocks][8]
    const int* blk_sys;   // particle block -> system
    const int* cblk_sys;  // cell block -> system (-1 past the systems' cells)
    const int* cblk0;     // first cell block of each system
    int ncblocks;         // allocated cell blocks
    // Run maps: the particle / cell blocks of the systems that advance in this
    // launch (uploaded, step budget not exhausted).  The step kernels' grids
    // cover only these, so idle slots of a batch cost nothing.
    const int* blk_run;   // global particle block ids
    int nrun;
    const int* cblk_run;  // global cell block ids
    int ncrun;
    const int* run_sys;   // the running systems, ascending
    int nrun_sys;
    // Rebuild work list, written on the device by k_rb_plan when a step
    // rebuilds: the systems that sort or rebuild, with prefix offsets of their
    // particle blocks and cell blocks (rb_poff / rb_coff have rb_n + 1 entries).
    // The rebuild kernels walk these virtual blocks with grid-stride loops.
    int* rb_sys;
    int* rb_poff;
    int* rb_coff;
    int* rb_n;
    const SysParams* sp;
    SysState* ss;
    const double* mat;
    const float* matf;   // fp32 copy of the material tables (mixed path)
    int nsys;
    int nblocks;
    long long P;       // total padded particles
    int hist_any;      // history arrays allocated
    // graph mode: k_initial's last block sets this IF-node condition to
    // "some system rebuilds (or sorts) this step"; 0 = no conditional
    unsigned long long cond;
    int use_cond;
    unsigned int* grid_ctr;
    unsigned long long* stat_ctr;  // [0] steps whose rebuild branch opened
};

// Two-float separation (x_j + s L) - x_i from positions stored relative to
// the box corner as hi + lo floats.  The shift is applied to the coordinate
// that sits next to the crossed face, which keeps the hi-part difference exact
// (Sterbenz); the result carries ~1e-7 relative error.
__device__ __forceinline__ float two_float_sep(float xj_hi, float xj_lo, float xi_hi, float xi_lo, int s, float Lh,
                                               float Ll) {
    float dh, dl;
    if (s > 0) {
        dh = xj_hi - (xi_hi - Lh);
        dl = xj_lo - (xi_lo - Ll);
    } else if (s < 0) {
        dh = (xj_hi - Lh) - xi_hi;
        dl = (xj_lo - Ll) - xi_lo;
    } else {
        dh = xj_hi - xi_hi;
        dl = xj_lo - xi_lo;
    }
    return dh + dl;
}

// (hi, lo) += t for a two-float value (Knuth two-sum, then renormalised).
__device__ __forceinline__ void two_float_add(float& hi, float& lo, float t) {
    const float s = hi + t;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (t - bb);
    const float l = lo + err;
    const float h2 = s + l;
    lo = l - (h2 - s);
    hi = h2;
}

// ---- kernel launchers (mdg_kernels_fp64.cu / mdg_kernels_mixed.cu) ----------
// Each returns the number of kernels it launched on `st`.
int launch_initial(const Dev& d, cudaStream_t st);
int launch_initial_mixed(const Dev& d, cudaStream_t st);
int launch_rebuild(const Dev& d, cudaStream_t st);
int launch_force_fp64(const Dev& d, int has_lj, int has_dem, int tpp, cudaStream_t st);
int launch_force_mixed(const Dev& d, int has_lj, int has_dem, int tpp, cudaStream_t st);
// device-side loop control of a multi-step WHILE graph
int launch_loop_ctl(const Dev& d, long long* counter, unsigned long long handle, cudaStream_t st);
int launch_final(const Dev& d, cudaStream_t st, int integrate);
int launch_ke_init(const Dev& d, cudaStream_t st);
// thermo reduction for all systems into out[nsys][16] (device pointer)
int launch_thermo(const Dev& d, double* out, cudaStream_t st);
// history injection/extraction helpers run on the host side of the API

}  // namespace mdg
