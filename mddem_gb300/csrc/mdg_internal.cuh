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

#include "../../include/mdg.h"  // MDG_MAX_WALLS, status and kind codes

namespace mdg {

constexpr int BLK = 128;               // particles per block (segment padding unit)
constexpr int IDX_BITS = 26;
constexpr uint32_t IDX_MASK = (1u << IDX_BITS) - 1u;
constexpr int NTAB = 14;               // material pair tables
// LJ multi-type pair tables (build_lj_pair_table, md_lj/src/lib.rs:334-384),
// packed in an LJ system's slot of the material tables with the same layout:
// entry (tab, a, b) at mat0 + (tab * nmat + a) * nmat + b
enum { TL_LJ1 = 0, TL_LJ2, TL_LJ3, TL_LJ4, TL_CUT2, NTAB_LJ };
constexpr int THERMO_W = 24;           // doubles per system in the thermo record

// device status bits (sticky per system)
enum : int {
    ST_OVERLAP = 1,
    ST_NAN = 2,
    ST_NBR_OVF = 4,
    ST_HIST_OVF = 8,
    ST_TIMEOUT = 16,
    ST_LOST = 32,
};

// material pair table ids (MaterialTable::build_pair_tables order)
enum : int {
    T_BETA = 0, T_FRICTION, T_ROLL_FRICTION, T_COHESION, T_SURFACE, T_EEFF, T_GEFF,
    T_TWIST_FRICTION, T_KN, T_KT, T_KROLL, T_GROLL, T_KTWIST, T_GTWIST
};

// A plane wall: a point on it, the unit outward normal, the active box,
// the wall velocity and its material index.
struct WallP {
    double p[3], nrm[3], lo[3], hi[3], vel[3];
    int mat;
};

struct SysParams {
    int kind;            // 0 DEM, 1 LJ
    int precision;       // 0 fp64, 1 mixed
    int contact_model, adhesion_model, rolling_model, twisting_model;
    int touch_only;      // DEM without a JKR pull-off range (no pair acts beyond r_i + r_j)
    int p0, n, npad;     // particle segment
    int b0, nb;          // first particle block; blocks holding the n particles
    int ncb;             // cell blocks of the system's cell segment
    // periodic axes (fixed axes: no images, no wrap) and plane walls
    int per[3];
    int nwall;
    WallP walls[MDG_MAX_WALLS];
    // Langevin ([langevin]): drag gamma, noise kT, seed of the counter-based stream
    int lv;
    double lv_gamma, lv_kT;
    unsigned long long lv_seed;
    int c0, ncell;       // ext-cell segment
    int nc[3];           // interior cells per axis
    int ext[3];          // extended grid (interior + 2*layers)
    int sl[3];           // ghost layers per side
    int win[3];          // enumeration half-width in interior cells
    int build_mode;      // list build: 0 warp per bin, 1 warp per particle, 2 thread per particle
    double lo[3], hi[3], L[3];
    double bin[3], inv_bin[3], origin[3];
    double max_cutoff, stencil_cut_sq;
    unsigned int stencil_bits[32];  // offsets in [-sl, sl]^3 that pass the stencil distance test
    float pre_cut2;      // fp32 prefilter radius^2 for the list build (conservative)
    float band_rel;      // relative error bound of the hi-only fp32 r^2 in the list build
    float ucut2f;        // fp32 copy of uniform_cutoff_sq
    float sf2f;          // fp32 copy of sf2
    float Lh[3], Ll[3];  // two-float split of the box lengths
    // fixed-point geometry of mixed LJ systems: u = (x - lo) 2^32 / L mod 2^32,
    // so an int32 difference is the minimum-image separation in units of L / 2^32
    double uinv[3];      // 2^32 / L
    float uscale[3];     // L / 2^32
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
    int rb_next;         // rebuild requests for the next step, gathered by the fused
                         // final + initial kernel while this step's flags are still read
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
    // mixed LJ systems: 32-bit fixed-point positions (x, y, z, 0) written by the
    // integrator every step and read by the pair kernel; lbpu: same at the last build
    uint4* posu;
    uint4* lbpu;
    // per-particle virial (6 x P) when any system accumulates it
    double* vir;
    // reductions
    double* blkpart;   // [nblocks][8]
    const int* blk_sys;   // particle block -> system
    const int* cblk_sys;  // cell block -> system (-1 past the systems' cells)
    const int* cblk0;     // first cell block of each system
    int* csum;            // particles per cell block (k_cells -> k_scan, cleared there)
    int* cbase;           // first particle of each cell block (k_scan -> k_cellscan)
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
    // the run map's blocks split by particle kind (ascending): the force
    // kernels of one kind launch over its blocks only
    const int* blk_run_kind[2];  // [0] DEM, [1] LJ
    int nrun_kind[2];
    // Rebuild work list, written on the device by k_rb_plan when a step
    // rebuilds: the systems that sort or rebuild, with prefix offsets of their
    // particle blocks and cell blocks (rb_poff / rb_coff have rb_n + 1 entries).
    // The rebuild kernels walk these virtual blocks with grid-stride loops.
    int* rb_sys;
    int* rb_poff;
    int* rb_coff;
    int* rb_n;
    // Mixed DEM contexts: per system, the particles that have list partners
    // (indices within the system, at the system's particle offset), built at
    // each rebuild; the force kernel visits only these.
    int* dem_wl;
    int* dem_wl_n;
    // Mixed DEM contexts: the particles (absolute indices, all systems) whose
    // rows hold a touching pair this step, appended by the screening pass and
    // consumed by the contact pass; dem_cl_n = {count, blocks done}, cleared
    // by the contact pass's last block.
    int* dem_cl;
    int* dem_cl_n;
    const SysParams* sp;
    SysState* ss;
    const double* mat;
    const float* matf;   // fp32 copy of the material tables (mixed path)
    int nsys;
    int nblocks;
    long long P;       // total padded particles
    int hist_any;      // history arrays allocated
    int lj_multi;      // some LJ system has a multi-type pair table (nmat > 1)
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

// 32-bit fixed-point position of a mixed LJ particle: round((x - lo) 2^32 / L)
// modulo 2^32 per axis.  Differences wrap like the periodic box, so
// (int)(u_j - u_i) * L / 2^32 is the minimum-image separation whenever it is
// below L / 2 (the list cutoff is), with ~L 2^-33 quantisation.
__device__ __forceinline__ uint4 fixed_pos(const SysParams& sp, const double4& x) {
    return make_uint4((unsigned int)__double2ll_rn((x.x - sp.lo[0]) * sp.uinv[0]),
                      (unsigned int)__double2ll_rn((x.y - sp.lo[1]) * sp.uinv[1]),
                      (unsigned int)__double2ll_rn((x.z - sp.lo[2]) * sp.uinv[2]), 0u);
}

__device__ __forceinline__ float3 fixed_sep(const SysParams& sp, const uint4& uj, const uint4& ui) {
    return make_float3((float)(int)(uj.x - ui.x) * sp.uscale[0], (float)(int)(uj.y - ui.y) * sp.uscale[1],
                       (float)(int)(uj.z - ui.z) * sp.uscale[2]);
}

// Conversions between double and float by integer operations.  On GB300 the
// hardware conversions run on the FP64 pipe at the rate of a DFMA (measured
// ~0.6 T/s, against ~36 T/s for FFMA), so the mixed integrators convert with
// these instead.  dbl_to_flt rounds to nearest (ties away from zero), so
// its errors carry no bias that a long run could accumulate (|x| < 2^-126
// gives a signed zero, finite |x| >= 2^128 infinity); flt_to_dbl is exact for
// normal floats (subnormals give zero).  Both keep infinities and NaNs, so a
// non-finite force still reaches the integrators' NaN check.
__device__ __forceinline__ float dbl_to_flt(double x) {
    const unsigned long long raw = (unsigned long long)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(raw >> 32) & 0x80000000u;
    if (((raw >> 52) & 0x7ffull) == 0x7ffull)  // inf or NaN
        return __uint_as_float(sign | 0x7f800000u | ((raw << 12) ? 0x400000u : 0u));
    // half of the 29 dropped mantissa bits; a carry moves into the exponent
    const unsigned long long b = raw + (1ull << 28);
    const int e = (int)((b >> 52) & 0x7ffull) - 896;  // rebias 1023 -> 127
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned int)e << 23) | ((unsigned int)(b >> 29) & 0x7fffffu));
}
__device__ __forceinline__ double flt_to_dbl(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)sign);
    const unsigned long long de = e == 255u ? 0x7ffull : (unsigned long long)(e + 896u);
    return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// -x when flip, else x: a sign-bit flip (no FP64 multiply by -1)
__device__ __forceinline__ double neg_if(double x, bool flip) {
    return __longlong_as_double(__double_as_longlong(x) ^ (flip ? (long long)0x8000000000000000ull : 0ll));
}
// x != 0 for a double, by its bits (no FP64 compare)
__device__ __forceinline__ bool dbl_nonzero(double x) {
    return ((unsigned long long)__double_as_longlong(x) << 1) != 0ull;
}

// Geometry copy of a mixed-precision particle after its drift (tx, ty, tz)
// to the fp64 position x, and its rebuild request (decide_rebuild's per-atom
// tests, neighbor.rs:564-674) when test is set: displacement since the last
// build in fp32 against a threshold 1e-5 on the safe side, every / check,
// and (reference policy) leaving the box on a periodic axis.  LJ systems keep
// the fixed-point copy (box exit tested on the fp64 position, as the
// reference does); DEM systems the two-float copy.
__device__ __forceinline__ bool mixed_drift(const Dev& d, const SysParams& sp, long long i, const double4& x,
                                            float tx, float ty, float tz, bool test, int ssb) {
    if (sp.kind == 1) {
        const uint4 u = fixed_pos(sp, x);
        d.posu[i] = u;
        if (!test) return false;
        const float3 m = fixed_sep(sp, u, d.lbpu[i]);
        bool nd = m.x * m.x + m.y * m.y + m.z * m.z > sp.disp_thr2f;
        if (sp.every > 0) nd = (sp.check && nd) || ssb >= sp.every;
        if (!nd && sp.policy == 0)
            nd = (sp.per[0] && (x.x < sp.lo[0] || x.x >= sp.hi[0])) || (sp.per[1] && (x.y < sp.lo[1] || x.y >= sp.hi[1])) ||
                 (sp.per[2] && (x.z < sp.lo[2] || x.z >= sp.hi[2]));
        return nd;
    }
    // advance the two-float copy by the same drift in fp32 (exact two-sum,
    // renormalised); it is re-derived from the fp64 position at every build
    float4 ph = d.pos2[2 * i], pl = d.pos2[2 * i + 1];
    two_float_add(ph.x, pl.x, tx);
    two_float_add(ph.y, pl.y, ty);
    two_float_add(ph.z, pl.z, tz);
    d.pos2[2 * i] = ph;
    d.pos2[2 * i + 1] = pl;
    if (!test) return false;
    const float4 bh = d.lbp2[2 * i], bl = d.lbp2[2 * i + 1];
    const float dx = (ph.x - bh.x) + (pl.x - bl.x);
    const float dy = (ph.y - bh.y) + (pl.y - bl.y);
    const float dz = (ph.z - bh.z) + (pl.z - bl.z);
    bool nd = dx * dx + dy * dy + dz * dz > sp.disp_thr2f;
    if (sp.every > 0) nd = (sp.check && nd) || ssb >= sp.every;
    if (!nd && sp.policy == 0) {
        const float rx = ph.x + pl.x, ry = ph.y + pl.y, rz = ph.z + pl.z;
        nd = (sp.per[0] && (rx < 0.f || rx >= sp.Lh[0])) || (sp.per[1] && (ry < 0.f || ry >= sp.Lh[1])) ||
             (sp.per[2] && (rz < 0.f || rz >= sp.Lh[2]));
    }
    return nd;
}

// The device view restricted to the running blocks of one particle kind
// (kind 0 DEM, 1 LJ): for kernels that only act on that kind.
__host__ __forceinline__ Dev kind_view(const Dev& d, int kind) {
    Dev k = d;
    k.blk_run = d.blk_run_kind[kind];
    k.nrun = d.nrun_kind[kind];
    return k;
}

// ---- kernel launchers (mdg_kernels_fp64.cu / mdg_kernels_mixed.cu) ----------
// Each returns the number of kernels it launched on `st`.
// Per-system reduction of NV doubles.  Every block of the system (gb = its
// global particle block id) contributes a partial; the last block to arrive sums the partials with a fixed order
// (strided lanes, then a fixed tree) so the result is deterministic.  Returns
// true on the last block (all threads), totals valid in out[] on thread 0.
// Every block of the system must be in the launch.
template <int NV>
__device__ bool system_reduce(const Dev& d, int s, int gb, const double (&v)[NV], double (&out)[NV]) {
    static_assert(NV <= 8, "blkpart holds 8 doubles per block");
    __shared__ double sh[NV][BLK];
    __shared__ int last;
    const SysParams& sp = d.sp[s];
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; k++) sh[k][t] = v[k];
    __syncthreads();
    for (int w = BLK / 2; w > 0; w >>= 1) {
        if (t < w) {
#pragma unroll
            for (int k = 0; k < NV; k++) sh[k][t] = sh[k][t] + sh[k][t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) d.blkpart[(size_t)gb * 8 + k] = sh[k][0];
        __threadfence();
        unsigned int prev = atomicAdd(&d.ss[s].red_count, 1u);
        last = (prev == (unsigned)(sp.nb - 1)) ? 1 : 0;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = 0.0;
    for (int b = t; b < sp.nb; b += BLK) {
        const volatile double* p = d.blkpart + (size_t)(sp.b0 + b) * 8;
#pragma unroll
        for (int k = 0; k < NV; k++) acc[k] = acc[k] + p[k];
    }
#pragma unroll
    for (int k = 0; k < NV; k++) sh[k][t] = acc[k];
    __syncthreads();
    for (int w = BLK / 2; w > 0; w >>= 1) {
        if (t < w) {
#pragma unroll
            for (int k = 0; k < NV; k++) sh[k][t] = sh[k][t] + sh[k][t + w];
        }
        __syncthreads();
    }
    if (t == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = sh[k][0];
        d.ss[s].red_count = 0;
    }
    return true;
}

__device__ __forceinline__ int vload(const int* p) { return *((const volatile int*)p); }

// The system sorts its particles this step / rebuilds its list this step.
__device__ __forceinline__ bool do_sort(const SysState* st) {
    return sys_active(st) && (vload(&st->rebuild) || vload(&st->periodic_sort));
}
__device__ __forceinline__ bool do_rebuild(const SysState* st) {
    return sys_active(st) && (vload(&st->rebuild) || (vload(&st->periodic_sort) && vload(&st->nonid)));
}

// End of a step for one system (one thread, after the system's last block
// of the final kernel): nh_post_final's half step of p_xi from the kinetic
// energy (m|v|^2 summed in ke2), then the next nh_pre_initial's half step
// (its compute_ke sees the same velocities) and its exp scale
// (md_thermostat/src/lib.rs:254-353); the virial; the rebuild / sort
// counters, step, step budget and history buffer flip; the overlap limit
// (contact.rs:197-216).
__device__ __forceinline__ void step_end(const SysParams& sp, SysState* st, double ke2, const double* vir,
                                         int integrate) {
    const double ke = 0.5 * ke2;
    const double dt = sp.dt;
    st->ke = ke;
    if (sp.nh && integrate) {
        const double post = st->p_xi_pre + (dt / 2.0) * (2.0 * ke - sp.nh_ndof * sp.nh_T);
        st->p_xi_post = post;
        const double pre = post + (dt / 2.0) * (2.0 * ke - sp.nh_ndof * sp.nh_T);
        st->p_xi_pre = pre;
        st->nh_scale = exp(-dt / 2.0 * pre / sp.nh_Q);
    }
    if (vir)
        for (int q = 0; q < 6; q++) st->vir[q] = vir[q];
    const bool rb = do_rebuild(st);
    if (integrate) {
        st->steps_since_build = rb ? 0 : st->steps_since_build + 1;
        st->sort_counter = st->periodic_sort ? 0 : st->sort_counter + 1;
        st->step += 1;
        if (st->remaining > 0) st->remaining -= 1;
    } else if (rb) {
        st->steps_since_build = 0;
    }
    if (sp.kind == 0) st->hcur ^= 1;  // the force kernel wrote the other history buffer
    if (rb) st->nbuilds += 1;
    if (st->overlap > 500) st->status |= ST_OVERLAP;
    st->overlap = 0;
    st->rebuild = 0;
    st->periodic_sort = 0;
    st->nonid = 0;
}

// True on the last block of system s to arrive (all threads); the block
// counter is reset there.  Every block of the system must call it.
__device__ __forceinline__ bool system_last(const Dev& d, int s) {
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(&d.ss[s].red_count, 1u);
        last = prev == (unsigned)(d.sp[s].nb - 1);
        if (last) d.ss[s].red_count = 0;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Langevin force at PostForce (langevin_force, md_thermostat/src/lib.rs:529-564):
// f += -gamma m v + sqrt(2 gamma m kT / dt) N(0,1) per component, with m the
// mass and v the half-kicked velocity.  N(0,1) by the Box-Muller cos branch
// of normal_sample (lib.rs:571-577) from two uniforms of a counter-based
// stream: the SplitMix64 finaliser (Steele, Lea & Flood 2014) over (seed,
// step, tag, draw), so each particle's noise is independent of its storage
// order.
__device__ __forceinline__ unsigned long long lv_mix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double lv_uniform(unsigned long long seed, long long step, unsigned int tag, int draw) {
    const unsigned long long h =
        lv_mix(seed + lv_mix((unsigned long long)step * 0x9e3779b97f4a7c15ull + lv_mix(((unsigned long long)tag << 3) + draw)));
    return (double)(h >> 11) * 0x1.0p-53;
}
__device__ __forceinline__ double lv_normal(unsigned long long seed, long long step, unsigned int tag, int k) {
    const double u1 = lv_uniform(seed, step, tag, 2 * k), u2 = lv_uniform(seed, step, tag, 2 * k + 1);
    return sqrt(-2.0 * log(fmax(u1, 1e-300))) * cos(6.283185307179586 * u2);
}
__device__ __forceinline__ void langevin_add(const Dev& d, const SysParams& sp, const SysState* st, long long i,
                                             const double4& v, double4& f) {
    const double drag = sp.lv_gamma * d.mass[i];
    const double rc = sqrt(2.0 * drag * sp.lv_kT / sp.dt);
    const unsigned int tag = d.tag[i];
    const long long step = st->step;
    f.x = f.x - drag * v.x;
    f.y = f.y - drag * v.y;
    f.z = f.z - drag * v.z;
    f.x = f.x + rc * lv_normal(sp.lv_seed, step, tag, 0);
    f.y = f.y + rc * lv_normal(sp.lv_seed, step, tag, 1);
    f.z = f.z + rc * lv_normal(sp.lv_seed, step, tag, 2);
    d.frc[i] = f;  // the reference changes atoms.force: the next initial kick uses it
}

// entry k of a prefix array off[0..n] with off[k] <= v < off[k+1]
__device__ __forceinline__ int rb_find(const int* off, int n, int v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Grid-stride loop over the particle blocks (s = system, lb = block within
// it) or cell blocks of the rebuild work list.
#define RB_FOR_PARTICLE_BLOCKS(BODY)                                  \
    {                                                                 \
        const int rbn_ = *d.rb_n;                                     \
        const int tot_ = d.rb_poff[rbn_];                             \
        for (int v_ = blockIdx.x; v_ < tot_; v_ += gridDim.x) {       \
            const int k_ = rb_find(d.rb_poff, rbn_, v_);              \
            BODY(d, d.rb_sys[k_], v_ - d.rb_poff[k_]);                \
        }                                                             \
    }
#define RB_FOR_PARTICLE_SUBS(BODY, SUB)                               \
    {                                                                 \
        const int rbn_ = *d.rb_n;                                     \
        const int tot_ = d.rb_poff[rbn_] * (SUB);                     \
        for (int v_ = blockIdx.x; v_ < tot_; v_ += gridDim.x) {       \
            const int pv_ = v_ % d.rb_poff[rbn_];                     \
            const int k_ = rb_find(d.rb_poff, rbn_, pv_);             \
            BODY(d, d.rb_sys[k_], pv_ - d.rb_poff[k_], v_ / d.rb_poff[rbn_]); \
        }                                                             \
    }
#define RB_FOR_CELL_BLOCKS(BODY, SUB)                                 \
    {                                                                 \
        const int rbn_ = *d.rb_n;                                     \
        const int tot_ = d.rb_coff[rbn_] * (SUB);                     \
        for (int v_ = blockIdx.x; v_ < tot_; v_ += gridDim.x) {       \
            const int cv_ = v_ / (SUB);                               \
            const int k_ = rb_find(d.rb_coff, rbn_, cv_);             \
            BODY(d, d.rb_sys[k_], cv_ - d.rb_coff[k_], v_ % (SUB));   \
        }                                                             \
    }

int launch_initial(const Dev& d, cudaStream_t st);
int launch_initial_mixed(const Dev& d, cudaStream_t st, int nh_only = 0, const long long* loop = nullptr);
int launch_step_mixed(const Dev& d, const long long* loop, cudaStream_t st);
int launch_walls(const Dev& d, int integrating, cudaStream_t st);
int launch_rdf(const Dev& d, int s, const SysParams& sp, float4* posf, double r_max, int nbins,
               unsigned long long* counts, cudaStream_t st);
int launch_msd_ref(const Dev& d, int s, int n, double* ref, cudaStream_t st);
int launch_msd(const Dev& d, int s, int n, const double* ref, double* part, cudaStream_t st);
int rdf_max_bins();
int launch_rebuild_tail_mixed(const Dev& d, int has_dem, cudaStream_t st);
int launch_final_mixed(const Dev& d, cudaStream_t st, int integrate);
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

// ---- seeded initial conditions on the device (mdg_generate.cu)
constexpr int GEN_MAX_TYPES = 8;
struct FccArgs {
    int nc[3];
    double lo[3], a[3];
    double temperature, skin;
    uint64_t seed;
    int ntypes;
    double frac[GEN_MAX_TYPES];   // cumulative type thresholds
    double tmass[GEN_MAX_TYPES];  // mass of each type (index 0 for a single type)
};
struct GasArgs {
    long long n;
    double rmin, rmax, density, sep;
    int inset, vel_mode;
    double speed;
    uint32_t material;
    uint64_t seed, max_proposals;
};
struct GasPlacement {
    double4* placed = nullptr;  // (x, y, z, r) in acceptance order
    size_t count = 0;
    uint64_t proposals = 0;
    double rmin = 0.0, rmax = 0.0;  // of the placed radii
    void release(cudaStream_t s);
};
// FCC lattice into system segment p (p.n atoms); velocities fixed to T
int gen_fcc(const Dev& d, const SysParams& p, const FccArgs& f, cudaStream_t s, long long* launches);
// parallel RSA into scratch (MDG_ERR_ARG when fewer than n fit in the proposal budget)
int gen_gas_place(const GasArgs& a, const double box_lo[3], const double box_hi[3], cudaStream_t s,
                  GasPlacement* out, long long* launches);
// placed spheres and their velocities into system segment p
int gen_gas_write(const Dev& d, const SysParams& p, const GasArgs& a, const GasPlacement& gp, cudaStream_t s,
                  long long* launches);

}  // namespace mdg
