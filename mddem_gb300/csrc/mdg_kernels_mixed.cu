// mdg_kernels_mixed.cu -- mixed-precision force kernels.
//
// Positions stay FP64 in the integrator; the pair kernels read a two-float
// copy relative to the box corner, x - lo = hi + lo_part (pos2 pairs),
// written by the integrator each step.  Pair separations are formed as
// (x_j,hi - x_i,hi) + (x_j,lo - x_i,lo), with a periodic shift applied to the
// coordinate that sits next to the crossed face so that the hi-part
// difference stays exact (Sterbenz); the separation then carries ~1e-7
// relative error.  Force arithmetic is FP32; per-particle sums use Kahan
// compensation (Kahan 1965) and are handed to the FP64 integrator as doubles.
#include "mdg_internal.cuh"

namespace mdg {

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return flt_to_dbl(s) - flt_to_dbl(c); }
};

// LJ 12-6 in FP32 with compensated per-particle sums (same list, same owner
// frames as the FP64 kernel).  Geometry from the 32-bit fixed-point copy: one
// 16-byte gather per list entry, and the wrapped integer difference is the
// minimum-image separation, so the entry's image code is not needed.  The
// separation carries the fixed-point quantisation (L 2^-33) plus one fp32
// rounding (2^-24 relative) and the fp32 scale (2^-24 relative, the same for
// every pair).
// Minimum resident blocks per SM asked of ptxas for k_lj_mixed (a compile-time
// tuning knob; 8 caps it at 64 registers).
#ifndef MDG_LJ_MINB
#define MDG_LJ_MINB 8
#endif
// VIR: systems with `virial` also write their per-particle virial (the
// owner-entry sum of d_a f_b, VirialStress::add_pair, virial.rs:61-68; fp32
// per lane, summed in fp64 at the thermo query); a separate instantiation so
// the common path keeps its registers.  MT: systems with a multi-type pair
// table gather the partner's type and look up lj1, lj2 and the squared cutoff
// (pair_table.get(ti, tj), fp32 copies); also its own instantiation.
// The LJ pair force is cut off without a shift, so it jumps by f(rc) at the
// cutoff (about 1e-3 of a particle's pair-force sum).  The fp32 separation
// can fall on the other side of rc than the fp64 one for a pair within
// rounding of it; such pairs (fp32 r^2 within LJ_CUT_BAND of rc^2, about 10x
// the fp32 separation's error) are decided with the fp64 path's own
// arithmetic (k_lj_fp64: the owner frame, image shift, fma sum), so both
// paths count the same pairs: k_lj_mixed leaves them out of its main loop and
// decides them in a second pass over the row, run only by a lane that met
// one.  At LJ 256k about two pairs lie that close to the cutoff in any step.
constexpr float LJ_CUT_BAND = 2e-6f;

__device__ __noinline__ bool lj_within_fp64(const Dev& d, const SysParams& sp, long long i, uint32_t e, double cut2) {
    const long long j = sp.p0 + (e & IDX_MASK);
    const uint32_t code = e >> IDX_BITS;
    const bool own = code >= 27u;
    const int sc = (int)(own ? code - 27u : code);
    const int s3[3] = {sc / 9 - 1, (sc / 3) % 3 - 1, sc % 3 - 1};
    const double4 xi = d.pos[i], xj = d.pos[j];
    const double a[3] = {own ? xj.x : xi.x, own ? xj.y : xi.y, own ? xj.z : xi.z};
    const double b[3] = {own ? xi.x : xj.x, own ? xi.y : xj.y, own ? xi.z : xj.z};
    double dd[3];
    for (int q = 0; q < 3; q++) {
        const int sq = own ? s3[q] : -s3[q];
        const double img = sq > 0 ? __dadd_rn(a[q], sp.L[q]) : (sq < 0 ? __dadd_rn(a[q], -sp.L[q]) : a[q]);
        dd[q] = __dsub_rn(img, b[q]);
    }
    const double r2 = fma(dd[0], dd[0], fma(dd[1], dd[1], __dmul_rn(dd[2], dd[2])));
    return r2 < cut2;
}

// One LJ pair's force on the particle (fp32, compensated sums) and, on owner
// entries of systems with `virial`, its virial terms.
template <bool VIR>
__device__ __forceinline__ void lj_pair_add(float dx, float dy, float dz, float r2, float lj1, float lj2, bool owner_vir,
                                            Kahan& kx, Kahan& ky, Kahan& kz, float& w0, float& w1, float& w2,
                                            float& w3, float& w4, float& w5) {
    const float r2inv = __frcp_rn(r2);
    const float r6inv = r2inv * r2inv * r2inv;
    const float fpair = r2inv * r6inv * (lj1 * r6inv - lj2);
    kx.add(-fpair * dx);
    ky.add(-fpair * dy);
    kz.add(-fpair * dz);
    if (VIR && owner_vir) {  // owner entry: the reference's half-list pair
        const float px = -fpair * dx, py = -fpair * dy, pz = -fpair * dz;
        w0 += dx * px;
        w1 += dy * py;
        w2 += dz * pz;
        w3 += dx * py;
        w4 += dx * pz;
        w5 += dy * pz;
    }
}

template <int TPP, bool VIR, bool MT>
__global__ void __launch_bounds__(BLK, MDG_LJ_MINB) k_lj_mixed(Dev d) {
    const int pb = d.blk_run[blockIdx.x / TPP];
    const int sub = blockIdx.x % TPP;
    const int s = d.blk_sys[pb];
    const SysParams& sp = d.sp[s];
    if (sp.kind != 1 || !sys_active(d.ss + s)) return;
    const int lane = threadIdx.x % TPP;
    const int li = (pb - sp.b0) * BLK + sub * (BLK / TPP) + threadIdx.x / TPP;
    const bool act = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    Kahan kx, ky, kz;
    const bool vir = VIR && sp.virial;
    float w0 = 0.f, w1 = 0.f, w2 = 0.f, w3 = 0.f, w4 = 0.f, w5 = 0.f;
    if (act) {
        const uint4 ui = d.posu[i];
        const int nn = d.nnum[i];
        const long long base = sp.lst0 + li;
        const float lj1_ = sp.lj1f, lj2_ = sp.lj2f;
        const float cut2_ = sp.lj_cut2f;
        const bool mt = MT && sp.nmat > 1;
        const long long tq = (long long)sp.nmat * sp.nmat;
        const long long trow = mt ? sp.mat0 + (long long)d.type[i] * sp.nmat : 0;
        const float s0 = sp.uscale[0], s1 = sp.uscale[1], s2 = sp.uscale[2];
        bool near = false;  // a pair within fp32 rounding of the cutoff
        const float in2_ = cut2_ * (1.f - LJ_CUT_BAND), out2_ = cut2_ * (1.f + LJ_CUT_BAND);
        // U entries in flight per lane: list loads first, then the gathers, then
        // the arithmetic, so each lane keeps U independent load chains open
        constexpr int U = 4;
        for (int k0 = lane; k0 < nn; k0 += U * TPP) {
            uint32_t e[U];
            uint4 uj[U];
            uint32_t tj[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int k = k0 + u * TPP;
                e[u] = k < nn ? __ldg(d.nlist + base + (long long)k * sp.npad) : 0xffffffffu;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const long long j = sp.p0 + (e[u] != 0xffffffffu ? (e[u] & IDX_MASK) : 0u);
                uj[u] = __ldg(d.posu + j);
                if (MT && mt) tj[u] = __ldg(d.type + j);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (e[u] == 0xffffffffu) continue;
                // d_i = x_j(+image) - x_i for owner and partner entries alike:
                // the force on i is -fpair d_i either way
                const float dx = (float)(int)(uj[u].x - ui.x) * s0;
                const float dy = (float)(int)(uj[u].y - ui.y) * s1;
                const float dz = (float)(int)(uj[u].z - ui.z) * s2;
                const float r2 = dx * dx + dy * dy + dz * dz;
                float lj1 = lj1_, lj2 = lj2_, cut2 = cut2_;
                if (MT && mt) {
                    const long long o = trow + tj[u];
                    lj1 = __ldg(d.matf + o + TL_LJ1 * tq);
                    lj2 = __ldg(d.matf + o + TL_LJ2 * tq);
                    cut2 = __ldg(d.matf + o + TL_CUT2 * tq);
                }
                // one compare for the pairs well inside the cutoff; those within
                // the band around it are decided after the loop
                const float in2 = (MT && mt) ? cut2 * (1.f - LJ_CUT_BAND) : in2_;
                if (r2 >= in2) {
                    near |= r2 <= ((MT && mt) ? cut2 * (1.f + LJ_CUT_BAND) : out2_);
                    continue;
                }
                lj_pair_add<VIR>(dx, dy, dz, r2, lj1, lj2, vir && (e[u] >> IDX_BITS) >= 27u, kx, ky, kz, w0, w1, w2,
                                 w3, w4, w5);
            }
        }
        if (near) {
            // rare: this lane's pairs within fp32 rounding of the cutoff, counted
            // when the fp64 arithmetic of k_lj_fp64 counts them
            for (int k = lane; k < nn; k += TPP) {
                const uint32_t e = __ldg(d.nlist + base + (long long)k * sp.npad);
                const long long j = sp.p0 + (e & IDX_MASK);
                const uint4 uj = __ldg(d.posu + j);
                const float dx = (float)(int)(uj.x - ui.x) * s0;
                const float dy = (float)(int)(uj.y - ui.y) * s1;
                const float dz = (float)(int)(uj.z - ui.z) * s2;
                const float r2 = dx * dx + dy * dy + dz * dz;
                float lj1 = lj1_, lj2 = lj2_, cut2 = cut2_;
                double c64 = sp.lj_cut2;
                if (MT && mt) {
                    const long long o = trow + __ldg(d.type + j);
                    lj1 = __ldg(d.matf + o + TL_LJ1 * tq);
                    lj2 = __ldg(d.matf + o + TL_LJ2 * tq);
                    cut2 = __ldg(d.matf + o + TL_CUT2 * tq);
                    c64 = __ldg(d.mat + o + TL_CUT2 * tq);
                }
                if (!(r2 >= cut2 * (1.f - LJ_CUT_BAND) && r2 <= cut2 * (1.f + LJ_CUT_BAND)) ||
                    !lj_within_fp64(d, sp, i, e, c64))
                    continue;
                lj_pair_add<VIR>(dx, dy, dz, r2, lj1, lj2, vir && (e >> IDX_BITS) >= 27u, kx, ky, kz, w0, w1, w2, w3,
                                 w4, w5);
            }
        }
    }
    if (TPP > 1) {
        // combine the lanes' compensated sums: sum the values, then the corrections
#pragma unroll
        for (int o = TPP / 2; o > 0; o >>= 1) {
            const float sx_ = __shfl_down_sync(0xffffffffu, kx.s, o, TPP), cx_ = __shfl_down_sync(0xffffffffu, kx.c, o, TPP);
            const float sy_ = __shfl_down_sync(0xffffffffu, ky.s, o, TPP), cy_ = __shfl_down_sync(0xffffffffu, ky.c, o, TPP);
            const float sz_ = __shfl_down_sync(0xffffffffu, kz.s, o, TPP), cz_ = __shfl_down_sync(0xffffffffu, kz.c, o, TPP);
            kx.add(sx_);
            kx.c += cx_;
            ky.add(sy_);
            ky.c += cy_;
            kz.add(sz_);
            kz.c += cz_;
        }
    }
    if (VIR && vir && TPP > 1) {
#pragma unroll
        for (int o = TPP / 2; o > 0; o >>= 1) {
            w0 += __shfl_down_sync(0xffffffffu, w0, o, TPP);
            w1 += __shfl_down_sync(0xffffffffu, w1, o, TPP);
            w2 += __shfl_down_sync(0xffffffffu, w2, o, TPP);
            w3 += __shfl_down_sync(0xffffffffu, w3, o, TPP);
            w4 += __shfl_down_sync(0xffffffffu, w4, o, TPP);
            w5 += __shfl_down_sync(0xffffffffu, w5, o, TPP);
        }
    }
    if (act && lane == 0) {
        d.frc[i] = make_double4(kx.value(), ky.value(), kz.value(), 0.0);
        if (VIR && vir) {
            const double half = sp.newton ? 1.0 : 0.5;
            d.vir[0 * d.P + i] = (double)w0 * half;
            d.vir[1 * d.P + i] = (double)w1 * half;
            d.vir[2 * d.P + i] = (double)w2 * half;
            d.vir[3 * d.P + i] = (double)w3 * half;
            d.vir[4 * d.P + i] = (double)w4 * half;
            d.vir[5 * d.P + i] = (double)w5 * half;
        }
    }
}

// ----------------------------------------------------------------------------
// Hertz-Mindlin / Hooke contact, mixed precision.
//
// Geometry: the overlap delta = (r1 + r2) - d cancels two millimetre-scale
// numbers, so it is formed as ((r1 + r2)^2 - d^2) / ((r1 + r2) + d) with both
// squares in double-float arithmetic (error-free fp32 transformations:
// Knuth two-sum, two-product via fma; Dekker 1971), from two-float separations
// and two-float radii.  Everything downstream (normal, damping, tangential
// force, torques) is fp32; the tangential / rolling / twisting spring
// integration (rotation into the tangent plane, v_t dt, Coulomb rescale) is
// fp64; per-particle sums are Kahan-compensated.  Each pair is evaluated in
// its owner's frame on both sides, so forces stay exactly antisymmetric.
// Same laws and branches as hm_pair (contact.rs:103-615, 622-990).
// ----------------------------------------------------------------------------
// The error-free transformations use round-to-nearest intrinsics: ptxas may
// otherwise contract a product with the sum that consumes it into one FMA
// (its choice depends on scheduling and register pressure), which keeps the
// rounded product in the error term but not in the sum and breaks exactness.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = fmaf(a, b, -p);
}

// separation component (x_p + s L) - x_o as an unevaluated sum dh + dl
__device__ __forceinline__ void sep_df(float hp, float lp, float ho, float lo_, int s, float Lh, float Ll, float& dh,
                                       float& dl) {
    float a = hp, b = ho, al = lp, bl = lo_;
    if (s > 0) {  // shift the owner (next to the crossed face) by -L
        float t, te;
        two_sum(ho, -Lh, t, te);
        b = t;
        bl = lo_ - Ll + te;
    } else if (s < 0) {
        float t, te;
        two_sum(hp, -Lh, t, te);
        a = t;
        al = lp - Ll + te;
    }
    float e;
    two_sum(a, -b, dh, e);
    dl = (al - bl) + e;
}

struct Kahan3 {
    Kahan x, y, z;
    __device__ __forceinline__ void add(float a, float b, float c) {
        x.add(a);
        y.add(b);
        z.add(c);
    }
};

__device__ __forceinline__ float mtf(const Dev& d, const SysParams& sp, int tab, int a, int b) {
    return d.matf[sp.mat0 + ((long long)tab * sp.nmat + a) * sp.nmat + b];
}

struct PairMixed {
    float fn[3], ft[3], ti[3], tj[3], tr[3], tw[3];
    double spring[7];
    bool hit, tang, overlap;
};

// o = owner, p = partner; geometry as double-float separation (dxh + dxl ...)
__device__ void hm_pair_mixed(const Dev& d, const SysParams& sp, const float (&dh)[3], const float (&dl)[3],
                              float r1h, float r1l, float r2h, float r2l, const double4& v_i, const double4& v_j,
                              const double4& w_i, const double4& w_j, int mi, int mj, uint32_t tag_i, uint32_t tag_j,
                              const double* stored, PairMixed& o) {
    const float kPi = 3.14159265358979f;
    const float SQRT_5_3 = 0.9128709291752768f;
    const float EPS = 1e-30f;
    const bool hooke = sp.contact_model == 1;
    const bool use_dmt = sp.adhesion_model == 1;
    o.hit = o.tang = o.overlap = false;
    // d^2 in double-float
    float Sh = 0.f, Sl = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float p, e;
        two_prod(dh[k], dh[k], p, e);
        float t, te;
        two_sum(Sh, p, t, te);
        Sh = t;
        // (dh + dl)^2 = dh^2 + dl (2 dh + dl): the dl^2 term matters in
        // large boxes, where dl (the lo parts of coordinates near L) reaches
        // ~1e-8 L and (r1 + r2)^2 - d^2 of a grazing contact is small
        Sl += te + e + dl[k] * (2.f * dh[k] + dl[k]);
    }
    // r1 + r2 in double-float
    float sh, se;
    two_sum(r1h, r2h, sh, se);
    const float sl = se + r1l + r2l;
    const float sum_r = sh + sl;
    const float surface_energy = hooke ? 0.f : mtf(d, sp, T_SURFACE, mi, mj);
    const float r_eff = (r1h * r2h) / sum_r;
    const float e_eff = mtf(d, sp, T_EEFF, mi, mj);
    float pulloff = 0.f;
    if (!hooke && surface_energy > 0.f && !use_dmt) {
        const float g = surface_energy;
        pulloff = cbrtf(kPi * kPi * g * g * r_eff / (4.f * e_eff * e_eff));
    }
    // (sum_r + pulloff)^2 - d^2 and (sum_r)^2 - d^2, double-float
    float ih, il;
    two_sum(sh, pulloff, ih, il);
    il += sl;
    float qh, qe;
    two_prod(ih, ih, qh, qe);
    float gap_h, gap_e;
    two_sum(qh, -Sh, gap_h, gap_e);
    const float range2 = gap_h + (gap_e + qe + 2.f * ih * il - Sl);
    if (!(range2 > 0.f)) return;  // dist_sq >= interaction_r^2
    const float dist_sq = Sh + Sl;
    const float distance = sqrtf(dist_sq);
    if (distance == 0.f) return;
    float ph, pe;
    two_prod(sh, sh, ph, pe);
    float ch, ce;
    two_sum(ph, -Sh, ch, ce);
    const float diff = ch + (ce + pe + 2.f * sh * sl - Sl);  // (r1 + r2)^2 - d^2
    const float r_min = fminf(r1h, r2h);
    const float delta = fminf(diff / (sum_r + distance), 0.5f * r_min);
    if (hooke && delta <= 0.f) return;
    if (delta > 0.f && distance / sum_r < 0.90f) o.overlap = true;
    if (!hooke && delta <= 0.f && surface_energy <= 0.f) return;
    o.hit = true;
    const float inv_dist = 1.f / distance;
    const float nx = (dh[0] + dl[0]) * inv_dist, ny = (dh[1] + dl[1]) * inv_dist, nz = (dh[2] + dl[2]) * inv_dist;
    const float g_eff = mtf(d, sp, T_GEFF, mi, mj);
    const float inv_m_i = dbl_to_flt(v_i.w), inv_m_j = dbl_to_flt(v_j.w);
    const float m_r = 1.f / (inv_m_i + inv_m_j);
    const float beta = mtf(d, sp, T_BETA, mi, mj);
    const float mu = mtf(d, sp, T_FRICTION, mi, mj);
    const float mu_r = mtf(d, sp, T_ROLL_FRICTION, mi, mj);
    const float mu_tw = mtf(d, sp, T_TWIST_FRICTION, mi, mj);
    const float cohesion_energy = mtf(d, sp, T_COHESION, mi, mj);
    const bool jkr_adhesion_only = !hooke && surface_energy > 0.f && !use_dmt && delta <= 0.f;
    float s_n = 0.f, k_n = 0.f, k_t = 0.f, kn = 0.f, kt = 0.f, gamma_n = 0.f;
    if (hooke) {
        kn = mtf(d, sp, T_KN, mi, mj);
        kt = mtf(d, sp, T_KT, mi, mj);
        gamma_n = 2.f * beta * sqrtf(kn * m_r);
    } else if (delta > 0.f) {
        const float sdr = sqrtf(delta * r_eff);
        s_n = 2.f * e_eff * sdr;
        k_n = 4.f / 3.f * e_eff * sdr;
        k_t = 8.f * g_eff * sdr;
    }
    const float r1 = r1h, r2 = r2h;
    const float oix = dbl_to_flt(w_i.x), oiy = dbl_to_flt(w_i.y), oiz = dbl_to_flt(w_i.z);
    const float ojx = dbl_to_flt(w_j.x), ojy = dbl_to_flt(w_j.y), ojz = dbl_to_flt(w_j.z);
    const float r1nx = r1 * nx, r1ny = r1 * ny, r1nz = r1 * nz;
    const float r2nx = r2 * nx, r2ny = r2 * ny, r2nz = r2 * nz;
    // relative contact velocity: translational difference first (cancellation in fp64)
    const float dvx = dbl_to_flt(v_j.x - v_i.x), dvy = dbl_to_flt(v_j.y - v_i.y), dvz = dbl_to_flt(v_j.z - v_i.z);
    const float vrx = dvx + (-ojy * r2nz + ojz * r2ny) - (oiy * r1nz - oiz * r1ny);
    const float vry = dvy + (-ojz * r2nx + ojx * r2nz) - (oiz * r1nx - oix * r1nz);
    const float vrz = dvz + (-ojx * r2ny + ojy * r2nx) - (oix * r1ny - oiy * r1nx);
    const float v_n = vrx * nx + vry * ny + vrz * nz;
    float f_n_mag;
    if (hooke) {
        if (cohesion_energy > 0.f) f_n_mag = kn * delta - gamma_n * v_n - cohesion_energy * kPi * delta * r_eff;
        else f_n_mag = fmaxf(kn * delta - gamma_n * v_n, 0.f);
    } else if (surface_energy > 0.f && use_dmt) {
        f_n_mag = k_n * delta - 2.f * beta * SQRT_5_3 * sqrtf(s_n * m_r) * v_n - 2.f * kPi * surface_energy * r_eff;
    } else if (surface_energy > 0.f) {
        const float f_adh = 1.5f * kPi * surface_energy * r_eff;
        if (jkr_adhesion_only) f_n_mag = -f_adh;
        else f_n_mag = k_n * delta - 2.f * beta * SQRT_5_3 * sqrtf(s_n * m_r) * v_n - f_adh;
    } else if (cohesion_energy > 0.f) {
        f_n_mag = k_n * delta - 2.f * beta * SQRT_5_3 * sqrtf(s_n * m_r) * v_n - cohesion_energy * kPi * delta * r_eff;
    } else {
        f_n_mag = fmaxf(k_n * delta - 2.f * beta * SQRT_5_3 * sqrtf(s_n * m_r) * v_n, 0.f);
    }
    o.fn[0] = f_n_mag * nx;
    o.fn[1] = f_n_mag * ny;
    o.fn[2] = f_n_mag * nz;
    if (jkr_adhesion_only) return;
    o.tang = true;
    const float vtx = vrx - v_n * nx, vty = vry - v_n * ny, vtz = vrz - v_n * nz;
    const bool flip = !(tag_i < tag_j);  // canonical (lower-tag) frame of the stored springs
    const double dt = sp.dt;
    const double ndx = flt_to_dbl(nx), ndy = flt_to_dbl(ny), ndz = flt_to_dbl(nz);
    // spring integration in fp64
    double sx = neg_if(stored[0], flip), sy = neg_if(stored[1], flip), sz = neg_if(stored[2], flip);
    const double sdn = sx * ndx + sy * ndy + sz * ndz;
    sx -= sdn * ndx;
    sy -= sdn * ndy;
    sz -= sdn * ndz;
    sx = fma(flt_to_dbl(vtx), dt, sx);
    sy = fma(flt_to_dbl(vty), dt, sy);
    sz = fma(flt_to_dbl(vtz), dt, sz);
    const float ktt = hooke ? kt : k_t;
    const float sfx = dbl_to_flt(sx), sfy = dbl_to_flt(sy), sfz = dbl_to_flt(sz);
    const float s_mag = sqrtf(sfx * sfx + sfy * sfy + sfz * sfz);
    const float fts = ktt * s_mag;
    const float ft_max = mu * fabsf(f_n_mag);
    if (fts > ft_max && fts > EPS) {
        const double sc = flt_to_dbl(ft_max / fts);
        sx *= sc;
        sy *= sc;
        sz *= sc;
    }
    const float gamma_t = 2.f * SQRT_5_3 * beta * sqrtf(ktt * m_r);
    float ftx = ktt * dbl_to_flt(sx) - gamma_t * vtx;
    float fty = ktt * dbl_to_flt(sy) - gamma_t * vty;
    float ftz = ktt * dbl_to_flt(sz) - gamma_t * vtz;
    const float ftm = sqrtf(ftx * ftx + fty * fty + ftz * ftz);
    if (ftm > ft_max && ftm > EPS) {
        const float sc = ft_max / ftm;
        ftx *= sc;
        fty *= sc;
        ftz *= sc;
    }
    o.ft[0] = ftx; o.ft[1] = fty; o.ft[2] = ftz;
    o.ti[0] = r1ny * ftz - r1nz * fty; o.ti[1] = r1nz * ftx - r1nx * ftz; o.ti[2] = r1nx * fty - r1ny * ftx;
    o.tj[0] = r2ny * ftz - r2nz * fty; o.tj[1] = r2nz * ftx - r2nx * ftz; o.tj[2] = r2nx * fty - r2ny * ftx;
    // relative spin from the fp64 angular velocities
    const float orx = dbl_to_flt(w_i.x - w_j.x), ory = dbl_to_flt(w_i.y - w_j.y), orz = dbl_to_flt(w_i.z - w_j.z);
    const float odn = orx * nx + ory * ny + orz * nz;
    const float rollx = orx - odn * nx, rolly = ory - odn * ny, rollz = orz - odn * nz;
    double rdx = neg_if(stored[3], flip), rdy = neg_if(stored[4], flip), rdz = neg_if(stored[5], flip);
    double twd = neg_if(stored[6], flip);
    o.tr[0] = o.tr[1] = o.tr[2] = 0.f;
    o.tw[0] = o.tw[1] = o.tw[2] = 0.f;
    if (mu_r > 0.f) {
        const float roll_mag = sqrtf(rollx * rollx + rolly * rolly + rollz * rollz);
        if (sp.rolling_model == 1) {
            const float k_roll = mtf(d, sp, T_KROLL, mi, mj);
            const float g_roll = mtf(d, sp, T_GROLL, mi, mj);
            const double rdn = rdx * ndx + rdy * ndy + rdz * ndz;
            rdx -= rdn * ndx; rdy -= rdn * ndy; rdz -= rdn * ndz;
            rdx = fma(flt_to_dbl(rollx), dt, rdx); rdy = fma(flt_to_dbl(rolly), dt, rdy); rdz = fma(flt_to_dbl(rollz), dt, rdz);
            float tx = -k_roll * dbl_to_flt(rdx) - g_roll * rollx;
            float ty = -k_roll * dbl_to_flt(rdy) - g_roll * rolly;
            float tz = -k_roll * dbl_to_flt(rdz) - g_roll * rollz;
            const float trm = sqrtf(tx * tx + ty * ty + tz * tz);
            const float tau_max = mu_r * fabsf(f_n_mag) * r_eff;
            if (trm > tau_max && trm > EPS) {
                const float sc = tau_max / trm;
                tx *= sc; ty *= sc; tz *= sc;
                if (k_roll > EPS) {
                    rdx = flt_to_dbl((tx + g_roll * rollx) / (-k_roll));
                    rdy = flt_to_dbl((ty + g_roll * rolly) / (-k_roll));
                    rdz = flt_to_dbl((tz + g_roll * rollz) / (-k_roll));
                }
            }
            o.tr[0] = tx; o.tr[1] = ty; o.tr[2] = tz;
        } else if (roll_mag > 1e-30f) {
            const float inv_roll = mu_r * fabsf(f_n_mag) * r_eff / roll_mag;
            o.tr[0] = -inv_roll * rollx; o.tr[1] = -inv_roll * rolly; o.tr[2] = -inv_roll * rollz;
        }
    }
    if (mu_tw > 0.f) {
        const float twist_vel = odn;
        if (sp.twisting_model == 1) {
            const float k_tw = mtf(d, sp, T_KTWIST, mi, mj);
            const float g_tw = mtf(d, sp, T_GTWIST, mi, mj);
            twd = fma(flt_to_dbl(twist_vel), dt, twd);
            float tau_tw = -k_tw * dbl_to_flt(twd) - g_tw * twist_vel;
            const float tau_max = mu_tw * fabsf(f_n_mag) * r_eff;
            if (fabsf(tau_tw) > tau_max) {
                tau_tw = copysignf(1.f, tau_tw) * tau_max;
                if (k_tw > EPS) twd = flt_to_dbl((tau_tw + g_tw * twist_vel) / (-k_tw));
            }
            o.tw[0] = tau_tw * nx; o.tw[1] = tau_tw * ny; o.tw[2] = tau_tw * nz;
        } else if (fabsf(twist_vel) > 1e-30f) {
            const float tau = mu_tw * fabsf(f_n_mag) * r_eff;
            const float sg = twist_vel > 0.f ? -1.f : 1.f;
            o.tw[0] = sg * tau * nx; o.tw[1] = sg * tau * ny; o.tw[2] = sg * tau * nz;
        }
    }
    o.spring[0] = neg_if(sx, flip); o.spring[1] = neg_if(sy, flip); o.spring[2] = neg_if(sz, flip);
    o.spring[3] = neg_if(rdx, flip); o.spring[4] = neg_if(rdy, flip); o.spring[5] = neg_if(rdz, flip);
    o.spring[6] = neg_if(twd, flip);
}

__device__ __forceinline__ bool hist_find_m(const Dev& d, const SysParams& sp, int hc, long long p, int lp, uint32_t t,
                                            double* out) {
    const int n = d.hcnt[hc][p];
    for (int c = 0; c < n; c++) {
        if (d.htag[hc][sp.h0 + (long long)c * sp.npad + lp] == t) {
            for (int q = 0; q < 7; q++) out[q] = d.hval[hc][sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + lp];
            return true;
        }
    }
    return false;
}

// Mixed DEM force, in two passes.
//
// Screen (k_dem_screen): one thread per particle of a system's worklist (the
// particles with listed partners).  With a touch-only contact law a listed
// pair acts only while the spheres overlap, so each partner is tested on the
// two-float separation (dh + dl, ~1e-7 of the distance) against r_i + r_j
// with a 2e-5 margin on the squares.  A particle with no touching partner
// gets its zero force, torque, virial and contact count written here; the
// others are appended to one list for the whole context (warp-aggregated; the
// order does not matter, each particle's force comes from its own row).
// Systems with a pull-off range (JKR) send every worklist particle on.  The
// screen needs few registers, so it runs at full occupancy with many
// partner gathers in flight, where the contact law's registers would not.
//
// Contact (k_dem_contact): a fixed grid walks the list and evaluates the
// contact law on every listed pair of each particle's row, owner frames on
// both sides, Kahan sums; its last block clears the list for the next step.

// True when some listed partner of particle i (row li of its system) may
// overlap it.
__device__ __forceinline__ bool dem_touching(const Dev& d, const SysParams& sp, long long i, int li) {
    const int nn = d.nnum[i];
    const float4 hi = d.pos2[2 * i], lo = d.pos2[2 * i + 1];
    const long long base = sp.lst0 + li;
    for (int k = 0; k < nn; k++) {
        const uint32_t e = d.nlist[base + (long long)k * sp.npad];
        const long long j = sp.p0 + (int)(e & IDX_MASK);
        const uint32_t code = e >> IDX_BITS;
        const int sc = (int)(code >= 27u ? code - 27u : code);
        const float4 hj = d.pos2[2 * j], lj4 = d.pos2[2 * j + 1];
        // |(x_j + s L) - x_i|: the same distance in either owner frame
        float dh, dl;
        sep_df(hj.x, lj4.x, hi.x, lo.x, sc / 9 - 1, sp.Lh[0], sp.Ll[0], dh, dl);
        const float x = dh + dl;
        sep_df(hj.y, lj4.y, hi.y, lo.y, (sc / 3) % 3 - 1, sp.Lh[1], sp.Ll[1], dh, dl);
        const float y = dh + dl;
        sep_df(hj.z, lj4.z, hi.z, lo.z, sc % 3 - 1, sp.Lh[2], sp.Ll[2], dh, dl);
        const float z = dh + dl;
        const float rs = hi.w + hj.w;
        if (x * x + y * y + z * z <= rs * rs * 1.00002f) return true;
    }
    return false;
}

__global__ void __launch_bounds__(BLK) k_dem_screen(Dev d) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (sp.kind != 0 || !sys_active(st)) return;  // uniform over the block
    const int k = (gb - sp.b0) * BLK + threadIdx.x;
    bool contact = false;
    long long i = 0;
    if (k < d.dem_wl_n[s]) {
        const int li = d.dem_wl[sp.p0 + k];
        i = (long long)sp.p0 + li;
        contact = !sp.touch_only || dem_touching(d, sp, i, li);
        if (!contact) {
            d.frc[i] = make_double4(0.0, 0.0, 0.0, 0.0);
            d.trq[i] = make_double4(0.0, 0.0, 0.0, 0.0);
            d.hcnt[st->hcur ^ 1][i] = 0;
            if (sp.virial)
                for (int q = 0; q < 6; q++) d.vir[q * d.P + i] = 0.0;
        }
    }
    const unsigned int m = __ballot_sync(0xffffffffu, contact);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(d.dem_cl_n, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (contact) d.dem_cl[base + __popc(m & ((1u << lane) - 1u))] = (int)i;
}

// Lanes per contact particle in the contact pass: lane e of a group evaluates
// row entries e, e + CG, e + 2 CG, ... of its particle, so a particle's pairs
// run side by side instead of one after another in one thread.
constexpr int CG = 8;

// Compensated (s, c) sum over the CG lanes of a group by a fixed shuffle
// tree (deterministic order); the total lands on the group's first lane.
__device__ __forceinline__ void group_sum(Kahan& k) {
#pragma unroll
    for (int o = CG / 2; o > 0; o >>= 1) {
        const float so = __shfl_down_sync(0xffffffffu, k.s, o, CG);
        const float co = __shfl_down_sync(0xffffffffu, k.c, o, CG);
        k.add(so);
        k.c += co;
    }
}

// Minimum resident blocks per SM asked of ptxas for k_dem_contact (a
// compile-time tuning knob: 4 caps it at 128 registers).
#ifndef MDG_DEM_MINB
#define MDG_DEM_MINB 4
#endif
constexpr int DEM_CONTACT_GRID = 152 * MDG_DEM_MINB;

// The contact law over the rows of the listed particles: force, torque, the
// next history buffer (owner tangential contacts in row order), the
// large-overlap count and (VIR) the owner-side virial sum of d_a f_b
// (hertz_mindlin_contact_force's add_pair, contact.rs:559-569; fp32 pair
// terms summed in fp64).  Each warp takes 32 / CG listed particles, warps
// numbered across blocks first so the list spreads over every SM.
template <bool VIR>
__global__ void __launch_bounds__(BLK, MDG_DEM_MINB) k_dem_contact(Dev d) {
    const int n = *((const volatile int*)d.dem_cl_n);
    const int lane = threadIdx.x & 31, el = lane % CG, sub = lane / CG;
    const unsigned int gmask = ((1u << CG) - 1u) << (sub * CG);
    const int nwarps = gridDim.x * (BLK / 32);
    for (int w = (int)(threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x; w * (32 / CG) < n; w += nwarps) {
        const int kk = w * (32 / CG) + sub;
        const bool has = kk < n;
        long long i = 0;
        int s = 0, nn = 0;
        if (has) {
            i = d.dem_cl[kk];
            s = d.blk_sys[i / BLK];
            nn = d.nnum[i];
        }
        int maxnn = nn;  // uniform over the warp: every lane runs the same chunks
        for (int o = 16; o > 0; o >>= 1) maxnn = max(maxnn, __shfl_xor_sync(0xffffffffu, maxnn, o));
        const SysParams& sp = d.sp[s];
        SysState* st = d.ss + s;
        const int li = (int)(i - sp.p0);
        const int hcur = st->hcur;
        const int hn = hcur ^ 1;
        float4 hi = make_float4(0, 0, 0, 0), lo = hi;
        double4 vi = make_double4(0, 0, 0, 0), wi = vi;
        int ti_ = 0;
        uint32_t tag_i = 0;
        if (has) {
            hi = d.pos2[2 * i];
            lo = d.pos2[2 * i + 1];
            vi = d.vel[i];
            wi = d.omg[i];
            ti_ = (int)d.type[i];
            tag_i = d.tag[i];
        }
        const long long base = sp.lst0 + li;
        const bool vir = VIR && sp.virial;
        const float vs = sp.newton ? 1.f : 0.5f;
        Kahan3 F, T;
        double V[6] = {0, 0, 0, 0, 0, 0};
        int nh = 0, nover = 0;
        for (int k0 = 0; k0 < maxnn; k0 += CG) {
            const int k = k0 + el;
            bool wh = false;  // this lane stores a history entry
            uint32_t tag_j = 0;
            PairMixed o;
            if (has && k < nn) {
                const uint32_t e = d.nlist[base + (long long)k * sp.npad];
                const int lj = (int)(e & IDX_MASK);
                const long long j = sp.p0 + lj;
                const uint32_t code = e >> IDX_BITS;
                const bool own = code >= 27u;
                const int sc = (int)(own ? code - 27u : code);
                const int sx = sc / 9 - 1, sy = (sc / 3) % 3 - 1, sz = sc % 3 - 1;
                const float4 hj = d.pos2[2 * j], lj4 = d.pos2[2 * j + 1];
                float dh[3], dl[3];
                if (own) {
                    sep_df(hj.x, lj4.x, hi.x, lo.x, sx, sp.Lh[0], sp.Ll[0], dh[0], dl[0]);
                    sep_df(hj.y, lj4.y, hi.y, lo.y, sy, sp.Lh[1], sp.Ll[1], dh[1], dl[1]);
                    sep_df(hj.z, lj4.z, hi.z, lo.z, sz, sp.Lh[2], sp.Ll[2], dh[2], dl[2]);
                } else {
                    // owner frame: owner j, partner i's image -s
                    sep_df(hi.x, lo.x, hj.x, lj4.x, -sx, sp.Lh[0], sp.Ll[0], dh[0], dl[0]);
                    sep_df(hi.y, lo.y, hj.y, lj4.y, -sy, sp.Lh[1], sp.Ll[1], dh[1], dl[1]);
                    sep_df(hi.z, lo.z, hj.z, lj4.z, -sz, sp.Lh[2], sp.Ll[2], dh[2], dl[2]);
                }
                const float rs = hi.w + hj.w;
                const float x = dh[0] + dl[0], y = dh[1] + dl[1], z = dh[2] + dl[2];
                // spheres clearly apart: no force, skip the partner's state and history
                if (!sp.touch_only || x * x + y * y + z * z <= rs * rs * 1.00002f) {
                    const double4 vj = d.vel[j];
                    const double4 wj = d.omg[j];
                    const int tj_ = (int)d.type[j];
                    tag_j = d.tag[j];
                    double stored[7] = {0, 0, 0, 0, 0, 0, 0};
                    if (own) {
                        hist_find_m(d, sp, hcur, i, li, tag_j, stored);
                        hm_pair_mixed(d, sp, dh, dl, hi.w, lo.w, hj.w, lj4.w, vi, vj, wi, wj, ti_, tj_, tag_i, tag_j,
                                      stored, o);
                        if (o.hit) {
                            F.add(-o.fn[0], -o.fn[1], -o.fn[2]);
                            if (o.overlap) nover++;
                            if (vir) {
                                // owner frame: separation owner -> partner, the owner's pair force
                                const float fx = (-o.fn[0] + (o.tang ? o.ft[0] : 0.f)) * vs;
                                const float fy = (-o.fn[1] + (o.tang ? o.ft[1] : 0.f)) * vs;
                                const float fz = (-o.fn[2] + (o.tang ? o.ft[2] : 0.f)) * vs;
                                V[0] += (double)(x * fx); V[1] += (double)(y * fy); V[2] += (double)(z * fz);
                                V[3] += (double)(x * fy); V[4] += (double)(x * fz); V[5] += (double)(y * fz);
                            }
                            if (o.tang) {
                                F.add(o.ft[0], o.ft[1], o.ft[2]);
                                T.add(o.ti[0] + o.tr[0] + o.tw[0], o.ti[1] + o.tr[1] + o.tw[1],
                                      o.ti[2] + o.tr[2] + o.tw[2]);
                                wh = true;
                            }
                        }
                    } else {
                        hist_find_m(d, sp, hcur, j, lj, tag_i, stored);
                        hm_pair_mixed(d, sp, dh, dl, hj.w, lj4.w, hi.w, lo.w, vj, vi, wj, wi, tj_, ti_, tag_j, tag_i,
                                      stored, o);
                        if (o.hit) {
                            F.add(o.fn[0], o.fn[1], o.fn[2]);
                            if (o.tang) {
                                F.add(-o.ft[0], -o.ft[1], -o.ft[2]);
                                T.add(o.tj[0] - o.tr[0] - o.tw[0], o.tj[1] - o.tr[1] - o.tw[1],
                                      o.tj[2] - o.tr[2] - o.tw[2]);
                            }
                        }
                    }
                }
            }
            // history slots in row order within the group
            const unsigned int bal = __ballot_sync(0xffffffffu, wh) & gmask;
            if (wh) {
                const int slot = nh + __popc(bal & ((1u << lane) - 1u));
                if (slot < sp.hcap) {
                    d.htag[hn][sp.h0 + (long long)slot * sp.npad + li] = tag_j;
                    for (int q = 0; q < 7; q++)
                        d.hval[hn][sp.h0 * 7 + (long long)(slot * 7 + q) * sp.npad + li] = o.spring[q];
                }
            }
            nh += __popc(bal);
        }
        group_sum(F.x); group_sum(F.y); group_sum(F.z);
        group_sum(T.x); group_sum(T.y); group_sum(T.z);
#pragma unroll
        for (int o = CG / 2; o > 0; o >>= 1) {
            nover += __shfl_down_sync(0xffffffffu, nover, o, CG);
            if (VIR)
                for (int q = 0; q < 6; q++) V[q] += __shfl_down_sync(0xffffffffu, V[q], o, CG);
        }
        if (has && el == 0) {
            if (nh > sp.hcap) {
                atomicOr(&st->status, ST_HIST_OVF);
                nh = sp.hcap;
            }
            d.hcnt[hn][i] = nh;
            if (nover) atomicAdd(&st->overlap, nover);
            d.frc[i] = make_double4(F.x.value(), F.y.value(), F.z.value(), 0.0);
            d.trq[i] = make_double4(T.x.value(), T.y.value(), T.z.value(), 0.0);
            if (vir)
                for (int q = 0; q < 6; q++) d.vir[q * d.P + i] = V[q];
        }
    }
    // every block has read the count: the last one to finish clears the list
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd((unsigned int*)d.dem_cl_n + 1, 1u) == gridDim.x - 1) {
            d.dem_cl_n[0] = 0;
            d.dem_cl_n[1] = 0;
        }
    }
}

// Per-particle pieces of the mixed integrators, shared by the separate
// initial / final kernels and the fused step kernel (so both give the same
// bits).  FP64 arithmetic is kept to the Verlet kicks and the drift (FMA
// form), the spin kicks and the quaternion sum; conversions go through
// dbl_to_flt / flt_to_dbl (integer operations), and the rotation increment is
// fp32.  A DEM particle-step costs 22 FP64-pipe operations.

// dt as an unevaluated fp32 sum hi + lo (one FP64 subtraction)
__device__ __forceinline__ float2 dt_split(double dt) {
    const float h = dbl_to_flt(dt);
    return make_float2(h, dbl_to_flt(dt - flt_to_dbl(h)));
}

// drift x += v dt (FMA) and the fp32 displacement for the geometry copy of
// the particle, v (rounded to fp32) times the two-float dt: unbiased, ~1e-7
// relative
__device__ __forceinline__ void drift_mixed(double4& x, const double4& v, double dt, float2 dts, float& tx, float& ty,
                                            float& tz) {
    x.x = fma(v.x, dt, x.x);
    x.y = fma(v.y, dt, x.y);
    x.z = fma(v.z, dt, x.z);
    const float vx = dbl_to_flt(v.x), vy = dbl_to_flt(v.y), vz = dbl_to_flt(v.z);
    tx = fmaf(vx, dts.x, vx * dts.y);
    ty = fmaf(vy, dts.x, vy * dts.y);
    tz = fmaf(vz, dts.x, vz * dts.y);
}

// initial_rotation's quaternion update (rotational.rs:59-84): q' = dq * q
// with dq = (cos(angle/2), sin(angle/2) w / |w|), angle = |w| dt.  The
// increment q' - q = (c1, a) * q, c1 = cos(angle/2) - 1 = -2 sin^2(angle/4)
// (full relative precision for small angles), is formed in fp32 from an
// fp32 copy of q and added to the fp64 q: its error is ~1e-7 of the
// increment, about 1e-7 x angle/2 per step.
__device__ __forceinline__ void rotate_mixed(const Dev& d, long long i, const double4& w, float dtf) {
    const float wx = dbl_to_flt(w.x), wy = dbl_to_flt(w.y), wz = dbl_to_flt(w.z);
    const float om = sqrtf(wx * wx + wy * wy + wz * wz);
    const float angle = om * dtf;
    if (!(angle > 1e-14f)) return;
    const float half = 0.5f * angle;
    const float sq = sinf(0.5f * half);
    const float c1 = -2.f * sq * sq;
    const float k = sinf(half) / om;
    const float a1 = wx * k, a2 = wy * k, a3 = wz * k;
    const double4 q = d.quat[i];
    const float qw = dbl_to_flt(q.x), qx = dbl_to_flt(q.y), qy = dbl_to_flt(q.z), qz = dbl_to_flt(q.w);
    const float rw = c1 * qw - (a1 * qx + a2 * qy + a3 * qz);
    const float rx = c1 * qx + (a1 * qw + a2 * qz - a3 * qy);
    const float ry = c1 * qy + (a2 * qw + a3 * qx - a1 * qz);
    const float rz = c1 * qz + (a3 * qw + a1 * qy - a2 * qx);
    d.quat[i] = make_double4(q.x + flt_to_dbl(rw), q.y + flt_to_dbl(rx), q.z + flt_to_dbl(ry), q.w + flt_to_dbl(rz));
}

// Initial integration of the mixed path: the same update as k_initial (NH
// scale, half kick, drift, two-float drift copy, fp32 rebuild test, half
// spin kick, quaternion update) with FP64 state for x, v, omega and q, FMA
// contraction, and the rotation of initial_rotation (rotational.rs:59-84)
// by rotate_mixed.
//
// nh_only: only thermostatted systems (the multi-step graph's fused kernel
// below does the others), and nothing on the first iteration of a launch
// (loop[0] == loop[1]), where the fused kernel does every system.
__global__ void __launch_bounds__(BLK) k_initial_mixed(Dev d, int nh_only, const long long* loop) {
    if (nh_only && loop[0] == loop[1]) return;  // uniform over the grid
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    const bool live = sys_active(st) && (!nh_only || sp.nh);
    const bool act = live && li < sp.n;
    const long long i = (long long)sp.p0 + li;
    const double dt = sp.dt;
    const double scale = sp.nh ? st->nh_scale : 1.0;
    if (li == 0 && live)
        st->periodic_sort =
            (sp.policy == 0 && sp.sort_every > 0 && st->sort_counter + 1 >= sp.sort_every) ? 1 : 0;
    const int already = *((const volatile int*)&st->rebuild);
    int need = 0;
    if (act) {
        double4 v = d.vel[i];
        const double4 f = d.frc[i];
        double4 x = d.pos[i];
        if (sp.nh) {
            v.x *= scale;
            v.y *= scale;
            v.z *= scale;
        }
        const double h = 0.5 * dt * v.w;
        v.x = fma(h, f.x, v.x);
        v.y = fma(h, f.y, v.y);
        v.z = fma(h, f.z, v.z);
        const float2 dts = dt_split(dt);
        const float dtf = dts.x;
        float tx, ty, tz;
        drift_mixed(x, v, dt, dts, tx, ty, tz);
        d.vel[i] = v;
        d.pos[i] = x;
        need = mixed_drift(d, sp, i, x, tx, ty, tz, !already, st->steps_since_build);
        if (sp.kind == 0) {
            double4 w = d.omg[i];
            if (dbl_nonzero(w.w)) {
                const double4 tq = d.trq[i];
                const double hw = 0.5 * dt * w.w;
                w.x = fma(hw, tq.x, w.x);
                w.y = fma(hw, tq.y, w.y);
                w.z = fma(hw, tq.z, w.z);
                rotate_mixed(d, i, w, dtf);
                d.omg[i] = w;
            }
        }
    }
    if (__any_sync(0xffffffffu, need) && (threadIdx.x & 31) == 0) atomicOr(&st->rebuild, 1);
    if (d.use_cond) {
        // grid-wide last block: open the rebuild branch of the step graph only
        // when some running system rebuilds or sorts
        __shared__ int last;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            last = atomicAdd(d.grid_ctr, 1u) == (unsigned)(gridDim.x - 1);
        }
        __syncthreads();
        if (last && threadIdx.x == 0) {
            __threadfence();
            unsigned int any = 0;
            for (int q = 0; q < d.nrun_sys; q++) {
                const SysState* o = d.ss + d.run_sys[q];
                if (sys_active(o))
                    any |= (unsigned)(*((const volatile int*)&o->rebuild) | *((const volatile int*)&o->periodic_sort));
            }
            *d.grid_ctr = 0;
            if (any) d.stat_ctr[0] += 1;
            cudaGraphSetConditional((cudaGraphConditionalHandle)d.cond, any ? 1u : 0u);
        }
    }
}

// After a DEM system's list build: particles with no listed partner get zero
// force, torque and contact-history count in both buffers (nothing writes
// them again until the next build); the others are appended to the system's
// worklist (warp-aggregated; any order: each particle's force is computed
// independently, so results do not depend on it).
__device__ __forceinline__ void dem_wl_block(const Dev& d, int s, int lb) {
    const SysParams& sp = d.sp[s];
    if (sp.kind != 0 || !do_rebuild(d.ss + s)) return;
    const int li = lb * BLK + threadIdx.x;
    const bool in = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    // with walls every particle is visited each step (the wall kernel adds to
    // the force the pair kernel writes)
    const bool has = in && (d.nnum[i] > 0 || sp.nwall > 0);
    if (in && !has) {
        d.frc[i] = make_double4(0.0, 0.0, 0.0, 0.0);
        d.trq[i] = make_double4(0.0, 0.0, 0.0, 0.0);
        d.hcnt[0][i] = 0;
        d.hcnt[1][i] = 0;
        if (sp.virial)
            for (int q = 0; q < 6; q++) d.vir[q * d.P + i] = 0.0;
    }
    const unsigned int m = __ballot_sync(0xffffffffu, has);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(&d.dem_wl_n[s], __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (has) d.dem_wl[sp.p0 + base + __popc(m & ((1u << lane) - 1u))] = li;
}
__global__ void __launch_bounds__(BLK) k_dem_wl(Dev d) RB_FOR_PARTICLE_BLOCKS(dem_wl_block)

int launch_rebuild_tail_mixed(const Dev& d, int has_dem, cudaStream_t st) {
    if (!has_dem) return 0;
    constexpr int CAP = 152 * 16;
    k_dem_wl<<<d.nrun < CAP ? d.nrun : CAP, BLK, 0, st>>>(d);
    return 1;
}

// final_integration + final_rotation (mddem_verlet/src/lib.rs:136-154,
// rotational.rs:87-100) and nh_post_final for the mixed path: FP64 state with
// FMA; the kinetic-energy reduction only for thermostatted systems (mixed
// contexts carry no virial).
__global__ void __launch_bounds__(BLK) k_final_mixed(Dev d, int integrate) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (!sys_active(st)) return;  // every block of a frozen system returns
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    const bool act = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    const double dt = sp.dt;
    double ke2 = 0.0;
    int bad = 0;
    if (act) {
        double4 f = d.frc[i];
        double4 v = d.vel[i];
        if (integrate && sp.lv) langevin_add(d, sp, st, i, v, f);
        if (integrate) {
            const double h = 0.5 * dt * v.w;
            v.x = fma(h, f.x, v.x);
            v.y = fma(h, f.y, v.y);
            v.z = fma(h, f.z, v.z);
            if (sp.nh) {
                const double scale = st->nh_scale;
                v.x *= scale;
                v.y *= scale;
                v.z *= scale;
            }
            d.vel[i] = v;
        }
        if (sp.nh) ke2 = d.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z);
        if (sp.kind == 0 && integrate) {
            double4 w = d.omg[i];
            if (dbl_nonzero(w.w)) {
                const double4 tq = d.trq[i];
                const double hw = 0.5 * dt * w.w;
                w.x = fma(hw, tq.x, w.x);
                w.y = fma(hw, tq.y, w.y);
                w.z = fma(hw, tq.z, w.z);
                d.omg[i] = w;
            }
        }
        const int ex = 0x7ff00000;
        bad = ((__double2hiint(v.x) & ex) == ex) | ((__double2hiint(v.y) & ex) == ex) |
              ((__double2hiint(v.z) & ex) == ex);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&st->status, ST_NAN);
    bool last;
    double tot = 0.0;
    if (sp.nh) {
        const double v1[1] = {ke2};
        double o1[1];
        last = system_reduce<1>(d, s, gb, v1, o1);
        tot = o1[0];
    } else {
        last = system_last(d, s);
    }
    if (last && threadIdx.x == 0) step_end(sp, st, tot, nullptr, integrate);
}

int launch_final_mixed(const Dev& d, cudaStream_t st, int integrate) {
    k_final_mixed<<<d.nrun, BLK, 0, st>>>(d, integrate);
    return 1;
}

// One iteration of the multi-step graph, mixed path: the final half of the
// previous step (k_final_mixed's update, step bookkeeping) fused with the
// initial half of this step (k_initial_mixed's update, rebuild test) in one
// pass over the particle arrays -- 424 instead of 648 bytes per DEM particle.
// The arithmetic is the same FMA sequence as the two kernels, so the state is
// bitwise identical.  loop = {iterations left, iterations of this launch}:
// the first iteration has no previous step to finish (the state is at a step
// boundary), and the launch's last step is finished by k_final_mixed after
// the loop.  Thermostatted systems get only the final half here: their
// initial half needs the system's kinetic energy after it, so
// k_initial_mixed (nh_only) follows.  A system whose step budget runs out with
// the finished step is not started again.
__global__ void __launch_bounds__(BLK) k_step_mixed(Dev d, const long long* loop) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    const long long i = (long long)sp.p0 + li;
    const double dt = sp.dt;
    const float2 dts = dt_split(dt);
    const float dtf = dts.x;
    const bool first = loop[0] == loop[1];
    // read before this system's last block updates the bookkeeping
    const long long rem = *((volatile const long long*)&st->remaining);
    const bool was = rem != 0;
    const bool fin = !first && was;
    const long long rem_after = (fin && rem > 0) ? rem - 1 : rem;
    const bool ini = rem_after != 0 && !(fin && sp.nh);
    int ssb = 0;
    if (ini && sp.every > 0) ssb = fin ? (do_rebuild(st) ? 0 : st->steps_since_build + 1) : st->steps_since_build;
    double ke2 = 0.0;
    int bad = 0, need = 0;
    if (li < sp.n && (fin || ini)) {
        double4 v = d.vel[i];
        double4 f = d.frc[i];
        const double h = 0.5 * dt * v.w;
        if (fin && sp.lv) langevin_add(d, sp, st, i, v, f);
        if (fin) {
            v.x = fma(h, f.x, v.x);
            v.y = fma(h, f.y, v.y);
            v.z = fma(h, f.z, v.z);
            if (sp.nh) {
                const double scale = st->nh_scale;
                v.x *= scale;
                v.y *= scale;
                v.z *= scale;
                ke2 = d.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z);
            }
            const int ex = 0x7ff00000;
            bad = ((__double2hiint(v.x) & ex) == ex) | ((__double2hiint(v.y) & ex) == ex) |
                  ((__double2hiint(v.z) & ex) == ex);
        }
        if (ini) {
            if (sp.nh) {  // first iteration only (fin && nh excludes ini)
                const double scale = st->nh_scale;
                v.x *= scale;
                v.y *= scale;
                v.z *= scale;
            }
            v.x = fma(h, f.x, v.x);
            v.y = fma(h, f.y, v.y);
            v.z = fma(h, f.z, v.z);
            double4 x = d.pos[i];
            float tx, ty, tz;
            drift_mixed(x, v, dt, dts, tx, ty, tz);
            d.pos[i] = x;
            need = mixed_drift(d, sp, i, x, tx, ty, tz, true, ssb);
        }
        d.vel[i] = v;
        if (sp.kind == 0) {
            double4 w = d.omg[i];
            if (dbl_nonzero(w.w)) {
                const double4 tq = d.trq[i];
                const double hw = 0.5 * dt * w.w;
                if (fin) {
                    w.x = fma(hw, tq.x, w.x);
                    w.y = fma(hw, tq.y, w.y);
                    w.z = fma(hw, tq.z, w.z);
                }
                if (ini) {
                    w.x = fma(hw, tq.x, w.x);
                    w.y = fma(hw, tq.y, w.y);
                    w.z = fma(hw, tq.z, w.z);
                    rotate_mixed(d, i, w, dtf);
                }
                d.omg[i] = w;
            }
        }
    }
    if (__any_sync(0xffffffffu, need) && (threadIdx.x & 31) == 0) atomicOr(&st->rb_next, 1);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&st->status, ST_NAN);
    if (was) {  // uniform over the system's blocks
        bool last;
        double tot = 0.0;
        if (fin && sp.nh) {
            const double v1[1] = {ke2};
            double o1[1];
            last = system_reduce<1>(d, s, gb, v1, o1);
            tot = o1[0];
        } else {
            last = system_last(d, s);
        }
        if (last && threadIdx.x == 0) {
            if (fin) step_end(sp, st, tot, nullptr, 1);  // clears this step's flags
            if (ini) {
                st->rebuild |= st->rb_next;
                st->periodic_sort =
                    (sp.policy == 0 && sp.sort_every > 0 && st->sort_counter + 1 >= sp.sort_every) ? 1 : 0;
            }
            st->rb_next = 0;
        }
    }
    if (d.use_cond) {
        // grid-wide last block: open the rebuild branch when some running
        // system rebuilds or sorts in the step that starts now
        __shared__ int glast;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            glast = atomicAdd(d.grid_ctr, 1u) == (unsigned)(gridDim.x - 1);
        }
        __syncthreads();
        if (glast && threadIdx.x == 0) {
            __threadfence();
            unsigned int any = 0;
            for (int q = 0; q < d.nrun_sys; q++) {
                const SysState* o = d.ss + d.run_sys[q];
                if (sys_active(o))
                    any |= (unsigned)(*((const volatile int*)&o->rebuild) | *((const volatile int*)&o->periodic_sort));
            }
            *d.grid_ctr = 0;
            if (any) d.stat_ctr[0] += 1;
            cudaGraphSetConditional((cudaGraphConditionalHandle)d.cond, any ? 1u : 0u);
        }
    }
}

int launch_step_mixed(const Dev& d, const long long* loop, cudaStream_t st) {
    k_step_mixed<<<d.nrun, BLK, 0, st>>>(d, loop);
    return 1;
}

int launch_initial_mixed(const Dev& d, cudaStream_t st, int nh_only, const long long* loop) {
    k_initial_mixed<<<d.nrun, BLK, 0, st>>>(d, nh_only, loop);
    return 1;
}


template <bool VIR, bool MT>
void launch_lj_mixed(const Dev& dall, int tpp, cudaStream_t st) {
    const Dev d = kind_view(dall, 1);
    switch (tpp) {
        case 2: k_lj_mixed<2, VIR, MT><<<d.nrun * 2, BLK, 0, st>>>(d); break;
        case 4: k_lj_mixed<4, VIR, MT><<<d.nrun * 4, BLK, 0, st>>>(d); break;
        case 8: k_lj_mixed<8, VIR, MT><<<d.nrun * 8, BLK, 0, st>>>(d); break;
        default: k_lj_mixed<1, VIR, MT><<<d.nrun, BLK, 0, st>>>(d); break;
    }
}

int launch_force_mixed(const Dev& d, int has_lj, int has_dem, int tpp, cudaStream_t st) {
    int n = 0;
    has_dem = has_dem && d.nrun_kind[0] > 0;
    has_lj = has_lj && d.nrun_kind[1] > 0;
    if (has_dem) {
        k_dem_screen<<<d.nrun_kind[0], BLK, 0, st>>>(kind_view(d, 0));
        if (d.vir)
            k_dem_contact<true><<<DEM_CONTACT_GRID, BLK, 0, st>>>(d);
        else
            k_dem_contact<false><<<DEM_CONTACT_GRID, BLK, 0, st>>>(d);
        n += 2;
    }
    if (has_lj) {
        if (d.lj_multi) {  // some system has a multi-type pair table
            if (d.vir)
                launch_lj_mixed<true, true>(d, tpp, st);
            else
                launch_lj_mixed<false, true>(d, tpp, st);
        } else if (d.vir) {  // some system asks for its virial
            launch_lj_mixed<true, false>(d, tpp, st);
        } else {
            launch_lj_mixed<false, false>(d, tpp, st);
        }
        n++;
    }
    return n;
}

}  // namespace mdg
