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
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// LJ 12-6 in FP32 with compensated per-particle sums (same list, same owner
// frames as the FP64 kernel).
template <int TPP>
__global__ void __launch_bounds__(BLK, 8) k_lj_mixed(Dev d) {
    const int pb = blockIdx.x / TPP;
    const int sub = blockIdx.x % TPP;
    const int s = d.blk_sys[pb];
    const SysParams& sp = d.sp[s];
    if (sp.kind != 1) return;
    const int lane = threadIdx.x % TPP;
    const int li = (pb - sp.b0) * BLK + sub * (BLK / TPP) + threadIdx.x / TPP;
    const bool act = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    Kahan kx, ky, kz;
    if (act) {
        const float4 hi = d.pos2[2 * i];
        const float4 lo = d.pos2[2 * i + 1];
        const int nn = d.nnum[i];
        const long long base = sp.lst0 + li;
        const float lj1 = sp.lj1f, lj2 = sp.lj2f;
        const float cut2 = sp.lj_cut2f;
        const float Lh0 = sp.Lh[0], Lh1 = sp.Lh[1], Lh2 = sp.Lh[2];
        const float Ll0 = sp.Ll[0], Ll1 = sp.Ll[1], Ll2 = sp.Ll[2];
        // U entries in flight per lane: list loads first, then the gathers, then
        // the arithmetic, so each lane keeps U independent load chains open
        constexpr int U = 4;
        for (int k0 = lane; k0 < nn; k0 += U * TPP) {
            uint32_t e[U];
            float4 hj[U], lj[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int k = k0 + u * TPP;
                e[u] = k < nn ? __ldg(d.nlist + base + (long long)k * sp.npad) : 0xffffffffu;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                const long long j = sp.p0 + (e[u] != 0xffffffffu ? (e[u] & IDX_MASK) : 0u);
                hj[u] = __ldg(d.pos2 + 2 * j);
                lj[u] = __ldg(d.pos2 + 2 * j + 1);
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (e[u] == 0xffffffffu) continue;
                const uint32_t code = e[u] >> IDX_BITS;
                const int sc = (int)(code >= 27u ? code - 27u : code);
                // d_i = x_j(+s) - x_i for owner and partner entries alike: the
                // force on i is -fpair d_i either way
                float dx, dy, dz;
                if (sc == 13) {  // no periodic image (most entries)
                    dx = (hj[u].x - hi.x) + (lj[u].x - lo.x);
                    dy = (hj[u].y - hi.y) + (lj[u].y - lo.y);
                    dz = (hj[u].z - hi.z) + (lj[u].z - lo.z);
                } else {
                    const int sx = sc / 9 - 1, sy = (sc / 3) % 3 - 1, sz = sc % 3 - 1;
                    dx = two_float_sep(hj[u].x, lj[u].x, hi.x, lo.x, sx, Lh0, Ll0);
                    dy = two_float_sep(hj[u].y, lj[u].y, hi.y, lo.y, sy, Lh1, Ll1);
                    dz = two_float_sep(hj[u].z, lj[u].z, hi.z, lo.z, sz, Lh2, Ll2);
                }
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 >= cut2) continue;
                const float r2inv = __frcp_rn(r2);
                const float r6inv = r2inv * r2inv * r2inv;
                const float fpair = r2inv * r6inv * (lj1 * r6inv - lj2);
                kx.add(-fpair * dx);
                ky.add(-fpair * dy);
                kz.add(-fpair * dz);
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
    if (act && lane == 0) d.frc[i] = make_double4(kx.value(), ky.value(), kz.value(), 0.0);
}

int launch_force_mixed(const Dev& d, int hcur, int has_lj, int has_dem, int tpp, cudaStream_t st) {
    (void)hcur;
    (void)has_dem;
    int n = 0;
    if (has_lj) {
        switch (tpp) {
            case 2: k_lj_mixed<2><<<d.nblocks * 2, BLK, 0, st>>>(d); break;
            case 4: k_lj_mixed<4><<<d.nblocks * 4, BLK, 0, st>>>(d); break;
            case 8: k_lj_mixed<8><<<d.nblocks * 8, BLK, 0, st>>>(d); break;
            default: k_lj_mixed<1><<<d.nblocks, BLK, 0, st>>>(d); break;
        }
        n++;
    }
    return n;
}

}  // namespace mdg
