// mdg_measure.cu -- measurement kernels after the step: radial distribution
// pair counts and mean square displacement (md_measure/src/lib.rs:333-600).
//
// Compiled with -fmad=false: the pair separations, squares and bin indices use
// the reference's arithmetic exactly, so pair counts per bin equal the
// reference's loop on the same positions.
#include <cstdint>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {

constexpr int RDF_TILE = 128;
constexpr int RDF_MAX_BINS = 4096;

// All pairs i < j of one system (the reference's local-local loop,
// lib.rs:379-400): fp32 screen on a float copy of the positions with a
// conservative margin, then the reference's fp64 minimum image, r^2 (no
// fma), sqrt and bin index.  Block histograms in shared memory, then 64-bit
// atomics: integer counts, so the result does not depend on the order.
__global__ void __launch_bounds__(RDF_TILE) k_rdf(const double4* __restrict__ pos, const float4* __restrict__ posf,
                                                  int n, double lx, double ly, double lz, double cut2, double dr,
                                                  float screen2, int nbins, unsigned long long* counts) {
    __shared__ float4 tile[RDF_TILE];
    __shared__ unsigned int hist[RDF_MAX_BINS];
    const int ti = blockIdx.x, tj = blockIdx.y;
    if (tj < ti) return;  // uniform over the block
    for (int b = threadIdx.x; b < nbins; b += RDF_TILE) hist[b] = 0u;
    const int j0 = tj * RDF_TILE;
    const int jl = j0 + threadIdx.x;
    if (jl < n) tile[threadIdx.x] = posf[jl];
    __syncthreads();
    const int i = ti * RDF_TILE + threadIdx.x;
    if (i < n) {
        const float4 fi = posf[i];
        const float flx = (float)lx, fly = (float)ly, flz = (float)lz;
        const double hx = lx * 0.5, hy = ly * 0.5, hz = lz * 0.5;
        double4 xi = make_double4(0, 0, 0, 0);
        bool have_i = false;
        const int jmax = min(RDF_TILE, n - j0);
        for (int t = 0; t < jmax; t++) {
            const int j = j0 + t;
            if (j <= i) continue;
            const float4 fj = tile[t];
            float ax = fabsf(fj.x - fi.x), ay = fabsf(fj.y - fi.y), az = fabsf(fj.z - fi.z);
            ax = fminf(ax, fabsf(ax - flx));
            ay = fminf(ay, fabsf(ay - fly));
            az = fminf(az, fabsf(az - flz));
            if (ax * ax + ay * ay + az * az > screen2) continue;
            if (!have_i) {
                xi = pos[i];
                have_i = true;
            }
            const double4 xj = pos[j];
            double dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
            if (dx > hx) dx -= lx; else if (dx < -hx) dx += lx;
            if (dy > hy) dy -= ly; else if (dy < -hy) dy += ly;
            if (dz > hz) dz -= lz; else if (dz < -hz) dz += lz;
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 >= cut2 || r2 < 1e-20) continue;
            const double bin = sqrt(r2) / dr;
            if (bin < (double)nbins) atomicAdd(&hist[(int)bin], 1u);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += RDF_TILE)
        if (hist[b]) atomicAdd(counts + b, (unsigned long long)hist[b]);
}

__global__ void k_to_float(const double4* __restrict__ pos, float4* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4 x = pos[i];
        out[i] = make_float4((float)x.x, (float)x.y, (float)x.z, 0.f);
    }
}

// Unwrapped position x + image L (the continuous trajectory the reference's
// MSD tracker accumulates, lib.rs:520-560).
__device__ __forceinline__ double3 unwrapped(const Dev& d, const SysParams& sp, long long i) {
    const double4 x = d.pos[i];
    const int4 im = d.img[i];
    return make_double3(x.x + (double)im.x * sp.L[0], x.y + (double)im.y * sp.L[1], x.z + (double)im.z * sp.L[2]);
}

__global__ void __launch_bounds__(BLK) k_msd_ref(Dev d, int s, double* ref) {
    const SysParams& sp = d.sp[s];
    const int li = blockIdx.x * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long i = (long long)sp.p0 + li;
    const double3 u = unwrapped(d, sp, i);
    const size_t t = d.tag[i];
    ref[3 * t] = u.x;
    ref[3 * t + 1] = u.y;
    ref[3 * t + 2] = u.z;
}

// Block sums of |u - u_ref|^2 into part[blockIdx.x] (fixed tree: deterministic).
__global__ void __launch_bounds__(BLK) k_msd(Dev d, int s, const double* ref, double* part) {
    __shared__ double sh[BLK];
    const SysParams& sp = d.sp[s];
    const int li = blockIdx.x * BLK + threadIdx.x;
    double v = 0.0;
    if (li < sp.n) {
        const long long i = (long long)sp.p0 + li;
        const double3 u = unwrapped(d, sp, i);
        const size_t t = d.tag[i];
        const double dx = u.x - ref[3 * t], dy = u.y - ref[3 * t + 1], dz = u.z - ref[3 * t + 2];
        v = dx * dx + dy * dy + dz * dz;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int w = BLK / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

int launch_rdf(const Dev& d, int s, const SysParams& sp, float4* posf, double r_max, int nbins,
               unsigned long long* counts, cudaStream_t st) {
    const int n = sp.n;
    const double4* pos = d.pos + sp.p0;
    k_to_float<<<(n + 255) / 256, 256, 0, st>>>(pos, posf, n);
    const int tiles = (n + RDF_TILE - 1) / RDF_TILE;
    const double cut2 = r_max * r_max;
    const double dr = r_max / (double)nbins;
    // screen: float positions carry <= 2^-23 |x| error each; 1e-3 r_max of slack
    const float sr = (float)(r_max * (1.0 + 1e-3) + 4e-7 * (sp.L[0] + sp.L[1] + sp.L[2] + 1.0));
    k_rdf<<<dim3(tiles, tiles), RDF_TILE, 0, st>>>(pos, posf, n, sp.L[0], sp.L[1], sp.L[2], cut2, dr, sr * sr,
                                                  nbins, counts);
    return 2;
}

int launch_msd_ref(const Dev& d, int s, int n, double* ref, cudaStream_t st) {
    k_msd_ref<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(d, s, ref);
    return 1;
}

int launch_msd(const Dev& d, int s, int n, const double* ref, double* part, cudaStream_t st) {
    k_msd<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(d, s, ref, part);
    return 1;
}

int rdf_max_bins() { return RDF_MAX_BINS; }

}  // namespace mdg
