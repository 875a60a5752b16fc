// mdg_noalloc.cu -- the granular-temperature reduction without any device
// allocation.
//
// mdg_thermo needs a context, and a context owns device memory it allocated
// with cudaMalloc.  Some callers cannot allocate: a host that reserves all of
// the GPU's memory up front for its own pool and refuses any allocation made
// behind its back, or a time-critical loop where an allocation may synchronize
// the device and stall every other stream.  mdg_granular_temp_noalloc serves
// them: the caller passes device buffers for the inputs and the output, and
// the only scratch memory is the file-scope array below, which is part of the
// library image and is held on every GPU that loads the library until the
// process exits.
//
// The computation mirrors print_granular_temperature
// (crates/dem_granular/src/granular_temp.rs:44-134) and compute_ke
// (crates/mddem_core/src/atom.rs:489-502): two passes, the second using the
// mass-weighted mean velocity of the first.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mdg.h"

namespace {

constexpr int NA_BLOCK = 256;                       // threads (= particles) per block
constexpr int NA_MAX_BLOCKS = 4096;                 // => at most 1,048,576 particles
constexpr int NA_SLOTS = 8;                         // doubles per block partial
constexpr int NA_TOTALS = NA_MAX_BLOCKS * NA_SLOTS; // offset of the pass-1 totals
constexpr int NA_COUNTER = NA_TOTALS + 8;           // arrival counter (one double slot)
constexpr int NA_DOUBLES = NA_COUNTER + 8;

}  // namespace

// All calls share this array and it keeps the last call's contents.  Calls
// that overlap on the GPU (different streams or threads at the same time) race
// on it: the caller must serialise them.
static __device__ __align__(256) double g_mdg_noalloc_scratch[NA_DOUBLES];

namespace {

// Fixed-order block reduction of NV values over NA_BLOCK threads.
template <int NV>
__device__ void block_sum(double (&v)[NV], double (*sh)[NA_BLOCK]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int k = 0; k < NV; k++) sh[k][t] = v[k];
    __syncthreads();
    for (int w = NA_BLOCK / 2; w > 0; w >>= 1) {
        if (t < w) {
#pragma unroll
            for (int k = 0; k < NV; k++) sh[k][t] = sh[k][t] + sh[k][t + w];
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = sh[k][0];
}

// Writes this block's partial, then the last block to arrive sums all partials
// in block order (strided lanes, fixed tree) into tot[], resets the counter
// and returns true.
template <int NV>
__device__ bool last_block_total(double* scr, const double (&part)[NV], double* tot, double (*sh)[NA_BLOCK]) {
    __shared__ int last;
    unsigned int* counter = reinterpret_cast<unsigned int*>(scr + NA_COUNTER);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) scr[(size_t)blockIdx.x * NA_SLOTS + k] = part[k];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += NA_BLOCK) {
        const volatile double* p = scr + (size_t)b * NA_SLOTS;
#pragma unroll
        for (int k = 0; k < NV; k++) acc[k] = acc[k] + p[k];
    }
    block_sum<NV>(acc, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) tot[k] = acc[k];
        *counter = 0u;
    }
    return true;
}

// pass 1: sum m, sum m v, sum m |v|^2
__global__ void __launch_bounds__(NA_BLOCK) k_na_pass1(const double* __restrict__ vel,
                                                       const double* __restrict__ mass, long long n, double* scr) {
    __shared__ double sh[5][NA_BLOCK];
    const long long i = (long long)blockIdx.x * NA_BLOCK + threadIdx.x;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < n) {
        const double m = mass[i];
        const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
        v[0] = m;
        v[1] = m * vx;
        v[2] = m * vy;
        v[3] = m * vz;
        v[4] = m * (vx * vx + vy * vy + vz * vz);
    }
    block_sum<5>(v, sh);
    last_block_total<5>(scr, v, scr + NA_TOTALS, sh);
}

// pass 2: sum m |v - vbar|^2, then the three outputs
__global__ void __launch_bounds__(NA_BLOCK) k_na_pass2(const double* __restrict__ vel,
                                                       const double* __restrict__ mass, long long n, double* scr,
                                                       double* out) {
    __shared__ double sh[1][NA_BLOCK];
    const double* tot = scr + NA_TOTALS;
    const long long i = (long long)blockIdx.x * NA_BLOCK + threadIdx.x;
    double v[1] = {0.0};
    if (i < n) {
        const double m = mass[i];
        const double ax = tot[1] / tot[0], ay = tot[2] / tot[0], az = tot[3] / tot[0];
        const double dx = vel[3 * i] - ax, dy = vel[3 * i + 1] - ay, dz = vel[3 * i + 2] - az;
        v[0] = m * (dx * dx) + m * (dy * dy) + m * (dz * dz);
    }
    block_sum<1>(v, sh);
    double res[1];
    if (last_block_total<1>(scr, v, res, sh) && threadIdx.x == 0) {
        out[0] = res[0] / (3.0 * tot[0]);
        out[1] = 0.5 * tot[4];
        out[2] = sqrt(tot[1] * tot[1] + tot[2] * tot[2] + tot[3] * tot[3]);
    }
}

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
double* g_na_scratch[NA_MAX_DEVICES] = {};

int na_status(cudaError_t e) {
    if (e == cudaSuccess) return MDG_OK;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MDG_ERR_NODEVICE;
    return MDG_ERR_CUDA;
}

}  // namespace

extern "C" int mdg_granular_temp_noalloc(const double* vel, const double* mass, size_t n, double* out3,
                                         void* stream) {
    if (!vel || !mass || !out3 || n == 0) return MDG_ERR_ARG;
    if (n > (size_t)NA_MAX_BLOCKS * NA_BLOCK) return MDG_ERR_ARG;  // beyond the scratch array
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_status(e);
    if (dev < 0 || dev >= NA_MAX_DEVICES) return MDG_ERR_ARG;
    double* scr = nullptr;
    {
        // once per device, with that device current: the device address of the
        // static scratch array (its host-side name is only a stand-in).  The
        // cached address belongs to the device's primary context; it assumes
        // that context lives as long as the process.  A caller that resets
        // the device (cudaDeviceReset) must not call this entry point again
        // in the same process.
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_scratch[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_mdg_noalloc_scratch);
            if (e != cudaSuccess) return na_status(e);
            g_na_scratch[dev] = static_cast<double*>(p);
        }
        scr = g_na_scratch[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the arrival counter must start at zero
    e = cudaMemsetAsync(scr + NA_COUNTER, 0, sizeof(double), st);
    if (e != cudaSuccess) return na_status(e);
    const unsigned int nb = (unsigned int)((n + NA_BLOCK - 1) / NA_BLOCK);
    k_na_pass1<<<nb, NA_BLOCK, 0, st>>>(vel, mass, (long long)n, scr);
    k_na_pass2<<<nb, NA_BLOCK, 0, st>>>(vel, mass, (long long)n, scr, out3);
    return na_status(cudaGetLastError());
}
