// mdg_generate.cu -- seeded initial conditions made on the device.
//
// Two generators write a system's particles straight into a context's device
// arrays, so a million-particle system is set up without a host loop or a
// host->device copy of its state:
//
// * FCC lattice: md_lattice's fcc_insert (crates/md_lattice/src/lib.rs:232-454)
//   -- 4-atom basis on unit cells stretched to tile the box, in (ix, iy, iz,
//   basis) order; types by cumulative fraction of (k + 0.5) / N; Gaussian
//   velocities N(0, sqrt(T/m)) per component; the mean velocity removed and
//   the velocities rescaled to T with 3N - 3 degrees of freedom.
// * Granular gas: dem_atom's random insertion (crates/dem_atom/src/insert.rs:
//   523-571) -- uniform candidates in the box inset by the largest radius, a
//   radius drawn per candidate, rejected when a placed sphere lies within
//   sep (r_i + r_j) under the minimum image -- as a grid-parallel random
//   sequential addition that reproduces the sequential result on its proposal
//   stream; speeds of fixed magnitude in isotropic directions, Maxwellian, or
//   Gaussian per component (insert.rs:580-592); omega 0, identity quaternions;
//   mass and inverse inertia as insert.rs:343-349.
//
// Random numbers are counter based: draw(seed, stream, i) is a hash of the
// three (splitmix64's finaliser, Steele, Lea & Flood 2014, applied twice), so
// a particle's draws do not depend on the launch shape, and a CPU
// restatement reproduces the stream.  Uniforms take the top 53 bits; normals
// come from the Box-Muller transform.
//
// Parallel RSA.  Proposal g = 0, 1, 2, ... is a centre and radius from draws
// 4g .. 4g+3 of stream 1.  Sequential RSA accepts g when it clears every
// sphere accepted before it.  The device takes the proposals in batches
// [g0, g0 + M): each is tested against the placed spheres of the 27 cells
// around it (cells at least one exclusion reach wide); the survivors are
// listed per cell; sweeps then settle them in proposal order -- a proposal is
// rejected as soon as an earlier proposal of the batch that it conflicts with
// is accepted, and accepted once every such earlier proposal is rejected.  The
// lowest undecided proposal is always settled by the next sweep, and the
// conflict chains are short, so a few sweeps settle a batch; the result is the
// sequential one.  A prefix sum over the batch numbers the accepted proposals;
// those numbered below n are placed, in proposal order.  The batch size only
// changes the speed, never the spheres.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {
namespace {

constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ull;
constexpr double kTwoM53 = 1.0 / 9007199254740992.0;  // 2^-53
constexpr double kPiD = 3.141592653589793;
constexpr int GEN_BLOCK = 256;
constexpr int RED_BLOCKS = 1024;     // fixed reduction grid: the same sums on every launch
constexpr int SCAN_BLOCK = 1024;     // proposals per scan block
constexpr int CAND_CAP = 16;         // listed proposals per cell and batch
constexpr int MAX_BATCH = 1 << 20;   // proposals per batch (<= SCAN_BLOCK^2)
constexpr int STREAM_PLACE = 1, STREAM_VEL = 2;

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__host__ __device__ inline uint64_t draw(uint64_t seed, uint32_t stream, uint64_t i) {
    return mix64(mix64(seed + kGolden * ((uint64_t)stream + 1)) + kGolden * (i + 1));
}

__device__ inline double uniform01(uint64_t h) { return (double)(h >> 11) * kTwoM53; }  // [0, 1)

// Two standard normals from draws (2k, 2k+1) of the stream at index base.
__device__ inline void normal_pair(uint64_t seed, uint32_t stream, uint64_t base, double& z0, double& z1) {
    const double u1 = ((double)(draw(seed, stream, base) >> 11) + 1.0) * kTwoM53;  // (0, 1]
    const double u2 = uniform01(draw(seed, stream, base + 1));
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// Three standard normals of particle i (draws 4i .. 4i+3; the fourth normal
// is dropped).
__device__ inline double3 normal3(uint64_t seed, uint64_t i) {
    double a, b, c, e;
    normal_pair(seed, STREAM_VEL, 4 * i, a, b);
    normal_pair(seed, STREAM_VEL, 4 * i + 2, c, e);
    return make_double3(a, b, c);
}

// The padding rows of a system segment, as mdg_upload_state writes them.
__device__ inline void write_pad(const Dev& d, size_t o, bool dem) {
    const double4 z = make_double4(0.0, 0.0, 0.0, 0.0);
    d.pos[o] = z;
    d.lbp[o] = z;
    d.vel[o] = z;
    d.frc[o] = z;
    d.mass[o] = 1.0;
    d.cutr[o] = 0.0;
    d.tag[o] = 0xffffffffu;
    d.type[o] = 0;
    d.img[o] = make_int4(0, 0, 0, 0);
    d.nnum[o] = 0;
    if (dem) {
        d.omg[o] = z;
        d.trq[o] = z;
        d.quat[o] = make_double4(1.0, 0.0, 0.0, 0.0);
        d.hcnt[0][o] = 0;
        d.hcnt[1][o] = 0;
    }
}

// ---------------------------------------------------------------- FCC lattice

__global__ void k_fcc_place(Dev d, int p0, int n, int npad, FccArgs f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    const size_t o = (size_t)p0 + i;
    if (i >= n) {
        write_pad(d, o, false);
        return;
    }
    const int b = i & 3, cid = i >> 2;
    const int iz = cid % f.nc[2];
    const int iy = (cid / f.nc[2]) % f.nc[1];
    const int ix = cid / (f.nc[2] * f.nc[1]);
    // basis (0,0,0), (1/2,1/2,0), (1/2,0,1/2), (0,1/2,1/2)
    const double bx = (b == 1 || b == 2) ? 0.5 : 0.0;
    const double by = (b == 1 || b == 3) ? 0.5 : 0.0;
    const double bz = (b == 2 || b == 3) ? 0.5 : 0.0;
    const double x = f.lo[0] + ((double)ix + bx) * f.a[0];
    const double y = f.lo[1] + ((double)iy + by) * f.a[1];
    const double z = f.lo[2] + ((double)iz + bz) * f.a[2];
    int t = 0;
    if (f.ntypes > 1) {
        const double fr = ((double)i + 0.5) / (double)n;
        t = f.ntypes - 1;
        for (int q = 0; q < f.ntypes; q++)
            if (fr < f.frac[q]) {
                t = q;
                break;
            }
    }
    const double m = f.tmass[t];
    const double sv = sqrt(f.temperature / m);
    const double3 g = normal3(f.seed, (uint64_t)i);
    const double4 p = make_double4(x, y, z, 0.0);
    d.pos[o] = p;
    d.lbp[o] = p;
    d.vel[o] = make_double4(sv * g.x, sv * g.y, sv * g.z, 1.0 / m);
    d.frc[o] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.mass[o] = m;
    d.cutr[o] = f.skin;
    d.tag[o] = (uint32_t)i;
    d.type[o] = (uint32_t)t;
    d.img[o] = make_int4(0, 0, 0, 0);
    d.nnum[o] = 0;
}

// Block partials over a system's particles: MODE 0 the velocity sums; MODE 1
// sum m |v - u|^2.  Fixed grid and tree order: the same sums on every launch.
template <int MODE>
__global__ void __launch_bounds__(GEN_BLOCK) k_gen_sum(const double4* __restrict__ vel, const double* __restrict__ mass,
                                                       int p0, int n, double ux, double uy, double uz,
                                                       double* __restrict__ part) {
    __shared__ double sh[3][GEN_BLOCK];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int i = blockIdx.x * GEN_BLOCK + threadIdx.x; i < n; i += RED_BLOCKS * GEN_BLOCK) {
        const double4 v = vel[p0 + i];
        if (MODE == 0) {
            a0 += v.x;
            a1 += v.y;
            a2 += v.z;
        } else {
            const double dx = v.x - ux, dy = v.y - uy, dz = v.z - uz;
            a0 += mass[p0 + i] * (dx * dx + dy * dy + dz * dz);
        }
    }
    sh[0][threadIdx.x] = a0;
    sh[1][threadIdx.x] = a1;
    sh[2][threadIdx.x] = a2;
    __syncthreads();
    for (int s = GEN_BLOCK / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 3; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) part[3 * blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// Totals of the RED_BLOCKS partials, in tree order.
__global__ void __launch_bounds__(RED_BLOCKS) k_gen_total(const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[3][RED_BLOCKS];
    for (int q = 0; q < 3; q++) sh[q][threadIdx.x] = part[3 * threadIdx.x + q];
    __syncthreads();
    for (int s = RED_BLOCKS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 3; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) out[threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_gen_adjust(double4* vel, int p0, int n, double ux, double uy, double uz, double scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4 v = vel[p0 + i];
    v.x = (v.x - ux) * scale;
    v.y = (v.y - uy) * scale;
    v.z = (v.z - uz) * scale;
    vel[p0 + i] = v;
}

// -------------------------------------------------------------- parallel RSA

struct RsaGrid {
    double L[3], lo[3];         // box
    double in_lo[3], in_w[3];   // proposal region in_lo + in_w u
    double cell[3];
    int nc[3];
    double rmin, rdelta, sep;
    uint64_t seed;
    int capp;                   // placed spheres per cell
};

__device__ inline int cell_of(const RsaGrid& g, double x, int d) {
    int c = (int)floor((x - g.lo[d]) / g.cell[d]);
    c %= g.nc[d];
    return c < 0 ? c + g.nc[d] : c;
}

__device__ inline int nbr(const RsaGrid& g, int c, int k, int d) {
    // distinct neighbour cells: 3 per axis, or every cell when fewer than 3
    return g.nc[d] >= 3 ? (c + k - 1 + g.nc[d]) % g.nc[d] : k;
}

__device__ inline int noff(const RsaGrid& g, int d) { return g.nc[d] >= 3 ? 3 : g.nc[d]; }

// b within the exclusion distance of a (minimum image); symmetric in a, b
__device__ inline bool conflict(const RsaGrid& g, const double4& a, const double4& b) {
    double r2 = 0.0;
    const double ad[3] = {a.x, a.y, a.z}, bd[3] = {b.x, b.y, b.z};
    for (int d = 0; d < 3; d++) {
        double dx = bd[d] - ad[d];
        dx -= g.L[d] * rint(dx / g.L[d]);
        r2 += dx * dx;
    }
    const double md = g.sep * (a.w + b.w);
    return r2 <= md * md;
}

__device__ inline double4 proposal(const RsaGrid& g, uint64_t k) {
    const double ux = uniform01(draw(g.seed, STREAM_PLACE, 4 * k));
    const double uy = uniform01(draw(g.seed, STREAM_PLACE, 4 * k + 1));
    const double uz = uniform01(draw(g.seed, STREAM_PLACE, 4 * k + 2));
    const double ur = uniform01(draw(g.seed, STREAM_PLACE, 4 * k + 3));
    return make_double4(g.in_lo[0] + g.in_w[0] * ux, g.in_lo[1] + g.in_w[1] * uy, g.in_lo[2] + g.in_w[2] * uz,
                        g.rdelta > 0.0 ? g.rmin + g.rdelta * ur : g.rmin);
}

// st: 0 undecided, 1 accepted, 2 rejected.  flags[0] |= 1: a cell's proposal
// list overflowed (the batch is redone smaller); |= 2: a cell's placed list
// overflowed (cannot happen within the packing bound).
__global__ void k_rsa_propose(RsaGrid g, uint64_t g0, int M, const double4* __restrict__ placed,
                              const int* __restrict__ pcnt, const int* __restrict__ plist, double4* __restrict__ cpos,
                              int* __restrict__ ccell, int* __restrict__ st, int* __restrict__ ccnt,
                              int* __restrict__ clist, int* __restrict__ flags) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    const double4 q = proposal(g, g0 + (uint64_t)c);
    cpos[c] = q;
    const int ci[3] = {cell_of(g, q.x, 0), cell_of(g, q.y, 1), cell_of(g, q.z, 2)};
    bool hit = false;
    for (int a = 0; a < noff(g, 0) && !hit; a++)
        for (int b = 0; b < noff(g, 1) && !hit; b++)
            for (int e = 0; e < noff(g, 2) && !hit; e++) {
                const int cc = (nbr(g, ci[0], a, 0) * g.nc[1] + nbr(g, ci[1], b, 1)) * g.nc[2] + nbr(g, ci[2], e, 2);
                const int m = min(pcnt[cc], g.capp);
                for (int k = 0; k < m; k++)
                    if (conflict(g, q, placed[plist[(size_t)cc * g.capp + k]])) {
                        hit = true;
                        break;
                    }
            }
    if (hit) {
        st[c] = 2;
        ccell[c] = -1;
        return;
    }
    st[c] = 0;
    const int cf = (ci[0] * g.nc[1] + ci[1]) * g.nc[2] + ci[2];
    ccell[c] = cf;
    const int k = atomicAdd(&ccnt[cf], 1);
    if (k < CAND_CAP) clist[(size_t)cf * CAND_CAP + k] = c;
    else atomicOr(flags, 1);
}

__global__ void k_rsa_settle(RsaGrid g, int M, const double4* __restrict__ cpos, const int* __restrict__ ccell,
                             int* st, const int* __restrict__ ccnt, const int* __restrict__ clist, int* undecided) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M) return;
    volatile int* vst = st;
    if (vst[c] != 0) return;
    const double4 q = cpos[c];
    const int cf = ccell[c];
    const int ci[3] = {cf / (g.nc[1] * g.nc[2]), (cf / g.nc[2]) % g.nc[1], cf % g.nc[2]};
    bool pending = false;
    for (int a = 0; a < noff(g, 0); a++)
        for (int b = 0; b < noff(g, 1); b++)
            for (int e = 0; e < noff(g, 2); e++) {
                const int cc = (nbr(g, ci[0], a, 0) * g.nc[1] + nbr(g, ci[1], b, 1)) * g.nc[2] + nbr(g, ci[2], e, 2);
                const int m = min(ccnt[cc], CAND_CAP);
                for (int k = 0; k < m; k++) {
                    const int j = clist[(size_t)cc * CAND_CAP + k];
                    if (j >= c) continue;
                    const int s = vst[j];
                    if (s == 2 || !conflict(g, q, cpos[j])) continue;
                    if (s == 1) {
                        vst[c] = 2;
                        return;
                    }
                    pending = true;
                }
            }
    if (pending) atomicAdd(undecided, 1);
    else vst[c] = 1;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_rsa_count(const int* __restrict__ st, int M, int* __restrict__ bcount) {
    __shared__ int ws[SCAN_BLOCK / 32];
    const int c = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const unsigned bal = __ballot_sync(0xffffffffu, c < M && st[c] == 1);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; w++) t += ws[w];
        bcount[blockIdx.x] = t;
    }
}

// Exclusive scan of nb <= SCAN_BLOCK block counts; boff[nb] = the total.
__global__ void __launch_bounds__(SCAN_BLOCK) k_rsa_scan(const int* __restrict__ bcount, int nb, int* __restrict__ boff) {
    __shared__ int sh[SCAN_BLOCK];
    const int t = threadIdx.x;
    sh[t] = t < nb ? bcount[t] : 0;
    __syncthreads();
    for (int s = 1; s < SCAN_BLOCK; s <<= 1) {
        const int v = t >= s ? sh[t - s] : 0;
        __syncthreads();
        sh[t] += v;
        __syncthreads();
    }
    if (t < nb) boff[t] = sh[t] - bcount[t];
    if (t == SCAN_BLOCK - 1) boff[nb] = sh[t];
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_rsa_commit(RsaGrid g, int M, long long placed0, long long n,
                                                           const int* __restrict__ st, const double4* __restrict__ cpos,
                                                           const int* __restrict__ ccell, const int* __restrict__ boff,
                                                           double4* __restrict__ placed, int* __restrict__ pcnt,
                                                           int* __restrict__ plist, int* __restrict__ ccnt,
                                                           int* __restrict__ flags) {
    __shared__ int ws[SCAN_BLOCK / 32];
    const int c = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const bool acc = c < M && st[c] == 1;
    const unsigned bal = __ballot_sync(0xffffffffu, acc);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) ws[w] = __popc(bal);
    __syncthreads();
    int before = 0;
    for (int q = 0; q < w; q++) before += ws[q];
    before += __popc(bal & ((1u << lane) - 1u));
    if (c < M && ccell[c] >= 0) ccnt[ccell[c]] = 0;  // the proposal lists are rebuilt by the next batch
    if (!acc) return;
    const long long idx = placed0 + boff[blockIdx.x] + before;
    if (idx >= n) return;
    const double4 q = cpos[c];
    placed[idx] = q;
    const int cf = (cell_of(g, q.x, 0) * g.nc[1] + cell_of(g, q.y, 1)) * g.nc[2] + cell_of(g, q.z, 2);
    const int k = atomicAdd(&pcnt[cf], 1);
    if (k < g.capp) plist[(size_t)cf * g.capp + k] = (int)idx;
    else atomicOr(flags, 2);
}

// min and max radius of the placed spheres (positive doubles order like their bits)
__global__ void k_rsa_minmax(const double4* __restrict__ placed, long long n, unsigned long long* mm) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long b = (unsigned long long)__double_as_longlong(placed[i].w);
    atomicMin(&mm[0], b);
    atomicMax(&mm[1], b);
}

__global__ void k_gas_write(Dev d, int p0, int n, int npad, const double4* __restrict__ placed, GasArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    const size_t o = (size_t)p0 + i;
    if (i >= n) {
        write_pad(d, o, true);
        return;
    }
    const double4 q = placed[i];
    const double r = q.w;
    const double m = ((a.density * 4.0) / 3.0) * kPiD * ((r * r) * r);
    const double inv_i = 1.0 / (((0.4 * m) * r) * r);
    double3 v;
    if (a.vel_mode == MDG_VEL_SPEED) {
        const double u1 = uniform01(draw(a.seed, STREAM_VEL, 4 * (uint64_t)i));
        const double u2 = uniform01(draw(a.seed, STREAM_VEL, 4 * (uint64_t)i + 1));
        const double z = 1.0 - 2.0 * u1;
        const double s = sqrt(fmax(0.0, 1.0 - z * z));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        v = make_double3(a.speed * (s * cs), a.speed * (s * sn), a.speed * z);
    } else {
        const double sg = a.vel_mode == MDG_VEL_MAXWELL_RMS ? a.speed / sqrt(3.0) : a.speed;
        const double3 g = normal3(a.seed, (uint64_t)i);
        v = make_double3(sg * g.x, sg * g.y, sg * g.z);
    }
    d.pos[o] = q;
    d.lbp[o] = q;
    d.vel[o] = make_double4(v.x, v.y, v.z, 1.0 / m);
    d.frc[o] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.mass[o] = m;
    d.cutr[o] = r;
    d.tag[o] = (uint32_t)i;
    d.type[o] = a.material;
    d.img[o] = make_int4(0, 0, 0, 0);
    d.nnum[o] = 0;
    d.omg[o] = make_double4(0.0, 0.0, 0.0, inv_i);
    d.trq[o] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.quat[o] = make_double4(1.0, 0.0, 0.0, 0.0);
    d.hcnt[0][o] = 0;
    d.hcnt[1][o] = 0;
}

int blocks_for(long long n, int b) { return (int)((n + b - 1) / b); }

int gen_err(cudaError_t e) {
    if (e == cudaSuccess) return MDG_OK;
    return e == cudaErrorMemoryAllocation ? MDG_ERR_OOM : MDG_ERR_CUDA;
}

int sync_err(cudaStream_t s) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    return gen_err(e);
}

}  // namespace

int gen_fcc(const Dev& d, const SysParams& p, const FccArgs& f, cudaStream_t s, long long* launches) {
    const int n = p.n;
    k_fcc_place<<<blocks_for(p.npad, GEN_BLOCK), GEN_BLOCK, 0, s>>>(d, p.p0, n, p.npad, f);
    double* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, (3 * RED_BLOCKS + 3) * sizeof(double), s);
    if (e != cudaSuccess) return gen_err(e);
    double tot[3];
    // mean velocity (fcc_insert: the plain mean over the atoms)
    k_gen_sum<0><<<RED_BLOCKS, GEN_BLOCK, 0, s>>>(d.vel, d.mass, p.p0, n, 0.0, 0.0, 0.0, buf);
    k_gen_total<<<1, RED_BLOCKS, 0, s>>>(buf, buf + 3 * RED_BLOCKS);
    cudaMemcpyAsync(tot, buf + 3 * RED_BLOCKS, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
    int r = sync_err(s);
    if (r) {
        cudaFreeAsync(buf, s);
        return r;
    }
    const double nn = (double)n;
    const double ux = tot[0] / nn, uy = tot[1] / nn, uz = tot[2] / nn;
    // kinetic energy after the mean is removed; rescale to T with 3N - 3 dof
    k_gen_sum<1><<<RED_BLOCKS, GEN_BLOCK, 0, s>>>(d.vel, d.mass, p.p0, n, ux, uy, uz, buf);
    k_gen_total<<<1, RED_BLOCKS, 0, s>>>(buf, buf + 3 * RED_BLOCKS);
    cudaMemcpyAsync(tot, buf + 3 * RED_BLOCKS, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
    r = sync_err(s);
    cudaFreeAsync(buf, s);
    if (r) return r;
    double scale = 1.0;
    const double ndof = 3.0 * nn - 3.0;
    if (ndof > 0.0) {
        const double ke = 0.5 * tot[0];
        const double cur = 2.0 * ke / ndof;
        if (cur > 1e-20) scale = std::sqrt(f.temperature / cur);
    }
    k_gen_adjust<<<blocks_for(n, GEN_BLOCK), GEN_BLOCK, 0, s>>>(d.vel, p.p0, n, ux, uy, uz, scale);
    *launches += 8;
    return sync_err(s);
}

void GasPlacement::release(cudaStream_t s) {
    if (placed) cudaFreeAsync(placed, s);
    placed = nullptr;
}

int gen_gas_place(const GasArgs& a, const double box_lo[3], const double box_hi[3], cudaStream_t s,
                  GasPlacement* out, long long* launches) {
    out->placed = nullptr;
    out->count = 0;
    const long long n = (long long)a.n;
    RsaGrid g{};
    const double reach = a.sep * 2.0 * a.rmax;
    long long ncell = 1;
    for (int d = 0; d < 3; d++) {
        g.lo[d] = box_lo[d];
        g.L[d] = box_hi[d] - box_lo[d];
        g.in_lo[d] = box_lo[d] + (a.inset ? a.rmax : 0.0);
        g.in_w[d] = (box_hi[d] - (a.inset ? a.rmax : 0.0)) - g.in_lo[d];
        if (!(g.L[d] > 0.0) || !(g.in_w[d] > 0.0)) return MDG_ERR_ARG;
        // cells wider than the reach by a margin: binning rounding cannot hide a conflict
        const double c = std::floor(g.L[d] / (reach * (1.0 + 1e-9)));
        g.nc[d] = c < 1.0 ? 1 : (c > 1024.0 ? 1024 : (int)c);
        g.cell[d] = g.L[d] / g.nc[d];
        ncell *= g.nc[d];
    }
    g.rmin = a.rmin;
    g.rdelta = a.rmax - a.rmin;
    g.sep = a.sep;
    g.seed = a.seed;
    // placed spheres per cell: exclusion balls of radius sep rmin are disjoint
    // and lie in the cell grown by that radius on every side
    const double h = a.sep * a.rmin;
    double vol = 1.0;
    for (int d = 0; d < 3; d++) vol *= g.cell[d] + 2.0 * h;
    const double capd = std::floor(vol / (4.0 / 3.0 * kPiD * h * h * h)) + 1.0;
    if (!(capd >= 1.0) || capd > 4096.0) return MDG_ERR_CONFIG;
    g.capp = (int)capd;
    if ((double)ncell * (g.capp + CAND_CAP) * sizeof(int) > 8e9) return MDG_ERR_CONFIG;
    // at most 2 proposals per cell on average: a cell's list (CAND_CAP = 16)
    // fills with probability below 1e-10
    const long long batch_cap = std::min<long long>(MAX_BATCH, 2 * ncell);
    const uint64_t limit = a.max_proposals ? a.max_proposals : (uint64_t)n * 20000ull;

    int err = MDG_OK;
    auto alloc = [&](void** p, size_t bytes) {
        if (err) return;
        cudaError_t e = cudaMallocAsync(p, bytes, s);
        if (e != cudaSuccess) err = gen_err(e);
    };
    double4 *placed = nullptr, *cpos = nullptr;
    int *pcnt = nullptr, *plist = nullptr, *ccnt = nullptr, *clist = nullptr, *ccell = nullptr, *st = nullptr;
    int *bcount = nullptr, *boff = nullptr, *flags = nullptr;
    unsigned long long* mm = nullptr;
    alloc((void**)&placed, (size_t)n * sizeof(double4));
    alloc((void**)&pcnt, (size_t)ncell * sizeof(int));
    alloc((void**)&plist, (size_t)ncell * g.capp * sizeof(int));
    alloc((void**)&ccnt, (size_t)ncell * sizeof(int));
    alloc((void**)&clist, (size_t)ncell * CAND_CAP * sizeof(int));
    alloc((void**)&cpos, (size_t)batch_cap * sizeof(double4));
    alloc((void**)&ccell, (size_t)batch_cap * sizeof(int));
    alloc((void**)&st, (size_t)batch_cap * sizeof(int));
    alloc((void**)&bcount, (size_t)SCAN_BLOCK * sizeof(int));
    alloc((void**)&boff, (size_t)(SCAN_BLOCK + 1) * sizeof(int));
    alloc((void**)&flags, 2 * sizeof(int));
    alloc((void**)&mm, 2 * sizeof(unsigned long long));
    auto release = [&]() {
        for (void* p : {(void*)cpos, (void*)pcnt, (void*)plist, (void*)ccnt, (void*)clist, (void*)ccell, (void*)st,
                        (void*)bcount, (void*)boff, (void*)flags, (void*)mm})
            if (p) cudaFreeAsync(p, s);
    };
    if (!err) {
        cudaMemsetAsync(pcnt, 0, (size_t)ncell * sizeof(int), s);
        cudaMemsetAsync(ccnt, 0, (size_t)ncell * sizeof(int), s);
    }
    long long count = 0;
    uint64_t g0 = 0;
    double rate = 1.0;             // acceptance of the last batch: sizes the next
    long long cap_now = batch_cap;  // halved when a cell's proposal list overflows
    while (!err && count < n && g0 < limit) {
        const long long want = (long long)std::ceil((double)(n - count) / std::max(rate, 1e-3) * 1.25) + 256;
        const long long M = std::min<long long>({cap_now, std::max<long long>(1024, want), (long long)(limit - g0)});
        int hflags[2] = {0, 0}, und = 0;
        cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
        k_rsa_propose<<<blocks_for(M, GEN_BLOCK), GEN_BLOCK, 0, s>>>(g, g0, (int)M, placed, pcnt, plist, cpos, ccell,
                                                                     st, ccnt, clist, flags);
        cudaMemcpyAsync(hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s);
        *launches += 1;
        if ((err = sync_err(s))) break;
        if (hflags[0] & 1) {  // a cell's proposal list overflowed: clear and redo the batch smaller
            cudaMemsetAsync(ccnt, 0, (size_t)ncell * sizeof(int), s);
            cap_now = std::max<long long>(1, M / 2);  // one proposal never overflows
            continue;
        }
        for (long long sweep = 0;; sweep++) {
            if (sweep > M) {  // unreachable: every sweep settles the lowest undecided proposal
                err = MDG_ERR_TIMEOUT;
                break;
            }
            cudaMemsetAsync(flags + 1, 0, sizeof(int), s);
            k_rsa_settle<<<blocks_for(M, GEN_BLOCK), GEN_BLOCK, 0, s>>>(g, (int)M, cpos, ccell, st, ccnt, clist,
                                                                        flags + 1);
            cudaMemcpyAsync(&und, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
            *launches += 1;
            if ((err = sync_err(s))) break;
            if (und == 0) break;
        }
        if (err) break;
        const int nb = blocks_for(M, SCAN_BLOCK);
        int total = 0;
        k_rsa_count<<<nb, SCAN_BLOCK, 0, s>>>(st, (int)M, bcount);
        k_rsa_scan<<<1, SCAN_BLOCK, 0, s>>>(bcount, nb, boff);
        k_rsa_commit<<<nb, SCAN_BLOCK, 0, s>>>(g, (int)M, count, n, st, cpos, ccell, boff, placed, pcnt, plist, ccnt,
                                               flags);
        cudaMemcpyAsync(&total, boff + nb, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s);
        *launches += 3;
        if ((err = sync_err(s))) break;
        if (hflags[0] & 2) {
            err = MDG_ERR_CONFIG;
            break;
        }
        count = std::min<long long>(n, count + total);
        rate = (double)total / (double)M;
        g0 += (uint64_t)M;
    }
    if (!err && count > 0) {
        unsigned long long hm[2] = {~0ull, 0ull};
        cudaMemcpyAsync(mm, hm, sizeof(hm), cudaMemcpyHostToDevice, s);
        k_rsa_minmax<<<blocks_for(count, GEN_BLOCK), GEN_BLOCK, 0, s>>>(placed, count, mm);
        cudaMemcpyAsync(hm, mm, sizeof(hm), cudaMemcpyDeviceToHost, s);
        *launches += 1;
        err = sync_err(s);
        if (!err) {
            double lo, hi;
            std::memcpy(&lo, &hm[0], sizeof(double));
            std::memcpy(&hi, &hm[1], sizeof(double));
            out->rmin = lo;
            out->rmax = hi;
        }
    }
    release();
    out->placed = placed;
    out->count = (size_t)count;
    out->proposals = g0;
    if (err) {
        out->release(s);
        return err;
    }
    return count == n ? MDG_OK : MDG_ERR_ARG;
}

int gen_gas_write(const Dev& d, const SysParams& p, const GasArgs& a, const GasPlacement& gp, cudaStream_t s,
                  long long* launches) {
    k_gas_write<<<blocks_for(p.npad, GEN_BLOCK), GEN_BLOCK, 0, s>>>(d, p.p0, p.n, p.npad, gp.placed, a);
    *launches += 1;
    return sync_err(s);
}

}  // namespace mdg

extern "C" uint64_t mdg_counter_draw(uint64_t seed, uint32_t stream, uint64_t index) {
    return mdg::draw(seed, stream, index);
}
