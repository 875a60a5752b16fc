// mdg_kernels_fp64.cu -- FP64 kernels of the hot path (the plain path).
//
// Compiled with -fmad=false: every multiply and add rounds separately, and
// fma() appears exactly where the reference uses f64::mul_add, so per-pair
// arithmetic is bit-identical to the reference's CPU path.  Per-particle sums
// run in a fixed per-row order (deterministic run to run) that differs from
// the reference's scatter-then-reverse-comm order, hence a 1e-12 relative
// bound on forces rather than bit equality.
//
// One timestep = k_initial -> [rebuild: k_rb_plan, k_cells, k_scan,
// k_scatter, k_cellsort, k_gather, k_copyback, k_build] -> force -> k_final.
// The rebuild kernels visit only the systems that sort or rebuild this step.
#include "mdg_internal.cuh"

namespace mdg {

// ----------------------------------------------------------------------------
// helpers
// ----------------------------------------------------------------------------
// Ghost position = pos + periodic_offset * size (comm.rs:281, 404-406); the
// offset is +-1.0, so the image coordinate is x + L or x + (-L) exactly.
__device__ __forceinline__ double img_coord(double x, int s, double L) {
    return s > 0 ? x + L : (s < 0 ? x + (-L) : x);
}

// ((p - bin_origin) * inv_bs).floor() as i32, clamped (neighbor.rs:848-853)
__device__ __forceinline__ int ext_cell_1d(double x, double origin, double inv_bin, int ext) {
    int c = (int)floor((x - origin) * inv_bin);
    return c < 0 ? 0 : (c > ext - 1 ? ext - 1 : c);
}

__device__ __forceinline__ void decode_shift(int sc, int& sx, int& sy, int& sz) {
    sx = sc / 9 - 1;
    sy = (sc / 3) % 3 - 1;
    sz = sc % 3 - 1;
}



// ----------------------------------------------------------------------------
// initial integration + rebuild decision
// ----------------------------------------------------------------------------
// nh_pre_initial (md_thermostat/src/lib.rs:254-301) or initial_integration
// (mddem_verlet/src/lib.rs:97-123) + initial_rotation (rotational.rs:59-84),
// fused with decide_rebuild's per-atom tests (neighbor.rs:564-674).
__global__ void __launch_bounds__(BLK) k_initial(Dev d) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    const bool live = sys_active(st);
    const bool act = live && li < sp.n;
    const long long i = (long long)sp.p0 + li;
    const double dt = sp.dt;
    // exp(-dt/2 p_xi / Q) after the pre-initial half step of p_xi, computed
    // once per system by the previous step's reduction (k_final / k_ke_init)
    const double scale = sp.nh ? st->nh_scale : 1.0;
    if (li == 0 && live)
        st->periodic_sort =
            (sp.policy == 0 && sp.sort_every > 0 && st->sort_counter + 1 >= sp.sort_every) ? 1 : 0;
    const int already = vload(&st->rebuild);
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
        v.x += h * f.x;
        v.y += h * f.y;
        v.z += h * f.z;
        const double tx = v.x * dt, ty = v.y * dt, tz = v.z * dt;
        x.x += tx;
        x.y += ty;
        x.z += tz;
        d.vel[i] = v;
        d.pos[i] = x;
        if (sp.precision == 1)
            need = mixed_drift(d, sp, i, x, (float)tx, (float)ty, (float)tz, !already, st->steps_since_build);
        if (sp.kind == 0) {
            double4 w = d.omg[i];
            if (w.w != 0.0) {
                const double4 tq = d.trq[i];
                w.x += 0.5 * dt * tq.x * w.w;
                w.y += 0.5 * dt * tq.y * w.w;
                w.z += 0.5 * dt * tq.z * w.w;
                const double om = sqrt(w.x * w.x + w.y * w.y + w.z * w.z);
                const double angle = om * dt;
                if (angle > 1e-14) {
                    const double inv = 1.0 / om;
                    const double half = angle * 0.5;
                    const double sn = sin(half), cs = cos(half);
                    const double a0 = cs, a1 = w.x * inv * sn, a2 = w.y * inv * sn, a3 = w.z * inv * sn;
                    const double4 q = d.quat[i];
                    double4 r;  // Hamilton product dq * q (rotational.rs:34-41)
                    r.x = a0 * q.x - a1 * q.y - a2 * q.z - a3 * q.w;
                    r.y = a0 * q.y + a1 * q.x + a2 * q.w - a3 * q.z;
                    r.z = a0 * q.z - a1 * q.w + a2 * q.x + a3 * q.y;
                    r.w = a0 * q.w + a1 * q.z - a2 * q.y + a3 * q.x;
                    d.quat[i] = r;
                }
                d.omg[i] = w;
            }
        }
        if (!already && sp.precision == 0) {
            bool disp = false;
            if (sp.every == 0 || sp.check) {
                const double4 b = d.lbp[i];
                double dx = x.x - b.x, dy = x.y - b.y, dz = x.z - b.z;
                const double hbx = sp.L[0] * 0.5, hby = sp.L[1] * 0.5, hbz = sp.L[2] * 0.5;
                if (sp.per[0]) { if (dx > hbx) dx -= sp.L[0]; else if (dx < -hbx) dx += sp.L[0]; }
                if (sp.per[1]) { if (dy > hby) dy -= sp.L[1]; else if (dy < -hby) dy += sp.L[1]; }
                if (sp.per[2]) { if (dz > hbz) dz -= sp.L[2]; else if (dz < -hbz) dz += sp.L[2]; }
                disp = dx * dx + dy * dy + dz * dz > sp.disp_thr_sq;
            }
            if (sp.every == 0) need = disp;
            else if (sp.check) need = (st->steps_since_build >= sp.every) || disp;
            else need = st->steps_since_build >= sp.every;
            if (!need && sp.policy == 0)
                need = (sp.per[0] && (x.x < sp.lo[0] || x.x >= sp.hi[0])) ||
                       (sp.per[1] && (x.y < sp.lo[1] || x.y >= sp.hi[1])) ||
                       (sp.per[2] && (x.z < sp.lo[2] || x.z >= sp.hi[2]));
        }
    }
    if (__any_sync(0xffffffffu, need) && (threadIdx.x & 31) == 0) atomicOr(&st->rebuild, 1);
    if (d.use_cond) {
        // grid-wide last block: open the rebuild branch of the step graph only
        // when some system rebuilds or sorts
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
            for (int q = 0; q < d.nsys; q++)
                if (sys_active(d.ss + q)) any |= (unsigned)(vload(&d.ss[q].rebuild) | vload(&d.ss[q].periodic_sort));
            *d.grid_ctr = 0;
            if (any) d.stat_ctr[0] += 1;
            cudaGraphSetConditional((cudaGraphConditionalHandle)d.cond, any ? 1u : 0u);
        }
    }
}

// ----------------------------------------------------------------------------
// rebuild pipeline
// ----------------------------------------------------------------------------


// Exclusive block-wide scan (1024 threads) of one int; total to `tot`.
__device__ __forceinline__ int block_scan1024(int v, int* wsum, int& tot) {
    const int t = threadIdx.x;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((t & 31) >= o) x += y;
    }
    if ((t & 31) == 31) wsum[t >> 5] = x;
    __syncthreads();
    if (t < 32) {
        int w = wsum[t];
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (t >= o) w += y;
        }
        wsum[t] = w;
    }
    __syncthreads();
    const int incl = x + ((t >> 5) ? wsum[(t >> 5) - 1] : 0);
    tot = wsum[31];
    __syncthreads();
    return incl - v;
}

// Rebuild work list of this step (one block of 1024 threads): the running
// systems that sort or rebuild, in ascending order, with the prefix offsets
// of their particle blocks and cell blocks.
__global__ void __launch_bounds__(1024) k_rb_plan(Dev d) {
    __shared__ int wsum[32];
    const int t = threadIdx.x;
    int cn = 0, cp = 0, cc = 0;  // carries (uniform across the block)
    for (int base = 0; base < d.nrun_sys; base += 1024) {
        const int k = base + t;
        const int s = k < d.nrun_sys ? d.run_sys[k] : -1;
        const bool f = s >= 0 && do_sort(d.ss + s);
        const int np = f ? d.sp[s].nb : 0, nc = f ? d.sp[s].ncb : 0;
        int tn, tp, tc;
        const int en = block_scan1024(f ? 1 : 0, wsum, tn);
        const int ep = block_scan1024(np, wsum, tp);
        const int ec = block_scan1024(nc, wsum, tc);
        if (f) {
            d.rb_sys[cn + en] = s;
            d.rb_poff[cn + en] = cp + ep;
            d.rb_coff[cn + en] = cc + ec;
        }
        cn += tn;
        cp += tp;
        cc += tc;
    }
    if (t == 0) {
        d.rb_poff[cn] = cp;
        d.rb_coff[cn] = cc;
        *d.rb_n = cn;
    }
}

// pbc (domain.rs:413-459, rebuild steps only) + bin key (neighbor.rs:721-738)
__device__ __forceinline__ void cells_block(const Dev& d, int s, int lb) {
    const SysParams& sp = d.sp[s];
    const SysState* st = d.ss + s;
    if (!do_sort(st)) return;  // uniform over the block
    const int li = lb * BLK + threadIdx.x;
    int key = -1;  // global cell block of the particle's cell
    if (li < sp.n) {
        const long long i = (long long)sp.p0 + li;
        double4 x = d.pos[i];
        if (vload(&st->rebuild)) {
            int4 im = d.img[i];
            const double hx = sp.lo[0] + sp.L[0], hy = sp.lo[1] + sp.L[1], hz = sp.lo[2] + sp.L[2];
            // wrap on periodic axes only; on a fixed axis a particle outside the box
            // (which pbc's slow path, domain.rs:434-452, removes) is an error
            if ((!sp.per[0] && (x.x < sp.lo[0] || x.x >= sp.hi[0])) || (!sp.per[1] && (x.y < sp.lo[1] || x.y >= sp.hi[1])) ||
                (!sp.per[2] && (x.z < sp.lo[2] || x.z >= sp.hi[2])))
                atomicOr(&d.ss[s].status, ST_LOST);
            if (sp.per[0]) { if (x.x < sp.lo[0]) { x.x += sp.L[0]; im.x -= 1; } else if (x.x >= hx) { x.x -= sp.L[0]; im.x += 1; } }
            if (sp.per[1]) { if (x.y < sp.lo[1]) { x.y += sp.L[1]; im.y -= 1; } else if (x.y >= hy) { x.y -= sp.L[1]; im.y += 1; } }
            if (sp.per[2]) { if (x.z < sp.lo[2]) { x.z += sp.L[2]; im.z -= 1; } else if (x.z >= hz) { x.z -= sp.L[2]; im.z += 1; } }
            d.pos[i] = x;
            d.img[i] = im;
        }
        const int cx = ext_cell_1d(x.x, sp.origin[0], sp.inv_bin[0], sp.ext[0]);
        const int cy = ext_cell_1d(x.y, sp.origin[1], sp.inv_bin[1], sp.ext[1]);
        const int cz = ext_cell_1d(x.z, sp.origin[2], sp.inv_bin[2], sp.ext[2]);
        const int flat = (cx * sp.ext[1] + cy) * sp.ext[2] + cz;
        d.cell[i] = flat;
        atomicAdd(&d.cnt[sp.c0 + flat], 1);
        key = d.cblk0[s] + flat / BLK;
    }
    // particle counts per 128-cell block, aggregated over the warp (particles
    // are in bin order after the first sort, so a warp mostly shares one block)
    const unsigned int grp = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&d.csum[key], __popc(grp));
}
__global__ void __launch_bounds__(BLK) k_cells(Dev d) RB_FOR_PARTICLE_BLOCKS(cells_block)

// Cell starts in two levels.  k_scan: per listed system (one block), the
// exclusive scan of its 128-cell block counts (k_cells' csum) -> block bases
// (absolute particle offsets); csum is cleared for the next rebuild.
// k_cellscan: per cell block, the scan of its 128 counts + the block base ->
// cstart (with the sentinel cstart[ncell] = p0 + n); counts are reset for use
// as scatter cursors.
__device__ void scan_system(const Dev& d, int s) {
    const SysParams& sp = d.sp[s];
    if (!do_sort(d.ss + s)) return;
    __shared__ int wsum[32];
    const int t = threadIdx.x;
    const int cb0 = d.cblk0[s];
    int carry = sp.p0;
    for (int base = 0; base < sp.ncb; base += 1024) {
        const int b = base + t;
        const int v = b < sp.ncb ? d.csum[cb0 + b] : 0;
        int tot;
        const int ex = block_scan1024(v, wsum, tot);
        if (b < sp.ncb) {
            d.cbase[cb0 + b] = carry + ex;
            d.csum[cb0 + b] = 0;
        }
        carry += tot;
    }
}
__global__ void __launch_bounds__(1024) k_scan(Dev d) {
    const int rbn = *d.rb_n;
    for (int k = blockIdx.x; k < rbn; k += gridDim.x) scan_system(d, d.rb_sys[k]);
}

__device__ __forceinline__ void cellscan_block(const Dev& d, int s, int lcb, int) {
    const SysParams& sp = d.sp[s];
    if (!do_sort(d.ss + s)) return;  // uniform over the block
    __shared__ int wsum[BLK / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int c = lcb * BLK + t;
    const int v = c < sp.ncell ? d.cnt[sp.c0 + c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int off = d.cbase[d.cblk0[s] + lcb];
    for (int q = 0; q < w; q++) off += wsum[q];
    if (c < sp.ncell) {
        d.cstart[sp.c0 + c] = off + x - v;
        d.cnt[sp.c0 + c] = 0;
    } else if (c == sp.ncell) {
        d.cstart[sp.c0 + c] = off + x - v;  // sentinel: p0 + n
    }
    __syncthreads();
}
__global__ void __launch_bounds__(BLK) k_cellscan(Dev d) RB_FOR_CELL_BLOCKS(cellscan_block, 1)

__device__ __forceinline__ void scatter_block(const Dev& d, int s, int lb) {
    const SysParams& sp = d.sp[s];
    if (!do_sort(d.ss + s)) return;
    const int li = lb * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long i = (long long)sp.p0 + li;
    const int c = d.cell[i];
    const int slot = d.cstart[sp.c0 + c] + atomicAdd(&d.cnt[sp.c0 + c], 1);
    d.perm[slot] = (int)i;
}
__global__ void __launch_bounds__(BLK) k_scatter(Dev d) RB_FOR_PARTICLE_BLOCKS(scatter_block)

// Stable order inside each cell (by old index): the sort of sort_atoms_by_bin
// made stable (documented deviation from sort_unstable_by_key,
// neighbor.rs:740).  Also detects a non-identity permutation, which turns a
// periodic sort into a rebuild (neighbor.rs:784-793).
// One warp per cell: the cell's keys (old indices, distinct) sit in registers,
// CS_K per lane; each key's rank is the count of smaller keys, gathered by
// warp shuffles; the keys are then written at their ranks.  Cells of more
// than 32 * CS_K particles fall back to an insertion sort on lane 0.
constexpr int CS_WARPS = BLK / 32;
constexpr int CS_SUBS = BLK / CS_WARPS;  // blocks per 128-cell block
constexpr int CS_K = 4;
__device__ __forceinline__ void cellsort_cells(const Dev& d, int s, int lcb, int sub) {
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (!do_sort(st)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lcb * BLK + sub * CS_WARPS + warp;
    if (c >= sp.ncell) return;
    const int start = d.cstart[sp.c0 + c];
    const int m = d.cnt[sp.c0 + c];
    int* p = d.perm + start;
    bool ident = true;
    if (m <= 32 * CS_K) {
        int key[CS_K], rank[CS_K];
#pragma unroll
        for (int k = 0; k < CS_K; k++) {
            const int a = lane + 32 * k;
            key[k] = a < m ? p[a] : 0x7fffffff;
            rank[k] = 0;
        }
#pragma unroll
        for (int kk = 0; kk < CS_K; kk++) {
            if (32 * kk >= m) break;  // uniform over the warp
            for (int t = 0; t < 32; t++) {
                const int other = __shfl_sync(0xffffffffu, key[kk], t);
#pragma unroll
                for (int k = 0; k < CS_K; k++) rank[k] += other < key[k] ? 1 : 0;
            }
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < CS_K; k++) {
            const int a = lane + 32 * k;
            if (a < m) {
                p[rank[k]] = key[k];
                if (key[k] != start + rank[k]) ident = false;
            }
        }
        ident = __all_sync(0xffffffffu, ident);
    } else if (lane == 0) {
        for (int a = 1; a < m; a++) {
            const int key = p[a];
            int b = a - 1;
            while (b >= 0 && p[b] > key) {
                p[b + 1] = p[b];
                b--;
            }
            p[b + 1] = key;
        }
        for (int a = 0; a < m; a++)
            if (p[a] != start + a) ident = false;
    }
    if (lane == 0) {
        d.cnt[sp.c0 + c] = 0;
        // one flag per system: read before the atomic, so that a first sort
        // (every cell permuted) does not queue an atomic per cell on one word
        if (!ident && !vload(&st->nonid)) atomicOr(&st->nonid, 1);
    }
}
__global__ void __launch_bounds__(BLK) k_cellsort(Dev d) RB_FOR_CELL_BLOCKS(cellsort_cells, CS_SUBS)

// Atom::apply_permutation + AtomDataRegistry::apply_permutation_all +
// ContactHistoryStore::apply_permutation (atom.rs:383-394, 197-202,
// tangential.rs:92-96): gather every per-atom array into scratch.
__device__ __forceinline__ void gather_block(const Dev& d, int s, int lb) {
    const SysParams& sp = d.sp[s];
    if (!do_rebuild(d.ss + s)) return;
    const int hcur = d.ss[s].hcur;
    const int li = lb * BLK + threadIdx.x;
    if (li == 0 && d.dem_wl_n) d.dem_wl_n[s] = 0;  // the worklist is rebuilt after the list
    if (li >= sp.n) return;
    const long long k = (long long)sp.p0 + li;
    const long long o = d.perm[k];
    d.s_pos[k] = d.pos[o];
    d.s_vel[k] = d.vel[o];
    d.s_mass[k] = d.mass[o];
    d.s_cutr[k] = d.cutr[o];
    d.s_tag[k] = d.tag[o];
    d.s_type[k] = d.type[o];
    d.s_img[k] = d.img[o];
    if (sp.kind == 0) {
        d.s_omg[k] = d.omg[o];
        d.s_quat[k] = d.quat[o];
        if (d.hist_any) {
            const long long lo_ = o - sp.p0;
            const int hc = d.hcnt[hcur][o];
            d.s_hcnt[k] = hc;
            for (int c = 0; c < hc; c++) {
                d.s_htag[sp.h0 + (long long)c * sp.npad + li] = d.htag[hcur][sp.h0 + (long long)c * sp.npad + lo_];
                for (int q = 0; q < 7; q++)
                    d.s_hval[sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + li] =
                        d.hval[hcur][sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + lo_];
            }
        }
    }
}

__global__ void __launch_bounds__(BLK) k_gather(Dev d) RB_FOR_PARTICLE_BLOCKS(gather_block)

__device__ __forceinline__ void copyback_block(const Dev& d, int s, int lb) {
    const SysParams& sp = d.sp[s];
    if (!do_rebuild(d.ss + s)) return;
    const int hcur = d.ss[s].hcur;
    const int li = lb * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long k = (long long)sp.p0 + li;
    const double4 x = d.s_pos[k];
    d.pos[k] = x;
    d.vel[k] = d.s_vel[k];
    d.mass[k] = d.s_mass[k];
    d.cutr[k] = d.s_cutr[k];
    d.tag[k] = d.s_tag[k];
    d.type[k] = d.s_type[k];
    d.img[k] = d.s_img[k];
    if (sp.kind == 0) {
        d.omg[k] = d.s_omg[k];
        d.quat[k] = d.s_quat[k];
        if (d.hist_any) {
            const int hc = d.s_hcnt[k];
            d.hcnt[hcur][k] = hc;
            for (int c = 0; c < hc; c++) {
                d.htag[hcur][sp.h0 + (long long)c * sp.npad + li] = d.s_htag[sp.h0 + (long long)c * sp.npad + li];
                for (int q = 0; q < 7; q++)
                    d.hval[hcur][sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + li] =
                        d.s_hval[sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + li];
            }
        }
    }
    // two-float geometry copy relative to the box corner (list build and the
    // mixed-precision pair kernels); w = cutoff radius
    const double rx = x.x - sp.lo[0], ry = x.y - sp.lo[1], rz = x.z - sp.lo[2];
    const float hx = (float)rx, hy = (float)ry, hz = (float)rz;
    const double cr = d.s_cutr[k];
    const float crh = (float)cr;
    const float4 ph = make_float4(hx, hy, hz, crh);
    const float4 pl = make_float4((float)(rx - (double)hx), (float)(ry - (double)hy), (float)(rz - (double)hz),
                                  (float)(cr - (double)crh));
    d.pos2[2 * k] = ph;
    d.pos2[2 * k + 1] = pl;
    if (sp.precision == 1) {
        d.lbp2[2 * k] = ph;
        d.lbp2[2 * k + 1] = pl;
        if (sp.kind == 1) {
            const uint4 u = fixed_pos(sp, x);
            d.posu[k] = u;
            d.lbpu[k] = u;
        }
    }
    // ext cell in the new order, with a flag when a bin coordinate lies within
    // 1e-9 of a bin edge (the list build then recomputes image cells in fp64)
    const double ux = (x.x - sp.origin[0]) * sp.inv_bin[0];
    const double uy = (x.y - sp.origin[1]) * sp.inv_bin[1];
    const double uz = (x.z - sp.origin[2]) * sp.inv_bin[2];
    const int cx = min(max((int)floor(ux), 0), sp.ext[0] - 1);
    const int cy = min(max((int)floor(uy), 0), sp.ext[1] - 1);
    const int cz = min(max((int)floor(uz), 0), sp.ext[2] - 1);
    const double fx = ux - floor(ux), fy = uy - floor(uy), fz = uz - floor(uz);
    const bool edge = fx < 1e-9 || fx > 1.0 - 1e-9 || fy < 1e-9 || fy > 1.0 - 1e-9 || fz < 1e-9 || fz > 1.0 - 1e-9;
    d.cell[k] = ((cx * sp.ext[1] + cy) * sp.ext[2] + cz) | (edge ? (int)0x80000000u : 0);
}
__global__ void __launch_bounds__(BLK) k_copyback(Dev d) RB_FOR_PARTICLE_BLOCKS(copyback_block)

// Stencil membership of a cell offset (compute_bin_grid's distance test,
// neighbor.rs:341-361, tabulated on the host).
__device__ __forceinline__ bool stencil_ok(const SysParams& sp, int dx, int dy, int dz) {
    if (abs(dx) > sp.sl[0] || abs(dy) > sp.sl[1] || abs(dz) > sp.sl[2]) return false;
    const int wy = 2 * sp.sl[1] + 1, wz = 2 * sp.sl[2] + 1;
    const int b = ((dx + sp.sl[0]) * wy + (dy + sp.sl[1])) * wz + (dz + sp.sl[2]);
    return (sp.stencil_bits[b >> 5] >> (b & 31)) & 1u;
}

// Owner rule of the reference's half list (bin_neighbor_list,
// neighbor.rs:938-1065): local `o`, in ext cell eo, scanning its self cell
// (entries after it in bin order) and its forward stencil cells finds the
// image of `p` that lies in ext cell g.  `ghost`: the image is a periodic copy
// (ghosts follow all locals in bin order).  newton=false: full stencil, all
// entries but self.
__device__ __forceinline__ bool owner_test(const SysParams& sp, int eox, int eoy, int eoz, int gx, int gy,
                                           int gz, bool ghost, long long o, long long p) {
    const int dx = gx - eox, dy = gy - eoy, dz = gz - eoz;
    if (!stencil_ok(sp, dx, dy, dz)) return false;
    const long long flat = ((long long)dx * sp.ext[1] + dy) * sp.ext[2] + dz;
    if (sp.newton) {
        if (flat > 0) return true;
        if (flat < 0) return false;
        return ghost || p > o;
    }
    return !(flat == 0 && !ghost && p == o);
}

// uniform: r2 < (2 r sf)^2; polydisperse: r2 < (s_i + s_j)^2 sf^2 (neighbor.rs:959-1060)
__device__ __forceinline__ bool cut_ok(const SysParams& sp, double r2, double so, double sq) {
    if (sp.uniform) return r2 < sp.uniform_cutoff_sq;
    const double ss = so + sq;
    return r2 < ss * ss * sp.sf2;
}

// ext cell of an image coordinate (fp64, exactly as the reference bins ghosts)
__device__ __forceinline__ void ext_cell3(const SysParams& sp, double x, double y, double z, int& cx, int& cy,
                                          int& cz) {
    cx = ext_cell_1d(x, sp.origin[0], sp.inv_bin[0], sp.ext[0]);
    cy = ext_cell_1d(y, sp.origin[1], sp.inv_bin[1], sp.ext[1]);
    cz = ext_cell_1d(z, sp.origin[2], sp.inv_bin[2], sp.ext[2]);
}

// Owner-rule decisions that depend only on the pair of bins: for a tile of
// candidates from source bin E (image shift s) seen from centre bin e.
struct TileRule {
    bool own;   // centre particle owns every pair of the tile
    bool oth;   // every candidate owns its pair with the centre particle
    bool same;  // same bin, no shift: ownership by index order
};

__device__ __forceinline__ TileRule tile_rule(const SysParams& sp, int ex, int ey, int ez, int Ex, int Ey, int Ez,
                                              int sx, int sy, int sz) {
    TileRule r{false, false, false};
    if (!(sx | sy | sz)) {
        const int dx = Ex - ex, dy = Ey - ey, dz = Ez - ez;
        if (!stencil_ok(sp, dx, dy, dz)) return r;
        const int flat = (dx * sp.ext[1] + dy) * sp.ext[2] + dz;
        if (!sp.newton) {
            r.own = true;  // full stencil; self excluded per pair
            r.same = flat == 0;
            return r;
        }
        r.own = flat > 0;
        r.oth = flat < 0;
        r.same = flat == 0;
        return r;
    }
    // periodic image: image bin of the candidate g, image bin of the centre h
    const int gx = min(max(Ex + sx * sp.nc[0], 0), sp.ext[0] - 1);
    const int gy = min(max(Ey + sy * sp.nc[1], 0), sp.ext[1] - 1);
    const int gz = min(max(Ez + sz * sp.nc[2], 0), sp.ext[2] - 1);
    const int hx = min(max(ex - sx * sp.nc[0], 0), sp.ext[0] - 1);
    const int hy = min(max(ey - sy * sp.nc[1], 0), sp.ext[1] - 1);
    const int hz = min(max(ez - sz * sp.nc[2], 0), sp.ext[2] - 1);
    r.own = owner_test(sp, ex, ey, ez, gx, gy, gz, true, 0, 1);
    r.oth = sp.newton && owner_test(sp, Ex, Ey, Ez, hx, hy, hz, true, 0, 1);
    return r;
}

// Neighbour list build.  Each particle walks the interior-cell window of its
// bin (with periodic image shifts) in the reference's stencil order; every
// candidate is screened by an fp32 test on the hi parts (conservative
// radius); survivors get the two-float separation, and the reference's own
// fp64 cutoff test (fma form) only within 1e-5 of the cutoff.  The
// reference's owner rule is applied twice: `own` (i holds the pair in the
// reference's half list) and `oth` (the partner holds it); both go into i's
// full row, so forces are summed per particle without atomics while pair
// arithmetic stays in the owner's frame.  Owner decisions depend only on the
// two bins (the tile rule) except for same-bin order and for particles within
// 1e-9 of a bin edge, whose image bins are recomputed in fp64.  Three modes
// give identical rows: a warp per bin (lanes over the bin's particles, for
// systems with enough bins to fill the GPU), a warp per particle (lanes over
// candidates, rows written in order by ballot, for small dense systems) and a
// thread per particle (dilute systems).  Also saves last_build_pos
// (neighbor.rs:545-561).
constexpr int BUILD_WARPS = 4;

// The survivors of the fp32 screen that lie near the cutoff, or that involve
// a particle within 1e-9 of a bin edge under a periodic shift: two-float
// separation, the reference's own fp64 cutoff test (fma form) inside the
// band, and image bins recomputed in fp64 for edge particles.  Returns bit 0
// when i owns the pair in the reference's half list, bit 1 when j does.
// Kept out of line: it is rare, and inlined it would set the register count
// of the whole build loop.
__device__ __noinline__ int near_pair(const Dev& d, const SysParams& sp, long long i, long long j, float4 hi, float4 lo,
                                      float4 hj, float4 lj, int sx, int sy, int sz, bool edge, int ex, int ey, int ez,
                                      int Ex, int Ey, int Ez, TileRule tr) {
    const float band_hi = 1.00001f, band_lo = 0.99999f;
    bool ok_i = true, ok_j = true;
    const float fx = two_float_sep(hj.x, lj.x, hi.x, lo.x, sx, sp.Lh[0], sp.Ll[0]);
    const float fy = two_float_sep(hj.y, lj.y, hi.y, lo.y, sy, sp.Lh[1], sp.Ll[1]);
    const float fz = two_float_sep(hj.z, lj.z, hi.z, lo.z, sz, sp.Lh[2], sp.Ll[2]);
    const float r2f = fx * fx + fy * fy + fz * fz;
    float c2f;
    if (sp.uniform) {
        c2f = sp.ucut2f;
    } else {
        const float ssum = hi.w + hj.w;
        c2f = ssum * ssum * sp.sf2f;
    }
    if (r2f > c2f * band_hi) return 0;
    if (r2f >= c2f * band_lo || edge) {
        const double4 xi = d.pos[i], xj = d.pos[j];
        const double si = d.cutr[i], sj = d.cutr[j];
        if (r2f >= c2f * band_lo) {
            // the reference's own test, in its own arithmetic
            const double dx = img_coord(xj.x, sx, sp.L[0]) - xi.x;
            const double dy = img_coord(xj.y, sy, sp.L[1]) - xi.y;
            const double dz = img_coord(xj.z, sz, sp.L[2]) - xi.z;
            ok_i = cut_ok(sp, fma(dx, dx, fma(dy, dy, dz * dz)), si, sj);
            if (sx | sy | sz) {
                const double ux = img_coord(xi.x, -sx, sp.L[0]) - xj.x;
                const double uy = img_coord(xi.y, -sy, sp.L[1]) - xj.y;
                const double uz = img_coord(xi.z, -sz, sp.L[2]) - xj.z;
                ok_j = cut_ok(sp, fma(ux, ux, fma(uy, uy, uz * uz)), sj, si);
            } else {
                ok_j = ok_i;
            }
            if (!ok_i && !ok_j) return 0;
        }
        if (edge) {
            int gx, gy, gz, hx, hy, hz;
            ext_cell3(sp, img_coord(xj.x, sx, sp.L[0]), img_coord(xj.y, sy, sp.L[1]), img_coord(xj.z, sz, sp.L[2]),
                      gx, gy, gz);
            ext_cell3(sp, img_coord(xi.x, -sx, sp.L[0]), img_coord(xi.y, -sy, sp.L[1]), img_coord(xi.z, -sz, sp.L[2]),
                      hx, hy, hz);
            const bool own = ok_i && owner_test(sp, ex, ey, ez, gx, gy, gz, true, i, j);
            const bool oth = sp.newton && ok_j && owner_test(sp, Ex, Ey, Ez, hx, hy, hz, true, j, i);
            return (own ? 1 : 0) | (oth ? 2 : 0);
        }
    }
    const bool own = ok_i && (tr.own || (tr.same && (sp.newton ? j > i : true)));
    const bool oth = ok_j && (tr.oth || (tr.same && sp.newton && i > j));
    return (own ? 1 : 0) | (oth ? 2 : 0);
}

constexpr int BUILD_SUBS = BLK / BUILD_WARPS;  // work units per 128-particle block (BUILD_WARPS warps each)

// Row of particle li of system s by one thread (dilute systems, and the
// rare particles whose window has particles in ghost-layer bins).
__device__ __noinline__ void build_one(const Dev& d, int s, int li) {
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    const long long i = (long long)sp.p0 + li;
    d.lbp[i] = d.pos[i];
    const float4 hi = d.pos2[2 * i], lo = d.pos2[2 * i + 1];
    const int cr = d.cell[i];
    const bool edge_i = cr < 0;
    const int c = cr & 0x7fffffff;
    const int ez = c % sp.ext[2];
    const int ey = (c / sp.ext[2]) % sp.ext[1];
    const int ex = c / (sp.ext[2] * sp.ext[1]);
    const int qx0 = min(max(ex - sp.sl[0], 0), sp.nc[0] - 1);
    const int qy0 = min(max(ey - sp.sl[1], 0), sp.nc[1] - 1);
    const int qz0 = min(max(ez - sp.sl[2], 0), sp.nc[2] - 1);
    const float brel = sp.band_rel;
    const long long base = sp.lst0 + li;
    int count = 0;
    for (int ox = -sp.win[0]; ox <= sp.win[0]; ox++) {
        int qx = qx0 + ox, sx = 0;
        if (qx < 0) { qx += sp.nc[0]; sx = -1; } else if (qx >= sp.nc[0]) { qx -= sp.nc[0]; sx = 1; }
        if (sx && !sp.per[0]) continue;  // fixed axis: no periodic image
        if (qx < 0 || qx >= sp.nc[0]) continue;
        for (int oy = -sp.win[1]; oy <= sp.win[1]; oy++) {
            int qy = qy0 + oy, sy = 0;
            if (qy < 0) { qy += sp.nc[1]; sy = -1; } else if (qy >= sp.nc[1]) { qy -= sp.nc[1]; sy = 1; }
            if (sy && !sp.per[1]) continue;
            if (qy < 0 || qy >= sp.nc[1]) continue;
            for (int oz = -sp.win[2]; oz <= sp.win[2]; oz++) {
                int qz = qz0 + oz, sz = 0;
                if (qz < 0) { qz += sp.nc[2]; sz = -1; } else if (qz >= sp.nc[2]) { qz -= sp.nc[2]; sz = 1; }
                if (sz && !sp.per[2]) continue;
                if (qz < 0 || qz >= sp.nc[2]) continue;
                const bool shifted = (sx | sy | sz) != 0;
                const uint32_t sc = (uint32_t)((sx + 1) * 9 + (sy + 1) * 3 + (sz + 1));
                const float hsx = hi.x - (float)sx * sp.Lh[0];
                const float hsy = hi.y - (float)sy * sp.Lh[1];
                const float hsz = hi.z - (float)sz * sp.Lh[2];
                const int axa = (qx == 0) ? -1 : 0, axb = (qx == sp.nc[0] - 1) ? 1 : 0;
                const int aya = (qy == 0) ? -1 : 0, ayb = (qy == sp.nc[1] - 1) ? 1 : 0;
                const int aza = (qz == 0) ? -1 : 0, azb = (qz == sp.nc[2] - 1) ? 1 : 0;
                for (int ax = axa; ax <= axb; ax++)
                    for (int ay = aya; ay <= ayb; ay++)
                        for (int az = aza; az <= azb; az++) {
                            const int Ex = qx + sp.sl[0] + ax, Ey = qy + sp.sl[1] + ay, Ez = qz + sp.sl[2] + az;
                            const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
                            const int m0 = d.cstart[sp.c0 + flatE], m1 = d.cstart[sp.c0 + flatE + 1];
                            if (m0 == m1) continue;
                            const TileRule tr = tile_rule(sp, ex, ey, ez, Ex, Ey, Ez, sx, sy, sz);
                            if (!tr.own && !tr.oth && !tr.same && !shifted) continue;
                            for (int jj = m0; jj < m1; jj++) {
                                const long long j = jj;
                                if (!shifted && j == i) continue;
                                const float4 hj = d.pos2[2 * j];
                                const float px = hj.x - hsx, py = hj.y - hsy, pz = hj.z - hsz;
                                const float r2h = px * px + py * py + pz * pz;
                                float c2h;
                                if (sp.uniform) {
                                    c2h = sp.ucut2f;
                                } else {
                                    const float ssum = hi.w + hj.w;
                                    c2h = ssum * ssum * sp.sf2f;
                                }
                                if (!(r2h <= c2h * (1.f + brel))) continue;
                                const bool near = r2h > c2h * (1.f - brel);
                                const bool edge = shifted && (edge_i || d.cell[j] < 0);
                                int bits;
                                if (!near && !edge) {
                                    bits = ((tr.own || (tr.same && (sp.newton ? j > i : true))) ? 1 : 0) |
                                           ((tr.oth || (tr.same && sp.newton && i > j)) ? 2 : 0);
                                } else {
                                    bits = near_pair(d, sp, i, j, hi, lo, hj, d.pos2[2 * j + 1], sx, sy, sz, edge, ex,
                                                     ey, ez, Ex, Ey, Ez, tr);
                                }
                                const uint32_t jl = (uint32_t)(j - sp.p0);
                                if (bits & 1) {
                                    if (count < sp.ncap)
                                        d.nlist[base + (long long)count * sp.npad] = jl | ((sc + 27u) << IDX_BITS);
                                    count++;
                                }
                                if (bits & 2) {
                                    if (count < sp.ncap) d.nlist[base + (long long)count * sp.npad] = jl | (sc << IDX_BITS);
                                    count++;
                                }
                            }
                        }
            }
        }
    }
    if (count > sp.ncap) {
        atomicOr(&st->status, ST_NBR_OVF);
        atomicMax(&st->max_nbr, count);
        count = sp.ncap;
    } else if (count > vload(&st->max_nbr)) {  // skip the atomic on one word when it cannot raise it
        atomicMax(&st->max_nbr, count);
    }
    d.nnum[i] = count;
}

// One warp per bin: bin `sub * BUILD_WARPS + warp` of cell block `lcb` of
// system s.  Warp-synchronous only (no block barrier), so warps may leave early.
// One warp per bin (large dense systems): bin `sub * BUILD_WARPS + warp` of
// block `lcb` of system s; the lanes are the bin's particles, 32 at a time.
// Warp-synchronous only (no block barrier), so warps may leave early.
__device__ __noinline__ void build_cells(const Dev& d, int s, int lcb, int sub) {
    __shared__ float4 tile_h[BUILD_WARPS][32], tile_l[BUILD_WARPS][32];
    __shared__ int tile_e[BUILD_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (!do_rebuild(st)) return;
    const int c = lcb * BLK + sub * BUILD_WARPS + warp;
    if (c >= sp.ncell) return;
    const int a0 = d.cstart[sp.c0 + c], a1 = d.cstart[sp.c0 + c + 1];
    if (a0 == a1) return;
    const int ez = c % sp.ext[2];
    const int ey = (c / sp.ext[2]) % sp.ext[1];
    const int ex = c / (sp.ext[2] * sp.ext[1]);
    const int qx0 = min(max(ex - sp.sl[0], 0), sp.nc[0] - 1);
    const int qy0 = min(max(ey - sp.sl[1], 0), sp.nc[1] - 1);
    const int qz0 = min(max(ez - sp.sl[2], 0), sp.nc[2] - 1);
    const float brel = sp.band_rel;
    for (int ib = a0; ib < a1; ib += 32) {
        const long long i = ib + lane;
        const bool act = i < a1;
        float4 hi = make_float4(0, 0, 0, 0), lo = make_float4(0, 0, 0, 0);
        bool edge_i = false;
        if (act) {
            d.lbp[i] = d.pos[i];
            hi = d.pos2[2 * i];
            lo = d.pos2[2 * i + 1];
            edge_i = d.cell[i] < 0;
        }
        const long long base = sp.lst0 + (i - sp.p0);
        int count = 0;
        // the window's cells in the reference's stencil order (ox, oy, oz
        // ascending), 32 at a time: lane k describes entry e0 + k -- validity,
        // periodic shift, boundary flags, its interior cell's ext index and
        // particle range, and the tile rule -- so the warp walks the window
        // with shuffles instead of dependent loads per cell
        const int wy = 2 * sp.win[1] + 1, wz = 2 * sp.win[2] + 1;
        const int nent = (2 * sp.win[0] + 1) * wy * wz;
        for (int e0 = 0; e0 < nent; e0 += 32) {
            int eq = 0, eE = 0, em0 = 0, em1 = 0;
            {
                const int e = e0 + lane;
                if (e < nent) {
                    int qx = qx0 + e / (wy * wz) - sp.win[0], sx = 0;
                    int qy = qy0 + (e / wz) % wy - sp.win[1], sy = 0;
                    int qz = qz0 + e % wz - sp.win[2], sz = 0;
                    if (qx < 0) { qx += sp.nc[0]; sx = -1; } else if (qx >= sp.nc[0]) { qx -= sp.nc[0]; sx = 1; }
                    if (qy < 0) { qy += sp.nc[1]; sy = -1; } else if (qy >= sp.nc[1]) { qy -= sp.nc[1]; sy = 1; }
                    if (qz < 0) { qz += sp.nc[2]; sz = -1; } else if (qz >= sp.nc[2]) { qz -= sp.nc[2]; sz = 1; }
                    // fixed axes have no periodic image
                    const bool ok = !(sx && !sp.per[0]) && !(sy && !sp.per[1]) && !(sz && !sp.per[2]) && qx >= 0 &&
                                    qx < sp.nc[0] && qy >= 0 && qy < sp.nc[1] && qz >= 0 && qz < sp.nc[2];
                    if (ok) {
                        const int Ex = qx + sp.sl[0], Ey = qy + sp.sl[1], Ez = qz + sp.sl[2];
                        const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
                        em0 = d.cstart[sp.c0 + flatE];
                        em1 = d.cstart[sp.c0 + flatE + 1];
                        const TileRule tr = tile_rule(sp, ex, ey, ez, Ex, Ey, Ez, sx, sy, sz);
                        eE = flatE;
                        eq = 1 | ((sx + 1) << 1) | ((sy + 1) << 3) | ((sz + 1) << 5) | (qx == 0 ? 1 << 7 : 0) |
                             (qx == sp.nc[0] - 1 ? 1 << 8 : 0) | (qy == 0 ? 1 << 9 : 0) |
                             (qy == sp.nc[1] - 1 ? 1 << 10 : 0) | (qz == 0 ? 1 << 11 : 0) |
                             (qz == sp.nc[2] - 1 ? 1 << 12 : 0) | (tr.own ? 1 << 13 : 0) | (tr.oth ? 1 << 14 : 0) |
                             (tr.same ? 1 << 15 : 0);
                    }
                }
            }
            const int ne = min(32, nent - e0);
            for (int k = 0; k < ne; k++) {
                const int q = __shfl_sync(0xffffffffu, eq, k);
                const int qE = __shfl_sync(0xffffffffu, eE, k);
                const int qm0 = __shfl_sync(0xffffffffu, em0, k);
                const int qm1 = __shfl_sync(0xffffffffu, em1, k);
                if (!(q & 1)) continue;  // uniform over the warp
                const int sx = ((q >> 1) & 3) - 1, sy = ((q >> 3) & 3) - 1, sz = ((q >> 5) & 3) - 1;
                const int Ez0 = qE % sp.ext[2], Ey0 = (qE / sp.ext[2]) % sp.ext[1], Ex0 = qE / (sp.ext[2] * sp.ext[1]);
                const bool shifted = (sx | sy | sz) != 0;
                const uint32_t sc = (uint32_t)((sx + 1) * 9 + (sy + 1) * 3 + (sz + 1));
                // centre position moved by -s L: the candidate's own hi part
                // then gives the prefilter separation directly
                const float hsx = hi.x - (float)sx * sp.Lh[0];
                const float hsy = hi.y - (float)sy * sp.Lh[1];
                const float hsz = hi.z - (float)sz * sp.Lh[2];
                // an interior cell on the box face also visits the adjacent
                // ghost-layer cells (particles binned there by rounding)
                const int axa = (q >> 7) & 1 ? -1 : 0, axb = (q >> 8) & 1 ? 1 : 0;
                const int aya = (q >> 9) & 1 ? -1 : 0, ayb = (q >> 10) & 1 ? 1 : 0;
                const int aza = (q >> 11) & 1 ? -1 : 0, azb = (q >> 12) & 1 ? 1 : 0;
                for (int ax = axa; ax <= axb; ax++)
                    for (int ay = aya; ay <= ayb; ay++)
                        for (int az = aza; az <= azb; az++) {
                            const int Ex = Ex0 + ax, Ey = Ey0 + ay, Ez = Ez0 + az;
                            int m0, m1;
                            TileRule tr;
                            if ((ax | ay | az) == 0) {
                                m0 = qm0;
                                m1 = qm1;
                                tr = TileRule{((q >> 13) & 1) != 0, ((q >> 14) & 1) != 0, ((q >> 15) & 1) != 0};
                            } else {
                                const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
                                m0 = d.cstart[sp.c0 + flatE];
                                m1 = d.cstart[sp.c0 + flatE + 1];
                                if (m0 == m1) continue;
                                tr = tile_rule(sp, ex, ey, ez, Ex, Ey, Ez, sx, sy, sz);
                            }
                            if (m0 == m1) continue;
                            // nothing in this bin pair can enter the list unless a
                            // bin-edge particle needs its image bin recomputed
                            const bool maybe_edge = shifted;
                            if (!tr.own && !tr.oth && !tr.same && !maybe_edge) continue;
                            for (int t0 = m0; t0 < m1; t0 += 32) {
                                const int nt = min(32, m1 - t0);
                                __syncwarp();
                                if (lane < nt) {
                                    tile_h[warp][lane] = d.pos2[2 * (long long)(t0 + lane)];
                                    tile_l[warp][lane] = d.pos2[2 * (long long)(t0 + lane) + 1];
                                    tile_e[warp][lane] = d.cell[t0 + lane] < 0;
                                }
                                __syncwarp();
                                if (!act) continue;
                                // pass 1: hi-part fp32 screen of the whole tile into two bit
                                // masks: clearly inside the cutoff / near it (precise path)
                                unsigned int mask = 0u, near = 0u;
        #pragma unroll 4
                                for (int t = 0; t < nt; t++) {
                                    const float4 hj = tile_h[warp][t];
                                    const float px = hj.x - hsx, py = hj.y - hsy, pz = hj.z - hsz;
                                    const float r2h = px * px + py * py + pz * pz;
                                    float c2h;
                                    if (sp.uniform) {
                                        c2h = sp.ucut2f;
                                    } else {
                                        const float ssum = hi.w + hj.w;
                                        c2h = ssum * ssum * sp.sf2f;
                                    }
                                    mask |= (r2h <= c2h * (1.f + brel) ? 1u : 0u) << t;
                                    near |= (r2h > c2h * (1.f - brel) ? 1u : 0u) << t;
                                }
                                if (!shifted && i >= t0 && i < t0 + nt) mask &= ~(1u << (int)(i - t0));
                                // pass 2: survivors only
                                while (mask) {
                                    const int t = __ffs(mask) - 1;
                                    mask &= mask - 1u;
                                    const long long j = t0 + t;
                                    const bool edge = shifted && (edge_i || tile_e[warp][t] != 0);
                                    int bits;
                                    if (!((near >> t) & 1u) && !edge) {
                                        // clearly inside: owner decision only
                                        bits = ((tr.own || (tr.same && (sp.newton ? j > i : true))) ? 1 : 0) |
                                               ((tr.oth || (tr.same && sp.newton && i > j)) ? 2 : 0);
                                    } else {
                                        bits = near_pair(d, sp, i, j, hi, lo, tile_h[warp][t], tile_l[warp][t], sx, sy,
                                                         sz, edge, ex, ey, ez, Ex, Ey, Ez, tr);
                                    }
                                    const uint32_t jl = (uint32_t)(j - sp.p0);
                                    if (bits & 1) {
                                        if (count < sp.ncap)
                                            d.nlist[base + (long long)count * sp.npad] = jl | ((sc + 27u) << IDX_BITS);
                                        count++;
                                    }
                                    if (bits & 2) {
                                        if (count < sp.ncap)
                                            d.nlist[base + (long long)count * sp.npad] = jl | (sc << IDX_BITS);
                                        count++;
                                    }
                                }
                            }
                        }
            }
        }
        if (act) {
            if (count > sp.ncap) {
                atomicOr(&st->status, ST_NBR_OVF);
                atomicMax(&st->max_nbr, count);
                count = sp.ncap;
            } else if (count > vload(&st->max_nbr)) {  // skip the atomic on one word when it cannot raise it
                atomicMax(&st->max_nbr, count);
            }
            d.nnum[i] = count;
        }
    }
}

// Row of particle li of system s by one warp: lane k describes window entry
// e0 + k (its main bin's particle range, shift and tile rule); the entries'
// candidates are laid end to end and screened 32 at a time, one per lane;
// hits are written in candidate order at ballot offsets.  A window with
// particles in a ghost-layer bin (rounding at the box face) falls back to
// build_one on lane 0.
__device__ __noinline__ void build_warp(const Dev& d, int s, int li) {
    __shared__ int s_pre[BUILD_WARPS][33], s_m0[BUILD_WARPS][32], s_q[BUILD_WARPS][32], s_E[BUILD_WARPS][32];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long i = (long long)sp.p0 + li;
    const int cr = d.cell[i];
    const bool edge_i = cr < 0;
    const int c = cr & 0x7fffffff;
    const int ez = c % sp.ext[2];
    const int ey = (c / sp.ext[2]) % sp.ext[1];
    const int ex = c / (sp.ext[2] * sp.ext[1]);
    const int qx0 = min(max(ex - sp.sl[0], 0), sp.nc[0] - 1);
    const int qy0 = min(max(ey - sp.sl[1], 0), sp.nc[1] - 1);
    const int qz0 = min(max(ez - sp.sl[2], 0), sp.nc[2] - 1);
    const int wy = 2 * sp.win[1] + 1, wz = 2 * sp.win[2] + 1;
    const int nent = (2 * sp.win[0] + 1) * wy * wz;
    // first pass: any particle in a ghost-layer bin next to a face cell?
    bool ghost = false;
    for (int e = lane; e < nent; e += 32) {
        int qx = qx0 + e / (wy * wz) - sp.win[0];
        int qy = qy0 + (e / wz) % wy - sp.win[1];
        int qz = qz0 + e % wz - sp.win[2];
        if (qx < 0) qx += sp.nc[0]; else if (qx >= sp.nc[0]) qx -= sp.nc[0];
        if (qy < 0) qy += sp.nc[1]; else if (qy >= sp.nc[1]) qy -= sp.nc[1];
        if (qz < 0) qz += sp.nc[2]; else if (qz >= sp.nc[2]) qz -= sp.nc[2];
        if (qx < 0 || qx >= sp.nc[0] || qy < 0 || qy >= sp.nc[1] || qz < 0 || qz >= sp.nc[2]) continue;
        const int axa = (qx == 0) ? -1 : 0, axb = (qx == sp.nc[0] - 1) ? 1 : 0;
        const int aya = (qy == 0) ? -1 : 0, ayb = (qy == sp.nc[1] - 1) ? 1 : 0;
        const int aza = (qz == 0) ? -1 : 0, azb = (qz == sp.nc[2] - 1) ? 1 : 0;
        for (int ax = axa; ax <= axb; ax++)
            for (int ay = aya; ay <= ayb; ay++)
                for (int az = aza; az <= azb; az++) {
                    if ((ax | ay | az) == 0) continue;
                    const int Ex = qx + sp.sl[0] + ax, Ey = qy + sp.sl[1] + ay, Ez = qz + sp.sl[2] + az;
                    const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
                    if (d.cstart[sp.c0 + flatE] != d.cstart[sp.c0 + flatE + 1]) ghost = true;
                }
    }
    if (__any_sync(0xffffffffu, ghost)) {
        if (lane == 0) build_one(d, s, li);
        return;
    }
    if (lane == 0) d.lbp[i] = d.pos[i];
    const float4 hi = d.pos2[2 * i], lo = d.pos2[2 * i + 1];
    const float brel = sp.band_rel;
    const long long base = sp.lst0 + li;
    int count = 0;  // uniform over the warp
    for (int e0 = 0; e0 < nent; e0 += 32) {
        int nseg = 0, eq = 0, eE = 0, em0 = 0;
        {
            const int e = e0 + lane;
            if (e < nent) {
                int qx = qx0 + e / (wy * wz) - sp.win[0], sx = 0;
                int qy = qy0 + (e / wz) % wy - sp.win[1], sy = 0;
                int qz = qz0 + e % wz - sp.win[2], sz = 0;
                if (qx < 0) { qx += sp.nc[0]; sx = -1; } else if (qx >= sp.nc[0]) { qx -= sp.nc[0]; sx = 1; }
                if (qy < 0) { qy += sp.nc[1]; sy = -1; } else if (qy >= sp.nc[1]) { qy -= sp.nc[1]; sy = 1; }
                if (qz < 0) { qz += sp.nc[2]; sz = -1; } else if (qz >= sp.nc[2]) { qz -= sp.nc[2]; sz = 1; }
                // fixed axes have no periodic image
                const bool ok = !(sx && !sp.per[0]) && !(sy && !sp.per[1]) && !(sz && !sp.per[2]) && qx >= 0 &&
                                qx < sp.nc[0] && qy >= 0 && qy < sp.nc[1] && qz >= 0 && qz < sp.nc[2];
                if (ok) {
                    const int Ex = qx + sp.sl[0], Ey = qy + sp.sl[1], Ez = qz + sp.sl[2];
                    const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
                    const TileRule tr = tile_rule(sp, ex, ey, ez, Ex, Ey, Ez, sx, sy, sz);
                    const bool shifted = (sx | sy | sz) != 0;
                    // nothing in this bin pair can enter the list unless a
                    // bin-edge particle needs its image bin recomputed
                    if (tr.own || tr.oth || tr.same || shifted) {
                        em0 = d.cstart[sp.c0 + flatE];
                        nseg = d.cstart[sp.c0 + flatE + 1] - em0;
                    }
                    eE = flatE;
                    eq = ((sx + 1) << 1) | ((sy + 1) << 3) | ((sz + 1) << 5) | (tr.own ? 1 << 13 : 0) |
                         (tr.oth ? 1 << 14 : 0) | (tr.same ? 1 << 15 : 0);
                }
            }
        }
        // entries' candidates laid end to end: exclusive offsets
        int incl = nseg;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        s_pre[warp][lane] = incl - nseg;
        s_m0[warp][lane] = em0;
        s_q[warp][lane] = eq;
        s_E[warp][lane] = eE;
        if (lane == 0) s_pre[warp][32] = total;
        __syncwarp();
        for (int p0 = 0; p0 < total; p0 += 32) {
            const int p = p0 + lane;
            int bits = 0, sc = 0;
            long long j = 0;
            if (p < total) {
                // the entry holding candidate p: last k with s_pre[k] <= p
                // (entries without candidates share the next one's offset)
                int k = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (k + step < 32 && s_pre[warp][k + step] <= p) k += step;
                const int q = s_q[warp][k];
                j = s_m0[warp][k] + (p - s_pre[warp][k]);
                const int sx = ((q >> 1) & 3) - 1, sy = ((q >> 3) & 3) - 1, sz = ((q >> 5) & 3) - 1;
                const bool shifted = (sx | sy | sz) != 0;
                sc = (sx + 1) * 9 + (sy + 1) * 3 + (sz + 1);
                if (shifted || j != i) {
                    const float4 hj = d.pos2[2 * j];
                    const float px = hj.x - (hi.x - (float)sx * sp.Lh[0]);
                    const float py = hj.y - (hi.y - (float)sy * sp.Lh[1]);
                    const float pz = hj.z - (hi.z - (float)sz * sp.Lh[2]);
                    const float r2h = px * px + py * py + pz * pz;
                    float c2h;
                    if (sp.uniform) {
                        c2h = sp.ucut2f;
                    } else {
                        const float ssum = hi.w + hj.w;
                        c2h = ssum * ssum * sp.sf2f;
                    }
                    if (r2h <= c2h * (1.f + brel)) {
                        const TileRule tr{((q >> 13) & 1) != 0, ((q >> 14) & 1) != 0, ((q >> 15) & 1) != 0};
                        const bool near = r2h > c2h * (1.f - brel);
                        const bool edge = shifted && (edge_i || d.cell[j] < 0);
                        if (!near && !edge) {
                            bits = ((tr.own || (tr.same && (sp.newton ? j > i : true))) ? 1 : 0) |
                                   ((tr.oth || (tr.same && sp.newton && i > j)) ? 2 : 0);
                        } else {
                            const int fE = s_E[warp][k];
                            const int Ez = fE % sp.ext[2], Ey = (fE / sp.ext[2]) % sp.ext[1],
                                      Ex = fE / (sp.ext[2] * sp.ext[1]);
                            bits = near_pair(d, sp, i, j, hi, lo, hj, d.pos2[2 * j + 1], sx, sy, sz, edge, ex, ey, ez,
                                             Ex, Ey, Ez, tr);
                        }
                    }
                }
            }
            // row entries in candidate order: owner entry first, then partner entry
            const int nb = __popc(bits);
            int off = nb;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, off, o);
                if (lane >= o) off += y;
            }
            const int tot = __shfl_sync(0xffffffffu, off, 31);
            int slot = count + off - nb;
            const uint32_t jl = (uint32_t)(j - sp.p0);
            if (bits & 1) {
                if (slot < sp.ncap) d.nlist[base + (long long)slot * sp.npad] = jl | ((uint32_t)(sc + 27) << IDX_BITS);
                slot++;
            }
            if (bits & 2) {
                if (slot < sp.ncap) d.nlist[base + (long long)slot * sp.npad] = jl | ((uint32_t)sc << IDX_BITS);
            }
            count += tot;
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (count > sp.ncap) {
            atomicOr(&st->status, ST_NBR_OVF);
            atomicMax(&st->max_nbr, count);
            count = sp.ncap;
        } else if (count > vload(&st->max_nbr)) {  // skip the atomic on one word when it cannot raise it
            atomicMax(&st->max_nbr, count);
        }
        d.nnum[i] = count;
    }
}

// Candidates one warp stages at a time in build_cells_staged (192: 27 KB of
// shared memory per block, which leaves room for the 6 blocks per SM below).
constexpr int STAGE_CAP = 192;

// One warp per bin, staged (systems with many dense bins): the candidates of
// the bin's window are gathered into shared memory in passes of 32 (every
// lane issues its loads together: one memory latency per pass instead of one
// per window bin), moved by their periodic image, and those farther than the
// list cutoff from the centre bin's box are dropped (no particle of the bin
// can pair with them; about 30 % of a dense window).  The staged candidates
// are screened from shared memory against the bin's particles (the lanes),
// with the system's parameters and each window bin's owner rule and image
// code in registers and shared memory.  Same candidates in the same order as
// build_cells, hence identical rows.  Falls back to build_cells for a window
// of more than 32 bins (bins smaller than the list cutoff) and when a window
// bin on a box face has particles in its adjacent ghost-layer bin (placed
// there by rounding).
__device__ void build_cells_staged(const Dev& d, int s, int lcb, int sub) {
    __shared__ float4 st_p[BUILD_WARPS][STAGE_CAP];  // hi part + image shift, cutoff radius
    __shared__ int st_m[BUILD_WARPS][STAGE_CAP];     // the row entry: local index | image code << 26 | edge << 31
    __shared__ int st_f[BUILD_WARPS][STAGE_CAP];     // own | oth << 1 | same << 2 | shifted << 3 | entry << 4
    __shared__ int st_pre[BUILD_WARPS][33], st_q[BUILD_WARPS][32], st_E[BUILD_WARPS][32], st_m0[BUILD_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (!do_rebuild(st)) return;
    const int c = lcb * BLK + sub * BUILD_WARPS + warp;
    if (c >= sp.ncell) return;
    const int a0 = d.cstart[sp.c0 + c], a1 = d.cstart[sp.c0 + c + 1];
    if (a0 == a1) return;
    const int wy = 2 * sp.win[1] + 1, wz = 2 * sp.win[2] + 1;
    const int nent = (2 * sp.win[0] + 1) * wy * wz;
    if (nent > 32) {  // uniform over the warp
        build_cells(d, s, lcb, sub);
        return;
    }
    const int ez = c % sp.ext[2];
    const int ey = (c / sp.ext[2]) % sp.ext[1];
    const int ex = c / (sp.ext[2] * sp.ext[1]);
    const int qx0 = min(max(ex - sp.sl[0], 0), sp.nc[0] - 1);
    const int qy0 = min(max(ey - sp.sl[1], 0), sp.nc[1] - 1);
    const int qz0 = min(max(ez - sp.sl[2], 0), sp.nc[2] - 1);
    // window entry `lane` (reference stencil order): image shift, tile rule
    // and candidate range of its bin
    int nseg = 0, eq = 0, eE = 0, em0 = 0;
    bool ghost = false;
    if (lane < nent) {
        const int e = lane;
        int qx = qx0 + e / (wy * wz) - sp.win[0], sx = 0;
        int qy = qy0 + (e / wz) % wy - sp.win[1], sy = 0;
        int qz = qz0 + e % wz - sp.win[2], sz = 0;
        if (qx < 0) { qx += sp.nc[0]; sx = -1; } else if (qx >= sp.nc[0]) { qx -= sp.nc[0]; sx = 1; }
        if (qy < 0) { qy += sp.nc[1]; sy = -1; } else if (qy >= sp.nc[1]) { qy -= sp.nc[1]; sy = 1; }
        if (qz < 0) { qz += sp.nc[2]; sz = -1; } else if (qz >= sp.nc[2]) { qz -= sp.nc[2]; sz = 1; }
        const bool ok = !(sx && !sp.per[0]) && !(sy && !sp.per[1]) && !(sz && !sp.per[2]) && qx >= 0 &&
                        qx < sp.nc[0] && qy >= 0 && qy < sp.nc[1] && qz >= 0 && qz < sp.nc[2];
        if (ok) {
            const int Ex = qx + sp.sl[0], Ey = qy + sp.sl[1], Ez = qz + sp.sl[2];
            const int flatE = (Ex * sp.ext[1] + Ey) * sp.ext[2] + Ez;
            const TileRule tr = tile_rule(sp, ex, ey, ez, Ex, Ey, Ez, sx, sy, sz);
            eE = flatE;
            eq = ((sx + 1) << 1) | ((sy + 1) << 3) | ((sz + 1) << 5) | (tr.own ? 1 << 13 : 0) |
                 (tr.oth ? 1 << 14 : 0) | (tr.same ? 1 << 15 : 0);
            if (tr.own || tr.oth || tr.same || (sx | sy | sz)) {
                em0 = d.cstart[sp.c0 + flatE];
                nseg = d.cstart[sp.c0 + flatE + 1] - em0;
            }
            const int axa = (qx == 0) ? -1 : 0, axb = (qx == sp.nc[0] - 1) ? 1 : 0;
            const int aya = (qy == 0) ? -1 : 0, ayb = (qy == sp.nc[1] - 1) ? 1 : 0;
            const int aza = (qz == 0) ? -1 : 0, azb = (qz == sp.nc[2] - 1) ? 1 : 0;
            for (int ax = axa; ax <= axb; ax++)
                for (int ay = aya; ay <= ayb; ay++)
                    for (int az = aza; az <= azb; az++) {
                        if ((ax | ay | az) == 0) continue;
                        const int g = ((Ex + ax) * sp.ext[1] + (Ey + ay)) * sp.ext[2] + (Ez + az);
                        if (d.cstart[sp.c0 + g] != d.cstart[sp.c0 + g + 1]) ghost = true;
                    }
        }
    }
    if (__any_sync(0xffffffffu, ghost)) {
        build_cells(d, s, lcb, sub);
        return;
    }
    int incl = nseg;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    st_pre[warp][lane] = incl - nseg;
    st_q[warp][lane] = eq;
    st_E[warp][lane] = eE;
    st_m0[warp][lane] = em0;
    if (lane == 0) st_pre[warp][32] = total;
    // the system's parameters the loops use, in registers (the list stores
    // could alias the global SysParams for all the compiler knows)
    const float brel = sp.band_rel;
    const bool uniform = sp.uniform != 0, newton = sp.newton != 0;
    const float ucut2 = sp.ucut2f, sf2 = sp.sf2f;
    const float in_f = 1.f + brel, near_f = 1.f - brel;
    const float Lx = sp.Lh[0], Ly = sp.Lh[1], Lz = sp.Lh[2];
    const long long sp0 = sp.p0;
    const int ncap = sp.ncap, npad = sp.npad;
    // the centre bin's box in the frame of the geometry copy (x - lo),
    // widened by 1e-6 of the box for rounding; uniform systems drop staged
    // candidates farther than the list cutoff (plus the band) from it
    const float bx0 = (float)((ex - sp.sl[0]) * sp.bin[0] - 1e-6 * sp.L[0]);
    const float by0 = (float)((ey - sp.sl[1]) * sp.bin[1] - 1e-6 * sp.L[1]);
    const float bz0 = (float)((ez - sp.sl[2]) * sp.bin[2] - 1e-6 * sp.L[2]);
    const float bx1 = (float)((ex - sp.sl[0] + 1) * sp.bin[0] + 1e-6 * sp.L[0]);
    const float by1 = (float)((ey - sp.sl[1] + 1) * sp.bin[1] + 1e-6 * sp.L[1]);
    const float bz1 = (float)((ez - sp.sl[2] + 1) * sp.bin[2] + 1e-6 * sp.L[2]);
    const float cull2 = ucut2 * in_f;
    for (int ib = a0; ib < a1; ib += 32) {
        const long long i = ib + lane;
        const bool act = i < a1;
        float4 hi = make_float4(0, 0, 0, 0), lo = make_float4(0, 0, 0, 0);
        bool edge_i = false;
        if (act) {
            d.lbp[i] = d.pos[i];
            hi = d.pos2[2 * i];
            lo = d.pos2[2 * i + 1];
            edge_i = d.cell[i] < 0;
        }
        uint32_t* row = d.nlist + sp.lst0 + (i - sp0);
        const int li = (int)(i - sp0);
        int count = 0;
        int q0 = 0;  // next candidate of the window sequence to stage
        while (q0 < total) {
            // stage: passes of 32 candidates, kept ones compacted by ballot
            __syncwarp();
            int np = 0;
            while (q0 < total && np + 32 <= STAGE_CAP) {
                const int q = q0 + lane;
                bool keep = false;
                float4 hj = make_float4(0, 0, 0, 0);
                int meta = 0, fl = 0;
                if (q < total) {
                    int k = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (st_pre[warp][k + step] <= q) k += step;
                    const int ek = st_q[warp][k];
                    const long long j = st_m0[warp][k] + (q - st_pre[warp][k]);
                    const int sx = ((ek >> 1) & 3) - 1, sy = ((ek >> 3) & 3) - 1, sz = ((ek >> 5) & 3) - 1;
                    hj = d.pos2[2 * j];
                    hj.x += (float)sx * Lx;
                    hj.y += (float)sy * Ly;
                    hj.z += (float)sz * Lz;
                    keep = true;
                    if (uniform) {
                        const float ox = fmaxf(fmaxf(bx0 - hj.x, hj.x - bx1), 0.f);
                        const float oy = fmaxf(fmaxf(by0 - hj.y, hj.y - by1), 0.f);
                        const float oz = fmaxf(fmaxf(bz0 - hj.z, hj.z - bz1), 0.f);
                        keep = ox * ox + oy * oy + oz * oz <= cull2;
                    }
                    const bool shifted = (sx | sy | sz) != 0;
                    const bool edge = keep && shifted && d.cell[j] < 0;
                    const int sc = (sx + 1) * 9 + (sy + 1) * 3 + (sz + 1);
                    meta = (int)(j - sp0) | (sc << IDX_BITS) | (edge ? (int)0x80000000u : 0);
                    fl = ((ek >> 13) & 7) | (shifted ? 8 : 0) | (k << 4);
                }
                const unsigned int kb = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int slot = np + __popc(kb & ((1u << lane) - 1u));
                    st_p[warp][slot] = hj;
                    st_m[warp][slot] = meta;
                    st_f[warp][slot] = fl;
                }
                np += __popc(kb);
                q0 += 32;
            }
            __syncwarp();
            if (!act) continue;
            for (int t0 = 0; t0 < np; t0 += 32) {
                const int nt = min(32, np - t0);
                // hi-part fp32 screen of 32 staged candidates into two bit masks:
                // within the cutoff band / near the cutoff (precise path)
                unsigned int mask = 0u, near = 0u;
                const float4* tile = &st_p[warp][t0];
                if (uniform) {
                    const float cin = ucut2 * in_f, cnear = ucut2 * near_f;
#pragma unroll 8
                    for (int t = 0; t < nt; t++) {
                        const float4 hj = tile[t];
                        const float px = hj.x - hi.x, py = hj.y - hi.y, pz = hj.z - hi.z;
                        const float r2h = px * px + py * py + pz * pz;
                        mask |= (r2h <= cin ? 1u : 0u) << t;
                        near |= (r2h > cnear ? 1u : 0u) << t;
                    }
                } else {
#pragma unroll 4
                    for (int t = 0; t < nt; t++) {
                        const float4 hj = tile[t];
                        const float px = hj.x - hi.x, py = hj.y - hi.y, pz = hj.z - hi.z;
                        const float r2h = px * px + py * py + pz * pz;
                        const float ssum = hi.w + hj.w;
                        const float c2h = ssum * ssum * sf2;
                        mask |= (r2h <= c2h * in_f ? 1u : 0u) << t;
                        near |= (r2h > c2h * near_f ? 1u : 0u) << t;
                    }
                }
                while (mask) {
                    const int t = __ffs(mask) - 1;
                    mask &= mask - 1u;
                    const int meta = st_m[warp][t0 + t];
                    const int fl = st_f[warp][t0 + t];
                    const int jl = meta & (int)IDX_MASK;
                    if (!(fl & 8) && jl == li) continue;  // itself
                    const bool edge = (fl & 8) && (edge_i || meta < 0);
                    int bits;
                    if (!((near >> t) & 1u) && !edge) {
                        // owner rule of the pair's two bins; same bin: by index
                        const bool same = (fl & 4) != 0;
                        bits = (((fl & 1) || (same && (!newton || jl > li))) ? 1 : 0) |
                               (((fl & 2) || (same && newton && jl < li)) ? 2 : 0);
                    } else {
                        const int sc = (meta >> IDX_BITS) & 31;
                        const int k = fl >> 4;
                        const int fE = st_E[warp][k];
                        const int Ez = fE % sp.ext[2], Ey = (fE / sp.ext[2]) % sp.ext[1],
                                  Ex = fE / (sp.ext[2] * sp.ext[1]);
                        bits = near_pair(d, sp, i, sp0 + jl, hi, lo, d.pos2[2 * (sp0 + jl)],
                                         d.pos2[2 * (sp0 + jl) + 1], sc / 9 - 1, (sc / 3) % 3 - 1, sc % 3 - 1, edge,
                                         ex, ey, ez, Ex, Ey, Ez,
                                         TileRule{(fl & 1) != 0, (fl & 2) != 0, (fl & 4) != 0});
                    }
                    const uint32_t code = (uint32_t)meta & 0x7fffffffu;  // local index | image code << 26
                    if (bits & 1) {
                        if (count < ncap) row[(size_t)count * npad] = code + (27u << IDX_BITS);
                        count++;
                    }
                    if (bits & 2) {
                        if (count < ncap) row[(size_t)count * npad] = code;
                        count++;
                    }
                }
            }
        }
        if (act) {
            if (count > ncap) {
                atomicOr(&st->status, ST_NBR_OVF);
                atomicMax(&st->max_nbr, count);
                count = ncap;
            } else if (count > vload(&st->max_nbr)) {  // skip the atomic on one word when it cannot raise it
                atomicMax(&st->max_nbr, count);
            }
            d.nnum[i] = count;
        }
    }
}

// Work unit (particle block pb, sub-unit sub) of system s, by the system's
// build mode: 2 (dilute) the block's particles with a thread each (sub-unit
// 0); 0 (many dense bins) a bin per warp, bins numbered like particle slots;
// 1 (few dense bins) a particle per warp, BUILD_WARPS per sub-unit.
__device__ void build_unit(const Dev& d, int s, int pb, int sub) {
    const SysParams& sp = d.sp[s];
    if (!do_rebuild(d.ss + s)) return;  // uniform over the block
    if (sp.build_mode == 2) {
        if (sub != 0) return;
        const int li = pb * BLK + (int)threadIdx.x;
        if (li < sp.n) build_one(d, s, li);
        return;
    }
    if (sp.build_mode == 0) {
        build_cells_staged(d, s, pb, sub);  // the system has no more bins than particle slots
        return;
    }
    const int li = pb * BLK + sub * BUILD_WARPS + (int)(threadIdx.x >> 5);
    if (li < sp.n) build_warp(d, s, li);  // uniform over the warp
}

// Minimum resident blocks per SM asked of ptxas for k_build: 6 caps it at 80
// registers (~180 B of spills in the staged loop).  Measured on GB300 against
// 4 blocks at 128 registers: warp per particle 12 % faster (LJ 256k 2.04 ->
// 1.79 ms per rebuild and force, polydisperse 200k 0.97 -> 0.86 ms), warp per
// bin 2 % faster (0.83 -> 0.81 ms); a compile-time tuning knob.
#ifndef MDG_BUILD_MINB
#define MDG_BUILD_MINB 6
#endif
__global__ void __launch_bounds__(BUILD_WARPS * 32, MDG_BUILD_MINB) k_build(Dev d)
    RB_FOR_PARTICLE_SUBS(build_unit, BUILD_SUBS)

// ----------------------------------------------------------------------------
// LJ 12-6 force (lj_force, md_lj/src/lib.rs:488-633) over the full list.
// TPP lanes share one particle's row and combine with warp shuffles.  MT:
// systems with a multi-type pair table look up lj1, lj2 and the squared
// cutoff by the two particles' types (pair_table.get(ti, tj)); a separate
// instantiation, so the single-type path keeps its code.
// ----------------------------------------------------------------------------
template <int TPP, bool MT>
__global__ void __launch_bounds__(BLK) k_lj_fp64(Dev d) {
    const int pb = d.blk_run[blockIdx.x / TPP];
    const int sub = blockIdx.x % TPP;
    const int s = d.blk_sys[pb];
    const SysParams& sp = d.sp[s];
    if (sp.kind != 1 || !sys_active(d.ss + s)) return;
    const int lane = threadIdx.x % TPP;
    const int li = (pb - sp.b0) * BLK + sub * (BLK / TPP) + threadIdx.x / TPP;
    const bool act = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    double fx = 0, fy = 0, fz = 0, pe = 0;
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0, v4 = 0, v5 = 0;
    if (act) {
        const double4 xi = d.pos[i];
        const int nn = d.nnum[i];
        const long long base = sp.lst0 + li;
        double lj1 = sp.lj1, lj2 = sp.lj2, cut2 = sp.lj_cut2;
        const double half = sp.newton ? 1.0 : 0.5;
        const bool mt = MT && sp.nmat > 1;
        const long long tq = (long long)sp.nmat * sp.nmat;
        const long long trow = mt ? sp.mat0 + (long long)d.type[i] * sp.nmat : 0;
        for (int k = lane; k < nn; k += TPP) {
            const uint32_t e = d.nlist[base + (long long)k * sp.npad];
            const long long j = sp.p0 + (e & IDX_MASK);
            if (MT && mt) {
                const long long o = trow + d.type[j];
                lj1 = d.mat[o + TL_LJ1 * tq];
                lj2 = d.mat[o + TL_LJ2 * tq];
                cut2 = d.mat[o + TL_CUT2 * tq];
            }
            const uint32_t code = e >> IDX_BITS;
            const bool own = code >= 27u;
            int sx, sy, sz;
            decode_shift((int)(own ? code - 27u : code), sx, sy, sz);
            const double4 xj = d.pos[j];
            double dx, dy, dz;
            if (own) {
                dx = img_coord(xj.x, sx, sp.L[0]) - xi.x;
                dy = img_coord(xj.y, sy, sp.L[1]) - xi.y;
                dz = img_coord(xj.z, sz, sp.L[2]) - xi.z;
            } else {  // owner frame: partner i's image seen from j
                dx = img_coord(xi.x, -sx, sp.L[0]) - xj.x;
                dy = img_coord(xi.y, -sy, sp.L[1]) - xj.y;
                dz = img_coord(xi.z, -sz, sp.L[2]) - xj.z;
            }
            const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
            if (r2 >= cut2) continue;
            const double r2inv = 1.0 / r2;
            const double r6inv = r2inv * r2inv * r2inv;
            const double fpair = r2inv * r6inv * fma(lj1, r6inv, -lj2);
            if (!sp.virial) {
                if (own) {
                    fx = fma(-fpair, dx, fx);
                    fy = fma(-fpair, dy, fy);
                    fz = fma(-fpair, dz, fz);
                } else {
                    fx = fma(fpair, dx, fx);
                    fy = fma(fpair, dy, fy);
                    fz = fma(fpair, dz, fz);
                }
            } else {
                const double px = -fpair * dx, py = -fpair * dy, pz = -fpair * dz;
                if (own) {
                    fx += px; fy += py; fz += pz;
                    v0 += dx * px * half; v1 += dy * py * half; v2 += dz * pz * half;
                    v3 += dx * py * half; v4 += dx * pz * half; v5 += dy * pz * half;
                } else {
                    fx -= px; fy -= py; fz -= pz;
                }
            }
        }
    }
    if (TPP > 1) {
#pragma unroll
        for (int o = TPP / 2; o > 0; o >>= 1) {
            fx += __shfl_down_sync(0xffffffffu, fx, o, TPP);
            fy += __shfl_down_sync(0xffffffffu, fy, o, TPP);
            fz += __shfl_down_sync(0xffffffffu, fz, o, TPP);
            pe += __shfl_down_sync(0xffffffffu, pe, o, TPP);
            if (sp.virial) {
                v0 += __shfl_down_sync(0xffffffffu, v0, o, TPP);
                v1 += __shfl_down_sync(0xffffffffu, v1, o, TPP);
                v2 += __shfl_down_sync(0xffffffffu, v2, o, TPP);
                v3 += __shfl_down_sync(0xffffffffu, v3, o, TPP);
                v4 += __shfl_down_sync(0xffffffffu, v4, o, TPP);
                v5 += __shfl_down_sync(0xffffffffu, v5, o, TPP);
            }
        }
    }
    if (act && lane == 0) {
        d.frc[i] = make_double4(fx, fy, fz, pe);
        if (sp.virial) {
            d.vir[0 * d.P + i] = v0; d.vir[1 * d.P + i] = v1; d.vir[2 * d.P + i] = v2;
            d.vir[3 * d.P + i] = v3; d.vir[4 * d.P + i] = v4; d.vir[5 * d.P + i] = v5;
        }
    }
}

// ----------------------------------------------------------------------------
// Hertz-Mindlin / Hooke contact with tangential history
// (hertz_mindlin_contact_force, contact.rs:103-615; hooke_contact_force,
// contact.rs:622-990).  The pair is always evaluated in the owner's frame
// (i = owner, j = partner), exactly as the reference's half list does.
// ----------------------------------------------------------------------------
struct PairOut {
    double fn[3];      // normal force (owner -= fn, partner += fn)
    double ft[3];      // tangential force (owner += ft, partner -= ft)
    double ti[3];      // tangential torque on the owner
    double tj[3];      // tangential torque on the partner (same sign rule)
    double tr[3];      // rolling torque (owner +=, partner -=)
    double tw[3];      // twisting torque (owner +=, partner -=)
    double spring[7];  // updated history, canonical frame
    double vir[6];     // owner-side virial contribution
    bool hit;          // a force was applied
    bool tang;         // tangential/rolling/twisting stage reached
    bool overlap;      // large-overlap warning (d / (r1 + r2) < 0.90)
};

__device__ __forceinline__ double mtab(const Dev& d, const SysParams& sp, int tab, int a, int b) {
    return d.mat[sp.mat0 + ((long long)tab * sp.nmat + a) * sp.nmat + b];
}

__device__ void hm_pair(const Dev& d, const SysParams& sp, double dx, double dy, double dz, double r1, double r2,
                        const double4& v_i, const double4& v_j, const double4& w_i, const double4& w_j,
                        double mass_i, double mass_j, int mi, int mj, uint32_t tag_i, uint32_t tag_j,
                        const double* stored, PairOut& o) {
    const double kPi = 3.14159265358979323846;
    const double SQRT_5_3 = 0.9128709291752768;  // dem_atom/src/lib.rs:63
    const double EPS = 1e-30;                    // TANGENTIAL_EPSILON
    const bool hooke = sp.contact_model == 1;
    const bool use_dmt = sp.adhesion_model == 1;
    const double dt = sp.dt;
    o.hit = false;
    o.tang = false;
    o.overlap = false;
    const double dist_sq = dx * dx + dy * dy + dz * dz;
    const double sum_r = r1 + r2;
    const double surface_energy = hooke ? 0.0 : mtab(d, sp, T_SURFACE, mi, mj);
    const double r_eff = (r1 * r2) / sum_r;
    const double e_eff = mtab(d, sp, T_EEFF, mi, mj);
    double delta_pulloff = 0.0;
    if (!hooke && surface_energy > 0.0 && !use_dmt) {
        const double g = surface_energy;
        delta_pulloff = cbrt(kPi * kPi * g * g * r_eff / (4.0 * e_eff * e_eff));
    }
    const double interaction_r = sum_r + delta_pulloff;
    if (dist_sq >= interaction_r * interaction_r) return;
    const double distance = sqrt(dist_sq);
    if (distance == 0.0) return;
    const double r_min = fmin(r1, r2);
    const double delta = fmin(sum_r - distance, 0.5 * r_min);
    if (hooke && delta <= 0.0) return;
    if (delta > 0.0 && distance / sum_r < 0.90) o.overlap = true;
    if (!hooke && delta <= 0.0 && surface_energy <= 0.0) return;
    o.hit = true;
    const double inv_dist = 1.0 / distance;
    const double nx = dx * inv_dist, ny = dy * inv_dist, nz = dz * inv_dist;
    const double g_eff = mtab(d, sp, T_GEFF, mi, mj);
    const double inv_m_i = v_i.w > 0.0 ? v_i.w : 1.0 / mass_i;
    const double inv_m_j = v_j.w > 0.0 ? v_j.w : 1.0 / mass_j;
    const double m_r = 1.0 / (inv_m_i + inv_m_j);
    const double beta = mtab(d, sp, T_BETA, mi, mj);
    const double mu = mtab(d, sp, T_FRICTION, mi, mj);
    const double mu_r = mtab(d, sp, T_ROLL_FRICTION, mi, mj);
    const double mu_tw = mtab(d, sp, T_TWIST_FRICTION, mi, mj);
    const double cohesion_energy = mtab(d, sp, T_COHESION, mi, mj);
    const bool jkr_adhesion_only = !hooke && surface_energy > 0.0 && !use_dmt && delta <= 0.0;
    double s_n = 0, k_n = 0, k_t = 0, kn = 0, kt = 0, gamma_n = 0;
    if (hooke) {
        kn = mtab(d, sp, T_KN, mi, mj);
        kt = mtab(d, sp, T_KT, mi, mj);
        gamma_n = 2.0 * beta * sqrt(kn * m_r);
    } else if (delta > 0.0) {
        const double sdr = sqrt(delta * r_eff);
        s_n = 2.0 * e_eff * sdr;
        k_n = 4.0 / 3.0 * e_eff * sdr;
        k_t = 8.0 * g_eff * sdr;
    }
    const double oix = w_i.x, oiy = w_i.y, oiz = w_i.z;
    const double ojx = w_j.x, ojy = w_j.y, ojz = w_j.z;
    const double r1nx = r1 * nx, r1ny = r1 * ny, r1nz = r1 * nz;
    const double vcix = v_i.x + (oiy * r1nz - oiz * r1ny);
    const double vciy = v_i.y + (oiz * r1nx - oix * r1nz);
    const double vciz = v_i.z + (oix * r1ny - oiy * r1nx);
    const double r2nx = r2 * nx, r2ny = r2 * ny, r2nz = r2 * nz;
    const double vcjx = v_j.x + (-ojy * r2nz + ojz * r2ny);
    const double vcjy = v_j.y + (-ojz * r2nx + ojx * r2nz);
    const double vcjz = v_j.z + (-ojx * r2ny + ojy * r2nx);
    const double vrx = vcjx - vcix, vry = vcjy - vciy, vrz = vcjz - vciz;
    const double v_n = vrx * nx + vry * ny + vrz * nz;
    double f_n_mag;
    if (hooke) {
        if (cohesion_energy > 0.0) {
            const double f_coh = cohesion_energy * kPi * delta * r_eff;
            f_n_mag = kn * delta - gamma_n * v_n - f_coh;
        } else {
            f_n_mag = fmax(kn * delta - gamma_n * v_n, 0.0);
        }
    } else if (surface_energy > 0.0 && use_dmt) {
        const double f_dmt = 2.0 * kPi * surface_energy * r_eff;
        const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
        f_n_mag = k_n * delta - f_diss - f_dmt;
    } else if (surface_energy > 0.0) {
        const double f_adh = 1.5 * kPi * surface_energy * r_eff;
        if (jkr_adhesion_only) {
            f_n_mag = -f_adh;
        } else {
            const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
            f_n_mag = k_n * delta - f_diss - f_adh;
        }
    } else if (cohesion_energy > 0.0) {
        const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
        const double f_coh = cohesion_energy * kPi * delta * r_eff;
        f_n_mag = k_n * delta - f_diss - f_coh;
    } else {
        const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
        f_n_mag = fmax(k_n * delta - f_diss, 0.0);
    }
    o.fn[0] = f_n_mag * nx;
    o.fn[1] = f_n_mag * ny;
    o.fn[2] = f_n_mag * nz;
    const double vs = sp.newton ? 1.0 : 0.5;
    if (jkr_adhesion_only) {
        const double fx = -o.fn[0] * vs, fy = -o.fn[1] * vs, fz = -o.fn[2] * vs;
        o.vir[0] = dx * fx; o.vir[1] = dy * fy; o.vir[2] = dz * fz;
        o.vir[3] = dx * fy; o.vir[4] = dx * fz; o.vir[5] = dy * fz;
        return;
    }
    o.tang = true;
    const double vtx = vrx - v_n * nx, vty = vry - v_n * ny, vtz = vrz - v_n * nz;
    const double sign = tag_i < tag_j ? 1.0 : -1.0;
    double sx = sign * stored[0], sy = sign * stored[1], sz = sign * stored[2];
    const double sdn = sx * nx + sy * ny + sz * nz;
    sx -= sdn * nx;
    sy -= sdn * ny;
    sz -= sdn * nz;
    sx += vtx * dt;
    sy += vty * dt;
    sz += vtz * dt;
    const double ktt = hooke ? kt : k_t;
    const double s_mag = sqrt(sx * sx + sy * sy + sz * sz);
    const double fts = ktt * s_mag;
    const double ft_max = mu * fabs(f_n_mag);
    if (fts > ft_max && fts > EPS) {
        const double sc = ft_max / fts;
        sx *= sc; sy *= sc; sz *= sc;
    }
    const double gamma_t = 2.0 * SQRT_5_3 * beta * sqrt(ktt * m_r);
    double ftx = ktt * sx - gamma_t * vtx;
    double fty = ktt * sy - gamma_t * vty;
    double ftz = ktt * sz - gamma_t * vtz;
    const double ftm = sqrt(ftx * ftx + fty * fty + ftz * ftz);
    if (ftm > ft_max && ftm > EPS) {
        const double sc = ft_max / ftm;
        ftx *= sc; fty *= sc; ftz *= sc;
    }
    o.ft[0] = ftx; o.ft[1] = fty; o.ft[2] = ftz;
    o.ti[0] = r1ny * ftz - r1nz * fty; o.ti[1] = r1nz * ftx - r1nx * ftz; o.ti[2] = r1nx * fty - r1ny * ftx;
    o.tj[0] = r2ny * ftz - r2nz * fty; o.tj[1] = r2nz * ftx - r2nx * ftz; o.tj[2] = r2nx * fty - r2ny * ftx;
    const double orx = oix - ojx, ory = oiy - ojy, orz = oiz - ojz;
    const double odn = orx * nx + ory * ny + orz * nz;
    const double rollx = orx - odn * nx, rolly = ory - odn * ny, rollz = orz - odn * nz;
    double rdx = sign * stored[3], rdy = sign * stored[4], rdz = sign * stored[5];
    double twd = sign * stored[6];
    o.tr[0] = o.tr[1] = o.tr[2] = 0.0;
    o.tw[0] = o.tw[1] = o.tw[2] = 0.0;
    if (mu_r > 0.0) {
        const double roll_mag = sqrt(rollx * rollx + rolly * rolly + rollz * rollz);
        if (sp.rolling_model == 1) {
            const double k_roll = mtab(d, sp, T_KROLL, mi, mj);
            const double g_roll = mtab(d, sp, T_GROLL, mi, mj);
            const double rdn = rdx * nx + rdy * ny + rdz * nz;
            rdx -= rdn * nx; rdy -= rdn * ny; rdz -= rdn * nz;
            rdx += rollx * dt; rdy += rolly * dt; rdz += rollz * dt;
            double tx = -k_roll * rdx - g_roll * rollx;
            double ty = -k_roll * rdy - g_roll * rolly;
            double tz = -k_roll * rdz - g_roll * rollz;
            const double trm = sqrt(tx * tx + ty * ty + tz * tz);
            const double tau_max = mu_r * fabs(f_n_mag) * r_eff;
            if (trm > tau_max && trm > EPS) {
                const double sc = tau_max / trm;
                tx *= sc; ty *= sc; tz *= sc;
                if (k_roll > EPS) {
                    rdx = (tx + g_roll * rollx) / (-k_roll);
                    rdy = (ty + g_roll * rolly) / (-k_roll);
                    rdz = (tz + g_roll * rollz) / (-k_roll);
                }
            }
            o.tr[0] = tx; o.tr[1] = ty; o.tr[2] = tz;
        } else if (roll_mag > 1e-30) {
            const double tau_mag = mu_r * fabs(f_n_mag) * r_eff;
            const double inv_roll = tau_mag / roll_mag;
            o.tr[0] = -inv_roll * rollx; o.tr[1] = -inv_roll * rolly; o.tr[2] = -inv_roll * rollz;
        }
    }
    if (mu_tw > 0.0) {
        const double twist_vel = odn;
        if (sp.twisting_model == 1) {
            const double k_tw = mtab(d, sp, T_KTWIST, mi, mj);
            const double g_tw = mtab(d, sp, T_GTWIST, mi, mj);
            twd += twist_vel * dt;
            double tau_tw = -k_tw * twd - g_tw * twist_vel;
            const double tau_max = mu_tw * fabs(f_n_mag) * r_eff;
            if (fabs(tau_tw) > tau_max) {
                tau_tw = copysign(1.0, tau_tw) * tau_max;
                if (k_tw > EPS) twd = (tau_tw + g_tw * twist_vel) / (-k_tw);
            }
            o.tw[0] = tau_tw * nx; o.tw[1] = tau_tw * ny; o.tw[2] = tau_tw * nz;
        } else if (fabs(twist_vel) > 1e-30) {
            const double tau = mu_tw * fabs(f_n_mag) * r_eff;
            const double sg = twist_vel > 0.0 ? -1.0 : 1.0;
            o.tw[0] = sg * tau * nx; o.tw[1] = sg * tau * ny; o.tw[2] = sg * tau * nz;
        }
    }
    {
        const double vfx = (-o.fn[0] + ftx) * vs, vfy = (-o.fn[1] + fty) * vs, vfz = (-o.fn[2] + ftz) * vs;
        o.vir[0] = dx * vfx; o.vir[1] = dy * vfy; o.vir[2] = dz * vfz;
        o.vir[3] = dx * vfy; o.vir[4] = dx * vfz; o.vir[5] = dy * vfz;
    }
    o.spring[0] = sign * sx; o.spring[1] = sign * sy; o.spring[2] = sign * sz;
    o.spring[3] = sign * rdx; o.spring[4] = sign * rdy; o.spring[5] = sign * rdz;
    o.spring[6] = sign * twd;
}

// Look up the spring stored by particle `p` (local index lp in its system)
// for partner tag `t` in history buffer `hc`.
__device__ __forceinline__ bool hist_find(const Dev& d, const SysParams& sp, int hc, long long p, int lp,
                                          uint32_t t, double* out) {
    const int n = d.hcnt[hc][p];
    for (int c = 0; c < n; c++) {
        if (d.htag[hc][sp.h0 + (long long)c * sp.npad + lp] == t) {
            for (int q = 0; q < 7; q++) out[q] = d.hval[hc][sp.h0 * 7 + (long long)(c * 7 + q) * sp.npad + lp];
            return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(BLK) k_dem_fp64(Dev d) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (sp.kind != 0 || !sys_active(st)) return;
    const int hcur = st->hcur;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long i = (long long)sp.p0 + li;
    const int hn = hcur ^ 1;
    const double4 xi = d.pos[i];
    const double4 vi = d.vel[i];
    const double4 wi = d.omg[i];
    const double mass_i = d.mass[i];
    const int ti_ = (int)d.type[i];
    const uint32_t tag_i = d.tag[i];
    const int nn = d.nnum[i];
    const long long base = sp.lst0 + li;
    double F[3] = {0, 0, 0}, T[3] = {0, 0, 0}, V[6] = {0, 0, 0, 0, 0, 0};
    int nh = 0, nover = 0;
    PairOut o;
    for (int k = 0; k < nn; k++) {
        const uint32_t e = d.nlist[base + (long long)k * sp.npad];
        const int lj = (int)(e & IDX_MASK);
        const long long j = sp.p0 + lj;
        const uint32_t code = e >> IDX_BITS;
        const bool own = code >= 27u;
        int sx, sy, sz;
        decode_shift((int)(own ? code - 27u : code), sx, sy, sz);
        const double4 xj = d.pos[j];
        const double4 vj = d.vel[j];
        const double4 wj = d.omg[j];
        const double mass_j = d.mass[j];
        const int tj_ = (int)d.type[j];
        const uint32_t tag_j = d.tag[j];
        double stored[7] = {0, 0, 0, 0, 0, 0, 0};
        if (own) {
            hist_find(d, sp, hcur, i, li, tag_j, stored);
            const double dx = img_coord(xj.x, sx, sp.L[0]) - xi.x;
            const double dy = img_coord(xj.y, sy, sp.L[1]) - xi.y;
            const double dz = img_coord(xj.z, sz, sp.L[2]) - xi.z;
            hm_pair(d, sp, dx, dy, dz, xi.w, xj.w, vi, vj, wi, wj, mass_i, mass_j, ti_, tj_, tag_i, tag_j, stored, o);
            if (!o.hit) continue;
            F[0] -= o.fn[0]; F[1] -= o.fn[1]; F[2] -= o.fn[2];
            if (o.overlap) nover++;
            for (int q = 0; q < 6; q++) V[q] += o.vir[q];
            if (!o.tang) continue;
            F[0] += o.ft[0]; F[1] += o.ft[1]; F[2] += o.ft[2];
            T[0] += o.ti[0]; T[1] += o.ti[1]; T[2] += o.ti[2];
            T[0] += o.tr[0]; T[1] += o.tr[1]; T[2] += o.tr[2];
            T[0] += o.tw[0]; T[1] += o.tw[1]; T[2] += o.tw[2];
            if (nh < sp.hcap) {
                d.htag[hn][sp.h0 + (long long)nh * sp.npad + li] = tag_j;
                for (int q = 0; q < 7; q++)
                    d.hval[hn][sp.h0 * 7 + (long long)(nh * 7 + q) * sp.npad + li] = o.spring[q];
            }
            nh++;
        } else {
            hist_find(d, sp, hcur, j, lj, tag_i, stored);
            const double dx = img_coord(xi.x, -sx, sp.L[0]) - xj.x;
            const double dy = img_coord(xi.y, -sy, sp.L[1]) - xj.y;
            const double dz = img_coord(xi.z, -sz, sp.L[2]) - xj.z;
            hm_pair(d, sp, dx, dy, dz, xj.w, xi.w, vj, vi, wj, wi, mass_j, mass_i, tj_, ti_, tag_j, tag_i, stored, o);
            if (!o.hit) continue;
            F[0] += o.fn[0]; F[1] += o.fn[1]; F[2] += o.fn[2];
            if (!o.tang) continue;
            F[0] -= o.ft[0]; F[1] -= o.ft[1]; F[2] -= o.ft[2];
            T[0] += o.tj[0]; T[1] += o.tj[1]; T[2] += o.tj[2];
            T[0] -= o.tr[0]; T[1] -= o.tr[1]; T[2] -= o.tr[2];
            T[0] -= o.tw[0]; T[1] -= o.tw[1]; T[2] -= o.tw[2];
        }
    }
    if (nh > sp.hcap) {
        atomicOr(&st->status, ST_HIST_OVF);
        nh = sp.hcap;
    }
    if (d.hist_any) d.hcnt[hn][i] = nh;
    if (nover) atomicAdd(&st->overlap, nover);
    d.frc[i] = make_double4(F[0], F[1], F[2], 0.0);
    d.trq[i] = make_double4(T[0], T[1], T[2], 0.0);
    if (sp.virial)
        for (int q = 0; q < 6; q++) d.vir[q * d.P + i] = V[q];
}

// ----------------------------------------------------------------------------
// final integration + thermostat half step + per-step bookkeeping
// ----------------------------------------------------------------------------
// final_integration (mddem_verlet/src/lib.rs:136-154), final_rotation
// (rotational.rs:87-100), nh_post_final (md_thermostat/src/lib.rs:313-353).
// integrate = 0: reductions and rebuild bookkeeping only (force-only evaluation).
__global__ void __launch_bounds__(BLK) k_final(Dev d, int integrate) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    SysState* st = d.ss + s;
    if (!sys_active(st)) return;  // every block of a frozen system returns
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    const bool act = li < sp.n;
    const long long i = (long long)sp.p0 + li;
    const double dt = sp.dt;
    double vals[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int bad = 0;
    if (act) {
        double4 f = d.frc[i];
        double4 v = d.vel[i];
        if (integrate && sp.lv) langevin_add(d, sp, st, i, v, f);
        if (integrate) {
            const double h = 0.5 * dt * v.w;
            v.x += h * f.x;
            v.y += h * f.y;
            v.z += h * f.z;
            if (sp.nh) {
                const double scale = st->nh_scale;
                v.x *= scale;
                v.y *= scale;
                v.z *= scale;
            }
            d.vel[i] = v;
        }
        // KE feeds only the thermostat (thermo output has its own reduction)
        if (sp.nh) vals[0] = d.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z);
        if (sp.kind == 0 && integrate) {
            double4 w = d.omg[i];
            if (w.w != 0.0) {
                const double4 tq = d.trq[i];
                w.x += 0.5 * dt * tq.x * w.w;
                w.y += 0.5 * dt * tq.y * w.w;
                w.z += 0.5 * dt * tq.z * w.w;
                d.omg[i] = w;
            }
        }
        if (sp.virial)
            for (int q = 0; q < 6; q++) vals[1 + q] = d.vir[q * d.P + i];
        // non-finite test on the exponent bits of v (integer ops only): a
        // non-finite force or position shows in v by the next step
        const int ex = 0x7ff00000;
        bad = ((__double2hiint(v.x) & ex) == ex) | ((__double2hiint(v.y) & ex) == ex) |
              ((__double2hiint(v.z) & ex) == ex);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&st->status, ST_NAN);
    double out[8];
    bool last;
    if (sp.virial) {
        last = system_reduce<8>(d, s, gb, vals, out);
    } else {
        const double v1[1] = {vals[0]};
        double o1[1];
        last = system_reduce<1>(d, s, gb, v1, o1);
        out[0] = o1[0];
    }
    if (last && threadIdx.x == 0) step_end(sp, st, out[0], sp.virial ? out + 1 : nullptr, integrate);
}

// KE of the uploaded velocities (the first nh_pre_initial's compute_ke).
__global__ void __launch_bounds__(BLK) k_ke_init(Dev d) {
    const int gb = blockIdx.x;
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    if (gb - sp.b0 >= sp.nb) return;  // past the particles: not in the reduction
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    double vals[1] = {0.0};
    if (li < sp.n) {
        const long long i = (long long)sp.p0 + li;
        const double4 v = d.vel[i];
        // KE feeds only the thermostat (thermo output has its own reduction)
        if (sp.nh) vals[0] = d.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z);
    }
    double out[1];
    if (system_reduce<1>(d, s, gb, vals, out) && threadIdx.x == 0) {
        SysState* st = d.ss + s;
        const double ke = 0.5 * out[0];
        st->ke = ke;
        if (sp.nh) {
            const double dt = sp.dt;
            const double pre = st->p_xi_post + (dt / 2.0) * (2.0 * ke - sp.nh_ndof * sp.nh_T);
            st->p_xi_pre = pre;
            st->nh_scale = exp(-dt / 2.0 * pre / sp.nh_Q);
        }
    }
}

// thermo pass 1: sum m, sum m v, compute_ke sum, pe  (granular_temp.rs:62-101, atom.rs:489-502)
__global__ void __launch_bounds__(BLK) k_thermo1(Dev d, double* out16) {
    const int gb = blockIdx.x;
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    if (gb - sp.b0 >= sp.nb) return;  // past the particles: not in the reduction
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    double vals[7] = {0, 0, 0, 0, 0, 0, 0};
    if (li < sp.n) {
        const long long i = (long long)sp.p0 + li;
        const double4 v = d.vel[i];
        const double m = d.mass[i];
        vals[0] = m;
        vals[1] = m * v.x;
        vals[2] = m * v.y;
        vals[3] = m * v.z;
        vals[4] = m * (v.x * v.x + v.y * v.y + v.z * v.z);
        vals[5] = d.frc[i].w;
        if (sp.kind == 0) {
            // rotational term I |omega|^2 with I = 0.4 m r^2
            // (examples/bench_sphere_haff_cooling/main.rs:88-100)
            const double r = d.pos[i].w;
            const double4 w = d.omg[i];
            const double inertia = 0.4 * m * r * r;
            vals[6] = inertia * (w.x * w.x + w.y * w.y + w.z * w.z);
        }
    }
    double out[7];
    if (system_reduce<7>(d, s, gb, vals, out) && threadIdx.x == 0) {
        double* o = out16 + (size_t)s * THERMO_W;
        o[0] = 0.5 * out[4];
        o[1] = out[5];
        o[5] = sqrt(out[1] * out[1] + out[2] * out[2] + out[3] * out[3]);
        o[6] = out[0] > 0.0 ? out[6] / (3.0 * out[0]) : 0.0;  // T_rot = sum I w^2 / (3 M)
        o[8 + 0] = out[0];
        o[8 + 1] = out[1] / out[0];
        o[8 + 2] = out[2] / out[0];
        o[8 + 3] = out[3] / out[0];
    }
}

// thermo pass 2: sum m |v - vbar|^2 -> granular temperature; for mixed
// systems with a virial, also the sum of the per-particle virials the force
// kernel wrote (the plain path reduces them every step in k_final)
__global__ void __launch_bounds__(BLK) k_thermo2(Dev d, double* out16) {
    const int gb = blockIdx.x;
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    if (gb - sp.b0 >= sp.nb) return;  // past the particles: not in the reduction
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    double* o = out16 + (size_t)s * THERMO_W;
    const bool vir = sp.precision == 1 && sp.virial;
    double vals[7] = {0, 0, 0, 0, 0, 0, 0};
    if (li < sp.n) {
        const long long i = (long long)sp.p0 + li;
        const double4 v = d.vel[i];
        const double m = d.mass[i];
        const double dx = v.x - o[9], dy = v.y - o[10], dz = v.z - o[11];
        vals[0] = m * (dx * dx) + m * (dy * dy) + m * (dz * dz);
        if (vir)
            for (int q = 0; q < 6; q++) vals[1 + q] = d.vir[q * d.P + i];
    }
    double out[7];
    if (vir) {
        if (system_reduce<7>(d, s, gb, vals, out) && threadIdx.x == 0) {
            o[4] = out[0] / (3.0 * o[8]);
            for (int q = 0; q < 6; q++) o[16 + q] = out[1 + q];
        }
    } else {
        const double v1[1] = {vals[0]};
        double o1[1];
        if (system_reduce<1>(d, s, gb, v1, o1) && threadIdx.x == 0) o[4] = o1[0] / (3.0 * o[8]);
    }
}

// LJ potential energy per particle (owner entries of the full row; the sum
// over particles is the sum over the reference's half-list pairs), fp64,
// written to frc.w.  Launched on demand by the thermo query.
__global__ void __launch_bounds__(BLK) k_lj_pe(Dev d) {
    const int gb = blockIdx.x;
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    if (gb - sp.b0 >= sp.nb) return;  // past the particles: not in the reduction
    if (sp.kind != 1) return;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long i = (long long)sp.p0 + li;
    const double4 xi = d.pos[i];
    const int nn = d.nnum[i];
    const long long base = sp.lst0 + li;
    const bool mt = sp.nmat > 1;  // multi-type pair table
    const long long tq = (long long)sp.nmat * sp.nmat;
    const long long trow = mt ? sp.mat0 + (long long)d.type[i] * sp.nmat : 0;
    double pe = 0.0;
    for (int k = 0; k < nn; k++) {
        const uint32_t e = d.nlist[base + (long long)k * sp.npad];
        const uint32_t code = e >> IDX_BITS;
        if (code < 27u) continue;
        int sx, sy, sz;
        decode_shift((int)(code - 27u), sx, sy, sz);
        const long long j = sp.p0 + (e & IDX_MASK);
        const double4 xj = d.pos[j];
        const double dx = img_coord(xj.x, sx, sp.L[0]) - xi.x;
        const double dy = img_coord(xj.y, sy, sp.L[1]) - xi.y;
        const double dz = img_coord(xj.z, sz, sp.L[2]) - xi.z;
        const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
        double lj3 = sp.lj3, lj4 = sp.lj4, cut2 = sp.lj_cut2;
        if (mt) {
            const long long o = trow + d.type[j];
            lj3 = d.mat[o + TL_LJ3 * tq];
            lj4 = d.mat[o + TL_LJ4 * tq];
            cut2 = d.mat[o + TL_CUT2 * tq];
        }
        if (r2 >= cut2) continue;
        const double r2inv = 1.0 / r2;
        const double r6inv = r2inv * r2inv * r2inv;
        pe += r6inv * (lj3 * r6inv - lj4) * (sp.newton ? 1.0 : 0.5);
    }
    d.frc[i].w = pe;
}

// ----------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------
int launch_initial(const Dev& d, cudaStream_t st) {
    k_initial<<<d.nrun, BLK, 0, st>>>(d);
    return 1;
}

// The rebuild kernels walk the device-built work list with grid-stride
// loops; their grids (fixed when a graph is captured) are the running blocks,
// capped at a few waves of the GPU.
int launch_rebuild(const Dev& d, cudaStream_t st) {
    constexpr int CAP = 152 * 16;
    const int gp = d.nrun < CAP ? d.nrun : CAP;
    const int gb = d.nrun * BUILD_SUBS < 2 * CAP ? d.nrun * BUILD_SUBS : 2 * CAP;
    const int gs = d.nrun_sys < 304 ? d.nrun_sys : 304;
    const int gc = d.ncrun < CAP ? d.ncrun : CAP;
    const int gs_ = d.ncrun * CS_SUBS < 2 * CAP ? d.ncrun * CS_SUBS : 2 * CAP;
    k_rb_plan<<<1, 1024, 0, st>>>(d);
    k_cells<<<gp, BLK, 0, st>>>(d);
    k_scan<<<gs, 1024, 0, st>>>(d);
    k_cellscan<<<gc, BLK, 0, st>>>(d);
    k_scatter<<<gp, BLK, 0, st>>>(d);
    k_cellsort<<<gs_, BLK, 0, st>>>(d);
    k_gather<<<gp, BLK, 0, st>>>(d);
    k_copyback<<<gp, BLK, 0, st>>>(d);
    k_build<<<gb, BUILD_WARPS * 32, 0, st>>>(d);
    return 9;
}

int launch_force_fp64(const Dev& dall, int has_lj, int has_dem, int tpp, cudaStream_t st) {
    int n = 0;
    has_dem = has_dem && dall.nrun_kind[0] > 0;
    has_lj = has_lj && dall.nrun_kind[1] > 0;
    if (has_lj) {
        const Dev d = kind_view(dall, 1);
        if (d.lj_multi) {
            switch (tpp) {
                case 2: k_lj_fp64<2, true><<<d.nrun * 2, BLK, 0, st>>>(d); break;
                case 4: k_lj_fp64<4, true><<<d.nrun * 4, BLK, 0, st>>>(d); break;
                case 8: k_lj_fp64<8, true><<<d.nrun * 8, BLK, 0, st>>>(d); break;
                default: k_lj_fp64<1, true><<<d.nrun, BLK, 0, st>>>(d); break;
            }
        } else {
            switch (tpp) {
                case 2: k_lj_fp64<2, false><<<d.nrun * 2, BLK, 0, st>>>(d); break;
                case 4: k_lj_fp64<4, false><<<d.nrun * 4, BLK, 0, st>>>(d); break;
                case 8: k_lj_fp64<8, false><<<d.nrun * 8, BLK, 0, st>>>(d); break;
                default: k_lj_fp64<1, false><<<d.nrun, BLK, 0, st>>>(d); break;
            }
        }
        n++;
    }
    if (has_dem) {
        const Dev d = kind_view(dall, 0);
        k_dem_fp64<<<d.nrun, BLK, 0, st>>>(d);
        n++;
    }
    return n;
}

// WHILE-graph loop control: one step done; continue while steps remain and
// some system is still active.
__global__ void k_loop_ctl(Dev d, long long* counter, unsigned long long handle) {
    if (threadIdx.x != 0) return;
    const long long left = *counter - 1;
    *counter = left;
    unsigned int any = 0;
    for (int q = 0; q < d.nsys && !any; q++) any = sys_active(d.ss + q) ? 1u : 0u;
    cudaGraphSetConditional((cudaGraphConditionalHandle)handle, (left > 0 && any) ? 1u : 0u);
}

int launch_loop_ctl(const Dev& d, long long* counter, unsigned long long handle, cudaStream_t st) {
    k_loop_ctl<<<1, 32, 0, st>>>(d, counter, handle);
    return 1;
}

// Plane walls (wall_contact_force, crates/dem_wall/src/lib.rs:848-990), added
// after the pair forces: sphere-wall Hertz with R* = r and m* = m, viscous
// damping, JKR / DMT / SJKR adhesion, no tangential force, and the constant
// twisting torque; the reference's fp64 arithmetic (this file: no fma).
// wall_contact_force for plane walls (dem_wall/src/lib.rs:848-985).  A wall
// with a constant velocity has moved by velocity * dt once per step before the
// force (wall_move, lib.rs:766-790): moves = steps done + 1 inside a step,
// steps done for a force evaluation outside one.
__global__ void __launch_bounds__(BLK) k_walls(Dev d, int integrating) {
    const int gb = d.blk_run[blockIdx.x];
    const int s = d.blk_sys[gb];
    const SysParams& sp = d.sp[s];
    if (sp.nwall == 0 || sp.kind != 0 || !sys_active(d.ss + s)) return;
    const int li = (gb - sp.b0) * BLK + threadIdx.x;
    if (li >= sp.n) return;
    const long long i = (long long)sp.p0 + li;
    const double PI = 3.141592653589793;
    const double SQRT_5_3 = 0.9128709291752768;
    const double4 x = d.pos[i];
    const double4 v = d.vel[i];
    const double4 w = d.omg[i];
    const double radius = x.w;
    const int mi = (int)d.type[i];
    double4 f = d.frc[i], tq = d.trq[i];
    bool touched = false;
    const double moves = (double)(d.ss[s].step + integrating);
    for (int k = 0; k < sp.nwall; k++) {
        const WallP& W = sp.walls[k];
        const double px = W.p[0] + moves * (W.vel[0] * sp.dt), py = W.p[1] + moves * (W.vel[1] * sp.dt),
                     pz = W.p[2] + moves * (W.vel[2] * sp.dt);
        if (!(x.x >= W.lo[0] && x.x <= W.hi[0] && x.y >= W.lo[1] && x.y <= W.hi[1] && x.z >= W.lo[2] &&
              x.z <= W.hi[2]))
            continue;
        const double dx = x.x - px, dy = x.y - py, dz = x.z - pz;
        const double distance = dx * W.nrm[0] + dy * W.nrm[1] + dz * W.nrm[2];
        if (distance <= 0.0) continue;
        const double r_eff = radius;
        const double e_eff = mtab(d, sp, T_EEFF, mi, W.mat);
        const double surface_energy = mtab(d, sp, T_SURFACE, mi, W.mat);
        const bool use_dmt = sp.adhesion_model == 1;
        const double delta_pulloff = (surface_energy > 0.0 && !use_dmt)
                                         ? cbrt(PI * PI * surface_energy * surface_energy * r_eff /
                                                (4.0 * e_eff * e_eff))
                                         : 0.0;
        const double delta = fmin(radius - distance, 0.5 * radius);
        if (delta <= 0.0 && surface_energy <= 0.0) continue;
        if (delta < -delta_pulloff) continue;
        const bool jkr_adhesion_only = surface_energy > 0.0 && !use_dmt && delta <= 0.0;
        double s_n = 0.0, k_n = 0.0;
        if (delta > 0.0) {
            const double sdr = sqrt(delta * r_eff);
            s_n = 2.0 * e_eff * sdr;
            k_n = 4.0 / 3.0 * e_eff * sdr;
        }
        const double m_r = d.mass[i];
        const double vx = v.x - W.vel[0], vy = v.y - W.vel[1], vz = v.z - W.vel[2];
        const double v_n = vx * W.nrm[0] + vy * W.nrm[1] + vz * W.nrm[2];
        const double beta = mtab(d, sp, T_BETA, mi, W.mat);
        const double cohesion_energy = mtab(d, sp, T_COHESION, mi, W.mat);
        double f_net;
        if (surface_energy > 0.0 && use_dmt) {
            const double f_dmt = 2.0 * PI * surface_energy * r_eff;
            const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
            f_net = k_n * delta - f_diss - f_dmt;
        } else if (surface_energy > 0.0) {
            const double f_adhesion = 1.5 * PI * surface_energy * r_eff;
            if (jkr_adhesion_only) {
                f_net = -f_adhesion;
            } else {
                const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
                f_net = k_n * delta - f_diss - f_adhesion;
            }
        } else if (cohesion_energy > 0.0) {
            const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
            const double f_cohesion = cohesion_energy * PI * delta * r_eff;
            f_net = k_n * delta - f_diss - f_cohesion;
        } else {
            const double f_diss = 2.0 * beta * SQRT_5_3 * sqrt(s_n * m_r) * v_n;
            f_net = fmax(k_n * delta - f_diss, 0.0);
        }
        f.x += f_net * W.nrm[0];
        f.y += f_net * W.nrm[1];
        f.z += f_net * W.nrm[2];
        if (delta > 0.0) {
            const double mu_tw = mtab(d, sp, T_TWIST_FRICTION, mi, W.mat);
            if (mu_tw > 0.0) {
                const double twist = w.x * W.nrm[0] + w.y * W.nrm[1] + w.z * W.nrm[2];
                if (fabs(twist) > 1e-30) {
                    const double tau = mu_tw * fabs(f_net) * r_eff;
                    const double sign_tw = twist > 0.0 ? -1.0 : 1.0;
                    tq.x += sign_tw * tau * W.nrm[0];
                    tq.y += sign_tw * tau * W.nrm[1];
                    tq.z += sign_tw * tau * W.nrm[2];
                }
            }
        }
        touched = true;
    }
    if (touched) {
        d.frc[i] = f;
        d.trq[i] = tq;
    }
}

int launch_walls(const Dev& d, int integrating, cudaStream_t st) {
    k_walls<<<d.nrun, BLK, 0, st>>>(d, integrating);
    return 1;
}

int launch_final(const Dev& d, cudaStream_t st, int integrate) {
    k_final<<<d.nrun, BLK, 0, st>>>(d, integrate);
    return 1;
}

int launch_ke_init(const Dev& d, cudaStream_t st) {
    k_ke_init<<<d.nblocks, BLK, 0, st>>>(d);
    return 1;
}

int launch_thermo(const Dev& d, double* out, cudaStream_t st) {
    k_lj_pe<<<d.nblocks, BLK, 0, st>>>(d);
    k_thermo1<<<d.nblocks, BLK, 0, st>>>(d, out);
    k_thermo2<<<d.nblocks, BLK, 0, st>>>(d, out);
    return 3;
}

}  // namespace mdg
