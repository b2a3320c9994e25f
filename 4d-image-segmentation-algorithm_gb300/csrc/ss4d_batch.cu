// ss4d_batch.cu — batched solves of many independent volumes (uneven sizes,
// per-volume parameters) in the plain FP64 form or the mixed form.
//
// Each volume owns a solver handle for its buffers, its coefficient assembly
// (which in the mixed form also forms the step's first refinement pass) and
// its pack/unpack (ss4d_api.cu), extrapolated start included.  What is
// batched is the SOR loop: every phase of a loop body walks the
// concatenated tile lists of all volumes (volume v owns tiles [tile0_v,
// tile0_{v+1})), every tile with its volume's own tile shape; a tile whose
// volume has stopped, or (mixed form) is in another phase of its loop, is
// skipped.  Residual partial sums are kept per (volume, block) in a fixed
// order, and one controller runs every volume's stopping test (the
// single-volume state machines of ss4d_sweep.cuh).  By default the whole
// loop is one persistent launch (k_bsolve: a co-resident grid, its phases
// separated by a bounded grid barrier, the controller in block 0);
// otherwise each phase is a kernel of a CUDA graph's while loop, which the
// controller keeps going while any volume is active.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ss4d_sweep.cuh"

using namespace ss4d;

#define BMAX SS4D_BATCH_MAX_VOLUMES
#define BWARPS 8 // 256 threads per block

namespace {

struct BVol {
    Geo g;
    Split sp;
    SweepCfg cfg;
    SplitBufs b;
    long long tile0;
};


ss4d_status bfail(ss4d_status st, const char *fmt, ...)
{
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error_text(buf);
    return st;
}

#define BCK(call)                                                                                                  \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            cudaGetLastError();                                                                                    \
            return bfail(e_ == cudaErrorMemoryAllocation ? SS4D_ERR_ALLOC : SS4D_ERR_CUDA, "%s failed: %s", #call, \
                         cudaGetErrorString(e_));                                                                  \
        }                                                                                                          \
    } while (0)

#define BCKS(expr)                                                                                                 \
    do {                                                                                                           \
        ss4d_status s_ = (expr);                                                                                   \
        if (s_ != SS4D_OK)                                                                                         \
            return s_;                                                                                             \
    } while (0)

// ---------------------------------------------------------------------------
// kernels

// The grid-stride tile index that jumps a block from volume v to its first
// tile of volume v + 1 (the loop's t += gridDim.x lands on it): a volume the
// kernel does not work on costs a block one step, not one per tile.
__device__ __forceinline__ long long skip_to_next_volume(const BVol *__restrict__ vols, int v)
{
    const long long n0 = vols[v + 1].tile0, G = gridDim.x;
    long long off = ((long long)blockIdx.x - n0) % G;
    if (off < 0)
        off += G;
    return n0 + off - G;
}

// Walks the block's tiles of all volumes (grid-stride over the concatenated
// tile lists).  For every target of a volume that want(v) admits it calls
// body(v, V, g, sp, tc, p, s); when the block moves on from volume v it calls
// flush(v) (uniform over the block: t is).  The volume's description is read
// per tile (it stays in L1): holding it in registers doubled them.
template <int COL, class Want, class Body, class Flush>
__device__ __forceinline__ void walk_targets(const BVol *__restrict__ vols, int nv, long long total, Want want,
                                             Body body, Flush flush)
{
    int v = 0;
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        if (v + 1 < nv && t >= vols[v + 1].tile0) {
            flush(v);
            do
                ++v;
            while (v + 1 < nv && t >= vols[v + 1].tile0);
        }
        if (!want(v)) { // the whole block skips: v is uniform
            if (v + 1 >= nv)
                break;
            t = skip_to_next_volume(vols, v);
            continue;
        }
        const BVol &V = vols[v];
        const Geo g = V.g;
        const Split sp = V.sp;
        const SweepCfg cfg = V.cfg;
        const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
        const TileCoord tc = tile_coord(g, cfg, t - V.tile0, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (COL + tc.j + tc.k + tc.l) & 1;
        if (2 * tc.xi + 2 - p > g.nx)
            continue;
        const long long s = (((long long)tc.l * g.kM + tc.k) * g.jM + tc.j) * sp.Hs + tc.xi + sp.A;
        body(v, V, g, sp, tc, p, s);
    }
    flush(v);
}

// per-(volume, block) residual sums: a thread's sum goes to its warp's slot
// of the volume at each volume change, the block's to partial[v * grid + b]
// for the volumes the kernel worked on (the partials of the others belong to
// the kernel of their phase in the same loop body)
struct VolumeSums {
    double (*wacc)[BMAX];
    __device__ void clear()
    {
        for (int q = threadIdx.x; q < BWARPS * BMAX; q += blockDim.x)
            (&wacc[0][0])[q] = 0.0;
        __syncthreads();
    }
    __device__ void add(int v, double acc)
    {
        acc = warp_sum(acc);
        if ((threadIdx.x & 31) == 0)
            wacc[threadIdx.x >> 5][v] += acc;
    }
    template <class Want>
    __device__ void write(int nv, double *partial, Want want)
    {
        __syncthreads();
        for (int q = threadIdx.x; q < nv; q += blockDim.x) {
            if (!want(q))
                continue;
            double sum = 0.0;
            for (int w = 0; w < BWARPS; ++w)
                sum += wacc[w][q];
            partial[(long long)q * gridDim.x + blockIdx.x] = sum;
        }
    }
};

// ---- plain FP64 form

// Its own loop rather than walk_targets: the walker form of this kernel
// measured 8 % slower on the 16-volume workload (A/B on one box).
template <int COL>
__device__ __forceinline__ void bsweep64(const BVol *__restrict__ vols, int nv, long long total,
                                         const LoopState *__restrict__ st, double *partial, double (*wacc)[BMAX])
{
    VolumeSums sums{wacc};
    sums.clear();
    int v = 0;
    double acc = 0.0;
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        if (v + 1 < nv && t >= vols[v + 1].tile0) {
            sums.add(v, acc);
            acc = 0.0;
            do
                ++v;
            while (v + 1 < nv && t >= vols[v + 1].tile0);
        }
        if (st[v].stop)
            continue; // the whole block skips: v is uniform (a jump to the next
                      // volume, as walk_targets does, measured 4 % slower here)
        const BVol &V = vols[v];
        const Geo g = V.g;
        const Split sp = V.sp;
        const SweepCfg cfg = V.cfg;
        const int z = st[v].z;
        const double *src;
        double *dst;
        const double *oth;
        if (COL == 0) {
            src = (z & 1) ? V.b.R[1] : V.b.R[0];
            dst = (z & 1) ? V.b.R[0] : V.b.R[1];
            oth = V.b.Bk;
        } else {
            src = V.b.Bk;
            dst = V.b.Bk;
            oth = (z & 1) ? V.b.R[1] : V.b.R[0];
        }
        const double *cf = V.b.coef[COL];
        const double *pv = V.b.P[COL];
        const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
        const TileCoord tc = tile_coord(g, cfg, t - V.tile0, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (COL + tc.j + tc.k + tc.l) & 1;
        const int i = 2 * tc.xi + 2 - p;
        if (i > g.nx)
            continue;
        const long long s = (((long long)tc.l * g.kM + tc.k) * g.jM + tc.j) * sp.Hs + tc.xi + sp.A;
        const double r = sweep64_target(g, sp, tc, p, s, src, dst, oth, cf, pv);
        acc = fma(r, r, acc);
    }
    sums.add(v, acc);
    sums.write(nv, partial, [&](int q) { return !st[q].stop; });
}

template <int COL>
__global__ void __launch_bounds__(256) k_bsweep64(const BVol *__restrict__ vols, int nv, long long total,
                                                  const LoopState *__restrict__ st, double *partial)
{
    __shared__ double wacc[BWARPS][BMAX];
    bsweep64<COL>(vols, nv, total, st, partial, wacc);
}

// ---- mixed form (the single-volume kernels k_apply_black, k_refine,
// k_zero_delta, k_sweep32 of ss4d_kernels_fast.cu, per volume in its mode)

// (not when the assembly formed the pass: its first-difference kernel added
// the correction, LoopState.pre)
__device__ __forceinline__ void bapply_black(const BVol *__restrict__ vols, int nv, long long total,
                                             const LoopState *__restrict__ st)
{
    walk_targets<1>(
        vols, nv, total, [&](int v) { return st[v].mode == 0 && !st[v].stop && !st[v].pre; },
        [&](int, const BVol &V, const Geo &, const Split &, const TileCoord &, int, long long s) {
            V.b.Bk[s] += f2d_bits(V.b.dB[s]);
        },
        [](int) {});
}

__global__ void __launch_bounds__(256) k_bapply_black(const BVol *__restrict__ vols, int nv, long long total,
                                                      const LoopState *__restrict__ st)
{
    bapply_black(vols, nv, total, st);
}

// a volume whose first pass the assembly formed (LoopState.pre) only reads
// that pass's residual, as k_refine does
template <int COL>
__device__ __forceinline__ void brefine(const BVol *__restrict__ vols, int nv, long long total,
                                        const LoopState *__restrict__ st, double *partial, double (*wacc)[BMAX])
{
    VolumeSums sums{wacc};
    sums.clear();
    double acc = 0.0;
    auto want = [&](int v) { return st[v].mode == 0 && !st[v].stop; };
    walk_targets<COL>(
        vols, nv, total, want,
        [&](int v, const BVol &V, const Geo &g, const Split &sp, const TileCoord &tc, int p, long long s) {
            double *own = COL == 0 ? V.b.R[0] : V.b.Bk;
            const float *down = st[v].dsrc ? V.b.dR[1] : V.b.dR[0];
            const double *oth = COL == 0 ? V.b.Bk : V.b.R[0];
            const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
            double r;
            if (st[v].pre) {
                r = ld_stream(V.b.rpre[COL] + s);
            } else {
                const RefineOut o =
                    refine_target<COL>(g, sp, tc, p, s, Hy, Hz, Hw, own, down, oth, V.b.coef[COL], V.b.P[COL]);
                r = o.r;
                if (COL == 0)
                    own[s] = o.u;
            }
            acc = fma(r, r, acc);
            V.b.r32[COL][s] = d2f_bits(-r);
        },
        [&](int v) {
            sums.add(v, acc);
            acc = 0.0;
        });
    sums.write(nv, partial, want);
}

template <int COL>
__global__ void __launch_bounds__(256) k_brefine(const BVol *__restrict__ vols, int nv, long long total,
                                                 const LoopState *__restrict__ st, double *partial)
{
    __shared__ double wacc[BWARPS][BMAX];
    brefine<COL>(vols, nv, total, st, partial, wacc);
}

// zero the corrections of the volumes that start a round (unless the round
// keeps the correction in place)
__device__ __forceinline__ void bzero_delta(const BVol *__restrict__ vols, int nv, const LoopState *__restrict__ st)
{
    for (int v = 0; v < nv; ++v) {
        if (st[v].mode != 1 || st[v].stop || st[v].keep)
            continue;
        const BVol &V = vols[v];
        for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < V.sp.cs;
             t += (long long)gridDim.x * blockDim.x) {
            V.b.dR[0][t] = 0.f;
            V.b.dR[1][t] = 0.f;
            V.b.dB[t] = 0.f;
        }
    }
}

__global__ void k_bzero_delta(const BVol *__restrict__ vols, int nv, const LoopState *__restrict__ st)
{
    bzero_delta(vols, nv, st);
}

template <int COL>
__device__ __forceinline__ void bsweep32(const BVol *__restrict__ vols, int nv, long long total,
                                         const LoopState *__restrict__ st, const DevParams *__restrict__ par,
                                         double *partial, double (*wacc)[BMAX])
{
    VolumeSums sums{wacc};
    sums.clear();
    float acc = 0.f;
    auto want = [&](int v) { return (COL == 0 ? st[v].mode != 0 : st[v].mode == 2) && !st[v].stop; };
    walk_targets<COL>(
        vols, nv, total, want,
        [&](int v, const BVol &V, const Geo &g, const Split &sp, const TileCoord &tc, int p, long long s) {
            const int ds = st[v].dsrc;
            const float *src;
            float *dst;
            const float *oth;
            if (COL == 0) {
                src = ds ? V.b.dR[1] : V.b.dR[0];
                dst = ds ? V.b.dR[0] : V.b.dR[1];
                oth = V.b.dB;
            } else {
                src = V.b.dB;
                dst = V.b.dB;
                oth = ds ? V.b.dR[1] : V.b.dR[0];
            }
            const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
            const Sweep32Out o = sweep32_target(g, sp, tc, p, s, Hy, Hz, Hw, src, oth, V.b.coefq[COL],
                                                V.b.coefs[COL], V.b.r32[COL], (float)par[v].omega);
            acc = fmaf(o.r, o.r, acc);
            dst[s] = o.u;
        },
        [&](int v) {
            sums.add(v, (double)acc);
            acc = 0.f;
        });
    sums.write(nv, partial, want);
}

template <int COL>
__global__ void __launch_bounds__(256) k_bsweep32(const BVol *__restrict__ vols, int nv, long long total,
                                                  const LoopState *__restrict__ st, const DevParams *__restrict__ par,
                                                  double *partial)
{
    __shared__ double wacc[BWARPS][BMAX];
    bsweep32<COL>(vols, nv, total, st, par, partial, wacc);
}

// z == 0: a fresh state (mode 0), whose first refinement pass the assembly
// formed where pre[v] says so (may be null)
__global__ void k_binit(LoopState *st, int nv, int z, const int *pre)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    if (z == 0) {
        memset(&st[v], 0, sizeof(LoopState));
        st[v].pre = pre ? pre[v] : 0;
    } else {
        st[v].z = z;
    }
}

// every volume's stopping test (as k_ctrl64 does for one volume); one
// block; returns (in every thread) whether a volume is still active
__device__ __forceinline__ int bctrl(const double *__restrict__ pred, const double *__restrict__ pblack, int grid,
                                     int nv, const DevParams *__restrict__ par, LoopState *st)
{
    __shared__ int any;
    if (threadIdx.x == 0)
        any = 0;
    __syncthreads();
    for (int v = 0; v < nv; ++v) {
        if (st[v].stop)
            continue;
        double a = 0.0, c = 0.0;
        for (int t = threadIdx.x; t < grid; t += blockDim.x) {
            a += pred[(long long)v * grid + t];
            c += pblack[(long long)v * grid + t];
        }
        a = block_sum(a);
        c = block_sum(c);
        if (threadIdx.x == 0 && !ctrl64_update(&st[v], a, c, &par[v]))
            any = 1;
        __syncthreads();
    }
    __syncthreads();
    return any;
}

__global__ void k_bctrl(const double *__restrict__ pred, const double *__restrict__ pblack, int grid, int nv,
                        const DevParams *__restrict__ par, LoopState *st, cudaGraphConditionalHandle h, int use_cond)
{
    const int any = bctrl(pred, pblack, grid, nv, par, st);
    if (threadIdx.x == 0 && use_cond)
        cudaGraphSetConditional(h, any ? 1u : 0u);
}

// every volume's mixed-form controller step (k_ctrl_mixed per volume)
__device__ __forceinline__ int bctrl_mixed(const double *__restrict__ pred, const double *__restrict__ pblack,
                                           int grid, int nv, const DevParams *__restrict__ par, LoopState *st)
{
    __shared__ int any;
    if (threadIdx.x == 0)
        any = 0;
    __syncthreads();
    for (int v = 0; v < nv; ++v) {
        if (st[v].stop)
            continue;
        const int mode = st[v].mode;
        double a = 0.0, c = 0.0;
        if (mode != 1)
            for (int t = threadIdx.x; t < grid; t += blockDim.x) {
                a += pred[(long long)v * grid + t];
                c += pblack[(long long)v * grid + t];
            }
        a = block_sum(a);
        c = block_sum(c);
        if (threadIdx.x == 0 && !ctrl_mixed_update(&st[v], a, c, &par[v]))
            any = 1;
        __syncthreads();
    }
    __syncthreads();
    return any;
}

__global__ void k_bctrl_mixed(const double *__restrict__ pred, const double *__restrict__ pblack, int grid, int nv,
                              const DevParams *__restrict__ par, LoopState *st, cudaGraphConditionalHandle h,
                              int use_cond)
{
    const int any = bctrl_mixed(pred, pblack, grid, nv, par, st);
    if (threadIdx.x == 0 && use_cond)
        cudaGraphSetConditional(h, any ? 1u : 0u);
}

// ---- the whole loop in one launch

// A grid-wide barrier for a co-resident grid (cooperative launch): the last
// block to arrive resets the count and advances the generation the others
// wait on.  The wait is bounded (about a second of clock cycles); one that
// runs out sets err and returns false, and the caller leaves its loop.
struct GridBar {
    unsigned count, gen;
    int err, any;
};

__device__ __forceinline__ bool grid_sync(GridBar *gb)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &gb->gen;
        const unsigned g0 = *gen;
        __threadfence();
        if (atomicAdd(&gb->count, 1u) == gridDim.x - 1) {
            gb->count = 0;
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == g0) {
                if (clock64() - t0 > (1LL << 31)) {
                    atomicExch(&gb->err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int *)&gb->err == 0;
}

// The SOR loop of every volume as one persistent launch: the loop body's
// phases (those of the graph's body: refinement, zeroed corrections, FP32
// black and red sweeps, controller; or the FP64 black and red sweeps and the
// controller) run back to back with a grid barrier between them, until the
// controller finds no volume active or max_bodies bodies have run.  In the
// mixed form a phase (and its barrier) is left out when no active volume is
// in a mode it works on; every block reads the modes at the start of the
// body, after the controller's barrier, so the choice is the same in all.
// Six blocks of 256 threads per SM, as the separate kernels run (42
// registers at most).
template <int MIXED>
__global__ void __launch_bounds__(256, 6) k_bsolve(const BVol *__restrict__ vols, int nv, long long total,
                                                   LoopState *st, const DevParams *__restrict__ par, double *pred,
                                                   double *pblack, GridBar *gb, int max_bodies)
{
    __shared__ double wacc[BWARPS][BMAX];
    const int grid = gridDim.x;
    for (int body = 0; body < max_bodies; ++body) {
        if (MIXED) {
            int m0 = 0, m1 = 0, m2 = 0; // active volumes in mode 0 (refine), 1 (start a round), 2 (sweep)
            for (int v = 0; v < nv; ++v) {
                if (st[v].stop)
                    continue;
                const int mode = st[v].mode;
                m0 |= mode == 0;
                m1 |= mode == 1;
                m2 |= mode == 2;
            }
            if (m0) {
                bapply_black(vols, nv, total, st);
                if (!grid_sync(gb))
                    return;
                brefine<0>(vols, nv, total, st, pred, wacc);
                if (!grid_sync(gb))
                    return;
                brefine<1>(vols, nv, total, st, pblack, wacc);
                if (!grid_sync(gb))
                    return;
            }
            if (m1) {
                bzero_delta(vols, nv, st);
                if (!grid_sync(gb))
                    return;
            }
            if (m2) {
                bsweep32<1>(vols, nv, total, st, par, pblack, wacc);
                if (!grid_sync(gb))
                    return;
            }
            if (m1 || m2)
                bsweep32<0>(vols, nv, total, st, par, pred, wacc);
        } else {
            bsweep64<1>(vols, nv, total, st, pblack, wacc);
            if (!grid_sync(gb))
                return;
            bsweep64<0>(vols, nv, total, st, pred, wacc);
        }
        if (!grid_sync(gb))
            return;
        if (blockIdx.x == 0) {
            const int any = MIXED ? bctrl_mixed(pred, pblack, grid, nv, par, st) : bctrl(pred, pblack, grid, nv, par, st);
            if (threadIdx.x == 0)
                *(volatile int *)&gb->any = any;
        }
        if (!grid_sync(gb))
            return;
        if (*(volatile int *)&gb->any == 0)
            return;
    }
}

int bsweep_blocks_per_sm()
{
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_bsweep64<0>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bsweep64<1>, 256, 0);
    const int m = a < b ? a : b;
    return m > 0 ? m : 1;
}

} // namespace

// ---------------------------------------------------------------------------
// the batch handle

struct ss4d_batch {
    int n;
    ss4d_solver *vol[BMAX];
    BVol h_vols[BMAX];
    BVol *d_vols;
    LoopState *d_st, *h_st;
    DevParams *d_par, *h_par;
    double *d_partial;
    int grid;
    long long total;
    int dirty;
    cudaStream_t stream, cap;
    cudaGraph_t graph[2]; // per form: plain FP64, mixed
    cudaGraphExec_t exec[2];
    int use_graph, graph_failed;
    int mixed;
    int *d_pre, *h_pre; // per volume: the assembly formed the step's first refinement pass
    GridBar *d_bar;     // the persistent loop's grid barrier and its "any volume active" flag
    int persistent;     // run the loop as one persistent launch (default) or as the graph's while loop
    int withhold_barrier; // test of the timeout path (ss4d_batch_set_test_withhold_barrier)
    int pgrid[2];       // co-resident blocks of k_bsolve<0/1> (0: not yet known)
};

static void bfree_graph(ss4d_batch *b)
{
    for (int f = 0; f < 2; ++f) {
        if (b->exec[f])
            cudaGraphExecDestroy(b->exec[f]);
        if (b->graph[f])
            cudaGraphDestroy(b->graph[f]);
        b->exec[f] = nullptr;
        b->graph[f] = nullptr;
    }
}

extern "C" ss4d_status ss4d_batch_destroy(ss4d_batch *b)
{
    if (!b)
        return SS4D_OK;
    cudaStreamSynchronize(b->stream);
    bfree_graph(b);
    for (int v = 0; v < b->n; ++v)
        ss4d_solver_destroy(b->vol[v]);
    if (b->d_vols)
        cudaFree(b->d_vols);
    if (b->d_st)
        cudaFree(b->d_st);
    if (b->d_par)
        cudaFree(b->d_par);
    if (b->d_partial)
        cudaFree(b->d_partial);
    if (b->d_pre)
        cudaFree(b->d_pre);
    if (b->d_bar)
        cudaFree(b->d_bar);
    if (b->h_pre)
        cudaFreeHost(b->h_pre);
    if (b->h_st)
        cudaFreeHost(b->h_st);
    if (b->h_par)
        cudaFreeHost(b->h_par);
    if (b->cap)
        cudaStreamDestroy(b->cap);
    free(b);
    return SS4D_OK;
}

// refresh the host descriptors (tile ranges follow the volumes' shapes)
static ss4d_status bdescribe(ss4d_batch *b)
{
    long long t0 = 0;
    for (int v = 0; v < b->n; ++v) {
        SolverView w;
        BCKS(solver_view(b->vol[v], &w));
        b->h_vols[v].g = w.g;
        b->h_vols[v].sp = w.sp;
        b->h_vols[v].cfg = w.cfg;
        b->h_vols[v].b = w.b;
        b->h_vols[v].tile0 = t0;
        t0 += w.cfg.ntiles;
    }
    if (t0 != b->total)
        bfree_graph(b); // the tile count is a kernel argument of the graph
    b->total = t0;
    BCK(cudaMemcpyAsync(b->d_vols, b->h_vols, sizeof(BVol) * b->n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream)); // h_vols may change before the next call
    b->dirty = 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_create(int n, const ss4d_dims *dims, void *stream, ss4d_batch **out)
{
    if (!out || !dims || n < 1 || n > BMAX)
        return bfail(SS4D_ERR_INVALID, "invalid argument: need 1..%d volumes, dims and out", BMAX);
    *out = nullptr;
    ss4d_batch *b = (ss4d_batch *)calloc(1, sizeof(ss4d_batch));
    if (!b)
        return SS4D_ERR_ALLOC;
    b->n = n;
    b->stream = (cudaStream_t)stream;
    b->use_graph = 1;
    b->persistent = 1;
    b->dirty = 1;
    ss4d_status st = SS4D_OK;
    for (int v = 0; v < n && st == SS4D_OK; ++v) {
        st = ss4d_solver_create(&dims[v], SS4D_ARITH_FP64, stream, &b->vol[v]);
        if (st == SS4D_OK) {
            SolverView w;
            st = solver_view(b->vol[v], &w); // allocate the split buffers now
        }
    }
    if (st != SS4D_OK) {
        ss4d_batch_destroy(b);
        return st;
    }
    const int sm = solver_sm_count(b->vol[0]);
    b->grid = sm * bsweep_blocks_per_sm();
    cudaError_t e = cudaMalloc((void **)&b->d_vols, sizeof(BVol) * n);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&b->d_st, sizeof(LoopState) * n);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&b->d_par, sizeof(DevParams) * n);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&b->d_partial, sizeof(double) * 2 * (size_t)n * b->grid);
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&b->h_st, sizeof(LoopState) * n);
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&b->h_par, sizeof(DevParams) * n);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&b->d_pre, sizeof(int) * n);
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&b->h_pre, sizeof(int) * n);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&b->d_bar, sizeof(GridBar));
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ss4d_batch_destroy(b);
        return bfail(SS4D_ERR_ALLOC, "batch allocation failed: %s", cudaGetErrorString(e));
    }
    *out = b;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_graph(ss4d_batch *b, int enable)
{
    if (!b)
        return bfail(SS4D_ERR_INVALID, "invalid argument: batch is NULL");
    b->use_graph = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_persistent(ss4d_batch *b, int enable)
{
    if (!b)
        return bfail(SS4D_ERR_INVALID, "invalid argument: batch is NULL");
    b->persistent = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_test_withhold_barrier(ss4d_batch *b, int enable)
{
    if (!b)
        return bfail(SS4D_ERR_INVALID, "invalid argument: batch is NULL");
    b->withhold_barrier = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_arith(ss4d_batch *b, ss4d_arith arith)
{
    if (!b || (arith != SS4D_ARITH_FP64 && arith != SS4D_ARITH_MIXED))
        return bfail(SS4D_ERR_INVALID, "invalid argument: batches run the FP64 or the mixed form");
    for (int v = 0; v < b->n; ++v)
        BCKS(ss4d_solver_set_arith(b->vol[v], arith));
    b->mixed = arith == SS4D_ARITH_MIXED;
    b->dirty = 1; // the mixed form's buffers enter the descriptions
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_extrapolation(ss4d_batch *b, int order)
{
    if (!b)
        return bfail(SS4D_ERR_INVALID, "invalid argument: batch is NULL");
    for (int v = 0; v < b->n; ++v)
        BCKS(ss4d_solver_set_extrapolation(b->vol[v], order));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_projection(ss4d_batch *b, int enable)
{
    if (!b)
        return bfail(SS4D_ERR_INVALID, "invalid argument: batch is NULL");
    for (int v = 0; v < b->n; ++v)
        BCKS(ss4d_solver_set_projection(b->vol[v], enable));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_set_shape(ss4d_batch *b, int v, int xt, int k_block)
{
    if (!b || v < 0 || v >= b->n)
        return bfail(SS4D_ERR_INVALID, "invalid argument: no volume %d", v);
    BCKS(solver_set_shape(b->vol[v], xt, k_block));
    b->dirty = 1;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_autotune(ss4d_batch *b, const ss4d_params *p, double *const *d_u,
                                           const double *const *d_g, int *xt_out, int *kb_out)
{
    if (!b || !p || !d_u || !d_g)
        return bfail(SS4D_ERR_INVALID, "invalid argument: NULL batch, params, u or g");
    static const int kbs[] = {1, 2, 4, 8};
    for (int v = 0; v < b->n; ++v) {
        BCKS(solver_prepare_step(b->vol[v], &p[v], d_u[v], d_g + 8 * v));
        SolverView w;
        BCKS(solver_view(b->vol[v], &w));
        int top = 8;
        while (top < w.sp.nxh && top < 256)
            top <<= 1;
        float best = 1e30f;
        int bxt = 0, bkb = 4;
        for (int xt = 8; xt <= top; xt <<= 1) {
            for (int kb : kbs) {
                if (kb > w.g.nz)
                    continue;
                BCKS(solver_set_shape(b->vol[v], xt, kb));
                float ms = 0.f;
                BCKS(solver_time_sweeps(b->vol[v], &p[v], 1, &ms)); // warm-up
                BCKS(solver_time_sweeps(b->vol[v], &p[v], 3, &ms));
                if (ms < best) {
                    best = ms;
                    bxt = xt;
                    bkb = kb;
                }
            }
        }
        BCKS(solver_set_shape(b->vol[v], bxt, bkb));
        if (xt_out)
            xt_out[v] = bxt;
        if (kb_out)
            kb_out[v] = bkb;
    }
    b->dirty = 1;
    return SS4D_OK;
}

static double *bpart(ss4d_batch *b, int colour)
{
    return b->d_partial + (colour ? (size_t)b->n * b->grid : 0);
}

static void launch_bsweep(ss4d_batch *b, int colour, cudaStream_t st)
{
    if (colour == 0)
        k_bsweep64<0><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, bpart(b, 0));
    else
        k_bsweep64<1><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, bpart(b, 1));
}

static void launch_bctrl(ss4d_batch *b, unsigned long long h, int use_cond, cudaStream_t st)
{
    k_bctrl<<<1, 256, 0, st>>>(bpart(b, 0), bpart(b, 1), b->grid, b->n, b->d_par, b->d_st,
                               (cudaGraphConditionalHandle)h, use_cond);
}

// one loop body of the plain form: black half-sweep, red half-sweep, test
static void launch_body64(ss4d_batch *b, unsigned long long h, int use_cond, cudaStream_t st)
{
    launch_bsweep(b, 1, st);
    launch_bsweep(b, 0, st);
    launch_bctrl(b, h, use_cond, st);
}

// one loop body of the mixed form, as the single-volume one: refinement pass
// (volumes in mode 0), zeroed corrections (mode 1), FP32 black sweep (mode 2)
// and red sweep (modes 1 and 2), every volume's controller step
static void launch_body_mixed(ss4d_batch *b, unsigned long long h, int use_cond, cudaStream_t st)
{
    k_bapply_black<<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st);
    k_brefine<0><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, bpart(b, 0));
    k_brefine<1><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, bpart(b, 1));
    k_bzero_delta<<<1024, 256, 0, st>>>(b->d_vols, b->n, b->d_st);
    k_bsweep32<1><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, b->d_par, bpart(b, 1));
    k_bsweep32<0><<<b->grid, 256, 0, st>>>(b->d_vols, b->n, b->total, b->d_st, b->d_par, bpart(b, 0));
    k_bctrl_mixed<<<1, 256, 0, st>>>(bpart(b, 0), bpart(b, 1), b->grid, b->n, b->d_par, b->d_st,
                                     (cudaGraphConditionalHandle)h, use_cond);
}

static ss4d_status bbuild_graph(ss4d_batch *b)
{
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle h;
    BCK(cudaGraphCreate(&graph, 0));
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    alignas(cudaGraphNodeParams) unsigned char store[sizeof(cudaGraphNodeParams)];
    memset(store, 0, sizeof store);
    cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(store);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess)
        e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(b->cap, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        if (b->mixed)
            launch_body_mixed(b, (unsigned long long)h, 1, b->cap);
        else
            launch_body64(b, (unsigned long long)h, 1, b->cap);
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(b->cap, &body);
    }
    const int f = b->mixed;
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&b->exec[f], graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(graph);
        b->exec[f] = nullptr;
        return bfail(SS4D_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
    }
    b->graph[f] = graph;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_batch_seg_time_step(ss4d_batch *b, const ss4d_params *p, double *const *d_u,
                                                const double *const *d_g, ss4d_step_stats *stats)
{
    if (!b || !p || !d_u || !d_g)
        return bfail(SS4D_ERR_INVALID, "invalid argument: NULL batch, params, u or g");
    if (stats)
        memset(stats, 0, sizeof(ss4d_step_stats) * b->n);
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    BCK(cudaEventRecord(e0, b->stream));
    for (int v = 0; v < b->n; ++v) {
        BCKS(solver_prepare_step(b->vol[v], &p[v], d_u[v], d_g + 8 * v, &b->h_pre[v]));
        b->h_par[v].c = p[v].tau / (p[v].h * p[v].h);
        b->h_par[v].omega = p[v].omega_c;
        b->h_par[v].h4 = p[v].h * p[v].h * p[v].h * p[v].h;
        b->h_par[v].tol = p[v].gsTol;
        b->h_par[v].maxit = p[v].maxNoGSIteration;
        b->h_par[v].pad_ = 0;
    }
    if (b->dirty)
        BCKS(bdescribe(b));
    for (int v = 0; v < b->n; ++v) // after the volumes are described
        b->h_par[v].near_band = fabs(p[v].gsTol) * (double)b->h_vols[v].g.nint * 0x1p-53;
    BCK(cudaMemcpyAsync(b->d_par, b->h_par, sizeof(DevParams) * b->n, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_pre, b->h_pre, sizeof(int) * b->n, cudaMemcpyHostToDevice, b->stream));
    const int ib = (b->n + 63) / 64;
    k_binit<<<ib, 64, 0, b->stream>>>(b->d_st, b->n, 0, b->d_pre); // mixed: mode 0, refine first
    if (b->mixed) // each volume's projected start (when enabled), on its own loop state
        for (int v = 0; v < b->n; ++v)
            BCKS(solver_project_start(b->vol[v], b->h_pre[v], b->d_st + v));
    if (!b->mixed) {
        launch_bsweep(b, 0, b->stream); // the first red half-sweep
        k_binit<<<ib, 64, 0, b->stream>>>(b->d_st, b->n, 1, nullptr);
    }
    BCK(cudaGetLastError());
    int maxit = 0;
    for (int v = 0; v < b->n; ++v)
        maxit = p[v].maxNoGSIteration > maxit ? p[v].maxNoGSIteration : maxit;
    // a mixed body advances a volume by at most one inner iteration, and
    // every round adds a start and a refinement body
    const int guard_max = b->mixed ? 4 * (maxit + 4) + 16 : maxit + 8;
    bool graphed = false, persisted = false;
    if (b->persistent) {
        const int f = b->mixed;
        if (!b->pgrid[f]) {
            int per = 0;
            BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f ? (const void *)k_bsolve<1> : (const void *)k_bsolve<0>,
                                                             256, 0));
            const int cap = per * solver_sm_count(b->vol[0]);
            b->pgrid[f] = cap < b->grid ? cap : b->grid; // the partial arrays hold b->grid blocks
        }
        if (b->pgrid[f] > 0) {
            BCK(cudaMemsetAsync(b->d_bar, 0, sizeof(GridBar), b->stream));
            if (b->withhold_barrier) // the arrival count starts beyond the grid: no arrival completes the barrier
                BCK(cudaMemsetAsync(&b->d_bar->count, 0x80, sizeof(unsigned), b->stream));
            const BVol *vols = b->d_vols;
            int nv = b->n, mb = guard_max;
            long long total = b->total;
            LoopState *st = b->d_st;
            const DevParams *par = b->d_par;
            double *pred = bpart(b, 0), *pblack = bpart(b, 1);
            GridBar *gb = b->d_bar;
            void *args[] = {(void *)&vols, &nv, &total, &st, (void *)&par, &pred, &pblack, &gb, &mb};
            BCK(cudaLaunchCooperativeKernel(f ? (const void *)k_bsolve<1> : (const void *)k_bsolve<0>,
                                            dim3(b->pgrid[f]), dim3(256), args, 0, b->stream));
            persisted = true;
        }
    }
    if (!persisted && b->use_graph && !b->graph_failed) {
        if (!b->exec[b->mixed] && bbuild_graph(b) != SS4D_OK)
            b->graph_failed = 1;
        if (b->exec[b->mixed]) {
            BCK(cudaGraphLaunch(b->exec[b->mixed], b->stream));
            graphed = true;
        }
    }
    if (!graphed && !persisted) {
        for (int guard = 0; guard < guard_max; ++guard) {
            if (b->mixed)
                launch_body_mixed(b, 0, 0, b->stream);
            else
                launch_body64(b, 0, 0, b->stream);
            BCK(cudaGetLastError());
            BCK(cudaMemcpyAsync(b->h_st, b->d_st, sizeof(LoopState) * b->n, cudaMemcpyDeviceToHost, b->stream));
            BCK(cudaStreamSynchronize(b->stream));
            int active = 0;
            for (int v = 0; v < b->n; ++v)
                active += !b->h_st[v].stop;
            if (!active)
                break;
        }
    }
    for (int v = 0; v < b->n; ++v)
        BCKS(solver_finish_step(b->vol[v], b->d_st + v, d_u[v]));
    BCK(cudaEventRecord(e1, b->stream));
    BCK(cudaMemcpyAsync(b->h_st, b->d_st, sizeof(LoopState) * b->n, cudaMemcpyDeviceToHost, b->stream));
    GridBar hb;
    memset(&hb, 0, sizeof hb);
    if (persisted)
        BCK(cudaMemcpyAsync(&hb, b->d_bar, sizeof(GridBar), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    if (hb.err) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return bfail(SS4D_ERR_TIMEOUT, "the persistent batch loop's grid barrier gave up a wait");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ss4d_status worst = SS4D_OK;
    for (int v = 0; v < b->n; ++v) {
        const LoopState &L = b->h_st[v];
        if (stats) {
            stats[v].iterations = L.z;
            stats[v].residual = L.R;
            stats[v].first_residual = L.R_first;
            stats[v].refinements = b->mixed ? L.refinements : 0;
            stats[v].status = L.status;
            stats[v].near_tolerance = L.near;
            stats[v].projected = b->mixed ? L.proj : 0;
            stats[v].ms = ms;
        }
        if (L.status != SS4D_OK)
            worst = (ss4d_status)L.status;
    }
    if (worst != SS4D_OK)
        return bfail(worst, "a volume's SOR residual became non-finite");
    return SS4D_OK;
}
