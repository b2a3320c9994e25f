// ss4d_project.cu — start of a mixed segmentation step's first FP32 round by
// projection onto the previous steps' changes.
//
// With the extrapolated start, the first refinement pass measures the FP64
// residual of u^n + e (e the cubic extrapolation of the last three changes
// d_{n-1}, d_{n-2}, d_{n-3} that the unpack left in dR[0] / dB) and hands the
// FP32 round the correction equation A d = rhs, rhs = b - A (u^n + e).  The
// round starts from d = 0.  Here it starts instead from the combination
// d0 = sum_k c_k v_k of the vectors v = {d_{n-1}, d_{n-2}, e} (the history
// arrays and the extrapolation; {d_{n-1}, d_{n-2}} after two steps) whose
// residual rhs - A d0 is least in the 2-norm: the normal equations H c = g
// with H_ij = <A v_i, A v_j>, g_i = <rhs, A v_i>.  This is the projection of
// the new solution onto the span of the previous ones (P. F. Fischer,
// "Projection techniques for iterative solution of Ax = b with successive
// right-hand sides", Comput. Methods Appl. Mech. Engrg. 163 (1998) 193-204),
// here over the last three changes.  The cubic extrapolation is one point of
// that span, so the start is never worse in the norm the products are formed
// in; A is the FP32 sweeps' operator (their compressed records) and the sums
// are FP32 per thread and FP64 across threads.  The FP64 refinement that ends
// the round measures the exact FP64 residual as always, so the stop rule and
// the tolerance do not depend on the start.
//
//   k_proj_dots<COL>: per block the nine sums H_00 H_01 H_02 H_11 H_12 H_22
//                     g_0 g_1 g_2 over a sample of the targets of colour
//                     COL (every PROJ_STRIDE-th tile);
//   k_proj_solve:     one block sums the partials of both colours in a fixed
//                     order and solves H c = g (Cholesky, FP64); a system that
//                     is not positive definite, or sums that are not finite,
//                     leave the start at zero;
//   k_proj_start:     d0 into the round's correction arrays (red: dR[dsrc],
//                     black: dB) and LoopState.keep, so that the round's start
//                     keeps it (k_zero_delta).
#include "ss4d_sweep.cuh"

namespace ss4d {

// the three vectors, per colour (split layout; their ghost cells are zero)
struct ProjVecs {
    const float *v[3][2];
};

// fraction f of a compressed record's packed fractions q, decoded where it
// is used (three products share a record; the decoded values are not held)
__device__ __forceinline__ float wq(const uint4 q, int f)
{
    const unsigned x = f < 2 ? q.x : f < 4 ? q.y : f < 6 ? q.z : q.w;
    return (f & 1) ? q16_hi(x) : q16_lo(x);
}

// sum of the eight fractions: their 16-bit integers summed (at most 20
// bits) and scaled, exactly the FP32 sum of the decoded fractions
__device__ __forceinline__ float qsum(const uint4 q)
{
    const unsigned a = (q.x & 0xFFFFu) + (q.x >> 16) + (q.y & 0xFFFFu) + (q.y >> 16) + (q.z & 0xFFFFu) + (q.z >> 16) +
                       (q.w & 0xFFFFu) + (q.w >> 16);
    return (float)a * 0x1p-16f;
}

// A v at the pair of targets s, s + 1 (the second only when `two`; row
// phase p) for one vector: its own values and its other-colour neighbours
// read as 8-byte pairs, as the FP32 sweep reads them (sweep32_pair)
__device__ __forceinline__ float2 av_pair(const float *__restrict__ own, const float *__restrict__ oth, unsigned s,
                                          int p, bool two, unsigned Hy, unsigned Hz, unsigned Hw, const uint4 q0,
                                          const uint4 q1, float sc0, float sc1, float dg0, float dg1)
{
    const float2 u = __ldg(reinterpret_cast<const float2 *>(own + s));
    const float2 vx = __ldg(reinterpret_cast<const float2 *>(oth + s));
    const float ex = __ldg(oth + (p ? s - 1 : s + 2));
    const float2 yp = __ldg(reinterpret_cast<const float2 *>(oth + s + Hy));
    const float2 ym = __ldg(reinterpret_cast<const float2 *>(oth + s - Hy));
    const float2 zp = __ldg(reinterpret_cast<const float2 *>(oth + s + Hz));
    const float2 zm = __ldg(reinterpret_cast<const float2 *>(oth + s - Hz));
    const float2 wp = __ldg(reinterpret_cast<const float2 *>(oth + s + Hw));
    const float2 wm = __ldg(reinterpret_cast<const float2 *>(oth + s - Hw));
    // record order: +x (column s_t - p + 1), -x (s_t - p), +y, -y, +z, -z, +w, -w
    const float n0[8] = {p ? vx.x : vx.y, p ? ex : vx.x, yp.x, ym.x, zp.x, zm.x, wp.x, wm.x};
    float T = wq(q0, 0) * n0[0];
#pragma unroll
    for (int f = 1; f < 8; ++f)
        T = fmaf(wq(q0, f), n0[f], T);
    float2 r;
    r.x = fmaf(dg0, u.x, -sc0 * T);
    r.y = 0.f;
    if (two) {
        const float n1[8] = {p ? vx.y : ex, p ? vx.x : vx.y, yp.y, ym.y, zp.y, zm.y, wp.y, wm.y};
        T = wq(q1, 0) * n1[0];
#pragma unroll
        for (int f = 1; f < 8; ++f)
            T = fmaf(wq(q1, f), n1[f], T);
        r.y = fmaf(dg1, u.y, -sc1 * T);
    }
    return r;
}

// The sums run over every PROJ_STRIDE-th tile of the pair configuration, a
// systematic sample of the volume (tiles go along x chunks, then j groups, k
// planes, frames; an odd stride steps through every x chunk and j group when
// their counts are powers of two, as at the benchmark's size).  Three
// coefficients fitted from a ninth of the targets (9 M of each colour at
// 256x256x128x20) start the round as well as from all of them: over 50 steps
// of that workload 328 FP32 iterations against 326, the three projection
// kernels 2.52 -> 0.97 ms per step.  A volume of fewer than PROJ_STRIDE
// tiles per colour samples its first tile; any sample gives a valid start,
// since the FP64 refinement judges the result.
constexpr int PROJ_STRIDE = 9;

// two adjacent targets per thread (pc: make_pair_cfg), 64 registers (four
// blocks per SM); every block of the launch writes its nine partials
template <int COL>
__global__ void __launch_bounds__(256, 4) k_proj_dots(Geo g, Split sp, SweepCfg pc, SplitBufs b, ProjVecs V, int m,
                                                      double *part)
{
    const unsigned Hy = (unsigned)sp.Hs, Hz = Hy * (unsigned)g.jM, Hw = Hz * (unsigned)g.kM;
    const uint4 *__restrict__ cq = b.coefq[COL];
    const float *__restrict__ cs = b.coefs[COL];
    const double *__restrict__ rp = b.rpre[COL];
    const int tx = threadIdx.x & (pc.XT - 1), ty = threadIdx.x / pc.XT;
    float acc[9];
#pragma unroll
    for (int q = 0; q < 9; ++q)
        acc[q] = 0.f;
    for (long long t = (long long)blockIdx.x * PROJ_STRIDE; t < pc.ntiles; t += (long long)gridDim.x * PROJ_STRIDE) {
        const TileCoord tc = tile_coord(g, pc, t, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (COL + tc.j + tc.k + tc.l) & 1;
        const int xi = 2 * tc.xi; // the pair's first target; the second is xi + 1
        const int i = 2 * xi + 2 - p;
        if (i > g.nx)
            continue;
        const bool two = i + 2 <= g.nx;
        const unsigned s = (((unsigned)tc.l * g.kM + tc.k) * g.jM + tc.j) * Hy + xi + sp.A;
        const unsigned tq = ((((unsigned)tc.l - 1) * g.nz + (tc.k - 1)) * g.ny + (tc.j - 1)) * sp.nxh + xi;
        const uint4 q0 = __ldcs(cq + tq);
        const float sc0 = __ldcs(cs + tq);
        uint4 q1 = make_uint4(0u, 0u, 0u, 0u);
        float sc1 = 0.f;
        if (two) {
            q1 = __ldcs(cq + tq + 1);
            sc1 = __ldcs(cs + tq + 1);
        }
        const float dg0 = fmaf(sc0, qsum(q0), 1.f);
        const float dg1 = two ? fmaf(sc1, qsum(q1), 1.f) : 0.f;
        // rpre holds A u0 - b: the correction equation's right-hand side is its negative
        const double2 r2 = __ldcs(reinterpret_cast<const double2 *>(rp + s));
        const float rh0 = -d2f_bits(r2.x), rh1 = two ? -d2f_bits(r2.y) : 0.f;
        float2 Av[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
            Av[k] = k < m ? av_pair(V.v[k][COL], V.v[k][COL ^ 1], s, p, two, Hy, Hz, Hw, q0, q1, sc0, sc1, dg0, dg1)
                          : make_float2(0.f, 0.f);
        // the second target's terms are zero when it does not exist
        acc[0] = fmaf(Av[0].x, Av[0].x, fmaf(Av[0].y, Av[0].y, acc[0]));
        acc[1] = fmaf(Av[0].x, Av[1].x, fmaf(Av[0].y, Av[1].y, acc[1]));
        acc[2] = fmaf(Av[0].x, Av[2].x, fmaf(Av[0].y, Av[2].y, acc[2]));
        acc[3] = fmaf(Av[1].x, Av[1].x, fmaf(Av[1].y, Av[1].y, acc[3]));
        acc[4] = fmaf(Av[1].x, Av[2].x, fmaf(Av[1].y, Av[2].y, acc[4]));
        acc[5] = fmaf(Av[2].x, Av[2].x, fmaf(Av[2].y, Av[2].y, acc[5]));
        acc[6] = fmaf(rh0, Av[0].x, fmaf(rh1, Av[0].y, acc[6]));
        acc[7] = fmaf(rh0, Av[1].x, fmaf(rh1, Av[1].y, acc[7]));
        acc[8] = fmaf(rh0, Av[2].x, fmaf(rh1, Av[2].y, acc[8]));
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double tot = block_sum((double)acc[q]);
        if (threadIdx.x == 0)
            part[(size_t)(COL * 9 + q) * gridDim.x + blockIdx.x] = tot;
    }
}

// c[0..2] for the start; st->keep = 1 when the start is used
__global__ void k_proj_solve(const double *__restrict__ part, int grid, int m, LoopState *st, float *c)
{
    __shared__ double sum[9];
    if (st->stop)
        return;
    for (int q = 0; q < 9; ++q) {
        double a = 0.0;
        for (int t = threadIdx.x; t < grid; t += blockDim.x)
            a += part[(size_t)q * grid + t] + part[(size_t)(9 + q) * grid + t];
        a = block_sum(a);
        if (threadIdx.x == 0)
            sum[q] = a;
        __syncthreads();
    }
    if (threadIdx.x != 0)
        return;
    const int iu[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    double H[3][3], x[3], L[3][3] = {{0.0}};
    bool ok = m >= 1;
    for (int i = 0; i < m; ++i) {
        x[i] = sum[6 + i];
        for (int j = 0; j < m; ++j)
            H[i][j] = sum[iu[i][j]];
    }
    // Cholesky H = L L^T; a pivot below 1e-12 of its diagonal entry (or not
    // finite) rejects the system
    for (int j = 0; j < m && ok; ++j) {
        double d = H[j][j];
        for (int k = 0; k < j; ++k)
            d -= L[j][k] * L[j][k];
        if (!(d > 1e-12 * H[j][j]) || !isfinite(d)) {
            ok = false;
            break;
        }
        L[j][j] = sqrt(d);
        for (int i = j + 1; i < m; ++i) {
            double e = H[i][j];
            for (int k = 0; k < j; ++k)
                e -= L[i][k] * L[j][k];
            L[i][j] = e / L[j][j];
        }
    }
    if (ok) {
        for (int i = 0; i < m; ++i) { // L y = g
            for (int k = 0; k < i; ++k)
                x[i] -= L[i][k] * x[k];
            x[i] /= L[i][i];
        }
        for (int i = m - 1; i >= 0; --i) { // L^T c = y
            for (int k = i + 1; k < m; ++k)
                x[i] -= L[k][i] * x[k];
            x[i] /= L[i][i];
        }
        for (int i = 0; i < m; ++i)
            ok = ok && isfinite(x[i]);
    }
    for (int i = 0; i < 3; ++i)
        c[i] = ok && i < m ? (float)x[i] : 0.f;
    st->keep = ok ? 1 : 0;
    st->proj = ok ? 1 : 0;
}

__global__ void __launch_bounds__(256) k_proj_start(Split sp, SplitBufs b, ProjVecs V, int m,
                                                    const float *__restrict__ c, const LoopState *__restrict__ st)
{
    if (st->stop || !st->keep)
        return;
    const float c0 = c[0], c1 = c[1], c2 = c[2];
    float *red = pick(b.dR, st->dsrc);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < sp.cs;
         t += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int col = 0; col < 2; ++col) {
            float d = c0 * V.v[0][col][t];
            if (m >= 2)
                d = fmaf(c1, V.v[1][col][t], d);
            if (m >= 3)
                d = fmaf(c2, V.v[2][col][t], d);
            (col == 0 ? red : b.dB)[t] = d;
        }
    }
}

void launch_projection(const Geo &g, const Split &sp, const SweepCfg &cfg, SplitBufs b, float *const *hist, int m,
                       double *part, float *c, LoopState *st, int sm_count, cudaStream_t s)
{
    ProjVecs V;
    for (int col = 0; col < 2; ++col) {
        V.v[0][col] = hist[col];     // d_{n-1}
        V.v[1][col] = hist[2 + col]; // d_{n-2}
    }
    V.v[2][0] = b.dR[0]; // the extrapolation (its red part is in dR[0])
    V.v[2][1] = b.dB;
    const SweepCfg pc = make_pair_cfg(g, sp, cfg);
    // co-resident blocks only (at most the solver's grid, whose partial
    // buffer part is sized for)
    static int per_sm = 0;
    if (!per_sm) {
        int a = 0, b1 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_proj_dots<0>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_proj_dots<1>, 256, 0);
        per_sm = a < b1 ? a : b1;
        if (per_sm < 1)
            per_sm = 1;
    }
    int grid = sm_count * per_sm;
    if (grid > cfg.grid)
        grid = cfg.grid;
    k_proj_dots<0><<<grid, 256, 0, s>>>(g, sp, pc, b, V, m, part);
    k_proj_dots<1><<<grid, 256, 0, s>>>(g, sp, pc, b, V, m, part);
    k_proj_solve<<<1, 256, 0, s>>>(part, grid, m, st, c);
    k_proj_start<<<sm_count * 8, 256, 0, s>>>(sp, b, V, m, c, st);
}

} // namespace ss4d
