// ss4d_ws.cu — the solver side of the learned warm start (mixed form).
//
// After the first FP64 refinement pass of a step, r32 holds the residual
// r0 = b - A u^n at u^n and LoopState::R_first its sum r0^2 h^4.  The exact
// first correction would be d = A^-1 r0 (u^{n+1} = u^n + d).  Here
//   features:  per interior voxel of frame l, 16 BF16 channels
//                0  r0/s            1, 2  r0/s at frames l-1, l+1 (0 outside 1..nt)
//                3  r0/(s diag)     (the first Jacobi iterate)
//                4..11  w_f = c a_f / diag for the faces e, w, n, s, t, b, fw, bw
//                12 1/diag          13 gbar (mean of the 8 face values of g)
//                14 u^n             15 I0 (the presmoothed image)
//              with s = sqrt(R_first / (N h^4)) the RMS of r0 and c a_f, diag the
//              step's own FP64 coefficient records;
//              stored channel-group planar, [nt][2][nz][ny][nx][8]
//   (the network maps them to d/s, ss4d_nn.cu)
//   apply:     the red and black corrections d = s * prediction;
//   check:     sum over both colours of (r0 - A32 d)^2 h^4, the correction
//              equation's residual at the prediction (FP32, as the sweeps);
//   decide:    keep the prediction as the start of the first FP32 round only if
//              that residual is below R_first (its value at d = 0); otherwise
//              the round starts from zero, as without the network.
#include <cuda_bf16.h>

#include "ss4d_conv_tc.cuh"
#include "ss4d_sweep.cuh"

namespace ss4d {

__device__ __forceinline__ float ws_inv_sigma(const Geo &g, const LoopState *st, const DevParams *dp)
{
    const double var = st->R_first / ((double)g.nint * dp->h4);
    return var > 0.0 ? rsqrtf(d2f_bits(var)) : 0.f;
}

__device__ __forceinline__ long long split_index(const Geo &g, const Split &sp, int i, int j, int k, int l)
{
    return (((long long)l * g.kM + k) * g.jM + j) * sp.Hs + ((i + 1) >> 1) + sp.A - 1;
}

__global__ void __launch_bounds__(256) k_ws_features(Geo g, Split sp, SplitBufs b, const double *__restrict__ i0,
                                                     CPtrs8 gin, const LoopState *__restrict__ st,
                                                     const DevParams *__restrict__ dp, __nv_bfloat16 *x0)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const float inv = ws_inv_sigma(g, st, dp);
    const int col = (i + j + k + l) & 1;
    const long long s = split_index(g, sp, i, j, k, l);
    float ch[16];
    ch[0] = pick(b.r32, col)[s] * inv;
    ch[1] = l > 1 ? pick(b.r32, col ^ 1)[split_index(g, sp, i, j, k, l - 1)] * inv : 0.f;
    ch[2] = l < g.nt ? pick(b.r32, col ^ 1)[split_index(g, sp, i, j, k, l + 1)] * inv : 0.f;
    const double *cv = pick(b.coef, col) + coef_at(coef_index(g, sp, i, j, k, l), 0, 10);
    const float idiag = 1.f / d2f_bits(cv[256]);
    ch[3] = ch[0] * idiag;
#pragma unroll
    for (int f = 0; f < 8; ++f)
        ch[4 + f] = d2f_bits(cv[32 * f]) * idiag;
    ch[12] = idiag;
    const long long o = nat_index(g, i, j, k, l);
    float gb = 0.f;
#pragma unroll
    for (int f = 0; f < 8; ++f)
        gb += d2f_bits(__ldg(gin.p[f] + o));
    ch[13] = gb * 0.125f;
    ch[14] = d2f_bits(col == 0 ? b.R[0][s] : b.Bk[s]);
    ch[15] = d2f_bits(__ldg(i0 + o));
    __nv_bfloat162 v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
        v[c] = __floats2bfloat162_rn(ch[2 * c], ch[2 * c + 1]);
    // planar: channels 0-7 and 8-15 in the frame's two planes
    const long long vol = (long long)g.nx * g.ny * g.nz;
    const long long vf = ((long long)(k - 1) * g.ny + (j - 1)) * g.nx + (i - 1);
    *reinterpret_cast<uint4 *>(x0 + tc::planar_off(l - 1, 0, 2, vol, vf)) = *reinterpret_cast<uint4 *>(&v[0]);
    *reinterpret_cast<uint4 *>(x0 + tc::planar_off(l - 1, 8, 2, vol, vf)) = *reinterpret_cast<uint4 *>(&v[4]);
}

__global__ void __launch_bounds__(256) k_ws_apply(Geo g, Split sp, SplitBufs b, const float *__restrict__ y,
                                                  const LoopState *__restrict__ st, const DevParams *__restrict__ dp)
{
    if (st->stop)
        return;
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const float inv = ws_inv_sigma(g, st, dp);
    const float sigma = inv > 0.f ? 1.f / inv : 0.f;
    const size_t vox = (((size_t)(l - 1) * g.nz + (k - 1)) * g.ny + (j - 1)) * g.nx + (i - 1);
    const float d = sigma * y[vox];
    const int col = (i + j + k + l) & 1;
    const long long s = split_index(g, sp, i, j, k, l);
    if (col == 0)
        pick(b.dR, st->dsrc)[s] = isfinite(d) ? d : 0.f;
    else
        b.dB[s] = isfinite(d) ? d : 0.f;
}

// (r0 - A32 d)^2 over the targets of one colour, as in k_sweep32 without the update
template <int COL>
__global__ void __launch_bounds__(256) k_ws_check(Geo g, Split sp, SweepCfg cfg, SplitBufs b,
                                                  const LoopState *__restrict__ st)
{
    double tot = 0.0;
    if (!st->stop) {
        const int ds = st->dsrc;
        const float *own = COL == 0 ? pick(b.dR, ds) : b.dB;
        const float *__restrict__ oth = COL == 0 ? b.dB : pick(b.dR, ds);
        const uint4 *__restrict__ cq = b.coefq[COL];
        const float *__restrict__ cs = b.coefs[COL];
        const float *__restrict__ rhs = b.r32[COL];
        const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
        const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
        float acc = 0.f;
        for (long long t = blockIdx.x; t < cfg.ntiles; t += gridDim.x) {
            const TileCoord tc = tile_coord(g, cfg, t, tx, ty);
            if (!tc.ok)
                continue;
            const int p = (COL + tc.j + tc.k + tc.l) & 1;
            if (2 * tc.xi + 2 - p > g.nx)
                continue;
            const long long s = (((long long)tc.l * g.kM + tc.k) * g.jM + tc.j) * Hy + tc.xi + sp.A;
            float w[8];
            const float sc = load_coef16(cq, cs, tile_coef_index(g, sp, tc), w);
            const float nb[8] = {oth[s - p + 1], oth[s - p], oth[s + Hy], oth[s - Hy],
                                 oth[s + Hz],    oth[s - Hz], oth[s + Hw], oth[s - Hw]};
            float diag;
            const float r = resid32(w, sc, nb, own[s], rhs[s], diag);
            acc = fmaf(r, r, acc);
        }
        tot = acc;
    }
    tot = block_sum(tot);
    if (threadIdx.x == 0)
        b.partial[COL][blockIdx.x] = tot;
}

__global__ void k_ws_decide(SplitBufs b, int nparts, const DevParams *__restrict__ dp, LoopState *st)
{
    if (st->stop)
        return;
    double a = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x)
        a += b.partial[0][t] + b.partial[1][t];
    a = block_sum(a);
    if (threadIdx.x == 0) {
        const double R = a * dp->h4;
        const int keep = isfinite(R) && R < st->R_first;
        st->keep = keep;
        st->warm = keep;
    }
}

static inline void ws_interior_grid(const Geo &g, dim3 &grid, dim3 &block)
{
    const int bx = g.nx >= 128 ? 128 : (g.nx >= 64 ? 64 : 32);
    const int by = 256 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((g.nx + bx - 1) / bx, (g.ny + by - 1) / by, g.nz * g.nt);
}

void launch_ws_features(const Geo &g, const Split &sp, SplitBufs b, const double *i0, CPtrs8 gin,
                        const LoopState *st, const DevParams *dp, void *x0, cudaStream_t s)
{
    dim3 gr, bl;
    ws_interior_grid(g, gr, bl);
    k_ws_features<<<gr, bl, 0, s>>>(g, sp, b, i0, gin, st, dp, reinterpret_cast<__nv_bfloat16 *>(x0));
}

void launch_ws_apply(const Geo &g, const Split &sp, SplitBufs b, const float *y, const LoopState *st,
                     const DevParams *dp, cudaStream_t s)
{
    dim3 gr, bl;
    ws_interior_grid(g, gr, bl);
    k_ws_apply<<<gr, bl, 0, s>>>(g, sp, b, y, st, dp);
}

void launch_ws_check_decide(const Geo &g, const Split &sp, const SweepCfg &cfg, SplitBufs b, LoopState *st,
                            const DevParams *dp, cudaStream_t s)
{
    k_ws_check<0><<<cfg.grid, 256, 0, s>>>(g, sp, cfg, b, st);
    k_ws_check<1><<<cfg.grid, 256, 0, s>>>(g, sp, cfg, b, st);
    k_ws_decide<<<1, 256, 0, s>>>(b, cfg.grid, dp, st);
}

} // namespace ss4d
