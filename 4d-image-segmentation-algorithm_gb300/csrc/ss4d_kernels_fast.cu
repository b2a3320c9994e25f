// ss4d_kernels_fast.cu — colour-split red-black SOR forms.
//
// Layout: every array is split by colour c = (i+j+k+l)&1 into two arrays of
// rows (l,k,j) x Hs columns (see Split in ss4d_common.cuh), so a half-sweep
// streams only the coefficients of its own colour and every warp load is a
// contiguous run.  The coefficients of a voxel (FP64: 32 records per
// component-major block, see coef_at; the FP32 sweeps: a 16-byte record of
// fixed-point fractions and an FP32 scale, see store_coef16 in ss4d_sweep.cuh)
// are c*a_f for the 8 faces (+x,-x,+y,-y,+z,-z,+w,-w = e,w,n,s,t,b,fw,bw),
// the diagonal 1 + c*sum a_f and omega/diagonal (c = tau/h^2), so one update is
//     r = diag*u - sum (c a_f) u_f - prev,   u <- u - (omega/diag) r
// which is the reference's u + omega (GS - u) (segmentation4D.c:237-256)
// rearranged, and r is the reference's residual of that voxel
// (segmentation4D.c:294-307) before the update.
//
// Residual without a third pass: in iteration z the red voxels' residual at
// the end of z is exactly the pre-update residual the red sweep of z+1
// computes (same red values, same black neighbours), and a black voxel's
// residual after its own update is (1-omega) times its pre-update residual
// (its neighbours are red and do not move during the black sweep).  The red
// sweep of z+1 writes into the other buffer of a red ping-pong pair, so when
// the test on the residual of z stops the loop, the red values of z are
// still there.  The loop controller is a one-block kernel that sums the
// per-block partials in a fixed order (deterministic) and, inside a CUDA
// graph, sets the while-node condition.
#include "ss4d_sweep.cuh"

namespace ss4d {

// ---------------------------------------------------------------------------
// helpers

// ---------------------------------------------------------------------------
// assembly: the reference's _gs_coefficients_ (segmentation4D.c:446-580) in
// two passes.  The reference evaluates every face twice (the east face of
// voxel i is the west face of voxel i+1, with identical bits); here k_faces
// evaluates each face once, for the face between v and v + e_d, and stores
// its norm |grad u|_eps and g/|grad u|_eps; k_voxel_coef then forms the voxel
// value vc = sqrt(mean^2 + eps2) and c*a_f = c*vc*g_f/|grad u|_f.
// 1/sqrt comes from an FP32 seed refined by one FP64 Newton step (relative
// error ~2e-14), which replaces an FP64 square root and division per face;
// FP64 runs at 1/68 of the FP32 rate on GB300, so these passes are bounded
// by the FP64 pipe, not by HBM.

// 1/sqrt(x), x > 0: FP32 seed + one Newton step
__device__ __forceinline__ double rsqrt_nr(double x)
{
    const double y0 = f2d_bits(rsqrtf(d2f_bits(x)));
    const double e = fma(-x * y0, y0, 1.0); // 1 - x y0^2
    return fma(0.5 * y0, e, y0);
}

// 1/x, x >= 1: FP32 seed + one Newton step
__device__ __forceinline__ double rcp_nr(double x)
{
    const double y0 = f2d_bits(__fdividef(1.0f, d2f_bits(x)));
    const double e = fma(-x, y0, 1.0);
    return fma(y0, e, y0);
}

// Coefficient record t of one voxel (layout: coef_at in ss4d_common.cuh):
// FP64 [c a_0..c a_7, diag, omega/diag] and, with want32, the FP32 sweeps'
// compressed record (store_coef16).
__device__ __forceinline__ void store_coef(double *cf, uint4 *cq, float *cs, long long t, const double ac[8],
                                           double diag, double winv, int want32)
{
#pragma unroll
    for (int f = 0; f < 8; ++f)
        __stcs(cf + coef_at(t, f, 10), ac[f]);
    __stcs(cf + coef_at(t, 8, 10), diag);
    __stcs(cf + coef_at(t, 9, 10), winv);
    if (want32) {
        float a[8];
#pragma unroll
        for (int f = 0; f < 8; ++f)
            a[f] = d2f_bits(ac[f]);
        store_coef16(cq, cs, t, a);
    }
}

// Threads cover voxels v with every index in [0, n_a]; face d of v (between
// v and v + e_d) is evaluated when v is interior on the other three axes, so
// index 0 on axis d yields the face the interior voxel 1 sees backwards.
__global__ void __launch_bounds__(256) k_faces(Geo g, const double *__restrict__ u, CPtrs8 gin, int has_g, double ih,
                                               double iq2, double eps2, SplitBufs b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z % (g.nz + 1), l = blockIdx.z / (g.nz + 1);
    if (i > g.nx || j > g.ny)
        return;
    const int idx[4] = {i, j, k, l};
    const long long o = nat_index(g, i, j, k, l);
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    const double uc = u[o];
    // central differences at v along each axis where v is interior
    double D[4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
        D[a] = idx[a] >= 1 ? u[o + st[a]] - u[o - st[a]] : 0.0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 4; ++a)
            if (a != d && idx[a] < 1)
                ok = false;
        if (!ok)
            continue;
        const long long nb = o + st[d];
        const double cn = (u[nb] - uc) * ih;
        double tt = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (a == d)
                continue;
            const double t = (u[nb + st[a]] - u[nb - st[a]]) + D[a];
            tt = fma(t, t, tt);
        }
        const double s2 = fma(tt, iq2, fma(cn, cn, eps2));
        const double y = rsqrt_nr(s2);
        double gv = 1.0;
        if (has_g)
            gv = idx[d] >= 1 ? __ldg(gin.p[2 * d] + o) : __ldg(gin.p[2 * d + 1] + nb);
        __stcs(b.fn[d] + o, s2 * y);
        __stcs(b.fq[d] + o, gv * y);
    }
}

__global__ void __launch_bounds__(256) k_voxel_coef(Geo g, Split sp, double eps2, double c, double omega, SplitBufs b,
                                                    int want32)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const long long o = nat_index(g, i, j, k, l);
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    double q[8], sum = 0.0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        sum += __ldg(b.fn[d] + o) + __ldg(b.fn[d] + o - st[d]);
        q[2 * d] = __ldg(b.fq[d] + o);
        q[2 * d + 1] = __ldg(b.fq[d] + o - st[d]);
    }
    const double x = fma(sum * sum, 1.0 / 64.0, eps2); // mean^2 + eps2
    const double cv = c * (x * rsqrt_nr(x));           // c * vc
    const int col = (i + j + k + l) & 1;
    double *cf = pick(b.coef, col);
    double ac[8], diag = 1.0;
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        ac[f] = cv * q[f];
        diag += ac[f];
    }
    store_coef(cf, pick(b.coefq, col), pick(b.coefs, col), coef_index(g, sp, i, j, k, l), ac, diag,
               omega * rcp_nr(diag), want32);
}

// given natural coefficient arrays e..bw (the reference's layout) -> split
// FP64 c*a_f, diagonal, omega/diagonal (+ the FP32 sweeps' records)
__global__ void __launch_bounds__(256) k_pack_coef(Geo g, Split sp, CPtrs8 a, double c, double omega, SplitBufs b,
                                                   int want32)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const long long o = nat_index(g, i, j, k, l);
    const int col = (i + j + k + l) & 1;
    double *cf = pick(b.coef, col);
    double ac[8], diag = 1.0;
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        ac[f] = c * a.p[f][o];
        diag += ac[f];
    }
    store_coef(cf, pick(b.coefq, col), pick(b.coefs, col), coef_index(g, sp, i, j, k, l), ac, diag, omega / diag,
               want32);
}

// natural -> split copies of u (both red buffers and black, ghosts
// included) and of prev (both colours).  A thread takes two neighbours
// (i = 2m, 2m + 1) of one row: they have opposite colours and land in
// columns m + A - 1 and m + A of their colour arrays.
__global__ void __launch_bounds__(256) k_pack(Geo g, Split sp, const double *__restrict__ u,
                                              const double *__restrict__ prev, SplitBufs b, FastDiv fpairs,
                                              unsigned q0, unsigned q1)
{
    // q: rows x pairs, below 2^31; [q0, q1) covers whole frames
    const unsigned npairs = fpairs.d;
    for (unsigned q = q0 + blockIdx.x * blockDim.x + threadIdx.x; q < q1; q += gridDim.x * blockDim.x) {
        const unsigned row = fdiv(q, fpairs);
        const int m = (int)(q - row * npairs);
        // row = (l kM + k) jM + j
        const unsigned rk = fdiv(row, g.fjM);
        const int j = (int)(row - rk * g.fjM.d);
        const unsigned l = fdiv(rk, g.fkM);
        const int k = (int)(rk - l * g.fkM.d);
        const int c0 = (j + k + (int)l) & 1; // colour of i = 2m
        const long long o = (long long)row * g.iM + 2 * m;
        const long long s = (long long)row * sp.Hs + m + sp.A - 1;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (2 * m + h >= g.iM)
                break;
            const int col = c0 ^ h;
            const double v = u[o + h];
            if (col == 0) {
                b.R[0][s + h] = v;
                b.R[1][s + h] = v;
            } else {
                b.Bk[s + h] = v;
            }
            pick(b.P, col)[s + h] = prev[o + h];
        }
    }
}

// split -> natural interior of u.  With terms > 0 (mixed form) also the next
// step's start correction, extrapolated in time from this step's change
// d = u - prev (FP32) and the changes of earlier steps h1, h2 (per colour):
// terms 1: d, 2: 2 d - h1, 3: 3 d - 3 h1 + h2, written into the interior of
// dR[0] / dB, where the next step's first refinement pass (or, when the
// assembly forms that pass, its first-difference kernel) adds it to u^{n+1}.  The history then shifts: h2 <- h1 (keep >= 2), h1 <- d (keep >= 1).
struct History {
    float *h1[2]; // per colour
    float *h2[2];
};

// what: UNPACK_ALL (u and the history), UNPACK_PAUSED (only u, formed from a
// loop paused before its last refinement pass: the split u plus the round's
// correction, with that pass's own FP64 additions, so it equals what the pass
// then writes), UNPACK_HISTORY (only the history and the next start)
__global__ void k_unpack(Geo g, Split sp, SplitBufs b, const LoopState *__restrict__ st, double *u, int terms,
                         int keep, History hs, int l_off, int what)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + l_off + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const int col = (i + j + k + l) & 1;
    const long long s = (((long long)l * g.kM + k) * g.jM + j) * sp.Hs + ((i + 1) >> 1) + sp.A - 1;
    if (what == UNPACK_PAUSED) {
        // the refinement's red update own + down (k_refine<0>) and black one
        // Bk += dB (k_apply_black)
        const double v = col == 0 ? b.R[0][s] + f2d_bits(pick(b.dR, st->dsrc)[s]) : b.Bk[s] + f2d_bits(b.dB[s]);
        u[nat_index(g, i, j, k, l)] = v;
        return;
    }
    if (what == UNPACK_HISTORY && terms <= 0)
        return;
    // every load before the first store (which could alias them for the
    // compiler): one round trip to memory, not two
    float *h1 = pick(hs.h1, col), *h2 = pick(hs.h2, col);
    double pv = 0.0;
    float p1 = 0.f, p2 = 0.f;
    if (terms > 0) {
        pv = pick(b.P, col)[s];
        if (terms >= 2)
            p1 = h1[s];
        if (terms >= 3)
            p2 = h2[s];
    }
    const int fr = st->final_red;
    const double v = col == 0 ? pick(b.R, fr)[s] : b.Bk[s];
    if (what != UNPACK_HISTORY)
        u[nat_index(g, i, j, k, l)] = v;
    if (terms > 0) {
        const float d = d2f_bits(v - pv);
        float guess = d;
        if (terms == 2)
            guess = fmaf(2.f, d, -p1);
        else if (terms == 3)
            guess = fmaf(3.f, d - p1, p2);
        if (keep >= 2 && terms >= 2) // h1 holds an earlier change from the second step on
            h2[s] = p1;
        if (keep >= 1)
            h1[s] = d;
        if (col == 0)
            b.dR[0][s] = guess;
        else
            b.dB[s] = guess;
    }
}

__global__ void k_loop_init(LoopState *st, int mode, int pre, int spec)
{
    st->pre = pre;
    st->spec = spec;
    st->paused = 0;
    st->z = 0;
    st->stop = 0;
    st->status = 0;
    st->mode = mode;
    st->refinements = 0;
    st->round_z = 0;
    st->dsrc = 0;
    st->final_red = 0;
    st->bodies = 0;
    st->keep = 0;
    st->warm = 0;
    st->near = 0;
    st->proj = 0;
    st->R = 0.0;
    st->R_first = 0.0;
    st->Rd = 0.0;
    st->target = 0.0;
}

__global__ void k_advance(LoopState *st)
{
    st->z = 1;
}

// ---------------------------------------------------------------------------
// FP64 half-sweep with fused residual

template <int COL>
__global__ void __launch_bounds__(256) k_sweep64(Geo g, Split sp, SweepCfg cfg, SplitBufs b,
                                                 const DevParams *__restrict__ dp, const LoopState *__restrict__ st)
{
    const int z = st->z;
    const double *src;
    double *dst;
    const double *__restrict__ oth;
    if (COL == 0) {
        src = pick(b.R, z & 1);
        dst = pick(b.R, (z + 1) & 1);
        oth = b.Bk;
    } else {
        src = b.Bk;
        dst = b.Bk;
        oth = pick(b.R, z & 1);
    }
    const double *__restrict__ cf = b.coef[COL];
    const double *__restrict__ pv = b.P[COL];
    const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
    double acc = 0.0;
    for (long long t = blockIdx.x; t < cfg.ntiles; t += gridDim.x) {
        const TileCoord tc = tile_coord(g, cfg, t, tx, ty);
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
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        b.partial[COL][blockIdx.x] = acc;
}

// sums the partials of both colours in a fixed order and decides
__global__ void k_ctrl64(SplitBufs b, int nparts, const DevParams *__restrict__ dp, LoopState *st,
                         cudaGraphConditionalHandle h, int use_cond)
{
    double a = 0.0, c = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x) {
        a += b.partial[0][t];
        c += b.partial[1][t];
    }
    a = block_sum(a);
    c = block_sum(c);
    if (threadIdx.x == 0) {
        const bool stop = ctrl64_update(st, a, c, dp);
        if (use_cond)
            cudaGraphSetConditional(h, stop ? 0u : 1u);
    }
}

// ---------------------------------------------------------------------------
// mixed precision: FP64 refinement passes + FP32 sweeps on the correction
// equation A d = r.  Modes (LoopState::mode): 0 refine, 1 start a round
// (zero d, first red sweep), 2 inner iteration (black sweep + next red sweep).

// A refinement pass is three launches: k_apply_black (black u += d_B), then
// k_refine<0> (red u += d_R and the red residual against the updated black
// values), then k_refine<1> (the black residual against the updated red
// values); r32 receives the residual for the next round.  Applying the black
// correction first spares the red pass adding it to each of 8 neighbours.
__global__ void __launch_bounds__(256) k_apply_black(Geo g, Split sp, SweepCfg cfg, SplitBufs b,
                                                     const LoopState *__restrict__ st)
{
    if (st->mode != 0 || st->stop || st->pre) // pre: the first-difference kernel added it
        return;
    const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
    for (long long t = blockIdx.x; t < cfg.ntiles; t += gridDim.x) {
        const TileCoord tc = tile_coord(g, cfg, t, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (1 + tc.j + tc.k + tc.l) & 1;
        if (2 * tc.xi + 2 - p > g.nx)
            continue;
        const long long s = (((long long)tc.l * g.kM + tc.k) * g.jM + tc.j) * sp.Hs + tc.xi + sp.A;
        b.Bk[s] += f2d_bits(b.dB[s]);
    }
}

template <int COL>
__global__ void __launch_bounds__(256) k_refine(Geo g, Split sp, SweepCfg cfg, SplitBufs b,
                                                const DevParams *__restrict__ dp, const LoopState *__restrict__ st)
{
    if (st->mode != 0 || st->stop)
        return;
    const int ds = st->dsrc;
    double *own = COL == 0 ? b.R[0] : b.Bk;
    const float *__restrict__ down = pick(b.dR, ds); // only used for COL == 0
    const double *__restrict__ oth = COL == 0 ? b.Bk : b.R[0];
    const double *__restrict__ cf = b.coef[COL];
    const double *__restrict__ pv = b.P[COL];
    float *__restrict__ rr = b.r32[COL];
    const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
    const int tx = threadIdx.x & (cfg.XT - 1), ty = threadIdx.x / cfg.XT;
    // pre: the first pass of a step whose residual the coefficient kernel
    // formed (with the same operations on the same values) and whose
    // correction the first-difference kernel added; only read here
    const bool pre = st->pre;
    const double *__restrict__ rp = b.rpre[COL];
    double acc = 0.0;
    for (long long t = blockIdx.x; t < cfg.ntiles; t += gridDim.x) {
        const TileCoord tc = tile_coord(g, cfg, t, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (COL + tc.j + tc.k + tc.l) & 1;
        const int i = 2 * tc.xi + 2 - p;
        if (i > g.nx)
            continue;
        const long long s = (((long long)tc.l * g.kM + tc.k) * g.jM + tc.j) * Hy + tc.xi + sp.A;
        double r;
        if (pre) {
            r = ld_stream(rp + s);
        } else {
            const RefineOut o = refine_target<COL>(g, sp, tc, p, s, Hy, Hz, Hw, own, down, oth, cf, pv);
            r = o.r;
            if (COL == 0)
                own[s] = o.u;
        }
        acc = fma(r, r, acc);
        rr[s] = d2f_bits(-r);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        b.partial[COL][blockIdx.x] = acc;
}

// clears the corrections at the start of a round (ghosts stay zero), unless
// the round is to start from the correction already in place (warm start)
__global__ void k_zero_delta(Split sp, SplitBufs b, const LoopState *__restrict__ st)
{
    if (st->mode != 1 || st->stop || st->keep)
        return;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < sp.cs; t += (long long)gridDim.x * blockDim.x) {
        b.dR[0][t] = 0.f;
        b.dR[1][t] = 0.f;
        b.dB[t] = 0.f;
    }
}

// FP32 half-sweep of colour COL: each thread updates two adjacent targets of
// a row (pc: make_pair_cfg), so the pair shares its index arithmetic and reads its
// own values, right-hand sides and the y/z/w neighbours as 8-byte pairs; each
// target's arithmetic is sweep32_target's (resid32 and the relaxed update).
// The launch has the solver's persistent grid, whose every block writes its
// partial residual sum.
template <int COL>
__global__ void __launch_bounds__(256) k_sweep32(Geo g, Split sp, SweepCfg pc, SplitBufs b,
                                                 const DevParams *__restrict__ dp, const LoopState *__restrict__ st)
{
    const int mode = st->mode;
    if ((COL == 0 ? (mode == 0) : (mode != 2)) || st->stop)
        return;
    const int ds = st->dsrc;
    const float *src;
    float *dst;
    const float *__restrict__ oth;
    if (COL == 0) {
        src = pick(b.dR, ds);
        dst = pick(b.dR, ds ^ 1);
        oth = b.dB;
    } else {
        src = b.dB;
        dst = b.dB;
        oth = pick(b.dR, ds);
    }
    const uint4 *__restrict__ cq = b.coefq[COL];
    const float *__restrict__ cs = b.coefs[COL];
    const float *__restrict__ rhs = b.r32[COL];
    const float omega = (float)dp->omega;
    // 32-bit offsets: a colour array holds fewer than 2^31 elements
    const unsigned Hy = (unsigned)sp.Hs, Hz = Hy * (unsigned)g.jM, Hw = Hz * (unsigned)g.kM;
    const int tx = threadIdx.x & (pc.XT - 1), ty = threadIdx.x / pc.XT;
    float acc = 0.f;
    for (long long t = blockIdx.x; t < pc.ntiles; t += gridDim.x) {
        const TileCoord tc = tile_coord(g, pc, t, tx, ty);
        if (!tc.ok)
            continue;
        const int p = (COL + tc.j + tc.k + tc.l) & 1;
        const int xi = 2 * tc.xi; // the pair's first target; the second is xi + 1
        const int i = 2 * xi + 2 - p;
        if (i > g.nx)
            continue;
        const unsigned s = (((unsigned)tc.l * g.kM + tc.k) * g.jM + tc.j) * Hy + xi + sp.A;
        const unsigned tq = ((((unsigned)tc.l - 1) * g.nz + (tc.k - 1)) * g.ny + (tc.j - 1)) * sp.nxh + xi;
        acc = sweep32_pair(p, s, tq, i + 2 <= g.nx, Hy, Hz, Hw, src, dst, oth, cq, cs, rhs, omega, acc);
    }
    const double tot = block_sum((double)acc);
    if (threadIdx.x == 0)
        b.partial[COL][blockIdx.x] = tot;
}

__global__ void k_ctrl_mixed(SplitBufs b, int nparts, const DevParams *__restrict__ dp, LoopState *st,
                             cudaGraphConditionalHandle h, int use_cond)
{
    if (st->stop) { // stopped before the loop (the warm-start prologue's test)
        if (threadIdx.x == 0 && use_cond)
            cudaGraphSetConditional(h, 0u);
        return;
    }
    const int mode = st->mode;
    double a = 0.0, c = 0.0;
    if (mode != 1) {
        for (int t = threadIdx.x; t < nparts; t += blockDim.x) {
            a += b.partial[0][t];
            if (mode == 0 || mode == 2)
                c += b.partial[1][t];
        }
    }
    a = block_sum(a);
    c = block_sum(c);
    if (threadIdx.x != 0)
        return;
    const bool stop = ctrl_mixed_update(st, a, c, dp);
    if (use_cond) // a paused loop leaves the graph too
        cudaGraphSetConditional(h, stop || st->paused ? 0u : 1u);
}

// ---------------------------------------------------------------------------
// host launchers

static int pow2_at_least(int v)
{
    int p = 1;
    while (p < v)
        p <<= 1;
    return p;
}

int max_blocks_sweep64()
{
    int a = 0, b = 0, c = 0, d = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_sweep64<0>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_sweep64<1>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_refine<0>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_refine<1>, 256, 0);
    int m = a < b ? a : b;
    m = m < c ? m : c;
    m = m < d ? m : d;
    return m > 0 ? m : 1;
}

int max_blocks_sweep32()
{
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_sweep32<0>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_sweep32<1>, 256, 0);
    int m = a < b ? a : b;
    return m > 0 ? m : 1;
}

SweepCfg make_sweep_cfg(const Geo &g, const Split &s, int sm_count, int kb)
{
    return make_sweep_cfg_xt(g, s, sm_count, kb, 0);
}

// xt: threads along x per tile (a power of two in [8, 256]); 0 picks the
// smallest power of two covering a row's targets, at most 128
SweepCfg make_sweep_cfg_xt(const Geo &g, const Split &s, int sm_count, int kb, int xt)
{
    SweepCfg c;
    c.threads = 256;
    c.XT = xt > 0 ? pow2_at_least(xt) : pow2_at_least(s.nxh);
    if (xt <= 0 && c.XT > 128)
        c.XT = 128;
    if (c.XT > 256)
        c.XT = 256;
    if (c.XT < 8)
        c.XT = 8;
    c.TJ = c.threads / c.XT;
    c.KB = kb < 1 ? 1 : (kb > g.nz ? g.nz : kb);
    c.nXC = (s.nxh + c.XT - 1) / c.XT;
    c.nJG = (g.ny + c.TJ - 1) / c.TJ;
    c.nKB = (g.nz + c.KB - 1) / c.KB;
    c.ntiles = (long long)c.nXC * c.nJG * c.KB * g.nt * c.nKB;
    c.dXC = make_fastdiv((unsigned)c.nXC);
    c.dJG = make_fastdiv((unsigned)c.nJG);
    c.dKB = make_fastdiv((unsigned)c.KB);
    c.dNT = make_fastdiv((unsigned)g.nt);
    int per_sm = max_blocks_sweep64();
    int p32 = max_blocks_sweep32();
    per_sm = per_sm < p32 ? per_sm : p32;
    long long grid = (long long)sm_count * per_sm;
    if (grid > c.ntiles)
        grid = c.ntiles;
    c.grid = (int)(grid > 0 ? grid : 1);
    return c;
}

static inline void interior_grid(const Geo &g, dim3 &grid, dim3 &block)
{
    const int bx = g.nx >= 128 ? 128 : (g.nx >= 64 ? 64 : 32);
    const int by = 256 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((g.nx + bx - 1) / bx, (g.ny + by - 1) / by, g.nz * g.nt);
}

void launch_assemble(const Geo &g, const Split &s, const double *u, CPtrs8 gin, int has_g, const ss4d_params &p,
                     SplitBufs b, int want32, cudaStream_t st)
{
    const int bx = g.nx + 1 >= 128 ? 128 : (g.nx + 1 >= 64 ? 64 : 32);
    const int by = 256 / bx;
    dim3 fb(bx, by, 1), fg((g.nx + 1 + bx - 1) / bx, (g.ny + 1 + by - 1) / by, (g.nz + 1) * (g.nt + 1));
    const double ih = 1.0 / p.h, iq = 1.0 / (4.0 * p.h);
    k_faces<<<fg, fb, 0, st>>>(g, u, gin, has_g, ih, iq * iq, p.eps2, b);
    dim3 gr, bl;
    interior_grid(g, gr, bl);
    const double c = p.tau / (p.h * p.h);
    k_voxel_coef<<<gr, bl, 0, st>>>(g, s, p.eps2, c, p.omega_c, b, want32);
}

void launch_pack(const Geo &g, const Split &s, const double *u, const double *prev, SplitBufs b, cudaStream_t st)
{
    launch_pack_range(g, s, u, prev, b, 0, g.lM, st);
}

void launch_pack_range(const Geo &g, const Split &s, const double *u, const double *prev, SplitBufs b, int l0, int l1,
                       cudaStream_t st)
{
    const unsigned npairs = (unsigned)((g.iM + 1) / 2), per_frame = (unsigned)(g.jM * g.kM) * npairs;
    k_pack<<<4096, 256, 0, st>>>(g, s, u, prev, b, make_fastdiv(npairs), per_frame * (unsigned)l0,
                                 per_frame * (unsigned)l1);
}

void launch_pack_coef(const Geo &g, const Split &s, CPtrs8 a, const ss4d_params &p, SplitBufs b, int want32,
                      cudaStream_t st)
{
    dim3 gr, bl;
    interior_grid(g, gr, bl);
    const double c = p.tau / (p.h * p.h);
    k_pack_coef<<<gr, bl, 0, st>>>(g, s, a, c, p.omega_c, b, want32);
}

void launch_unpack(const Geo &g, const Split &s, SplitBufs b, const LoopState *state, double *u, cudaStream_t st,
                   int terms, int keep, float *const *hist)
{
    launch_unpack_range(g, s, b, state, u, st, terms, keep, hist, 1, g.lM - 1);
}

void launch_unpack_range(const Geo &g, const Split &s, SplitBufs b, const LoopState *state, double *u, cudaStream_t st,
                         int terms, int keep, float *const *hist, int l0, int l1, int what)
{
    dim3 gr, bl;
    interior_grid(g, gr, bl);
    gr.z = g.nz * (l1 - l0);
    History hs;
    for (int c = 0; c < 2; ++c) {
        hs.h1[c] = hist ? hist[c] : nullptr;
        hs.h2[c] = hist ? hist[2 + c] : nullptr;
    }
    k_unpack<<<gr, bl, 0, st>>>(g, s, b, state, u, terms, keep, hs, l0 - 1, what);
}

void launch_loop_init(LoopState *state, int mode, cudaStream_t st, int pre, int spec)
{
    k_loop_init<<<1, 1, 0, st>>>(state, mode, pre, spec);
}

void launch_advance(LoopState *state, cudaStream_t st)
{
    k_advance<<<1, 1, 0, st>>>(state);
}

void launch_sweep64(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                    LoopState *state, cudaStream_t st)
{
    if (colour == 0)
        k_sweep64<0><<<cfg.grid, cfg.threads, 0, st>>>(g, s, cfg, b, dp, state);
    else
        k_sweep64<1><<<cfg.grid, cfg.threads, 0, st>>>(g, s, cfg, b, dp, state);
}

void launch_ctrl64(SplitBufs b, int nparts, const DevParams *dp, LoopState *state, unsigned long long cond_handle,
                   int use_cond, cudaStream_t st)
{
    k_ctrl64<<<1, 256, 0, st>>>(b, nparts, dp, state, (cudaGraphConditionalHandle)cond_handle, use_cond);
}

void launch_refine(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                   LoopState *state, cudaStream_t st)
{
    if (colour == 0) {
        k_apply_black<<<cfg.grid, cfg.threads, 0, st>>>(g, s, cfg, b, state);
        k_refine<0><<<cfg.grid, cfg.threads, 0, st>>>(g, s, cfg, b, dp, state);
    } else {
        k_refine<1><<<cfg.grid, cfg.threads, 0, st>>>(g, s, cfg, b, dp, state);
    }
}

void launch_zero_delta(const Split &s, SplitBufs b, LoopState *state, cudaStream_t st)
{
    k_zero_delta<<<1024, 256, 0, st>>>(s, b, state);
}

// Tiles of the paired FP32 sweep: the cfg.XT targets of a row chunk are
// taken by cfg.XT / 2 threads with two adjacent targets each, so a tile has
// twice the rows; the tile order and the grid stay the solver's.
SweepCfg make_pair_cfg(const Geo &g, const Split &s, const SweepCfg &cfg)
{
    SweepCfg c = cfg;
    c.XT = cfg.XT >= 2 ? cfg.XT / 2 : 1;
    c.TJ = c.threads / c.XT;
    c.nXC = (s.nxh + 2 * c.XT - 1) / (2 * c.XT);
    c.nJG = (g.ny + c.TJ - 1) / c.TJ;
    c.ntiles = (long long)c.nXC * c.nJG * c.KB * g.nt * c.nKB;
    c.dXC = make_fastdiv((unsigned)c.nXC);
    c.dJG = make_fastdiv((unsigned)c.nJG);
    return c;
}

void launch_sweep32(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                    LoopState *state, int start_mode, cudaStream_t st)
{
    (void)start_mode;
    const SweepCfg pc = make_pair_cfg(g, s, cfg);
    if (colour == 0)
        k_sweep32<0><<<cfg.grid, cfg.threads, 0, st>>>(g, s, pc, b, dp, state);
    else
        k_sweep32<1><<<cfg.grid, cfg.threads, 0, st>>>(g, s, pc, b, dp, state);
}

void launch_ctrl_mixed(SplitBufs b, int nparts, const DevParams *dp, LoopState *state, unsigned long long cond_handle,
                       int use_cond, cudaStream_t st)
{
    k_ctrl_mixed<<<1, 256, 0, st>>>(b, nparts, dp, state, (cudaGraphConditionalHandle)cond_handle, use_cond);
}

} // namespace ss4d
