// ss4d_sweep.cuh — the tile schedule and the FP64 red-black update shared by
// the single-volume sweeps (ss4d_kernels_fast.cu) and the batched sweeps
// (ss4d_batch.cu).  Layouts: ss4d_common.cuh (Split, coef_at).
#pragma once

#include "ss4d_kernels.cuh"

namespace ss4d {

// streamed once per sweep: evict first
__device__ __forceinline__ double ld_stream(const double *p)
{
    return __ldcs(p);
}
__device__ __forceinline__ float ld_stream(const float *p)
{
    return __ldcs(p);
}
__device__ __forceinline__ double2 ld_stream2(const double *p)
{
    return __ldcs(reinterpret_cast<const double2 *>(p));
}
__device__ __forceinline__ float4 ld_stream4(const float *p)
{
    return __ldcs(reinterpret_cast<const float4 *>(p));
}

// FP32 <-> FP64 conversions by integer bit operations.  On this GPU a
// conversion instruction to or from FP64 issues at the FP64 rate (1/68 of
// FP32); these run on the integer pipe instead.
// Exact float -> double for zero, normal numbers, Inf and NaN (FP32
// subnormals, below 1.2e-38, become signed zero).
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    const unsigned de = e == 0xFFu ? 0x7FFu : e + 896u;
    const unsigned hi = e == 0u ? sign : (sign | (de << 20) | (m >> 3));
    const unsigned lo = e == 0u ? 0u : (m & 7u) << 29;
    return __hiloint2double((int)hi, (int)lo);
}
// double -> float by truncating the mantissa (error below 2^-23 relative);
// magnitudes outside the FP32 normal range become zero or Inf, NaN stays NaN.
__device__ __forceinline__ float d2f_bits(double d)
{
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const int fe = e - 896;
    unsigned r;
    if (e == 0x7FF)
        r = sign | 0x7F800000u | (m ? 0x400000u : 0u);
    else if (fe <= 0)
        r = sign;
    else if (fe >= 255)
        r = sign | 0x7F800000u;
    else
        r = sign | ((unsigned)fe << 23) | m;
    return __uint_as_float(r);
}

// read-only for the whole kernel (the other colour)
template <typename T>
__device__ __forceinline__ T ld_ro(const T *p)
{
    return __ldg(p);
}

// Select one of a pair held in a by-value kernel parameter without a runtime
// array index (which would copy the parameter struct to local memory).
template <typename T>
__device__ __forceinline__ T *pick(T *const (&a)[2], int i)
{
    return i ? a[1] : a[0];
}

struct TileCoord {
    int j, k, l, xi;
    bool ok;
};

// Tile order: x chunk fastest, then j group, then k inside a k block, then
// frame l, then k block.  Consecutive tiles (which a persistent grid works on
// at the same time) thus cover a few k planes (one with the default block
// depth of 1) of all frames, so the neighbouring-plane reads of the other
// colour hit in L2.
__device__ __forceinline__ TileCoord tile_coord(const Geo &g, const SweepCfg &cfg, long long t, int tx, int ty)
{
    TileCoord c;
    unsigned r = (unsigned)t; // t < ntiles < 2^31
    unsigned q = fdiv(r, cfg.dXC);
    const int xc = (int)(r - q * cfg.dXC.d);
    r = q;
    q = fdiv(r, cfg.dJG);
    const int jg = (int)(r - q * cfg.dJG.d);
    r = q;
    q = fdiv(r, cfg.dKB);
    const int kin = (int)(r - q * cfg.dKB.d);
    r = q;
    q = fdiv(r, cfg.dNT);
    const int lt = (int)(r - q * cfg.dNT.d);
    const int kb = (int)q;
    c.k = 1 + kb * cfg.KB + kin;
    c.l = 1 + lt;
    c.j = 1 + jg * cfg.TJ + ty;
    c.xi = xc * cfg.XT + tx;
    c.ok = c.k <= g.nz && c.j <= g.ny;
    return c;
}

// compact per-colour interior index of voxel (i, j, k, l)
__device__ __forceinline__ long long coef_index(const Geo &g, const Split &sp, int i, int j, int k, int l)
{
    return ((((long long)(l - 1) * g.nz + (k - 1)) * g.ny + (j - 1)) * sp.nxh) + ((i - 1) >> 1);
}

// compact per-colour interior index of a sweep target
__device__ __forceinline__ long long tile_coef_index(const Geo &g, const Split &sp, const TileCoord &tc)
{
    return ((((long long)(tc.l - 1) * g.nz + (tc.k - 1)) * g.ny + (tc.j - 1)) * sp.nxh) + tc.xi;
}

// One FP64 update of the target at split index s (row phase p):
//   r = diag*u - (prev + sum_f c a_f u_f),   dst = u - (omega/diag) r.
// Returns the pre-update residual r.
__device__ __forceinline__ double sweep64_target(const Geo &g, const Split &sp, const TileCoord &tc, int p,
                                                 long long s, const double *src, double *dst,
                                                 const double *__restrict__ oth, const double *__restrict__ cf,
                                                 const double *__restrict__ pv)
{
    const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
    const double u0 = src[s];
    const double *cv = cf + coef_at(tile_coef_index(g, sp, tc), 0, 10); // component f at cv[32 f]
    double S = fma(ld_stream(cv), ld_ro(oth + s - p + 1), ld_stream(pv + s));
    S = fma(ld_stream(cv + 32), ld_ro(oth + s - p), S);
    S = fma(ld_stream(cv + 64), ld_ro(oth + s + Hy), S);
    S = fma(ld_stream(cv + 96), ld_ro(oth + s - Hy), S);
    S = fma(ld_stream(cv + 128), ld_ro(oth + s + Hz), S);
    S = fma(ld_stream(cv + 160), ld_ro(oth + s - Hz), S);
    S = fma(ld_stream(cv + 192), ld_ro(oth + s + Hw), S);
    S = fma(ld_stream(cv + 224), ld_ro(oth + s - Hw), S);
    const double diag = ld_stream(cv + 256);
    const double winv = ld_stream(cv + 288);
    const double r = fma(diag, u0, -S); // S includes prev
    dst[s] = fma(-winv, r, u0);
    return r;
}

// ---------------------------------------------------------------------------
// mixed form: FP64 refinement and FP32 correction sweeps (single-volume
// kernels in ss4d_kernels_fast.cu, batched ones in ss4d_batch.cu)

// Refinement at a target of colour COL (Hy, Hz, Hw: the split strides of
// j, k, l): the red pass first adds the red correction (down) to u; then
// r = diag*u - (prev + sum_f c a_f u_f) against the other colour, whose
// correction is already in place.  Returns r and the target's u; the caller
// stores u (red pass) and -r into r32, the right-hand side of the next
// correction equation (r = A u - b here; the correction d with A d = b - A u
// moves u to the solution).
struct RefineOut {
    double r, u;
};
template <int COL>
__device__ __forceinline__ RefineOut refine_target(const Geo &g, const Split &sp, const TileCoord &tc, int p,
                                                   long long s, long long Hy, long long Hz, long long Hw,
                                                   const double *own, const float *__restrict__ down,
                                                   const double *__restrict__ oth, const double *__restrict__ cf,
                                                   const double *__restrict__ pv)
{
    const long long nb[8] = {s - p + 1, s - p, s + Hy, s - Hy, s + Hz, s - Hz, s + Hw, s - Hw};
    const double u0 = COL == 0 ? own[s] + f2d_bits(down[s]) : own[s];
    const double *cv = cf + coef_at(tile_coef_index(g, sp, tc), 0, 10);
    double S = ld_stream(pv + s); // prev + sum_f c a_f u_f
#pragma unroll
    for (int f = 0; f < 8; ++f)
        S = fma(ld_stream(cv + 32 * f), oth[nb[f]], S);
    const double diag = ld_stream(cv + 256);
    return RefineOut{fma(diag, u0, -S), u0};
}

// One FP32 SOR update of the correction at a target (diag = 1 + sum c a_f,
// formed from the record): returns the pre-update residual of the correction
// equation and the updated value, which the caller stores.
struct Sweep32Out {
    float r, u;
};
__device__ __forceinline__ Sweep32Out sweep32_target(const Geo &g, const Split &sp, const TileCoord &tc, int p,
                                                     long long s, long long Hy, long long Hz, long long Hw,
                                                     const float *src, const float *__restrict__ oth,
                                                     const float *__restrict__ cf, const float *__restrict__ rhs,
                                                     float omega)
{
    const float u0 = src[s];
    const float *cv = cf + 8 * tile_coef_index(g, sp, tc);
    const float4 c03 = ld_stream4(cv), c47 = ld_stream4(cv + 4);
    const float a0 = c03.x, a1 = c03.y, a2 = c03.z, a3 = c03.w, a4 = c47.x, a5 = c47.y, a6 = c47.z, a7 = c47.w;
    float S = a0 * ld_ro(oth + s - p + 1);
    S = fmaf(a1, ld_ro(oth + s - p), S);
    S = fmaf(a2, ld_ro(oth + s + Hy), S);
    S = fmaf(a3, ld_ro(oth + s - Hy), S);
    S = fmaf(a4, ld_ro(oth + s + Hz), S);
    S = fmaf(a5, ld_ro(oth + s - Hz), S);
    S = fmaf(a6, ld_ro(oth + s + Hw), S);
    S = fmaf(a7, ld_ro(oth + s - Hw), S);
    const float diag = 1.f + (((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7)));
    const float r = fmaf(diag, u0, -(S + ld_stream(rhs + s)));
    return Sweep32Out{r, fmaf(-omega / diag, r, u0)};
}

// ---------------------------------------------------------------------------
// stopping tests, one volume: a and c are the summed red and black partials
// of the body that just ran.  Both return true when the loop stops.

// plain FP64 form: R after iteration z.  A body is the black half-sweep of
// iteration z and the red one of z + 1, both summing pre-update residuals:
// the red ones are those of iteration z's values; an SOR update scales a
// black target's residual by (1 - omega), so the black sums are scaled by
// (1 - omega)^2.
__device__ inline bool ctrl64_update(LoopState *st, double a, double c, const DevParams *dp)
{
    const double om1 = 1.0 - dp->omega;
    const double R = (a + om1 * om1 * c) * dp->h4;
    const int z = st->z;
    st->bodies += 1;
    if (z == 1)
        st->R_first = R;
    st->R = R;
    if (fabs(R - dp->tol) <= dp->near_band)
        st->near = 1;
    const bool fin = isfinite(R);
    const bool stop = !fin || !(R > dp->tol) || z >= dp->maxit;
    if (!fin)
        st->status = SS4D_ERR_NONFINITE;
    if (stop) {
        st->stop = 1;
        st->final_red = z & 1; // red buffer holding the values of iteration z
    } else {
        st->z = z + 1;
    }
    return stop;
}

// mixed form: mode 0 (refinement: the FP64 residual test), 1 (a round has
// started), 2 (an inner iteration: the correction equation's residual
// against the round's target)
__device__ inline bool ctrl_mixed_update(LoopState *st, double a, double c, const DevParams *dp)
{
    const int mode = st->mode;
    st->bodies += 1;
    bool stop = false;
    if (mode == 0) {
        st->pre = 0; // later passes form their own residual
        const double R = (a + c) * dp->h4;
        if (st->refinements == 0)
            st->R_first = R;
        st->refinements += 1;
        st->R = R;
        if (fabs(R - dp->tol) <= dp->near_band)
            st->near = 1;
        const bool fin = isfinite(R);
        if (!fin)
            st->status = SS4D_ERR_NONFINITE;
        if (!fin || !(R > dp->tol) || st->z >= dp->maxit) {
            stop = true;
        } else {
            st->mode = 1;
            // aim the round just under the tolerance (the FP32 correction
            // residual tracks the FP64 one after refinement to about 1e-5
            // relative; a round that falls short only costs another round),
            // but not below what FP32 corrections can resolve relative to
            // the current residual
            st->target = fmax(0.9 * dp->tol, 1e-11 * R);
        }
    } else if (mode == 1) {
        st->mode = 2;
        st->dsrc ^= 1;
        st->round_z = 0;
        st->keep = 0;
    } else {
        const double om1 = 1.0 - dp->omega;
        const double Rd = (a + om1 * om1 * c) * dp->h4;
        st->Rd = Rd;
        st->z += 1;
        st->round_z += 1;
        if (!isfinite(Rd) || !(Rd > st->target) || st->z >= dp->maxit) {
            st->mode = 0; // refine with the red correction of this iteration
        } else {
            st->dsrc ^= 1;
        }
    }
    if (stop) {
        st->stop = 1;
        st->final_red = 0;
    }
    return stop;
}

} // namespace ss4d
