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

// Records of the FP32 correction sweeps.  The sweeps stream their records
// once per half-sweep and are bound by HBM, so a record is compressed: per
// target the scale s = sum_f c a_f in FP32 and the eight fractions
// w_f = c a_f / s in [0, 1] as 16-bit fixed-point numbers q_f (w_f = q_f /
// 2^16 rounded to nearest, 65535 at most): 20 bytes instead of 32 for eight
// FP32 values.  A sweep uses c a_f = s q_f / 2^16 and the diagonal
// 1 + s sum_f q_f / 2^16, so every row keeps the FP64 operator's structure
// diag - sum_f c a_f = 1: the rounding only moves weight between the target
// and its neighbours, and changes A d by sum_f da_f (d - d_f) with |da_f| <=
// 2^-17 s, small where the correction d is smooth.  The FP64 refinement
// measures the residual with the FP64 records, so the stop rule and the
// tolerance are those of the FP64 operator.
__device__ __forceinline__ void store_coef16(uint4 *__restrict__ cq, float *__restrict__ cs, long long t,
                                             const float a[8])
{
    const float s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    // the scale of the rounding need not be exact: a sweep forms its
    // diagonal from the stored fractions themselves
    const float k = s > 0.f ? __fdividef(65536.f, s) : 0.f;
    unsigned q[8];
#pragma unroll
    for (int f = 0; f < 8; ++f)
        q[f] = min(__float2uint_rn(a[f] * k), 65535u);
    __stcs(cq + t, make_uint4(q[0] | (q[1] << 16), q[2] | (q[3] << 16), q[4] | (q[5] << 16), q[6] | (q[7] << 16)));
    __stcs(cs + t, s);
}

// q / 2^16 for the low / high 16 bits of x, exactly: the bits under the
// exponent of 2^23 give 2^23 + q, and (2^23 + q) 2^-16 - 128 rounds nowhere
__device__ __forceinline__ float q16_lo(unsigned x)
{
    return fmaf(__uint_as_float((x & 0xFFFFu) | 0x4B000000u), 0x1p-16f, -128.f);
}
__device__ __forceinline__ float q16_hi(unsigned x)
{
    return fmaf(__uint_as_float((x >> 16) | 0x4B000000u), 0x1p-16f, -128.f);
}

// the fractions w[8] and the scale of record t
__device__ __forceinline__ float load_coef16(const uint4 *__restrict__ cq, const float *__restrict__ cs, long long t,
                                             float w[8])
{
    const uint4 v = __ldcs(cq + t);
    w[0] = q16_lo(v.x);
    w[1] = q16_hi(v.x);
    w[2] = q16_lo(v.y);
    w[3] = q16_hi(v.y);
    w[4] = q16_lo(v.z);
    w[5] = q16_hi(v.z);
    w[6] = q16_lo(v.w);
    w[7] = q16_hi(v.w);
    return __ldcs(cs + t);
}

// residual of the correction equation at a target: diag u0 - (s sum_f w_f
// u_f + rhs), diag = 1 + s sum_f w_f; nb[f] the neighbours in record order
__device__ __forceinline__ float resid32(const float w[8], float sc, const float nb[8], float u0, float rhs,
                                         float &diag)
{
    float T = w[0] * nb[0];
#pragma unroll
    for (int f = 1; f < 8; ++f)
        T = fmaf(w[f], nb[f], T);
    diag = fmaf(sc, ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7])), 1.f);
    return fmaf(diag, u0, -fmaf(sc, T, rhs));
}

// One FP32 SOR update of the correction at a target: returns the pre-update
// residual of the correction equation and the updated value, which the
// caller stores.
struct Sweep32Out {
    float r, u;
};
__device__ __forceinline__ Sweep32Out sweep32_target(const Geo &g, const Split &sp, const TileCoord &tc, int p,
                                                     long long s, long long Hy, long long Hz, long long Hw,
                                                     const float *src, const float *__restrict__ oth,
                                                     const uint4 *__restrict__ cq, const float *__restrict__ cs,
                                                     const float *__restrict__ rhs, float omega)
{
    const float u0 = src[s];
    float w[8];
    const float sc = load_coef16(cq, cs, tile_coef_index(g, sp, tc), w);
    const float nb[8] = {ld_ro(oth + s - p + 1), ld_ro(oth + s - p), ld_ro(oth + s + Hy), ld_ro(oth + s - Hy),
                         ld_ro(oth + s + Hz),    ld_ro(oth + s - Hz), ld_ro(oth + s + Hw), ld_ro(oth + s - Hw)};
    float diag;
    const float r = resid32(w, sc, nb, u0, ld_stream(rhs + s), diag);
    // the relaxation weight omega / diag to a few ulp (diag in [1, 2^126))
    return Sweep32Out{r, fmaf(-__fdividef(omega, diag), r, u0)};
}

// Two adjacent targets xi, xi + 1 of one row of an FP32 half-sweep (the
// second only when `two`), row phase p, split index s of the first (even:
// xi, Hs and A are), compact record index tq of the first; 32-bit offsets
// (a colour array holds fewer than 2^31 elements).  The pair reads its own
// values, right-hand sides and y/z/w neighbours as 8-byte pairs and shares
// its index arithmetic; each target's arithmetic is sweep32_target's.
// Returns acc plus the squared pre-update residuals (first target first).
__device__ __forceinline__ float sweep32_pair(int p, unsigned s, unsigned tq, bool two, unsigned Hy, unsigned Hz,
                                              unsigned Hw, const float *src, float *dst, const float *__restrict__ oth,
                                              const uint4 *__restrict__ cq, const float *__restrict__ cs,
                                              const float *__restrict__ rhs, float omega, float acc)
{
    const float2 u = *reinterpret_cast<const float2 *>(src + s);
    const float2 rh = __ldcs(reinterpret_cast<const float2 *>(rhs + s));
    float w0[8], w1[8];
    const float sc0 = load_coef16(cq, cs, tq, w0);
    float sc1 = 0.f;
    if (two)
        sc1 = load_coef16(cq, cs, tq + 1, w1);
    // x neighbours of the pair: the other colour's columns s - p .. s - p + 2
    const float2 vx = ld_ro(reinterpret_cast<const float2 *>(oth + s));
    const float ex = ld_ro(oth + (p ? s - 1 : s + 2));
    const float2 yp = ld_ro(reinterpret_cast<const float2 *>(oth + s + Hy));
    const float2 ym = ld_ro(reinterpret_cast<const float2 *>(oth + s - Hy));
    const float2 zp = ld_ro(reinterpret_cast<const float2 *>(oth + s + Hz));
    const float2 zm = ld_ro(reinterpret_cast<const float2 *>(oth + s - Hz));
    const float2 wp = ld_ro(reinterpret_cast<const float2 *>(oth + s + Hw));
    const float2 wm = ld_ro(reinterpret_cast<const float2 *>(oth + s - Hw));
    // record order: +x (column s_t - p + 1), -x (s_t - p), +y, -y, +z, -z, +w, -w
    const float nb0[8] = {p ? vx.x : vx.y, p ? ex : vx.x, yp.x, ym.x, zp.x, zm.x, wp.x, wm.x};
    float d0;
    const float r0 = resid32(w0, sc0, nb0, u.x, rh.x, d0);
    const float o0 = fmaf(-__fdividef(omega, d0), r0, u.x);
    acc = fmaf(r0, r0, acc);
    if (two) {
        const float nb1[8] = {p ? vx.y : ex, p ? vx.x : vx.y, yp.y, ym.y, zp.y, zm.y, wp.y, wm.y};
        float d1;
        const float r1 = resid32(w1, sc1, nb1, u.y, rh.y, d1);
        acc = fmaf(r1, r1, acc);
        *reinterpret_cast<float2 *>(dst + s) = make_float2(o0, fmaf(-__fdividef(omega, d1), r1, u.y));
    } else {
        dst[s] = o0;
    }
    return acc;
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
        st->pre = 0;    // later passes form their own residual
        st->paused = 0; // the pass a paused loop left for later has now run
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
            st->mode = 0;          // refine with the red correction of this iteration
            st->paused = st->spec; // (and, with spec, leave that pass to the caller)
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
