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
// at the same time) thus cover a few k planes of all frames, so the
// neighbouring-plane reads of the other colour hit in L2.
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

} // namespace ss4d
