// ss4d_common.cuh — geometry, launch helpers and reductions shared by the
// solver's kernels.  Device code only uses what is declared here plus the
// public ss4d.h types.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ss4d.h"

namespace ss4d {

// ---------------------------------------------------------------------------
// Division by a fixed divisor d of numerators below 2^31:
// q = (n * m) >> sh with m = ceil(2^sh / d), sh = 31 + ceil(log2 d)
// (the error term stays below 1/d for every such n).
struct FastDiv {
    unsigned d, m;
    int sh;
};

inline FastDiv make_fastdiv(unsigned d)
{
    FastDiv f;
    f.d = d;
    int s = 0;
    while ((1ull << s) < d)
        ++s;
    f.m = (unsigned)(((1ull << (31 + s)) + d - 1) / d);
    f.sh = 31 + s;
    return f;
}

__host__ __device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv &f)
{
    return (unsigned)(((unsigned long long)n * f.m) >> f.sh);
}

// ---------------------------------------------------------------------------
// Plane pk and frame fl (both from 0) of block z of a grid over P planes of
// F frames: frame by frame (kb <= 0 or kb >= P), else in blocks of kb
// planes, the planes of a block for each frame in turn (the last block
// holds the remaining P mod kb planes).  The divisors are fixed per launch:
// PlaneOrder carries them with their FastDiv multipliers (z < 2^31), since a
// thread of the float-float faces and coefficient kernels, which use this
// order, handles one voxel, and three integer divisions per thread cost the
// issue-bound faces kernel a few per cent.
struct PlaneOrder {
    int blocked;              // 0: frame by frame
    int P, kb, blk, full, rest; // blk = kb F, full = P / kb, rest = P - full kb
    FastDiv fP, fkb, fblk, frest;
};

inline PlaneOrder make_plane_order(int P, int F, int kb)
{
    PlaneOrder o;
    o.blocked = !(kb <= 0 || kb >= P);
    o.P = P;
    o.kb = o.blocked ? kb : 1;
    o.blk = o.kb * F;
    o.full = P / o.kb;
    o.rest = P - o.full * o.kb;
    o.fP = make_fastdiv((unsigned)P);
    o.fkb = make_fastdiv((unsigned)o.kb);
    o.fblk = make_fastdiv((unsigned)(o.blk > 0 ? o.blk : 1));
    o.frest = make_fastdiv((unsigned)(o.rest > 0 ? o.rest : 1));
    return o;
}

__host__ __device__ __forceinline__ void plane_frame(unsigned z, const PlaneOrder &o, int &pk, int &fl)
{
    if (!o.blocked) {
        const unsigned q = fdiv(z, o.fP);
        pk = (int)(z - q * (unsigned)o.P);
        fl = (int)q;
        return;
    }
    const unsigned b = fdiv(z, o.fblk);
    if (b < (unsigned)o.full) {
        const unsigned r = z - b * (unsigned)o.blk, q = fdiv(r, o.fkb);
        fl = (int)q;
        pk = (int)(b * (unsigned)o.kb + (r - q * (unsigned)o.kb));
    } else {
        const unsigned r = z - (unsigned)o.full * (unsigned)o.blk, q = fdiv(r, o.frest);
        fl = (int)q;
        pk = (int)((unsigned)o.full * (unsigned)o.kb + (r - q * (unsigned)o.rest));
    }
}

// ---------------------------------------------------------------------------
// Natural (reference) layout: ((l*kM + k)*jM + j)*iM + i, one ghost per side.
struct Geo {
    int iM, jM, kM, lM;   // padded extents
    int nx, ny, nz, nt;   // interior extents
    long long sy, sz, sw; // strides of j, k, l (i stride is 1)
    long long n;          // padded voxel count (below 2^31)
    long long nint;       // interior voxel count
    FastDiv fiM, fjM, fkM;
};

inline Geo make_geo(const ss4d_dims &d)
{
    Geo g;
    g.iM = d.iMax; g.jM = d.jMax; g.kM = d.kMax; g.lM = d.lMax;
    g.nx = g.iM - 2; g.ny = g.jM - 2; g.nz = g.kM - 2; g.nt = g.lM - 2;
    g.sy = g.iM;
    g.sz = (long long)g.iM * g.jM;
    g.sw = g.sz * g.kM;
    g.n = g.sw * g.lM;
    g.nint = (long long)g.nx * g.ny * g.nz * g.nt;
    g.fiM = make_fastdiv((unsigned)g.iM);
    g.fjM = make_fastdiv((unsigned)g.jM);
    g.fkM = make_fastdiv((unsigned)g.kM);
    return g;
}

// (i, j, k, l) of natural index o < 2^31
__device__ __forceinline__ void nat_coords(const Geo &g, unsigned o, int &i, int &j, int &k, int &l)
{
    unsigned q = fdiv(o, g.fiM);
    i = (int)(o - q * g.fiM.d);
    o = q;
    q = fdiv(o, g.fjM);
    j = (int)(o - q * g.fjM.d);
    o = q;
    q = fdiv(o, g.fkM);
    k = (int)(o - q * g.fkM.d);
    l = (int)q;
}

__host__ __device__ inline long long nat_index(const Geo &g, int i, int j, int k, int l)
{
    return (((long long)l * g.kM + k) * g.jM + j) * g.iM + i;
}

// ---------------------------------------------------------------------------
// Colour-split layout used by the fast forms.  Voxel (i,j,k,l) of colour
// c = (i+j+k+l)&1 lives in colour array c at row (l*kM + k)*jM + j and
// column xs = ((i+1)>>1) + A - 1.  In a row, the interior voxels of either
// colour occupy columns A .. A + nxh - 1 (so interior data starts on an
// aligned boundary), the x-ghosts sit at A-1 and A+nxh.  For a target voxel
// of the row's phase p = (c+j+k+l)&1 at column xs, its x-neighbours (other
// colour) are at xs-p (i-1) and xs-p+1 (i+1); its j/k/l neighbours are in
// the neighbouring rows at the same column xs.
struct Split {
    int A;          // first interior column
    int Hs;         // row pitch in elements (multiple of 8)
    int nxh;        // (nx+1)/2: interior columns per row (upper bound)
    long long rows; // jM*kM*lM
    long long cs;   // elements per colour array (rows*Hs)
    long long ct;   // coefficient records per colour: ny*nz*nt*nxh rounded up to 32
};

// Coefficients are indexed by a compact interior index per colour,
//   t = (((l-1)*nz + (k-1))*ny + (j-1))*nxh + (i-1)/2,
// and stored 32 records at a time, component-major ("AoSoA"): component f of
// record t sits at ((t/32)*nf + f)*32 + t%32.  A warp's 32 consecutive
// targets then read each component as one contiguous segment, and its whole
// record set is one contiguous run.
__host__ __device__ inline long long coef_at(long long t, int f, int nf)
{
    return (((t >> 5) * nf + f) << 5) + (t & 31);
}

inline Split make_split(const Geo &g)
{
    Split s;
    s.A = 8;
    s.nxh = (g.nx + 1) / 2;
    int need = s.A + s.nxh + 1;
    s.Hs = (need + 7) & ~7;
    s.rows = (long long)g.jM * g.kM * g.lM;
    s.cs = s.rows * s.Hs;
    s.ct = (((long long)g.ny * g.nz * g.nt * s.nxh) + 31) & ~31LL;
    return s;
}

// ---------------------------------------------------------------------------
// Deterministic block reduction of one double (any blockDim multiple of 32,
// up to 1024).  Returns the block total in thread 0.
template <typename T>
__device__ inline T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ inline T block_sum(T v)
{
    __shared__ T red_smem[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0)
        red_smem[wid] = v;
    __syncthreads();
    T t = 0;
    if (wid == 0) {
        t = lane < nw ? red_smem[lane] : T(0);
        t = warp_sum(t);
    }
    return t;
}

__device__ inline double block_min(double v)
{
    __shared__ double mn_smem[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0)
        mn_smem[wid] = v;
    __syncthreads();
    double t = 1e308;
    if (wid == 0) {
        t = lane < nw ? mn_smem[lane] : 1e308;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            t = fmin(t, __shfl_down_sync(0xffffffffu, t, o));
    }
    return t;
}

__device__ inline double block_max(double v)
{
    return -block_min(-v);
}

} // namespace ss4d
