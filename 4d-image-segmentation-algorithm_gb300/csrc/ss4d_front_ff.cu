// ss4d_front_ff.cu — the edge detector of the mixed form in float-float
// arithmetic: the presmoothing's red-black SOR (segmentation4D.c:337-409) and
// the 8 face g values (segmentation4D.c:594-821, _gFunction_ :67-70), with
// about 48 significant bits on the FP32 pipe instead of FP64.  The plain and
// reference forms keep the reference's FP64 rounding (ss4d_kernels_ref.cu);
// on GB300 that work is bound by the FP64 pipe, this form by memory.
//
// The image and the presmoothing's copy of its input (the reference's
// prev_u) are converted to float-float arrays (float2) once; the SOR
// iterations read and write those; the interior is written back as doubles
// at the end (h + l is exact in a double), the ghosts of the double image
// keep the values the reflection gave them.  Relative error of the results
// against the FP64 forms: about 1e-14 for the smoothed image, 1e-13 for g.
#include "ss4d_ff.cuh"

namespace ss4d {

using namespace ffa;

namespace {

__device__ __forceinline__ ff ffc(FFc c)
{
    return ff_make(c.h, c.l);
}

// sum over a 2D block (flattened thread index); the result in thread (0, 0)
__device__ double block_sum_flat(double v)
{
    __shared__ double part[32];
    const int t = threadIdx.y * blockDim.x + threadIdx.x, lane = t & 31, wid = t >> 5;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    v = warp_sum(v);
    if (lane == 0)
        part[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < nw ? part[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// the voxels of one colour, one per thread (every lane busy): thread x
// indexes the pairs (i, i+1) of a row
__device__ __forceinline__ bool colour_voxel(const Geo &g, int colour, int &i, int &j, int &k, int &l)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = blockIdx.z;
    k = 1 + kl % g.nz;
    l = 1 + kl / g.nz;
    i = 1 + 2 * t + ((colour + j + k + l + 1) & 1);
    return i <= g.nx && j <= g.ny;
}

__device__ __forceinline__ ff sum8(const float2 *v, long long o, const Geo &g)
{
    ff s = ff_add(ld_ff2(v, o + 1), ld_ff2(v, o - 1));
    s = ff_add(s, ld_ff2(v, o - g.sy));
    s = ff_add(s, ld_ff2(v, o + g.sy));
    s = ff_add(s, ld_ff2(v, o - g.sz));
    s = ff_add(s, ld_ff2(v, o + g.sz));
    s = ff_add(s, ld_ff2(v, o - g.sw));
    return ff_add(s, ld_ff2(v, o + g.sw));
}

__global__ void k_to_ff(long long n, const double *__restrict__ a, float2 *__restrict__ out)
{
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x)
        st_ff2(out, o, ff_from_d(a[o]));
}

__global__ void k_from_ff(Geo g, const float2 *__restrict__ v, double *__restrict__ out)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = 1 + blockIdx.z % g.nz, l = 1 + blockIdx.z / g.nz;
    if (i > g.nx || j > g.ny)
        return;
    const long long o = nat_index(g, i, j, k, l);
    out[o] = ff_to_d(ld_ff2(v, o));
}

// gs = (prev + c sum_8 v_nb) / (1 + 8c), v += omega (gs - v); inv_d = 1/(1 + 8c)
__global__ void k_presmooth_half_ff(Geo g, float2 *v, const float2 *__restrict__ prev, FFc c, FFc inv_d, FFc omega,
                                    int colour)
{
    int i, j, k, l;
    if (!colour_voxel(g, colour, i, j, k, l))
        return;
    const long long o = nat_index(g, i, j, k, l);
    const ff gs = ff_mul(ff_add(ld_ff2(prev, o), ff_mul(ffc(c), sum8(v, o, g))), ffc(inv_d));
    const ff vo = ld_ff2(v, o);
    st_ff2(v, o, ff_add(vo, ff_mul(ffc(omega), ff_add(gs, ff_neg(vo)))));
}

#define FRONT_RESID_K 4

// r = v (1 + 8c) - c sum_8 v_nb - prev; a thread sums r^2 over FRONT_RESID_K
// planes (FP32: the sum decides the stop test only), the block in FP64
__global__ void k_presmooth_resid_ff(Geo g, const float2 *__restrict__ v, const float2 *__restrict__ prev, FFc c,
                                     FFc d, double h4, double *partial)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int nkb = (g.nz + FRONT_RESID_K - 1) / FRONT_RESID_K;
    const int k0 = 1 + (blockIdx.z % nkb) * FRONT_RESID_K, l = 1 + blockIdx.z / nkb;
    float acc = 0.f;
    if (i <= g.nx && j <= g.ny) {
        for (int k = k0; k < k0 + FRONT_RESID_K && k <= g.nz; ++k) {
            const long long o = nat_index(g, i, j, k, l);
            const ff r = ff_add(ff_add(ff_mul(ld_ff2(v, o), ffc(d)), ff_neg(ff_mul(ffc(c), sum8(v, o, g)))),
                                ff_neg(ld_ff2(prev, o)));
            acc = fmaf(r.h, r.h, acc);
        }
    }
    const double tot = block_sum_flat((double)acc * h4);
    if (threadIdx.x == 0 && threadIdx.y == 0)
        partial[(blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = tot;
}

// face_sq of the face between o and o + st[D] (the reference's face formula)
template <int D>
__device__ __forceinline__ ff face_sq_ff(const float2 *v, long long o, const long long st[4], ff ih, ff iq)
{
    const long long nb = o + st[D];
    ff s = ff_make(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ff comp;
        if (a == D) {
            comp = ff_mul(ff_add(ld_ff2(v, nb), ff_neg(ld_ff2(v, o))), ih);
        } else {
            const ff plus = ff_add(ld_ff2(v, nb + st[a]), ld_ff2(v, o + st[a]));
            const ff minus = ff_add(ld_ff2(v, nb - st[a]), ld_ff2(v, o - st[a]));
            comp = ff_mul(ff_add(plus, ff_neg(minus)), iq);
        }
        s = ff_add_nr(s, ff_sqr(comp)); // positive terms
    }
    return ff_norm(s);
}

struct FaceConst {
    FFc ih, iq, K, theta, rho;
};

// each face shared by two voxels once, as k_gfaces: the thread at o (every
// coordinate 0..n) computes the + face along D when o's other coordinates
// are interior and stores it as g[2D][o] and g[2D+1][o + st[D]]
template <int D>
__device__ __forceinline__ void gface_plus_ff(const int c[4], const int n[4], long long o, const long long st[4],
                                              const float2 *i0, const float2 *ithr, GPtrs8 &gout, const FaceConst &F)
{
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (a != D && c[a] < 1)
            return;
    const ff ih = ffc(F.ih), iq = ffc(F.iq);
    ff s = ff_mul(ffc(F.theta), face_sq_ff<D>(i0, o, st, ih, iq));
    if (ithr)
        s = ff_add(s, ff_mul(ffc(F.rho), face_sq_ff<D>(ithr, o, st, ih, iq)));
    const double gv = ff_to_d(ff_rcp(ff_add(ff_make(1.f, 0.f), ff_mul(ffc(F.K), s))));
    if (c[D] >= 1)
        gout.p[2 * D][o] = gv;
    if (c[D] < n[D])
        gout.p[2 * D + 1][o + st[D]] = gv;
}

// 6 blocks per SM (40 registers) rather than 4 (56): the mixed edge
// detector at 256^2 x 128 x 20 went from 71.5 to 70.6 ms (8 blocks spilled
// and gained less)
__global__ void __launch_bounds__(256, 6) k_gfaces_ff(Geo g, const float2 *__restrict__ i0, const float2 *__restrict__ ithr, GPtrs8 gout,
                            FaceConst F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = blockIdx.z;
    const int k = kl % (g.nz + 1), l = kl / (g.nz + 1);
    if (i > g.nx || j > g.ny)
        return;
    const int c[4] = {i, j, k, l};
    const int n[4] = {g.nx, g.ny, g.nz, g.nt};
    const long long o = nat_index(g, i, j, k, l);
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    gface_plus_ff<0>(c, n, o, st, i0, ithr, gout, F);
    gface_plus_ff<1>(c, n, o, st, i0, ithr, gout, F);
    gface_plus_ff<2>(c, n, o, st, i0, ithr, gout, F);
    gface_plus_ff<3>(c, n, o, st, i0, ithr, gout, F);
}

dim3 row_block(int nx)
{
    const int bx = nx >= 128 ? 128 : (nx >= 64 ? 64 : 32);
    return dim3(bx, 256 / bx, 1);
}

} // namespace

FFc split_ff(double v)
{
    FFc c;
    c.h = (float)v;
    c.l = (float)(v - (double)c.h);
    return c;
}

void launch_to_ff(const Geo &g, const double *a, float2 *out, cudaStream_t st)
{
    k_to_ff<<<2048, 256, 0, st>>>(g.n, a, out);
}

void launch_from_ff(const Geo &g, const float2 *v, double *out, cudaStream_t st)
{
    const dim3 bl = row_block(g.nx);
    k_from_ff<<<dim3((g.nx + bl.x - 1) / bl.x, (g.ny + bl.y - 1) / bl.y, g.nz * g.nt), bl, 0, st>>>(g, v, out);
}

void launch_presmooth_half_ff(const Geo &g, float2 *v, const float2 *prev, double c, double omega, int colour,
                              cudaStream_t st)
{
    const int nxh = (g.nx + 1) / 2;
    const dim3 bl = row_block(nxh);
    const dim3 gr((nxh + bl.x - 1) / bl.x, (g.ny + bl.y - 1) / bl.y, g.nz * g.nt);
    k_presmooth_half_ff<<<gr, bl, 0, st>>>(g, v, prev, split_ff(c), split_ff(1.0 / (1 + c * 8)), split_ff(omega),
                                           colour);
}

long long front_resid_blocks(const Geo &g)
{
    const dim3 bl = row_block(g.nx);
    return (long long)((g.nx + bl.x - 1) / bl.x) * ((g.ny + bl.y - 1) / bl.y) *
           ((g.nz + FRONT_RESID_K - 1) / FRONT_RESID_K) * g.nt;
}

void launch_presmooth_resid_ff(const Geo &g, const float2 *v, const float2 *prev, double c, double h4,
                               double *partial, cudaStream_t st)
{
    const dim3 bl = row_block(g.nx);
    const dim3 gr((g.nx + bl.x - 1) / bl.x, (g.ny + bl.y - 1) / bl.y,
                  ((g.nz + FRONT_RESID_K - 1) / FRONT_RESID_K) * g.nt);
    k_presmooth_resid_ff<<<gr, bl, 0, st>>>(g, v, prev, split_ff(c), split_ff(1 + c * 8), h4, partial);
}

void launch_gfaces_ff(const Geo &g, const float2 *i0, const float2 *ithr, GPtrs8 gout, double h, double K,
                      double theta, double rho, cudaStream_t st)
{
    const dim3 bl = row_block(g.nx + 1);
    const dim3 gr((g.nx + 1 + bl.x - 1) / bl.x, (g.ny + 1 + bl.y - 1) / bl.y, (g.nz + 1) * (g.nt + 1));
    FaceConst F;
    F.ih = split_ff(1.0 / h);
    F.iq = split_ff(1.0 / (4.0 * h));
    F.K = split_ff(K);
    F.theta = split_ff(theta);
    F.rho = split_ff(rho);
    k_gfaces_ff<<<gr, bl, 0, st>>>(g, i0, ithr, gout, F);
}

} // namespace ss4d
