// ss4d_assemble_ff.cu — coefficient assembly of the mixed form in
// float-float arithmetic.
//
// The FP64 assembly (k_faces + k_voxel_coef, ss4d_kernels_fast.cu) executes
// about 125 FP64 instructions per voxel and is bounded by GB300's FP64 pipe
// (roughly 1/70 of its FP32 rate).  Here every quantity after the first
// differences of u is carried as an unevaluated sum of two floats (h + l,
// 48 significant bits; Dekker's and Knuth's error-free transformations: the
// rounding error of a float sum is recovered with the two-sum of Knuth, that
// of a product with one fused multiply-add), so the work runs on the FP32
// pipe.  FP64 instructions are left only where a double enters or leaves
// the float-float form: one subtraction per first difference of u and one
// addition per coefficient written (a double is split into two floats by
// integer operations).
//
//   k_fdiff:          F_a(v) = u(v + e_a) - u(v) for the 4 axes (FP64
//                     difference, split into two floats), natural layout;
//   k_faces_ff:       per face between v and v + e_d, from F only:
//                     |grad u|^2 = F_d^2/h^2 + sum_{a != d} (D_a(v+e_d) + D_a(v))^2/(4h)^2
//                     with D_a(x) = F_a(x) + F_a(x - e_a) the central difference
//                     (the reference's face formula, segmentation4D.c:446-580),
//                     s2 = |grad u|^2 + eps2, fn = s2 / sqrt(s2), fq = g / sqrt(s2);
//   k_voxel_coef_ff:  vc = sqrt(mean(fn)^2 + eps2), c a_f = c vc fq_f,
//                     diag = 1 + sum c a_f; written as FP64 records
//                     (refinement) and the FP32 sweeps' records (16-bit
//                     fractions of sum c a_f and that sum, store_coef16).
//
// Relative error of the coefficients: below 1e-12 (1/sqrt from an FP32 seed
// and one Newton step, about 1.5 (2^-22)^2 each; sums and products to 2^-46).  The mixed form's refinement passes measure the FP64 residual
// against these coefficients; the residual of its result against exact FP64
// coefficients meets the same tolerance (tested), the coefficient error
// entering it only squared, far below any tolerance.
#include <math.h>

#include "ss4d_ff.cuh"

namespace ss4d {

using namespace ffa;


struct FFConst {
    float ih2h, ih2l;   // 1/h^2
    float iq2h, iq2l;   // 1/(4h)^2
    float eps2h, eps2l; // eps2
    float ch, cl;       // tau/h^2
    int pow2;           // 1/h^2 and 1/(4h)^2 are powers of two (h is): exact scaling
};

// forward differences of every voxel that has a neighbour along the axis
// voxels [o0, o1) (whole frames).  With PACK also the split copies of u that
// k_pack makes when prev is u (red voxels into both red buffers, black ones
// into the black buffer, every voxel into prev of its colour): this kernel
// is bound by its FP64 subtractions, and the copy rides along on the
// memory bandwidth it leaves, reading u once for both.  PACK 2 also adds the
// first refinement pass's start correction to the interior of the u copies
// the pass would update (red: R[0], black: Bk) with the pass's own FP64
// addition: the correction in dR[0] / dB (withd) or zero.
template <int PACK>
__global__ void __launch_bounds__(256) k_fdiff(Geo g, Split sp, const double *__restrict__ u, SplitBufs b,
                                               long long o0, long long o1, int withd)
{
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    for (long long o = o0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; o < o1;
         o += (long long)gridDim.x * blockDim.x) {
        int i, j, k, l;
        nat_coords(g, (unsigned)o, i, j, k, l);
        const int idx[4] = {i, j, k, l};
        const int top[4] = {g.iM - 1, g.jM - 1, g.kM - 1, g.lM - 1};
        const double uc = u[o];
#pragma unroll
        for (int a = 0; a < 4; ++a)
            st_ff(b.fd[a], o, idx[a] < top[a] ? ff_from_d(u[o + st[a]] - uc) : ff_make(0.f, 0.f));
        if (PACK) {
            const long long s = (((long long)l * g.kM + k) * g.jM + j) * sp.Hs + ((i + 1) >> 1) + sp.A - 1;
            const bool red = ((i + j + k + l) & 1) == 0;
            double u0 = uc;
            if (PACK == 2 && i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz && l >= 1 &&
                l <= g.nt)
                u0 = uc + (withd ? f2d_bits(red ? b.dR[0][s] : b.dB[s]) : 0.0);
            if (red) {
                b.R[0][s] = u0;
                b.R[1][s] = uc;
                b.P[0][s] = uc;
            } else {
                b.Bk[s] = u0;
                b.P[1][s] = uc;
            }
        }
    }
}

// --- faces ------------------------------------------------------------------
// A block takes a tile of FTX x FTY voxels (i, j) of one (k, l) plane.  The
// central differences D_a of every voxel are formed once, by its own thread,
// and the i- and j-faces read those of their upper neighbour from shared
// memory (the tile plus one column and one row of halo); the k- and l-faces
// form them at v + e_k and v + e_l.  Each quantity is computed with the same
// operations in the same order as a per-face evaluation would.  Offsets are
// 32-bit (padded volumes below 2^31 voxels).
constexpr int FTX = 32, FTY = 8;

__device__ __forceinline__ ff ldf(const float2 *__restrict__ p, unsigned x)
{
    const float2 v = __ldg(p + x);
    return ff_make(v.x, v.y);
}

// D_a(x) = F_a(x) + F_a(x - e_a), unnormalised (it is added again)
__device__ __forceinline__ ff cdiff(const float2 *__restrict__ fa, unsigned x, unsigned sa)
{
    return ff_add_nr(ldf(fa, x), ldf(fa, x - sa));
}

// the face between v and v + e_D: Dv, Dn the central differences at v and
// v + e_D along the axes a != D, cn = F_D(v), gv its g; gives
// r = |grad u|_eps and q = g / |grad u|_eps
template <int D>
__device__ __forceinline__ void face_val(const FFConst &K, const ff Dv[4], const ff Dn[4], ff cn, ff gv, ff &r, ff &q)
{
    // sum of squares of the tangential central differences: positive terms,
    // renormalised once; the first term starts the sum (adding it to zero
    // would give the same pair)
    ff tt;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (a == D)
            continue;
        const ff t = ff_add(Dn[a], Dv[a]); // may cancel: renormalised before squaring
        const float p = t.h * t.h;
        const ff sq = ff_make(p, fmaf(2.f * t.h, t.l, fmaf(t.h, t.h, -p)));
        tt = a == (D == 0 ? 1 : 0) ? sq : ff_add_nr(tt, sq);
    }
    tt = ff_norm(tt);
    const ff cn2 = ff_sqr(cn);
    const ff a1 = K.pow2 ? ff_make(cn2.h * K.ih2h, cn2.l * K.ih2h) : ff_mul(cn2, ff_make(K.ih2h, K.ih2l));
    const ff a2 = K.pow2 ? ff_make(tt.h * K.iq2h, tt.l * K.iq2h) : ff_mul(tt, ff_make(K.iq2h, K.iq2l));
    const ff s2 = ff_add(ff_add_nr(a1, a2), ff_make(K.eps2h, K.eps2l));
    const ff y = ff_rsqrt(s2);
    r = ff_mul(s2, y);
    q = ff_mul(gv, y);
}

// face_val, written as fn and fq at v
template <int D>
__device__ __forceinline__ void face_ff(const FFConst &K, const ff Dv[4], const ff Dn[4], ff cn, ff gv,
                                        const SplitBufs &b, unsigned o)
{
    ff r, q;
    face_val<D>(K, Dv, Dn, cn, gv, r, q);
    __stcs(reinterpret_cast<float2 *>(b.fn[D]) + o, make_float2(r.h, r.l));
    __stcs(reinterpret_cast<float2 *>(b.fq[D]) + o, make_float2(q.h, q.l));
}

// g of the face between v and v + e_D: stored at v (g_e, g_n, ...) where v is
// interior along D, else at v + e_D (g_w, g_s, ...)
template <int D, int UPPER>
__device__ __forceinline__ ff face_g(const CPtrs8 &gin, int has_g, unsigned x)
{
    return has_g ? ff_from_pos_d(__ldg(gin.p[2 * D + UPPER] + x)) : ff_make(1.f, 0.f);
}

// the single face along D of a voxel v whose index along D is 0 (and >= 1
// along the others): the face between the ghost v and v + e_D
template <int D>
__device__ __forceinline__ void boundary_face(const FFConst &K, const CPtrs8 &gin, int has_g, const SplitBufs &b,
                                              const float2 *const F[4], const unsigned st[4], unsigned o,
                                              const ff Dn[4])
{
    ff Dv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
        Dv[a] = a == D ? ff_make(0.f, 0.f) : cdiff(F[a], o, st[a]);
    face_ff<D>(K, Dv, Dn, ldf(F[D], o), face_g<D, 1>(gin, has_g, o + st[D]), b, o);
}

// the faces of every voxel v with all indices in [0, n_a] whose faces
// between v and v + e_d have v and v + e_d in the extended box: all four for
// interior v, the one along a where v's index along a is 0 (and none where
// two indices are); frames l_off .. l_off + gridDim.z / (nz + 1) - 1
// Bound by the latency of its global loads: 8 blocks per SM (32 registers,
// a few bytes of spill) ran 6.28 ms at 256^2 x 128 x 20 against 6.93 ms
// at 5 blocks (48 registers) and 6.74 ms at 6.
__global__ void __launch_bounds__(FTX *FTY, 8) k_faces_ff(Geo g, CPtrs8 gin, int has_g, FFConst K, SplitBufs b,
                                                           int l_off, PlaneOrder po)
{
    __shared__ float2 sD[4][FTY + 1][FTX + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = 1 + blockIdx.x * FTX, j0 = 1 + blockIdx.y * FTY;
    const int i = i0 + tx, j = j0 + ty;
    int k, lf;
    plane_frame(blockIdx.z, po, k, lf);
    const int l = l_off + lf;
    const unsigned st[4] = {1u, (unsigned)g.sy, (unsigned)g.sz, (unsigned)g.sw};
    const float2 *const F[4] = {reinterpret_cast<const float2 *>(b.fd[0]), reinterpret_cast<const float2 *>(b.fd[1]),
                                reinterpret_cast<const float2 *>(b.fd[2]), reinterpret_cast<const float2 *>(b.fd[3])};
    const unsigned o = (((unsigned)l * g.kM + k) * g.jM + j) * g.iM + i;
    if (k == 0 || l == 0) { // ghost plane or frame: its one face along k or l
        if (k == l || i > g.nx || j > g.ny)
            return;
        ff Dn[4];
        if (k == 0) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
                Dn[a] = a == 2 ? ff_make(0.f, 0.f) : cdiff(F[a], o + st[2], st[a]);
            boundary_face<2>(K, gin, has_g, b, F, st, o, Dn);
        } else {
#pragma unroll
            for (int a = 0; a < 4; ++a)
                Dn[a] = a == 3 ? ff_make(0.f, 0.f) : cdiff(F[a], o + st[3], st[a]);
            boundary_face<3>(K, gin, has_g, b, F, st, o, Dn);
        }
        return;
    }
    // central differences of the tile (ghost column / row included) ...
    ff Dv[4];
    if (i <= g.nx + 1 && j <= g.ny + 1) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            Dv[a] = cdiff(F[a], o, st[a]);
            sD[a][ty][tx] = make_float2(Dv[a].h, Dv[a].l);
        }
    }
    // ... and of its halo: row j0 + FTY (for the j-faces of the tile's last
    // row) and column i0 + FTX (for the i-faces of its last column), where
    // those faces exist
    if (ty == 0) {
        if (i <= g.nx && j0 + FTY <= g.ny + 1) {
            const unsigned oh = o + FTY * st[1];
#pragma unroll
            for (int a = 0; a < 4; ++a)
                if (a != 1) {
                    const ff d = cdiff(F[a], oh, st[a]);
                    sD[a][FTY][tx] = make_float2(d.h, d.l);
                }
        }
    } else if (ty == 1 && tx < FTY) {
        if (i0 + FTX <= g.nx + 1 && j0 + tx <= g.ny) {
            const unsigned oh = (((unsigned)l * g.kM + k) * g.jM + (j0 + tx)) * g.iM + (i0 + FTX);
#pragma unroll
            for (int a = 1; a < 4; ++a) {
                const ff d = cdiff(F[a], oh, st[a]);
                sD[a][tx][FTX] = make_float2(d.h, d.l);
            }
        }
    }
    __syncthreads();
    if (i > g.nx || j > g.ny)
        return;
    ff Dn[4];
    // i-face and j-face: the upper neighbour's differences from the tile
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float2 v = sD[a][ty][tx + 1];
        Dn[a] = ff_make(v.x, v.y);
    }
    face_ff<0>(K, Dv, Dn, ldf(F[0], o), face_g<0, 0>(gin, has_g, o), b, o);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float2 v = sD[a][ty + 1][tx];
        Dn[a] = ff_make(v.x, v.y);
    }
    face_ff<1>(K, Dv, Dn, ldf(F[1], o), face_g<1, 0>(gin, has_g, o), b, o);
    // k-face and l-face: the differences at v + e_k and v + e_l
#pragma unroll
    for (int a = 0; a < 4; ++a)
        Dn[a] = a == 2 ? ff_make(0.f, 0.f) : cdiff(F[a], o + st[2], st[a]);
    face_ff<2>(K, Dv, Dn, ldf(F[2], o), face_g<2, 0>(gin, has_g, o), b, o);
#pragma unroll
    for (int a = 0; a < 4; ++a)
        Dn[a] = a == 3 ? ff_make(0.f, 0.f) : cdiff(F[a], o + st[3], st[a]);
    face_ff<3>(K, Dv, Dn, ldf(F[3], o), face_g<3, 0>(gin, has_g, o), b, o);
    // the faces between the ghosts i = 0 / j = 0 and the first voxel: the
    // thread of that voxel (its differences are the upper side's)
    if (i == 1)
        boundary_face<0>(K, gin, has_g, b, F, st, o - 1, Dv);
    if (j == 1)
        boundary_face<1>(K, gin, has_g, b, F, st, o - st[1], Dv);
}

// Memory-bound, its warps waiting on loads: 8 blocks per SM (32 registers)
// rather than 7 took the assembly from 13.5 to 13.0 ms at 256^2 x 128 x 20.
// With PRE it also forms the first refinement pass's FP64 residual at the
// target exactly as k_refine forms it (prev, then the products of the eight
// coefficients just written with the other colour's u in record order, then
// diag u0, with the same fused multiply-adds) on the split copies of u whose
// start correction the first-difference kernel added, into rpre.
// The records of interior voxel (i, j, k, l) (and with PRE the first pass's
// residual) from its 8 faces: fp[d], fm[d] the |grad u|_eps of its faces
// towards v + e_d and v - e_d, q[2d], q[2d+1] their g / |grad u|_eps
template <int PRE>
__device__ __forceinline__ void voxel_coef(const Geo &g, const Split &sp, const FFConst &K, const SplitBufs &b, int i,
                                           int j, int k, int l, const ff fp[4], const ff fm[4], const ff q[8])
{
    ff sum = ff_make(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 4; ++d) // positive terms: renormalised once
        sum = ff_add_nr(sum, ff_add_nr(fp[d], fm[d]));
    sum = ff_norm(sum);
    // mean^2 + eps2 with mean = sum / 8 (exact scaling)
    const ff m = ff_make(sum.h * 0.125f, sum.l * 0.125f);
    const ff x = ff_add(ff_sqr(m), ff_make(K.eps2h, K.eps2l));
    const ff cv = ff_mul(ff_make(K.ch, K.cl), ff_mul(x, ff_rsqrt(x))); // c * vc
    const int col = (i + j + k + l) & 1;
    double *cf = pick(b.coef, col);
    const long long t = coef_index(g, sp, i, j, k, l);
    // split index of the target and its neighbours (row phase p = i & 1)
    const long long Hy = sp.Hs, Hz = Hy * g.jM, Hw = Hz * g.kM;
    const long long sx = (((long long)l * g.kM + k) * g.jM + j) * Hy + ((i + 1) >> 1) + sp.A - 1;
    const int p = i & 1;
    const long long nb[8] = {sx - p + 1, sx - p, sx + Hy, sx - Hy, sx + Hz, sx - Hz, sx + Hw, sx - Hw};
    const double *__restrict__ oth = col == 0 ? b.Bk : b.R[0];
    double S = PRE ? __ldg(pick(b.P, col) + sx) : 0.0;
    ff diag = ff_make(1.f, 0.f);
    float a32[8];
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        const ff a = ff_mul(cv, q[f]);
        diag = ff_add_nr(diag, a); // positive terms: renormalised after the loop
        const double ad = ff_to_d(a);
        __stcs(cf + coef_at(t, f, 10), ad);
        a32[f] = a.h;
        if (PRE)
            S = fma(ad, __ldg(oth + nb[f]), S);
    }
    diag = ff_norm(diag);
    const double dd = ff_to_d(diag);
    __stcs(cf + coef_at(t, 8, 10), dd);
    if (PRE)
        pick(b.rpre, col)[sx] = fma(dd, __ldg((col == 0 ? b.R[0] : b.Bk) + sx), -S);
    // component 9 (omega/diag) serves only the FP64 sweep, whose form always
    // assembles its own records: not written here
    store_coef16(pick(b.coefq, col), pick(b.coefs, col), t, a32);
}

template <int PRE>
__global__ void __launch_bounds__(256, PRE ? 6 : 8) k_voxel_coef_ff(Geo g, Split sp, FFConst K, SplitBufs b, int l_off,
                                                                    PlaneOrder po)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    int kk, lf;
    plane_frame(blockIdx.z, po, kk, lf);
    const int k = 1 + kk, l = 1 + l_off + lf;
    if (i > g.nx || j > g.ny)
        return;
    const long long o = nat_index(g, i, j, k, l);
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    ff fp[4], fm[4], q[8];
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        fp[d] = ld_ff(b.fn[d], o);
        fm[d] = ld_ff(b.fn[d], o - st[d]);
        q[2 * d] = ld_ff(b.fq[d], o);
        q[2 * d + 1] = ld_ff(b.fq[d], o - st[d]);
    }
    voxel_coef<PRE>(g, sp, K, b, i, j, k, l, fp, fm, q);
}

static void split_host(double v, float &h, float &l)
{
    h = (float)v;
    l = (float)(v - (double)h);
}

template <int PACK> static int max_blocks_fdiff()
{
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_fdiff<PACK>, 256, 0);
    return a > 0 ? a : 1;
}

void launch_fdiff_range(const Geo &g, const double *u, SplitBufs b, int l0, int l1, int sm_count, cudaStream_t st)
{
    k_fdiff<0><<<sm_count * max_blocks_fdiff<0>(), 256, 0, st>>>(g, Split{}, u, b, (long long)l0 * g.sw,
                                                                  (long long)l1 * g.sw, 0);
}

void launch_fdiff_pack_range(const Geo &g, const Split &s, const double *u, SplitBufs b, int l0, int l1, int sm_count,
                             cudaStream_t st, int pre)
{
    if (pre)
        k_fdiff<2><<<sm_count * max_blocks_fdiff<2>(), 256, 0, st>>>(g, s, u, b, (long long)l0 * g.sw,
                                                                      (long long)l1 * g.sw, pre == 2);
    else
        k_fdiff<1><<<sm_count * max_blocks_fdiff<1>(), 256, 0, st>>>(g, s, u, b, (long long)l0 * g.sw,
                                                                      (long long)l1 * g.sw, 0);
}

void launch_assemble_ff(const Geo &g, const Split &s, const double *u, CPtrs8 gin, int has_g, const ss4d_params &p,
                        SplitBufs b, int pack, int sm_count, cudaStream_t st, int pre, int kblock)
{
    if (pack)
        launch_fdiff_pack_range(g, s, u, b, 0, g.lM, sm_count, st, pre);
    else
        launch_fdiff_range(g, u, b, 0, g.lM, sm_count, st);
    launch_assemble_ff_faces(g, s, gin, has_g, p, b, st, pack ? pre : 0, kblock);
}

void launch_assemble_ff_faces(const Geo &g, const Split &s, CPtrs8 gin, int has_g, const ss4d_params &p, SplitBufs b,
                              cudaStream_t st, int pre, int kblock)
{
    launch_assemble_ff_faces_range(g, s, gin, has_g, p, b, 0, g.nt + 1, 1, g.nt + 1, st, pre, kblock);
}

static FFConst make_ffconst(const ss4d_params &p)
{
    FFConst K;
    split_host(1.0 / (p.h * p.h), K.ih2h, K.ih2l);
    split_host(1.0 / (16.0 * p.h * p.h), K.iq2h, K.iq2l);
    split_host(p.eps2, K.eps2h, K.eps2l);
    split_host(p.tau / (p.h * p.h), K.ch, K.cl);
    int e1 = 0, e2 = 0;
    K.pow2 = K.ih2l == 0.f && K.iq2l == 0.f && frexp((double)K.ih2h, &e1) == 0.5 && frexp((double)K.iq2h, &e2) == 0.5;
    return K;
}

void launch_assemble_ff_faces_range(const Geo &g, const Split &s, CPtrs8 gin, int has_g, const ss4d_params &p,
                                    SplitBufs b, int f0, int f1, int v0, int v1, cudaStream_t st, int pre, int kblock)
{
    const FFConst K = make_ffconst(p);
    if (f1 > f0) {
        dim3 gr((g.nx + FTX - 1) / FTX, (g.ny + FTY - 1) / FTY, (g.nz + 1) * (f1 - f0));
        k_faces_ff<<<gr, dim3(FTX, FTY, 1), 0, st>>>(g, gin, has_g, K, b, f0,
                                                     make_plane_order(g.nz + 1, f1 - f0, kblock));
    }
    {
        const int bx = g.nx >= 128 ? 128 : (g.nx >= 64 ? 64 : 32);
        const int by = 256 / bx;
        dim3 bl(bx, by, 1);
        dim3 gr((g.nx + bx - 1) / bx, (g.ny + by - 1) / by, g.nz * (v1 - v0));
        const PlaneOrder po = make_plane_order(g.nz, v1 - v0, kblock);
        if (v1 > v0 && pre)
            k_voxel_coef_ff<1><<<gr, bl, 0, st>>>(g, s, K, b, v0 - 1, po);
        else if (v1 > v0)
            k_voxel_coef_ff<0><<<gr, bl, 0, st>>>(g, s, K, b, v0 - 1, po);
    }
}

} // namespace ss4d
