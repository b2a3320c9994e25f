// ss4d_kernels_ref.cu — natural-layout FP64 kernels in the reference's
// expression order.
//
// This translation unit is compiled with --fmad=false: every multiply and add
// is rounded separately, the way the x86-64 reference build rounds them, and
// division and square root are IEEE round-to-nearest.  The voxel updates here
// therefore reproduce the reference's arithmetic; only the order of the
// residual/norm summations differs (a parallel reduction instead of one
// serial sum).  They serve the SS4D_ARITH_REFERENCE form, the edge detector of
// every form (run once per segmentation), the MCF boundary and exact
// solution, the rescale, the mask and the norms.
#include "ss4d_kernels.cuh"

namespace ss4d {

// ---------------------------------------------------------------------------
// launch geometry over interior voxels: x along threadIdx.x, y along
// threadIdx.y, (k, l) along blockIdx.z.

__device__ inline bool interior_ijkl(const Geo &g, int &i, int &j, int &k, int &l)
{
    i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = blockIdx.z;
    k = 1 + kl % g.nz;
    l = 1 + kl / g.nz;
    return i <= g.nx && j <= g.ny;
}

// the voxels of one colour ((i + j + k + l) & 1 == colour), one per thread:
// thread x indexes the pairs (i, i+1) of a row, so every lane of a warp
// updates a voxel (a lane masked off by a colour test costs the FP64 pipe as
// much as an active one)
__device__ inline bool colour_ijkl(const Geo &g, int colour, int &i, int &j, int &k, int &l)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int kl = blockIdx.z;
    k = 1 + kl % g.nz;
    l = 1 + kl / g.nz;
    i = 1 + 2 * t + ((colour + j + k + l + 1) & 1);
    return i <= g.nx && j <= g.ny;
}

__device__ inline unsigned block_linear()
{
    return (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

__device__ inline int flat_tid()
{
    return threadIdx.y * blockDim.x + threadIdx.x;
}

// Block reduction over a 2D block (flattened thread order).
__device__ inline double block_sum2d(double v)
{
    __shared__ double s2[32];
    const int t = flat_tid();
    const int lane = t & 31, wid = t >> 5;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0)
        s2[wid] = v;
    __syncthreads();
    double r = 0;
    if (wid == 0) {
        r = lane < nw ? s2[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// ---------------------------------------------------------------------------
// Neumann reflection, one axis per launch (segmentation4D.c:826-864 runs the
// axes in x, y, z, w order over full padded ranges).

__global__ void k_reflect_axis(Geo g, double *u, int axis)
{
    // enumerate the padded cross-section orthogonal to `axis`
    long long cnt;
    int e[3];
    long long st[3], sa;
    int Ma;
    if (axis == 0) { e[0] = g.jM; e[1] = g.kM; e[2] = g.lM; st[0] = g.sy; st[1] = g.sz; st[2] = g.sw; sa = 1; Ma = g.iM; }
    else if (axis == 1) { e[0] = g.iM; e[1] = g.kM; e[2] = g.lM; st[0] = 1; st[1] = g.sz; st[2] = g.sw; sa = g.sy; Ma = g.jM; }
    else if (axis == 2) { e[0] = g.iM; e[1] = g.jM; e[2] = g.lM; st[0] = 1; st[1] = g.sy; st[2] = g.sw; sa = g.sz; Ma = g.kM; }
    else { e[0] = g.iM; e[1] = g.jM; e[2] = g.kM; st[0] = 1; st[1] = g.sy; st[2] = g.sz; sa = g.sw; Ma = g.lM; }
    cnt = (long long)e[0] * e[1] * e[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < cnt; t += (long long)gridDim.x * blockDim.x) {
        long long r = t;
        int a0 = (int)(r % e[0]); r /= e[0];
        int a1 = (int)(r % e[1]);
        int a2 = (int)(r / e[1]);
        long long base = a0 * st[0] + a1 * st[1] + a2 * st[2];
        u[base] = u[base + sa];
        u[base + (Ma - 1) * sa] = u[base + (Ma - 2) * sa];
    }
}

// ---------------------------------------------------------------------------
// x / d, rounded to nearest, for a divisor d > 0 known in advance with
// y = 1/d rounded to nearest (y == 0: no fast path).  A quotient from the
// reciprocal and one remainder correction (Markstein's iteration), then an
// exact acceptance test: the remainder x - q d (one FMA, correctly rounded) must
// be below d times half the spacing from q to its nearer neighbour; since
// that bound is a power-of-two multiple of d, hence exact, and rounding is
// monotonic, passing it proves q is the double nearest to x / d.  Otherwise
// (near a tie, zero, q outside [2^-400, 2^601)) the IEEE division decides.
__device__ inline double div_by_const(double x, double d, double y)
{
    if (y != 0.0) {
        const double q0 = x * y;
        const double q = fma(fma(-q0, d, x), y, q0);
        const long long b = __double_as_longlong(q);
        const int E = (int)((b >> 52) & 0x7ff) - 1023;
        if (E >= -400 && E <= 600) {
            const int e = E - 53 - ((b & 0xfffffffffffffLL) == 0 ? 1 : 0); // half spacing 2^e
            // d 2^e (a normal number: d in [2^-300, 2^300]) by adding e to d's
            // exponent, and |r| < d 2^e compared as the bit patterns of two
            // non-negative doubles: integer work only
            const long long lim = __double_as_longlong(d) + ((long long)e << 52);
            if ((__double_as_longlong(fma(-q, d, x)) & 0x7fffffffffffffffLL) < lim)
                return q;
        }
    }
    return x / d;
}

// reciprocal for div_by_const, or 0 where the divisor is outside the range
// its test needs (d in [2^-300, 2^300])
static inline double div_const_recip(double d)
{
    return (d >= 0x1p-300 && d <= 0x1p300) ? 1.0 / d : 0.0;
}

// ---------------------------------------------------------------------------
// presmoothing (segmentation4D.c:352-404); d = 1 + 8c (the same rounding on
// the host), y its reciprocal for div_by_const

__global__ void k_presmooth_half(Geo g, double *v, const double *prev, double c, double d, double y, double omega,
                                 int colour)
{
    int i, j, k, l;
    if (!colour_ijkl(g, colour, i, j, k, l))
        return;
    const long long o = nat_index(g, i, j, k, l);
    double gs = div_by_const(prev[o] + c * (v[o + 1] + v[o - 1] + v[o - g.sy] + v[o + g.sy] + v[o - g.sz]
                                            + v[o + g.sz] + v[o - g.sw] + v[o + g.sw]),
                             d, y);
    v[o] = v[o] + omega * (gs - v[o]);
}

// residual passes: a thread sums RESID_K k-planes before the block reduction
#define RESID_K 4

__device__ inline bool resid_ijl(const Geo &g, int &i, int &j, int &k0, int &l)
{
    i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int nkb = (g.nz + RESID_K - 1) / RESID_K;
    k0 = 1 + (blockIdx.z % nkb) * RESID_K;
    l = 1 + blockIdx.z / nkb;
    return i <= g.nx && j <= g.ny;
}

__global__ void k_presmooth_resid(Geo g, const double *v, const double *prev, double c, double d, double h4,
                                  double *partial)
{
    int i, j, k0, l;
    double acc = 0.0;
    if (resid_ijl(g, i, j, k0, l)) {
        for (int k = k0; k < k0 + RESID_K && k <= g.nz; ++k) {
            const long long o = nat_index(g, i, j, k, l);
            double r = v[o] * d
                       - c * (v[o + 1] + v[o - 1] + v[o - g.sy] + v[o + g.sy] + v[o - g.sz] + v[o + g.sz]
                              + v[o - g.sw] + v[o + g.sw])
                       - prev[o];
            acc += (r * r) * h4;
        }
    }
    acc = block_sum2d(acc);
    if (flat_tid() == 0)
        partial[block_linear()] = acc;
}

// explicit smoother (segmentation4D.c:422-441): one Jacobi-style step from
// prev over i = 1 .. iMax-3 (the reference's x loop stops one column short)
// and the interior j, k, l; the neighbours are summed in the reference's order

__global__ void k_presmooth_explicit(Geo g, double *v, const double *prev, double coeff)
{
    int i, j, k, l;
    if (!interior_ijkl(g, i, j, k, l) || i > g.nx - 1)
        return;
    const long long o = nat_index(g, i, j, k, l);
    v[o] = (1.0 - 8.0 * coeff) * prev[o]
           + coeff * (prev[o + 1] + prev[o - 1] + prev[o + g.sy] + prev[o - g.sy] + prev[o + g.sz] + prev[o - g.sz]
                      + prev[o + g.sw] + prev[o - g.sw]);
}

// ---------------------------------------------------------------------------
// separable Gaussian along one axis (an option beside the reference's
// implicit presmoothing, which is not a Gaussian): out = sum_{m=-R..R}
// w[|m|] in(c + m) in order of m, each term added by a fused multiply-add
// (explicit fma: one rounding, the same on the host, whatever --fmad says),
// the coordinate mirrored about the volume's faces as the reference's
// reflection does (ghost 0 = voxel 1: x < 1 -> 1 - x, x > n -> 2n + 1 - x);
// interior voxels only

__device__ inline int gauss_mirror(int x, int n)
{
    // each two reflections move x by 2n towards [1, n]: |x| <= R + n needs
    // fewer than 2 R / n + 2 steps (R <= SS4D_GAUSS_MAX_RADIUS)
    for (int q = 0; q < 4 * SS4D_GAUSS_MAX_RADIUS + 4; ++q) {
        if (x < 1)
            x = 1 - x;
        else if (x > n)
            x = 2 * n + 1 - x;
        else
            break;
    }
    return x;
}

template <int AXIS>
__global__ void k_gauss_axis(Geo g, const double *__restrict__ in, double *__restrict__ out, GaussWeights W)
{
    int i, j, k, l;
    if (!interior_ijkl(g, i, j, k, l))
        return;
    const int c[4] = {i, j, k, l};
    const int n[4] = {g.nx, g.ny, g.nz, g.nt};
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    const long long o = nat_index(g, i, j, k, l);
    const long long base = o - (long long)c[AXIS] * st[AXIS];
    double acc = 0.0;
    for (int m = -W.R; m <= W.R; ++m)
        acc = fma(W.w[m < 0 ? -m : m], in[base + (long long)gauss_mirror(c[AXIS] + m, n[AXIS]) * st[AXIS]], acc);
    out[o] = acc;
}

// ---------------------------------------------------------------------------
// face gradients (segmentation4D.c:455-548, :594-821): normal component
// (v[nb]-v[c])/h, tangential ((v[nb+a]+v[c+a]) - (v[nb-a]+v[c-a]))/(4h),
// squares summed in x, y, z, w order.

__device__ inline double face_sq(const double *v, long long c, long long nb, const long long st[4], int d,
                                 double h, double q)
{
    double comp[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (a == d)
            comp[a] = (v[nb] - v[c]) / h;
        else
            comp[a] = ((v[nb + st[a]] + v[c + st[a]]) - (v[nb - st[a]] + v[c - st[a]])) / q;
    }
    return (comp[0] * comp[0]) + (comp[1] * comp[1]) + (comp[2] * comp[2]) + (comp[3] * comp[3]);
}

// face_sq of the face between o and o + st[d], in the reference's expression
// order.  POW2: h is a power of two, so x / h == x * (1/h) and x / (4h) ==
// x * (1/(4h)) exactly (one rounding of the same real number); otherwise the
// divisions by h and 4h go through div_by_const (ih, iq: its reciprocals).
template <bool POW2, int D>
__device__ inline double face_sq_plus(const double *v, long long o, const long long st[4], double h, double q,
                                      double ih, double iq)
{
    const long long nb = o + st[D];
    double comp[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (a == D) {
            const double t = v[nb] - v[o];
            comp[a] = POW2 ? t * ih : div_by_const(t, h, ih);
        } else {
            const double t = (v[nb + st[a]] + v[o + st[a]]) - (v[nb - st[a]] + v[o - st[a]]);
            comp[a] = POW2 ? t * iq : div_by_const(t, q, iq);
        }
    }
    return (comp[0] * comp[0]) + (comp[1] * comp[1]) + (comp[2] * comp[2]) + (comp[3] * comp[3]);
}

// The 8 g faces of every interior voxel, each shared face computed once.  The
// reference's value for the + face of voxel o along axis d and for the - face
// of voxel o + st[d] is the same number: the normal difference only changes
// sign (exactly) before it is squared, and the tangential sums add the same
// pairs (IEEE addition is commutative).  The thread at o computes the + face
// along d when o's other coordinates are interior, and stores it as g[2d][o]
// (o interior along d) and g[2d+1][o + st[d]] (o + st[d] interior along d).
// Threads cover coordinates 0..n along every axis.
template <bool POW2, int D>
__device__ inline void gface_plus(const Geo &g, const int c[4], const int n[4], long long o, const long long st[4],
                                  const double *i0, const double *ithr, GPtrs8 &gout, double h, double q, double ih,
                                  double iq, double K, double theta, double rho)
{
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (a != D && c[a] < 1)
            return;
    const double s0 = face_sq_plus<POW2, D>(i0, o, st, h, q, ih, iq);
    const double s1 = ithr ? face_sq_plus<POW2, D>(ithr, o, st, h, q, ih, iq) : 0.0;
    const double gv = 1.0 / (1 + K * (theta * s0 + rho * s1));
    if (c[D] >= 1)
        gout.p[2 * D][o] = gv;
    if (c[D] < n[D])
        gout.p[2 * D + 1][o + st[D]] = gv;
}

template <bool POW2>
__global__ void k_gfaces(Geo g, const double *i0, const double *ithr, GPtrs8 gout, double h, double K, double theta,
                         double rho, double ih, double iq)
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
    const double q = 4.0 * h;
    gface_plus<POW2, 0>(g, c, n, o, st, i0, ithr, gout, h, q, ih, iq, K, theta, rho);
    gface_plus<POW2, 1>(g, c, n, o, st, i0, ithr, gout, h, q, ih, iq, K, theta, rho);
    gface_plus<POW2, 2>(g, c, n, o, st, i0, ithr, gout, h, q, ih, iq, K, theta, rho);
    gface_plus<POW2, 3>(g, c, n, o, st, i0, ithr, gout, h, q, ih, iq, K, theta, rho);
}

// _gs_coefficients_ / _gs_coefficients_mcf in reference order
__global__ void k_coef_ref(Geo g, const double *u, CPtrs8 gin, int has_g, GPtrs8 coef, double h, double eps2)
{
    int i, j, k, l;
    if (!interior_ijkl(g, i, j, k, l))
        return;
    const long long o = nat_index(g, i, j, k, l);
    const long long st[4] = {1, g.sy, g.sz, g.sw};
    const double q = 4.0 * h;
    double nf[8];
#pragma unroll
    for (int f = 0; f < 8; ++f) {
        const int d = f >> 1;
        const long long nb = (f & 1) ? o - st[d] : o + st[d];
        nf[f] = sqrt(face_sq(u, o, nb, st, d, h, q) + eps2);
    }
    double mean = ((nf[0] + nf[1] + nf[2] + nf[3] + nf[4] + nf[5] + nf[6] + nf[7]) / 8.0);
    double vc = sqrt(mean * mean + eps2);
#pragma unroll
    for (int f = 0; f < 8; ++f)
        coef.p[f][o] = has_g ? vc * gin.p[f][o] * (1.0 / nf[f]) : vc * (1.0 / nf[f]);
}

// ---------------------------------------------------------------------------
// red-black SOR in reference order (segmentation4D.c:232-308)

__global__ void k_sor_half_ref(Geo g, double *u, const double *prev, CPtrs8 a, double c, double omega, int colour)
{
    int i, j, k, l;
    if (!colour_ijkl(g, colour, i, j, k, l))
        return;
    const long long o = nat_index(g, i, j, k, l);
    const double E = a.p[0][o], W = a.p[1][o], N = a.p[2][o], S = a.p[3][o];
    const double T = a.p[4][o], B = a.p[5][o], FW = a.p[6][o], BW = a.p[7][o];
    double gs = (prev[o] + c * ((E * u[o + 1]) + (W * u[o - 1]) + (S * u[o - g.sy]) + (N * u[o + g.sy])
                                + (B * u[o - g.sz]) + (T * u[o + g.sz]) + (BW * u[o - g.sw]) + (FW * u[o + g.sw])))
                / (1 + c * (E + W + N + S + T + B + FW + BW));
    u[o] = u[o] + omega * (gs - u[o]);
}

__global__ void k_sor_resid_ref(Geo g, const double *u, const double *prev, CPtrs8 a, double c, double h4,
                                double *partial)
{
    int i, j, k0, l;
    double acc = 0.0;
    if (resid_ijl(g, i, j, k0, l)) {
        for (int k = k0; k < k0 + RESID_K && k <= g.nz; ++k) {
            const long long o = nat_index(g, i, j, k, l);
            const double E = a.p[0][o], W = a.p[1][o], N = a.p[2][o], S = a.p[3][o];
            const double T = a.p[4][o], B = a.p[5][o], FW = a.p[6][o], BW = a.p[7][o];
            double r = u[o] * (1 + c * (E + W + N + S + T + B + FW + BW))
                       - c * ((E * u[o + 1]) + (W * u[o - 1]) + (S * u[o - g.sy]) + (N * u[o + g.sy])
                              + (B * u[o - g.sz]) + (T * u[o + g.sz]) + (BW * u[o - g.sw]) + (FW * u[o + g.sw]))
                       - prev[o];
            acc += (r * r) * h4;
        }
    }
    acc = block_sum2d(acc);
    if (flat_tid() == 0)
        partial[block_linear()] = acc;
}

// ---------------------------------------------------------------------------
// deterministic final reductions: one block, fixed order

// first stage of a long reduction: block b combines in[b*per, (b+1)*per)
__global__ void k_reduce_sum_part(const double *in, long long n, long long per, double *out)
{
    const long long beg = blockIdx.x * per, end = beg + per < n ? beg + per : n;
    double acc = 0.0;
    for (long long t = beg + threadIdx.x; t < end; t += blockDim.x)
        acc += in[t];
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        out[blockIdx.x] = acc;
}

__global__ void k_reduce_sum(const double *partial, long long n, double *out)
{
    double acc = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x)
        acc += partial[t];
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        *out = acc;
}

// partial holds n (min, max) pairs; out[0] = min, out[1] = max,
// out[2] = min + level*(max-min)
__global__ void k_reduce_minmax(const double *partial, long long n, double level, double *out)
{
    double mn = 1e308, mx = -1e308;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
        mn = fmin(mn, partial[2 * t]);
        mx = fmax(mx, partial[2 * t + 1]);
    }
    mn = block_min(mn);
    mx = block_max(mx);
    if (threadIdx.x == 0) {
        out[0] = mn;
        out[1] = mx;
        out[2] = mn + level * (mx - mn);
    }
}

// ---------------------------------------------------------------------------
// norms over every padded voxel (segmentation4D.c:194-213, :317-335)

__global__ void k_l2_partial(long long n, const double *a, const double *b, double h4, double *partial)
{
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        double d = a[t] - b[t];
        acc += (d * d) * h4;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = acc;
}

__global__ void k_mass_partial(long long n, const double *a, double h4, double *partial)
{
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        acc += (a[t] * h4);
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = acc;
}

// ---------------------------------------------------------------------------
// MCF exact solution and Dirichlet ghosts (mcf_4D.c:344-461)

__device__ inline double mcf_coord(int i, double h)
{
    return ((i - 1) * h) + (h / 2.) - 1.25;
}

__device__ inline double mcf_value(double x, double y, double z, double w, double t)
{
    return ((x * x + y * y + z * z + w * w - 1.0) / 6.0) + t;
}

__global__ void k_mcf_field(Geo g, double *u, double h, double t, int ghosts_only)
{
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < g.n; o += (long long)gridDim.x * blockDim.x) {
        long long r = o;
        const int i = (int)(r % g.iM); r /= g.iM;
        const int j = (int)(r % g.jM); r /= g.jM;
        const int k = (int)(r % g.kM);
        const int l = (int)(r / g.kM);
        const int idx[4] = {i, j, k, l};
        const int M[4] = {g.iM, g.jM, g.kM, g.lM};
        double x[4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
            x[a] = mcf_coord(idx[a], h);
        if (ghosts_only) {
            // the reference's eight passes run x-lo, x-hi, ..., w-hi over full
            // ranges: the last pass touching a ghost decides its value, and it
            // uses the special face coordinate on its own axis only.
            int last = -1;
#pragma unroll
            for (int a = 0; a < 4; ++a)
                if (idx[a] == 0 || idx[a] == M[a] - 1)
                    last = a;
            if (last < 0)
                continue;
            x[last] = idx[last] == M[last] - 1 ? (h / 2.) + 1.25 : -(h / 2.) - 1.25;
            if (M[last] == 1)
                x[last] = (h / 2.) + 1.25;
        }
        u[o] = mcf_value(x[0], x[1], x[2], x[3], t);
    }
}

// ---------------------------------------------------------------------------
// rescale to [0,1] per ball (segmentation4D.c:1020-1104): one block per
// frame; the balls of a frame are processed in their order because each
// ball's min/max sees the values the earlier balls rescaled.

__global__ void k_rescale_balls(Geo g, double *v, const int *frame_first, const int *frame_count, const double *bx,
                                const double *by, const double *bz, double R, int l0)
{
    const int l = l0 + blockIdx.x;
    const int first = frame_first[l], count = frame_count[l];
    for (int c = 0; c < count; ++c) {
        const double cx = bx[first + c], cy = by[first + c], cz = bz[first + c];
        const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
        const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
        const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
        const int ni = i1 - i0 + 1, nj = j1 - j0 + 1, nk = k1 - k0 + 1;
        const long long cnt = (long long)ni * nj * nk;
        double mn = 100000, mx = 0;
        for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int i = i0 + (int)(t % ni), j = j0 + (int)((t / ni) % nj), k = k0 + (int)(t / ((long long)ni * nj));
            const double dx = i - cx, dy = j - cy, dz = k - cz;
            if (sqrt((dx * dx) + (dy * dy) + (dz * dz)) <= R) {
                const double val = v[nat_index(g, i, j, k, l)];
                mn = val < mn ? val : mn;
                mx = val > mx ? val : mx;
            }
        }
        mn = block_min(mn);
        mx = block_max(mx);
        __shared__ double qo[2];
        if (threadIdx.x == 0) {
            // ball values never exceed the reference's starting bounds in a
            // meaningful run; keep its initial values 100000 / 0 exactly
            const double lo = mn < 100000 ? mn : 100000, hi = mx > 0 ? mx : 0;
            const double quot = 1. / (hi - lo);
            qo[0] = quot;
            qo[1] = lo * quot;
        }
        __syncthreads();
        const double quot = qo[0], off = qo[1];
        for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int i = i0 + (int)(t % ni), j = j0 + (int)((t / ni) % nj), k = k0 + (int)(t / ((long long)ni * nj));
            const double dx = i - cx, dy = j - cy, dz = k - cz;
            if (sqrt((dx * dx) + (dy * dy) + (dz * dz)) <= R) {
                const long long o = nat_index(g, i, j, k, l);
                const double nv = (quot * v[o]) - off;
                if (c == 0 || v[o] < nv)
                    v[o] = nv;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// initial segmentation (segmentation4D.c:876-1018, 1106-1147).  One block per
// frame walks that frame's balls in order, as k_rescale_balls does.

// minimum (from 100000) and maximum (from 0) of frame l inside the ball of
// radius R: _get3DMinWithinR_ / _get3DMaxWithinR_ (segmentation4D.c:897-969);
// the results in every thread
__device__ void ball_min_max(const Geo &g, const double *v, int l, double cx, double cy, double cz, double R,
                             double &mn_out, double &mx_out)
{
    const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
    const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
    const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
    const int ni = i1 - i0 + 1, nj = j1 - j0 + 1, nk = k1 - k0 + 1;
    const long long cnt = (long long)ni * nj * nk;
    double mn = 100000, mx = 0;
    for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
        const int i = i0 + (int)(t % ni), j = j0 + (int)((t / ni) % nj), k = k0 + (int)(t / ((long long)ni * nj));
        const double dx = i - cx, dy = j - cy, dz = k - cz;
        if (sqrt((dx * dx) + (dy * dy) + (dz * dz)) <= R) {
            const double val = v[nat_index(g, i, j, k, l)];
            mn = val < mn ? val : mn;
            mx = val > mx ? val : mx;
        }
    }
    mn = block_min(mn);
    mx = block_max(mx);
    __shared__ double r2[2];
    if (threadIdx.x == 0) {
        r2[0] = mn;
        r2[1] = mx;
    }
    __syncthreads();
    mn_out = r2[0];
    mx_out = r2[1];
    __syncthreads();
}

__global__ void k_ball_min_max(Geo g, const double *v, int l, double cx, double cy, double cz, double R, double *out)
{
    double mn, mx;
    ball_min_max(g, v, l, cx, cy, cz, R, mn, mx);
    if (threadIdx.x == 0) {
        out[0] = mn;
        out[1] = mx;
    }
}

// _locallyThreshold4Ddata_ (segmentation4D.c:971-1018): per ball the level
// alpha min + beta max of the input inside it; thr = the global maximum
// (from 0, _get4DMax_) wherever the input inside the ball exceeds it
__global__ void k_local_threshold(Geo g, const double *in, double *thr, const int *frame_first, const int *frame_count,
                                  const double *bx, const double *by, const double *bz, double R, double alpha,
                                  double beta, const double *minmax)
{
    const int l = 1 + blockIdx.x;
    const double gmax = minmax[1] > 0 ? minmax[1] : 0;
    const int first = frame_first[l], count = frame_count[l];
    for (int c = 0; c < count; ++c) {
        const double cx = bx[first + c], cy = by[first + c], cz = bz[first + c];
        double mn, mx;
        ball_min_max(g, in, l, cx, cy, cz, R, mn, mx);
        const double level = alpha * mn + beta * mx;
        const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
        const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
        const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
        const int ni = i1 - i0 + 1, nj = j1 - j0 + 1, nk = k1 - k0 + 1;
        const long long cnt = (long long)ni * nj * nk;
        for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int i = i0 + (int)(t % ni), j = j0 + (int)((t / ni) % nj), k = k0 + (int)(t / ((long long)ni * nj));
            const double dx = i - cx, dy = j - cy, dz = k - cz;
            if (sqrt((dx * dx) + (dy * dy) + (dz * dz)) <= R) {
                const long long o = nat_index(g, i, j, k, l);
                if (in[o] > level)
                    thr[o] = gmax;
            }
        }
    }
}

// _generate4DsegmFunct_ (segmentation4D.c:1106-1147): in each ball's box
// (half-width R + 0.5) and within the fixed distance 12 of its centre,
// u = max(u, |1/(r + 0.5) - 1/12.5|) and Mmask = 1; balls in order
__global__ void k_generate_segm(Geo g, double *u, double *Mmask, const int *frame_first, const int *frame_count,
                                const double *bx, const double *by, const double *bz, double R)
{
    const int l = 1 + blockIdx.x;
    const double v = 0.5, Rf = 12.;
    const int first = frame_first[l], count = frame_count[l];
    for (int c = 0; c < count; ++c) {
        const double cx = bx[first + c], cy = by[first + c], cz = bz[first + c];
        const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
        const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
        const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
        const int ni = i1 - i0 + 1, nj = j1 - j0 + 1, nk = k1 - k0 + 1;
        const long long cnt = (long long)ni * nj * nk;
        for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int i = i0 + (int)(t % ni), j = j0 + (int)((t / ni) % nj), k = k0 + (int)(t / ((long long)ni * nj));
            const double dx = i - cx, dy = j - cy, dz = k - cz;
            if (sqrt((dx * dx) + (dy * dy) + (dz * dz)) <= Rf) {
                const double nv = fabs((1. / (sqrt((dx * dx) + (dy * dy) + (dz * dz)) + v)) - (1. / (Rf + v)));
                const long long o = nat_index(g, i, j, k, l);
                if (u[o] < nv)
                    u[o] = nv;
                Mmask[o] = 1.;
            }
        }
        __syncthreads(); // the next ball may cover the same voxels
    }
}

// ---------------------------------------------------------------------------
// one frame's interior <-> the bytes of its file (x fastest, then y, z):
// _load3dDataArrayVTK_ (segmentation4D.c:1317-1320), _writeData_ (:1250-1254),
// _writeData_mpi_ (segmentation4D_mpi.c:1466-1473)

// byte / 255. from a table of the 256 quotients (the same IEEE divisions),
// built once per block; a block walks FRAME_Z_PER_BLOCK planes
#define FRAME_Z_PER_BLOCK 32
__global__ void k_frame_from_bytes(Geo g, double *img, int l, const uint8_t *__restrict__ bytes)
{
    __shared__ double lut[256];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if (t < 256)
        lut[t] = t / 255.;
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= g.nx || y >= g.ny)
        return;
    for (int z = blockIdx.z; z < g.nz; z += gridDim.z) {
        const long long q = ((long long)z * g.ny + y) * g.nx + x;
        img[nat_index(g, x + 1, y + 1, z + 1, l)] = lut[bytes[q]];
    }
}

// mode 0: (unsigned char)(255 v + 0.5), clamped to [0, 255] (the reference's
// conversion is undefined outside); mode 1: 1 where v >= 0.5, else 0
__global__ void k_frame_to_bytes(Geo g, const double *img, int l, int mode, uint8_t *__restrict__ bytes)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.nx || y >= g.ny)
        return;
    const long long q = ((long long)z * g.ny + y) * g.nx + x;
    const double v = img[nat_index(g, x + 1, y + 1, z + 1, l)];
    uint8_t out;
    if (mode == 1) {
        out = v >= 0.5 ? 1 : 0;
    } else {
        const double w = 255 * v + 0.5;
        out = w >= 255. ? 255 : (w > 0. ? (uint8_t)(int)w : 0);
    }
    bytes[q] = out;
}

__global__ void k_mask_zero(Geo g, double *v, const double *Mmask, int l_off)
{
    int i, j, k, l;
    if (!interior_ijkl(g, i, j, k, l))
        return;
    l += l_off;
    const long long o = nat_index(g, i, j, k, l);
    if (Mmask[o] == 0)
        v[o] = 0;
}

// ---------------------------------------------------------------------------
// threshold to mask (segmentation4D_mpi.c:1470-1478)

// ordered 64-bit keys of doubles: a signed comparison of two keys compares the
// numbers (-0 below +0); the map is its own inverse.  NaN is skipped.
__device__ inline long long dkey(long long b)
{
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

#define MINMAX_BLOCKS 2048
// interior min and max of u per block, as (min, max) pairs in partial; a
// block walks whole rows (threads along x), comparing integer keys so the
// FP64 pipe is not used; a block without a number reports (1e308, -1e308)
__global__ void k_minmax_partial(Geo g, const double *u, double *partial)
{
    long long mn = 0x7fffffffffffffffLL, mx = -0x7fffffffffffffffLL - 1;
    const int rows = g.ny * g.nz * g.nt;
    for (int r = blockIdx.x * blockDim.y + threadIdx.y; r < rows; r += gridDim.x * blockDim.y) {
        const int j = r % g.ny, kl = r / g.ny;
        const long long base = nat_index(g, 0, j + 1, 1 + kl % g.nz, 1 + kl / g.nz);
        for (int i = 1 + threadIdx.x; i <= g.nx; i += blockDim.x) {
            const long long b = __double_as_longlong(u[base + i]);
            if ((b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL) {
                const long long key = dkey(b);
                mn = key < mn ? key : mn;
                mx = key > mx ? key : mx;
            }
        }
    }
    __shared__ long long smn[32], smx[32];
    const int t = flat_tid(), lane = t & 31, wid = t >> 5, nw = (blockDim.x * blockDim.y + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long a = __shfl_down_sync(0xffffffffu, mn, o), b = __shfl_down_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    if (lane == 0) {
        smn[wid] = mn;
        smx[wid] = mx;
    }
    __syncthreads();
    if (wid == 0) {
        mn = lane < nw ? smn[lane] : 0x7fffffffffffffffLL;
        mx = lane < nw ? smx[lane] : -0x7fffffffffffffffLL - 1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long a = __shfl_down_sync(0xffffffffu, mn, o), b = __shfl_down_sync(0xffffffffu, mx, o);
            mn = a < mn ? a : mn;
            mx = b > mx ? b : mx;
        }
        if (lane == 0) {
            const bool none = mn == 0x7fffffffffffffffLL;
            partial[2 * blockIdx.x] = none ? 1e308 : __longlong_as_double(dkey(mn));
            partial[2 * blockIdx.x + 1] = none ? -1e308 : __longlong_as_double(dkey(mx));
        }
    }
}

__global__ void k_threshold(Geo g, const double *u, const double *level_dev, double level, uint8_t *mask)
{
    int i, j, k, l;
    if (!interior_ijkl(g, i, j, k, l))
        return;
    const double lev = level_dev ? level_dev[2] : level;
    const long long m = ((((long long)(l - 1) * g.nz + (k - 1)) * g.ny + (j - 1)) * g.nx) + (i - 1);
    mask[m] = u[nat_index(g, i, j, k, l)] >= lev ? 1 : 0;
}

// ---------------------------------------------------------------------------
// host-side launch wrappers

static inline void interior_cfg(const Geo &g, dim3 &grid, dim3 &block)
{
    const int bx = g.nx >= 128 ? 128 : (g.nx >= 64 ? 64 : 32);
    const int by = 256 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((g.nx + bx - 1) / bx, (g.ny + by - 1) / by, g.nz * g.nt);
}

long long interior_blocks(const Geo &g)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    return (long long)gr.x * gr.y * gr.z;
}

void launch_reflect(const Geo &g, double *u, cudaStream_t st)
{
    for (int a = 0; a < 4; ++a)
        k_reflect_axis<<<256, 256, 0, st>>>(g, u, a);
}

// one colour: ceil(nx/2) threads along a row
static inline void colour_cfg(const Geo &g, dim3 &grid, dim3 &block)
{
    const int nxh = (g.nx + 1) / 2;
    const int bx = nxh >= 128 ? 128 : (nxh >= 64 ? 64 : 32);
    const int by = 256 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((nxh + bx - 1) / bx, (g.ny + by - 1) / by, g.nz * g.nt);
}

void launch_presmooth_half(const Geo &g, double *v, const double *prev, double c, double omega, int colour,
                           cudaStream_t st)
{
    dim3 gr, bl;
    colour_cfg(g, gr, bl);
    const double d = 1 + c * 8;
    k_presmooth_half<<<gr, bl, 0, st>>>(g, v, prev, c, d, div_const_recip(d), omega, colour);
}

static inline void resid_cfg(const Geo &g, dim3 &grid, dim3 &block)
{
    interior_cfg(g, grid, block);
    grid.z = ((g.nz + RESID_K - 1) / RESID_K) * g.nt;
}

long long resid_blocks(const Geo &g)
{
    dim3 gr, bl;
    resid_cfg(g, gr, bl);
    return (long long)gr.x * gr.y * gr.z;
}

void launch_presmooth_resid(const Geo &g, const double *v, const double *prev, double c, double h4, double *partial,
                            cudaStream_t st)
{
    dim3 gr, bl;
    resid_cfg(g, gr, bl);
    k_presmooth_resid<<<gr, bl, 0, st>>>(g, v, prev, c, 1 + c * 8, h4, partial);
}

void launch_gauss_axis(const Geo &g, int axis, const double *in, double *out, const GaussWeights &W,
                       cudaStream_t st)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    if (axis == 0)
        k_gauss_axis<0><<<gr, bl, 0, st>>>(g, in, out, W);
    else if (axis == 1)
        k_gauss_axis<1><<<gr, bl, 0, st>>>(g, in, out, W);
    else if (axis == 2)
        k_gauss_axis<2><<<gr, bl, 0, st>>>(g, in, out, W);
    else
        k_gauss_axis<3><<<gr, bl, 0, st>>>(g, in, out, W);
}

void launch_presmooth_explicit(const Geo &g, double *v, const double *prev, double coeff, cudaStream_t st)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    k_presmooth_explicit<<<gr, bl, 0, st>>>(g, v, prev, coeff);
}

void launch_gfaces(const Geo &g, const double *i0, const double *ithr, GPtrs8 gout, double h, double K, double theta,
                   double rho, cudaStream_t st)
{
    const int bx = g.nx + 1 >= 128 ? 128 : (g.nx + 1 >= 64 ? 64 : 32);
    const int by = 256 / bx;
    dim3 bl(bx, by, 1), gr((g.nx + 1 + bx - 1) / bx, (g.ny + 1 + by - 1) / by, (g.nz + 1) * (g.nt + 1));
    int e = 0;
    const double m = frexp(h, &e);
    const double ih = 1.0 / h, iq = 1.0 / (4.0 * h);
    // a power of two whose reciprocals are normal numbers
    if (m == 0.5 && ih * h == 1.0 && iq * (4.0 * h) == 1.0 && isnormal(ih) && isnormal(iq) && isnormal(4.0 * h))
        k_gfaces<true><<<gr, bl, 0, st>>>(g, i0, ithr, gout, h, K, theta, rho, ih, iq);
    else
        k_gfaces<false><<<gr, bl, 0, st>>>(g, i0, ithr, gout, h, K, theta, rho, div_const_recip(h),
                                           div_const_recip(4.0 * h));
}

void launch_coef_ref(const Geo &g, const double *u, CPtrs8 gin, int has_g, GPtrs8 coef, double h, double eps2,
                     cudaStream_t st)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    k_coef_ref<<<gr, bl, 0, st>>>(g, u, gin, has_g, coef, h, eps2);
}

void launch_sor_half_ref(const Geo &g, double *u, const double *prev, CPtrs8 a, double c, double omega, int colour,
                         cudaStream_t st)
{
    dim3 gr, bl;
    colour_cfg(g, gr, bl);
    k_sor_half_ref<<<gr, bl, 0, st>>>(g, u, prev, a, c, omega, colour);
}

void launch_sor_resid_ref(const Geo &g, const double *u, const double *prev, CPtrs8 a, double c, double h4,
                          double *partial, cudaStream_t st)
{
    dim3 gr, bl;
    resid_cfg(g, gr, bl);
    k_sor_resid_ref<<<gr, bl, 0, st>>>(g, u, prev, a, c, h4, partial);
}

// n partials: one block when n is small; else up to 1024 blocks first, their
// results written behind the partials (partial[n ..]), then one block.
// Returns the number of launches.
static long long reduce_split(long long n, long long &per)
{
    per = 4096;
    long long nb = (n + per - 1) / per;
    if (nb > 1024) {
        per = (n + 1023) / 1024;
        nb = (n + per - 1) / per;
    }
    return nb;
}

int launch_reduce_sum(double *partial, long long n, double *out, cudaStream_t st)
{
    if (n <= 16384) {
        k_reduce_sum<<<1, 1024, 0, st>>>(partial, n, out);
        return 1;
    }
    long long per;
    const long long nb = reduce_split(n, per);
    k_reduce_sum_part<<<(unsigned)nb, 256, 0, st>>>(partial, n, per, partial + n);
    k_reduce_sum<<<1, 1024, 0, st>>>(partial + n, nb, out);
    return 2;
}

void launch_l2(const Geo &g, const double *a, const double *b, double h4, double *partial, int nblk, cudaStream_t st)
{
    k_l2_partial<<<nblk, 256, 0, st>>>(g.n, a, b, h4, partial);
}

void launch_mass(const Geo &g, const double *a, double h4, double *partial, int nblk, cudaStream_t st)
{
    k_mass_partial<<<nblk, 256, 0, st>>>(g.n, a, h4, partial);
}

void launch_mcf_field(const Geo &g, double *u, double h, double t, int ghosts_only, cudaStream_t st)
{
    k_mcf_field<<<1024, 256, 0, st>>>(g, u, h, t, ghosts_only);
}

void launch_rescale_balls(const Geo &g, double *v, const int *frame_first, const int *frame_count, const double *bx,
                          const double *by, const double *bz, double R, cudaStream_t st)
{
    launch_rescale_balls_range(g, v, frame_first, frame_count, bx, by, bz, R, 1, g.lM - 1, st);
}

void launch_rescale_balls_range(const Geo &g, double *v, const int *frame_first, const int *frame_count,
                                const double *bx, const double *by, const double *bz, double R, int l0, int l1,
                                cudaStream_t st)
{
    k_rescale_balls<<<l1 - l0, 256, 0, st>>>(g, v, frame_first, frame_count, bx, by, bz, R, l0);
}

void launch_mask_zero(const Geo &g, double *v, const double *Mmask, cudaStream_t st)
{
    launch_mask_zero_range(g, v, Mmask, 1, g.lM - 1, st);
}

void launch_mask_zero_range(const Geo &g, double *v, const double *Mmask, int l0, int l1, cudaStream_t st)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    gr.z = g.nz * (l1 - l0);
    k_mask_zero<<<gr, bl, 0, st>>>(g, v, Mmask, l0 - 1);
}

void launch_ball_min_max(const Geo &g, const double *v, int l, double cx, double cy, double cz, double R, double *out2,
                         cudaStream_t st)
{
    k_ball_min_max<<<1, 256, 0, st>>>(g, v, l, cx, cy, cz, R, out2);
}

void launch_local_threshold(const Geo &g, const double *in, double *thr, const int *frame_first, const int *frame_count,
                            const double *bx, const double *by, const double *bz, double R, double alpha, double beta,
                            const double *minmax, cudaStream_t st)
{
    k_local_threshold<<<g.nt, 256, 0, st>>>(g, in, thr, frame_first, frame_count, bx, by, bz, R, alpha, beta, minmax);
}

void launch_generate_segm(const Geo &g, double *u, double *Mmask, const int *frame_first, const int *frame_count,
                          const double *bx, const double *by, const double *bz, double R, cudaStream_t st)
{
    k_generate_segm<<<g.nt, 256, 0, st>>>(g, u, Mmask, frame_first, frame_count, bx, by, bz, R);
}

void launch_frame_bytes(const Geo &g, double *img_out, const double *img_in, int l, int mode, const uint8_t *bytes_in,
                        uint8_t *bytes_out, cudaStream_t st)
{
    const int bx = g.nx >= 128 ? 128 : (g.nx >= 64 ? 64 : 32);
    dim3 bl(bx, 256 / bx, 1), gr((g.nx + bx - 1) / bx, (g.ny + 256 / bx - 1) / (256 / bx), g.nz);
    if (img_out) {
        gr.z = (g.nz + FRAME_Z_PER_BLOCK - 1) / FRAME_Z_PER_BLOCK;
        k_frame_from_bytes<<<gr, bl, 0, st>>>(g, img_out, l, bytes_in);
    } else {
        k_frame_to_bytes<<<gr, bl, 0, st>>>(g, img_in, l, mode, bytes_out);
    }
}

int launch_minmax(const Geo &g, const double *u, double *partial, double level, double *out3, cudaStream_t st)
{
    const long long rows = (long long)g.ny * g.nz * g.nt;
    const int nb = (int)(rows / 2 < MINMAX_BLOCKS ? (rows + 1) / 2 : MINMAX_BLOCKS);
    k_minmax_partial<<<nb, dim3(128, 2, 1), 0, st>>>(g, u, partial);
    k_reduce_minmax<<<1, 1024, 0, st>>>(partial, nb, level, out3);
    return 2;
}

void launch_threshold(const Geo &g, const double *u, const double *level_dev, double level, uint8_t *mask,
                      cudaStream_t st)
{
    dim3 gr, bl;
    interior_cfg(g, gr, bl);
    k_threshold<<<gr, bl, 0, st>>>(g, u, level_dev, level, mask);
}

} // namespace ss4d
