/*
 * ss4d_oracle.c — TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement, in plain C99, of the reference's semi-implicit
 * subjective-surfaces / mean-curvature-flow path (segmentation4D.c and
 * mcf_4D.c of 88MARK08/4D-image-segmentation-algorithm).  It is the checker
 * the CUDA path is compared with; nothing in the product links or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Parity pin: tests/test_oracle_golden.py checks every function here against
 * fixtures produced by the reference itself (compiled from its own sources by
 * oracle/Makefile into oracle/_ref/, fixtures generated by
 * tests/golden/make_golden.py).  To be bit-comparable with the reference this
 * file keeps the reference's evaluation order in every floating-point
 * expression and calls pow() where the reference calls pow(); it must be built
 * with -ffp-contract=off so that no compiler fuses a multiply and an add that
 * the x86 reference build rounds separately.
 *
 * Differences from the reference, none of which change a result:
 *  - state is passed explicitly (dims, params, arrays) instead of globals;
 *  - loops over frames carry OpenMP pragmas in the manner of mcf_4D_openmp.c
 *    (parallel over l, reduction of the residual); with one thread the
 *    summation order is the reference's serial order;
 *  - the ball loops of the rescale refuse centres whose box leaves the array
 *    (the reference reads out of bounds there, segmentation4D.c:1043-1045).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/ss4d.h"

/* ---------------------------------------------------------------------- */
/* layout                                                                   */

typedef struct {
    int iM, jM, kM, lM;
    ptrdiff_t sx, sy, sz, sw; /* strides of i, j, k, l */
    ptrdiff_t n;              /* padded voxel count   */
} geo_t;

static geo_t geo_of(const ss4d_dims *d)
{
    geo_t g;
    g.iM = d->iMax; g.jM = d->jMax; g.kM = d->kMax; g.lM = d->lMax;
    g.sx = 1;
    g.sy = g.iM;
    g.sz = (ptrdiff_t)g.iM * g.jM;
    g.sw = g.sz * g.kM;
    g.n = g.sw * g.lM;
    return g;
}

/* ijkl() of segmentation4D.c:61-65 */
static inline ptrdiff_t at(const geo_t *g, int i, int j, int k, int l)
{
    return (((ptrdiff_t)l * g->kM + k) * g->jM + j) * g->iM + i;
}

static int g_threads = 1;

void or_set_threads(int n)
{
    g_threads = n > 0 ? n : 1;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}

int or_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

/* _copy4DdataFromSrcToDest_ (segmentation4D.c:866-874) */
void or_copy(const ss4d_dims *d, const double *src, double *dst)
{
    geo_t g = geo_of(d);
    memcpy(dst, src, sizeof(double) * (size_t)g.n);
}

/* ---------------------------------------------------------------------- */
/* face gradients                                                           */

/*
 * |grad v|^2 on the face between voxel c and its neighbour nb = c + st[d]
 * (or c - st[d]) along axis d, as written out face by face in
 * segmentation4D.c:455-548 and :594-821: the normal component is the
 * one-sided difference (v[nb] - v[c]) / h, every tangential component a
 * is ((v[nb+a] + v[c+a]) - (v[nb-a] + v[c-a])) / (4h), and the four squares
 * are summed in x, y, z, w order.  The reference writes some tangential sums
 * as (v[c+a] + v[nb+a]); IEEE addition commutes, so the bits agree.
 */
static inline double face_sq(const double *v, ptrdiff_t c, ptrdiff_t nb, const ptrdiff_t st[4],
                             int d, double h, double q)
{
    double comp[4];
    for (int a = 0; a < 4; ++a) {
        if (a == d)
            comp[a] = (v[nb] - v[c]) / h;
        else
            comp[a] = ((v[nb + st[a]] + v[c + st[a]]) - (v[nb - st[a]] + v[c - st[a]])) / q;
    }
    return (comp[0] * comp[0]) + (comp[1] * comp[1]) + (comp[2] * comp[2]) + (comp[3] * comp[3]);
}

/* Face order of the reference's coefficient arrays: e, w, n, s, t, b, fw, bw
 * = (+x, -x, +y, -y, +z, -z, +w, -w). */
static const int face_axis[8] = {0, 0, 1, 1, 2, 2, 3, 3};
static const int face_sign[8] = {+1, -1, +1, -1, +1, -1, +1, -1};

/* ---------------------------------------------------------------------- */
/* boundary                                                                 */

/* _reflection4Ddata_ (segmentation4D.c:826-864): copy the first/last interior
 * layer into the ghost layer, axis by axis in x, y, z, w order over the full
 * padded ranges (so edge and corner ghosts take the value of the last axis). */
void or_reflect(const ss4d_dims *d, double *u)
{
    geo_t g = geo_of(d);
    int i, j, k, l;
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (j = 0; j < g.jM; j++) {
                u[at(&g, 0, j, k, l)] = u[at(&g, 1, j, k, l)];
                u[at(&g, g.iM - 1, j, k, l)] = u[at(&g, g.iM - 2, j, k, l)];
            }
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (i = 0; i < g.iM; i++) {
                u[at(&g, i, 0, k, l)] = u[at(&g, i, 1, k, l)];
                u[at(&g, i, g.jM - 1, k, l)] = u[at(&g, i, g.jM - 2, k, l)];
            }
    for (l = 0; l < g.lM; l++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++) {
                u[at(&g, i, j, 0, l)] = u[at(&g, i, j, 1, l)];
                u[at(&g, i, j, g.kM - 1, l)] = u[at(&g, i, j, g.kM - 2, l)];
            }
    for (k = 0; k < g.kM; k++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++) {
                u[at(&g, i, j, k, 0)] = u[at(&g, i, j, k, 1)];
                u[at(&g, i, j, k, g.lM - 1)] = u[at(&g, i, j, k, g.lM - 2)];
            }
}

/* Cell-centre coordinate of index i on [-1.25, 1.25] (mcf_4D.c:453-456). */
static inline double mcf_coord(int i, double h)
{
    return ((i - 1) * h) + (h / 2.) - 1.25;
}

static inline double mcf_value(double x, double y, double z, double w, double t)
{
    return ((x * x + y * y + z * z + w * w - 1.0) / 6.0) + t;
}

/* _exactSolution_mcf (mcf_4D.c:444-461) */
void or_mcf_exact_solution(const ss4d_dims *d, double h, double t, double *out)
{
    geo_t g = geo_of(d);
    int l;
#pragma omp parallel for schedule(static)
    for (l = 0; l < g.lM; l++)
        for (int k = 0; k < g.kM; k++)
            for (int j = 0; j < g.jM; j++)
                for (int i = 0; i < g.iM; i++)
                    out[at(&g, i, j, k, l)] = mcf_value(mcf_coord(i, h), mcf_coord(j, h),
                                                        mcf_coord(k, h), mcf_coord(l, h), t);
}

/* _set4DBoundaryToExactValues_mcf (mcf_4D.c:344-443): eight passes, low then
 * high ghost face of x, y, z, w, each over the full padded range of the other
 * axes.  On its own axis a pass uses -(h/2)-1.25 or (h/2)+1.25; the other
 * coordinates follow mcf_coord.  Later passes overwrite edges and corners. */
void or_mcf_set_boundary(const ss4d_dims *d, double h, double t, double *u)
{
    geo_t g = geo_of(d);
    const double lo = -(h / 2.) - 1.25, hi = (h / 2.) + 1.25;
    int i, j, k, l;
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (j = 0; j < g.jM; j++)
                u[at(&g, 0, j, k, l)] = mcf_value(lo, mcf_coord(j, h), mcf_coord(k, h), mcf_coord(l, h), t);
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (j = 0; j < g.jM; j++)
                u[at(&g, g.iM - 1, j, k, l)] = mcf_value(hi, mcf_coord(j, h), mcf_coord(k, h), mcf_coord(l, h), t);
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, 0, k, l)] = mcf_value(mcf_coord(i, h), lo, mcf_coord(k, h), mcf_coord(l, h), t);
    for (l = 0; l < g.lM; l++)
        for (k = 0; k < g.kM; k++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, g.jM - 1, k, l)] = mcf_value(mcf_coord(i, h), hi, mcf_coord(k, h), mcf_coord(l, h), t);
    for (l = 0; l < g.lM; l++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, j, 0, l)] = mcf_value(mcf_coord(i, h), mcf_coord(j, h), lo, mcf_coord(l, h), t);
    for (l = 0; l < g.lM; l++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, j, g.kM - 1, l)] = mcf_value(mcf_coord(i, h), mcf_coord(j, h), hi, mcf_coord(l, h), t);
    for (k = 0; k < g.kM; k++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, j, k, 0)] = mcf_value(mcf_coord(i, h), mcf_coord(j, h), mcf_coord(k, h), lo, t);
    for (k = 0; k < g.kM; k++)
        for (j = 0; j < g.jM; j++)
            for (i = 0; i < g.iM; i++)
                u[at(&g, i, j, k, g.lM - 1)] = mcf_value(mcf_coord(i, h), mcf_coord(j, h), mcf_coord(k, h), hi, t);
}

/* ---------------------------------------------------------------------- */
/* presmoothing: constant-coefficient implicit heat step                    */

/* _presmoothStep_ (segmentation4D.c:337-409).  scratch plays the reference's
 * global prev_u.  Returns the iteration count; *res receives the last
 * sum r^2 h^4. */
int or_presmooth(const ss4d_dims *d, const ss4d_params *p, double *v, double *scratch, double *res)
{
    geo_t g = geo_of(d);
    const double c = p->sigma / (p->h * p->h);
    const double h4 = p->h * p->h * p->h * p->h;
    const ptrdiff_t sx = g.sx, sy = g.sy, sz = g.sz, sw = g.sw;
    double R = 0.0;
    int z = 0, l;

    or_copy(d, v, scratch);
    or_reflect(d, v);
    do {
        z = z + 1;
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (l = 1; l <= g.lM - 2; l++)
                for (int k = 1; k <= g.kM - 2; k++)
                    for (int j = 1; j <= g.jM - 2; j++)
                        for (int i = 1; i <= g.iM - 2; i++) {
                            if ((i + j + k + l) % 2 != colour)
                                continue;
                            ptrdiff_t o = at(&g, i, j, k, l);
                            double gs = (scratch[o] + c * (v[o + sx] + v[o - sx] + v[o - sy] + v[o + sy]
                                                           + v[o - sz] + v[o + sz] + v[o - sw] + v[o + sw]))
                                        / (1 + c * 8);
                            v[o] = v[o] + p->omega_sigma * (gs - v[o]);
                        }
        }
        R = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : R)
        for (l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i <= g.iM - 2; i++) {
                        ptrdiff_t o = at(&g, i, j, k, l);
                        R += (pow(v[o] * (1 + c * 8) - c * (v[o + sx] + v[o - sx] + v[o - sy] + v[o + sy]
                                                            + v[o - sz] + v[o + sz] + v[o - sw] + v[o + sw])
                                      - scratch[o], 2) * h4);
                    }
    } while (R > p->gsTol && z < p->maxNoGSIteration_sigma);
    if (res)
        *res = R;
    return z;
}

/* _presmoothStepEXP_ (segmentation4D.c:410-444), the explicit smoother the
 * reference declares but its main never calls: scratch (the reference's
 * prev_u) <- v, reflect v, then `steps` times: v <- (1 - 8c) prev + c * (sum
 * of the 8 neighbours of prev, in the order i+1, i-1, j+1, j-1, k+1, k-1,
 * l+1, l-1) over i = 1 .. iMax-3 (the reference's loop stops one short of the
 * last interior column) and the interior j, k, l, and reflect v.  prev is
 * not refreshed between the steps, as in the reference. */
void or_presmooth_explicit(const ss4d_dims *d, const ss4d_params *p, int steps, double *v, double *scratch)
{
    geo_t g = geo_of(d);
    const double coeff = p->sigma / (p->h * p->h);
    const ptrdiff_t sx = g.sx, sy = g.sy, sz = g.sz, sw = g.sw;
    int l;
    or_copy(d, v, scratch);
    or_reflect(d, v);
    for (int t = 0; t < steps; t++) {
#pragma omp parallel for schedule(static)
        for (l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i < g.iM - 2; i++) {
                        ptrdiff_t o = at(&g, i, j, k, l);
                        v[o] = (1.0 - 8.0 * coeff) * scratch[o]
                               + coeff * (scratch[o + sx] + scratch[o - sx] + scratch[o + sy] + scratch[o - sy]
                                          + scratch[o + sz] + scratch[o - sz] + scratch[o + sw] + scratch[o - sw]);
                    }
        or_reflect(d, v);
    }
}

/* A true Gaussian beside the reference's implicit presmoothing (no
 * counterpart in the reference): per axis with sigma > 0, taps w_m =
 * exp(-m^2 / (2 sigma^2)) / (w_0 + 2 w_1 + ... ), |m| <= ceil(3 sigma), the
 * sum over m = -R..R in order, each term by fma() (correctly rounded, as the
 * GPU's), coordinates mirrored about the volume's faces
 * (x < 1 -> 1 - x, x > n -> 2n + 1 - x, as the reference's reflection
 * copies voxel 1 into ghost 0); then the ghost layer by reflection.
 * Returns -1 when a radius exceeds 32. */
static int mirror_idx(int x, int n)
{
    while (x < 1 || x > n)
        x = x < 1 ? 1 - x : 2 * n + 1 - x;
    return x;
}

int or_gaussian(const ss4d_dims *d, const double sigma[4], double *v, double *scratch)
{
    geo_t g = geo_of(d);
    const ptrdiff_t st[4] = {g.sx, g.sy, g.sz, g.sw};
    const int n[4] = {g.iM - 2, g.jM - 2, g.kM - 2, g.lM - 2};
    double *src = v, *dst = scratch;
    for (int a = 0; a < 4; ++a) {
        if (!(sigma[a] > 0.0))
            continue;
        const double r = ceil(3.0 * sigma[a]);
        if (r > 32)
            return -1;
        const int R = (int)r;
        double w[33], sum = 0.0;
        for (int m = 0; m <= R; ++m) {
            w[m] = exp(-(double)(m * m) / (2.0 * sigma[a] * sigma[a]));
            sum += (m ? 2.0 : 1.0) * w[m];
        }
        for (int m = 0; m <= R; ++m)
            w[m] = w[m] / sum;
        int l;
#pragma omp parallel for schedule(static)
        for (l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i <= g.iM - 2; i++) {
                        const int c[4] = {i, j, k, l};
                        const ptrdiff_t o = at(&g, i, j, k, l);
                        const ptrdiff_t base = o - (ptrdiff_t)c[a] * st[a];
                        double acc = 0.0;
                        for (int m = -R; m <= R; ++m)
                            acc = fma(w[m < 0 ? -m : m], src[base + (ptrdiff_t)mirror_idx(c[a] + m, n[a]) * st[a]], acc);
                        dst[o] = acc;
                    }
        double *t = src;
        src = dst;
        dst = t;
    }
    if (src != v)
        or_copy(d, src, v);
    or_reflect(d, v);
    return 0;
}

/* ---------------------------------------------------------------------- */
/* edge detector                                                            */

/* The face loop of _gf_inputImage_plus_thresholdedImage_
 * (segmentation4D.c:594-821): g_f = 1/(1 + K (theta |grad i0|_f^2 +
 * rho |grad ithr|_f^2)) for the 8 faces of every interior voxel
 * (_gFunction_, segmentation4D.c:67-70). */
void or_gfaces(const ss4d_dims *d, const ss4d_params *p, const double *i0, const double *ithr,
               double *const gout[8])
{
    geo_t g = geo_of(d);
    const ptrdiff_t st[4] = {g.sx, g.sy, g.sz, g.sw};
    const double q = 4.0 * p->h;
    int l;
#pragma omp parallel for schedule(static)
    for (l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++) {
                    ptrdiff_t o = at(&g, i, j, k, l);
                    for (int f = 0; f < 8; ++f) {
                        ptrdiff_t nb = o + face_sign[f] * st[face_axis[f]];
                        double s0 = face_sq(i0, o, nb, st, face_axis[f], p->h, q);
                        double s1 = face_sq(ithr, o, nb, st, face_axis[f], p->h, q);
                        gout[f][o] = 1.0 / (1 + p->K * (p->theta_img * s0 + p->rho_thr * s1));
                    }
                }
}

/* _gf_inputImage_plus_thresholdedImage_: presmooth both images, then g. */
void or_edge_detector(const ss4d_dims *d, const ss4d_params *p, double *i0, double *ithr,
                      double *scratch, double *const gout[8], int *z_i0, int *z_thr)
{
    int a = or_presmooth(d, p, i0, scratch, NULL);
    int b = or_presmooth(d, p, ithr, scratch, NULL);
    if (z_i0)
        *z_i0 = a;
    if (z_thr)
        *z_thr = b;
    or_gfaces(d, p, i0, ithr, gout);
}

/* ---------------------------------------------------------------------- */
/* coefficient assembly                                                     */

/* _gs_coefficients_ (segmentation4D.c:446-580) when gin != NULL, else
 * _gs_coefficients_mcf (mcf_4D.c:208-342).  Per interior voxel: the 8 face
 * norms |grad u|_f = sqrt(|grad u|_f^2 + eps2), their mean, the voxel value
 * vc = sqrt(mean^2 + eps2), and a_f = vc * g_f * (1/|grad u|_f). */
void or_coefficients(const ss4d_dims *d, const ss4d_params *p, const double *u,
                     const double *const gin[8], double *const coef[8])
{
    geo_t g = geo_of(d);
    const ptrdiff_t st[4] = {g.sx, g.sy, g.sz, g.sw};
    const double q = 4.0 * p->h;
    int l;
#pragma omp parallel for schedule(static)
    for (l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++) {
                    ptrdiff_t o = at(&g, i, j, k, l);
                    double nf[8];
                    for (int f = 0; f < 8; ++f) {
                        ptrdiff_t nb = o + face_sign[f] * st[face_axis[f]];
                        nf[f] = sqrt(face_sq(u, o, nb, st, face_axis[f], p->h, q) + p->eps2);
                    }
                    double mean = ((nf[0] + nf[1] + nf[2] + nf[3] + nf[4] + nf[5] + nf[6] + nf[7]) / 8.0);
                    double vc = sqrt(pow(mean, 2) + p->eps2);
                    for (int f = 0; f < 8; ++f) {
                        if (gin)
                            coef[f][o] = vc * gin[f][o] * (1.0 / nf[f]);
                        else
                            coef[f][o] = vc * (1.0 / nf[f]);
                    }
                }
}

/* ---------------------------------------------------------------------- */
/* red-black SOR                                                            */

/* The do/while of _segTimeStep_ (segmentation4D.c:228-309), identical in
 * _mcfTimeStep (mcf_4D.c:121-200): red sweep ((i+j+k+l) even), black sweep,
 * then R = sum r^2 h^4 with r = u(1 + c sum a) - c sum a u_nb - prev; repeat
 * while R > gsTol && z < maxNoGSIteration.  The numerator visits the faces in
 * the order e, w, s, n, b, t, bw, fw and the diagonal in e, w, n, s, t, b,
 * fw, bw, as the reference does. */
int or_sor(const ss4d_dims *d, const ss4d_params *p, double *u, const double *prev,
           const double *const a[8], double *res)
{
    geo_t g = geo_of(d);
    const double c = p->tau / (p->h * p->h);
    const double h4 = p->h * p->h * p->h * p->h;
    const ptrdiff_t sx = g.sx, sy = g.sy, sz = g.sz, sw = g.sw;
    const double *E = a[0], *W = a[1], *N = a[2], *S = a[3], *T = a[4], *B = a[5], *FW = a[6], *BW = a[7];
    double R = 0.0;
    int z = 0, l;
    do {
        z = z + 1;
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (l = 1; l <= g.lM - 2; l++)
                for (int k = 1; k <= g.kM - 2; k++)
                    for (int j = 1; j <= g.jM - 2; j++)
                        for (int i = 1; i <= g.iM - 2; i++) {
                            if ((i + j + k + l) % 2 != colour)
                                continue;
                            ptrdiff_t o = at(&g, i, j, k, l);
                            double gs = (prev[o] + c * ((E[o] * u[o + sx]) + (W[o] * u[o - sx]) + (S[o] * u[o - sy])
                                                        + (N[o] * u[o + sy]) + (B[o] * u[o - sz]) + (T[o] * u[o + sz])
                                                        + (BW[o] * u[o - sw]) + (FW[o] * u[o + sw])))
                                        / (1 + c * (E[o] + W[o] + N[o] + S[o] + T[o] + B[o] + FW[o] + BW[o]));
                            u[o] = u[o] + p->omega_c * (gs - u[o]);
                        }
        }
        R = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : R)
        for (l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i <= g.iM - 2; i++) {
                        ptrdiff_t o = at(&g, i, j, k, l);
                        R += (pow(u[o] * (1 + c * (E[o] + W[o] + N[o] + S[o] + T[o] + B[o] + FW[o] + BW[o]))
                                      - c * ((E[o] * u[o + sx]) + (W[o] * u[o - sx]) + (S[o] * u[o - sy])
                                             + (N[o] * u[o + sy]) + (B[o] * u[o - sz]) + (T[o] * u[o + sz])
                                             + (BW[o] * u[o - sw]) + (FW[o] * u[o + sw]))
                                      - prev[o], 2) * h4);
                    }
    } while (R > p->gsTol && z < p->maxNoGSIteration);
    if (res)
        *res = R;
    return z;
}

/* One half-sweep of or_sor's loop (the red or the black loop of
 * segmentation4D.c:234-285, identical in _segTimeStep_mpi_,
 * segmentation4D_mpi.c:300-359) over the interior of the given array; with
 * or_sor_residual the pieces a slab of a volume split by frames runs between
 * its ghost-frame exchanges.  Same evaluation order as or_sor. */
void or_sor_half(const ss4d_dims *d, const ss4d_params *p, double *u, const double *prev, const double *const a[8],
                 int colour)
{
    geo_t g = geo_of(d);
    const double c = p->tau / (p->h * p->h);
    const ptrdiff_t sx = g.sx, sy = g.sy, sz = g.sz, sw = g.sw;
    const double *E = a[0], *W = a[1], *N = a[2], *S = a[3], *T = a[4], *B = a[5], *FW = a[6], *BW = a[7];
    int l;
#pragma omp parallel for schedule(static)
    for (l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++) {
                    if ((i + j + k + l) % 2 != colour)
                        continue;
                    ptrdiff_t o = at(&g, i, j, k, l);
                    double gs = (prev[o] + c * ((E[o] * u[o + sx]) + (W[o] * u[o - sx]) + (S[o] * u[o - sy])
                                                + (N[o] * u[o + sy]) + (B[o] * u[o - sz]) + (T[o] * u[o + sz])
                                                + (BW[o] * u[o - sw]) + (FW[o] * u[o + sw])))
                                / (1 + c * (E[o] + W[o] + N[o] + S[o] + T[o] + B[o] + FW[o] + BW[o]));
                    u[o] = u[o] + p->omega_c * (gs - u[o]);
                }
}

/* The residual sum of or_sor's loop (segmentation4D.c:288-308) over the
 * interior of the given array (summed in (l, k, j, i) order when one thread
 * runs it). */
double or_sor_residual(const ss4d_dims *d, const ss4d_params *p, const double *u, const double *prev,
                       const double *const a[8])
{
    geo_t g = geo_of(d);
    const double c = p->tau / (p->h * p->h);
    const double h4 = p->h * p->h * p->h * p->h;
    const ptrdiff_t sx = g.sx, sy = g.sy, sz = g.sz, sw = g.sw;
    const double *E = a[0], *W = a[1], *N = a[2], *S = a[3], *T = a[4], *B = a[5], *FW = a[6], *BW = a[7];
    double R = 0.0;
    int l;
#pragma omp parallel for schedule(static) reduction(+ : R)
    for (l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++) {
                    ptrdiff_t o = at(&g, i, j, k, l);
                    R += (pow(u[o] * (1 + c * (E[o] + W[o] + N[o] + S[o] + T[o] + B[o] + FW[o] + BW[o]))
                                  - c * ((E[o] * u[o + sx]) + (W[o] * u[o - sx]) + (S[o] * u[o - sy])
                                         + (N[o] * u[o + sy]) + (B[o] * u[o - sz]) + (T[o] * u[o + sz])
                                         + (BW[o] * u[o - sw]) + (FW[o] * u[o + sw]))
                                  - prev[o], 2) * h4);
                }
    return R;
}

/* ---------------------------------------------------------------------- */
/* rescale / mask                                                           */

static int ball_box_ok(const geo_t *g, double cx, double cy, double cz, double R)
{
    int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
    int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
    int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
    return k0 >= 0 && j0 >= 0 && i0 >= 0 && k1 < g->kM && j1 < g->jM && i1 < g->iM;
}

/* _rescale4DdataToZeroOne_ (segmentation4D.c:1020-1104).  Balls are given
 * flattened in (frame, centre) order.  Returns 0, or -1 if a ball box leaves
 * the array (the reference would read outside it). */
int or_rescale(const ss4d_dims *d, double R, double *v, const double *Mmask, int nb, const int *bl,
               const double *bx, const double *by, const double *bz)
{
    geo_t g = geo_of(d);
    for (int b = 0; b < nb; ++b)
        if (!ball_box_ok(&g, bx[b], by[b], bz[b], R))
            return -1;
    for (int l = 1; l <= g.lM - 2; l++) {
        int c = 0;
        for (int b = 0; b < nb; ++b) {
            if (bl[b] != l)
                continue;
            const double cx = bx[b], cy = by[b], cz = bz[b];
            int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
            int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
            int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
            double mx = 0, mn = 100000;
            for (int k = k0; k <= k1; k++)
                for (int j = j0; j <= j1; j++)
                    for (int i = i0; i <= i1; i++) {
                        double dx = i - cx, dy = j - cy, dz = k - cz;
                        double r = sqrt((dx * dx) + (dy * dy) + (dz * dz));
                        if (r <= R) {
                            double val = v[at(&g, i, j, k, l)];
                            if (val < mn)
                                mn = val;
                            if (val > mx)
                                mx = val;
                        }
                    }
            double quot = 1. / (mx - mn);
            double off = mn * quot;
            for (int k = k0; k <= k1; k++)
                for (int j = j0; j <= j1; j++)
                    for (int i = i0; i <= i1; i++) {
                        double dx = i - cx, dy = j - cy, dz = k - cz;
                        double r = sqrt((dx * dx) + (dy * dy) + (dz * dz));
                        ptrdiff_t o = at(&g, i, j, k, l);
                        double nv = (quot * v[o]) - off;
                        if (r <= R) {
                            if (c == 0)
                                v[o] = nv;
                            else if (v[o] < nv)
                                v[o] = nv;
                        }
                    }
            ++c;
        }
    }
    if (Mmask) {
        for (int l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i <= g.iM - 2; i++) {
                        ptrdiff_t o = at(&g, i, j, k, l);
                        if (Mmask[o] == 0)
                            v[o] = 0;
                    }
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* initial segmentation: local thresholding, initial function              */

/* _get4DMax_ (segmentation4D.c:876-895): the largest interior value, the
 * search starting from 0 (so the result is never negative). */
double or_max4d(const ss4d_dims *d, const double *v)
{
    geo_t g = geo_of(d);
    double mx = 0;
    for (int l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++)
                    if (v[at(&g, i, j, k, l)] > mx)
                        mx = v[at(&g, i, j, k, l)];
    return mx;
}

/* _get3DMinWithinR_ / _get3DMaxWithinR_ (segmentation4D.c:897-969): over the
 * voxels of frame l whose distance to the centre is at most R, the searches
 * starting from 100000 and 0.  Returns -1 if the ball's box leaves the array. */
int or_ball_min_max(const ss4d_dims *d, const double *v, int l, double cx, double cy, double cz, double R,
                    double *mn_out, double *mx_out)
{
    geo_t g = geo_of(d);
    if (!ball_box_ok(&g, cx, cy, cz, R) || l < 0 || l >= g.lM)
        return -1;
    int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
    int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
    int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
    double mn = 100000, mx = 0;
    for (int k = k0; k <= k1; k++)
        for (int j = j0; j <= j1; j++)
            for (int i = i0; i <= i1; i++) {
                double dx = i - cx, dy = j - cy, dz = k - cz;
                double r = sqrt((dx * dx) + (dy * dy) + (dz * dz));
                if (r <= R) {
                    double val = v[at(&g, i, j, k, l)];
                    if (val < mn)
                        mn = val;
                    if (val > mx)
                        mx = val;
                }
            }
    *mn_out = mn;
    *mx_out = mx;
    return 0;
}

/* _locallyThreshold4Ddata_ (segmentation4D.c:971-1018): per ball of radius R
 * the level alpha min + beta max of the input inside it; inside the ball the
 * thresholded image becomes the global maximum wherever the input exceeds the
 * level (elsewhere it is left as it is).  Balls flattened in (frame, centre)
 * order; -1 if a ball box leaves the array. */
int or_local_threshold(const ss4d_dims *d, double alpha, double beta, double R, const double *in, double *thr, int nb,
                       const int *bl, const double *bx, const double *by, const double *bz)
{
    geo_t g = geo_of(d);
    for (int b = 0; b < nb; ++b)
        if (!ball_box_ok(&g, bx[b], by[b], bz[b], R))
            return -1;
    const double gmax = or_max4d(d, in);
    for (int b = 0; b < nb; ++b) {
        const int l = bl[b];
        const double cx = bx[b], cy = by[b], cz = bz[b];
        double mn, mx;
        or_ball_min_max(d, in, l, cx, cy, cz, R, &mn, &mx);
        const double level = alpha * mn + beta * mx;
        int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
        int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
        int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    double dx = i - cx, dy = j - cy, dz = k - cz;
                    double r = sqrt((dx * dx) + (dy * dy) + (dz * dz));
                    if (r <= R && in[at(&g, i, j, k, l)] > level)
                        thr[at(&g, i, j, k, l)] = gmax;
                }
    }
    return 0;
}

/* _generate4DsegmFunct_ (segmentation4D.c:1106-1147): in the box of each
 * ball (half-width R + 0.5, R = ballRadius) and within the fixed distance 12
 * of its centre, u = max(u, |1/(r + 0.5) - 1/12.5|) and Mmask = 1.  -1 if a
 * ball box leaves the array. */
int or_generate_segm(const ss4d_dims *d, double R, double *u, double *Mmask, int nb, const int *bl, const double *bx,
                     const double *by, const double *bz)
{
    geo_t g = geo_of(d);
    const double v = 0.5, Rf = 12.;
    for (int b = 0; b < nb; ++b)
        if (!ball_box_ok(&g, bx[b], by[b], bz[b], R))
            return -1;
    for (int b = 0; b < nb; ++b) {
        const int l = bl[b];
        const double cx = bx[b], cy = by[b], cz = bz[b];
        int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
        int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
        int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    double dx = i - cx, dy = j - cy, dz = k - cz;
                    double r = sqrt((dx * dx) + (dy * dy) + (dz * dz));
                    if (r <= Rf) {
                        double nv = fabs((1. / (sqrt((dx * dx) + (dy * dy) + (dz * dz)) + v)) - (1. / (Rf + v)));
                        ptrdiff_t o = at(&g, i, j, k, l);
                        if (u[o] < nv)
                            u[o] = nv;
                        Mmask[o] = 1.;
                    }
                }
    }
    return 0;
}

/* Threshold of _writeData_mpi_ (segmentation4D_mpi.c:1470-1478): one byte per
 * interior voxel, 1 where u >= level, frames in (l, k, j, i) order.  With
 * normalise the level is min + level (max - min) over the interior. */
void or_threshold_mask(const ss4d_dims *d, const double *u, double level, int normalise, uint8_t *mask)
{
    geo_t g = geo_of(d);
    double lev = level;
    if (normalise) {
        double mn = INFINITY, mx = -INFINITY;
        for (int l = 1; l <= g.lM - 2; l++)
            for (int k = 1; k <= g.kM - 2; k++)
                for (int j = 1; j <= g.jM - 2; j++)
                    for (int i = 1; i <= g.iM - 2; i++) {
                        double val = u[at(&g, i, j, k, l)];
                        if (val < mn)
                            mn = val;
                        if (val > mx)
                            mx = val;
                    }
        lev = mn + level * (mx - mn);
    }
    size_t m = 0;
    for (int l = 1; l <= g.lM - 2; l++)
        for (int k = 1; k <= g.kM - 2; k++)
            for (int j = 1; j <= g.jM - 2; j++)
                for (int i = 1; i <= g.iM - 2; i++)
                    mask[m++] = u[at(&g, i, j, k, l)] >= lev ? 1 : 0;
}

/* ---------------------------------------------------------------------- */
/* norms                                                                    */

/* _l2norm_ (segmentation4D.c:194-213): over every padded voxel. */
double or_l2norm(const ss4d_dims *d, double h, const double *a, const double *b)
{
    geo_t g = geo_of(d);
    const double h4 = h * h * h * h;
    double s = 0;
    for (ptrdiff_t o = 0; o < g.n; ++o)
        s += (pow(a[o] - b[o], 2) * h4);
    return sqrt(s);
}

/* _mass4D_ (segmentation4D.c:317-335) */
double or_mass(const ss4d_dims *d, double h, const double *a)
{
    geo_t g = geo_of(d);
    const double h4 = h * h * h * h;
    double s = 0;
    for (ptrdiff_t o = 0; o < g.n; ++o)
        s += (a[o] * h4);
    return s;
}

/* ---------------------------------------------------------------------- */
/* time steps                                                               */

/* _segTimeStep_ (segmentation4D.c:215-315): prev <- u, coefficients, SOR,
 * rescale.  Returns the SOR iteration count. */
int or_seg_time_step(const ss4d_dims *d, const ss4d_params *p, double *u, double *prev,
                     const double *const gin[8], double *const coef[8], const double *Mmask, int nb,
                     const int *bl, const double *bx, const double *by, const double *bz, double *res)
{
    or_copy(d, u, prev);
    or_coefficients(d, p, u, gin, coef);
    int z = or_sor(d, p, u, prev, (const double *const *)coef, res);
    or_rescale(d, p->ballRadius, u, Mmask, nb, bl, bx, by, bz);
    return z;
}

/* _mcfTimeStep (mcf_4D.c:102-205): prev <- u, coefficients with g == 1,
 * exact Dirichlet ghosts at t = tau * step, SOR. */
int or_mcf_time_step(const ss4d_dims *d, const ss4d_params *p, int step, double *u, double *prev,
                     double *const coef[8], double *res)
{
    double t = p->tau * step;
    or_copy(d, u, prev);
    or_coefficients(d, p, u, NULL, coef);
    or_mcf_set_boundary(d, p->h, t, u);
    return or_sor(d, p, u, prev, (const double *const *)coef, res);
}
