/*
 * ss4d_compat_seg.c — segmentation4D.c's entry points and globals over the
 * GB300 solver (libss4d_seg.so).  See include/ss4d_compat.h for the contract.
 *
 * The globals below carry the names and types of segmentation4D.c:14-58 so a
 * driver written for the reference sets them unchanged.  Each host array has
 * a device mirror; the functions move the caller-visible arrays across and
 * run the device path of include/ss4d.h.
 */
#include <ctype.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/ss4d.h"
#include "../../include/ss4d_compat.h"

/* ---- the reference's globals (segmentation4D.c:14-58) ------------------ */
int kMax, iMax, jMax, lMax;
double *u, *prev_u, *i0, *Mmask;
double *e, *w, *n, *s, *t, *b, *fw, *bw;
double *g_e, *g_w, *g_n, *g_s, *g_t, *g_b, *g_fw, *g_bw;
int *no_of_centers;
double **center_x, **center_y, **center_z;
double spacing_x, spacing_y, spacing_z;
double origin_x, origin_y, origin_z;
int maxNoGSIteration;
double eps2;
double K;
int numberOfTimeStep;
int maxNoOfTimeSteps;
double segTol;
double tau, h, omega_c, gsTol, omega_sigma;
double theta_img, rho_thr, alpha, beta;
int mod;
double sigma;
double maxNoGSIteration_sigma;
int timeStepsNum;
double ballRadius;

/* ---- device mirrors ----------------------------------------------------- */
enum { A_U, A_PREV, A_I0, A_MASK, A_E, A_W, A_N, A_S, A_T, A_B, A_FW, A_BW,
       A_GE, A_GW, A_GN, A_GS, A_GT, A_GB, A_GFW, A_GBW, A_COUNT };

static ss4d_solver *g_solver;
static double *g_dev[A_COUNT];
static double *g_tmp;         /* device buffer for a pointer that is not a global */
static double *g_tmp2;
static size_t g_bytes;        /* bytes of one padded array */
static int g_strict;
static ss4d_step_stats g_last;
static uint8_t *g_frame_dev, *g_frame_host; /* one frame's file bytes (device, page-locked host) */

static double **host_slot(int a)
{
    double **tab[A_COUNT] = {&u, &prev_u, &i0, &Mmask, &e, &w, &n, &s, &t, &b, &fw, &bw,
                             &g_e, &g_w, &g_n, &g_s, &g_t, &g_b, &g_fw, &g_bw};
    return tab[a];
}

static void report(const char *what, ss4d_status st)
{
    if (st != SS4D_OK)
        fprintf(stderr, "ss4d: %s failed (status %d): %s\n", what, (int)st, ss4d_last_error());
}

static ss4d_params params_from_globals(void)
{
    ss4d_params p;
    memset(&p, 0, sizeof p);
    p.K = K;
    p.eps2 = eps2;
    p.tau = tau;
    p.h = h;
    p.omega_c = omega_c;
    p.gsTol = gsTol;
    p.maxNoGSIteration = maxNoGSIteration;
    p.maxNoOfTimeSteps = maxNoOfTimeSteps;
    p.segTol = segTol;
    p.sigma = sigma;
    p.omega_sigma = omega_sigma;
    p.maxNoGSIteration_sigma = maxNoGSIteration_sigma;
    p.theta_img = theta_img;
    p.rho_thr = rho_thr;
    p.ballRadius = ballRadius;
    return p;
}

static ss4d_arith arith_from_env(void)
{
    const char *v = getenv("SS4D_ARITH");
    if (v && strcmp(v, "reference") == 0)
        return SS4D_ARITH_REFERENCE;
    if (v && strcmp(v, "mixed") == 0)
        return SS4D_ARITH_MIXED;
    return SS4D_ARITH_FP64;
}

/* device mirror of a host pointer: a global's mirror, else a scratch buffer */
static double *mirror_of(const double *hp, double *scratch)
{
    for (int a = 0; a < A_COUNT; ++a)
        if (*host_slot(a) == hp)
            return g_dev[a];
    return scratch;
}

static bool up(const double *hp, double *dp)
{
    ss4d_status st = ss4d_copy_to_device(g_solver, dp, hp, g_bytes);
    report("upload", st);
    return st == SS4D_OK;
}

static bool down(double *hp, const double *dp)
{
    ss4d_status st = ss4d_copy_to_host(g_solver, hp, dp, g_bytes);
    report("download", st);
    return st == SS4D_OK;
}

static bool finish(void)
{
    ss4d_status st = ss4d_synchronize(g_solver);
    report("synchronize", st);
    return st == SS4D_OK;
}

bool ss4d_compat_sync_host(void)
{
    if (!g_solver)
        return false;
    for (int a = A_E; a < A_COUNT; ++a)
        if (!down(*host_slot(a), g_dev[a]))
            return false;
    return finish();
}

bool ss4d_compat_last_stats(struct ss4d_step_stats *out)
{
    if (!out)
        return false;
    *out = g_last;
    return true;
}

static bool sync_if_strict(int first, int last)
{
    if (!g_strict)
        return true;
    for (int a = first; a <= last; ++a)
        if (!down(*host_slot(a), g_dev[a]))
            return false;
    return true;
}

/* ---- allocation (segmentation4D.c:71-192) ------------------------------ */
bool _allocateMem_(void)
{
    if (g_solver)
        _deallocateMem_();
    ss4d_dims d = {iMax, jMax, kMax, lMax};
    ss4d_status st = ss4d_solver_create(&d, arith_from_env(), NULL, &g_solver);
    report("solver_create", st);
    if (st != SS4D_OK)
        return false;
    const char *sv = getenv("SS4D_COMPAT_STRICT");
    g_strict = sv && sv[0] == '1';
    const char *xv = getenv("SS4D_EXTRAPOLATE"); /* mixed form: extrapolation order 1..3 */
    if (xv && xv[0] >= '1' && xv[0] <= '3')
        ss4d_solver_set_extrapolation(g_solver, xv[0] - '0');
    const char *pv = getenv("SS4D_PROJECT"); /* with order 3: projected start of the first round */
    if (pv && pv[0] == '1')
        ss4d_solver_set_projection(g_solver, 1);
    g_bytes = sizeof(double) * (size_t)iMax * jMax * kMax * lMax;
    for (int a = 0; a < A_COUNT; ++a) {
        void *hp = NULL, *dp = NULL;
        if (ss4d_host_alloc(g_bytes, &hp) != SS4D_OK || ss4d_dev_alloc(g_bytes, &dp) != SS4D_OK)
            return false;
        memset(hp, 0, g_bytes); /* the reference zero-fills every array (segmentation4D.c:106-135) */
        *host_slot(a) = (double *)hp;
        g_dev[a] = (double *)dp;
        if (!up(hp, dp))
            return false;
    }
    void *t1 = NULL, *t2 = NULL;
    if (ss4d_dev_alloc(g_bytes, &t1) != SS4D_OK || ss4d_dev_alloc(g_bytes, &t2) != SS4D_OK)
        return false;
    g_tmp = (double *)t1;
    g_tmp2 = (double *)t2;
    center_x = (double **)calloc((size_t)lMax, sizeof(double *));
    center_y = (double **)calloc((size_t)lMax, sizeof(double *));
    center_z = (double **)calloc((size_t)lMax, sizeof(double *));
    if (!center_x || !center_y || !center_z)
        return false;
    for (int l = 0; l < lMax; ++l) {
        int c = no_of_centers ? no_of_centers[l] : 0;
        center_x[l] = (double *)malloc(sizeof(double) * (size_t)(c > 0 ? c : 1));
        center_y[l] = (double *)malloc(sizeof(double) * (size_t)(c > 0 ? c : 1));
        center_z[l] = (double *)malloc(sizeof(double) * (size_t)(c > 0 ? c : 1));
        if (!center_x[l] || !center_y[l] || !center_z[l])
            return false;
    }
    return finish();
}

bool _deallocateMem_(void)
{
    if (!g_solver)
        return true;
    ss4d_synchronize(g_solver);
    for (int a = 0; a < A_COUNT; ++a) {
        ss4d_host_free(*host_slot(a));
        ss4d_dev_free(g_dev[a]);
        *host_slot(a) = NULL;
        g_dev[a] = NULL;
    }
    ss4d_dev_free(g_tmp);
    ss4d_dev_free(g_tmp2);
    g_tmp = g_tmp2 = NULL;
    ss4d_dev_free(g_frame_dev);
    ss4d_host_free(g_frame_host);
    g_frame_dev = NULL;
    g_frame_host = NULL;
    if (center_x) {
        for (int l = 0; l < lMax; ++l) {
            free(center_x[l]);
            free(center_y[l]);
            free(center_z[l]);
        }
    }
    free(center_x);
    free(center_y);
    free(center_z);
    center_x = center_y = center_z = NULL;
    ss4d_solver_destroy(g_solver);
    g_solver = NULL;
    return true;
}

/* ---- small host utilities (index / scalar formula, no array work) ------ */
int ijkl(int i, int j, int k, int l)
{
    return ((l * kMax + k) * jMax + j) * iMax + i;
}

double _gFunction_(double value, double coef)
{
    return 1.0 / (1 + coef * value);
}

void _copy4DdataFromSrcToDest_(double *srcDataPtr, double *destDataPtr)
{
    memcpy(destDataPtr, srcDataPtr, g_bytes);
}

/* ---- device-backed entry points ---------------------------------------- */

/* centres of the per-ball rescale in (frame, centre) order */
typedef struct {
    int nb;
    int *l;
    double *x, *y, *z;
} balls_t;

static void balls_free(balls_t *bb)
{
    free(bb->l);
    free(bb->x);
    free(bb->y);
    free(bb->z);
}

static bool balls_make(balls_t *bb)
{
    memset(bb, 0, sizeof *bb);
    if (!no_of_centers)
        return true;
    int tot = 0;
    for (int l = 1; l <= lMax - 2; ++l)
        tot += no_of_centers[l] > 0 ? no_of_centers[l] : 0;
    if (tot == 0)
        return true;
    bb->l = (int *)malloc(sizeof(int) * tot);
    bb->x = (double *)malloc(sizeof(double) * tot);
    bb->y = (double *)malloc(sizeof(double) * tot);
    bb->z = (double *)malloc(sizeof(double) * tot);
    if (!bb->l || !bb->x || !bb->y || !bb->z)
        return false;
    int m = 0;
    for (int l = 1; l <= lMax - 2; ++l)
        for (int c = 0; c < no_of_centers[l]; ++c) {
            bb->l[m] = l;
            bb->x[m] = center_x[l][c];
            bb->y[m] = center_y[l][c];
            bb->z[m] = center_z[l][c];
            ++m;
        }
    bb->nb = tot;
    return true;
}

static bool rescale_dev(double *d_img)
{
    balls_t bb;
    if (!balls_make(&bb))
        return false;
    ss4d_balls B = {bb.nb, bb.l, bb.x, bb.y, bb.z};
    ss4d_params p = params_from_globals();
    ss4d_status st = ss4d_rescale_to_zero_one(g_solver, &p, d_img, g_dev[A_MASK], &B);
    balls_free(&bb);
    report("rescale", st);
    return st == SS4D_OK;
}

bool _rescale4DdataToZeroOne_(double *imagePtr)
{
    if (!g_solver || !imagePtr)
        return false;
    double *d = mirror_of(imagePtr, g_tmp);
    if (!up(imagePtr, d) || !up(Mmask, g_dev[A_MASK]))
        return false;
    if (!rescale_dev(d))
        return false;
    return down(imagePtr, d) && finish();
}

/* ---- initial segmentation (segmentation4D.c:876-1018, 1106-1147) ------- */

double _get4DMax_(double *imagePtr)
{
    if (!imagePtr)
        exit(1); /* as the reference (segmentation4D.c:880) */
    if (!g_solver)
        return 0;
    double *d = mirror_of(imagePtr, g_tmp);
    double mx = 0;
    if (!up(imagePtr, d))
        return 0;
    ss4d_status st = ss4d_max4d(g_solver, d, &mx);
    report("max4d", st);
    return mx;
}

static double ball_extreme(double *imagePtr, int l, double cx, double cy, double cz, double R, int want_max)
{
    if (!imagePtr)
        exit(1); /* as the reference (segmentation4D.c:901, 938) */
    if (!g_solver)
        return 0;
    double *d = mirror_of(imagePtr, g_tmp);
    double mn = 0, mx = 0;
    if (!up(imagePtr, d))
        return 0;
    ss4d_status st = ss4d_ball_min_max(g_solver, d, l, cx, cy, cz, R, &mn, &mx);
    report("ball min/max", st);
    return want_max ? mx : mn;
}

double _get3DMinWithinR_(double *imagePtr, int l, double center_x, double center_y, double center_z, double R)
{
    return ball_extreme(imagePtr, l, center_x, center_y, center_z, R, 0);
}

double _get3DMaxWithinR_(double *imagePtr, int l, double center_x, double center_y, double center_z, double R)
{
    return ball_extreme(imagePtr, l, center_x, center_y, center_z, R, 1);
}

bool _locallyThreshold4Ddata_(double *inputImagePtr, double *thresholdedImagePtr)
{
    if (!g_solver || !inputImagePtr || !thresholdedImagePtr)
        return false;
    double *di = mirror_of(inputImagePtr, g_tmp);
    double *dt = mirror_of(thresholdedImagePtr, g_tmp2);
    if (!up(inputImagePtr, di) || !up(thresholdedImagePtr, dt))
        return false;
    balls_t bb;
    if (!balls_make(&bb))
        return false;
    ss4d_balls B = {bb.nb, bb.l, bb.x, bb.y, bb.z};
    ss4d_status st = ss4d_local_threshold(g_solver, alpha, beta, ballRadius, di, dt, &B);
    balls_free(&bb);
    report("local threshold", st);
    return st == SS4D_OK && down(thresholdedImagePtr, dt) && finish();
}

bool _generate4DsegmFunct_(double *segmFuntionPtr)
{
    if (!g_solver || !segmFuntionPtr)
        return false;
    double *d = mirror_of(segmFuntionPtr, g_tmp);
    if (!up(segmFuntionPtr, d) || !up(Mmask, g_dev[A_MASK]))
        return false;
    balls_t bb;
    if (!balls_make(&bb))
        return false;
    ss4d_balls B = {bb.nb, bb.l, bb.x, bb.y, bb.z};
    ss4d_status st = ss4d_generate_segm_function(g_solver, ballRadius, d, g_dev[A_MASK], &B);
    balls_free(&bb);
    report("initial function", st);
    return st == SS4D_OK && down(segmFuntionPtr, d) && down(Mmask, g_dev[A_MASK]) && finish();
}

/* ---- file formats (segmentation4D.c:1149-1324) --------------------------- */

static size_t frame_voxels(void)
{
    return (size_t)(iMax - 2) * (jMax - 2) * (kMax - 2);
}

static bool frame_buffers(void)
{
    if (g_frame_dev)
        return true;
    ss4d_status st = ss4d_dev_alloc(frame_voxels(), (void **)&g_frame_dev);
    if (st == SS4D_OK)
        st = ss4d_host_alloc(frame_voxels(), (void **)&g_frame_host);
    report("frame buffers", st);
    return st == SS4D_OK;
}

/* file bytes of frame l into the device image d (host -> device: one byte per voxel) */
static bool frame_in(double *d, int l, const char *path)
{
    ss4d_status st = ss4d_vtk_read_frame(path, iMax - 2, jMax - 2, kMax - 2, g_frame_host);
    if (st == SS4D_OK)
        st = ss4d_copy_to_device(g_solver, g_frame_dev, g_frame_host, frame_voxels());
    if (st == SS4D_OK)
        st = ss4d_frame_from_bytes(g_solver, d, l, g_frame_dev);
    report("frame read", st);
    return st == SS4D_OK;
}

void _readNumberFromFile_(char *dim, FILE *input_file)
{
    int count = 0, var;
    do {
        var = fgetc(input_file);
        dim[count++] = (char)var;
    } while (var != EOF && !isspace(var));
}

void _readMetaData_(FILE *input_file)
{
    int c;
    while ((c = getc(input_file)) == '#')
        while ((c = getc(input_file)) != '\n' && c != EOF)
            ;
    for (int h = 0; h < 3 && c != EOF; ++h)
        while ((c = getc(input_file)) != '\n' && c != EOF)
            ;
}

bool _load3dDataArrayVTK_(double *imageDataPtr, int l, unsigned char *pathPtr)
{
    if (!imageDataPtr || !pathPtr || !g_solver || l < 1 || l > lMax - 2 || !frame_buffers())
        return false;
    double *d = mirror_of(imageDataPtr, g_tmp);
    /* the other frames and the ghosts of the host array stay as they are */
    if (!up(imageDataPtr, d) || !frame_in(d, l, (const char *)pathPtr))
        return false;
    return down(imageDataPtr, d) && finish();
}

void _readData_(double *inputImage, unsigned char *fileDirectory)
{
    if (!inputImage || !fileDirectory || !g_solver || !frame_buffers())
        exit(1);
    double *d = mirror_of(inputImage, g_tmp);
    if (!up(inputImage, d))
        exit(1);
    const double sp[3] = {spacing_x, spacing_y, spacing_z};
    char path[1024];
    for (int l = 1; l <= lMax - 2; ++l) {
        snprintf(path, sizeof path, "%s/movingBalls_457_at_time_%03d.vtk", (const char *)fileDirectory, l);
        if (!frame_in(d, l, path))
            exit(1); /* as the reference, for a missing frame file */
        snprintf(path, sizeof path, "%s/movingBalls_457_centers_at_timestep_%03d.vtk", (const char *)fileDirectory,
                 l);
        int np = 0;
        const int cap = no_of_centers ? no_of_centers[l] : 0;
        ss4d_status st = ss4d_vtk_read_centers(path, sp, cap, center_x[l], center_y[l], center_z[l], &np);
        report("centre file", st);
        if (st != SS4D_OK)
            exit(1); /* missing file, or more centres than no_of_centers[l] allocated */
    }
    if (!down(inputImage, d) || !finish())
        exit(1);
}

bool _writeData_(double *array4DPtr, unsigned char *pathPtr)
{
    if (!array4DPtr || !pathPtr || !g_solver || !frame_buffers())
        return false;
    double *d = mirror_of(array4DPtr, g_tmp);
    if (!up(array4DPtr, d))
        return false;
    const double origin[3] = {origin_x, origin_y, origin_z};
    const double sp[3] = {spacing_x, spacing_y, spacing_z};
    char path[1024];
    for (int l = 1; l <= lMax - 2; ++l) {
        ss4d_status st = ss4d_frame_to_bytes(g_solver, d, l, 0, g_frame_dev);
        if (st == SS4D_OK)
            st = ss4d_copy_to_host(g_solver, g_frame_host, g_frame_dev, frame_voxels());
        if (st == SS4D_OK)
            st = ss4d_synchronize(g_solver);
        snprintf(path, sizeof path, "%s_at_time_%03d.vtk", (const char *)pathPtr, l);
        if (st == SS4D_OK)
            st = ss4d_vtk_write_frame(path, iMax - 2, jMax - 2, kMax - 2, origin, sp, g_frame_host);
        report("frame write", st);
        if (st != SS4D_OK)
            puts("File could not be opened."); /* as the reference; it goes on with the next frame */
    }
    return true;
}

bool _reflection4Ddata_(double *v)
{
    if (!g_solver || !v)
        return false;
    double *d = mirror_of(v, g_tmp);
    if (!up(v, d))
        return false;
    ss4d_status st = ss4d_reflect(g_solver, d);
    report("reflect", st);
    return st == SS4D_OK && down(v, d) && finish();
}

bool _presmoothStep_(double *v)
{
    if (!g_solver || !v)
        return false;
    double *d = mirror_of(v, g_tmp);
    if (!up(v, d))
        return false;
    ss4d_params p = params_from_globals();
    /* the reference keeps the copy of the input in its global prev_u */
    ss4d_status st = ss4d_presmooth_step(g_solver, &p, d, g_dev[A_PREV], &g_last);
    report("presmooth", st);
    return st == SS4D_OK && down(v, d) && down(prev_u, g_dev[A_PREV]) && finish();
}

void _presmoothStepEXP_(double *v)
{
    if (!g_solver || !v)
        return;
    double *d = mirror_of(v, g_tmp);
    if (!up(v, d))
        return;
    ss4d_params p = params_from_globals();
    ss4d_status st = ss4d_presmooth_explicit(g_solver, &p, timeStepsNum, d, g_dev[A_PREV]);
    report("explicit presmoothing", st);
    if (st == SS4D_OK && down(v, d) && down(prev_u, g_dev[A_PREV]))
        finish();
}

bool _gf_inputImage_plus_thresholdedImage_(double *img, double *thr)
{
    if (!g_solver || !img || !thr)
        return false;
    double *di = mirror_of(img, g_tmp);
    double *dt = mirror_of(thr, g_tmp2);
    if (!up(img, di) || !up(thr, dt))
        return false;
    ss4d_params p = params_from_globals();
    double *dg[8];
    for (int f = 0; f < 8; ++f)
        dg[f] = g_dev[A_GE + f];
    /* the reference presmooths both images in place with prev_u as scratch */
    ss4d_status st = ss4d_edge_detector(g_solver, &p, di, dt, g_dev[A_PREV], dg);
    report("edge detector", st);
    if (st != SS4D_OK)
        return false;
    return down(img, di) && down(thr, dt) && down(prev_u, g_dev[A_PREV]) && sync_if_strict(A_GE, A_GBW) && finish();
}

bool _gs_coefficients_(void)
{
    if (!g_solver)
        return false;
    if (!up(u, g_dev[A_U]))
        return false;
    ss4d_params p = params_from_globals();
    const double *dg[8];
    double *dc[8];
    for (int f = 0; f < 8; ++f) {
        dg[f] = g_dev[A_GE + f];
        dc[f] = g_dev[A_E + f];
    }
    ss4d_status st = ss4d_gs_coefficients(g_solver, &p, g_dev[A_U], dg, dc);
    report("coefficients", st);
    return st == SS4D_OK && sync_if_strict(A_E, A_BW) && finish();
}

bool _segTimeStep_(void)
{
    if (!g_solver)
        return false;
    ss4d_params p = params_from_globals();
    const double *dg[8];
    for (int f = 0; f < 8; ++f)
        dg[f] = g_dev[A_GE + f];
    balls_t bb;
    if (!balls_make(&bb))
        return false;
    ss4d_balls B = {bb.nb, bb.l, bb.x, bb.y, bb.z};
    ss4d_status st;
    if (!g_strict) {
        /* prev_u <- u as the reference's step begins (segmentation4D.c:224),
         * u up and down in frame chunks overlapped with the step's first and
         * last kernels, Mmask up beside the solve */
        st = ss4d_seg_time_step_host(g_solver, &p, u, g_dev[A_U], prev_u, Mmask, g_dev[A_MASK], dg, &B, &g_last);
        balls_free(&bb);
        report("segmentation time step", st);
        return st == SS4D_OK && finish();
    }
    /* strict: the plain sequence, which also leaves prev_u on the device for
     * the refresh of the reference-layout coefficients */
    if (!up(u, g_dev[A_U]) || !up(Mmask, g_dev[A_MASK])) {
        balls_free(&bb);
        return false;
    }
    st = ss4d_seg_time_step(g_solver, &p, g_dev[A_U], g_dev[A_PREV], dg, g_dev[A_MASK], &B, &g_last);
    balls_free(&bb);
    report("segmentation time step", st);
    if (st != SS4D_OK)
        return false;
    double *dc[8];
    for (int f = 0; f < 8; ++f)
        dc[f] = g_dev[A_E + f];
    st = ss4d_gs_coefficients(g_solver, &p, g_dev[A_PREV], dg, dc);
    report("coefficients", st);
    if (st != SS4D_OK || !sync_if_strict(A_E, A_BW))
        return false;
    return down(u, g_dev[A_U]) && down(prev_u, g_dev[A_PREV]) && finish();
}

double _l2norm_(double *a, double *bb)
{
    if (!g_solver || !a || !bb)
        return false;
    double *da = mirror_of(a, g_tmp), *db = mirror_of(bb, g_tmp2);
    if (da == db && a != bb)
        db = g_tmp2;
    if (!up(a, da) || !up(bb, db))
        return false;
    double out = 0;
    ss4d_status st = ss4d_l2norm(g_solver, h, da, db, &out);
    report("l2norm", st);
    return st == SS4D_OK ? out : 0.0;
}

double _mass4D_(double *a)
{
    if (!g_solver || !a)
        return false;
    double *da = mirror_of(a, g_tmp);
    if (!up(a, da))
        return false;
    double out = 0;
    ss4d_status st = ss4d_mass(g_solver, h, da, &out);
    report("mass", st);
    return st == SS4D_OK ? out : 0.0;
}
