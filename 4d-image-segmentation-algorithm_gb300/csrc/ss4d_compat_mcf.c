/*
 * ss4d_compat_mcf.c — mcf_4D.c's entry points and globals over the GB300
 * solver (libss4d_mcf.so).  Same contract as libss4d_seg.so (see
 * include/ss4d_compat.h); it serves drivers of mcf_4D.c and of its OpenMP
 * form mcf_4D_openmp.c, which share one interface (mcf_4D.h).
 */
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/ss4d.h"
#include "../../include/ss4d_compat.h"

/* ---- the reference's globals (mcf_4D.c:12-34) --------------------------- */
int kMax, iMax, jMax, lMax;
double *u, *prev_u, *exact_u;
double *e, *w, *n, *s, *t, *b, *fw, *bw;
int maxNoGSIteration;
double eps2;
int numberOfTimeStep;
int maxNoOfTimeSteps;
double mcfTol;
double tau, h, omega_c, gsTol;

enum { A_U, A_PREV, A_EXACT, A_E, A_W, A_N, A_S, A_T, A_B, A_FW, A_BW, A_COUNT };

static ss4d_solver *g_solver;
static double *g_dev[A_COUNT];
static double *g_tmp, *g_tmp2;
static size_t g_bytes;
static int g_strict;
static ss4d_step_stats g_last;

static double **host_slot(int a)
{
    double **tab[A_COUNT] = {&u, &prev_u, &exact_u, &e, &w, &n, &s, &t, &b, &fw, &bw};
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
    p.eps2 = eps2;
    p.tau = tau;
    p.h = h;
    p.omega_c = omega_c;
    p.gsTol = gsTol;
    p.maxNoGSIteration = maxNoGSIteration;
    p.maxNoOfTimeSteps = maxNoOfTimeSteps;
    p.segTol = mcfTol;
    return p;
}

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

bool _allocateMem_mcf(void)
{
    if (g_solver)
        _deallocateMem_mcf();
    ss4d_dims d = {iMax, jMax, kMax, lMax};
    const char *v = getenv("SS4D_ARITH");
    ss4d_arith ar = SS4D_ARITH_FP64;
    if (v && strcmp(v, "reference") == 0)
        ar = SS4D_ARITH_REFERENCE;
    else if (v && strcmp(v, "mixed") == 0)
        ar = SS4D_ARITH_MIXED;
    ss4d_status st = ss4d_solver_create(&d, ar, NULL, &g_solver);
    report("solver_create", st);
    if (st != SS4D_OK)
        return false;
    const char *sv = getenv("SS4D_COMPAT_STRICT");
    g_strict = sv && sv[0] == '1';
    g_bytes = sizeof(double) * (size_t)iMax * jMax * kMax * lMax;
    for (int a = 0; a < A_COUNT; ++a) {
        void *hp = NULL, *dp = NULL;
        if (ss4d_host_alloc(g_bytes, &hp) != SS4D_OK || ss4d_dev_alloc(g_bytes, &dp) != SS4D_OK)
            return false;
        memset(hp, 0, g_bytes);
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
    return finish();
}

bool _deallocateMem_mcf(void)
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
    ss4d_solver_destroy(g_solver);
    g_solver = NULL;
    return true;
}

int ijkl(int i, int j, int k, int l)
{
    return ((l * kMax + k) * jMax + j) * iMax + i;
}

void _copy4DdataFromSrcToDest_mcf(double *src, double *dst)
{
    memcpy(dst, src, g_bytes);
}

double _l2norm_mcf(double *a, double *bb)
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

bool _gs_coefficients_mcf(void)
{
    if (!g_solver || !up(u, g_dev[A_U]))
        return false;
    ss4d_params p = params_from_globals();
    double *dc[8];
    for (int f = 0; f < 8; ++f)
        dc[f] = g_dev[A_E + f];
    ss4d_status st = ss4d_gs_coefficients(g_solver, &p, g_dev[A_U], NULL, dc);
    report("coefficients", st);
    if (st != SS4D_OK)
        return false;
    if (g_strict)
        for (int a = A_E; a <= A_BW; ++a)
            if (!down(*host_slot(a), g_dev[a]))
                return false;
    return finish();
}

bool _set4DBoundaryToExactValues_mcf(double time)
{
    if (!g_solver || !up(u, g_dev[A_U]))
        return false;
    ss4d_status st = ss4d_mcf_set_boundary_exact(g_solver, h, time, g_dev[A_U]);
    report("boundary", st);
    return st == SS4D_OK && down(u, g_dev[A_U]) && finish();
}

void _exactSolution_mcf(double time)
{
    if (!g_solver)
        return;
    ss4d_status st = ss4d_mcf_exact_solution(g_solver, h, time, g_dev[A_EXACT]);
    report("exact solution", st);
    if (st == SS4D_OK)
        down(exact_u, g_dev[A_EXACT]);
    finish();
}

bool _mcfTimeStep(void)
{
    if (!g_solver || !up(u, g_dev[A_U]))
        return false;
    ss4d_params p = params_from_globals();
    ss4d_status st = ss4d_mcf_time_step(g_solver, &p, numberOfTimeStep, g_dev[A_U], g_dev[A_PREV], &g_last);
    report("mcf time step", st);
    if (st != SS4D_OK)
        return false;
    if (g_strict) {
        double *dc[8];
        for (int f = 0; f < 8; ++f)
            dc[f] = g_dev[A_E + f];
        if (ss4d_gs_coefficients(g_solver, &p, g_dev[A_PREV], NULL, dc) != SS4D_OK)
            return false;
        for (int a = A_E; a <= A_BW; ++a)
            if (!down(*host_slot(a), g_dev[a]))
                return false;
    }
    return down(u, g_dev[A_U]) && down(prev_u, g_dev[A_PREV]) && finish();
}
