/*
 * ss4d_scene.c — seeded synthetic 4D (3D + time) scenes.
 *
 * The reference reads uchar VTK frames of microscopy data from a directory
 * that is not distributed with it (segmentation4D.c:1149-1215, 1289-1324), so
 * every test, benchmark and oracle run here is fed by this generator instead.
 * It writes, in the reference's padded layout:
 *   i0 : intensities quantised to 8 bits and divided by 255, as the
 *        reference loader does (segmentation4D.c:1320); ghosts are 0 like the
 *        reference's zero-initialised arrays (segmentation4D.c:106-135);
 *   u0 : the initial level-set function 1/(|x - s| + 1) on every voxel,
 *        ghosts included (the ghosts of u are frozen Dirichlet data during
 *        the segmentation steps).
 *
 * Scene kinds (coordinates in padded voxel units, frames t = l - 1):
 *  1  one ellipsoid at the volume centre, radii (10, 8, 7) * nx/32, each
 *     modulated by 1 + 0.15 sin(2 pi t / 8 + phase), phases 0, 2pi/3, 4pi/3;
 *     intensity 200 on background 50; Gaussian noise sigma 20; in every
 *     frame the boundary shell (normalised radius 0.7..1) is set to the
 *     background over one random 30-degree azimuthal sector.
 *  2  as 1 with noise sigma 25 and two erased 30-degree sectors per frame.
 *  3  three ellipsoids, radii U[20, 50] * min(nx, ny, nz)/128, centres
 *     uniform with the object inside the volume, intensities U[150, 230] on
 *     background 50, radii modulated by 1 + 0.15 sin(2 pi t / nt + phase),
 *     one random 36-degree erased sector (10 % of the boundary) per object
 *     and frame, a global intensity drift from -10 % to +10 % over t, and
 *     Gaussian noise sigma 30.
 * s is the object centre in the middle frame (kind 3: u0 is the largest of
 * the three per-object values).
 *
 * Noise and per-frame choices come from a counter-based generator
 * (splitmix64 of seed and voxel index), so the scene does not depend on the
 * number of threads.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/ss4d.h"

static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform in (0, 1) from stream `s`, counter `n` */
static inline double unif(uint64_t seed, uint64_t s, uint64_t n)
{
    uint64_t r = mix64(mix64(seed ^ (s * 0xD1B54A32D192ED03ull)) + n);
    return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static inline double gauss(uint64_t seed, uint64_t n)
{
    double a = unif(seed, 1, 2 * n), b = unif(seed, 1, 2 * n + 1);
    return sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
}

#define MAX_OBJ 3
#define MAX_SECT 2

typedef struct {
    double cx, cy, cz;      /* centre */
    double r[3];            /* base radii */
    double ph[3];           /* modulation phases */
    double inten;           /* object intensity */
} object_t;

ss4d_status ss4d_scene_generate(int kind, int nx, int ny, int nz, int nt, uint64_t seed,
                                double *h_i0, double *h_u0, int nthreads)
{
    if (kind < 1 || kind > 3 || nx < 1 || ny < 1 || nz < 1 || nt < 1 || (!h_i0 && !h_u0))
        return SS4D_ERR_INVALID;
    const int iM = nx + 2, jM = ny + 2, kM = nz + 2, lM = nt + 2;
    const double two_pi = 6.283185307179586;
    object_t obj[MAX_OBJ];
    int nobj, nsect;
    double noise, period, sect_width, background = 50.0;

    memset(obj, 0, sizeof obj);
    if (kind == 1 || kind == 2) {
        double s = nx / 32.0;
        nobj = 1;
        obj[0].cx = (nx + 1) / 2.0;
        obj[0].cy = (ny + 1) / 2.0;
        obj[0].cz = (nz + 1) / 2.0;
        obj[0].r[0] = 10 * s;
        obj[0].r[1] = 8 * s;
        obj[0].r[2] = 7 * s;
        obj[0].ph[0] = 0.0;
        obj[0].ph[1] = two_pi / 3.0;
        obj[0].ph[2] = 2.0 * two_pi / 3.0;
        obj[0].inten = 200.0;
        noise = kind == 1 ? 20.0 : 25.0;
        nsect = kind == 1 ? 1 : 2;
        period = 8.0;
        sect_width = two_pi / 12.0; /* 30 degrees */
    } else {
        int mn = nx < ny ? nx : ny;
        mn = mn < nz ? mn : nz;
        double s = mn / 128.0;
        nobj = 3;
        for (int o = 0; o < nobj; ++o) {
            double rmax = 0;
            for (int a = 0; a < 3; ++a) {
                obj[o].r[a] = (20.0 + 30.0 * unif(seed, 100 + o, a)) * s;
                obj[o].ph[a] = two_pi * unif(seed, 100 + o, 3 + a);
                if (obj[o].r[a] > rmax)
                    rmax = obj[o].r[a];
            }
            double m = rmax * 1.15 + 1.0; /* room for the modulation */
            const int n3[3] = {nx, ny, nz};
            double c[3];
            for (int a = 0; a < 3; ++a) {
                double lo = 1.0 + m, hi = n3[a] - m;
                c[a] = lo < hi ? lo + (hi - lo) * unif(seed, 100 + o, 6 + a) : (n3[a] + 1) / 2.0;
            }
            obj[o].cx = c[0];
            obj[o].cy = c[1];
            obj[o].cz = c[2];
            obj[o].inten = 150.0 + 80.0 * unif(seed, 100 + o, 9);
        }
        noise = 30.0;
        nsect = 1;
        period = (double)nt;
        sect_width = two_pi / 10.0; /* 36 degrees = 10 % of the boundary */
    }

    /* per-frame sector start angles, one per object and sector */
    double *sect = (double *)malloc(sizeof(double) * (size_t)lM * MAX_OBJ * MAX_SECT);
    if (!sect)
        return SS4D_ERR_ALLOC;
    for (int l = 0; l < lM; ++l)
        for (int o = 0; o < MAX_OBJ; ++o)
            for (int q = 0; q < MAX_SECT; ++q)
                sect[((size_t)l * MAX_OBJ + o) * MAX_SECT + q] = two_pi * unif(seed, 200 + o, (uint64_t)l * MAX_SECT + q);

    const double lmid = (nt + 1) / 2.0;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    long long lM_ll = lM;
#pragma omp parallel for schedule(dynamic, 1)
    for (long long lk = 0; lk < lM_ll * kM; ++lk) {
        int l = (int)(lk / kM), k = (int)(lk % kM);
        double t = l - 1.0;
        double drift = kind == 3 ? 1.0 + 0.1 * (nt > 1 ? (2.0 * t / (nt - 1) - 1.0) : 0.0) : 1.0;
        for (int j = 0; j < jM; ++j)
            for (int i = 0; i < iM; ++i) {
                size_t o = (((size_t)l * kM + k) * jM + j) * iM + i;
                if (h_u0) {
                    double best = 0;
                    for (int b = 0; b < nobj; ++b) {
                        double dx = i - obj[b].cx, dy = j - obj[b].cy, dz = k - obj[b].cz, dw = l - lmid;
                        double v = 1.0 / (sqrt(dx * dx + dy * dy + dz * dz + dw * dw) + 1.0);
                        if (v > best)
                            best = v;
                    }
                    h_u0[o] = best;
                }
                if (!h_i0)
                    continue;
                if (i == 0 || j == 0 || k == 0 || l == 0 || i == iM - 1 || j == jM - 1 || k == kM - 1 || l == lM - 1) {
                    h_i0[o] = 0.0;
                    continue;
                }
                double val = background;
                for (int b = 0; b < nobj; ++b) {
                    double rr[3];
                    for (int a = 0; a < 3; ++a)
                        rr[a] = obj[b].r[a] * (1.0 + 0.15 * sin(two_pi * t / period + obj[b].ph[a]));
                    double dx = i - obj[b].cx, dy = j - obj[b].cy, dz = k - obj[b].cz;
                    double rho2 = (dx / rr[0]) * (dx / rr[0]) + (dy / rr[1]) * (dy / rr[1]) + (dz / rr[2]) * (dz / rr[2]);
                    if (rho2 > 1.0)
                        continue;
                    int erased = 0;
                    if (rho2 >= 0.49) {
                        double az = atan2(dy, dx);
                        if (az < 0)
                            az += two_pi;
                        for (int q = 0; q < nsect; ++q) {
                            double a0 = sect[((size_t)l * MAX_OBJ + b) * MAX_SECT + q];
                            double rel = az - a0;
                            if (rel < 0)
                                rel += two_pi;
                            if (rel < sect_width)
                                erased = 1;
                        }
                    }
                    if (!erased && obj[b].inten > val)
                        val = obj[b].inten;
                }
                val = val * drift + noise * gauss(seed, (uint64_t)o);
                double qv = floor(val + 0.5);
                if (qv < 0)
                    qv = 0;
                if (qv > 255)
                    qv = 255;
                h_i0[o] = qv / 255.;
            }
    }
    free(sect);
    return SS4D_OK;
}
