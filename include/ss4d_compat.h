/*
 * ss4d_compat.h — the reference's own entry points and globals, backed by the
 * GB300 solver.
 *
 * Two libraries, one per reference program, because the reference programs
 * define the same global names (u, iMax, e, ...) and cannot share a link unit:
 *
 *   libss4d_seg.so  replaces segmentation4D.c  (prototypes: segmentation4D.h:8-62)
 *   libss4d_mcf.so  replaces mcf_4D.c / mcf_4D_openmp.c (prototypes: mcf_4D.h:8-23)
 *
 * A reference driver (its main(), or any harness written against those
 * headers) links against one of them unchanged: it sets the same globals
 * (iMax..lMax, tau, h, K, eps2, omega_c, gsTol, maxNoGSIteration, sigma,
 * omega_sigma, maxNoGSIteration_sigma, theta_img, rho_thr, ballRadius,
 * no_of_centers, center_x/y/z ...), calls _allocateMem_(), fills the host
 * arrays and calls the same functions.
 *
 * Host arrays are page-locked copies of device arrays.  Every call uploads
 * the caller-visible arrays it reads (u, prev_u, i0, Mmask, the image it is
 * given) and downloads the ones it writes, so host reads and writes between
 * calls behave as with the reference.  The coefficient arrays e..bw and the
 * edge-detector arrays g_e..g_bw are produced and consumed on the device;
 * their host copies are refreshed by ss4d_compat_sync_host(), or after every
 * call when the environment variable SS4D_COMPAT_STRICT=1 is set.
 * SS4D_ARITH=reference|fp64|mixed selects the arithmetic form (default fp64);
 * with mixed, SS4D_EXTRAPOLATE=1, 2 or 3 starts each step from the extrapolation
 * of that order of the earlier steps (ss4d_solver_set_extrapolation), and with
 * order 3 SS4D_PROJECT=1 starts each step's first FP32 round from the
 * projection onto the earlier changes (ss4d_solver_set_projection).
 *
 * Behaviour the reference leaves undefined is an error here instead:
 * a rescale ball whose box leaves the array makes _rescale4DdataToZeroOne_
 * return false (the reference reads out of bounds, segmentation4D.c:1043).
 */
#ifndef SS4D_COMPAT_H
#define SS4D_COMPAT_H

#include <stdbool.h>
#include <stdio.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- libss4d_seg.so: segmentation4D.h ---------------------------------- */
bool _allocateMem_(void);                                               /* segmentation4D.c:71   */
bool _deallocateMem_(void);                                             /* segmentation4D.c:155  */
double _l2norm_(double *a, double *b);                                  /* segmentation4D.c:194  */
bool _gs_coefficients_(void);                                           /* segmentation4D.c:446  */
bool _segTimeStep_(void);                                               /* segmentation4D.c:215  */
bool _presmoothStep_(double *u);                                        /* segmentation4D.c:337  */
void _presmoothStepEXP_(double *u);                                     /* segmentation4D.c:410  */
bool _rescale4DdataToZeroOne_(double *imagePtr);                        /* segmentation4D.c:1020 */
bool _gf_inputImage_plus_thresholdedImage_(double *i0, double *i0_thr); /* segmentation4D.c:582  */
void _copy4DdataFromSrcToDest_(double *srcDataPtr, double *destDataPtr);/* segmentation4D.c:866  */
int ijkl(int i, int j, int k, int l);                                   /* segmentation4D.c:61   */
double _gFunction_(double value, double coef);                          /* segmentation4D.c:67   */
bool _reflection4Ddata_(double *u);                                     /* segmentation4D.c:826  */
double _mass4D_(double *a);                                             /* segmentation4D.c:317  */
double _get4DMax_(double *imagePtr);                                    /* segmentation4D.c:876  */
double _get3DMinWithinR_(double *imagePtr, int l, double center_x, double center_y,
                         double center_z, double R);                    /* segmentation4D.c:897  */
double _get3DMaxWithinR_(double *imagePtr, int l, double center_x, double center_y,
                         double center_z, double R);                    /* segmentation4D.c:934  */
bool _locallyThreshold4Ddata_(double *inputImagePtr, double *thresholdedImagePtr); /* segmentation4D.c:971 */
bool _generate4DsegmFunct_(double *segmFuntionPtr);                     /* segmentation4D.c:1106 */
void _readData_(double *inputImage, unsigned char *fileDirectory);      /* segmentation4D.c:1149 */
bool _writeData_(double *array4DPtr, unsigned char *pathPtr);           /* segmentation4D.c:1217 */
void _readNumberFromFile_(char *dim, FILE *input_file);                 /* segmentation4D.c:1262 */
void _readMetaData_(FILE *input_file);                                  /* segmentation4D.c:1275 */
bool _load3dDataArrayVTK_(double *imageDataPtr, int l, unsigned char *pathPtr); /* segmentation4D.c:1289 */

/* ---- libss4d_mcf.so: mcf_4D.h ------------------------------------------- */
bool _allocateMem_mcf(void);                                            /* mcf_4D.c:42   */
bool _deallocateMem_mcf(void);                                          /* mcf_4D.c:65   */
double _l2norm_mcf(double *a, double *b);                               /* mcf_4D.c:81   */
bool _gs_coefficients_mcf(void);                                        /* mcf_4D.c:208  */
bool _mcfTimeStep(void);                                                /* mcf_4D.c:102  */
bool _set4DBoundaryToExactValues_mcf(double t);                         /* mcf_4D.c:344  */
void _exactSolution_mcf(double t);                                      /* mcf_4D.c:444  */
void _copy4DdataFromSrcToDest_mcf(double *src, double *dst);            /* mcf_4D.c:463  */

/* ---- additions of this library (both) ---------------------------------- */
/* Download e..bw (and g_e..g_bw in libss4d_seg.so) into the host arrays. */
bool ss4d_compat_sync_host(void);
/* The statistics of the last SOR solve (iterations, residual, device ms). */
struct ss4d_step_stats;
bool ss4d_compat_last_stats(struct ss4d_step_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* SS4D_COMPAT_H */
