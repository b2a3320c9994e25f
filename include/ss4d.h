/*
 * ss4d.h — native C ABI of the GB300 semi-implicit subjective-surfaces /
 * mean-curvature-flow solver (4D, red-black SOR).
 *
 * Every entry point here replaces one function of the reference C programs
 * segmentation4D.c and mcf_4D.c / mcf_4D_openmp.c (88MARK08/4D-image-
 * segmentation-algorithm); the citation beside each declaration names it.
 * The reference works on process-global host arrays; this ABI works on
 * caller-owned DEVICE arrays with exactly the reference's volume layout:
 *
 *     double array of iMax*jMax*kMax*lMax voxels, index
 *     ((l*kMax + k)*jMax + j)*iMax + i   (x fastest)        segmentation4D.c:61-65
 *     one ghost voxel per side on every axis: iMax = nx + 2  segmentation4D.c:14
 *
 * and the reference's parameter names (struct ss4d_params).  A solver handle
 * owns the device workspaces the fast forms need (colour-split copies of u,
 * coefficient arrays, reduction buffers) and the CUDA stream every call is
 * issued on.  Calls are asynchronous with respect to the host except where a
 * result is returned by value (norms, stats): those synchronise the stream.
 *
 * No CPU fallback exists: without a CUDA device every compute call returns
 * SS4D_ERR_NO_DEVICE.  Reference-named wrappers over host arrays (a drop-in
 * for a reference main) live in ss4d_compat.h.
 */
#ifndef SS4D_H
#define SS4D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: ss4d_step_stats.near_tolerance; 3: .projected, SS4D_K_PROJECT */
#define SS4D_ABI_VERSION 3

typedef enum ss4d_status {
    SS4D_OK = 0,
    SS4D_ERR_INVALID = 1,     /* NULL pointer, bad size or parameter; the reference returns false (segmentation4D.c:100-103) */
    SS4D_ERR_ALLOC = 2,       /* a device/host allocation failed (reference: _allocateMem_ returns false) */
    SS4D_ERR_CUDA = 3,        /* a CUDA runtime call failed; text via ss4d_last_error() */
    SS4D_ERR_NONFINITE = 4,   /* the SOR residual became NaN or Inf */
    SS4D_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    SS4D_ERR_UNSUPPORTED = 6, /* combination not built (e.g. unknown arithmetic mode) */
    SS4D_ERR_NO_DEVICE = 7    /* no CUDA device visible */
} ss4d_status;

/* Arithmetic form of the SOR solve. */
typedef enum ss4d_arith {
    /* FP64 in the reference's expression order on the natural layout, three
     * passes per iteration like segmentation4D.c:228-309.  Slow; it is the
     * parity anchor (u agrees with the reference to rounding of pow()). */
    SS4D_ARITH_REFERENCE = 0,
    /* FP64 on a colour-split layout: fused residual, precomputed diagonal and
     * relaxation factor, whole sweep loop in one CUDA graph.  The plain form. */
    SS4D_ARITH_FP64 = 1,
    /* FP32 red-black sweeps on the correction equation, FP64 residual,
     * convergence test and refinement of u; same FP64 stopping tolerance. */
    SS4D_ARITH_MIXED = 2
} ss4d_arith;

/* Padded extents, as the reference's iMax, jMax, kMax, lMax globals
 * (segmentation4D.c:14).  Each must be >= 3; the product must stay below 2^31
 * like the reference's int indexing (segmentation4D.c:61-65). */
typedef struct ss4d_dims {
    int iMax, jMax, kMax, lMax;
} ss4d_dims;

/* The reference's tunables, same names and meaning (segmentation4D.c:45-58,
 * mcf_4D.c:25-33).  eps2 is used as eps^2 inside sqrt(|grad u|^2 + eps2). */
typedef struct ss4d_params {
    double K;                      /* edge-detector constant in g = 1/(1 + K s)           */
    double eps2;                   /* Evans-Spruck regularisation                          */
    double tau;                    /* time step                                            */
    double h;                      /* grid spacing                                         */
    double omega_c;                /* SOR relaxation of the time step                      */
    double gsTol;                  /* stop when sum r^2 h^4 <= gsTol                       */
    int    maxNoGSIteration;       /* SOR iteration cap per time step                      */
    int    maxNoOfTimeSteps;       /* driver loop cap (used by ss4d_seg_run)               */
    double segTol;                 /* driver stop on ||u^{n+1}-u^n||_2 (ss4d_seg_run)      */
    double sigma;                  /* presmoothing (implicit heat) step                    */
    double omega_sigma;            /* SOR relaxation of the presmoothing                   */
    double maxNoGSIteration_sigma; /* iteration cap of the presmoothing (a double, as in
                                      segmentation4D.c:56)                                  */
    double theta_img;              /* weight of the image gradient in g                    */
    double rho_thr;                /* weight of the thresholded-image gradient in g        */
    double ballRadius;             /* radius of the per-centre rescale balls              */
} ss4d_params;

/* Per-frame rescale centres (segmentation4D.c:38-39, no_of_centers/center_*),
 * flattened in (frame, centre) order: entries with the same l must be
 * consecutive and in the reference's centre order.  n == 0 and an all-ones
 * Mmask make the rescale the identity. */
typedef struct ss4d_balls {
    int n;
    const int *l;          /* frame index of each centre (1..lMax-2), host memory */
    const double *cx, *cy, *cz;
} ss4d_balls;

/* What one solve reports instead of the reference's printf
 * ("Mean square residue is %e and total number of RBSOR is %d"). */
typedef struct ss4d_step_stats {
    int    iterations;      /* SOR iterations z at loop exit (mixed: FP32 sweeps)     */
    int    status;          /* ss4d_status of the step                                */
    double residual;        /* sum r^2 h^4 at exit, in FP64                           */
    double first_residual;  /* residual after the first iteration                     */
    int    refinements;     /* mixed form: FP64 residual/refinement passes            */
    int    warm_started;    /* 1 when the learned predictor supplied the start        */
    float  ms;              /* device time of the call (CUDA events on the stream)    */
    int    near_tolerance;  /* 1 when a stop test saw |sum - gsTol| within nint * 2^-53
                               * gsTol: the reference's serial sum of the same terms
                               * could have decided that test the other way (one
                               * iteration more or fewer); reported, not corrected   */
    int    projected;       /* mixed form: 1 when the first FP32 round started from the
                               projection onto the previous steps' changes
                               (ss4d_solver_set_projection)                          */
} ss4d_step_stats;

typedef struct ss4d_solver ss4d_solver;

/* ---- library / device ------------------------------------------------- */
int         ss4d_abi_version(void);
const char *ss4d_last_error(void);            /* thread-local text of the last failure */
ss4d_status ss4d_device_count(int *count);    /* SS4D_ERR_NO_DEVICE when none visible   */

/* Solver handle.  `stream` is a cudaStream_t (NULL = legacy default stream).
 * Allocates nothing until a call needs it; all workspaces are sized from dims.
 * Replaces the allocation role of _allocateMem_ (segmentation4D.c:71-154)
 * for everything except the caller-visible arrays. */
ss4d_status ss4d_solver_create(const ss4d_dims *dims, ss4d_arith arith, void *stream,
                               ss4d_solver **out);
ss4d_status ss4d_solver_destroy(ss4d_solver *s);
ss4d_status ss4d_solver_set_stream(ss4d_solver *s, void *stream);
ss4d_status ss4d_solver_set_arith(ss4d_solver *s, ss4d_arith arith);
/* Tile schedule of the colour-split sweeps: k_block = depth of the k blocks
 * in the tile order (>= 1), max_grid caps the persistent grid (0 = as many
 * blocks as fit on the device).  Results do not depend on either. */
ss4d_status ss4d_solver_set_tiling(ss4d_solver *s, int k_block, int max_grid);
/* Block order of the mixed form's coefficient assembly (its faces and
 * coefficient kernels): 0 = frame by frame; planes >= 1 = in blocks of that
 * many k planes, each block's planes for every frame in turn (default 4).
 * Results do not depend on it. */
ss4d_status ss4d_solver_set_assembly_order(ss4d_solver *s, int planes);
/* Mixed form, segmentation steps: start the solve of step n from an
 * extrapolation in time instead of from u^n.  order 1: u^n + d_{n-1};
 * order 2: u^n + 2 d_{n-1} - d_{n-2}; order 3: u^n + 3 d_{n-1} - 3 d_{n-2}
 * + d_{n-3} (lower orders while fewer earlier steps exist), with d_m the
 * change u^{m+1} - u^m of an earlier step on this handle, kept in FP32;
 * 0 (default): off.  The FP64 stop rule is unchanged, so only the iteration
 * count depends on it.  With a warm-start network attached the network
 * predicts the correction left at the extrapolated start.  The history is
 * dropped by this call, by ss4d_solver_set_arith and by any other solve on
 * the handle.  No counterpart in the reference (each of its solves starts
 * from u^n). */
ss4d_status ss4d_solver_set_extrapolation(ss4d_solver *s, int order);
/* Mixed form with extrapolation of order 3: start each step's first FP32
 * round not from zero but from the combination of the last changes d_{n-1},
 * d_{n-2} and the extrapolation (d_{n-1}, d_{n-2} after two steps) whose
 * residual in the correction equation is least in the 2-norm (a projection
 * onto the previous solutions, Fischer 1998; enable 1, default 0).  The
 * FP64 stop rule is unchanged, so only the iteration count depends on it;
 * ss4d_step_stats.projected reports the steps that used it (batched solves:
 * ss4d_batch_set_projection).  No counterpart in the reference. */
ss4d_status ss4d_solver_set_projection(ss4d_solver *s, int enable);
/* Mixed form: relaxation factor of the FP32 sweeps on the correction
 * equation (0, the default: the step's omega_c).  Only the iteration count
 * depends on it: the stop rule is the FP64 residual of u.  No counterpart in
 * the reference. */
ss4d_status ss4d_solver_set_inner_omega(ss4d_solver *s, double omega);
/* Use (1) or bypass (0) the CUDA-graph form of the sweep loop (default 1). */
ss4d_status ss4d_solver_set_graph(ss4d_solver *s, int enable);
/* Per-kernel timing.  While enabled, the sweep loop runs host-driven (not
 * as a graph) and every launch of the kernels below is bracketed by CUDA
 * events on the handle's stream; totals accumulate until reset. */
typedef enum ss4d_kernel_kind {
    SS4D_K_SWEEP64 = 0,   /* FP64 red or black half-sweep with fused residual */
    SS4D_K_SWEEP32 = 1,   /* FP32 half-sweep of the correction equation       */
    SS4D_K_REFINE = 2,    /* FP64 refinement + residual pass (one colour)     */
    SS4D_K_ASSEMBLE = 3,  /* coefficient assembly                             */
    SS4D_K_PACK = 4,      /* natural <-> colour-split copies                  */
    SS4D_K_WARM = 5,      /* learned warm start: features, network, checks    */
    SS4D_K_PROJECT = 6,   /* start projected onto the previous steps' changes  */
    SS4D_K_COUNT = 7
} ss4d_kernel_kind;
ss4d_status ss4d_solver_set_timing(ss4d_solver *s, int enable);
ss4d_status ss4d_solver_kernel_time(const ss4d_solver *s, int kind, double *total_ms, long long *launches);
ss4d_status ss4d_solver_reset_timing(ss4d_solver *s);
/* Device bytes currently held by the handle. */
ss4d_status ss4d_solver_workspace_bytes(const ss4d_solver *s, size_t *bytes);
/* Kernel launches issued by this handle since creation (sweeps, passes,
 * reductions; a graph launch counts the kernels it contains). */
ss4d_status ss4d_solver_launch_count(const ss4d_solver *s, long long *count);

/* ---- hot-path entry points (device arrays, reference layout) ---------- */

/* _reflection4Ddata_ (segmentation4D.c:826-864): Neumann ghost layer. */
ss4d_status ss4d_reflect(ss4d_solver *s, double *d_img);

/* _presmoothStep_ (segmentation4D.c:337-409): one implicit heat step
 * (I - sigma*Laplace) v = img solved in place by red-black SOR with omega_sigma;
 * d_scratch receives the copy of the input that the reference keeps in its
 * global prev_u (may be NULL: the handle then uses its own).  The reference
 * and FP64 forms keep the reference's FP64 rounding bit for bit; the mixed
 * form iterates in float-float arithmetic (about 48 significant bits, within
 * 1e-13 of it), as does its ss4d_edge_detector. */
ss4d_status ss4d_presmooth_step(ss4d_solver *s, const ss4d_params *p, double *d_img,
                                double *d_scratch, ss4d_step_stats *stats);

/* _presmoothStepEXP_ (segmentation4D.c:410-444), the explicit smoother the
 * reference declares next to _presmoothStep_: d_scratch (the reference's
 * prev_u; NULL = internal) <- d_img, reflect d_img, then timeStepsNum times
 * d_img <- (1 - 8c) prev + c * (sum of prev's 8 neighbours), c = sigma/h^2,
 * over i = 1 .. iMax-3 (as the reference's loop) and the interior j, k, l,
 * and reflect d_img.  As in the reference, prev is not refreshed between the
 * steps, so any timeStepsNum >= 1 gives the result of one step.
 * Asynchronous on the handle's stream. */
ss4d_status ss4d_presmooth_explicit(ss4d_solver *s, const ss4d_params *p, int timeStepsNum,
                                    double *d_img, double *d_scratch);

/* A true Gaussian G_sigma, an option beside the reference's "G_sigma"
 * (the implicit heat step of ss4d_presmooth_step; no counterpart in the
 * reference): d_img is convolved axis by axis (x, y, z, t) with the
 * normalised taps w_m = exp(-m^2 / (2 sigma_a^2)) / sum, |m| <= R_a =
 * ceil(3 sigma_a) (sigma_a == 0 leaves axis a alone), over the interior
 * voxels, the volume mirrored about its faces as the reference's reflection
 * mirrors it (ghost 0 = voxel 1); then the ghost layer is set by that
 * reflection.  Each tap sum runs in order of m, a fused multiply-add per
 * tap, in FP64 in every arithmetic form.  R_a must not
 * exceed SS4D_GAUSS_MAX_RADIUS.  d_scratch (NULL = internal) is overwritten. */
#define SS4D_GAUSS_MAX_RADIUS 32
ss4d_status ss4d_gaussian_smooth(ss4d_solver *s, const double sigma[4], double *d_img, double *d_scratch);

/* The edge detector's second half (segmentation4D.c:594-821, _gFunction_
 * :67-70): the 8 face g values from images already smoothed (by
 * ss4d_gaussian_smooth, for instance), in the handle's arithmetic form as
 * ss4d_edge_detector computes them.  d_i0_thr may be NULL when rho_thr == 0. */
ss4d_status ss4d_gfaces(ss4d_solver *s, const ss4d_params *p, const double *d_i0, const double *d_i0_thr,
                        double *const d_g[8]);

/* _gf_inputImage_plus_thresholdedImage_ (segmentation4D.c:582-823): presmooth
 * d_i0 and d_i0_thr in place, then the 8 face values of the edge detector
 * g_f = 1/(1 + K (theta_img |grad I0|_f^2 + rho_thr |grad Ithr|_f^2)) into
 * d_g[0..7] = g_e, g_w, g_n, g_s, g_t, g_b, g_fw, g_bw.  d_i0_thr may be NULL
 * when rho_thr == 0 (its presmoothing is then skipped).  d_scratch plays the
 * reference's prev_u as in ss4d_presmooth_step (may be NULL). */
ss4d_status ss4d_edge_detector(ss4d_solver *s, const ss4d_params *p, double *d_i0,
                               double *d_i0_thr, double *d_scratch, double *const d_g[8]);

/* _gs_coefficients_ (segmentation4D.c:446-580) with d_g != NULL, or
 * _gs_coefficients_mcf (mcf_4D.c:208-342) with d_g == NULL: the 8 co-volume
 * coefficients e, w, n, s, t, b, fw, bw of every interior voxel. */
ss4d_status ss4d_gs_coefficients(ss4d_solver *s, const ss4d_params *p, const double *d_u,
                                 const double *const d_g[8], double *const d_coef[8]);

/* The red-black SOR loop of _segTimeStep_ (segmentation4D.c:228-309) on
 * given coefficients: solves (1 + c sum a) u - c sum a u_nb = prev, c = tau/h^2,
 * from the current d_u, until sum r^2 h^4 <= gsTol or maxNoGSIteration. */
ss4d_status ss4d_sor_solve(ss4d_solver *s, const ss4d_params *p, double *d_u,
                           const double *d_prev_u, const double *const d_coef[8],
                           ss4d_step_stats *stats);

/* _segTimeStep_ (segmentation4D.c:215-315): prev_u <- u, coefficients from u
 * and the face g, SOR solve, then _rescale4DdataToZeroOne_ with d_Mmask/balls.
 * d_prev_u may be NULL (not returned); d_Mmask may be NULL (all ones). */
ss4d_status ss4d_seg_time_step(ss4d_solver *s, const ss4d_params *p, double *d_u,
                               double *d_prev_u, const double *const d_g[8],
                               const double *d_Mmask, const ss4d_balls *balls,
                               ss4d_step_stats *stats);

/* ss4d_seg_time_step on HOST arrays, as a reference driver calls
 * _segTimeStep_: h_u (page-locked, read and written), d_u its device
 * mirror; h_prev (page-locked, may be NULL) receives the step's input u on
 * host threads, as the reference's step begins (segmentation4D.c:224);
 * h_Mmask (page-locked, NULL = all ones) goes up into d_Mmask beside the
 * solve, since only the final rescale reads it.  In the FP64 and mixed forms
 * u goes up in SS4D_HOST_CHUNKS chunks of frames on the handle's side stream
 * while the step's first kernels (the pack; in the mixed form the whole
 * coefficient assembly) work on the frames that have arrived, and comes down
 * in chunks as the unpack and the rescale finish them.  In the mixed form
 * the SOR loop pauses after each round of FP32 sweeps, and u formed from
 * that round goes down while the refinement pass decides whether it meets
 * gsTol; when it does, that download is the result, otherwise the loop goes
 * on and u goes down again at its end.  The results equal
 * ss4d_seg_time_step's.  Returns when h_u holds the result. */
#define SS4D_HOST_CHUNKS 16
ss4d_status ss4d_seg_time_step_host(ss4d_solver *s, const ss4d_params *p, double *h_u, double *d_u,
                                    double *h_prev, const double *h_Mmask, double *d_Mmask,
                                    const double *const d_g[8], const ss4d_balls *balls,
                                    ss4d_step_stats *stats);

/* _mcfTimeStep (mcf_4D.c:102-205): prev_u <- u, coefficients (g == 1), exact
 * Dirichlet ghosts at t = tau*numberOfTimeStep, SOR solve. */
ss4d_status ss4d_mcf_time_step(ss4d_solver *s, const ss4d_params *p, int numberOfTimeStep,
                               double *d_u, double *d_prev_u, ss4d_step_stats *stats);

/* _rescale4DdataToZeroOne_ (segmentation4D.c:1020-1104). */
ss4d_status ss4d_rescale_to_zero_one(ss4d_solver *s, const ss4d_params *p, double *d_img,
                                     const double *d_Mmask, const ss4d_balls *balls);

/* The same rescale without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory: a host application that owns the whole GPU memory budget
 * through its own pool and forbids further cudaMalloc, or a per-frame loop
 * that must not pay cudaMalloc's implicit device synchronisation.  It takes
 * no solver handle (a handle allocates its workspaces); the centre table and
 * the per-frame index tables are staged in a fixed-size array inside this
 * library (32 KB per device, kept until the process exits), which limits it
 * to SS4D_NOALLOC_MAX_BALLS centres and lMax <= SS4D_NOALLOC_MAX_FRAMES;
 * larger inputs return SS4D_ERR_INVALID.  The first call on a device looks
 * up that array's device address (cudaGetSymbolAddress).  All calls share
 * the one array, so calls
 * whose GPU work overlaps (different streams, or different host threads
 * without ordering) race on it; issue them in one stream.  `stream` is a
 * cudaStream_t (NULL = legacy default stream); the call is asynchronous. */
#define SS4D_NOALLOC_MAX_BALLS 1024
#define SS4D_NOALLOC_MAX_FRAMES 1024
ss4d_status ss4d_rescale_to_zero_one_noalloc(const ss4d_dims *dims, const ss4d_params *p, double *d_img,
                                             const double *d_Mmask, const ss4d_balls *balls, void *stream);

/* ---- file formats (segmentation4D.c:1149-1324, segmentation4D_mpi.c:
 * 1424-1482): a frame file is a VTK STRUCTURED_POINTS header of ten lines
 * followed by nx*ny*nz unsigned bytes, x fastest; a centre file lists the
 * balls of one frame.  The files are read and written on the host; the
 * byte <-> double conversion of a frame runs on the GPU, so a frame crosses
 * the bus as one byte per voxel. ----------------------------------------- */
/* Write the reference's header (DIMENSIONS, ORIGIN, SPACING as it prints
 * them) and the bytes. */
ss4d_status ss4d_vtk_write_frame(const char *path, int nx, int ny, int nz, const double origin[3],
                                 const double spacing[3], const uint8_t *h_bytes);
/* Skip ten header lines as _load3dDataArrayVTK_ does and read nx*ny*nz
 * bytes; SS4D_ERR_INVALID if the file holds fewer. */
ss4d_status ss4d_vtk_read_frame(const char *path, int nx, int ny, int nz, uint8_t *h_bytes);
/* The centre-file parse of _readData_ (with _readMetaData_ and
 * _readNumberFromFile_): *n points, each centre (double)(int)(x / spacing +
 * 0.5) per axis; SS4D_ERR_INVALID if there are more than max_points. */
ss4d_status ss4d_vtk_read_centers(const char *path, const double spacing[3], int max_points, double *cx,
                                  double *cy, double *cz, int *n);
/* Interior of frame l (1..lMax-2) of d_img = byte / 255. */
ss4d_status ss4d_frame_from_bytes(ss4d_solver *s, double *d_img, int l, const uint8_t *d_bytes);
/* Interior of frame l to bytes: mode 0 (unsigned char)(255 v + 0.5) as
 * _writeData_ writes (clamped to 0..255; the reference's conversion is
 * undefined outside), mode 1 the mask v >= 0.5 of _writeData_mpi_. */
ss4d_status ss4d_frame_to_bytes(ss4d_solver *s, const double *d_img, int l, int mode, uint8_t *d_bytes);

/* ---- initial segmentation (the reference main's pipeline before the time
 * steps, segmentation4D.c:1383-1393) ------------------------------------ */
/* _get4DMax_ (segmentation4D.c:876-895): largest interior value, the search
 * starting from 0. Synchronises. */
ss4d_status ss4d_max4d(ss4d_solver *s, const double *d_img, double *out);
/* _get3DMinWithinR_ / _get3DMaxWithinR_ (segmentation4D.c:897-969): minimum
 * (from 100000) and maximum (from 0) of frame l over the voxels within
 * distance R of (cx, cy, cz).  SS4D_ERR_INVALID if the ball's box leaves the
 * array.  Synchronises. */
ss4d_status ss4d_ball_min_max(ss4d_solver *s, const double *d_img, int l, double cx, double cy, double cz,
                              double R, double *min, double *max);
/* _locallyThreshold4Ddata_ (segmentation4D.c:971-1018): for each ball
 * (radius ballRadius) the level alpha*min + beta*max of d_in inside it;
 * d_thr becomes the global maximum of d_in where d_in exceeds the level
 * inside the ball and is left unchanged elsewhere.  alpha and beta are the
 * reference's globals of the same names. */
ss4d_status ss4d_local_threshold(ss4d_solver *s, double alpha, double beta, double ballRadius,
                                 const double *d_in, double *d_thr, const ss4d_balls *balls);
/* _generate4DsegmFunct_ (segmentation4D.c:1106-1147): inside each ball's box
 * (half-width ballRadius + 0.5) and within distance 12 of the centre (the
 * reference's fixed radius), u = max(u, |1/(r + 0.5) - 1/12.5|) and
 * Mmask = 1. */
ss4d_status ss4d_generate_segm_function(ss4d_solver *s, double ballRadius, double *d_u, double *d_Mmask,
                                        const ss4d_balls *balls);

/* Level-set threshold to a mask, as _writeData_mpi_ (segmentation4D_mpi.c:
 * 1470-1478): mask = (u >= level) for every interior voxel, written frame by
 * frame in (l, k, j, i) order, nx*ny*nz*nt bytes of 0/1.  With normalise != 0
 * the level is taken relative to the interior range: min + level*(max-min). */
ss4d_status ss4d_threshold_mask(ss4d_solver *s, const double *d_u, double level, int normalise,
                                uint8_t *d_mask);

/* _l2norm_ (segmentation4D.c:194-213) / _l2norm_mcf (mcf_4D.c:81-100):
 * sqrt(sum over ALL padded voxels of (a-b)^2 h^4). Synchronises. */
ss4d_status ss4d_l2norm(ss4d_solver *s, double h, const double *d_a, const double *d_b,
                        double *out);
/* _mass4D_ (segmentation4D.c:317-335). Synchronises. */
ss4d_status ss4d_mass(ss4d_solver *s, double h, const double *d_a, double *out);

/* _set4DBoundaryToExactValues_mcf (mcf_4D.c:344-443) and _exactSolution_mcf
 * (mcf_4D.c:444-461): u = (x^2+y^2+z^2+w^2-1)/6 + t on [-1.25,1.25]^4. */
ss4d_status ss4d_mcf_set_boundary_exact(ss4d_solver *s, double h, double t, double *d_u);
ss4d_status ss4d_mcf_exact_solution(ss4d_solver *s, double h, double t, double *d_out);

/* ---- batched volumes --------------------------------------------------- */
/* Many independent volumes, of different sizes and parameters, advanced
 * together in the plain FP64 form (default) or the mixed form
 * (ss4d_batch_set_arith).  The SOR loop of all volumes is ONE persistent
 * launch (a co-resident grid whose phases, the half-sweeps and in the mixed
 * form the refinement passes, walk the concatenated tiles of all volumes,
 * with a bounded grid barrier between phases: SS4D_ERR_TIMEOUT if one gives
 * up); ss4d_batch_set_persistent(b, 0) runs the same phases as kernels of a
 * CUDA graph's while loop instead.  Each volume keeps its own stopping test
 * (sum r^2 h^4 <= its gsTol, or its maxNoGSIteration) and once it has
 * stopped its tiles return at once.  In the mixed form each volume's
 * coefficient assembly also forms its step's first refinement pass, as
 * ss4d_seg_time_step does.  The
 * reference runs one volume per process, so these entry points have no
 * counterpart there; per volume the arithmetic is that of ss4d_seg_time_step
 * in the same form without the rescale (no centres, Mmask == 1).  At most
 * SS4D_BATCH_MAX_VOLUMES volumes. */
#define SS4D_BATCH_MAX_VOLUMES 64
typedef struct ss4d_batch ss4d_batch;
ss4d_status ss4d_batch_create(int n, const ss4d_dims *dims, void *stream, ss4d_batch **out);
ss4d_status ss4d_batch_destroy(ss4d_batch *b);
ss4d_status ss4d_batch_set_graph(ss4d_batch *b, int enable);
/* 1 (default): the SOR loop as one persistent launch; 0: as the graph's
 * while loop (or host-driven, with ss4d_batch_set_graph(b, 0)).  Results do
 * not depend on it except through the residual's summation order. */
ss4d_status ss4d_batch_set_persistent(ss4d_batch *b, int enable);
/* Test of the timeout path, no fault: with enable the persistent loop's grid
 * barrier starts with its arrival count beyond the grid, so no arrival
 * completes it; every block's first wait runs out after about a second and
 * the step returns SS4D_ERR_TIMEOUT with the context usable.  The volumes'
 * states after such a step are undefined. */
ss4d_status ss4d_batch_set_test_withhold_barrier(ss4d_batch *b, int enable);
/* Arithmetic form of the batched steps: SS4D_ARITH_FP64 (the default) or
 * SS4D_ARITH_MIXED, each volume as ss4d_seg_time_step does it in that form
 * (mixed: float-float assembly, FP32 correction sweeps, FP64 refinement and
 * the FP64 stop test), every loop kernel one launch for all volumes. */
ss4d_status ss4d_batch_set_arith(ss4d_batch *b, ss4d_arith arith);
/* Mixed form: start every volume's step from the extrapolation of order
 * 0..3 of its earlier steps (ss4d_solver_set_extrapolation per volume). */
ss4d_status ss4d_batch_set_extrapolation(ss4d_batch *b, int order);
/* Mixed form with extrapolation of order 3: every volume's first FP32 round
 * starts from its projected start (ss4d_solver_set_projection per volume). */
ss4d_status ss4d_batch_set_projection(ss4d_batch *b, int enable);
/* Tile shape of volume v: xt threads along x (power of two, 8..256; 0 =
 * automatic) and k-block depth k_block (>= 1).  Results do not depend on it. */
ss4d_status ss4d_batch_set_shape(ss4d_batch *b, int v, int xt, int k_block);
/* Autotuner: for every volume, time candidate tile shapes on that volume's
 * own sweeps (coefficients of d_u[v], d_g[8v..8v+7]; u is not modified) and
 * keep the fastest.  xt_out/kb_out (n entries each, may be NULL) receive the
 * chosen shapes. */
ss4d_status ss4d_batch_autotune(ss4d_batch *b, const ss4d_params *p, double *const *d_u,
                                const double *const *d_g, int *xt_out, int *kb_out);
/* One time step of every volume: parameters p[v], u d_u[v] (updated in
 * place), edge-detector faces d_g[8v + f]; stats[v] (may be NULL). */
ss4d_status ss4d_batch_seg_time_step(ss4d_batch *b, const ss4d_params *p, double *const *d_u,
                                     const double *const *d_g, ss4d_step_stats *stats);

/* ---- learned warm start ------------------------------------------------ */
/* A 4-layer convolutional network (3x3x3 kernels over each frame, 16 input
 * features -> 24 -> 24 -> 24 hidden channels with ReLU -> 1, BF16 weights and
 * activations, FP32 accumulation) that predicts the first correction
 * d = A^-1 r0 of a mixed-form time step from the residual r0 = b - A u^n
 * (normalised by its RMS s, at frames l and l+-1), the step's coefficients
 * (c a_f / diag, 1/diag), the first Jacobi iterate, gbar, u^n and the
 * presmoothed image; u^n + s * prediction starts the FP32 rounds and SOR
 * finishes to the unchanged FP64 tolerance.  When the prediction does not
 * lower the correction equation's residual the step starts from zero instead.
 * Training and inference are this library's own kernels.  No counterpart in
 * the reference.  Feature tensors are BF16 and channel-group planar,
 * [F][2][nz][ny][nx][8] (interior voxels, F frames; channels 0-7 in the first
 * plane of a frame, 8-15 in the second), the layout the tensor-core
 * convolutions load; parameters are FP32, per layer weights [27][cout][cin]
 * (tap = 9 dz + 3 dy + dx) then biases [cout]. */
typedef struct ss4d_wsnet ss4d_wsnet;
size_t ss4d_wsnet_param_count(void);
ss4d_status ss4d_wsnet_create(void *stream, ss4d_wsnet **out);
ss4d_status ss4d_wsnet_destroy(ss4d_wsnet *n);
ss4d_status ss4d_wsnet_set_stream(ss4d_wsnet *n, void *stream);
ss4d_status ss4d_wsnet_init(ss4d_wsnet *n, uint64_t seed);
ss4d_status ss4d_wsnet_set_params(ss4d_wsnet *n, const float *h_params);
ss4d_status ss4d_wsnet_get_params(ss4d_wsnet *n, float *h_params);
/* prediction [F][nz][ny][nx] FP32; asynchronous on the network's stream.  A
 * convolution whose bounded wait (about a second) gave up makes the whole
 * prediction NaN, which the warm start's check discards. */
ss4d_status ss4d_wsnet_forward(ss4d_wsnet *n, const void *d_x0, int nx, int ny, int nz, int nf, float *d_out);
/* Synchronise the network's stream; SS4D_ERR_TIMEOUT if a convolution of the
 * last forward (and any backward after it) gave up a wait, else SS4D_OK. */
ss4d_status ss4d_wsnet_check(ss4d_wsnet *n);
/* Test of the timeout path, no fault: with enable the convolutions issue no
 * halo loads, so each one's waits run out after about a second and its
 * output is made NaN. */
ss4d_status ss4d_wsnet_set_test_withhold_loads(ss4d_wsnet *n, int enable);
/* one Adam step on a batch of crops (frames F of nx*ny*nz voxels): mean
 * squared error against d_target over voxels at least `margin` from a crop's
 * border; lr == 0 only evaluates; d_grad (may be NULL) gets the gradient. */
ss4d_status ss4d_wsnet_train_step(ss4d_wsnet *n, const void *d_x0, const float *d_target, int nx, int ny,
                                  int nz, int nf, int margin, float lr, float *loss_out, float *d_grad);
/* Features of the time step from d_u (training data): assembles the step's
 * system, computes r0 in FP64 and writes the feature tensor of all nt frames
 * to d_x0 and s to *sigma.  d_u is not modified. */
ss4d_status ss4d_ws_features(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *const d_g[8],
                             const double *d_i0, void *d_x0, double *sigma);
/* Attach a network (NULL detaches) to a solver; d_i0 is the presmoothed
 * image.  Used by SS4D_ARITH_MIXED segmentation steps. */
ss4d_status ss4d_solver_set_warm_start(ss4d_solver *s, ss4d_wsnet *n, const double *d_i0);
/* Run the attached network in a segmentation step only when the handle's
 * previous mixed step needed at least min_iterations FP32 sweeps (0, the
 * default: every step).  The network costs about as much as a fixed number
 * of sweeps; once the extrapolated start leaves fewer than that to save,
 * the gate keeps it idle.  The first step after attaching always runs it. */
ss4d_status ss4d_solver_set_warm_start_gate(ss4d_solver *s, int min_iterations);

/* ---- one volume split across ranks by frames (t-slabs) ----------------
 * The reference's MPI program (segmentation4D_mpi.c) splits the frames of one
 * volume into slabs, one per process, exchanges one ghost frame with each
 * neighbour after every half-sweep (_communication_mpi_, :485-526; called at
 * :330 and :361), sums the residual over all processes every iteration
 * (MPI_Allreduce, :386) and picks the red voxels by the global index sum
 * (:307, :338).  Here a rank holds its slab as an ordinary padded volume
 * (lMax = its frames + 2, frame 0 and lMax-1 the ghosts) and the caller
 * supplies the communication (NCCL, MPI, ...) as two callbacks; the library
 * runs the loop.  Slabs are cut by ss4d_slab_partition so that every slab
 * starts on an even global frame offset: the red voxels of a slab are then
 * those with (i + j + k + l_local) even, the global red set, on every rank
 * (the reference's offset N * rank is wrong for uneven slabs). */

/* Cut nt frames into nranks slabs: rank r holds global interior frames
 * first[r] .. first[r] + count[r] - 1 (1-based).  Every slab but the last has
 * an even number of frames; SS4D_ERR_INVALID when nt < 2 nranks - 1. */
ss4d_status ss4d_slab_partition(int nt, int nranks, int *first, int *count);

typedef struct ss4d_slab_comm {
    void *ctx;
    /* Exchange the ghost frames of u (lMax frames of frame_elems doubles):
     * send frame 1 to the rank below and frame lMax-2 to the rank above;
     * receive the rank below's last interior frame into frame 0 and the rank
     * above's first into frame lMax-1.  At the volume's ends nothing is sent
     * or received (those ghosts keep the boundary values).  u is device
     * memory for the GPU entry points, whose work is queued on `stream` (a
     * cudaStream_t; NULL for host work): the exchange must come after it in
     * that stream (an NCCL call on it) or wait for it.  Returns 0 on success. */
    int (*exchange)(void *ctx, double *u, long long frame_elems, int lMax, void *stream);
    /* *value <- the sum of *value over all ranks (host memory).  0 on success. */
    int (*allreduce_sum)(void *ctx, double *value);
} ss4d_slab_comm;

/* The local work of one slab's SOR loop: a half-sweep of colour 0 (red) or 1
 * (black) over the slab's interior, and the slab's part of the residual
 * sum r^2 h^4 over its interior.  Returns 0 on success. */
typedef struct ss4d_slab_ops {
    void *ctx;
    int (*half_sweep)(void *ctx, int colour);
    int (*residual)(void *ctx, double *partial);
    double *u;              /* the slab's u, handed to the exchange */
    long long frame_elems;  /* iMax * jMax * kMax */
    int lMax;               /* the slab's padded frame count */
    void *stream;           /* where the ops' work is queued (cudaStream_t; NULL: host) */
} ss4d_slab_ops;

/* The slab SOR loop of _segTimeStep_mpi_ (segmentation4D_mpi.c:297-387):
 * repeat { red; exchange; black; exchange; residual; sum over ranks } while
 * sum > gsTol && z < maxNoGSIteration.  nint_global = the whole volume's
 * interior voxel count (the near_tolerance band).  Host code only: the ops
 * decide where the work runs. */
ss4d_status ss4d_slab_sor_loop(const ss4d_slab_ops *ops, const ss4d_slab_comm *comm, const ss4d_params *p,
                               long long nint_global, ss4d_step_stats *stats);

/* ss4d_slab_sor_loop on the GPU: the solver's dims are the slab's; d_u,
 * d_prev_u, d_coef in its natural layout (device).  The half-sweeps and the
 * residual are the reference-order FP64 kernels (SS4D_ARITH_REFERENCE), so
 * slab iterates equal the single-volume iterates bit for bit. */
ss4d_status ss4d_slab_sor_solve(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *d_prev_u,
                                const double *const d_coef[8], const ss4d_slab_comm *comm, long long nint_global,
                                ss4d_step_stats *stats);

/* _segTimeStep_mpi_ (segmentation4D_mpi.c:282-397) for one slab: exchange
 * u's ghost frames, prev_u <- u, coefficients (reference order) from u and
 * the slab's g faces, ss4d_slab_sor_solve, then the rescale of the slab's
 * frames (d_Mmask may be NULL; balls with frame indices local to the slab).
 * d_prev_u may be NULL (the handle's own). */
ss4d_status ss4d_slab_seg_time_step(ss4d_solver *s, const ss4d_params *p, double *d_u, double *d_prev_u,
                                    const double *const d_g[8], const double *d_Mmask, const ss4d_balls *balls,
                                    const ss4d_slab_comm *comm, long long nint_global, ss4d_step_stats *stats);

/* ---- memory helpers (used by the reference-named layer) --------------- */
/* Device / pinned-host allocations and copies on the handle's stream.  They
 * exist so that C callers without the CUDA headers (ss4d_compat.c) can mirror
 * host arrays; copies between pinned host and device are asynchronous. */
ss4d_status ss4d_dev_alloc(size_t bytes, void **out);
ss4d_status ss4d_dev_free(void *p);
ss4d_status ss4d_host_alloc(size_t bytes, void **out);   /* page-locked */
ss4d_status ss4d_host_free(void *p);
ss4d_status ss4d_copy_to_device(ss4d_solver *s, void *d_dst, const void *h_src, size_t bytes);
ss4d_status ss4d_copy_to_host(ss4d_solver *s, void *h_dst, const void *d_src, size_t bytes);
/* Host -> device copy on the handle's side stream, after the work already
 * queued on the handle's stream, so that it overlaps the calls that follow;
 * ss4d_join_side makes the handle's stream wait for the side copies issued
 * so far.  h_src must be page-locked for the copy to run asynchronously. */
ss4d_status ss4d_copy_to_device_side(ss4d_solver *s, void *d_dst, const void *h_src, size_t bytes);
ss4d_status ss4d_join_side(ss4d_solver *s);
ss4d_status ss4d_copy_device(ss4d_solver *s, void *d_dst, const void *d_src, size_t bytes);
ss4d_status ss4d_synchronize(ss4d_solver *s);

/* ---- synthetic scenes (host; the same generator feeds every test) ----- */
/* Writes the padded image i0 (intensities/255, as the reference loader,
 * segmentation4D.c:1320) and the initial u0 of scene `kind`
 * (1 = single deforming ellipsoid, 2 = large ellipsoid with two erased
 * sectors, 3 = multi-object drifting scene) for interior nx,ny,nz,nt. */
ss4d_status ss4d_scene_generate(int kind, int nx, int ny, int nz, int nt, uint64_t seed,
                                double *h_i0, double *h_u0, int nthreads);

#ifdef __cplusplus
}
#endif
#endif /* SS4D_H */
