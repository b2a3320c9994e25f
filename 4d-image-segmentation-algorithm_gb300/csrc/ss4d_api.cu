// ss4d_api.cu — the extern "C" ABI of include/ss4d.h: solver handles,
// workspaces, the SOR loop drivers (host loop and CUDA-graph while loop) and
// argument checking.  All device work is issued on the handle's stream.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <thread>
#include <vector>

#include "ss4d_kernels.cuh"

using namespace ss4d;

// ---------------------------------------------------------------------------
// errors

static thread_local char g_err[512] = "";

static void set_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

#define CK(call)                                                                                                   \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);                   \
            return e_ == cudaErrorMemoryAllocation ? SS4D_ERR_ALLOC                                                \
                                                   : (e_ == cudaErrorNoDevice ? SS4D_ERR_NO_DEVICE : SS4D_ERR_CUDA); \
        }                                                                                                          \
    } while (0)

#define CKS(expr)                                                                                                  \
    do {                                                                                                           \
        ss4d_status s_ = (expr);                                                                                   \
        if (s_ != SS4D_OK)                                                                                         \
            return s_;                                                                                             \
    } while (0)

#define REQ(cond, msg)                                                                                             \
    do {                                                                                                           \
        if (!(cond)) {                                                                                             \
            set_err("invalid argument: %s", msg);                                                                  \
            return SS4D_ERR_INVALID;                                                                               \
        }                                                                                                          \
    } while (0)

// error text for entry points defined in other translation units
void ss4d::set_error_text(const char *msg)
{
    snprintf(g_err, sizeof g_err, "%s", msg);
}

// the same for this library's C translation units (ss4d_vtk.c)
extern "C" void ss4d_set_error_text_c(const char *msg)
{
    snprintf(g_err, sizeof g_err, "%s", msg);
}

static ss4d_status last_launch()
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_err("kernel launch failed: %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// the handle

struct ss4d_solver {
    ss4d_dims dims;
    Geo geo;
    Split sp;
    SweepCfg cfg;
    ss4d_arith arith;
    cudaStream_t stream;
    cudaStream_t cap;
    cudaStream_t side;   // ss4d_copy_to_device_side, the chunked copies of ss4d_seg_time_step_host
    cudaEvent_t side_ev; // the last side copy
    cudaEvent_t chunk_ev[SS4D_HOST_CHUNKS], mask_ev;
    int device;
    int sm_count;
    int use_graph;
    int asm_kblock; // block order of the float-float faces and coefficient kernels (launch_assemble_ff_faces_range)
    long long launches;
    size_t bytes;

    // reductions / scalars
    double *d_partial;
    long long n_partial;
    double *d_scalar; // 8 doubles
    double *h_scalar; // pinned mirror
    // natural-layout scratch
    double *d_scratch;
    float2 *d_ff;      // mixed form's edge detector: 3 float-float volumes (image, thresholded image, prev)
    double *d_coef_nat; // 8 arrays (reference arithmetic)
    // split form
    SplitBufs sb;
    int have_split, have_mixed;
    LoopState *d_state;
    LoopState *h_state;
    DevParams *d_params;
    DevParams *h_params;
    // graphs
    cudaGraph_t graph64, graphmx;
    cudaGraphExec_t exec64, execmx;
    unsigned long long cond64, condmx;
    int graph_failed;
    int last_graphed; // the last solve ran as a graph
    // rescale balls
    int *d_frame_first, *d_frame_count;
    double *d_bx, *d_by, *d_bz;
    int balls_cap;
    cudaEvent_t ev0, ev1;
    // learned warm start (mixed form)
    ss4d_wsnet *ws_net;
    const double *ws_i0;
    void *ws_x0;   // BF16 features, planar [nt][2][nz][ny][nx][8]
    float *ws_y;   // prediction [nt][nz][ny][nx]
    CPtrs8 cur_g;  // g of the segmentation step in progress
    int have_g;
    int ws_gate;       // the network runs when the previous mixed step took >= ws_gate FP32 sweeps (0: always)
    int ws_last_iters; // FP32 sweeps of the previous mixed step (-1: none yet)
    // mixed form: start from an extrapolation in time (ss4d_solver_set_extrapolation)
    int extrap;      // 0 off, else the extrapolation order 1..3
    int have_dprev;  // steps in a row whose change was kept: dR[0] / dB hold the next start correction
    int pre_next;    // the next mixed loop's first refinement pass was formed by the assembly
    float *hist[4];  // earlier steps' changes (split layout): h1 red, h1 black, h2 red, h2 black
    int proj;        // start the first round from the projection onto the earlier changes (ss4d_project.cu)
    double *d_proj;  // its per-block sums (18 * n_partial / 2 doubles) and coefficients (3 floats after them)
    double inner_omega; // mixed form: relaxation factor of the FP32 sweeps (0: omega_c)
    // per-kernel timing (ss4d_solver_set_timing)
    int timing;
    double ktime[SS4D_K_COUNT];
    long long kcount[SS4D_K_COUNT];
    cudaEvent_t tev0, tev1;
};

// Launch `fn` and, when timing is on, bracket it with events on the
// handle's stream and add its device time to kernel kind `kind`.
template <typename F>
static void timed(ss4d_solver *s, int kind, bool count, F &&fn)
{
    if (!s->timing || !count) {
        fn();
        return;
    }
    cudaEventRecord(s->tev0, s->stream);
    fn();
    cudaEventRecord(s->tev1, s->stream);
    if (cudaEventSynchronize(s->tev1) == cudaSuccess) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->tev0, s->tev1);
        s->ktime[kind] += ms;
        s->kcount[kind] += 1;
    }
}

static ss4d_status dmalloc(ss4d_solver *s, void **p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return SS4D_ERR_ALLOC;
    }
    if (s)
        s->bytes += bytes;
    return SS4D_OK;
}

extern "C" int ss4d_abi_version(void)
{
    return SS4D_ABI_VERSION;
}

extern "C" const char *ss4d_last_error(void)
{
    return g_err;
}

extern "C" ss4d_status ss4d_device_count(int *count)
{
    REQ(count, "count is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        *count = 0;
        set_err("no CUDA device: %s", cudaGetErrorString(e));
        return SS4D_ERR_NO_DEVICE;
    }
    *count = n;
    return SS4D_OK;
}

static ss4d_status check_dims(const ss4d_dims *d)
{
    REQ(d, "dims is NULL");
    REQ(d->iMax >= 3 && d->jMax >= 3 && d->kMax >= 3 && d->lMax >= 3, "every padded extent must be >= 3");
    const long long n = (long long)d->iMax * d->jMax * d->kMax * d->lMax;
    REQ(n < (1LL << 31), "padded volume must hold fewer than 2^31 voxels (the reference's int indexing)");
    REQ((long long)(d->kMax - 1) * (d->lMax - 1) <= 65535, "(kMax-1)*(lMax-1) must not exceed 65535");
    const Split sp = make_split(make_geo(*d));
    REQ(sp.cs < (1LL << 31) && sp.ct < (1LL << 31), "a colour-split array must hold fewer than 2^31 elements");
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_create(const ss4d_dims *dims, ss4d_arith arith, void *stream, ss4d_solver **out)
{
    REQ(out, "out is NULL");
    *out = nullptr;
    CKS(check_dims(dims));
    REQ(arith == SS4D_ARITH_REFERENCE || arith == SS4D_ARITH_FP64 || arith == SS4D_ARITH_MIXED, "unknown arithmetic");
    int ndev = 0;
    CKS(ss4d_device_count(&ndev));
    ss4d_solver *s = (ss4d_solver *)calloc(1, sizeof(ss4d_solver));
    if (!s)
        return SS4D_ERR_ALLOC;
    s->dims = *dims;
    s->geo = make_geo(*dims);
    s->sp = make_split(s->geo);
    s->arith = arith;
    s->stream = (cudaStream_t)stream;
    s->use_graph = 1;
    s->asm_kblock = 4; // blocks of 4 planes across the frames: measured best of 0, 2, 4, 8, 16, 32 (by 2 %)
    ss4d_status st = SS4D_OK;
#define FAIL_IF(call)                                                                                              \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            set_err("%s failed: %s", #call, cudaGetErrorString(e_));                                               \
            st = e_ == cudaErrorMemoryAllocation ? SS4D_ERR_ALLOC : SS4D_ERR_CUDA;                                  \
            goto fail;                                                                                             \
        }                                                                                                          \
    } while (0)
    FAIL_IF(cudaGetDevice(&s->device));
    FAIL_IF(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
    // k blocks of one plane: at 256^2 x 128 x 20 the FP32 half-sweep took
    // 0.693 ms against 0.714 ms with blocks of 4 planes, the FP64 one 1.685
    // against 1.751 ms (a refinement kernel 2.023 against 1.996 ms)
    s->cfg = make_sweep_cfg(s->geo, s->sp, s->sm_count, 1);
    FAIL_IF(cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking));
    FAIL_IF(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
    FAIL_IF(cudaEventCreateWithFlags(&s->side_ev, cudaEventDisableTiming));
    for (int c = 0; c < SS4D_HOST_CHUNKS; ++c)
        FAIL_IF(cudaEventCreateWithFlags(&s->chunk_ev[c], cudaEventDisableTiming));
    FAIL_IF(cudaEventCreateWithFlags(&s->mask_ev, cudaEventDisableTiming));
    FAIL_IF(cudaEventCreate(&s->ev0));
    FAIL_IF(cudaEventCreate(&s->ev1));
    FAIL_IF(cudaEventCreate(&s->tev0));
    FAIL_IF(cudaEventCreate(&s->tev1));
    {
        long long nb = interior_blocks(s->geo);
        long long need = nb * 2 + 4096; // per-block partials (min/max pairs) and a second reduction stage
        if (need < 8192)
            need = 8192;
        // room for the partials of the largest persistent grid any tiling allows
        const long long gmax = (long long)s->sm_count * (max_blocks_sweep64() > max_blocks_sweep32()
                                                             ? max_blocks_sweep64()
                                                             : max_blocks_sweep32());
        if (need < 2LL * gmax)
            need = 2LL * gmax;
        s->n_partial = need;
    }
    if ((st = dmalloc(s, (void **)&s->d_partial, sizeof(double) * s->n_partial)) != SS4D_OK)
        goto fail;
    if ((st = dmalloc(s, (void **)&s->d_scalar, sizeof(double) * 8)) != SS4D_OK)
        goto fail;
    if ((st = dmalloc(s, (void **)&s->d_state, sizeof(LoopState))) != SS4D_OK)
        goto fail;
    if ((st = dmalloc(s, (void **)&s->d_params, sizeof(DevParams))) != SS4D_OK)
        goto fail;
    FAIL_IF(cudaMallocHost((void **)&s->h_scalar, sizeof(double) * 8));
    FAIL_IF(cudaMallocHost((void **)&s->h_state, sizeof(LoopState)));
    FAIL_IF(cudaMallocHost((void **)&s->h_params, sizeof(DevParams)));
#undef FAIL_IF
    *out = s;
    return SS4D_OK;
fail:
    ss4d_solver_destroy(s);
    return st;
}

static void free_graphs(ss4d_solver *s)
{
    if (s->exec64)
        cudaGraphExecDestroy(s->exec64);
    if (s->graph64)
        cudaGraphDestroy(s->graph64);
    if (s->execmx)
        cudaGraphExecDestroy(s->execmx);
    if (s->graphmx)
        cudaGraphDestroy(s->graphmx);
    s->exec64 = nullptr;
    s->graph64 = nullptr;
    s->execmx = nullptr;
    s->graphmx = nullptr;
}

extern "C" ss4d_status ss4d_solver_destroy(ss4d_solver *s)
{
    if (!s)
        return SS4D_OK;
    if (s->stream || s->cap)
        cudaStreamSynchronize(s->stream);
    free_graphs(s);
    // allocation bases only: R[1], Bk, P[1], coef[1], ... point inside them
    void *dev[] = {s->d_partial, s->d_scalar, s->d_state, s->d_params, s->d_scratch, s->d_coef_nat,
                   s->sb.R[0], s->sb.P[0], s->sb.coef[0], s->sb.coefq[0], s->sb.dR[0], s->sb.r32[0], s->sb.fn[0],
                   s->d_frame_first, s->d_frame_count, s->d_bx, s->d_by, s->d_bz, s->ws_x0, s->ws_y,
                   s->hist[0], s->hist[1], s->hist[2], s->hist[3], s->sb.fd[0], s->d_ff, s->d_proj};
    for (void *p : dev)
        if (p)
            cudaFree(p);
    if (s->h_scalar)
        cudaFreeHost(s->h_scalar);
    if (s->h_state)
        cudaFreeHost(s->h_state);
    if (s->h_params)
        cudaFreeHost(s->h_params);
    if (s->ev0)
        cudaEventDestroy(s->ev0);
    if (s->ev1)
        cudaEventDestroy(s->ev1);
    if (s->tev0)
        cudaEventDestroy(s->tev0);
    if (s->tev1)
        cudaEventDestroy(s->tev1);
    if (s->cap)
        cudaStreamDestroy(s->cap);
    if (s->side) {
        cudaStreamSynchronize(s->side);
        cudaStreamDestroy(s->side);
    }
    if (s->side_ev)
        cudaEventDestroy(s->side_ev);
    for (int c = 0; c < SS4D_HOST_CHUNKS; ++c)
        if (s->chunk_ev[c])
            cudaEventDestroy(s->chunk_ev[c]);
    if (s->mask_ev)
        cudaEventDestroy(s->mask_ev);
    free(s);
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_stream(ss4d_solver *s, void *stream)
{
    REQ(s, "solver is NULL");
    s->stream = (cudaStream_t)stream;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_arith(ss4d_solver *s, ss4d_arith arith)
{
    REQ(s, "solver is NULL");
    REQ(arith == SS4D_ARITH_REFERENCE || arith == SS4D_ARITH_FP64 || arith == SS4D_ARITH_MIXED, "unknown arithmetic");
    s->arith = arith;
    s->have_dprev = 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_tiling(ss4d_solver *s, int k_block, int max_grid)
{
    REQ(s, "solver is NULL");
    REQ(k_block >= 1 && max_grid >= 0, "k_block must be >= 1 and max_grid >= 0");
    SweepCfg c = make_sweep_cfg(s->geo, s->sp, s->sm_count, k_block);
    if (max_grid > 0 && c.grid > max_grid)
        c.grid = max_grid;
    REQ(2LL * c.grid <= s->n_partial, "grid larger than the partial-sum buffer");
    s->cfg = c;
    s->sb.partial[1] = s->d_partial + c.grid;
    free_graphs(s); // kernel arguments changed
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_assembly_order(ss4d_solver *s, int planes)
{
    REQ(s, "solver is NULL");
    REQ(planes >= 0, "planes must be >= 0");
    s->asm_kblock = planes;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_graph(ss4d_solver *s, int enable)
{
    REQ(s, "solver is NULL");
    s->use_graph = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_workspace_bytes(const ss4d_solver *s, size_t *bytes)
{
    REQ(s && bytes, "NULL argument");
    *bytes = s->bytes;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_launch_count(const ss4d_solver *s, long long *count)
{
    REQ(s && count, "NULL argument");
    *count = s->launches;
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// workspaces

static ss4d_status ensure_scratch(ss4d_solver *s)
{
    if (!s->d_scratch)
        CKS(dmalloc(s, (void **)&s->d_scratch, sizeof(double) * s->geo.n));
    return SS4D_OK;
}

static ss4d_status ensure_ff_front(ss4d_solver *s)
{
    if (!s->d_ff)
        CKS(dmalloc(s, (void **)&s->d_ff, sizeof(float2) * 3 * s->geo.n));
    return SS4D_OK;
}

static ss4d_status ensure_coef_nat(ss4d_solver *s)
{
    if (!s->d_coef_nat) {
        CKS(dmalloc(s, (void **)&s->d_coef_nat, sizeof(double) * 8 * s->geo.n));
        CK(cudaMemsetAsync(s->d_coef_nat, 0, sizeof(double) * 8 * s->geo.n, s->stream));
    }
    return SS4D_OK;
}

static ss4d_status ensure_split(ss4d_solver *s, int mixed)
{
    const long long cs = s->sp.cs;
    if (!s->have_split) {
        double *u3 = nullptr, *p2 = nullptr, *cf = nullptr;
        CKS(dmalloc(s, (void **)&u3, sizeof(double) * 3 * cs));
        CKS(dmalloc(s, (void **)&p2, sizeof(double) * 2 * cs));
        CKS(dmalloc(s, (void **)&cf, sizeof(double) * 20 * s->sp.ct));
        CK(cudaMemsetAsync(u3, 0, sizeof(double) * 3 * cs, s->stream));
        CK(cudaMemsetAsync(p2, 0, sizeof(double) * 2 * cs, s->stream));
        CK(cudaMemsetAsync(cf, 0, sizeof(double) * 20 * s->sp.ct, s->stream));
        s->sb.R[0] = u3;
        s->sb.R[1] = u3 + cs;
        s->sb.Bk = u3 + 2 * cs;
        s->sb.P[0] = p2;
        s->sb.P[1] = p2 + cs;
        s->sb.coef[0] = cf;
        s->sb.coef[1] = cf + 10 * s->sp.ct;
        s->sb.partial[0] = s->d_partial;
        s->sb.partial[1] = s->d_partial + s->cfg.grid;
        double *faces = nullptr; // 4 face norms + 4 face g/norm arrays, natural layout
        CKS(dmalloc(s, (void **)&faces, sizeof(double) * 8 * (size_t)s->geo.n));
        for (int d = 0; d < 4; ++d) {
            s->sb.fn[d] = faces + (size_t)d * s->geo.n;
            s->sb.fq[d] = faces + (size_t)(4 + d) * s->geo.n;
        }
        s->have_split = 1;
    }
    if (mixed && !s->have_mixed) {
        float *c32 = nullptr, *d3 = nullptr, *r2 = nullptr;
        // per colour: ct 16-byte fraction records, then (after both) ct scales
        CKS(dmalloc(s, (void **)&c32, sizeof(float) * 10 * s->sp.ct));
        CKS(dmalloc(s, (void **)&d3, sizeof(float) * 3 * cs));
        CKS(dmalloc(s, (void **)&r2, sizeof(float) * 2 * cs));
        CK(cudaMemsetAsync(c32, 0, sizeof(float) * 10 * s->sp.ct, s->stream));
        CK(cudaMemsetAsync(d3, 0, sizeof(float) * 3 * cs, s->stream));
        CK(cudaMemsetAsync(r2, 0, sizeof(float) * 2 * cs, s->stream));
        s->sb.coefq[0] = reinterpret_cast<uint4 *>(c32);
        s->sb.coefq[1] = reinterpret_cast<uint4 *>(c32 + 4 * s->sp.ct);
        s->sb.coefs[0] = c32 + 8 * s->sp.ct;
        s->sb.coefs[1] = c32 + 9 * s->sp.ct;
        s->sb.dR[0] = d3;
        s->sb.dR[1] = d3 + cs;
        s->sb.dB = d3 + 2 * cs;
        s->sb.r32[0] = r2;
        s->sb.r32[1] = r2 + cs;
        double *fd = nullptr; // float-float forward differences, 4 axes, natural layout
        CKS(dmalloc(s, (void **)&fd, sizeof(double) * 4 * (size_t)s->geo.n));
        for (int d = 0; d < 4; ++d)
            s->sb.fd[d] = fd + (size_t)d * s->geo.n;
        double *rp = nullptr; // the first refinement pass's residual, per colour (split layout)
        CKS(dmalloc(s, (void **)&rp, sizeof(double) * 2 * cs));
        CK(cudaMemsetAsync(rp, 0, sizeof(double) * 2 * cs, s->stream));
        s->sb.rpre[0] = rp;
        s->sb.rpre[1] = rp + cs;
        s->have_mixed = 1;
        free_graphs(s); // kernel arguments changed
    }
    return SS4D_OK;
}

static ss4d_status check_params(const ss4d_params *p)
{
    REQ(p, "params is NULL");
    REQ(p->h > 0 && isfinite(p->h), "h must be positive");
    REQ(isfinite(p->tau) && isfinite(p->eps2) && isfinite(p->omega_c) && isfinite(p->gsTol), "non-finite parameter");
    return SS4D_OK;
}

// The residual is a sum of nint non-negative terms; a serial left-to-right
// sum of them (the reference's) differs from any other order by at most
// about nint * 2^-53 relative.  A stop test with R that close to the
// tolerance is reported (ss4d_step_stats.near_tolerance): there the
// reference could have stopped one iteration earlier or later.
static double near_band(double tol, long long nint)
{
    return fabs(tol) * (double)nint * 0x1p-53;
}

static ss4d_status upload_params(ss4d_solver *s, const ss4d_params *p)
{
    s->h_params->c = p->tau / (p->h * p->h);
    // the mixed form's FP32 sweeps may relax with their own factor
    s->h_params->omega = s->arith == SS4D_ARITH_MIXED && s->inner_omega > 0.0 ? s->inner_omega : p->omega_c;
    s->h_params->h4 = p->h * p->h * p->h * p->h;
    s->h_params->tol = p->gsTol;
    s->h_params->maxit = p->maxNoGSIteration;
    s->h_params->pad_ = 0;
    s->h_params->near_band = near_band(p->gsTol, s->geo.nint);
    // the host mirror is only rewritten after the previous copy completed:
    // every solve ends with a stream synchronisation
    CK(cudaMemcpyAsync(s->d_params, s->h_params, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    return SS4D_OK;
}

static ss4d_status read_scalar(ss4d_solver *s, int idx, double *out)
{
    CK(cudaMemcpyAsync(s->h_scalar, s->d_scalar + idx, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = s->h_scalar[0];
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// SOR loop drivers

// reference arithmetic: red, black, residual pass, host test (segmentation4D.c:228-309)
static ss4d_status sor_reference(ss4d_solver *s, const ss4d_params *p, double *u, const double *prev, CPtrs8 a,
                                 ss4d_step_stats *stats)
{
    const Geo &g = s->geo;
    const double c = p->tau / (p->h * p->h), h4 = p->h * p->h * p->h * p->h;
    const long long nb = resid_blocks(g);
    const double band = near_band(p->gsTol, g.nint);
    double R = 0.0, R1 = 0.0;
    int z = 0, near = 0;
    do {
        z = z + 1;
        launch_sor_half_ref(g, u, prev, a, c, p->omega_c, 0, s->stream);
        launch_sor_half_ref(g, u, prev, a, c, p->omega_c, 1, s->stream);
        launch_sor_resid_ref(g, u, prev, a, c, h4, s->d_partial, s->stream);
        s->launches += 3 + launch_reduce_sum(s->d_partial, nb, s->d_scalar, s->stream);
        CKS(last_launch());
        CKS(read_scalar(s, 0, &R));
        if (z == 1)
            R1 = R;
        near |= fabs(R - p->gsTol) <= band;
    } while (R > p->gsTol && z < p->maxNoGSIteration);
    if (stats) {
        stats->iterations = z;
        stats->residual = R;
        stats->first_residual = R1;
        stats->refinements = 0;
        stats->near_tolerance = near;
        stats->status = isfinite(R) ? SS4D_OK : SS4D_ERR_NONFINITE;
    }
    return isfinite(R) ? SS4D_OK : SS4D_ERR_NONFINITE;
}

static ss4d_status build_graph(ss4d_solver *s, int mixed)
{
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle h;
    CK(cudaGraphCreate(&graph, 0));
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        set_err("cudaGraphConditionalHandleCreate: %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    // the C++ view of this union-holding struct has no default constructor:
    // build it in zeroed storage, as the C API expects unused bytes zero
    alignas(cudaGraphNodeParams) unsigned char cp_store[sizeof(cudaGraphNodeParams)];
    memset(cp_store, 0, sizeof cp_store);
    cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_store);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        set_err("cudaGraphAddNode(conditional): %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(s->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        set_err("cudaStreamBeginCaptureToGraph: %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    const unsigned long long hv = (unsigned long long)h;
    if (!mixed) {
        launch_sweep64(s->geo, s->sp, s->cfg, 1, s->sb, s->d_params, s->d_state, s->cap);
        launch_sweep64(s->geo, s->sp, s->cfg, 0, s->sb, s->d_params, s->d_state, s->cap);
        launch_ctrl64(s->sb, s->cfg.grid, s->d_params, s->d_state, hv, 1, s->cap);
    } else {
        launch_refine(s->geo, s->sp, s->cfg, 0, s->sb, s->d_params, s->d_state, s->cap);
        launch_refine(s->geo, s->sp, s->cfg, 1, s->sb, s->d_params, s->d_state, s->cap);
        launch_zero_delta(s->sp, s->sb, s->d_state, s->cap);
        launch_sweep32(s->geo, s->sp, s->cfg, 1, s->sb, s->d_params, s->d_state, 0, s->cap);
        launch_sweep32(s->geo, s->sp, s->cfg, 0, s->sb, s->d_params, s->d_state, 0, s->cap);
        launch_ctrl_mixed(s->sb, s->cfg.grid, s->d_params, s->d_state, hv, 1, s->cap);
    }
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(s->cap, &captured);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(graph);
        set_err("cudaStreamEndCapture: %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(graph);
        set_err("cudaGraphInstantiate: %s", cudaGetErrorString(e));
        return SS4D_ERR_CUDA;
    }
    if (mixed) {
        s->graphmx = graph;
        s->execmx = exec;
        s->condmx = hv;
    } else {
        s->graph64 = graph;
        s->exec64 = exec;
        s->cond64 = hv;
    }
    return SS4D_OK;
}

static ss4d_status finish_stats(ss4d_solver *s, ss4d_step_stats *stats, int mixed)
{
    CK(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const LoopState &L = *s->h_state;
    if (mixed)
        s->ws_last_iters = L.z;
    if (stats) {
        stats->iterations = L.z;
        stats->residual = L.R;
        stats->first_residual = L.R_first;
        stats->refinements = mixed ? L.refinements : 0;
        stats->status = L.status;
        stats->warm_started = L.warm;
        stats->near_tolerance = L.near;
        stats->projected = mixed ? L.proj : 0;
    }
    if (L.status != SS4D_OK) {
        set_err("SOR residual became non-finite at iteration %d", L.z);
        return (ss4d_status)L.status;
    }
    return SS4D_OK;
}

// coefficient assembly from u into the split records: FP64 (plain form,
// FP64 throughout) or float-float (mixed form, FP32 records for its sweeps).
// With pack, the mixed form also makes the split copies of u (prev = u) in
// its first-difference kernel: packed_by_assembly() says whether that
// replaces the caller's launch_pack.
static bool packed_by_assembly(int mixed)
{
    return mixed != 0;
}

static void assemble(ss4d_solver *s, const ss4d_params *p, const double *d_u, CPtrs8 gi, int has_g, int mixed,
                     int pack = 0, int pre = 0)
{
    if (mixed) {
        launch_assemble_ff(s->geo, s->sp, d_u, gi, has_g, *p, s->sb, pack, s->sm_count, s->stream, pre, s->asm_kblock);
        s->launches += 3;
    } else {
        launch_assemble(s->geo, s->sp, d_u, gi, has_g, *p, s->sb, 0, s->stream);
        s->launches += 2;
    }
}

static ss4d_status ensure_ws_buffers(ss4d_solver *s)
{
    if (!s->ws_x0) {
        CKS(dmalloc(s, &s->ws_x0, (size_t)s->geo.nint * 32));
        CKS(dmalloc(s, (void **)&s->ws_y, (size_t)s->geo.nint * 4));
    }
    return SS4D_OK;
}

// mixed form, state in mode 0 with zero corrections: the first FP64
// refinement pass at u^n (r0 into r32, R_first) and the controller's test;
// then the network's features, its prediction of the first correction, the
// check of that prediction and the keep/discard decision (ss4d_ws.cu)
static ss4d_status ws_first_pass(ss4d_solver *s)
{
    const SweepCfg &cfg = s->cfg;
    launch_refine(s->geo, s->sp, cfg, 0, s->sb, s->d_params, s->d_state, s->stream);
    launch_refine(s->geo, s->sp, cfg, 1, s->sb, s->d_params, s->d_state, s->stream);
    launch_ctrl_mixed(s->sb, cfg.grid, s->d_params, s->d_state, 0, 0, s->stream);
    s->launches += 4; // a refinement pass is 3 launches
    return last_launch();
}

static ss4d_status warm_start_prologue(ss4d_solver *s)
{
    const Geo &g = s->geo;
    CKS(ensure_ws_buffers(s));
    CKS(ws_first_pass(s));
    ss4d_status st = SS4D_OK;
    timed(s, SS4D_K_WARM, true, [&] {
        launch_ws_features(g, s->sp, s->sb, s->ws_i0, s->cur_g, s->d_state, s->d_params, s->ws_x0, s->stream);
        st = ss4d_wsnet_set_stream(s->ws_net, s->stream);
        if (st == SS4D_OK)
            st = ss4d_wsnet_forward(s->ws_net, s->ws_x0, g.nx, g.ny, g.nz, g.nt, s->ws_y);
        launch_ws_apply(g, s->sp, s->sb, s->ws_y, s->d_state, s->d_params, s->stream);
        launch_ws_check_decide(g, s->sp, s->cfg, s->sb, s->d_state, s->d_params, s->stream);
    });
    CKS(st);
    s->launches += 1 + 4 + 1 + 3;
    return last_launch();
}

extern "C" ss4d_status ss4d_solver_set_warm_start(ss4d_solver *s, ss4d_wsnet *n, const double *d_i0)
{
    REQ(s, "solver is NULL");
    REQ(!n || d_i0, "the warm start needs the presmoothed image");
    s->ws_net = n;
    s->ws_i0 = n ? d_i0 : nullptr;
    s->ws_last_iters = -1;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_warm_start_gate(ss4d_solver *s, int min_iterations)
{
    REQ(s, "solver is NULL");
    REQ(min_iterations >= 0, "the gate is a non-negative iteration count");
    s->ws_gate = min_iterations;
    return SS4D_OK;
}

// this step's solve starts from the network's prediction
static bool ws_this_step(const ss4d_solver *s, int mixed)
{
    return mixed && s->ws_net && s->have_g &&
           (s->ws_gate <= 0 || s->ws_last_iters < 0 || s->ws_last_iters >= s->ws_gate);
}

extern "C" ss4d_status ss4d_ws_features(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *const d_g[8],
                                        const double *d_i0, void *d_x0, double *sigma)
{
    REQ(s && d_u && d_g && d_i0 && d_x0 && sigma, "NULL argument");
    CKS(check_params(p));
    CPtrs8 gi;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        gi.p[f] = d_g[f];
    }
    CKS(ensure_split(s, 1));
    s->have_dprev = 0; // the corrections are overwritten below
    const Split &sp = s->sp;
    assemble(s, p, d_u, gi, 1, 1, 1);
    CKS(upload_params(s, p));
    const size_t fb = sizeof(float) * sp.cs;
    CK(cudaMemsetAsync(s->sb.dR[0], 0, fb, s->stream));
    CK(cudaMemsetAsync(s->sb.dR[1], 0, fb, s->stream));
    CK(cudaMemsetAsync(s->sb.dB, 0, fb, s->stream));
    launch_loop_init(s->d_state, 0, s->stream);
    CKS(ws_first_pass(s));
    launch_ws_features(s->geo, sp, s->sb, d_i0, gi, s->d_state, s->d_params, d_x0, s->stream);
    s->launches += 2;
    CKS(last_launch());
    CK(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const double h4 = p->h * p->h * p->h * p->h;
    *sigma = sqrt(s->h_state->R_first / ((double)s->geo.nint * h4));
    return SS4D_OK;
}

// a segmentation step of the mixed form that starts from u^n + (u^n - u^{n-1})
static bool extrapolating(const ss4d_solver *s)
{
    return s->arith == SS4D_ARITH_MIXED && s->extrap && s->have_dprev && s->have_g;
}

// A mixed segmentation step (not with the learned warm start, which runs
// its own first pass before its prediction) has the assembly form its first
// refinement pass: the first-difference kernel adds the start correction to
// the split copies of u with the pass's FP64 addition, the coefficient
// kernel evaluates the pass's FP64 residual with the pass's operations on
// the same values, and the pass only reads that residual (LoopState.pre).
// The step's results are those of the pass run in full.  Returns 0 (not
// this step), 1 (start correction zero) or 2 (the extrapolation that
// extrapolating() will find in dR[0] / dB).
static int pre_form(const ss4d_solver *s, int mixed)
{
    if (!mixed)
        return 0;
    return s->extrap && s->have_dprev ? 2 : 1;
}

// the mixed loop's start correction: zero, or the extrapolation the previous
// step's unpack left in dR[0] / dB (applied by the first refinement pass, or
// by the first-difference kernel when the assembly formed that pass)
static ss4d_status clear_corrections(ss4d_solver *s)
{
    const size_t fb = sizeof(float) * s->sp.cs;
    if (!extrapolating(s)) {
        CK(cudaMemsetAsync(s->sb.dR[0], 0, fb, s->stream));
        CK(cudaMemsetAsync(s->sb.dB, 0, fb, s->stream));
    }
    CK(cudaMemsetAsync(s->sb.dR[1], 0, fb, s->stream));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_inner_omega(ss4d_solver *s, double omega)
{
    REQ(s, "solver is NULL");
    REQ(omega == 0.0 || (omega > 0.0 && omega < 2.0), "inner omega must be 0 or in (0, 2)");
    s->inner_omega = omega;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_extrapolation(ss4d_solver *s, int order)
{
    REQ(s, "solver is NULL");
    REQ(order >= 0 && order <= 3, "extrapolation order must be 0, 1, 2 or 3");
    s->extrap = order;
    s->have_dprev = 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_set_projection(ss4d_solver *s, int enable)
{
    REQ(s, "solver is NULL");
    s->proj = enable ? 1 : 0;
    return SS4D_OK;
}

// the first round's start projected onto the earlier changes: with the
// extrapolation of order 3 applied by the assembly (whose first refinement
// pass's residual is then in rpre) and at least two earlier changes, when no
// learned warm start supplies the start
static ss4d_status project_start(ss4d_solver *s, int pre, LoopState *d_state)
{
    if (!s->proj || !pre || s->extrap != 3 || !extrapolating(s) || s->have_dprev < 2 || ws_this_step(s, 1))
        return SS4D_OK;
    for (int q = 0; q < 4; ++q)
        if (!s->hist[q])
            return SS4D_OK;
    if (!s->d_proj) {
        const size_t nd = 9 * (size_t)s->n_partial; // 18 * grid with n_partial >= 2 * grid
        CKS(dmalloc(s, (void **)&s->d_proj, sizeof(double) * nd + 4 * sizeof(float)));
    }
    float *c = reinterpret_cast<float *>(s->d_proj + 9 * (size_t)s->n_partial);
    const int m = s->have_dprev >= 3 ? 3 : 2;
    timed(s, SS4D_K_PROJECT, true, [&] {
        launch_projection(s->geo, s->sp, s->cfg, s->sb, s->hist, m, s->d_proj, c, d_state, s->sm_count, s->stream);
    });
    s->launches += 4;
    return SS4D_OK;
}

static ss4d_status drive_loop(ss4d_solver *s, const ss4d_params *p, int mixed, int mode);

// the loop on the split buffers; u/prev already packed, coefficients assembled.
// spec (mixed form): the loop pauses when a round ends, before that round's
// refinement pass (LoopState.paused), for the caller to run that pass itself
static ss4d_status run_split_loop(ss4d_solver *s, const ss4d_params *p, int mixed, int spec = 0)
{
    const int pre = mixed ? s->pre_next : 0; // consumed by this loop only
    s->pre_next = 0;
    const Geo &g = s->geo;
    const Split &sp = s->sp;
    const SweepCfg &cfg = s->cfg;
    CKS(upload_params(s, p));
    if (!mixed) {
        launch_loop_init(s->d_state, 0, s->stream);
        timed(s, SS4D_K_SWEEP64, true,
              [&] { launch_sweep64(g, sp, cfg, 0, s->sb, s->d_params, s->d_state, s->stream); });
        launch_advance(s->d_state, s->stream);
        s->launches += 3;
    } else {
        // the first refinement pass adds the correction in dR[0] / dB to u
        // (or the assembly did, and formed the pass's residual: pre_next)
        CKS(clear_corrections(s));
        launch_loop_init(s->d_state, 0, s->stream, pre, spec);
        s->launches += 1;
        if (ws_this_step(s, mixed))
            CKS(warm_start_prologue(s));
        CKS(project_start(s, pre, s->d_state));
    }
    CKS(last_launch());
    // the mode the controller left for the first body
    return drive_loop(s, p, mixed, mixed && ws_this_step(s, mixed) ? 1 : 0);
}

// the loop from the state the controller left (mode: that state's mode),
// as the graph's while loop or host-driven, until it stops or pauses
static ss4d_status drive_loop(ss4d_solver *s, const ss4d_params *p, int mixed, int mode)
{
    const Geo &g = s->geo;
    const Split &sp = s->sp;
    const SweepCfg &cfg = s->cfg;
    bool graphed = false;
    if (s->use_graph && !s->graph_failed && !s->timing) {
        cudaGraphExec_t ex = mixed ? s->execmx : s->exec64;
        if (!ex) {
            if (build_graph(s, mixed) != SS4D_OK)
                s->graph_failed = 1; // fall back to the host loop from now on
            ex = mixed ? s->execmx : s->exec64;
        }
        if (ex) {
            CK(cudaGraphLaunch(ex, s->stream));
            graphed = true;
        }
    }
    if (!graphed) {
        // host-driven form of the same loop: one small readback per iteration
        for (int guard = 0; guard < 4 * (p->maxNoGSIteration + 4) + 16; ++guard) {
            if (!mixed) {
                timed(s, SS4D_K_SWEEP64, true,
                      [&] { launch_sweep64(g, sp, cfg, 1, s->sb, s->d_params, s->d_state, s->stream); });
                timed(s, SS4D_K_SWEEP64, true,
                      [&] { launch_sweep64(g, sp, cfg, 0, s->sb, s->d_params, s->d_state, s->stream); });
                launch_ctrl64(s->sb, cfg.grid, s->d_params, s->d_state, 0, 0, s->stream);
                s->launches += 3;
            } else {
                // kernels whose mode does not match return at once: only the
                // ones that do the work are timed
                timed(s, SS4D_K_REFINE, mode == 0,
                      [&] { launch_refine(g, sp, cfg, 0, s->sb, s->d_params, s->d_state, s->stream); });
                timed(s, SS4D_K_REFINE, mode == 0,
                      [&] { launch_refine(g, sp, cfg, 1, s->sb, s->d_params, s->d_state, s->stream); });
                launch_zero_delta(sp, s->sb, s->d_state, s->stream);
                timed(s, SS4D_K_SWEEP32, mode == 2,
                      [&] { launch_sweep32(g, sp, cfg, 1, s->sb, s->d_params, s->d_state, 0, s->stream); });
                timed(s, SS4D_K_SWEEP32, mode != 0,
                      [&] { launch_sweep32(g, sp, cfg, 0, s->sb, s->d_params, s->d_state, 0, s->stream); });
                launch_ctrl_mixed(s->sb, cfg.grid, s->d_params, s->d_state, 0, 0, s->stream);
                s->launches += 7;
            }
            CKS(last_launch());
            CK(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            if (s->h_state->stop || s->h_state->paused)
                break;
            mode = s->h_state->mode;
        }
    }
    s->last_graphed = graphed ? 1 : 0;
    return SS4D_OK;
}

// the refinement pass a paused loop left for later (one host-driven body in
// mode 0: only the refinement kernels and the controller do work)
static ss4d_status refine_paused(ss4d_solver *s)
{
    const Geo &g = s->geo;
    const Split &sp = s->sp;
    const SweepCfg &cfg = s->cfg;
    timed(s, SS4D_K_REFINE, true, [&] { launch_refine(g, sp, cfg, 0, s->sb, s->d_params, s->d_state, s->stream); });
    timed(s, SS4D_K_REFINE, true, [&] { launch_refine(g, sp, cfg, 1, s->sb, s->d_params, s->d_state, s->stream); });
    launch_ctrl_mixed(s->sb, cfg.grid, s->d_params, s->d_state, 0, 0, s->stream);
    s->launches += 4;
    return last_launch();
}

// count the kernels of a graphed loop after the fact: the controller counts
// the loop bodies it ran
static void count_graph_launches(ss4d_solver *s, int mixed)
{
    if (!s->last_graphed)
        return;
    s->launches += (long long)(mixed ? 7 : 3) * s->h_state->bodies;
}

extern "C" ss4d_status ss4d_solver_set_timing(ss4d_solver *s, int enable)
{
    REQ(s, "solver is NULL");
    s->timing = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_kernel_time(const ss4d_solver *s, int kind, double *total_ms, long long *launches)
{
    REQ(s && total_ms && launches, "NULL argument");
    REQ(kind >= 0 && kind < SS4D_K_COUNT, "unknown kernel kind");
    *total_ms = s->ktime[kind];
    *launches = s->kcount[kind];
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_solver_reset_timing(ss4d_solver *s)
{
    REQ(s, "solver is NULL");
    for (int k = 0; k < SS4D_K_COUNT; ++k) {
        s->ktime[k] = 0.0;
        s->kcount[k] = 0;
    }
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// balls

static ss4d_status upload_balls(ss4d_solver *s, const ss4d_balls *b, double R, int *have)
{
    *have = 0;
    if (!b || b->n == 0)
        return SS4D_OK;
    REQ(b->n > 0 && b->l && b->cx && b->cy && b->cz, "balls arrays are NULL");
    const Geo &g = s->geo;
    std::vector<int> first(g.lM, 0), count(g.lM, 0);
    int prev_l = -1;
    for (int i = 0; i < b->n; ++i) {
        const int l = b->l[i];
        REQ(l >= 1 && l <= g.lM - 2, "ball frame index out of range");
        REQ(l >= prev_l, "balls must be ordered by frame");
        if (l != prev_l)
            first[l] = i;
        count[l] += 1;
        prev_l = l;
        const int k0 = (int)(b->cz[i] - R - 0.5), k1 = (int)(b->cz[i] + R + 0.5);
        const int j0 = (int)(b->cy[i] - R - 0.5), j1 = (int)(b->cy[i] + R + 0.5);
        const int i0 = (int)(b->cx[i] - R - 0.5), i1 = (int)(b->cx[i] + R + 0.5);
        REQ(k0 >= 0 && j0 >= 0 && i0 >= 0 && k1 < g.kM && j1 < g.jM && i1 < g.iM,
            "a ball's box leaves the array (the reference would read out of bounds)");
    }
    if (s->balls_cap < b->n) {
        if (s->d_bx)
            cudaFree(s->d_bx), cudaFree(s->d_by), cudaFree(s->d_bz);
        CKS(dmalloc(s, (void **)&s->d_bx, sizeof(double) * b->n));
        CKS(dmalloc(s, (void **)&s->d_by, sizeof(double) * b->n));
        CKS(dmalloc(s, (void **)&s->d_bz, sizeof(double) * b->n));
        s->balls_cap = b->n;
    }
    if (!s->d_frame_first) {
        CKS(dmalloc(s, (void **)&s->d_frame_first, sizeof(int) * g.lM));
        CKS(dmalloc(s, (void **)&s->d_frame_count, sizeof(int) * g.lM));
    }
    // synchronous copies: the host vectors die with this call
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(s->d_frame_first, first.data(), sizeof(int) * g.lM, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_frame_count, count.data(), sizeof(int) * g.lM, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_bx, b->cx, sizeof(double) * b->n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_by, b->cy, sizeof(double) * b->n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_bz, b->cz, sizeof(double) * b->n, cudaMemcpyHostToDevice));
    *have = 1;
    return SS4D_OK;
}

static ss4d_status rescale_impl(ss4d_solver *s, const ss4d_params *p, double *d_img, const double *d_Mmask,
                                const ss4d_balls *balls)
{
    int have = 0;
    CKS(upload_balls(s, balls, p->ballRadius, &have));
    if (have) {
        launch_rescale_balls(s->geo, d_img, s->d_frame_first, s->d_frame_count, s->d_bx, s->d_by, s->d_bz,
                             p->ballRadius, s->stream);
        s->launches += 1;
    }
    if (d_Mmask) {
        launch_mask_zero(s->geo, d_img, d_Mmask, s->stream);
        s->launches += 1;
    }
    return last_launch();
}

// ---------------------------------------------------------------------------
// entry points

extern "C" ss4d_status ss4d_reflect(ss4d_solver *s, double *d_img)
{
    REQ(s && d_img, "NULL argument");
    launch_reflect(s->geo, d_img, s->stream);
    s->launches += 4;
    return last_launch();
}

// The mixed form's presmoothing: the same SOR on float-float copies of the
// image (slot 0 or 1 of d_ff) and of its input (slot 2), written back to
// the image's interior at the end; the float-float result stays in its slot
// for the g faces.  prev (the reference's prev_u) receives the input as in
// the FP64 forms.
static ss4d_status presmooth_ff(ss4d_solver *s, const ss4d_params *p, double *d_img, double *prev, int slot,
                                ss4d_step_stats *stats)
{
    CKS(ensure_ff_front(s));
    const Geo &g = s->geo;
    float2 *v = s->d_ff + (size_t)slot * g.n, *pf = s->d_ff + 2 * (size_t)g.n;
    CK(cudaEventRecord(s->ev0, s->stream));
    CK(cudaMemcpyAsync(prev, d_img, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    launch_reflect(g, d_img, s->stream);
    launch_to_ff(g, d_img, v, s->stream);
    launch_to_ff(g, prev, pf, s->stream);
    s->launches += 6;
    const double c = p->sigma / (p->h * p->h), h4 = p->h * p->h * p->h * p->h;
    const long long nb = front_resid_blocks(g);
    // the residual's squares are summed in FP32 per thread: a test within
    // 1e-6 of gsTol is reported as near the tolerance
    const double band = fabs(p->gsTol) * 1e-6;
    double R = 0.0, R1 = 0.0;
    int z = 0, near = 0;
    do {
        z = z + 1;
        launch_presmooth_half_ff(g, v, pf, c, p->omega_sigma, 0, s->stream);
        launch_presmooth_half_ff(g, v, pf, c, p->omega_sigma, 1, s->stream);
        launch_presmooth_resid_ff(g, v, pf, c, h4, s->d_partial, s->stream);
        s->launches += 3 + launch_reduce_sum(s->d_partial, nb, s->d_scalar, s->stream);
        CKS(last_launch());
        CKS(read_scalar(s, 0, &R));
        if (z == 1)
            R1 = R;
        near |= fabs(R - p->gsTol) <= band;
    } while (R > p->gsTol && z < p->maxNoGSIteration_sigma);
    launch_from_ff(g, v, d_img, s->stream);
    s->launches += 1;
    CKS(last_launch());
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->iterations = z;
        stats->residual = R;
        stats->first_residual = R1;
        stats->near_tolerance = near;
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
        stats->status = isfinite(R) ? SS4D_OK : SS4D_ERR_NONFINITE;
    }
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_presmooth_step(ss4d_solver *s, const ss4d_params *p, double *d_img, double *d_scratch,
                                           ss4d_step_stats *stats)
{
    REQ(s && d_img, "NULL argument");
    CKS(check_params(p));
    double *prev = d_scratch;
    if (!prev) {
        CKS(ensure_scratch(s));
        prev = s->d_scratch;
    }
    if (s->arith == SS4D_ARITH_MIXED)
        return presmooth_ff(s, p, d_img, prev, 0, stats);
    const Geo &g = s->geo;
    CK(cudaEventRecord(s->ev0, s->stream));
    CK(cudaMemcpyAsync(prev, d_img, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    launch_reflect(g, d_img, s->stream);
    s->launches += 4;
    const double c = p->sigma / (p->h * p->h), h4 = p->h * p->h * p->h * p->h;
    const long long nb = resid_blocks(g);
    const double band = near_band(p->gsTol, g.nint);
    double R = 0.0, R1 = 0.0;
    int z = 0, near = 0;
    do {
        z = z + 1;
        launch_presmooth_half(g, d_img, prev, c, p->omega_sigma, 0, s->stream);
        launch_presmooth_half(g, d_img, prev, c, p->omega_sigma, 1, s->stream);
        launch_presmooth_resid(g, d_img, prev, c, h4, s->d_partial, s->stream);
        s->launches += 3 + launch_reduce_sum(s->d_partial, nb, s->d_scalar, s->stream);
        CKS(last_launch());
        CKS(read_scalar(s, 0, &R));
        if (z == 1)
            R1 = R;
        near |= fabs(R - p->gsTol) <= band;
    } while (R > p->gsTol && z < p->maxNoGSIteration_sigma);
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->iterations = z;
        stats->residual = R;
        stats->first_residual = R1;
        stats->near_tolerance = near;
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
        stats->status = isfinite(R) ? SS4D_OK : SS4D_ERR_NONFINITE;
    }
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_presmooth_explicit(ss4d_solver *s, const ss4d_params *p, int timeStepsNum, double *d_img,
                                               double *d_scratch)
{
    REQ(s && d_img, "NULL argument");
    CKS(check_params(p));
    REQ(timeStepsNum >= 0, "timeStepsNum must not be negative");
    double *prev = d_scratch;
    if (!prev) {
        CKS(ensure_scratch(s));
        prev = s->d_scratch;
    }
    const Geo &g = s->geo;
    CK(cudaMemcpyAsync(prev, d_img, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    launch_reflect(g, d_img, s->stream);
    s->launches += 4;
    // prev is not refreshed between the reference's steps, so every step after
    // the first recomputes the same values: one step is the result of any
    // number >= 1 (bit for bit)
    if (timeStepsNum > 0) {
        launch_presmooth_explicit(g, d_img, prev, p->sigma / (p->h * p->h), s->stream);
        launch_reflect(g, d_img, s->stream);
        s->launches += 5;
    }
    return last_launch();
}

// taps of ss4d_gaussian_smooth: w_m = exp(-m^2 / (2 sigma^2)) / sum over
// |m| <= R = ceil(3 sigma), the sum formed as w_0 + 2 w_1 + 2 w_2 + ... (the
// doubling is exact, so a multiply-add gives the same sum)
static ss4d_status gauss_weights(double sigma, GaussWeights *W)
{
    const double r = ceil(3.0 * sigma);
    REQ(r <= SS4D_GAUSS_MAX_RADIUS, "a Gaussian radius ceil(3 sigma) exceeds SS4D_GAUSS_MAX_RADIUS");
    W->R = (int)r;
    double sum = 0.0;
    for (int m = 0; m <= W->R; ++m) {
        W->w[m] = exp(-(double)(m * m) / (2.0 * sigma * sigma));
        sum += (m ? 2.0 : 1.0) * W->w[m];
    }
    for (int m = 0; m <= W->R; ++m)
        W->w[m] = W->w[m] / sum;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_gaussian_smooth(ss4d_solver *s, const double sigma[4], double *d_img, double *d_scratch)
{
    REQ(s && sigma && d_img, "NULL argument");
    GaussWeights W[4];
    for (int a = 0; a < 4; ++a) {
        REQ(isfinite(sigma[a]) && sigma[a] >= 0.0, "sigma must be finite and >= 0");
        if (sigma[a] > 0.0)
            CKS(gauss_weights(sigma[a], &W[a]));
    }
    double *tmp = d_scratch;
    if (!tmp) {
        CKS(ensure_scratch(s));
        tmp = s->d_scratch;
    }
    const Geo &g = s->geo;
    double *src = d_img, *dst = tmp;
    for (int a = 0; a < 4; ++a) {
        if (sigma[a] == 0.0)
            continue;
        launch_gauss_axis(g, a, src, dst, W[a], s->stream);
        s->launches += 1;
        double *t = src;
        src = dst;
        dst = t;
    }
    if (src != d_img)
        CK(cudaMemcpyAsync(d_img, src, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    launch_reflect(g, d_img, s->stream);
    s->launches += 4;
    return last_launch();
}

extern "C" ss4d_status ss4d_gfaces(ss4d_solver *s, const ss4d_params *p, const double *d_i0, const double *d_i0_thr,
                                   double *const d_g[8])
{
    REQ(s && d_i0 && d_g, "NULL argument");
    CKS(check_params(p));
    REQ(d_i0_thr || p->rho_thr == 0.0, "i0_thr may only be NULL when rho_thr == 0");
    GPtrs8 go;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        go.p[f] = d_g[f];
    }
    const Geo &g = s->geo;
    if (s->arith == SS4D_ARITH_MIXED) {
        CKS(ensure_ff_front(s));
        launch_to_ff(g, d_i0, s->d_ff, s->stream);
        if (d_i0_thr)
            launch_to_ff(g, d_i0_thr, s->d_ff + g.n, s->stream);
        launch_gfaces_ff(g, s->d_ff, d_i0_thr ? s->d_ff + g.n : nullptr, go, p->h, p->K, p->theta_img, p->rho_thr,
                         s->stream);
        s->launches += d_i0_thr ? 3 : 2;
    } else {
        launch_gfaces(g, d_i0, d_i0_thr, go, p->h, p->K, p->theta_img, p->rho_thr, s->stream);
        s->launches += 1;
    }
    return last_launch();
}

extern "C" ss4d_status ss4d_edge_detector(ss4d_solver *s, const ss4d_params *p, double *d_i0, double *d_i0_thr,
                                          double *d_scratch, double *const d_g[8])
{
    REQ(s && d_i0 && d_g, "NULL argument");
    CKS(check_params(p));
    REQ(d_i0_thr || p->rho_thr == 0.0, "i0_thr may only be NULL when rho_thr == 0");
    GPtrs8 go;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        go.p[f] = d_g[f];
    }
    if (s->arith == SS4D_ARITH_MIXED) {
        // float-float presmoothing of both images, g faces from the
        // float-float results
        double *prev = d_scratch;
        if (!prev) {
            CKS(ensure_scratch(s));
            prev = s->d_scratch;
        }
        CKS(presmooth_ff(s, p, d_i0, prev, 0, nullptr));
        if (d_i0_thr)
            CKS(presmooth_ff(s, p, d_i0_thr, prev, 1, nullptr));
        launch_gfaces_ff(s->geo, s->d_ff, d_i0_thr ? s->d_ff + s->geo.n : nullptr, go, p->h, p->K, p->theta_img,
                         p->rho_thr, s->stream);
        s->launches += 1;
        return last_launch();
    }
    CKS(ss4d_presmooth_step(s, p, d_i0, d_scratch, nullptr));
    if (d_i0_thr)
        CKS(ss4d_presmooth_step(s, p, d_i0_thr, d_scratch, nullptr));
    launch_gfaces(s->geo, d_i0, d_i0_thr, go, p->h, p->K, p->theta_img, p->rho_thr, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_gs_coefficients(ss4d_solver *s, const ss4d_params *p, const double *d_u,
                                            const double *const d_g[8], double *const d_coef[8])
{
    REQ(s && d_u && d_coef, "NULL argument");
    CKS(check_params(p));
    CPtrs8 gi;
    GPtrs8 co;
    for (int f = 0; f < 8; ++f) {
        gi.p[f] = d_g ? d_g[f] : nullptr;
        REQ(!d_g || d_g[f], "a g array is NULL");
        REQ(d_coef[f], "a coefficient array is NULL");
        co.p[f] = d_coef[f];
    }
    launch_coef_ref(s->geo, d_u, gi, d_g ? 1 : 0, co, p->h, p->eps2, s->stream);
    s->launches += 1;
    return last_launch();
}

// solve on the split buffers from natural u/prev; coefficients already in place
// split -> natural u after a loop whose state is d_state; in mixed
// segmentation steps with extrapolation it also keeps the next step's start
// correction: an extrapolation from this step's change and up to order-1
// earlier ones
struct UnpackPlan {
    int save, terms, keep;
};

// the extrapolation terms and history depth of this step's unpack
static ss4d_status unpack_plan(ss4d_solver *s, int mixed, UnpackPlan *u)
{
    u->save = mixed && s->extrap && s->have_g;
    u->terms = u->keep = 0;
    if (u->save) {
        u->keep = s->extrap - 1;
        for (int q = 0; q < 2 * u->keep; ++q) {
            if (!s->hist[q]) {
                CKS(dmalloc(s, (void **)&s->hist[q], sizeof(float) * s->sp.cs));
                // ghost and padding cells stay zero (the projection reads them as neighbours)
                CK(cudaMemsetAsync(s->hist[q], 0, sizeof(float) * s->sp.cs, s->stream));
            }
        }
        u->terms = s->have_dprev + 1 < s->extrap ? s->have_dprev + 1 : s->extrap;
    }
    return SS4D_OK;
}

static void unpack_done(ss4d_solver *s, const UnpackPlan &u)
{
    s->have_dprev = u.save ? (s->have_dprev < 3 ? s->have_dprev + 1 : 3) : 0;
}

static ss4d_status unpack_step(ss4d_solver *s, const LoopState *d_state, double *d_u, int mixed)
{
    UnpackPlan u;
    CKS(unpack_plan(s, mixed, &u));
    timed(s, SS4D_K_PACK, true,
          [&] { launch_unpack(s->geo, s->sp, s->sb, d_state, d_u, s->stream, u.terms, u.keep, s->hist); });
    unpack_done(s, u);
    s->launches += 1;
    return last_launch();
}

// packed: the split copies of u and prev are made already
static ss4d_status split_solve(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *d_prev,
                               ss4d_step_stats *stats, bool packed = false)
{
    const int mixed = s->arith == SS4D_ARITH_MIXED;
    if (!packed) {
        timed(s, SS4D_K_PACK, true, [&] { launch_pack(s->geo, s->sp, d_u, d_prev, s->sb, s->stream); });
        s->launches += 1;
        CKS(last_launch());
    }
    CKS(run_split_loop(s, p, mixed));
    CKS(unpack_step(s, s->d_state, d_u, mixed));
    ss4d_status st = finish_stats(s, stats, mixed);
    count_graph_launches(s, mixed);
    return st;
}

extern "C" ss4d_status ss4d_sor_solve(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *d_prev_u,
                                      const double *const d_coef[8], ss4d_step_stats *stats)
{
    REQ(s && d_u && d_prev_u && d_coef, "NULL argument");
    CKS(check_params(p));
    CPtrs8 a;
    for (int f = 0; f < 8; ++f) {
        REQ(d_coef[f], "a coefficient array is NULL");
        a.p[f] = d_coef[f];
    }
    if (stats)
        memset(stats, 0, sizeof *stats);
    CK(cudaEventRecord(s->ev0, s->stream));
    ss4d_status st;
    if (s->arith == SS4D_ARITH_REFERENCE) {
        st = sor_reference(s, p, d_u, d_prev_u, a, stats);
    } else {
        const int mixed = s->arith == SS4D_ARITH_MIXED;
        CKS(ensure_split(s, mixed));
        launch_pack_coef(s->geo, s->sp, a, *p, s->sb, mixed, s->stream);
        s->launches += 1;
        CKS(last_launch());
        st = split_solve(s, p, d_u, d_prev_u, stats);
    }
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats)
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
    return st;
}

extern "C" ss4d_status ss4d_seg_time_step(ss4d_solver *s, const ss4d_params *p, double *d_u, double *d_prev_u,
                                          const double *const d_g[8], const double *d_Mmask, const ss4d_balls *balls,
                                          ss4d_step_stats *stats)
{
    REQ(s && d_u && d_g, "NULL argument");
    CKS(check_params(p));
    CPtrs8 gi;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        gi.p[f] = d_g[f];
    }
    if (stats)
        memset(stats, 0, sizeof *stats);
    const Geo &g = s->geo;
    CK(cudaEventRecord(s->ev0, s->stream));
    ss4d_status st;
    if (s->arith == SS4D_ARITH_REFERENCE) {
        double *prev = d_prev_u;
        if (!prev) {
            CKS(ensure_scratch(s));
            prev = s->d_scratch;
        }
        CKS(ensure_coef_nat(s));
        CK(cudaMemcpyAsync(prev, d_u, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
        GPtrs8 co;
        CPtrs8 ca;
        for (int f = 0; f < 8; ++f) {
            co.p[f] = s->d_coef_nat + (size_t)f * g.n;
            ca.p[f] = co.p[f];
        }
        launch_coef_ref(g, d_u, gi, 1, co, p->h, p->eps2, s->stream);
        s->launches += 1;
        CKS(last_launch());
        st = sor_reference(s, p, d_u, prev, ca, stats);
    } else {
        const int mixed = s->arith == SS4D_ARITH_MIXED;
        CKS(ensure_split(s, mixed));
        if (d_prev_u)
            CK(cudaMemcpyAsync(d_prev_u, d_u, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
        const int pre = pre_form(s, mixed);
        timed(s, SS4D_K_ASSEMBLE, true, [&] { assemble(s, p, d_u, gi, 1, mixed, 1, pre); });
        CKS(last_launch());
        s->cur_g = gi;
        s->have_g = 1;
        s->pre_next = pre != 0;
        st = split_solve(s, p, d_u, d_u, stats, packed_by_assembly(mixed));
        s->have_g = 0;
    }
    if (st == SS4D_OK)
        st = rescale_impl(s, p, d_u, d_Mmask, balls);
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats)
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
    return st;
}

// ---------------------------------------------------------------------------
// a time step on host arrays, the copies overlapped with the step's work

// prev <- u on host threads (the reference's copy at the start of a step)
struct HostCopy {
    std::vector<std::thread> th;
    void start(double *dst, const double *src, size_t n)
    {
        if (!dst)
            return;
        const int T = 8;
        const size_t per = (n + T - 1) / T;
        for (int t = 0; t < T; ++t) {
            const size_t a = per * t < n ? per * t : n, e = a + per < n ? a + per : n;
            if (e > a)
                th.emplace_back([=] { memcpy(dst + a, src + a, sizeof(double) * (e - a)); });
        }
    }
    void join()
    {
        for (auto &t : th)
            t.join();
        th.clear();
    }
    ~HostCopy() { join(); }
};

extern "C" ss4d_status ss4d_seg_time_step_host(ss4d_solver *s, const ss4d_params *p, double *h_u, double *d_u,
                                               double *h_prev, const double *h_Mmask, double *d_Mmask,
                                               const double *const d_g[8], const ss4d_balls *balls,
                                               ss4d_step_stats *stats)
{
    REQ(s && h_u && d_u && d_g, "NULL argument");
    REQ(!h_Mmask || d_Mmask, "h_Mmask needs d_Mmask");
    CKS(check_params(p));
    const Geo &g = s->geo;
    const size_t frame = (size_t)g.sw, all = (size_t)g.n;
    HostCopy hc;
    hc.start(h_prev, h_u, all);
    if (s->arith == SS4D_ARITH_REFERENCE || s->timing) {
        // the plain sequence (the reference form has no split layout to
        // overlap; per-kernel timing wants the kernels in their own order)
        CK(cudaMemcpyAsync(d_u, h_u, sizeof(double) * all, cudaMemcpyHostToDevice, s->stream));
        if (h_Mmask)
            CK(cudaMemcpyAsync(d_Mmask, h_Mmask, sizeof(double) * all, cudaMemcpyHostToDevice, s->stream));
        CKS(ss4d_seg_time_step(s, p, d_u, nullptr, d_g, h_Mmask ? d_Mmask : nullptr, balls, stats));
        hc.join();
        CK(cudaMemcpyAsync(h_u, d_u, sizeof(double) * all, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        return SS4D_OK;
    }
    CPtrs8 gi;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        gi.p[f] = d_g[f];
    }
    if (stats)
        memset(stats, 0, sizeof *stats);
    const int mixed = s->arith == SS4D_ARITH_MIXED;
    CKS(ensure_split(s, mixed));
    // the centre tables now: they are read only by the rescale, and a copy
    // from pageable memory later could wait for the loop
    int have_balls = 0;
    CKS(upload_balls(s, balls, p->ballRadius, &have_balls));
    CK(cudaEventRecord(s->ev0, s->stream));
    // u goes up in chunks of padded frames on the side stream, after the
    // work already queued on the handle's stream (d_u may be in use there)
    const int C = g.lM < SS4D_HOST_CHUNKS ? g.lM : SS4D_HOST_CHUNKS;
    int F[SS4D_HOST_CHUNKS + 1];
    for (int c = 0; c <= C; ++c)
        F[c] = (int)((long long)c * g.lM / C);
    CK(cudaEventRecord(s->side_ev, s->stream));
    CK(cudaStreamWaitEvent(s->side, s->side_ev, 0));
    for (int c = 0; c < C; ++c) {
        CK(cudaMemcpyAsync(d_u + F[c] * frame, h_u + F[c] * frame, sizeof(double) * frame * (F[c + 1] - F[c]),
                           cudaMemcpyHostToDevice, s->side));
        CK(cudaEventRecord(s->chunk_ev[c], s->side));
    }
    if (h_Mmask) { // needed by the rescale only
        CK(cudaMemcpyAsync(d_Mmask, h_Mmask, sizeof(double) * all, cudaMemcpyHostToDevice, s->side));
        CK(cudaEventRecord(s->mask_ev, s->side));
    }
    // stage c, once chunks c and c + 1 are up (a first difference reads the
    // next frame): the pack of chunk c's frames and, in the mixed form (whose
    // first-difference kernel makes the pack's copies), their first
    // differences and the faces and coefficients whose inputs are then
    // complete (faces of frame l read the differences of l-1 .. l+1, the
    // coefficients of l the faces of l-1 and l); the last stage does the rest
    int fh = 0, vh = 1; // next frame of faces / of coefficients
    const int pre = pre_form(s, mixed);
    for (int c = 0; c < C; ++c) {
        CK(cudaStreamWaitEvent(s->stream, s->chunk_ev[c], 0));
        if (c + 1 < C)
            CK(cudaStreamWaitEvent(s->stream, s->chunk_ev[c + 1], 0));
        if (mixed) {
            launch_fdiff_pack_range(g, s->sp, d_u, s->sb, F[c], F[c + 1], s->sm_count, s->stream, pre);
            const bool last = c + 1 == C;
            int fe = last ? g.nt + 1 : F[c + 1] - 1;
            fe = fe < fh ? fh : (fe > g.nt + 1 ? g.nt + 1 : fe);
            const int ve = fe < vh ? vh : fe;
            launch_assemble_ff_faces_range(g, s->sp, gi, 1, *p, s->sb, fh, fe, vh, ve, s->stream, pre, s->asm_kblock);
            s->launches += 1 + (fe > fh) + (ve > vh);
            fh = fe;
            vh = ve;
        } else {
            launch_pack_range(g, s->sp, d_u, d_u, s->sb, F[c], F[c + 1], s->stream);
            s->launches += 1;
        }
    }
    if (!mixed) {
        launch_assemble(g, s->sp, d_u, gi, 1, *p, s->sb, 0, s->stream);
        s->launches += 2;
    }
    CKS(last_launch());
    s->cur_g = gi;
    s->have_g = 1;
    s->pre_next = pre != 0;
    // mixed form: the loop pauses when a round ends; u formed from that round
    // goes down while its refinement pass decides (below)
    CKS(run_split_loop(s, p, mixed, mixed));
    // the unpack and the rescale per chunk of interior frames, each chunk's
    // download on the side stream as soon as it is done
    UnpackPlan up;
    CKS(unpack_plan(s, mixed, &up));
    if (h_Mmask)
        CK(cudaStreamWaitEvent(s->stream, s->mask_ev, 0));
    hc.join(); // prev has its copy of u before any chunk of u comes down
    const int nt = g.lM - 2, Ci = nt < SS4D_HOST_CHUNKS ? nt : SS4D_HOST_CHUNKS;
    auto download = [&](int what) -> ss4d_status {
        // the side stream's earlier downloads of d_u first (a retried round)
        CK(cudaEventRecord(s->side_ev, s->side));
        CK(cudaStreamWaitEvent(s->stream, s->side_ev, 0));
        for (int c = 0; c < Ci; ++c) {
            const int a = 1 + (int)((long long)c * nt / Ci), e = 1 + (int)((long long)(c + 1) * nt / Ci);
            launch_unpack_range(g, s->sp, s->sb, s->d_state, d_u, s->stream, up.terms, up.keep, s->hist, a, e, what);
            s->launches += 1;
            if (have_balls) {
                launch_rescale_balls_range(g, d_u, s->d_frame_first, s->d_frame_count, s->d_bx, s->d_by, s->d_bz,
                                           p->ballRadius, a, e, s->stream);
                s->launches += 1;
            }
            if (h_Mmask) {
                launch_mask_zero_range(g, d_u, d_Mmask, a, e, s->stream);
                s->launches += 1;
            }
            CK(cudaEventRecord(s->chunk_ev[c], s->stream));
            CK(cudaStreamWaitEvent(s->side, s->chunk_ev[c], 0));
            CK(cudaMemcpyAsync(h_u + a * frame, d_u + a * frame, sizeof(double) * frame * (e - a),
                               cudaMemcpyDeviceToHost, s->side));
        }
        return last_launch();
    };
    // A paused loop's u (the split u plus the round's correction, added as
    // its refinement pass adds it) goes down at once; the pass runs beside the
    // download, and when it ends the step (as a round aimed below the
    // tolerance almost always does) that u is the step's result: only the
    // extrapolation history is left to write.  Otherwise the loop resumes and
    // the result of a later round goes down.
    bool done = false;
    for (int guard = 0; mixed && guard < 4 * (p->maxNoGSIteration + 4) + 16; ++guard) {
        CK(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->h_state->stop || !s->h_state->paused)
            break; // stopped at the step's first refinement pass: as without pausing
        CKS(download(UNPACK_PAUSED));
        CKS(refine_paused(s));
        CK(cudaMemcpyAsync(s->h_state, s->d_state, sizeof(LoopState), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->h_state->stop) {
            if (up.terms > 0) {
                launch_unpack_range(g, s->sp, s->sb, s->d_state, d_u, s->stream, up.terms, up.keep, s->hist, 1,
                                    g.lM - 1, UNPACK_HISTORY);
                s->launches += 1;
            }
            done = true;
            break;
        }
        CKS(drive_loop(s, p, mixed, s->h_state->mode));
    }
    if (!done)
        CKS(download(UNPACK_ALL));
    CKS(last_launch());
    unpack_done(s, up);
    s->have_g = 0;
    ss4d_status st = finish_stats(s, stats, mixed);
    count_graph_launches(s, mixed);
    CK(cudaEventRecord(s->side_ev, s->side));
    CK(cudaStreamWaitEvent(s->stream, s->side_ev, 0));
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats)
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
    return st;
}

extern "C" ss4d_status ss4d_mcf_time_step(ss4d_solver *s, const ss4d_params *p, int numberOfTimeStep, double *d_u,
                                          double *d_prev_u, ss4d_step_stats *stats)
{
    REQ(s && d_u, "NULL argument");
    CKS(check_params(p));
    if (stats)
        memset(stats, 0, sizeof *stats);
    const Geo &g = s->geo;
    const double t = p->tau * numberOfTimeStep;
    double *prev = d_prev_u;
    if (!prev) {
        CKS(ensure_scratch(s));
        prev = s->d_scratch;
    }
    CK(cudaEventRecord(s->ev0, s->stream));
    CK(cudaMemcpyAsync(prev, d_u, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    CPtrs8 none;
    for (int f = 0; f < 8; ++f)
        none.p[f] = nullptr;
    ss4d_status st;
    if (s->arith == SS4D_ARITH_REFERENCE) {
        CKS(ensure_coef_nat(s));
        GPtrs8 co;
        CPtrs8 ca;
        for (int f = 0; f < 8; ++f) {
            co.p[f] = s->d_coef_nat + (size_t)f * g.n;
            ca.p[f] = co.p[f];
        }
        launch_coef_ref(g, d_u, none, 0, co, p->h, p->eps2, s->stream);
        launch_mcf_field(g, d_u, p->h, t, 1, s->stream);
        s->launches += 2;
        CKS(last_launch());
        st = sor_reference(s, p, d_u, prev, ca, stats);
    } else {
        const int mixed = s->arith == SS4D_ARITH_MIXED;
        CKS(ensure_split(s, mixed));
        timed(s, SS4D_K_ASSEMBLE, true, [&] { assemble(s, p, d_u, none, 0, mixed); });
        launch_mcf_field(g, d_u, p->h, t, 1, s->stream);
        s->launches += 1;
        CKS(last_launch());
        st = split_solve(s, p, d_u, prev, stats);
    }
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats)
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
    return st;
}

extern "C" ss4d_status ss4d_rescale_to_zero_one(ss4d_solver *s, const ss4d_params *p, double *d_img,
                                                const double *d_Mmask, const ss4d_balls *balls)
{
    REQ(s && p && d_img, "NULL argument");
    return rescale_impl(s, p, d_img, d_Mmask, balls);
}

extern "C" ss4d_status ss4d_frame_from_bytes(ss4d_solver *s, double *d_img, int l, const uint8_t *d_bytes)
{
    REQ(s && d_img && d_bytes, "NULL argument");
    REQ(l >= 1 && l <= s->geo.nt, "frame index out of range (interior frames are 1..lMax-2)");
    launch_frame_bytes(s->geo, d_img, nullptr, l, 0, d_bytes, nullptr, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_frame_to_bytes(ss4d_solver *s, const double *d_img, int l, int mode, uint8_t *d_bytes)
{
    REQ(s && d_img && d_bytes, "NULL argument");
    REQ(l >= 1 && l <= s->geo.nt, "frame index out of range (interior frames are 1..lMax-2)");
    REQ(mode == 0 || mode == 1, "mode must be 0 (scaled bytes) or 1 (mask)");
    launch_frame_bytes(s->geo, nullptr, d_img, l, mode, nullptr, d_bytes, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_max4d(ss4d_solver *s, const double *d_img, double *out)
{
    REQ(s && d_img && out, "NULL argument");
    s->launches += launch_minmax(s->geo, d_img, s->d_partial, 0.0, s->d_scalar, s->stream);
    CKS(last_launch());
    CK(cudaMemcpyAsync(s->h_scalar, s->d_scalar, sizeof(double) * 2, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *out = s->h_scalar[1] > 0 ? s->h_scalar[1] : 0.0; // the reference's search starts from 0
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_ball_min_max(ss4d_solver *s, const double *d_img, int l, double cx, double cy, double cz,
                                         double R, double *mn, double *mx)
{
    REQ(s && d_img && mn && mx, "NULL argument");
    const Geo &g = s->geo;
    REQ(l >= 0 && l < g.lM, "frame index out of range");
    const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
    const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
    const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
    REQ(k0 >= 0 && j0 >= 0 && i0 >= 0 && k1 < g.kM && j1 < g.jM && i1 < g.iM,
        "the ball's box leaves the array (the reference would read out of bounds)");
    launch_ball_min_max(g, d_img, l, cx, cy, cz, R, s->d_scalar, s->stream);
    s->launches += 1;
    CKS(last_launch());
    CK(cudaMemcpyAsync(s->h_scalar, s->d_scalar, sizeof(double) * 2, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *mn = s->h_scalar[0];
    *mx = s->h_scalar[1];
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_local_threshold(ss4d_solver *s, double alpha, double beta, double ballRadius,
                                            const double *d_in, double *d_thr, const ss4d_balls *balls)
{
    REQ(s && d_in && d_thr, "NULL argument");
    int have = 0;
    CKS(upload_balls(s, balls, ballRadius, &have));
    if (!have)
        return SS4D_OK;
    s->launches += launch_minmax(s->geo, d_in, s->d_partial, 0.0, s->d_scalar, s->stream);
    launch_local_threshold(s->geo, d_in, d_thr, s->d_frame_first, s->d_frame_count, s->d_bx, s->d_by, s->d_bz,
                           ballRadius, alpha, beta, s->d_scalar, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_generate_segm_function(ss4d_solver *s, double ballRadius, double *d_u, double *d_Mmask,
                                                   const ss4d_balls *balls)
{
    REQ(s && d_u && d_Mmask, "NULL argument");
    int have = 0;
    CKS(upload_balls(s, balls, ballRadius, &have));
    if (!have)
        return SS4D_OK;
    launch_generate_segm(s->geo, d_u, d_Mmask, s->d_frame_first, s->d_frame_count, s->d_bx, s->d_by, s->d_bz,
                         ballRadius, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_threshold_mask(ss4d_solver *s, const double *d_u, double level, int normalise,
                                           uint8_t *d_mask)
{
    REQ(s && d_u && d_mask, "NULL argument");
    if (normalise) {
        s->launches += launch_minmax(s->geo, d_u, s->d_partial, level, s->d_scalar, s->stream);
        launch_threshold(s->geo, d_u, s->d_scalar, level, d_mask, s->stream);
        s->launches += 1;
    } else {
        launch_threshold(s->geo, d_u, nullptr, level, d_mask, s->stream);
        s->launches += 1;
    }
    return last_launch();
}

extern "C" ss4d_status ss4d_l2norm(ss4d_solver *s, double h, const double *d_a, const double *d_b, double *out)
{
    REQ(s && d_a && d_b && out, "NULL argument");
    const int nblk = 1024;
    launch_l2(s->geo, d_a, d_b, h * h * h * h, s->d_partial, nblk, s->stream);
    s->launches += 1 + launch_reduce_sum(s->d_partial, nblk, s->d_scalar, s->stream);
    CKS(last_launch());
    double v = 0;
    CKS(read_scalar(s, 0, &v));
    *out = sqrt(v);
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_mass(ss4d_solver *s, double h, const double *d_a, double *out)
{
    REQ(s && d_a && out, "NULL argument");
    const int nblk = 1024;
    launch_mass(s->geo, d_a, h * h * h * h, s->d_partial, nblk, s->stream);
    s->launches += 1 + launch_reduce_sum(s->d_partial, nblk, s->d_scalar, s->stream);
    CKS(last_launch());
    return read_scalar(s, 0, out);
}

extern "C" ss4d_status ss4d_mcf_set_boundary_exact(ss4d_solver *s, double h, double t, double *d_u)
{
    REQ(s && d_u, "NULL argument");
    launch_mcf_field(s->geo, d_u, h, t, 1, s->stream);
    s->launches += 1;
    return last_launch();
}

extern "C" ss4d_status ss4d_mcf_exact_solution(ss4d_solver *s, double h, double t, double *d_out)
{
    REQ(s && d_out, "NULL argument");
    launch_mcf_field(s->geo, d_out, h, t, 0, s->stream);
    s->launches += 1;
    return last_launch();
}

// ---------------------------------------------------------------------------
// memory helpers

extern "C" ss4d_status ss4d_dev_alloc(size_t bytes, void **out)
{
    REQ(out, "out is NULL");
    *out = nullptr;
    return dmalloc(nullptr, out, bytes ? bytes : 1);
}

extern "C" ss4d_status ss4d_dev_free(void *p)
{
    if (p)
        CK(cudaFree(p));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_host_alloc(size_t bytes, void **out)
{
    REQ(out, "out is NULL");
    *out = nullptr;
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err("cudaMallocHost(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return SS4D_ERR_ALLOC;
    }
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_host_free(void *p)
{
    if (p)
        CK(cudaFreeHost(p));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_copy_to_device(ss4d_solver *s, void *d_dst, const void *h_src, size_t bytes)
{
    REQ(s && d_dst && h_src, "NULL argument");
    CK(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, s->stream));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_copy_to_device_side(ss4d_solver *s, void *d_dst, const void *h_src, size_t bytes)
{
    REQ(s && d_dst && h_src, "NULL argument");
    // after what the handle's stream has queued (d_dst may be in use there)
    CK(cudaEventRecord(s->side_ev, s->stream));
    CK(cudaStreamWaitEvent(s->side, s->side_ev, 0));
    CK(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, s->side));
    CK(cudaEventRecord(s->side_ev, s->side));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_join_side(ss4d_solver *s)
{
    REQ(s, "solver is NULL");
    CK(cudaStreamWaitEvent(s->stream, s->side_ev, 0));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_copy_to_host(ss4d_solver *s, void *h_dst, const void *d_src, size_t bytes)
{
    REQ(s && h_dst && d_src, "NULL argument");
    CK(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, s->stream));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_copy_device(ss4d_solver *s, void *d_dst, const void *d_src, size_t bytes)
{
    REQ(s && d_dst && d_src, "NULL argument");
    CK(cudaMemcpyAsync(d_dst, d_src, bytes, cudaMemcpyDeviceToDevice, s->stream));
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_synchronize(ss4d_solver *s)
{
    REQ(s, "solver is NULL");
    CK(cudaStreamSynchronize(s->stream));
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// a handle's colour-split machinery, for the batched solver (ss4d_batch.cu)

int ss4d::solver_sm_count(const ss4d_solver *s)
{
    return s->sm_count;
}

ss4d_status ss4d::solver_view(ss4d_solver *s, SolverView *out)
{
    REQ(s && out, "NULL argument");
    CKS(ensure_split(s, s->arith == SS4D_ARITH_MIXED));
    out->g = s->geo;
    out->sp = s->sp;
    out->cfg = s->cfg;
    out->b = s->sb;
    return SS4D_OK;
}

ss4d_status ss4d::solver_set_shape(ss4d_solver *s, int xt, int kb)
{
    REQ(s && kb >= 1 && xt >= 0 && xt <= 256, "bad tile shape");
    SweepCfg c = make_sweep_cfg_xt(s->geo, s->sp, s->sm_count, kb, xt);
    REQ(2LL * c.grid <= s->n_partial, "grid larger than the partial-sum buffer");
    s->cfg = c;
    s->sb.partial[1] = s->d_partial + c.grid;
    free_graphs(s);
    return SS4D_OK;
}

ss4d_status ss4d::solver_prepare_step(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *const d_g[8],
                                      int *pre_out)
{
    REQ(s && d_u && d_g, "NULL argument");
    CKS(check_params(p));
    CPtrs8 gi;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        gi.p[f] = d_g[f];
    }
    const int mixed = s->arith == SS4D_ARITH_MIXED;
    CKS(ensure_split(s, mixed));
    const int pre = pre_out ? pre_form(s, mixed) : 0;
    if (pre_out)
        *pre_out = pre;
    timed(s, SS4D_K_ASSEMBLE, true, [&] { assemble(s, p, d_u, gi, 1, mixed, 1, pre); });
    CKS(last_launch());
    if (!packed_by_assembly(mixed)) {
        timed(s, SS4D_K_PACK, true, [&] { launch_pack(s->geo, s->sp, d_u, d_u, s->sb, s->stream); });
        s->launches += 1;
    }
    if (mixed) {
        s->have_g = 1; // a segmentation step: its change feeds the extrapolation
        CKS(clear_corrections(s));
    }
    return last_launch();
}

ss4d_status ss4d::solver_project_start(ss4d_solver *s, int pre, LoopState *d_state)
{
    return project_start(s, pre == 2, d_state);
}

ss4d_status ss4d::solver_finish_step(ss4d_solver *s, const LoopState *d_state, double *d_u)
{
    REQ(s && d_state && d_u, "NULL argument");
    const int mixed = s->arith == SS4D_ARITH_MIXED;
    ss4d_status st = unpack_step(s, d_state, d_u, mixed);
    s->have_g = 0;
    return st;
}

ss4d_status ss4d::solver_time_sweeps(ss4d_solver *s, const ss4d_params *p, int iters, float *ms)
{
    REQ(s && p && ms && iters > 0, "bad argument");
    CKS(ensure_split(s, 0));
    CKS(upload_params(s, p));
    launch_loop_init(s->d_state, 0, s->stream); // z stays 0: fixed buffers, as in a real loop
    CK(cudaEventRecord(s->tev0, s->stream));
    for (int it = 0; it < iters; ++it) {
        launch_sweep64(s->geo, s->sp, s->cfg, 1, s->sb, s->d_params, s->d_state, s->stream);
        launch_sweep64(s->geo, s->sp, s->cfg, 0, s->sb, s->d_params, s->d_state, s->stream);
    }
    CK(cudaEventRecord(s->tev1, s->stream));
    CKS(last_launch());
    CK(cudaEventSynchronize(s->tev1));
    CK(cudaEventElapsedTime(ms, s->tev0, s->tev1));
    s->launches += 1 + 2LL * iters;
    return SS4D_OK;
}

// ---------------------------------------------------------------------------
// one slab of a volume split by frames (ss4d_slab.c runs the loop): the
// reference-order kernels on the slab's natural layout

namespace {
struct SlabGpu {
    ss4d_solver *s;
    const ss4d_params *p;
    double *u;
    const double *prev;
    CPtrs8 a;
};

int slab_half_sweep(void *ctx, int colour)
{
    SlabGpu *q = static_cast<SlabGpu *>(ctx);
    launch_sor_half_ref(q->s->geo, q->u, q->prev, q->a, q->p->tau / (q->p->h * q->p->h), q->p->omega_c, colour,
                        q->s->stream);
    q->s->launches += 1;
    return last_launch() != SS4D_OK;
}

int slab_residual(void *ctx, double *partial)
{
    SlabGpu *q = static_cast<SlabGpu *>(ctx);
    const Geo &g = q->s->geo;
    const double h2 = q->p->h * q->p->h;
    launch_sor_resid_ref(g, q->u, q->prev, q->a, q->p->tau / h2, h2 * h2, q->s->d_partial, q->s->stream);
    q->s->launches += 1 + launch_reduce_sum(q->s->d_partial, resid_blocks(g), q->s->d_scalar, q->s->stream);
    if (last_launch() != SS4D_OK)
        return 1;
    return read_scalar(q->s, 0, partial) != SS4D_OK;
}
} // namespace

extern "C" ss4d_status ss4d_slab_sor_solve(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *d_prev_u,
                                           const double *const d_coef[8], const ss4d_slab_comm *comm,
                                           long long nint_global, ss4d_step_stats *stats)
{
    REQ(s && d_u && d_prev_u && d_coef && comm, "NULL argument");
    CKS(check_params(p));
    SlabGpu q{s, p, d_u, d_prev_u, {}};
    for (int f = 0; f < 8; ++f) {
        REQ(d_coef[f], "a coefficient array is NULL");
        q.a.p[f] = d_coef[f];
    }
    const Geo &g = s->geo;
    ss4d_slab_ops ops{&q, slab_half_sweep, slab_residual, d_u, g.sw, g.lM, (void *)s->stream};
    CK(cudaEventRecord(s->ev0, s->stream));
    ss4d_status st = ss4d_slab_sor_loop(&ops, comm, p, nint_global, stats);
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    if (stats)
        cudaEventElapsedTime(&stats->ms, s->ev0, s->ev1);
    return st;
}

extern "C" ss4d_status ss4d_slab_seg_time_step(ss4d_solver *s, const ss4d_params *p, double *d_u, double *d_prev_u,
                                               const double *const d_g[8], const double *d_Mmask,
                                               const ss4d_balls *balls, const ss4d_slab_comm *comm,
                                               long long nint_global, ss4d_step_stats *stats)
{
    REQ(s && d_u && d_g && comm && comm->exchange, "NULL argument");
    CKS(check_params(p));
    CPtrs8 gi;
    for (int f = 0; f < 8; ++f) {
        REQ(d_g[f], "a g array is NULL");
        gi.p[f] = d_g[f];
    }
    const Geo &g = s->geo;
    double *prev = d_prev_u;
    if (!prev) {
        CKS(ensure_scratch(s));
        prev = s->d_scratch;
    }
    CKS(ensure_coef_nat(s));
    // the coefficients of the slab's first and last frames read u in the
    // neighbours' frames: bring the ghosts up to date first
    if (comm->exchange(comm->ctx, d_u, g.sw, g.lM, (void *)s->stream)) {
        set_err("ss4d_slab_seg_time_step: the ghost-frame exchange failed");
        return SS4D_ERR_CUDA;
    }
    CK(cudaMemcpyAsync(prev, d_u, sizeof(double) * g.n, cudaMemcpyDeviceToDevice, s->stream));
    GPtrs8 co;
    const double *ca[8];
    for (int f = 0; f < 8; ++f) {
        co.p[f] = s->d_coef_nat + (size_t)f * g.n;
        ca[f] = co.p[f];
    }
    launch_coef_ref(g, d_u, gi, 1, co, p->h, p->eps2, s->stream);
    s->launches += 1;
    CKS(last_launch());
    ss4d_step_stats local;
    ss4d_status st = ss4d_slab_sor_solve(s, p, d_u, prev, ca, comm, nint_global, stats ? stats : &local);
    if (st == SS4D_OK)
        st = rescale_impl(s, p, d_u, d_Mmask, balls);
    // as the reference's rescale ends (segmentation4D_mpi.c:1256): the ghosts
    // hold the neighbours' rescaled frames
    if (st == SS4D_OK && comm->exchange(comm->ctx, d_u, g.sw, g.lM, (void *)s->stream)) {
        set_err("ss4d_slab_seg_time_step: the ghost-frame exchange failed");
        return SS4D_ERR_CUDA;
    }
    CK(cudaStreamSynchronize(s->stream));
    return st;
}
