// ss4d_noalloc.cu — the per-step rescale (_rescale4DdataToZeroOne_,
// segmentation4D.c:1020-1104) for callers that cannot allocate device memory.
//
// ss4d_rescale_to_zero_one stages the centre table and the per-frame index
// tables in buffers its solver handle cudaMalloc's.  A caller whose device
// memory is owned entirely by its own pool, or that must not pay the implicit
// synchronisation of cudaMalloc inside its per-frame loop, cannot use that
// path.  This entry point takes no handle and allocates nothing: it stages
// the same tables in one fixed array of this library and launches the same
// kernels.  The array holds at most SS4D_NOALLOC_MAX_BALLS centres and
// SS4D_NOALLOC_MAX_FRAMES frames (32 KB); every device that loads the library
// keeps it until the process exits.
//
// Sharing: every call writes the whole table region it uses (its centres and
// all lMax frame counts, so frames without centres read zero) before its
// kernels run, in stream order, and copies only that region (3n + lMax
// doubles).  Calls whose GPU work overlaps race on the array.
#include <cuda_runtime.h>

#include <math.h>
#include <mutex>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "ss4d_kernels.cuh"

using namespace ss4d;

// A call with n centres and lMax frames uses the first 3n + lMax doubles:
// cx[n] cy[n] cz[n] | frame_first[lMax] frame_count[lMax] (ints, two per double),
// packed so that one copy of exactly that many bytes stages them.
#define NOALLOC_DOUBLES (3 * SS4D_NOALLOC_MAX_BALLS + SS4D_NOALLOC_MAX_FRAMES)

static __device__ __align__(256) double g_rescale_scratch[NOALLOC_DOUBLES];

// device address of g_rescale_scratch per device; in host code the symbol
// itself is only a host-side stand-in
#define NOALLOC_MAX_DEVICES 64
static double *g_scratch_dev[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;

static ss4d_status fail(ss4d_status st, const char *fmt, ...)
{
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error_text(buf);
    return st;
}

// once per device, with that device current
static ss4d_status scratch_address(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorNoDevice ? SS4D_ERR_NO_DEVICE : SS4D_ERR_CUDA, "cudaGetDevice failed: %s",
                    cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(SS4D_ERR_UNSUPPORTED, "device ordinal %d beyond %d", dev, NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_rescale_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(SS4D_ERR_CUDA, "cudaGetSymbolAddress(rescale scratch) failed: %s", cudaGetErrorString(e));
        }
        g_scratch_dev[dev] = (double *)p;
    }
    *out = g_scratch_dev[dev];
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_rescale_to_zero_one_noalloc(const ss4d_dims *dims, const ss4d_params *p, double *d_img,
                                                        const double *d_Mmask, const ss4d_balls *balls, void *stream)
{
    if (!dims || !p || !d_img)
        return fail(SS4D_ERR_INVALID, "invalid argument: NULL dims, params or image");
    if (dims->iMax < 3 || dims->jMax < 3 || dims->kMax < 3 || dims->lMax < 3)
        return fail(SS4D_ERR_INVALID, "invalid argument: every padded extent must be >= 3");
    if ((long long)dims->iMax * dims->jMax * dims->kMax * dims->lMax >= (1LL << 31))
        return fail(SS4D_ERR_INVALID, "invalid argument: padded volume must hold fewer than 2^31 voxels");
    if ((long long)(dims->kMax - 2) * (dims->lMax - 2) > 65535)
        return fail(SS4D_ERR_INVALID, "invalid argument: (kMax-2)*(lMax-2) must not exceed 65535");
    if (dims->lMax > SS4D_NOALLOC_MAX_FRAMES)
        return fail(SS4D_ERR_INVALID, "lMax = %d exceeds the %d frames the allocation-free rescale holds", dims->lMax,
                    SS4D_NOALLOC_MAX_FRAMES);
    const int nb = balls ? balls->n : 0;
    if (nb < 0 || nb > SS4D_NOALLOC_MAX_BALLS)
        return fail(SS4D_ERR_INVALID, "%d centres exceed the %d the allocation-free rescale holds", nb,
                    SS4D_NOALLOC_MAX_BALLS);
    const Geo g = make_geo(*dims);
    cudaStream_t st = (cudaStream_t)stream;
    const double R = p->ballRadius;

    if (nb > 0) {
        if (!balls->l || !balls->cx || !balls->cy || !balls->cz)
            return fail(SS4D_ERR_INVALID, "invalid argument: balls arrays are NULL");
        // host staging on the stack: pageable, so the copy below has read it
        // by the time cudaMemcpyAsync returns
        double stage[NOALLOC_DOUBLES];
        const size_t used = 3 * (size_t)nb + (size_t)g.lM;  // doubles this call stages
        int *first = (int *)(stage + 3 * nb);
        int *count = first + g.lM;
        memset(first, 0, sizeof(int) * 2 * (size_t)g.lM);
        int prev_l = -1;
        for (int i = 0; i < nb; ++i) {
            const int l = balls->l[i];
            if (l < 1 || l > g.lM - 2)
                return fail(SS4D_ERR_INVALID, "invalid argument: ball frame index %d out of range", l);
            if (l < prev_l)
                return fail(SS4D_ERR_INVALID, "invalid argument: balls must be ordered by frame");
            if (l != prev_l)
                first[l] = i;
            count[l] += 1;
            prev_l = l;
            const double cx = balls->cx[i], cy = balls->cy[i], cz = balls->cz[i];
            const int k0 = (int)(cz - R - 0.5), k1 = (int)(cz + R + 0.5);
            const int j0 = (int)(cy - R - 0.5), j1 = (int)(cy + R + 0.5);
            const int i0 = (int)(cx - R - 0.5), i1 = (int)(cx + R + 0.5);
            if (k0 < 0 || j0 < 0 || i0 < 0 || k1 >= g.kM || j1 >= g.jM || i1 >= g.iM)
                return fail(SS4D_ERR_INVALID,
                            "invalid argument: a ball's box leaves the array (the reference would read out of bounds)");
            stage[i] = cx;
            stage[nb + i] = cy;
            stage[2 * nb + i] = cz;
        }
        double *scratch = nullptr;
        ss4d_status s0 = scratch_address(&scratch);
        if (s0 != SS4D_OK)
            return s0;
        cudaError_t e = cudaMemcpyAsync(scratch, stage, used * sizeof(double), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SS4D_ERR_CUDA, "staging the centre table failed: %s", cudaGetErrorString(e));
        }
        const int *d_first = (const int *)(scratch + 3 * nb);
        launch_rescale_balls(g, d_img, d_first, d_first + g.lM, scratch, scratch + nb, scratch + 2 * nb, R, st);
    }
    if (d_Mmask)
        launch_mask_zero(g, d_img, d_Mmask, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(SS4D_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return SS4D_OK;
}
