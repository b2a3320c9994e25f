// ss4d_nn.cu — the learned warm start: a 4-layer 3x3x3 convolutional network
// (BF16 weights and activations, FP32 accumulation) with its forward, its
// gradients and its optimiser, as hand-written kernels.
//
// Tensors are channel-group planar: [F][C/8][nz][ny][nx][8] with C = 16 or
// 32 BF16 channels (16 input features; 24 hidden channels, the rest zero).  Every
// convolution, forward and data gradient, runs on the tcgen05 tensor cores
// (ss4d_conv_tc.cu): an implicit GEMM per frame, M = voxels, N = output
// channels, K = 27 taps x input channels.  The data gradient of a layer is
// the same convolution with the taps reversed and the channel roles swapped;
// the weight gradient is an FP32 reduction over voxels with a fixed
// summation order (this file).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ss4d_conv_tc.cuh"
#include "ss4d_kernels.cuh"

namespace ss4d {
namespace nn {

constexpr int TX = 8, TY = 8, TZ = 4;
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int TV = TX * TY * TZ; // 256 output voxels per tile
constexpr int HV = HX * HY * HZ; // 600 input voxels per tile

// dW[tap][co][ci] and db[co] summed over the voxels of each block's tiles
// (FP32); X: planar, CIN channels (the layer input), dY: planar, YS channels
// of which COUT are used.  Each block writes its partial sums; k_reduce_cols adds them in
// block order.
__host__ __device__ constexpr int wgrad_smem_bytes(int cin, int cout)
{
    return (HV * cin + TV * cout) * 4;
}

template <int CIN, int COUT, int YS>
__global__ void __launch_bounds__(256) k_wgrad(const __nv_bfloat16 *__restrict__ x,
                                               const __nv_bfloat16 *__restrict__ dy, int nx, int ny, int nz, int nf,
                                               float *partial)
{
    constexpr int NOUT = 27 * COUT * CIN;
    constexpr int NP = (COUT * CIN + 255) / 256; // (co, ci) pairs per thread
    extern __shared__ float wsm[];
    float *sx = wsm;
    float *sd = wsm + HV * CIN;
    float acc[NP][27], bacc = 0.f;
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
        for (int t = 0; t < 27; ++t)
            acc[p][t] = 0.f;
    const int tid = threadIdx.x;
    const int ntx = (nx + TX - 1) / TX, nty = (ny + TY - 1) / TY, ntz = (nz + TZ - 1) / TZ;
    const long long ntiles = (long long)ntx * nty * ntz * nf;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        long long r = tile;
        const int tx0 = (int)(r % ntx) * TX;
        r /= ntx;
        const int ty0 = (int)(r % nty) * TY;
        r /= nty;
        const int tz0 = (int)(r % ntz) * TZ;
        const int f = (int)(r / ntz);
        __syncthreads();
        for (int q = tid; q < HV * CIN; q += blockDim.x) {
            const int v = q / CIN, c = q % CIN;
            const int gx = tx0 + v % HX - 1, gy = ty0 + (v / HX) % HY - 1, gz = tz0 + v / (HX * HY) - 1;
            float val = 0.f;
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz)
                val = __bfloat162float(
                    x[tc::planar_off(f, c, CIN / 8, (long long)nx * ny * nz, ((long long)gz * ny + gy) * nx + gx)]);
            sx[q] = val;
        }
        for (int q = tid; q < TV * COUT; q += blockDim.x) {
            const int m = q / COUT, c = q % COUT;
            const int ox = tx0 + m % TX, oy = ty0 + (m / TX) % TY, oz = tz0 + m / (TX * TY);
            float val = 0.f;
            if (ox < nx && oy < ny && oz < nz)
                val = __bfloat162float(
                    dy[tc::planar_off(f, c, YS / 8, (long long)nx * ny * nz, ((long long)oz * ny + oy) * nx + ox)]);
            sd[q] = val;
        }
        __syncthreads();
        for (int m = 0; m < TV; ++m) {
            const int hbase = ((m / (TX * TY) + 1) * HY + ((m / TX) % TY) + 1) * HX + (m % TX) + 1;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const int q = tid + 256 * p;
                if (q < COUT * CIN) {
                    const int co = q / CIN, ci = q % CIN;
                    const float d = sd[m * COUT + co];
                    const float *xb = sx + hbase * CIN + ci;
#pragma unroll
                    for (int t = 0; t < 27; ++t)
                        acc[p][t] = fmaf(xb[(((t / 9 - 1) * HY + ((t / 3) % 3 - 1)) * HX + (t % 3 - 1)) * CIN], d,
                                         acc[p][t]);
                }
            }
            if (tid < COUT)
                bacc += sd[m * COUT + tid];
        }
    }
    // partial row of this block: [27][COUT][CIN] then [COUT]
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int q = tid + 256 * p;
        if (q < COUT * CIN)
#pragma unroll
            for (int t = 0; t < 27; ++t)
                partial[(size_t)blockIdx.x * (NOUT + COUT) + (size_t)t * COUT * CIN + q] = acc[p][t];
    }
    if (tid < COUT)
        partial[(size_t)blockIdx.x * (NOUT + COUT) + NOUT + tid] = bacc;
}

// out[c] = sum over rows r of in[r][c], rows in order
__global__ void k_reduce_cols(const float *__restrict__ in, int rows, int cols, float *out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols)
        return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r)
        s += in[(size_t)r * cols + c];
    out[c] = s;
}

// squared error over the voxels at least `margin` from the crop border;
// dy (channel 0 of 16, planar) = d(mean squared error)/d out
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ target, int nx, int ny, int nz, int nf,
                      int margin, float inv_count, __nv_bfloat16 *dy, float *partial)
{
    float acc = 0.f;
    const long long n = (long long)nx * ny * nz * nf;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        long long r = v;
        const int x = (int)(r % nx);
        r /= nx;
        const int y = (int)(r % ny);
        r /= ny;
        const int z = (int)(r % nz);
        const bool inside = x >= margin && x < nx - margin && y >= margin && y < ny - margin && z >= margin &&
                            z < nz - margin;
        float g = 0.f;
        if (inside) {
            const float d = out[v] - target[v];
            acc += d * d;
            g = 2.f * d * inv_count;
        }
        const long long vol = (long long)nx * ny * nz, f = v / vol, vf = v - f * vol;
        __nv_bfloat162 *g0 = reinterpret_cast<__nv_bfloat162 *>(dy + tc::planar_off((int)f, 0, 2, vol, vf));
        __nv_bfloat162 *g1 = reinterpret_cast<__nv_bfloat162 *>(dy + tc::planar_off((int)f, 8, 2, vol, vf));
        g0[0] = __floats2bfloat162_rn(g, 0.f);
#pragma unroll
        for (int c = 1; c < 4; ++c)
            g0[c] = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            g1[c] = __floats2bfloat162_rn(0.f, 0.f);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0)
        partial[blockIdx.x] = acc;
}

// Adam on the FP32 master parameters
__global__ void k_adam(float *p, const float *__restrict__ g, float *m, float *v, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// gradient rows of the weight partials -> master layout [27][cout][cin_real] + bias
__global__ void k_unpack_grad(const float *__restrict__ gsum, int cout, int cinp, int cin, float *gw, float *gb)
{
    const int n = 27 * cout * cin;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) {
        const int tap = q / (cout * cin), r = q % (cout * cin), co = r / cin, ci = r % cin;
        gw[q] = gsum[((size_t)tap * cout + co) * cinp + ci];
    } else if (q < n + cout) {
        gb[q - n] = gsum[27 * cout * cinp + (q - n)];
    }
}

} // namespace nn
} // namespace ss4d

// ===========================================================================
// host side: the network handle

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

using namespace ss4d;
using namespace ss4d::nn;

namespace {

struct Layer {
    int cin, cout;   // real channels
    int cinp, nout;  // stored input channels (the convolution's CIN), output channels computed (its N)
    int coutp_t;     // channels of this layer's output gradient as a data-gradient input (16 or 32)
    size_t w_off, b_off;
};

// 16 -> 24 -> 24 -> 24 -> 1; a tcgen05 MMA with M = 128 computes N = 32 (or
// 16) output channels, the ones beyond cout with zero weights
const Layer kLayers[4] = {
    {16, 24, 16, 32, 32, 0, 0},
    {24, 24, 32, 32, 32, 0, 0},
    {24, 24, 32, 32, 32, 0, 0},
    {24, 1, 32, 16, 16, 0, 0},
};

ss4d_status nfail(ss4d_status st, const char *fmt, ...)
{
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error_text(buf);
    return st;
}

#define NCK(call)                                                                                                  \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            cudaGetLastError();                                                                                    \
            return nfail(e_ == cudaErrorMemoryAllocation ? SS4D_ERR_ALLOC : SS4D_ERR_CUDA, "%s failed: %s", #call, \
                         cudaGetErrorString(e_));                                                                  \
        }                                                                                                          \
    } while (0)

} // namespace

struct ss4d_wsnet {
    cudaStream_t stream;
    int sm;
    size_t nparam;
    float *p, *g, *m, *v;          // master parameters, gradients, Adam moments (FP32, flat)
    __nv_bfloat16 *wf[4], *wt[4];  // forward / data-gradient weights as tcgen05 B operands (tc::pack_tc)
    int *err;                      // set by a convolution that gave up a bounded wait (reset per forward)
    int withhold_loads;            // test of the timeout path (ss4d_wsnet_set_test_withhold_loads)
    float *bias[4];                // views into p
    // activations and gradients, sized for `cap` voxels
    size_t cap;
    __nv_bfloat16 *a[3], *dz16, *dz32[2];
    float *y;
    float *partial;                // weight-gradient partials
    size_t partial_cap;
    float *gsum;                   // reduced weight gradient of one layer
    float *loss_part;
    float h_loss;
    long long step;
    int launch_failed;
};

static size_t layer_offsets(size_t *w_off, size_t *b_off)
{
    size_t off = 0;
    for (int L = 0; L < 4; ++L) {
        w_off[L] = off;
        off += (size_t)27 * kLayers[L].cout * kLayers[L].cin;
        b_off[L] = off;
        off += kLayers[L].cout;
    }
    return off;
}

extern "C" size_t ss4d_wsnet_param_count(void)
{
    size_t w[4], b[4];
    return layer_offsets(w, b);
}

extern "C" ss4d_status ss4d_wsnet_destroy(ss4d_wsnet *n)
{
    if (!n)
        return SS4D_OK;
    cudaStreamSynchronize(n->stream);
    void *ptrs[] = {n->p, n->g, n->m, n->v, n->a[0], n->a[1], n->a[2], n->dz16, n->dz32[0], n->dz32[1], n->y,
                    n->partial, n->gsum, n->loss_part, n->err};
    for (void *q : ptrs)
        if (q)
            cudaFree(q);
    for (int L = 0; L < 4; ++L) {
        if (n->wf[L])
            cudaFree(n->wf[L]);
        if (n->wt[L])
            cudaFree(n->wt[L]);
    }
    free(n);
    return SS4D_OK;
}

static void set_conv_attrs()
{
    static bool done = false;
    if (done)
        return;
    cudaFuncSetAttribute(k_wgrad<16, 24, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, wgrad_smem_bytes(16, 24));
    cudaFuncSetAttribute(k_wgrad<32, 24, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, wgrad_smem_bytes(32, 24));
    cudaFuncSetAttribute(k_wgrad<32, 1, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, wgrad_smem_bytes(32, 1));
    done = true;
}

extern "C" ss4d_status ss4d_wsnet_create(void *stream, ss4d_wsnet **out)
{
    if (!out)
        return nfail(SS4D_ERR_INVALID, "invalid argument: out is NULL");
    *out = nullptr;
    ss4d_wsnet *n = (ss4d_wsnet *)calloc(1, sizeof(ss4d_wsnet));
    if (!n)
        return SS4D_ERR_ALLOC;
    n->stream = (cudaStream_t)stream;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n->sm, cudaDevAttrMultiProcessorCount, dev);
    size_t woff[4], boff[4];
    n->nparam = layer_offsets(woff, boff);
    cudaError_t e = cudaMalloc((void **)&n->p, n->nparam * 4);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->g, n->nparam * 4);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->m, n->nparam * 4);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->v, n->nparam * 4);
    for (int L = 0; L < 4 && e == cudaSuccess; ++L) {
        e = cudaMalloc((void **)&n->wf[L], tc::packed_tc_elems(kLayers[L].cinp, kLayers[L].nout) * 2);
        if (e == cudaSuccess && L > 0)
            e = cudaMalloc((void **)&n->wt[L], tc::packed_tc_elems(kLayers[L].coutp_t, 32) * 2);
        n->bias[L] = n->p + boff[L];
    }
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->err, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->gsum, (size_t)(27 * 24 * 32 + 24) * 4);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&n->loss_part, 4096 * 4);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ss4d_wsnet_destroy(n);
        return nfail(SS4D_ERR_ALLOC, "network allocation failed: %s", cudaGetErrorString(e));
    }
    cudaMemsetAsync(n->m, 0, n->nparam * 4, n->stream);
    cudaMemsetAsync(n->v, 0, n->nparam * 4, n->stream);
    cudaMemsetAsync(n->err, 0, sizeof(int), n->stream);
    set_conv_attrs();
    *out = n;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_wsnet_set_stream(ss4d_wsnet *n, void *stream)
{
    if (!n)
        return nfail(SS4D_ERR_INVALID, "invalid argument: network is NULL");
    n->stream = (cudaStream_t)stream;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_wsnet_set_test_withhold_loads(ss4d_wsnet *n, int enable)
{
    if (!n)
        return nfail(SS4D_ERR_INVALID, "invalid argument: network is NULL");
    n->withhold_loads = enable ? 1 : 0;
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_wsnet_check(ss4d_wsnet *n)
{
    if (!n)
        return nfail(SS4D_ERR_INVALID, "invalid argument: network is NULL");
    int h = 0;
    NCK(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
    if (h)
        return nfail(SS4D_ERR_TIMEOUT, "a tensor-core convolution gave up a bounded wait; its output was made NaN");
    return SS4D_OK;
}

static ss4d_status pack_all(ss4d_wsnet *n)
{
    size_t woff[4], boff[4];
    layer_offsets(woff, boff);
    for (int L = 0; L < 4; ++L) {
        const Layer &l = kLayers[L];
        tc::pack_tc(n->p + woff[L], l.cout, l.cin, 0, l.cinp, l.nout, n->wf[L], n->stream);
        if (L > 0) // data gradient: input = this layer's output gradient, output = its input channels
            tc::pack_tc(n->p + woff[L], l.cout, l.cin, 1, l.coutp_t, 32, n->wt[L], n->stream);
    }
    NCK(cudaGetLastError());
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_wsnet_set_params(ss4d_wsnet *n, const float *h_params)
{
    if (!n || !h_params)
        return nfail(SS4D_ERR_INVALID, "invalid argument: NULL network or parameters");
    NCK(cudaMemcpyAsync(n->p, h_params, n->nparam * 4, cudaMemcpyHostToDevice, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
    return pack_all(n);
}

extern "C" ss4d_status ss4d_wsnet_get_params(ss4d_wsnet *n, float *h_params)
{
    if (!n || !h_params)
        return nfail(SS4D_ERR_INVALID, "invalid argument: NULL network or buffer");
    NCK(cudaMemcpyAsync(h_params, n->p, n->nparam * 4, cudaMemcpyDeviceToHost, n->stream));
    NCK(cudaStreamSynchronize(n->stream));
    return SS4D_OK;
}

// He-normal weights (std sqrt(2 / (27 cin))), the output layer scaled by
// 1/10 so an untrained network predicts almost no correction; zero biases
extern "C" ss4d_status ss4d_wsnet_init(ss4d_wsnet *n, uint64_t seed)
{
    if (!n)
        return nfail(SS4D_ERR_INVALID, "invalid argument: network is NULL");
    float *h = (float *)calloc(n->nparam, 4);
    if (!h)
        return SS4D_ERR_ALLOC;
    size_t woff[4], boff[4];
    layer_offsets(woff, boff);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int L = 0; L < 4; ++L) {
        const double sd = sqrt(2.0 / (27.0 * kLayers[L].cin)) * (L == 3 ? 0.1 : 1.0);
        const size_t nw = (size_t)27 * kLayers[L].cout * kLayers[L].cin;
        for (size_t q = 0; q < nw; ++q)
            h[woff[L] + q] = (float)(sd * sqrt(-2.0 * log(next())) * cos(6.283185307179586 * next()));
    }
    ss4d_status st = ss4d_wsnet_set_params(n, h);
    free(h);
    cudaMemsetAsync(n->m, 0, n->nparam * 4, n->stream);
    cudaMemsetAsync(n->v, 0, n->nparam * 4, n->stream);
    n->step = 0;
    return st;
}

static ss4d_status ensure_act(ss4d_wsnet *n, size_t vox, bool train)
{
    if (vox <= n->cap && (!train || n->dz16))
        return SS4D_OK;
    void *old[] = {n->a[0], n->a[1], n->a[2], n->dz16, n->dz32[0], n->dz32[1], n->y};
    for (void *q : old)
        if (q)
            cudaFree(q);
    n->a[0] = n->a[1] = n->a[2] = n->dz16 = n->dz32[0] = n->dz32[1] = nullptr;
    n->y = nullptr;
    const size_t cap = vox > n->cap ? vox : n->cap;
    NCK(cudaMalloc((void **)&n->a[0], cap * 64));
    NCK(cudaMalloc((void **)&n->a[1], cap * 64));
    NCK(cudaMalloc((void **)&n->y, cap * 4));
    if (train) {
        NCK(cudaMalloc((void **)&n->a[2], cap * 64));
        NCK(cudaMalloc((void **)&n->dz16, cap * 32));
        NCK(cudaMalloc((void **)&n->dz32[0], cap * 64));
        NCK(cudaMalloc((void **)&n->dz32[1], cap * 64));
    }
    n->cap = cap;
    return SS4D_OK;
}

static int conv_grid(const ss4d_wsnet *n, int nx, int ny, int nz, int nf)
{
    const long long tiles = (long long)((nx + TX - 1) / TX) * ((ny + TY - 1) / TY) * ((nz + TZ - 1) / TZ) * nf;
    const long long g = (long long)n->sm * 2;
    return (int)(tiles < g ? tiles : g);
}

// one convolution on the tensor cores: cin input channels (16 or 32), nout
// computed output channels (32, or 16 for the output layer), cout of them real
static void conv(ss4d_wsnet *n, int cin, int nout, int cout, const __nv_bfloat16 *x, const __nv_bfloat16 *w,
                 const float *bias, const __nv_bfloat16 *mask, __nv_bfloat16 *y, float *yf, int nx, int ny, int nz,
                 int nf, int relu)
{
    tc::TcArgs a;
    a.w = w;
    a.bias = bias;
    a.mask = mask;
    a.y = y;
    a.yf = yf;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.nf = nf;
    a.cout = cout;
    a.ystride = 32;
    a.mstride = 32;
    a.relu = relu;
    a.err = n->err;
    a.withhold_loads = n->withhold_loads;
    if (tc::conv_tc(cin, nout, x, a, n->sm, n->stream) != cudaSuccess)
        n->launch_failed = 1;
}

// forward over F frames of extents nx, ny, nz; x0 planar [F][2][nz][ny][nx][8] BF16.
// With train, a[0..2] keep the three hidden activations for the backward.
static ss4d_status forward(ss4d_wsnet *n, const __nv_bfloat16 *x0, int nx, int ny, int nz, int nf, bool train,
                           float *out)
{
    const size_t vox = (size_t)nx * ny * nz * nf;
    NCK(ensure_act(n, vox, train) == SS4D_OK ? cudaSuccess : cudaErrorMemoryAllocation);
    __nv_bfloat16 *a1 = n->a[0], *a2 = n->a[1], *a3 = train ? n->a[2] : n->a[0];
    n->launch_failed = 0;
    NCK(cudaMemsetAsync(n->err, 0, sizeof(int), n->stream)); // this forward's waits only
    conv(n, 16, 32, 24, x0, n->wf[0], n->bias[0], nullptr, a1, nullptr, nx, ny, nz, nf, 1);
    conv(n, 32, 32, 24, a1, n->wf[1], n->bias[1], nullptr, a2, nullptr, nx, ny, nz, nf, 1);
    conv(n, 32, 32, 24, a2, n->wf[2], n->bias[2], nullptr, a3, nullptr, nx, ny, nz, nf, 1);
    float *y = out ? out : n->y;
    conv(n, 32, 16, 1, a3, n->wf[3], n->bias[3], nullptr, nullptr, y, nx, ny, nz, nf, 0);
    tc::poison_if_err(n->err, y, (long long)vox, n->stream);
    NCK(cudaGetLastError());
    if (n->launch_failed)
        return nfail(SS4D_ERR_CUDA, "a tensor-core convolution could not be launched (tensor map or launch)");
    return SS4D_OK;
}

extern "C" ss4d_status ss4d_wsnet_forward(ss4d_wsnet *n, const void *d_x0, int nx, int ny, int nz, int nf,
                                          float *d_out)
{
    if (!n || !d_x0 || !d_out || nx < 1 || ny < 1 || nz < 1 || nf < 1)
        return nfail(SS4D_ERR_INVALID, "invalid argument to the network forward");
    return forward(n, (const __nv_bfloat16 *)d_x0, nx, ny, nz, nf, false, d_out);
}

template <int CIN, int COUT, int YS>
static ss4d_status wgrad(ss4d_wsnet *n, const __nv_bfloat16 *x, const __nv_bfloat16 *dy, int nx, int ny, int nz,
                         int nf, int cin_real, float *gw, float *gb)
{
    const int grid = conv_grid(n, nx, ny, nz, nf);
    const size_t cols = (size_t)27 * COUT * CIN + COUT;
    if (n->partial_cap < cols * grid) {
        if (n->partial)
            cudaFree(n->partial);
        n->partial = nullptr;
        NCK(cudaMalloc((void **)&n->partial, cols * grid * 4));
        n->partial_cap = cols * grid;
    }
    k_wgrad<CIN, COUT, YS><<<grid, 256, wgrad_smem_bytes(CIN, COUT), n->stream>>>(x, dy, nx, ny, nz, nf, n->partial);
    k_reduce_cols<<<(int)((cols + 255) / 256), 256, 0, n->stream>>>(n->partial, grid, (int)cols, n->gsum);
    const int nmaster = 27 * COUT * cin_real + COUT;
    k_unpack_grad<<<(nmaster + 255) / 256, 256, 0, n->stream>>>(n->gsum, COUT, CIN, cin_real, gw, gb);
    NCK(cudaGetLastError());
    return SS4D_OK;
}

// one Adam step on crops: x0 planar [F][2][nz][ny][nx][8] BF16 features, target
// [F][nz][ny][nx] FP32; the loss is the mean squared error over voxels at
// least `margin` from the crop borders.  d_grad (nparam floats, may be NULL)
// receives the gradient; lr == 0 computes loss and gradient without updating.
extern "C" ss4d_status ss4d_wsnet_train_step(ss4d_wsnet *n, const void *d_x0, const float *d_target, int nx, int ny,
                                             int nz, int nf, int margin, float lr, float *loss_out, float *d_grad)
{
    if (!n || !d_x0 || !d_target || nx <= 2 * margin || ny <= 2 * margin || nz <= 2 * margin || nf < 1)
        return nfail(SS4D_ERR_INVALID, "invalid argument to the training step");
    const __nv_bfloat16 *x0 = (const __nv_bfloat16 *)d_x0;
    if (forward(n, x0, nx, ny, nz, nf, true, nullptr) != SS4D_OK)
        return SS4D_ERR_CUDA;
    size_t woff[4], boff[4];
    layer_offsets(woff, boff);
    const long long inner = (long long)(nx - 2 * margin) * (ny - 2 * margin) * (nz - 2 * margin) * nf;
    const int lb = 1024;
    k_mse<<<lb, 256, 0, n->stream>>>(n->y, d_target, nx, ny, nz, nf, margin, 1.f / (float)inner, n->dz16,
                                     n->loss_part);
    // layer 4 (3 -> out): weights and data gradient (masked by a3 > 0)
    if (wgrad<32, 1, 16>(n, n->a[2], n->dz16, nx, ny, nz, nf, 24, n->g + woff[3], n->g + boff[3]) != SS4D_OK)
        return SS4D_ERR_CUDA;
    conv(n, 16, 32, 24, n->dz16, n->wt[3], nullptr, n->a[2], n->dz32[0], nullptr, nx, ny, nz, nf, 0);
    // layer 3
    if (wgrad<32, 24, 32>(n, n->a[1], n->dz32[0], nx, ny, nz, nf, 24, n->g + woff[2], n->g + boff[2]) != SS4D_OK)
        return SS4D_ERR_CUDA;
    conv(n, 32, 32, 24, n->dz32[0], n->wt[2], nullptr, n->a[1], n->dz32[1], nullptr, nx, ny, nz, nf, 0);
    // layer 2
    if (wgrad<32, 24, 32>(n, n->a[0], n->dz32[1], nx, ny, nz, nf, 24, n->g + woff[1], n->g + boff[1]) != SS4D_OK)
        return SS4D_ERR_CUDA;
    conv(n, 32, 32, 24, n->dz32[1], n->wt[1], nullptr, n->a[0], n->dz32[0], nullptr, nx, ny, nz, nf, 0);
    // layer 1
    if (wgrad<16, 24, 32>(n, x0, n->dz32[0], nx, ny, nz, nf, 16, n->g + woff[0], n->g + boff[0]) != SS4D_OK)
        return SS4D_ERR_CUDA;
    if (n->launch_failed)
        return nfail(SS4D_ERR_CUDA, "a tensor-core convolution could not be launched (tensor map or launch)");
    if (d_grad)
        NCK(cudaMemcpyAsync(d_grad, n->g, n->nparam * 4, cudaMemcpyDeviceToDevice, n->stream));
    if (lr > 0.f) {
        n->step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - powf(b1, (float)n->step)), c2 = 1.f / (1.f - powf(b2, (float)n->step));
        k_adam<<<(int)((n->nparam + 255) / 256), 256, 0, n->stream>>>(n->p, n->g, n->m, n->v, (int)n->nparam, lr, b1,
                                                                       b2, 1e-8f, c1, c2);
        if (pack_all(n) != SS4D_OK)
            return SS4D_ERR_CUDA;
    }
    NCK(cudaGetLastError());
    if (loss_out) {
        float hp[1024];
        NCK(cudaMemcpyAsync(hp, n->loss_part, sizeof hp, cudaMemcpyDeviceToHost, n->stream));
        NCK(cudaStreamSynchronize(n->stream));
        double s = 0;
        for (int i = 0; i < lb; ++i)
            s += hp[i];
        *loss_out = (float)(s / (double)inner);
    }
    return SS4D_OK;
}
