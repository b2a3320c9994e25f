// ss4d_conv_tc.cuh — shapes, descriptors and the epilogue of the tcgen05
// convolution (ss4d_conv_tc.cu), shared with the network's host code.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace ss4d {
namespace tc {

// output tile: 8 (x) x 16 (y) voxels = one M = 128 accumulator per z plane,
// TZ planes per tile; its input halo tile is HX x HY x HZ voxels
constexpr int TX = 8, TY = 16, TZ = 2;
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
constexpr int HV = HX * HY * HZ;
// one 8-channel group of the halo tile, 16 bytes per voxel, each group on a
// 1024-byte boundary (TMA destinations)
constexpr int PLANE = ((HV * 16 + 1023) / 1024) * 1024;

template <int CIN, int N> struct TcCfg {
    static_assert(CIN % 16 == 0 && N % 16 == 0 && N >= 16 && N <= 256, "M = 128 needs N a multiple of 16");
    static constexpr int NCG = CIN / 8;                      // channel groups (TMA boxes per tile)
    static constexpr int KC = CIN / 16;                      // K chunks of 16 per tap
    static constexpr int BOX_BYTES = HV * 16;                // bytes one box writes
    static constexpr int WBLK = N * 32;                      // one (tap, kc) B operand: 2 K groups x N rows x 16 B
    static constexpr int WBYTES = 27 * KC * WBLK;
    static constexpr int HALO = NCG * PLANE;                 // one halo buffer
    static constexpr int SMEM = 1024 + 2 * HALO + WBYTES + 64;
    static constexpr int TCOLS = 2 * TZ * N < 32 ? 32 : 2 * TZ * N; // two accumulator buffers (a power of two here)
    static_assert((TCOLS & (TCOLS - 1)) == 0, "tensor memory is allocated in powers of two columns");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

struct TcArgs {
    const __nv_bfloat16 *w;    // B blocks of the layer (pack_tc)
    const float *bias;         // [cout] or null
    const __nv_bfloat16 *mask; // [voxel][mstride]: keep channel c where mask > 0 (or null)
    __nv_bfloat16 *y;          // [voxel][ystride] BF16 output, or null
    float *yf;                 // [voxel] channel 0 in FP32, or null
    int nx, ny, nz, nf;
    int cout;                  // real output channels; channels cout .. ystride-1 are written as zero
    int ystride, mstride;
    int relu;
    int *err;                  // set to 1 when a bounded wait ran out
};

inline long long tc_tiles(int nx, int ny, int nz, int nf)
{
    return (long long)((nx + TX - 1) / TX) * ((ny + TY - 1) / TY) * ((nz + TZ - 1) / TZ) * nf;
}

// shared-memory matrix descriptor: no swizzle, K-major; lbo = byte stride of
// the core matrices along K, sbo = along M (or N); version 1 (bits 46-47)
__host__ __device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// one voxel's N accumulated channels -> bias, ReLU, mask -> global
template <int N>
__device__ __forceinline__ void epilogue_store(const TcArgs &a, float (&v)[N], size_t vox)
{
#pragma unroll
    for (int c = 0; c < N; ++c) {
        float x = c < a.cout ? v[c] : 0.f;
        if (a.bias && c < a.cout)
            x += a.bias[c];
        if (a.relu)
            x = fmaxf(x, 0.f);
        v[c] = x;
    }
    if (a.mask) {
        const __nv_bfloat162 *mk = reinterpret_cast<const __nv_bfloat162 *>(a.mask + vox * a.mstride);
#pragma unroll
        for (int c = 0; c < N; c += 2) {
            if (c >= a.mstride)
                break;
            const __nv_bfloat162 m2 = mk[c / 2];
            if (!(__low2float(m2) > 0.f))
                v[c] = 0.f;
            if (!(__high2float(m2) > 0.f))
                v[c + 1] = 0.f;
        }
    }
    if (a.y) {
        uint4 *dst = reinterpret_cast<uint4 *>(a.y + vox * a.ystride);
#pragma unroll
        for (int c = 0; c < N; c += 8) {
            if (c >= a.ystride)
                break;
            __nv_bfloat162 b0 = __floats2bfloat162_rn(v[c], v[c + 1]), b1 = __floats2bfloat162_rn(v[c + 2], v[c + 3]),
                           b2 = __floats2bfloat162_rn(v[c + 4], v[c + 5]), b3 = __floats2bfloat162_rn(v[c + 6], v[c + 7]);
            uint4 q;
            q.x = *reinterpret_cast<uint32_t *>(&b0);
            q.y = *reinterpret_cast<uint32_t *>(&b1);
            q.z = *reinterpret_cast<uint32_t *>(&b2);
            q.w = *reinterpret_cast<uint32_t *>(&b3);
            dst[c / 8] = q;
        }
        for (int c = N; c < a.ystride; c += 8) // channels beyond N: zero
            dst[c / 8] = make_uint4(0, 0, 0, 0);
    }
    if (a.yf)
        a.yf[vox] = v[0];
}

// launch one convolution (cin 16 or 32 input channels, N 32 or 16 computed
// output channels) on x [nf][nz][ny][nx][cin] BF16; sm_count CTAs at most
cudaError_t conv_tc(int cin, int n, const void *x, const TcArgs &a, int sm_count, cudaStream_t st);
// weights W[27][cout][cin] FP32 -> the B blocks of a (cinp, n) convolution;
// reverse: the data-gradient weights (taps reversed, channel roles swapped)
void pack_tc(const float *w, int cout, int cin, int reverse, int cinp, int n, __nv_bfloat16 *out, cudaStream_t st);
constexpr size_t packed_tc_elems(int cinp, int n) { return (size_t)27 * (cinp / 16) * 2 * n * 8; }
// y[0..n) <- NaN when *err is set (a convolution before it gave up a wait)
void poison_if_err(const int *err, float *y, long long n, cudaStream_t st);

} // namespace tc
} // namespace ss4d
