// ss4d_conv_tc.cuh — shapes, descriptors and the epilogue of the tcgen05
// convolution (ss4d_conv_tc.cu), shared with the network's host code.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace ss4d {
namespace tc {

// Activations are stored channel-group planar: a tensor of C channels over
// F frames of nx*ny*nz voxels is [F][C/8][nz][ny][nx][8] BF16, element
// (f, c, voxel v of its frame) at ((f * C/8 + c/8) * nx*ny*nz + v) * 8 + c%8:
// the 8 channels of a group are the 16 bytes of one operand row, and a row
// of the halo tile (10 voxels) is 160 contiguous bytes for the TMA.
__host__ __device__ __forceinline__ size_t planar_off(int f, int c, int groups, long long vol, long long v)
{
    return (((size_t)f * groups + (c >> 3)) * (size_t)vol + (size_t)v) * 8 + (c & 7);
}

// output tile: 8 (x) x 16 (y) voxels = one M = 128 accumulator per z plane,
// TZ planes per tile; its input halo tile is HX x HY x HZ voxels
constexpr int TX = 8, TY = 16, TZ = 4;
constexpr int STAGES = 2; // halo tiles in flight
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
    // one (dy, dx, kc) B operand: the three dz taps stacked along N (rows dz*N + co),
    // 2 K groups x 3N rows x 16 B
    static constexpr int WBLK = 3 * N * 32;
    static constexpr int WBYTES = 9 * KC * WBLK;
    static constexpr int HALO = NCG * PLANE;                 // one halo buffer
    static constexpr int ZBYTES = 4096;                      // a zero A operand (128 rows x 16 K) for clearing
    static constexpr int SMEM = 1024 + STAGES * HALO + WBYTES + ZBYTES + 128; // + mbarriers, the TMEM address, a flag
    static constexpr int TCOLS = 2 * TZ * N < 32 ? 32 : 2 * TZ * N; // two accumulator buffers (a power of two here)
    static_assert(TZ * N <= 256 && 3 * N <= 256, "one MMA covers at most 256 columns");
    static_assert((TCOLS & (TCOLS - 1)) == 0, "tensor memory is allocated in powers of two columns");
    static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};

struct TcArgs {
    const __nv_bfloat16 *w;    // B blocks of the layer (pack_tc)
    const float *bias;         // [cout] or null
    const __nv_bfloat16 *mask; // planar, mstride channels: keep channel c where mask > 0 (or null)
    __nv_bfloat16 *y;          // planar, ystride channels: BF16 output, or null
    float *yf;                 // [voxel] channel 0 in FP32, or null
    int nx, ny, nz, nf;
    int cout;                  // real output channels; channels cout .. ystride-1 are written as zero
    int ystride, mstride;
    int relu;
    int *err;                  // set to 1 when a bounded wait ran out
    int withhold_loads;        // test of the timeout path: issue no halo loads, so every wait runs out
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

// one voxel's N accumulated channels -> bias, ReLU, mask -> global; voxel vf
// of frame f, vol voxels per frame
template <int N>
__device__ __forceinline__ void epilogue_store(const TcArgs &a, float (&v)[N], int f, long long vf, long long vol)
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
#pragma unroll
        for (int c = 0; c < N; c += 8) {
            if (c >= a.mstride)
                break;
            const uint4 q = *reinterpret_cast<const uint4 *>(a.mask + planar_off(f, c, a.mstride / 8, vol, vf));
            const __nv_bfloat162 *m2 = reinterpret_cast<const __nv_bfloat162 *>(&q);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (!(__low2float(m2[e]) > 0.f))
                    v[c + 2 * e] = 0.f;
                if (!(__high2float(m2[e]) > 0.f))
                    v[c + 2 * e + 1] = 0.f;
            }
        }
    }
    if (a.y) {
        const int G = a.ystride / 8;
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
            *reinterpret_cast<uint4 *>(a.y + planar_off(f, c, G, vol, vf)) = q;
        }
        for (int c = N; c < a.ystride; c += 8) // channels beyond N: zero
            *reinterpret_cast<uint4 *>(a.y + planar_off(f, c, G, vol, vf)) = make_uint4(0, 0, 0, 0);
    }
    if (a.yf)
        a.yf[(size_t)f * vol + vf] = v[0];
}

// launch one convolution (cin 16 or 32 input channels, N 32 or 16 computed
// output channels) on x (planar, cin channels, nf frames) BF16; persistent
// CTAs, as many as fit on sm_count SMs
cudaError_t conv_tc(int cin, int n, const void *x, const TcArgs &a, int sm_count, cudaStream_t st);
// weights W[27][cout][cin] FP32 -> the B blocks of a (cinp, n) convolution
// (per (dy, dx, K chunk) the three dz taps stacked along N); reverse: the
// data-gradient weights (taps reversed, channel roles swapped)
void pack_tc(const float *w, int cout, int cin, int reverse, int cinp, int n, __nv_bfloat16 *out, cudaStream_t st);
constexpr size_t packed_tc_elems(int cinp, int n) { return (size_t)27 * (cinp / 16) * 2 * n * 8; }
// y[0..n) <- NaN when *err is set (a convolution before it gave up a wait)
void poison_if_err(const int *err, float *y, long long n, cudaStream_t st);

} // namespace tc
} // namespace ss4d
