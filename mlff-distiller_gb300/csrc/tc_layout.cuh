// Shared-memory operand layouts and helpers of the tcgen05 kernels
// (edge filters in tc_edge.cu, per-atom update MLP in tc_update.cu).
#pragma once
#include <cuda_fp16.h>
#include "tc_ptx.cuh"

namespace mlff {
namespace tc {

constexpr long long WAIT_BUDGET = 1LL << 32;   // ~2 s at 2 GHz

// ----------------------------------------------------- operand layouts
// A operand (weights): 128 rows x 16 K fp16, K-major, no swizzle:
//   off(m, k) = (k / 8) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2
constexpr uint32_t A_TILE = 4096;
constexpr uint32_t A_LBO = 2048;
constexpr uint32_t A_SBO = 128;
constexpr uint32_t A_PAIR = 2 * A_TILE;       // hi tile then lo tile of one 128 x 16 block

__host__ __device__ constexpr uint32_t a_off(int m, int k) {
    return (uint32_t)((k >> 3) * 2048 + (m >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

// B operand (edge rows x K, fp16) in the K-major 128-byte-swizzle layout:
// K-blocks of 64 columns, each n_rows x 128 bytes; inside a block, 8-row
// groups of 1024 bytes, and row r's 16-byte chunk j (columns 8j..8j+7) sits
// at chunk position j ^ (r % 8).  A warp storing 32 consecutive columns of
// one row touches one 128-byte line, and the MMA reads whole lines.
__host__ __device__ constexpr uint32_t b_block(int n_rows) { return (uint32_t)n_rows * 128; }
__device__ __forceinline__ uint32_t b_off(int n_rows, int row, int k) {
    return (uint32_t)((k >> 6) * b_block(n_rows) + (row >> 3) * 1024 + (row & 7) * 128 +
                      ((((k >> 3) & 7) ^ (row & 7)) << 4) + (k & 7) * 2);
}
// descriptor start offset of K-step s (columns 16s..16s+15)
__host__ __device__ constexpr uint32_t b_kstep_off(int n_rows, int s) {
    return (uint32_t)((s >> 2) * b_block(n_rows) + (s & 3) * 32);
}
__device__ __forceinline__ uint64_t sdesc_b(uint32_t saddr) {
    return sdesc(saddr, 16, 1024) | ((uint64_t)2 << 61);   // layout 2: 128-byte swizzle
}

constexpr uint32_t align1k(uint32_t x) { return (x + 1023u) & ~1023u; }

// sigmoid / SiLU helpers
// sigmoid via the fast exponential and reciprocal; silu = z s,
// silu' = s (1 + z (1 - s)).  Both are exact in the limits z -> +-inf.
__device__ __forceinline__ float fast_sigmoid(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

// x = hi + lo for two values at once (packed conversions)
__device__ __forceinline__ void split2(float a, float b, __half2& hi, __half2& lo) {
    hi = __floats2half2_rn(a, b);
    const float2 f = __half22float2(hi);
    lo = __floats2half2_rn(a - f.x, b - f.y);
}

// hi and lo fp16 halves of the pair (a, b), each packed in one 32-bit word
// (a in the low half)
__device__ __forceinline__ void split_pack(float a, float b, uint32_t& hi, uint32_t& lo) {
    __half2 h, l;
    split2(a, b, h, l);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Shared-memory address of the 16-byte chunk of a K-major 128-byte-swizzle
// B tile of n_rows rows that holds row `row`, K values k0 .. k0 + 7 (k0 a
// multiple of 8): the destination of one stmatrix row.
__device__ __forceinline__ uint32_t b_chunk(uint32_t tile, int n_rows, int row, int k0) {
    return tile + (uint32_t)((k0 >> 6) * b_block(n_rows) + (row >> 3) * 1024 + (row & 7) * 128 +
                             ((((k0 >> 3) & 7) ^ (row & 7)) << 4));
}

// store 16 consecutive K values (one K-step, both 8-column chunks) of one
// row as split fp16 into a B-operand tile (hi half, lo half)
__device__ __forceinline__ void store_row16(unsigned char* tile, uint32_t half_bytes, int n_rows, int row, int s,
                                            const float (&v)[16]) {
    __align__(16) __half2 hi[8];
    __align__(16) __half2 lo[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) split2(v[2 * i], v[2 * i + 1], hi[i], lo[i]);
    const uint32_t o0 = b_off(n_rows, row, 16 * s);
    const uint32_t o1 = b_off(n_rows, row, 16 * s + 8);
    *reinterpret_cast<uint4*>(tile + o0) = *reinterpret_cast<const uint4*>(&hi[0]);
    *reinterpret_cast<uint4*>(tile + o1) = *reinterpret_cast<const uint4*>(&hi[4]);
    *reinterpret_cast<uint4*>(tile + half_bytes + o0) = *reinterpret_cast<const uint4*>(&lo[0]);
    *reinterpret_cast<uint4*>(tile + half_bytes + o1) = *reinterpret_cast<const uint4*>(&lo[4]);
}

// Rows row and row+1, column k of a B-operand tile: store the split fp16
// values of a pair of edges.
__device__ __forceinline__ void store_col_pair(unsigned char* tile, uint32_t half_bytes, int n_rows, int row, int k,
                                               float a, float b) {
    __half2 hi, lo;
    split2(a, b, hi, lo);
    const uint32_t o0 = b_off(n_rows, row, k), o1 = b_off(n_rows, row + 1, k);
    *reinterpret_cast<__half*>(tile + o0) = __low2half(hi);
    *reinterpret_cast<__half*>(tile + o1) = __high2half(hi);
    *reinterpret_cast<__half*>(tile + half_bytes + o0) = __low2half(lo);
    *reinterpret_cast<__half*>(tile + half_bytes + o1) = __high2half(lo);
}

// Column k of a B tile written by the thread that owns it, rows row0 + i
// with row0 a multiple of 8 (then row0 + i sits i * 128 bytes further and
// its swizzle key is i % 8): the k-dependent part of b_off is computed once,
// each pair store costs an add and an xor when i is a compile-time constant.
struct BColumn {
    unsigned char* base;   // tile + K-block of k + row0 * 128 + (k % 8) * 2
    uint32_t half_bytes;
    uint32_t kj;           // 16-byte chunk of k within its 128-byte row
    __device__ __forceinline__ BColumn(unsigned char* tile, uint32_t half, int n_rows, int row0, int k)
        : base(tile + (k >> 6) * b_block(n_rows) + row0 * 128 + (k & 7) * 2), half_bytes(half), kj((k >> 3) & 7) {}
    // rows row0 + i and row0 + i + 1: the split fp16 values of a and b
    __device__ __forceinline__ void put_pair(int i, float a, float b) const {
        __half2 hi, lo;
        split2(a, b, hi, lo);
        const uint32_t o0 = (uint32_t)i * 128 + ((kj ^ (uint32_t)(i & 7)) << 4);
        const uint32_t o1 = (uint32_t)(i + 1) * 128 + ((kj ^ (uint32_t)((i + 1) & 7)) << 4);
        *reinterpret_cast<__half*>(base + o0) = __low2half(hi);
        *reinterpret_cast<__half*>(base + o1) = __high2half(hi);
        *reinterpret_cast<__half*>(base + half_bytes + o0) = __low2half(lo);
        *reinterpret_cast<__half*>(base + half_bytes + o1) = __high2half(lo);
    }
    // row row0 + i alone (any i): the split fp16 value of a
    __device__ __forceinline__ void put_one(int i, float a) const {
        const __half hi = __float2half_rn(a);
        const __half lo = __float2half_rn(a - __half2float(hi));
        const uint32_t o = (uint32_t)i * 128 + ((kj ^ (uint32_t)(i & 7)) << 4);
        *reinterpret_cast<__half*>(base + o) = hi;
        *reinterpret_cast<__half*>(base + half_bytes + o) = lo;
    }
};

}  // namespace tc
}  // namespace mlff
