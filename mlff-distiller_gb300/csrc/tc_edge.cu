// Tensor-core (tcgen05) fused edge kernels.
//
// Same algorithm as the CUDA-core kernels in tuned.cu (receiver-sorted
// tiles, persistent CTAs over receiver ranges, register-carried receiver
// sums, forward-mode df/dd in the reverse pass), with the filter MLP
// (Linear(R,128) - SiLU - Linear(128,384), student_model.py:318-322,350) on
// the 5th-generation tensor cores:
//
//   * transposed GEMMs: D[channel][edge] = W[channel][k] * X[edge][k]^T, so
//     a TMEM lane is a hidden unit / output channel and a TMEM column is an
//     edge; the epilogue thread that owns lane c reads channel c of 32
//     consecutive edges and runs the receiver-segmented sum directly, with
//     coalesced gathers of the senders' feature rows;
//   * split-FP16 operands: x = hi + lo (both fp16), three MMAs per K-step
//     (hi*hi + hi*lo + lo*hi) with FP32 accumulation in TMEM;
//   * operands resident for the whole launch: W1 (128 x 32), the hi half
//     of W2 (384 x 128) and the lo half of W2's third chunk in shared
//     memory, the lo halves of chunks 0 and 1 in TMEM (A operands of
//     tcgen05.mma with A in tensor memory);
//   * the [E; E'] tiles (RBF x cutoff and its d-derivative, split fp16) are
//     computed once per call for all layers and bulk-copied per edge tile
//     (the forward kernel copies the E rows only); per-tile edge arrays are
//     fetched with cp.async while the previous tile's epilogue runs;
//   * GEMM2's three 128-channel chunks are issued by three threads: a thread
//     stalls on tcgen05.mma issue while the tensor core is busy (about one
//     MMA per 50 cycles from one thread), three keep it saturated;
//   * every wait is bounded (clock64 budget); on expiry the kernel records
//     MLFF_ERR_TIMEOUT, drains its own copies, frees TMEM and returns.
//
// TMEM (512 columns): [0,128) lo halves of W2 chunks 0 and 1; [128,512) two
// pipelines of 192 columns each, three 64-column accumulator chunks per
// pipeline (forward: 64-edge tiles, one chunk per W2 chunk; reverse: 32-edge
// tiles with [f | f'] per chunk, f' = df/dd in forward mode, chunks 0-1 for
// GEMM2 and the third for GEMM3).  GEMM1's output aliases one chunk until
// epilogue 1 has read it: chunk 0 in the forward kernel, the third chunk
// ([z | z']) in the reverse kernel.
#include <cuda_fp16.h>
#include <mutex>
#include "common.cuh"
#include <type_traits>
#include "workspace.h"
#include "edge_common.cuh"
#include "profile.h"
#include "tc_ptx.cuh"
#include "tc_layout.cuh"

namespace mlff {
using namespace tc;

// ----------------------------------------------------- operand layouts
constexpr uint32_t SLAB = 2 * A_TILE;         // hi + lo of one 128 x 16 block (W1)
constexpr int W2_TILES = 24;                  // 3 channel chunks x 8 K-steps, q = g * 8 + s
constexpr uint32_t W1_BYTES = 2 * SLAB;       // 2 K-steps
constexpr uint32_t W2_HALF = W2_TILES * A_TILE;   // all hi tiles (96 KB), then all lo tiles
constexpr uint32_t W2L_BYTES = 8 * A_TILE;    // lo tiles of W2 chunk 2 (resident in shared memory)

// TMEM columns (512 allocated): [0,128) the lo halves of W2 chunks 0 and 1
// as MMA A operands (chunk g, K-step s at 64 g + 8 s); [128,512) two
// pipelines' GEMM accumulators, 192 columns each (see the kernels).
constexpr uint32_t TM_W2LO = 0;

// ------------------------------------------------------------- packing
// W1 [H][RMAX] -> 2 K-step blocks (hi, lo); W2 [3H][H] -> 24 hi tiles
// followed by the 24 matching lo tiles; W2's third chunk transposed
// (rows = hidden units, K = channels) -> 8 K-step pairs (hi tile, lo tile)
// for the per-atom Q rows of the reverse pass.
__global__ void pack_tc_kernel(const float* __restrict__ w1, const float* __restrict__ w2,
                               unsigned char* __restrict__ w1_out, unsigned char* __restrict__ w2_out,
                               uint32_t* __restrict__ w2_tm, unsigned char* __restrict__ w2q_out) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 8 * 128 * 16; i += stride) {
        const int s = i / 2048, m = (i / 16) % 128, kk = i % 16;
        __half hi, lo;
        split_f16(w2[(2 * H + 16 * s + kk) * H + m], hi, lo);
        *reinterpret_cast<__half*>(w2q_out + s * A_PAIR + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(w2q_out + s * A_PAIR + A_TILE + a_off(m, kk)) = lo;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * 128 * 16; i += stride) {
        const int s = i / 2048, m = (i / 16) % 128, kk = i % 16;
        __half hi, lo;
        split_f16(w1[m * RMAX + 16 * s + kk], hi, lo);
        *reinterpret_cast<__half*>(w1_out + s * SLAB + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(w1_out + s * SLAB + A_TILE + a_off(m, kk)) = lo;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < W2_TILES * 128 * 16; i += stride) {
        const int q = i / 2048, m = (i / 16) % 128, kk = i % 16;
        const int g = q / 8, s = q % 8;
        __half hi, lo;
        split_f16(w2[(g * 128 + m) * H + 16 * s + kk], hi, lo);
        *reinterpret_cast<__half*>(w2_out + q * A_TILE + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(w2_out + W2_HALF + q * A_TILE + a_off(m, kk)) = lo;
    }
    // TMEM image of the lo halves of chunks 0 and 1: word (r, v, m) is TMEM
    // lane m, column 32 r + v, holding k = 2 (v % 8), 2 (v % 8) + 1 of
    // K-step 4 r + v / 8 (low half first)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * 32 * 128; i += stride) {
        const int m = i % 128, v = (i / 128) % 32, r = i / (32 * 128);
        const int ks = 4 * r + v / 8, g = ks >> 3, s = ks & 7, j = v % 8;
        const float* row = w2 + (size_t)(g * 128 + m) * H + 16 * s;
        __half hi0, lo0, hi1, lo1;
        split_f16(row[2 * j], hi0, lo0);
        split_f16(row[2 * j + 1], hi1, lo1);
        __half2 pr = __halves2half2(lo0, lo1);
        w2_tm[i] = *reinterpret_cast<uint32_t*>(&pr);
    }
}

int pack_update_tc(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st);

int pack_bf16(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st) {
    for (int l = 0; l < d.n_layers; ++l) {
        const LayerOffsets& L = o.layer[l];
        pack_tc_kernel<<<64, 256, 0, st>>>(out + L.w1, out + L.w2, reinterpret_cast<unsigned char*>(out + L.w1_bf),
                                           reinterpret_cast<unsigned char*>(out + L.w2_bf),
                                           reinterpret_cast<uint32_t*>(out + L.w2_tm),
                                           reinterpret_cast<unsigned char*>(out + L.w2q_tc));
        MLFF_LAUNCH_CHECK("pack_tc");
    }
    return pack_update_tc(d, out, o, st);
}

// -------------------------------------------------------- shared pieces
constexpr int NT = 512;                        // threads per CTA (16 warps)
// Test hook (EdgeArgs::stall_test): the first main-loop wait of a partition
// also waits on an mbarrier that nothing arrives at, for STALL_BUDGET
// cycles, and so takes the timeout path of a real stalled wait.
constexpr long long STALL_BUDGET = 1LL << 16;
constexpr int WHERE_STALL_TEST = 99;

__device__ __forceinline__ void signal_timeout(const EdgeArgs& a, volatile int* abort_flag, int where) {
    set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, where);
    *abort_flag = 1;
}

// Lo halves of W2 chunks 0 and 1 into TMEM columns [0,128), as A operands,
// from their packed TMEM image: warp (q, r) writes rows 32q..32q+31 (its
// TMEM lane quarter), columns 32r..32r+31 (K-steps 4r..4r+3 of the 16).
__device__ __forceinline__ void load_w2_lo_tmem(uint32_t lane_base, const uint32_t* w2tm, int r, int m) {
    uint32_t v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __ldg(w2tm + (r * 32 + i) * 128 + m);
    tmem_st32u(lane_base + TM_W2LO + 32 * r, v);
}

// Resident W2 operands on one mbarrier: all 24 hi tiles (six 16 KB bulk
// copies), then the 8 lo tiles of chunk 2 (the lo tiles of chunks 0 and 1 are
// TMEM operands).
__device__ __forceinline__ void load_w2_resident(unsigned char* hi, unsigned char* lo2, const unsigned char* w2g,
                                                 uint64_t* bar) {
    mbar_expect_tx(bar, W2_HALF + W2L_BYTES);
#pragma unroll
    for (int i = 0; i < 6; ++i) bulk_g2s(hi + i * (W2_HALF / 6), w2g + i * (W2_HALF / 6), W2_HALF / 6, bar);
    bulk_g2s(lo2, w2g + W2_HALF + 16 * A_TILE, W2L_BYTES, bar);
}

// rbf(d)_r * fc(d) for r in [r0, r0 + 16) (0 beyond R or for padding edges)
__device__ __forceinline__ void rbf16(float d, bool valid, int r0, int R, const float* cent, const float* gam,
                                      float rc, float (&out)[16]) {
    const float fc = cutoff_fn(d, rc);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = r0 + i;
        const float diff = d - cent[r];
        out[i] = (valid && r < R) ? __expf(-gam[r] * diff * diff) * fc : 0.0f;
    }
}
__device__ __forceinline__ void rbf16_d(float d, bool valid, int r0, int R, const float* cent, const float* gam,
                                        float rc, float (&out)[16]) {
    float fc, dfc;
    cutoff_fn_d(d, rc, fc, dfc);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = r0 + i;
        const float diff = d - cent[r];
        const float g = __expf(-gam[r] * diff * diff);
        out[i] = (valid && r < R) ? g * (dfc - 2.0f * gam[r] * diff * fc) : 0.0f;
    }
}

// ------------------------------------------------------ E tiles (per call)
// [E; E'] tiles: for every 32 consecutive edges of a receiver partition, the
// RBF x cutoff rows (rows 0-31) and their d-derivatives (rows 32-63) as
// split fp16 in a K-major no-swizzle layout (16-byte core matrices of 8 rows
// x 8 columns: the 8-column chunks of an 8-row group 128 bytes apart, the
// groups 512 bytes apart; the hi image, then the lo image), computed once
// per call for all layers.  Each image holds the E rows in its first 2 KB
// and the E' rows in its second.  Tile k of partition p is the reverse
// kernel's k-th tile of p; the forward kernel's 64-edge tile k copies only
// the E rows of tiles 2k and 2k + 1.
constexpr uint32_t ET_ROWS = 64;
constexpr uint32_t ET_BYTES = ET_ROWS * 128, ET_HALF = ET_ROWS * 64;   // 8 KB, hi then lo
constexpr uint32_t ET_LBO = 128, ET_SBO = 512;     // chunk and row-group strides
constexpr uint32_t ET_E = 32 * 64;                 // the E rows of one image: 2 KB
__device__ __forceinline__ uint32_t et_off(int row, int k) {
    return (uint32_t)((row >> 3) * ET_SBO + (k >> 3) * ET_LBO + (row & 7) * 16 + (k & 7) * 2);
}

// Tile counts of all partitions (32 edges per tile), then their exclusive
// scan (one block, 1024 partitions at a time): bases at base[0..P].
__global__ void __launch_bounds__(1024) etile_index_kernel(const int32_t* __restrict__ row_ptr,
                                                           const int32_t* __restrict__ part, int P,
                                                           int32_t* __restrict__ base) {
    pdl_wait();
    pdl_trigger();
    __shared__ int cb[1024];
    __shared__ int carry;
    const int t = threadIdx.x;
    if (t == 0) carry = 0;
    __syncthreads();
    for (int p0 = 0; p0 < P; p0 += 1024) {
        const int p = p0 + t;
        int nb = 0;
        if (p < P) {
            const int E = row_ptr[part[p + 1]] - row_ptr[part[p]];
            nb = (E + 31) / 32;
        }
        cb[t] = nb;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {   // inclusive scan (Hillis-Steele)
            const int xb = t >= o ? cb[t - o] : 0;
            __syncthreads();
            cb[t] += xb;
            __syncthreads();
        }
        if (p < P) base[p] = carry + cb[t] - nb;
        __syncthreads();
        if (t == 1023) carry += cb[1023];
        __syncthreads();
    }
    if (t == 0) base[P] = carry;
}

__global__ void __launch_bounds__(256) etile_fill_kernel(EdgeArgs a, const int32_t* __restrict__ base,
                                                         unsigned char* __restrict__ out) {
    pdl_wait();
    pdl_trigger();
    __shared__ float cent[RMAX], gam[RMAX];
    if (threadIdx.x < RMAX) {
        cent[threadIdx.x] = a.centers[threadIdx.x];
        gam[threadIdx.x] = a.gamma[threadIdx.x];
    }
    __syncthreads();
    if (a.st->code != 0) return;
    constexpr int TE = 32;                              // edges per tile
    constexpr int ROWS = ET_ROWS;
    constexpr int PER = 2 * ROWS;                       // threads per tile: (row, K-step)
    constexpr int TPI = 256 / PER;                      // tiles per block iteration
    const int t = threadIdx.x, sub = t / PER, loc = t % PER;
    const int row = loc % ROWS, s = loc / ROWS;
    const int which = row >> 5, erow = row & 31;
    for (int p = blockIdx.x; p < a.nparts; p += gridDim.x) {
        const int e0 = a.row_ptr[a.part[p]], e1 = a.row_ptr[a.part[p + 1]];
        const int b0 = base[p];
        for (int k = blockIdx.y * TPI + sub; e0 + k * TE < e1; k += gridDim.y * TPI) {
            const int e = e0 + k * TE + erow;
            const bool valid = e < e1;
            const float d = valid ? a.geo[e].w : 0.f;
            float v[16];
            if (which == 0) rbf16(d, valid, 16 * s, a.R, cent, gam, a.cutoff, v);
            else rbf16_d(d, valid, 16 * s, a.R, cent, gam, a.cutoff, v);
            __align__(16) __half2 hi[8];
            __align__(16) __half2 lo[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) split2(v[2 * i], v[2 * i + 1], hi[i], lo[i]);
            unsigned char* tile = out + (size_t)(b0 + k) * ET_BYTES;
            *reinterpret_cast<uint4*>(tile + et_off(row, 16 * s)) = *reinterpret_cast<const uint4*>(&hi[0]);
            *reinterpret_cast<uint4*>(tile + et_off(row, 16 * s + 8)) = *reinterpret_cast<const uint4*>(&hi[4]);
            *reinterpret_cast<uint4*>(tile + ET_HALF + et_off(row, 16 * s)) = *reinterpret_cast<const uint4*>(&lo[0]);
            *reinterpret_cast<uint4*>(tile + ET_HALF + et_off(row, 16 * s + 8)) =
                *reinterpret_cast<const uint4*>(&lo[4]);
        }
    }
}

int launch_etiles(const EdgeArgs& a, int32_t* base, unsigned char* tiles, cudaStream_t st) {
    MLFF_LAUNCH_PDL("etile_index", etile_index_kernel, 1, 1024, 0, st, a.row_ptr, a.part, a.nparts, base);
    // tiles of a partition spread over gridDim.y blocks
    MLFF_LAUNCH_PDL("etile_fill", etile_fill_kernel, dim3(a.nparts, 16), 256, 0, st, a, base, tiles);
    return MLFF_OK;
}

// Per-edge arrays of a tile, fetched asynchronously for the next tile while
// the current one runs: (u, d), sender, receiver (padding: 0, 0, -1) and,
// when ea is given, the edges' accumulated (dE/dd, dE/du) of the layers
// processed so far.
__device__ __forceinline__ void fetch_tile_edges(const EdgeArgs& a, int t, int tn, int t0, int n, float4* us,
                                                 int* src_s, int* rcv_s, float4* ea = nullptr) {
    if (t < tn) {
        if (t < n) {
            cp_async16(us + t, a.geo + t0 + t);
            cp_async4(src_s + t, a.col + t0 + t);
            cp_async4(rcv_s + t, a.erecv + t0 + t);
            if (ea) cp_async16(ea + t, a.eacc + t0 + t);
        } else {
            us[t] = make_float4(0.f, 0.f, 0.f, 0.f);
            src_s[t] = 0;
            rcv_s[t] = -1;
        }
    }
    cp_async_commit();
}

// Per-tile prep by the threads that fetched the tile's edge arrays: sender
// (and receiver) row offsets, u components, and a bitmask of the edges whose
// receiver differs from the previous edge's (edge 0 compares with prev).
template <int N>
__device__ __forceinline__ void tile_prep(int e, int n, int prev, const int* src_s, const int* rcv_s,
                                          const float4* us, int* soff, int* roff, float* uc, uint32_t* chg) {
    const bool valid = e < n;
    const int ra = rcv_s[e];
    soff[e] = src_s[e] * 2 * H;   // row offsets in float2 units of the pair layout
    if (roff) roff[e] = max(ra, 0) * 2 * H;
    if (uc) {
        const float4 u = us[e];
        uc[e] = u.x;
        uc[N + e] = u.y;
        uc[2 * N + e] = u.z;
    }
    const int before = e == 0 ? prev : rcv_s[e - 1];
    const unsigned m = __ballot_sync(0xffffffffu, valid && ra != before);
    if ((e & 31) == 0) chg[e >> 5] = m;
}

// Sum 8 per-lane values over the 32 lanes of a warp with 9 shuffles
// (reduce-scatter).  Afterwards lanes with (lane & 3) == 0 hold the sum of
// value index = bits 4..2 of the lane id.
__device__ __forceinline__ float warp_reduce_scatter8(const float (&v)[8], int lane) {
    float w4[4], w2[2];
    const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float send = b16 ? v[j] : v[j + 4];
        const float keep = b16 ? v[j + 4] : v[j];
        w4[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float send = b8 ? w4[j] : w4[j + 2];
        const float keep = b8 ? w4[j + 2] : w4[j];
        w2[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const float send = b4 ? w2[0] : w2[1];
    const float keep = b4 ? w2[1] : w2[0];
    float w1 = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    w1 += __shfl_xor_sync(0xffffffffu, w1, 2);
    w1 += __shfl_xor_sync(0xffffffffu, w1, 1);
    return w1;
}
__device__ __forceinline__ int reduce_scatter8_index(int lane) {
    return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// Chunk g of GEMM2 for one B tile of NR rows: D (TMEM columns dcol) +=
// W2[g] B^T with B the split-fp16 tile at Hs (hi half, then lo half
// 2 * b_block(NR) bytes later).  Per K-step: the resident hi tile times both
// halves of B, then the lo tile (TMEM for chunks 0 and 1, shared memory for
// chunk 2) times the hi half.  Every MMA accumulates (the epilogue filled
// TMEM with the bias).  The three chunks are issued by three threads in
// parallel: a thread issues about one MMA per 50 cycles and stalls while the
// tensor core is busy, so one issuer adds its own latency to every MMA; each
// chunk keeps a fixed accumulation order.
template <int NR>
__device__ __forceinline__ void issue_gemm2_chunk(int g, uint32_t tmem, uint32_t dcol, const unsigned char* w2h,
                                                  const unsigned char* w2l, const unsigned char* Hs) {
    constexpr uint32_t idesc = idesc_f16(NR);
    constexpr uint64_t DA = A_TILE >> 4, DH = (2 * b_block(NR)) >> 4;
    const uint64_t a_hi = sdesc(smem_u32(w2h), A_LBO, A_SBO) + (uint64_t)(8 * g) * DA;
    const uint64_t a_lo = sdesc(smem_u32(w2l), A_LBO, A_SBO);
    const uint64_t b0 = sdesc_b(smem_u32(Hs));
    const uint32_t d = tmem + dcol;
#pragma unroll 1
    for (int s = 0; s < 8; ++s) {
        const uint64_t bh = b0 + (uint64_t)(b_kstep_off(NR, s) >> 4);
        const uint64_t ah = a_hi + (uint64_t)s * DA;
        mma_f16(d, ah, bh, idesc, 1);
        mma_f16(d, ah, bh + DH, idesc, 1);
        if (g < 2) mma_f16_ts(d, tmem + TM_W2LO + 64 * g + 8 * s, bh, idesc, 1);
        else mma_f16(d, a_lo + (uint64_t)s * DA, bh, idesc, 1);
    }
}

// out = base + (sum over the receiver's edges): receivers in [j0, j1)
// without edges get the base row (the epilogues store base + sum once per
// receiver that has edges); out in the component-major layout, base in the
// pair layout.
__device__ __forceinline__ void copy_empty_rows(float* out, const float* base, const int32_t* row_ptr, int j0, int j1,
                                                int w, int lane, int nwarps = NT / 32) {
    for (int j = j0 + w; j < j1; j += nwarps)
        if (row_ptr[j] == row_ptr[j + 1])
            for (int k = lane; k < 4 * H; k += 32) {
                const int comp = k / H, ch = k % H;
                out[(int64_t)j * 4 * H + k] = base[(int64_t)j * 4 * H + pair_off(comp, ch)];
            }
}

// ------------------------------------------------ pipelines (both kernels)
// Each kernel runs two independent pipelines per CTA, warps 0-7 and 8-15,
// each on its own receiver partition (CTA b: partitions 2b and 2b + 1, then
// 2b + 2G ...), so that one pipeline's MMAs, copies and barrier waits overlap
// the other pipeline's CUDA-core epilogues.  A pipeline owns 192 TMEM
// columns (three filter chunks of 64), an H tile, its barriers and a named
// CTA barrier.
constexpr int PT = 256;                              // threads per pipeline
__device__ __forceinline__ void pipe_sync(int pp) {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + pp), "r"(PT) : "memory");
}
// Pipeline barrier that also ORs v over the pipeline's threads: every thread
// gets the same answer.
__device__ __forceinline__ bool pipe_sync_or(int pp, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + pp), "r"(PT)
        : "memory");
    return r != 0;
}
// the first n threads (whole warps) of pipeline pp
__device__ __forceinline__ void pipe_sync_first(int pp, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(3 + pp), "r"(n) : "memory");
}
// The warps that read the TMEM columns the next tile's GEMM1 writes (n
// threads, warp 0 of the pipeline among them) signal that their reads are
// done (arrive, no wait); warp 0 waits for them, then issues that GEMM1 while
// the rest of the pipeline is still in epilogue 2.
__device__ __forceinline__ void cols_free_arrive(int pp, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(5 + pp), "r"(n) : "memory");
}
__device__ __forceinline__ void cols_free_sync(int pp, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(5 + pp), "r"(n) : "memory");
}

// ------------------------------------------------------- forward kernel
// 64-edge tiles per pipeline: GEMM1 (z = W1 e, two N = 32 halves, one per
// [E; E'] tile) into the columns of the pipeline's chunk 0, epilogue 1
// (h = silu(z + b1) into the H tile, bias refills), GEMM2 (three 128 x 64
// chunks), epilogue 2: warp (q, h) of the
// pipeline reads TMEM lane quarter q (channels 32q..32q+31) and sums two
// feature components of every edge per receiver in registers (h = 0 the
// scalar and v_x, h = 1 v_y and v_z), Xt = X + messages written once per
// receiver.  Padding edges of a partition's last tile get h = 0 and a zero
// bias fill (a fix-up after epilogue 1): their filter is exactly zero and
// every gather runs unpredicated.
constexpr int QN = 64;                               // edges per forward tile
constexpr uint32_t Q_HH = 2 * b_block(QN);           // one half (hi or lo) of the H tile: 16 KB
constexpr uint32_t Q_SB_US = 0;
constexpr uint32_t Q_SB_SRC = Q_SB_US + QN * 16;
constexpr uint32_t Q_SB_RCV = Q_SB_SRC + QN * 4;
constexpr uint32_t Q_SB_SOFF = Q_SB_RCV + QN * 4;
constexpr uint32_t Q_SB_UC = Q_SB_SOFF + QN * 4;
constexpr uint32_t Q_SB_CHG = Q_SB_UC + 3 * QN * 4;
constexpr uint32_t Q_SB_BYTES = Q_SB_CHG + 16;
constexpr uint32_t Q_OFF_W1 = 0;
constexpr uint32_t Q_OFF_W2H = Q_OFF_W1 + W1_BYTES;
constexpr uint32_t Q_OFF_H = align1k(Q_OFF_W2H + W2_HALF);   // pipeline p's H tile at + 2 Q_HH p
constexpr uint32_t Q_OFF_W2L = align1k(Q_OFF_H + 4 * Q_HH);
constexpr uint32_t Q_OFF_SB = Q_OFF_W2L + W2L_BYTES;        // [pipeline][buffer] edge arrays
constexpr uint32_t Q_OFF_B1 = Q_OFF_SB + 4 * Q_SB_BYTES;
constexpr uint32_t Q_OFF_B2 = Q_OFF_B1 + H * 4;
constexpr uint32_t Q_OFF_BAR = Q_OFF_B2 + H3 * 4;
constexpr uint32_t Q_OFF_MISC = Q_OFF_BAR + 8 * 8;
constexpr uint32_t Q_SMEM = align1k(Q_OFF_MISC + 16);
static_assert(4 * ET_E <= 2 * Q_HH, "the E rows of two [E; E'] tiles fit in the H tile's space");
static_assert(Q_SB_BYTES % 16 == 0, "edge array alignment");
static_assert(Q_SMEM <= 232448, "forward kernel shared memory");

__global__ void __launch_bounds__(NT, 1) edge_fwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                            const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + Q_OFF_W1;
    unsigned char* w2h = smem + Q_OFF_W2H;
    unsigned char* w2l = smem + Q_OFF_W2L;        // resident lo tiles of W2 chunk 2
    float* b1s = reinterpret_cast<float*>(smem + Q_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + Q_OFF_B2);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + Q_OFF_BAR);
    uint64_t* w2h_bar = bars;                       // resident W2 operands
    uint64_t* never_bar = bars + 1;                 // test hook: nothing arrives here
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + Q_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + Q_OFF_MISC + 4);

    // waits for the previous kernel at entry: reading the status word first
    // and returning early keeps the main loop's register allocation lean
    pdl_wait();
    if (a.st->code != 0) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w == 0) {
        tmem_alloc(tslot, 512);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(w2h_bar, 1);
        mbar_init(never_bar, 1);
        for (int p = 0; p < 2; ++p) {
            mbar_init(bars + 2 + 3 * p, 1);   // GEMM1
            mbar_init(bars + 3 + 3 * p, 1);   // E tile
            mbar_init(bars + 4 + 3 * p, 3);   // GEMM2: one commit per chunk issuer
        }
        fence_mbar_init();
        *abort_flag = 0;
    }
    for (int i = t; i < (int)(W1_BYTES / 16); i += NT)
        reinterpret_cast<uint4*>(w1s)[i] = reinterpret_cast<const uint4*>(w1g)[i];
    if (t < H) b1s[t] = a.P[a.lo.b1 + t];
    for (int i = t; i < H3; i += NT) b2s[i] = a.P[a.lo.b2 + i];
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    if (t == 32) load_w2_resident(w2h, w2l, w2g, w2h_bar);
    const int q = w & 3;
    const int c = 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    load_w2_lo_tmem(lane_base, reinterpret_cast<const uint32_t*>(a.P + a.lo.w2_tm), w >> 2, c);
    tmem_st_wait();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    pdl_trigger();   // after the TMEM allocation

    // ---- this thread's pipeline
    const int pp = w >> 3, wl = w & 7, tp = t & (PT - 1), hh = wl >> 2;
    const uint32_t TB = 128 + 192 * pp;             // the pipeline's TMEM columns: chunk g at TB + 64 g
    unsigned char* Hs = smem + Q_OFF_H + pp * 2 * Q_HH;   // H hi, then lo
    unsigned char* Es = Hs;                         // [E; E'] tiles (bulk-copied) before H is written
    uint64_t* mma_bar = bars + 2 + 3 * pp;
    uint64_t* e_bar = bars + 3 + 3 * pp;
    uint64_t* g2_bar = bars + 4 + 3 * pp;
    unsigned char* sbase = smem + Q_OFF_SB + 2 * pp * Q_SB_BYTES;
    // components 2 hh and 2 hh + 1: one float2 of the pair layout of X,
    // H floats apart in the component-major Xt
    const float2* xx = reinterpret_cast<const float2*>(a.X + pair_off(2 * hh, c));
    float* out = a.Xt + 2 * hh * H + c;

    uint32_t mma_phase = 0, g2_phase = 0;   // GEMM1 / GEMM2 barrier phases
    uint32_t e_phase = 0, e_issued = 0;     // E-tile copies: barrier phase, copies issued (thread tp 64)
    bool w2h_ready = false;                 // (GEMM2 issuers)
    bool aborted = false;
    auto prep = [&](unsigned char* sbx, int nn, int prev) {
        tile_prep<QN>(tp, nn, prev, reinterpret_cast<int*>(sbx + Q_SB_SRC), reinterpret_cast<int*>(sbx + Q_SB_RCV),
                      reinterpret_cast<float4*>(sbx + Q_SB_US), reinterpret_cast<int*>(sbx + Q_SB_SOFF), nullptr,
                      reinterpret_cast<float*>(sbx + Q_SB_UC), reinterpret_cast<uint32_t*>(sbx + Q_SB_CHG));
    };
    auto fetch = [&](unsigned char* sbx, int t0, int nn) {
        fetch_tile_edges(a, tp, QN, t0, nn, reinterpret_cast<float4*>(sbx + Q_SB_US),
                         reinterpret_cast<int*>(sbx + Q_SB_SRC), reinterpret_cast<int*>(sbx + Q_SB_RCV));
    };
    // z^T = W1 e^T into chunk 0's columns, once the copies have landed
    // (thread tp 0): the tile's 64 edges are the E rows (0-31) of nt
    // consecutive [E; E'] tiles, copied to Es (edges 32 j .. 32 j + 31 from
    // tile j: its hi E rows at 4 KB j, its lo E rows 2 KB further)
    auto issue_gemm1 = [&](int nt) {
        if (!mbar_wait(e_bar, e_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 8);
        fence_after_sync();
        constexpr uint32_t idesc = idesc_f16(32);
        for (int j = 0; j < nt; ++j)
#pragma unroll
            for (int s = 0; s < 2; ++s)
#pragma unroll
                for (int pr = 0; pr < 3; ++pr) {
                    const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                    const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                    const uint64_t bd =
                        sdesc(smem_u32(Es + j * 2 * ET_E + bhl * ET_E + s * 2 * ET_LBO), ET_LBO, ET_SBO);
                    mma_f16(tmem + TB + 32 * j, ad, bd, idesc, (s | pr) != 0);
                }
        mma_commit(mma_bar);
    };
    // copies of the E rows of the [E; E'] tiles of forward tile k (thread tp QN)
    auto copy_etiles = [&](const unsigned char* etiles, int nrev, int k) {
        const int nt = min(2, nrev - 2 * k);
        mbar_expect_tx(e_bar, nt * 2 * ET_E);
        for (int j = 0; j < nt; ++j) {
            const unsigned char* src = etiles + (size_t)(2 * k + j) * ET_BYTES;
            bulk_g2s(Es + j * 2 * ET_E, src, ET_E, e_bar);                     // hi image
            bulk_g2s(Es + j * 2 * ET_E + ET_E, src + ET_HALF, ET_E, e_bar);    // lo image
        }
        ++e_issued;
    };
    for (int p = 2 * blockIdx.x + pp; p < a.nparts && !aborted; p += 2 * gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        const int ntl = (e1 - e0 + QN - 1) / QN;
        const int nrev = (e1 - e0 + 31) / 32;   // [E; E'] tiles of the partition
        const unsigned char* etiles = a.etile + (size_t)a.etile_base[p] * ET_BYTES;
        copy_empty_rows(a.Xt, a.X, a.row_ptr, j0, j1, wl, lane, PT / 32);
        int cur = j0;
        float acc0 = 0.f, acc1 = 0.f;   // message sums of the current receiver, two components
        // X of the current receiver (the residual term of Xt)
        float2 base = xx[(int64_t)cur * 2 * H];
        if (ntl > 0) {   // the partition's first tile: edge arrays and E tiles
            fetch(sbase, e0, min(QN, e1 - e0));
            if (tp == QN) copy_etiles(etiles, nrev, 0);
            cp_async_wait_all();
            pipe_sync(pp);
            if (tp < QN) prep(sbase, min(QN, e1 - e0), j0);
            pipe_sync(pp);
        }
        for (int k = 0; k < ntl; ++k) {
            const int t0 = e0 + k * QN, n = min(QN, e1 - t0), buf = k & 1;
            unsigned char* sb = sbase + buf * Q_SB_BYTES;
            unsigned char* sbn = sbase + (buf ^ 1) * Q_SB_BYTES;
            const int* rcv_s = reinterpret_cast<const int*>(sb + Q_SB_RCV);
            const int* soff = reinterpret_cast<const int*>(sb + Q_SB_SOFF);
            const float* uc = reinterpret_cast<const float*>(sb + Q_SB_UC);
            const uint32_t* chg = reinterpret_cast<const uint32_t*>(sb + Q_SB_CHG);
            // z^T = W1 e^T on the bulk-copied tile, into chunk 0's columns (read
            // by the scalar warps until the end of the previous tile's epilogue 2)
            if (tp == 0) issue_gemm1((n + 31) / 32);
            e_phase ^= 1;
            if (wl == 0) {
                __syncwarp();
                // one warp polls the MMA barrier; the others wait at the pipeline barrier
                if ((a.stall_test & 1) && k == 0 && !mbar_wait(never_bar, 0, STALL_BUDGET))
                    signal_timeout(a, abort_flag, WHERE_STALL_TEST);
                if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 1);
            }
            mma_phase ^= 1;
            fence_before_sync();
            pipe_sync(pp);
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1) -> H tile (split fp16); warp (q, hh) takes
                // hidden unit c of edges 32 hh .. 32 hh + 31
                const int col = 32 * hh, nv = n - col;
                const float bias = b1s[c];
                const BColumn hc(Hs, Q_HH, QN, col, c);
                // GEMM2 accumulates onto b2 (0 for padding edges): this warp refills the
                // chunk-0 cells it has just read and all 64 columns of chunk 1 + hh
                float bv[16];
                const float b0c = b2s[c], bch = b2s[(1 + hh) * H + c];
#pragma unroll
                for (int i0 = 0; i0 < 32; i0 += 16) {   // 16 edges per TMEM load
                    float z[16];
                    tmem_ld16(lane_base + TB + col + i0, z);
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 16; i += 2) {
                        const float z0 = z[i] + bias, z1 = z[i + 1] + bias;
                        hc.put_pair(i0 + i, z0 * fast_sigmoid(z0), z1 * fast_sigmoid(z1));
                    }
                }
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = b0c;
                tmem_st16(lane_base + TB + col, bv);
                tmem_st16(lane_base + TB + col + 16, bv);
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = bch;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) tmem_st16(lane_base + TB + 64 * (1 + hh) + 16 * kk, bv);
                if (n < QN) {   // the last tile of a partition: its padding edges get h = 0 and no bias
                    tmem_st_wait();   // the fills above land before the zeros below
#pragma unroll 1
                    for (int i = max(nv, 0); i < 32; ++i) hc.put_one(i, 0.f);
#pragma unroll 1
                    for (int i = max(nv, 0); i < 32; ++i) tmem_st1(lane_base + TB + col + i, 0.f);
#pragma unroll 1
                    for (int i = n; i < QN; ++i) tmem_st1(lane_base + TB + 64 * (1 + hh) + i, 0.f);
                }
                tmem_st_wait();
            }
            fence_async_smem();
            fence_before_sync();
            pipe_sync(pp);
            // epilogue 2's first two 8-edge blocks of sender features are
            // gathered while GEMM2 runs (padding edges read row 0)
            float xa0[8], xa1[8], xb0[8], xb1[8];
            auto gather8 = [&](float (&x0)[8], float (&x1)[8], int col) {
#pragma unroll
                for (int i = 0; i < 8; i += 4) {
                    const int4 so = *reinterpret_cast<const int4*>(soff + col + i);
                    const int sv[4] = {so.x, so.y, so.z, so.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float2 v = __ldg(xx + sv[j]);
                        x0[i + j] = v.x;
                        x1[i + j] = v.y;
                    }
                }
            };
            gather8(xa0, xa1, 0);
            if (8 < n) gather8(xb0, xb1, 8);
            if (wl < 3 && lane == 0) {   // f^T = W2 h^T, chunk wl issued by warp wl
                fence_after_sync();
                if (!w2h_ready) {
                    if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) signal_timeout(a, abort_flag, 6);
                    w2h_ready = true;
                }
                issue_gemm2_chunk<QN>(wl, tmem, TB + 64 * wl, w2h, w2l, Hs);
                mma_commit(g2_bar);
            }
            if (wl < 3) __syncwarp();   // lanes 1-31 of the issuing warps wait here, not in a spin loop
            if (wl == 0 && !mbar_wait(g2_bar, g2_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 4);
            g2_phase ^= 1;
            fence_before_sync();
            // the abort decision is the same for every thread of the pipeline
            const bool abort_now = pipe_sync_or(pp, *abort_flag != 0);
            fence_after_sync();
            // the H tile is free: the next tile's E tile and edge arrays arrive
            // while epilogue 2 runs
            const bool more = k + 1 < ntl && !abort_now;
            if (more) {
                fetch(sbn, t0 + QN, min(QN, e1 - t0 - QN));
                if (tp == QN) copy_etiles(etiles, nrev, k + 1);
            }
            if (wl == 2) __syncwarp();
            {   // epilogue 2: components 2 hh, 2 hh + 1 of the message sums, segmented
                // by receiver; 8-edge blocks, the next block's gathers in flight
                const float* u0 = uc + (hh == 0 ? 0 : QN);        // u component of comp. 2 hh (hh = 1: y)
                const float* u1 = uc + (hh == 0 ? 0 : 2 * QN);    // of comp. 2 hh + 1 (x or z)
                // (compiled once per warp half: hc is std::integral_constant<int, hh>)
                auto process8 = [&](auto hc, const float (&x0)[8], const float (&x1)[8], int col) {
                    constexpr int HH = decltype(hc)::value;
                    float fa[8], f1[8], f2[8];
                    if (HH == 0) tmem_ld8(lane_base + TB + col, fa);   // phi_s
                    tmem_ld8(lane_base + TB + 64 + col, f1);            // phi_v1
                    tmem_ld8(lane_base + TB + 128 + col, f2);           // phi_v2
                    const uint32_t m = (chg[col >> 5] >> (col & 31)) & 0xFFu;
                    // the block's u components, two 16-byte shared loads per array
                    // (u arrays and col are 32-byte aligned)
                    float ua[8], ub[8];
                    *reinterpret_cast<float4*>(ub) = *reinterpret_cast<const float4*>(u1 + col);
                    *reinterpret_cast<float4*>(ub + 4) = *reinterpret_cast<const float4*>(u1 + col + 4);
                    if (HH != 0) {
                        *reinterpret_cast<float4*>(ua) = *reinterpret_cast<const float4*>(u0 + col);
                        *reinterpret_cast<float4*>(ua + 4) = *reinterpret_cast<const float4*>(u0 + col + 4);
                    }
                    tmem_ld_wait();
                    // message terms of edge i added to the sums, the same expressions on
                    // both branches (a block's branch depends on where the tile starts)
                    auto add_m = [&](int i) {
                        if (HH == 0) acc0 = fmaf(x0[i], fa[i], acc0);
                        else acc0 = fmaf(x0[i], f1[i], fmaf(ua[i], f2[i], acc0));
                        acc1 = fmaf(x1[i], f1[i], fmaf(ub[i], f2[i], acc1));
                    };
                    if (m == 0) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) add_m(i);
                    } else {   // a receiver starts in this block: store the finished sums
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            if (m & (1u << i)) {
                                out[(int64_t)cur * 4 * H] = base.x + acc0;
                                out[(int64_t)cur * 4 * H + H] = base.y + acc1;
                                cur = rcv_s[col + i];
                                base = xx[(int64_t)cur * 2 * H];
                                acc0 = 0.f;
                                acc1 = 0.f;
                            }
                            add_m(i);
                        }
                    }
                };
                auto blocks = [&](auto hc) {
                    for (int col = 0; col < n; col += 16) {   // blocks col and col + 8 are in flight
                        process8(hc, xa0, xa1, col);
                        if (col + 8 >= n) break;
                        if (col + 16 < n) gather8(xa0, xa1, col + 16);
                        process8(hc, xb0, xb1, col + 8);
                        if (col + 24 < n) gather8(xb0, xb1, col + 24);
                    }
                };
                if (hh == 0) blocks(std::integral_constant<int, 0>{});
                else blocks(std::integral_constant<int, 1>{});
            }
            if (more && tp < QN) {   // the next tile's prep, by the two warps that fetched it
                cp_async_wait_all();
                pipe_sync_first(pp, QN);
                prep(sbn, min(QN, e1 - t0 - QN), rcv_s[QN - 1]);
            }
            fence_before_sync();
            pipe_sync(pp);
            if (abort_now) {
                aborted = true;
                break;
            }
        }
        if (!aborted) {
            out[(int64_t)cur * 4 * H] = base.x + acc0;
            out[(int64_t)cur * 4 * H + H] = base.y + acc1;
        }
    }
    // drain: every MMA and copy this CTA issued must be complete before it
    // frees its tensor memory and exits (a wait on the parity of the phase
    // before the current one returns at once)
    __syncthreads();
    if (tp == 0) {
        if (!mbar_wait(mma_bar, mma_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 3);
        if (!mbar_wait(g2_bar, g2_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 5);
    }
    if (tp == QN) {
        if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 7);
        if (e_issued > 0 && !mbar_wait(e_bar, (e_issued - 1) & 1, WAIT_BUDGET))
            set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 9);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------- reverse kernel
// Two independent pipelines per CTA, warps 0-7 and 8-15, each on its own
// receiver partition (CTA b: partitions 2b and 2b + 1, then 2b + 2G ...),
// so that one pipeline's MMAs, copies and barrier waits overlap the other
// pipeline's CUDA-core epilogues.  A pipeline processes 32-edge tiles with
// E and E' (then H and H') stacked as rows 0-31 / 32-63 of one 64-row B
// tile: every MMA is 128 x 64 x 16 and one pass gives the filter and its
// d-derivative (forward mode, no transposed GEMM, no stored activation).
//
// The third filter chunk (phi_v2, the u-direction term) enters the reverse
// pass only through sums over channels with the receiver's v adjoint:
//   dE/du_k(e) = sum_c dE/dXt_{v_k}(i)[c] phi_v2(e)[c] = Q_k(i) . h_e + beta_k(i)
//   its dE/dd term = sum_k u_k(e) Q_k(i) . h'_e
// with Q_k(i) = W2[2H:3H]^T dE/dXt_{v_k}(i) and beta_k(i) = b2[2H:3H] .
// dE/dXt_{v_k}(i) precomputed per atom (vq_kernel).  So GEMM2 computes
// chunks 0 and 1 only, and GEMM3 multiplies the Q rows of the tile's
// receivers (rows 3 r + k, 21 receivers per round) with the same [H; H']
// tile: its outputs are already summed over channels.
//
// TMEM (512 columns): [0,128) the lo halves of W2 chunks 0-1 (shared A
// operands); pipeline p owns [128 + 192 p, 320 + 192 p): chunk g (0, 1) at
// + 64 g with f in its first 32 columns and f' in the next 32; GEMM1's
// [z | z'] output at + 128 until epilogue 1 has read it, then GEMM3's
// [Q h | Q h'].
//
// Epilogue 2 roles: warp (q, h) of a pipeline reads TMEM lane quarter q
// (channels 32q..32q+31) and handles two feature components of every edge
// of the tile: h = 0 the scalar and v_x, h = 1 v_y and v_z.  Node adjoints
// are gathered from the sender side (exact: f(d_ab) = f(d_ba)) and summed per
// receiver in registers; each thread's share of the remaining dE/dd terms
// is reduced across lanes (one value per edge).  Epilogue 3: the threads
// owning GEMM3's rows (warps of quarters 0 and 1) scatter dE/du and the
// u-term of dE/dd of their receiver's edges.
// Padding edges of a partial tile get h = h' = 0 and a zero bias fill, so
// their filter is exactly zero and every gather runs unpredicated (padding
// gathers read row 0).
constexpr int PN = 32;                               // edges per reverse tile
constexpr uint32_t P_HH = 2 * b_block(2 * PN);       // one half (hi or lo) of a [H; H'] tile: 16 KB
constexpr int QR = 21;                               // receivers per GEMM3 round (rows 3 r + k < 64)
constexpr uint32_t QT_HALF = 8 * 2048;               // one half (hi or lo) of a Q tile: 64 rows x K 128
constexpr uint32_t R_SB_US = 0;
constexpr uint32_t R_SB_SRC = R_SB_US + PN * 16;
constexpr uint32_t R_SB_RCV = R_SB_SRC + PN * 4;
constexpr uint32_t R_SB_SOFF = R_SB_RCV + PN * 4;
constexpr uint32_t R_SB_ROFF = R_SB_SOFF + PN * 4;
constexpr uint32_t R_SB_UC = R_SB_ROFF + PN * 4;
constexpr uint32_t R_SB_CHG = R_SB_UC + 3 * PN * 4;
constexpr uint32_t R_SB_EACC = R_SB_CHG + 16;
constexpr uint32_t R_SB_BYTES = R_SB_EACC + PN * 16;
constexpr uint32_t R_OFF_W1 = 0;
constexpr uint32_t R_OFF_W2H = R_OFF_W1 + W1_BYTES;           // hi tiles of W2 chunks 0-1
constexpr uint32_t R_OFF_H = align1k(R_OFF_W2H + 16 * A_TILE);  // pipeline p's [H; H'] tile at + 2 P_HH p
constexpr uint32_t R_OFF_Q = align1k(R_OFF_H + 4 * P_HH);       // pipeline p's Q tile (hi, lo) at + 2 QT_HALF p
constexpr uint32_t R_OFF_SB = R_OFF_Q + 4 * QT_HALF;            // [pipeline][buffer] edge arrays
constexpr uint32_t R_OFF_B1 = R_OFF_SB + 4 * R_SB_BYTES;
constexpr uint32_t R_OFF_B2 = R_OFF_B1 + H * 4;                // b2 of chunks 0-1
constexpr uint32_t R_OFF_RED = R_OFF_B2 + 2 * H * 4;           // [pipeline] per-edge partial sums
constexpr uint32_t R_RED_DU = 8 * PN;                          // red: [8 warps][PN] dE/dd shares,
constexpr uint32_t R_RED_DDU = R_RED_DU + 3 * PN;              //      [3][PN] dE/du_k, [3][PN] u_k terms of dE/dd
constexpr uint32_t R_RED_FLOATS = R_RED_DDU + 3 * PN;
constexpr uint32_t R_OFF_BAR = R_OFF_RED + 2 * R_RED_FLOATS * 4;
constexpr uint32_t R_OFF_MISC = R_OFF_BAR + 10 * 8;
constexpr uint32_t R_SMEM = align1k(R_OFF_MISC + 16);
static_assert(ET_BYTES <= 2 * P_HH, "E tile fits in the H tile's space");
static_assert(R_SB_EACC % 16 == 0 && R_SB_BYTES % 16 == 0, "edge array alignment");
// GEMM3 is an M = 128 MMA on a 64-row A tile: its rows 64-127 read the
// 1 KB after each K-step (the next K-step, the next half or tile, and after
// the last Q half the edge arrays), results never read back
static_assert(4 * R_SB_BYTES >= 1024, "bytes behind the last Q half");
static_assert(3 * QR <= 64, "Q rows of a round");
static_assert(R_SMEM <= 232448, "reverse kernel shared memory");

// GEMM3: D (64 TMEM columns at dcol) = Q [H; H']^T, the Q tile at qt (hi
// half, then lo half QT_HALF bytes later; K-major, no swizzle, rows 0-63,
// LBO 1024, K-steps 2048 bytes apart), B the split-fp16 [H; H'] tile.
__device__ __forceinline__ void issue_gemm3(uint32_t tmem, uint32_t dcol, const unsigned char* qt,
                                            const unsigned char* Hs) {
    constexpr uint32_t idesc = idesc_f16(2 * PN);
    constexpr uint64_t DH = (2 * b_block(2 * PN)) >> 4;
    const uint64_t a0 = sdesc(smem_u32(qt), 1024, 128);
    const uint64_t b0 = sdesc_b(smem_u32(Hs));
    const uint32_t d = tmem + dcol;
#pragma unroll 1
    for (int s = 0; s < 8; ++s) {
        const uint64_t bh = b0 + (uint64_t)(b_kstep_off(2 * PN, s) >> 4);
        const uint64_t ah = a0 + (uint64_t)((2048 * s) >> 4), al = ah + (uint64_t)(QT_HALF >> 4);
        mma_f16(d, ah, bh, idesc, s > 0 ? 1u : 0u);
        mma_f16(d, ah, bh + DH, idesc, 1);
        mma_f16(d, al, bh, idesc, 1);
    }
}

// Per-atom Q rows of the reverse kernel (one layer), on the tensor cores:
// for atom i and k in {x, y, z}, Q_k(i)[h] = sum_c W2[2H + c][h]
// dE/dXt[i][1 + k][c], stored as split fp16 (128 hi, then 128 lo), and
// beta_k(i) = sum_c b2[2H + c] dE/dXt[i][1 + k][c].  Persistent, one CTA per
// SM, 64-atom tiles: B = the tile's 192 rows (atom, k) of dE/dXt_v (K = 128
// channels, split fp16, 128-byte swizzle), A = the packed transpose of W2's
// third chunk (resident), D = Q^T in TMEM (lane = hidden unit, column = row);
// the epilogue thread of hidden unit h writes its values of 48 rows.  Two
// CTAs per SM, 32-atom tiles.
constexpr int VQ_TA = 32, VQ_TR = 3 * VQ_TA, VQ_NT = 256;
constexpr uint32_t VQ_BH = 2 * b_block(VQ_TR);                 // one half of the B tile (K = 128)
constexpr uint32_t VQ_OFF_A = 0;                               // 8 K-step pairs, 64 KB
constexpr uint32_t VQ_OFF_B = VQ_OFF_A + 8 * A_PAIR;
constexpr uint32_t VQ_OFF_BAR = VQ_OFF_B + 2 * VQ_BH;
constexpr uint32_t VQ_SMEM = align1k(VQ_OFF_BAR + 32);
static_assert(VQ_SMEM <= 232448, "vq shared memory");

__global__ void __launch_bounds__(VQ_NT, 2) vq_tc_kernel(const float* __restrict__ P, LayerOffsets lo,
                                                        const float* __restrict__ xtbar, int n_atoms,
                                                        unsigned char* __restrict__ qs, float* __restrict__ qb,
                                                        Status* st) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* As = smem + VQ_OFF_A;
    unsigned char* Bs = smem + VQ_OFF_B;
    uint64_t* a_bar = reinterpret_cast<uint64_t*>(smem + VQ_OFF_BAR);
    uint64_t* mma_bar = a_bar + 1;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + VQ_OFF_BAR + 16);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + VQ_OFF_BAR + 20);
    pdl_wait();
    if (st->code != 0) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w == 0) {
        tmem_alloc(tslot, 128);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(a_bar, 1);
        mbar_init(mma_bar, 1);
        fence_mbar_init();
        *abort_flag = 0;
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    pdl_trigger();   // after the TMEM allocation
    if (t == 0) {
        const unsigned char* src = reinterpret_cast<const unsigned char*>(P + lo.w2q_tc);
        mbar_expect_tx(a_bar, 8 * A_PAIR);
#pragma unroll
        for (int i = 0; i < 4; ++i) bulk_g2s(As + i * 2 * A_PAIR, src + i * 2 * A_PAIR, 2 * A_PAIR, a_bar);
    }
    float4 bb;   // b2[2H + 4 lane .. 4 lane + 3]
    bb = reinterpret_cast<const float4*>(P + lo.b2 + 2 * H)[lane];
    const int q = w & 3, ch = w >> 2;       // epilogue: lane quarter q, column half ch
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    const int h = 32 * q + lane;
    uint32_t phase = 0;
    bool a_ready = false;
    const int ntiles = (n_atoms + VQ_TA - 1) / VQ_TA;
    for (int tile = blockIdx.x; tile < ntiles && !*abort_flag; tile += gridDim.x) {
        const int a0 = tile * VQ_TA;
        // B tile: warp w builds rows w, w + 8, ..., w + 88 (all loads issued
        // first); lane takes channels 4 lane .. 4 lane + 3; beta by warp sums
        {
            // (dE/dXt in the pair layout: component k of channels 4 lane .. +3
            // is every other float of two 16-byte words)
            float4 x[12];
#pragma unroll
            for (int u = 0; u < 12; ++u) {
                const int row = w + 8 * u, atom = a0 + row / 3, comp = 1 + row % 3;
                if (atom < n_atoms) {
                    const float4* pr = reinterpret_cast<const float4*>(xtbar + (int64_t)atom * 4 * H + (comp >> 1) * 2 * H);
                    const float4 p0 = pr[2 * lane], p1 = pr[2 * lane + 1];
                    x[u] = (comp & 1) ? make_float4(p0.y, p0.w, p1.y, p1.w) : make_float4(p0.x, p0.z, p1.x, p1.z);
                } else {
                    x[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
#pragma unroll
            for (int u = 0; u < 12; ++u) {
                const int row = w + 8 * u, atom = a0 + row / 3;
                __half2 h0, l0, h1, l1;
                split2(x[u].x, x[u].y, h0, l0);
                split2(x[u].z, x[u].w, h1, l1);
                const uint32_t o = b_off(VQ_TR, row, 4 * lane);
                uint2 hv, lv;
                hv.x = *reinterpret_cast<uint32_t*>(&h0);
                hv.y = *reinterpret_cast<uint32_t*>(&h1);
                lv.x = *reinterpret_cast<uint32_t*>(&l0);
                lv.y = *reinterpret_cast<uint32_t*>(&l1);
                *reinterpret_cast<uint2*>(Bs + o) = hv;
                *reinterpret_cast<uint2*>(Bs + VQ_BH + o) = lv;
                float b = fmaf(bb.x, x[u].x, fmaf(bb.y, x[u].y, fmaf(bb.z, x[u].z, bb.w * x[u].w)));
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) b += __shfl_xor_sync(0xffffffffu, b, off);
                if (lane == 0 && atom < n_atoms) qb[(int64_t)a0 * 3 + row] = b;
            }
        }
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (t == 0) {   // Q^T = W2q^T B^T: 8 K-steps x (hi hi, hi lo, lo hi)
            fence_after_sync();
            if (!a_ready) {
                if (!mbar_wait(a_bar, 0, WAIT_BUDGET)) {
                    set_status(st, MLFF_ERR_TIMEOUT, 40);
                    *abort_flag = 1;
                }
                a_ready = true;
            }
            constexpr uint32_t idesc = idesc_f16(VQ_TR);
            const uint64_t b0 = sdesc_b(smem_u32(Bs));
#pragma unroll 1
            for (int s = 0; s < 8; ++s) {
                const uint64_t ah = sdesc(smem_u32(As + s * A_PAIR), A_LBO, A_SBO);
                const uint64_t al = sdesc(smem_u32(As + s * A_PAIR + A_TILE), A_LBO, A_SBO);
                const uint64_t bh = b0 + (uint64_t)(b_kstep_off(VQ_TR, s) >> 4);
                mma_f16(tmem, ah, bh, idesc, s > 0 ? 1u : 0u);
                mma_f16(tmem, ah, bh + (VQ_BH >> 4), idesc, 1);
                mma_f16(tmem, al, bh, idesc, 1);
            }
            mma_commit(mma_bar);
        }
        if (w == 0) {
            __syncwarp();
            if (!mbar_wait(mma_bar, phase, WAIT_BUDGET)) {
                set_status(st, MLFF_ERR_TIMEOUT, 41);
                *abort_flag = 1;
            }
        }
        phase ^= 1;
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        // epilogue: thread of hidden unit h, rows 48 ch .. 48 ch + 47
        {
            float v[48];
            tmem_ld32(lane_base + 48 * ch, *reinterpret_cast<float(*)[32]>(v));
            tmem_ld16(lane_base + 48 * ch + 32, *reinterpret_cast<float(*)[16]>(v + 32));
            tmem_ld_wait();
            const int nrow = min(48, 3 * (n_atoms - a0) - 48 * ch);
#pragma unroll
            for (int i = 0; i < 48; ++i) {
                if (i >= nrow) break;
                __half hi, lo;
                split_f16(v[i], hi, lo);
                __half* dst = reinterpret_cast<__half*>(qs + ((int64_t)a0 * 3 + 48 * ch + i) * 2 * (2 * H));
                dst[h] = hi;
                dst[H + h] = lo;
            }
        }
        fence_before_sync();
        __syncthreads();   // D and the B tile are free for the next tile
        fence_after_sync();
    }
    // drain: the weight copy and the last MMAs are complete before the TMEM
    // is freed (a wait on the phase before the current one returns at once)
    if (t == 0) {
        if (!mbar_wait(a_bar, 0, WAIT_BUDGET)) set_status(st, MLFF_ERR_TIMEOUT, 42);
        if (!mbar_wait(mma_bar, phase ^ 1, WAIT_BUDGET)) set_status(st, MLFF_ERR_TIMEOUT, 43);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 128);
}

__global__ void __launch_bounds__(NT, 1) edge_bwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                            const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + R_OFF_W1;
    unsigned char* w2h = smem + R_OFF_W2H;
    float* b1s = reinterpret_cast<float*>(smem + R_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + R_OFF_B2);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + R_OFF_BAR);
    uint64_t* w2h_bar = bars;                       // resident W2 operands
    uint64_t* never_bar = bars + 1;                 // test hook: nothing arrives here
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + R_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + R_OFF_MISC + 4);

    // waits for the previous kernel at entry: reading the status word first
    // and returning early keeps the main loop's register allocation lean
    pdl_wait();
    if (a.st->code != 0) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w == 0) {
        tmem_alloc(tslot, 512);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(w2h_bar, 1);
        mbar_init(never_bar, 1);
        for (int p = 0; p < 2; ++p) {
            mbar_init(bars + 2 + 4 * p, 1);   // GEMM1
            mbar_init(bars + 3 + 4 * p, 1);   // E tile
            mbar_init(bars + 4 + 4 * p, 2);   // GEMM2: one commit per chunk issuer
            mbar_init(bars + 5 + 4 * p, 1);   // GEMM3
        }
        fence_mbar_init();
        *abort_flag = 0;
    }
    for (int i = t; i < (int)(W1_BYTES / 16); i += NT)
        reinterpret_cast<uint4*>(w1s)[i] = reinterpret_cast<const uint4*>(w1g)[i];
    if (t < H) b1s[t] = a.P[a.lo.b1 + t];
    for (int i = t; i < 2 * H; i += NT) b2s[i] = a.P[a.lo.b2 + i];
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    if (t == 32) {   // hi tiles of W2 chunks 0-1 (the first 16 tiles of the packed hi half)
        mbar_expect_tx(w2h_bar, 16 * A_TILE);
#pragma unroll
        for (int i = 0; i < 4; ++i) bulk_g2s(w2h + i * 4 * A_TILE, w2g + i * 4 * A_TILE, 4 * A_TILE, w2h_bar);
    }
    const int q = w & 3;
    const int c = 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    load_w2_lo_tmem(lane_base, reinterpret_cast<const uint32_t*>(a.P + a.lo.w2_tm), w >> 2, c);
    tmem_st_wait();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    pdl_trigger();   // after the TMEM allocation

    // ---- this thread's pipeline
    const int pp = w >> 3, wl = w & 7, tp = t & (PT - 1), hh = wl >> 2;
    const uint32_t TB = 128 + 192 * pp;             // the pipeline's TMEM columns
    unsigned char* Hs = smem + R_OFF_H + pp * 2 * P_HH;   // [H; H'] hi, then lo
    unsigned char* Es = Hs;                         // [E; E'] tile (bulk-copied) before H is written
    unsigned char* qt = smem + R_OFF_Q + pp * 2 * QT_HALF;   // Q tile hi, then lo
    uint64_t* mma_bar = bars + 2 + 4 * pp;
    uint64_t* e_bar = bars + 3 + 4 * pp;
    uint64_t* g2_bar = bars + 4 + 4 * pp;
    uint64_t* g3_bar = bars + 5 + 4 * pp;
    float* red = reinterpret_cast<float*>(smem + R_OFF_RED) + pp * R_RED_FLOATS;
    unsigned char* sbase = smem + R_OFF_SB + 2 * pp * R_SB_BYTES;
    const int rs8_idx = reduce_scatter8_index(lane);
    // components 2 hh and 2 hh + 1: one float2 of the pair layout of dE/dXt
    // and X, H floats apart in the component-major dE/dX
    const float2* xtb = reinterpret_cast<const float2*>(a.xtbar + pair_off(2 * hh, c));
    const float2* xx = reinterpret_cast<const float2*>(a.X + pair_off(2 * hh, c));
    float* out = a.xbar + 2 * hh * H + c;

    uint32_t mma_phase = 0, g2_phase = 0, g3_phase = 0;   // GEMM1 / GEMM2 / GEMM3 barrier phases
    uint32_t e_phase = 0, e_issued = 0;     // E-tile copies: barrier phase, copies issued (thread tp 32)
    bool w2h_ready = false;                 // (GEMM2 issuers)
    bool aborted = false;
    auto prep = [&](unsigned char* sbx, int nn, int prev) {
        tile_prep<PN>(tp, nn, prev, reinterpret_cast<int*>(sbx + R_SB_SRC), reinterpret_cast<int*>(sbx + R_SB_RCV),
                      reinterpret_cast<float4*>(sbx + R_SB_US), reinterpret_cast<int*>(sbx + R_SB_SOFF),
                      reinterpret_cast<int*>(sbx + R_SB_ROFF), reinterpret_cast<float*>(sbx + R_SB_UC),
                      reinterpret_cast<uint32_t*>(sbx + R_SB_CHG));
    };
    auto fetch = [&](unsigned char* sbx, int t0, int nn) {
        fetch_tile_edges(a, tp, PN, t0, nn, reinterpret_cast<float4*>(sbx + R_SB_US),
                         reinterpret_cast<int*>(sbx + R_SB_SRC), reinterpret_cast<int*>(sbx + R_SB_RCV),
                         a.eacc_init ? nullptr : reinterpret_cast<float4*>(sbx + R_SB_EACC));
    };
    // [z; z']^T = W1 [e; e']^T on the [E; E'] tile at Es into the [z | z']
    // columns, once its copy has landed (thread tp 0)
    auto issue_gemm1 = [&]() {
        if (!mbar_wait(e_bar, e_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 18);
        fence_after_sync();
        constexpr uint32_t idesc = idesc_f16(2 * PN);
#pragma unroll
        for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int pr = 0; pr < 3; ++pr) {
                const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                const uint64_t bd = sdesc(smem_u32(Es + bhl * ET_HALF + s * 2 * ET_LBO), ET_LBO, ET_SBO);
                mma_f16(tmem + TB + 128, ad, bd, idesc, (s | pr) != 0);
            }
        mma_commit(mma_bar);
    };
    for (int p = 2 * blockIdx.x + pp; p < a.nparts && !aborted; p += 2 * gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        const int ntl = (e1 - e0 + PN - 1) / PN;
        const unsigned char* etiles = a.etile + (size_t)a.etile_base[p] * ET_BYTES;
        // dE/dX = dE/dXt + the gathered sums: receivers without edges get their dE/dXt row
        if (a.write_nodes) copy_empty_rows(a.xbar, a.xtbar, a.row_ptr, j0, j1, wl, lane, PT / 32);
        int cur = j0;
        float acc0 = 0.f, acc1 = 0.f;   // gathered node adjoints of the current receiver, two components
        float cr0, cr1;                 // its dE/dXt rows (the same two components)
        {
            const float2 r = __ldg(xtb + (int64_t)j0 * 2 * H);
            cr0 = r.x;
            cr1 = r.y;
        }
        if (ntl > 0) {   // the partition's first tile: edge arrays and [E; E'] tile
            fetch(sbase, e0, min(PN, e1 - e0));
            if (tp == 32) {
                mbar_expect_tx(e_bar, ET_BYTES);
                bulk_g2s(Es, etiles, ET_BYTES, e_bar);
                ++e_issued;
            }
            cp_async_wait_all();
            pipe_sync(pp);
            if (tp < PN) prep(sbase, min(PN, e1 - e0), j0);
            pipe_sync(pp);
        }
        for (int k = 0; k < ntl; ++k) {
            const int t0 = e0 + k * PN, n = min(PN, e1 - t0), buf = k & 1;
            unsigned char* sb = sbase + buf * R_SB_BYTES;
            unsigned char* sbn = sbase + (buf ^ 1) * R_SB_BYTES;
            const int* rcv_s = reinterpret_cast<const int*>(sb + R_SB_RCV);
            const int* soff = reinterpret_cast<const int*>(sb + R_SB_SOFF);
            const int* roff = reinterpret_cast<const int*>(sb + R_SB_ROFF);
            const float* uc = reinterpret_cast<const float*>(sb + R_SB_UC);
            const uint32_t chw = *reinterpret_cast<const uint32_t*>(sb + R_SB_CHG);
            // the tile's receivers: local receiver r starts at edge r_first(r)
            const uint32_t starts = chw & ~1u;
            const int nrcv = 1 + __popc(starts);
            auto r_first = [&](int r) { return r == 0 ? 0 : (int)__fns(starts, 0, r); };
            // Q rows of receivers QR b .. QR b + 20 into the Q tile (row 3 r' + k)
            auto fill_q = [&](int b) {
                const int nrow = 3 * min(QR, nrcv - QR * b);
                for (int i = tp; i < 32 * nrow; i += PT) {
                    const int m = i >> 5, j = i & 15, hl = (i >> 4) & 1;
                    const int atom = rcv_s[r_first(QR * b + m / 3)];
                    const unsigned char* src = a.qs + (((int64_t)atom * 3 + m % 3) * 2 + hl) * (2 * H) + 16 * j;
                    cp_async16(qt + hl * QT_HALF + (j >> 1) * 2048 + (j & 1) * 1024 + (m >> 3) * 128 + (m & 7) * 16,
                               src);
                }
                cp_async_commit();
            };
            fill_q(0);
            // [z; z']^T = W1 [e; e']^T on the bulk-copied tile: the partition's
            // first tile here, later tiles at the end of the previous tile's
            // epilogue 2
            if (k == 0 && tp == 0) issue_gemm1();
            e_phase ^= 1;
            if (wl == 0) {
                __syncwarp();
                // one warp polls the MMA barrier; the others wait at the
                // pipeline barrier instead of spinning
                if ((a.stall_test & 2) && k == 0 && !mbar_wait(never_bar, 0, STALL_BUDGET))
                    signal_timeout(a, abort_flag, WHERE_STALL_TEST);
                if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 11);
            }
            mma_phase ^= 1;
            fence_before_sync();
            pipe_sync(pp);
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1) (rows 0-31), h' = silu'(z + b1) z'
                // (rows 32-63); warp (q, hh) takes hidden units 32 q .. 32 q + 31 of
                // edges 16 hh .. 16 hh + 15 in the 16x256b fragment -- thread t holds
                // hidden units 16 g + t/4 and 16 g + 8 + t/4 of lane group g, edges
                // 2 (t % 4), + 1 and the same + 8 --, which is the m8n8 fragment of
                // 8 x 8 (hidden x edge) blocks: stmatrix .trans writes each block's
                // edge rows as the 16-byte chunks of the K-major tile
                const int col = 16 * hh, nv = n - col;   // valid edges among this warp's 16
                const int r4 = lane >> 2, c2 = 2 * (lane & 3);
                // this thread's stmatrix row: row R = lane % 8 of block m = lane / 8
                // (edge half s = m / 2, hidden half w = m % 2)
                const int mb = lane >> 3, R = lane & 7;
                const uint32_t rowaddr = smem_u32(Hs) + (uint32_t)((q >> 1) * b_block(2 * PN) +
                                                                   ((col >> 3) + (mb >> 1)) * 1024 + R * 128);
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    float z[8], zd[8];
                    tmem_ld16x256_x2(lane_base + ((uint32_t)(16 * g) << 16) + TB + 128 + col, z);
                    tmem_ld16x256_x2(lane_base + ((uint32_t)(16 * g) << 16) + TB + 128 + PN + col, zd);
                    const float bA = b1s[32 * q + 16 * g + r4], bB = b1s[32 * q + 16 * g + 8 + r4];
                    tmem_ld_wait();
                    float hv[8], hd[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {   // value i: edge 8 (i / 4) + c2 + i % 2, hidden block (i / 2) % 2
                        const float zz = z[i] + (((i >> 1) & 1) ? bB : bA);
                        const float sg = fast_sigmoid(zz);
                        const bool valid = 8 * (i >> 2) + c2 + (i & 1) < nv;
                        hv[i] = valid ? zz * sg : 0.f;
                        hd[i] = valid ? sg * (1.0f + zz * (1.0f - sg)) * zd[i] : 0.f;
                    }
                    // block m (registers 4 (m / 2) + 2 (m % 2), + 1) -> 16-byte rows
                    uint32_t fh[4], fl[4], dh[4], dl[4];
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
                        const int i0 = 4 * (m >> 1) + 2 * (m & 1);
                        split_pack(hv[i0], hv[i0 + 1], fh[m], fl[m]);
                        split_pack(hd[i0], hd[i0 + 1], dh[m], dl[m]);
                    }
                    const uint32_t a = rowaddr + ((((4 * (q & 1) + 2 * g + (mb & 1)) ^ R)) << 4);
                    stmatrix_x4_trans(a, fh[0], fh[1], fh[2], fh[3]);                       // h hi
                    stmatrix_x4_trans(a + P_HH, fl[0], fl[1], fl[2], fl[3]);                // h lo
                    stmatrix_x4_trans(a + 4 * 1024, dh[0], dh[1], dh[2], dh[3]);            // h' hi (rows + 32)
                    stmatrix_x4_trans(a + 4 * 1024 + P_HH, dl[0], dl[1], dl[2], dl[3]);     // h' lo
                }
                // f = W2 h accumulates onto b2 (0 for padding edges), f' = W2 h'
                // onto 0: this warp refills chunk hh (f: 32 columns, f': 32
                // columns); GEMM3 overwrites the [z | z'] columns
                float bv[16], bz[16];
                const float bch = b2s[hh * H + c];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    bv[i] = i < n ? bch : 0.0f;
                    bz[i] = 0.0f;
                }
                tmem_st16(lane_base + TB + 64 * hh, bv);
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = 16 + i < n ? bch : 0.0f;
                tmem_st16(lane_base + TB + 64 * hh + 16, bv);
                tmem_st16(lane_base + TB + 64 * hh + PN, bz);
                tmem_st16(lane_base + TB + 64 * hh + PN + 16, bz);
                tmem_st_wait();
            }
            cp_async_wait_all();   // this thread's Q-tile rows
            fence_async_smem();
            fence_before_sync();
            pipe_sync(pp);
            // epilogue 2's first two 4-edge blocks of gathers are issued while
            // GEMM2 runs: the senders' dE/dXt and X rows and, when a receiver
            // starts at the block's first edge, that receiver's dE/dXt rows
            // (receivers that start inside a block load theirs in epilogue 2;
            // otherwise the rows carry over from the previous block)
            float tba0[4], tba1[4], xba0[4], xba1[4], ra0 = 0.f, ra1 = 0.f;
            float tbb0[4], tbb1[4], xbb0[4], xbb1[4], rb0 = 0.f, rb1 = 0.f;
            auto gather4 = [&](float (&tb0)[4], float (&tb1)[4], float (&xb0)[4], float (&xb1)[4], float& r0,
                               float& r1, int col) {
                const int4 so = *reinterpret_cast<const int4*>(soff + col);
                const int sv[4] = {so.x, so.y, so.z, so.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float2 t = __ldg(xtb + sv[i]), x = __ldg(xx + sv[i]);
                    tb0[i] = t.x;
                    tb1[i] = t.y;
                    xb0[i] = x.x;
                    xb1[i] = x.y;
                }
                if ((chw >> col) & 1u) {
                    const float2 r = __ldg(xtb + roff[col]);
                    r0 = r.x;
                    r1 = r.y;
                }
            };
            gather4(tba0, tba1, xba0, xba1, ra0, ra1, 0);
            if (4 < n) gather4(tbb0, tbb1, xbb0, xbb1, rb0, rb1, 4);
            if (wl < 3 && lane == 0) {   // GEMM2 chunks 0, 1 (warps 0, 1), GEMM3 (warp 2)
                fence_after_sync();
                if (wl < 2) {
                    if (!w2h_ready) {
                        if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) signal_timeout(a, abort_flag, 16);
                        w2h_ready = true;
                    }
                    issue_gemm2_chunk<2 * PN>(wl, tmem, TB + 64 * wl, w2h, w2h, Hs);   // (chunk 2's lo tile unused)
                    mma_commit(g2_bar);
                } else {
                    issue_gemm3(tmem, TB + 128, qt, Hs);
                    mma_commit(g3_bar);
                }
            }
            if (wl < 3) __syncwarp();   // lanes 1-31 of the issuing warps wait here, not in a spin loop
            if (wl == 0 && !mbar_wait(g2_bar, g2_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 14);
            if (wl == 3 && !mbar_wait(g3_bar, g3_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 30);
            g2_phase ^= 1;
            g3_phase ^= 1;
            fence_before_sync();
            // the abort decision is the same for every thread of the pipeline
            const bool abort_now = pipe_sync_or(pp, *abort_flag != 0);
            fence_after_sync();
            // epilogue 3 (warps of lane quarters 0-1): GEMM3 row l = 3 r' + kk is
            // receiver QR b + r', component kk; its columns are the tile's edges
            // ([Q h | Q h']); the row owner writes the values of its receiver's edges
            auto epi3 = [&](int b) {
                if (q >= 2) return;
                const int l = 32 * q + lane, r = QR * b + l / 3, kk = l % 3;
                const bool on = l < 3 * QR && r < nrcv;
                if (!__any_sync(0xffffffffu, on)) return;   // no receiver row of this round in this warp
                const int s0 = on ? r_first(r) : 0;
                const int s1 = on ? (r + 1 < nrcv ? r_first(r + 1) : n) : 0;
                float v[32];
                tmem_ld32(lane_base + TB + 128 + 32 * hh, v);   // hh 0: Q h, hh 1: Q h'
                tmem_ld_wait();
                if (hh == 0) {   // dE/du_kk = Q h + beta
                    const float beta = on ? __ldg(a.qb + (int64_t)rcv_s[s0] * 3 + kk) : 0.f;
                    float* dst = red + R_RED_DU + kk * PN;
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        if (i >= s0 && i < s1) dst[i] = v[i] + beta;
                } else {         // u_kk (Q h') of dE/dd
                    float* dst = red + R_RED_DDU + kk * PN;
                    const float4* u4 = reinterpret_cast<const float4*>(uc + kk * PN);   // 16-byte aligned
#pragma unroll
                    for (int i4 = 0; i4 < 8; ++i4) {
                        const float4 u = u4[i4];
                        const float uu[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int i = 4 * i4 + j;
                            if (i >= s0 && i < s1) dst[i] = uu[j] * v[i];
                        }
                    }
                }
            };
            epi3(0);
            const int nround = (nrcv + QR - 1) / QR;
            for (int b = 1; b < nround && !abort_now; ++b) {   // tiles of more than 21 receivers
                tmem_ld_wait();
                fence_before_sync();
                pipe_sync(pp);   // round b - 1's rows are read: refill the Q tile
                fill_q(b);
                cp_async_wait_all();
                fence_async_smem();
                fence_before_sync();
                pipe_sync(pp);
                if (wl == 2 && lane == 0) {
                    fence_after_sync();
                    issue_gemm3(tmem, TB + 128, qt, Hs);
                    mma_commit(g3_bar);
                }
                if (wl == 2) __syncwarp();
                if (wl == 3 && !mbar_wait(g3_bar, g3_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 31);
                g3_phase ^= 1;
                fence_before_sync();
                pipe_sync(pp);
                fence_after_sync();
                epi3(b);
            }
            // epilogue 3's TMEM reads are done: the [z | z'] columns are free for
            // the next tile's GEMM1 (issued by warp 5, an epilogue-3 warp that
            // does no prep, after its epilogue 2)
            if (q < 2 && wl != 5) {
                fence_before_sync();
                cols_free_arrive(pp, 128);
            }
            // the H tile is free: the next tile's [E; E'] tile and edge arrays
            // arrive while epilogue 2 runs
            const bool more = k + 1 < ntl && !abort_now;
            if (more) {
                fetch(sbn, t0 + PN, min(PN, e1 - t0 - PN));
                if (tp == 32) {
                    mbar_expect_tx(e_bar, ET_BYTES);
                    bulk_g2s(Es, etiles + (size_t)(k + 1) * ET_BYTES, ET_BYTES, e_bar);
                    ++e_issued;
                }
            }
            if (wl == 1) __syncwarp();
            {   // epilogue 2 over 4-edge blocks, the next block's gathers in flight
                // (compiled once per warp half: hc is std::integral_constant<int, hh>)
                auto process4 = [&](auto hc, const float (&tb0)[4], const float (&tb1)[4], const float (&xb0)[4],
                                    const float (&xb1)[4], float rn0, float rn1, int col, float* pv) {
                    constexpr int HH = decltype(hc)::value;
                    float fa[4], da[4], f1[4], d1[4];
                    if (HH == 0) {
                        tmem_ld4(lane_base + TB + col, fa);        // phi_s (bias included)
                        tmem_ld4(lane_base + TB + PN + col, da);   // dphi_s / dd
                    }
                    tmem_ld4(lane_base + TB + 64 + col, f1);       // phi_v1
                    tmem_ld4(lane_base + TB + 64 + PN + col, d1);
                    const uint32_t m = (chw >> col) & 0xFu;
                    tmem_ld_wait();
                    if (HH != 0) {
#pragma unroll
                        for (int i = 0; i < 4; ++i) fa[i] = f1[i];
                    }
                    // this thread's share of dE/dd of edge i (sender features and
                    // phi_s', phi_v1'), given the receiver's dE/dXt rows t0, t1;
                    // the same expressions on both branches below (a block's branch
                    // depends on where the tile starts)
                    float r0 = cr0, r1 = cr1;   // the current receiver's dE/dXt rows
                    auto edge_term = [&](int i, float t0, float t1) {
                        if (HH == 0) pv[i] = fmaf(t0 * xb0[i], da[i], t1 * xb1[i] * d1[i]);
                        else pv[i] = fmaf(t0, xb0[i], t1 * xb1[i]) * d1[i];
                    };
                    if (m == 0) {   // one receiver for the whole block, no sum finishes here
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            acc0 = fmaf(tb0[i], fa[i], acc0);
                            acc1 = fmaf(tb1[i], f1[i], acc1);
                            edge_term(i, r0, r1);
                        }
                    } else {   // a receiver starts in this block: store the finished sums
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            if (m & (1u << i)) {
                                if (a.write_nodes) {
                                    out[(int64_t)cur * 4 * H] = r0 + acc0;
                                    out[(int64_t)cur * 4 * H + H] = r1 + acc1;
                                }
                                cur = rcv_s[col + i];
                                acc0 = 0.f;
                                acc1 = 0.f;
                                if (i > 0) {
                                    const float2 r = __ldg(xtb + roff[col + i]);
                                    r0 = r.x;
                                    r1 = r.y;
                                } else {   // edge 0's receiver rows came with the gathers
                                    r0 = rn0;
                                    r1 = rn1;
                                }
                            }
                            acc0 = fmaf(tb0[i], fa[i], acc0);
                            acc1 = fmaf(tb1[i], f1[i], acc1);
                            edge_term(i, r0, r1);
                        }
                    }
                    cr0 = r0;
                    cr1 = r1;
                };
                // the shares of dE/dd of blocks col and col + 4 are reduced
                // across lanes together (9 shuffles for 8 edges); a missing
                // second block (padding edges, never read) contributes zeros
                auto blocks = [&](auto hc) {
                    for (int col = 0; col < n; col += 8) {   // blocks col and col + 4 are in flight
                        float pv[8];
                        process4(hc, tba0, tba1, xba0, xba1, ra0, ra1, col, pv);
                        if (col + 4 < n) {
                            if (col + 8 < n) gather4(tba0, tba1, xba0, xba1, ra0, ra1, col + 8);
                            process4(hc, tbb0, tbb1, xbb0, xbb1, rb0, rb1, col + 4, pv + 4);
                            if (col + 12 < n) gather4(tbb0, tbb1, xbb0, xbb1, rb0, rb1, col + 12);
                        } else {
#pragma unroll
                            for (int i = 4; i < 8; ++i) pv[i] = 0.f;
                        }
                        const float s8 = warp_reduce_scatter8(pv, lane);
                        if ((lane & 3) == 0) red[wl * PN + col + rs8_idx] = s8;
                    }
                };
                if (hh == 0) blocks(std::integral_constant<int, 0>{});
                else blocks(std::integral_constant<int, 1>{});
            }
            if (wl == 5) {   // the next tile's GEMM1, once epilogue 3's warps are through
                fence_before_sync();
                cols_free_sync(pp, 128);
                if (more && lane == 0) issue_gemm1();
                __syncwarp();
            }
            if (more && tp < PN) {   // the next tile's prep, by the warp that fetched it
                cp_async_wait_all();
                __syncwarp();
                prep(sbn, min(PN, e1 - t0 - PN), rcv_s[PN - 1]);
            }
            fence_before_sync();
            pipe_sync(pp);
            // per-edge sums, fixed order, by the pipeline's last warp (the next
            // tile's GEMM1 is already running): dE/dd = the 8 warps' shares +
            // the three u terms; dE/du from epilogue 3
            const int te = tp - (PT - 32);
            if (te >= 0 && te < n) {
                float dd = 0.f;
#pragma unroll
                for (int ww = 0; ww < 8; ++ww) dd += red[ww * PN + te];
                dd += (red[R_RED_DDU + te] + red[R_RED_DDU + PN + te]) + red[R_RED_DDU + 2 * PN + te];
                float4 ea = a.eacc_init ? make_float4(0.f, 0.f, 0.f, 0.f)
                                        : reinterpret_cast<const float4*>(sb + R_SB_EACC)[te];
                ea.x += dd;
                ea.y += red[R_RED_DU + te];
                ea.z += red[R_RED_DU + PN + te];
                ea.w += red[R_RED_DU + 2 * PN + te];
                a.eacc[t0 + te] = ea;
            }
            if (abort_now) {
                aborted = true;
                break;
            }
        }
        if (!aborted && a.write_nodes) {
            out[(int64_t)cur * 4 * H] = cr0 + acc0;
            out[(int64_t)cur * 4 * H + H] = cr1 + acc1;
        }
    }
    // drain: every MMA and copy this CTA issued must be complete before it
    // frees its tensor memory and exits (after a timed-out wait the work it
    // waited for may still be running).  A wait on the parity of the phase
    // before the current one returns at once, so these also hold when
    // nothing was issued.
    __syncthreads();
    if (tp == 0) {
        if (!mbar_wait(mma_bar, mma_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 13);
        if (!mbar_wait(g2_bar, g2_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 15);
        if (!mbar_wait(g3_bar, g3_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 32);
    }
    if (tp == 32) {
        if (t == 32 && !mbar_wait(w2h_bar, 0, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 17);
        if (e_issued > 0 && !mbar_wait(e_bar, (e_issued - 1) & 1, WAIT_BUDGET))
            set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 19);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 512);
}

static int tc_grid(int nparts) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 152;
    }
    return std::max(1, std::min(sms, nparts));
}

int launch_edge_fwd_tc(const EdgeArgs& a, int layer, cudaStream_t st) {
    (void)layer;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(edge_fwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, Q_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "edge_fwd_tc smem attribute");
    const unsigned char* w1 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w1_bf);
    const unsigned char* w2 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w2_bf);
    // two pipelines (partitions) per CTA
    MLFF_LAUNCH_PDL("edge_fwd_tc", edge_fwd_tc_kernel, tc_grid((a.nparts + 1) / 2), NT, Q_SMEM, st, a, w1, w2);
    return MLFF_OK;
}

int launch_edge_bwd_tc(const EdgeArgs& a, int layer, cudaStream_t st) {
    (void)layer;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(edge_bwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, R_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "edge_bwd_tc smem attribute");
    const unsigned char* w1 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w1_bf);
    const unsigned char* w2 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w2_bf);
    // two pipelines (partitions) per CTA
    MLFF_LAUNCH_PDL("edge_bwd_tc", edge_bwd_tc_kernel, tc_grid((a.nparts + 1) / 2), NT, R_SMEM, st, a, w1, w2);
    return MLFF_OK;
}

int launch_vq(const float* P, const LayerOffsets& lo, const float* xtbar, int n_atoms, unsigned char* qs, float* qb,
              Status* st_word, cudaStream_t st) {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(vq_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, VQ_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "vq_tc smem attribute");
    const int tiles = (n_atoms + VQ_TA - 1) / VQ_TA;
    const int grid = std::max(1, std::min(tiles, 2 * num_sms()));
    MLFF_LAUNCH_PDL("vq_tc", vq_tc_kernel, grid, VQ_NT, VQ_SMEM, st, P, lo, xtbar, n_atoms, qs, qb, st_word);
    return MLFF_OK;
}

}  // namespace mlff
