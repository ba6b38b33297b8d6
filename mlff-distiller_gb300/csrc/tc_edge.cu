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
//   * the E tiles (RBF x cutoff, split fp16) are computed once per call for
//     all layers and bulk-copied per edge tile; per-tile edge arrays are
//     fetched with cp.async while the previous tile's epilogue runs;
//   * GEMM2's three 128-channel chunks are issued by three threads: a thread
//     stalls on tcgen05.mma issue while the tensor core is busy (about one
//     MMA per 50 cycles from one thread), three keep it saturated;
//   * every wait is bounded (clock64 budget); on expiry the kernel records
//     MLFF_ERR_TIMEOUT, drains its own copies, frees TMEM and returns.
//
// TMEM (512 columns): [0,128) lo halves of W2 chunks 0 and 1; [128,512) the
// GEMM2 accumulators (forward: 128-edge tiles, chunk g at 128 + 128 g;
// reverse: 64-edge tiles with [f | f'] per chunk, f' = df/dd in forward
// mode); GEMM1's output aliases one chunk until epilogue 1 has read it:
// chunk 0 in the forward kernel (read by the scalar warps only, so the next
// tile's GEMM1 is issued while the vector warps finish epilogue 2), chunk 2
// ([z; z']) in the reverse kernel.
#include <cuda_fp16.h>
#include <mutex>
#include "common.cuh"
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
// as MMA A operands (chunk g, K-step s at 64 g + 8 s); [128,512) the GEMM2
// accumulators, chunk g at 128 + 128 g; GEMM1 writes z into the columns
// of chunk 0 (forward) or 2 (reverse, TM_Z), which epilogue 1 reads before
// it refills them with the bias.
constexpr uint32_t TM_W2LO = 0;
constexpr uint32_t TM_F = 128;
constexpr uint32_t TM_Z = 384;

// ------------------------------------------------------------- packing
// W1 [H][RMAX] -> 2 K-step blocks (hi, lo); W2 [3H][H] -> 24 hi tiles
// followed by the 24 matching lo tiles.
__global__ void pack_tc_kernel(const float* __restrict__ w1, const float* __restrict__ w2,
                               unsigned char* __restrict__ w1_out, unsigned char* __restrict__ w2_out,
                               uint32_t* __restrict__ w2_tm) {
    const int stride = gridDim.x * blockDim.x;
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
                                           reinterpret_cast<uint32_t*>(out + L.w2_tm));
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

// Barrier 1 over the first n threads (whole warps) of the CTA.
__device__ __forceinline__ void bar_sync_first(int n) { asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory"); }

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
// The RBF x cutoff rows of every edge tile as split fp16 in the K-major
// no-swizzle layout (16-byte core matrices: K-step s at 4096 s, its second 8
// columns 2048 further, 8-row groups 128 apart; the hi image, then the lo
// image 8 KB later), computed once per call for all layers: forward tiles of
// 128 edges, reverse tiles of 64 edges with the d-derivative rows 64-127.
// Tiles follow the receiver partitions, so tile k of partition p is the k-th
// tile its CTA processes.
constexpr uint32_t ET_BYTES = 16384, ET_HALF = 8192;
__device__ __forceinline__ uint32_t et_off(int row, int k) {
    return (uint32_t)((k >> 4) * 4096 + ((k >> 3) & 1) * 2048 + (row >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// tile counts of all partitions, then an exclusive scan (one block, the
// partitions taken 1024 at a time)
__global__ void __launch_bounds__(1024) etile_index_kernel(const int32_t* __restrict__ row_ptr,
                                                           const int32_t* __restrict__ part, int P,
                                                           int32_t* __restrict__ base) {
    pdl_wait();
    pdl_trigger();
    __shared__ int cf[1024], cb[1024];
    __shared__ int carry[2];
    const int t = threadIdx.x;
    if (t == 0) carry[0] = carry[1] = 0;
    __syncthreads();
    for (int p0 = 0; p0 < P; p0 += 1024) {
        const int p = p0 + t;
        int nf = 0, nb = 0;
        if (p < P) {
            const int E = row_ptr[part[p + 1]] - row_ptr[part[p]];
            nf = (E + 127) / 128;
            nb = (E + 63) / 64;
        }
        cf[t] = nf;
        cb[t] = nb;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {   // inclusive scan (Hillis-Steele)
            const int xf = t >= o ? cf[t - o] : 0, xb = t >= o ? cb[t - o] : 0;
            __syncthreads();
            cf[t] += xf;
            cb[t] += xb;
            __syncthreads();
        }
        if (p < P) {
            base[p] = carry[0] + cf[t] - nf;
            base[P + 1 + p] = carry[1] + cb[t] - nb;
        }
        __syncthreads();
        if (t == 1023) {
            carry[0] += cf[1023];
            carry[1] += cb[1023];
        }
        __syncthreads();
    }
    if (t == 0) {
        base[P] = carry[0];
        base[2 * P + 1] = carry[1];
    }
}

template <bool REV>
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
    constexpr int TN = REV ? 64 : 128;
    const int t = threadIdx.x;
    const int row = t & (TN - 1), s = (t / TN) & 1, which = REV ? (t >> 7) : 0;
    for (int p = blockIdx.x; p < a.nparts; p += gridDim.x) {
        const int e0 = a.row_ptr[a.part[p]], e1 = a.row_ptr[a.part[p + 1]];
        const int b0 = base[(REV ? a.nparts + 1 : 0) + p];
        for (int k = blockIdx.y; e0 + k * TN < e1; k += gridDim.y) {
            const int e = e0 + k * TN + row;
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
            const int trow = which * 64 + row;
            *reinterpret_cast<uint4*>(tile + et_off(trow, 16 * s)) = *reinterpret_cast<const uint4*>(&hi[0]);
            *reinterpret_cast<uint4*>(tile + et_off(trow, 16 * s + 8)) = *reinterpret_cast<const uint4*>(&hi[4]);
            *reinterpret_cast<uint4*>(tile + ET_HALF + et_off(trow, 16 * s)) = *reinterpret_cast<const uint4*>(&lo[0]);
            *reinterpret_cast<uint4*>(tile + ET_HALF + et_off(trow, 16 * s + 8)) = *reinterpret_cast<const uint4*>(&lo[4]);
        }
    }
}

int launch_etiles(const EdgeArgs& a, int32_t* base, unsigned char* fwd, unsigned char* rev, cudaStream_t st) {
    MLFF_LAUNCH_PDL("etile_index", etile_index_kernel, 1, 1024, 0, st, a.row_ptr, a.part, a.nparts, base);
    // tiles of a partition spread over gridDim.y blocks
    MLFF_LAUNCH_PDL("etile_fill_fwd", etile_fill_kernel<false>, dim3(a.nparts, 16), 256, 0, st, a, base, fwd);
    if (rev) {
        MLFF_LAUNCH_PDL("etile_fill_rev", etile_fill_kernel<true>, dim3(a.nparts, 32), 256, 0, st, a, base, rev);
    }
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
    soff[e] = src_s[e] * 4 * H;
    if (roff) roff[e] = max(ra, 0) * 4 * H;
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

// Chunk g of GEMM2 for one 128-row B tile: D (TMEM columns 128 + 128 g) +=
// W2[g] B^T with B the split-fp16 tile at Hs (hi half, then lo half HALF128
// bytes later).  Per K-step: the resident hi tile times both halves of B,
// then the lo tile (TMEM for chunks 0 and 1, shared memory for chunk 2)
// times the hi half.  Every MMA accumulates (the epilogue filled TMEM with
// the bias).  The three chunks are issued by three threads in parallel: a
// thread issues about one MMA per 50 cycles and stalls while the tensor core
// is busy, so one issuer adds its own latency to every MMA; each chunk keeps
// a fixed accumulation order.
constexpr uint32_t HALF128 = 2 * b_block(128);   // K = 128: two K-blocks
__device__ __forceinline__ void issue_gemm2_chunk(int g, uint32_t tmem, const unsigned char* w2h,
                                                  const unsigned char* w2l, const unsigned char* Hs) {
    constexpr uint32_t idesc = idesc_f16(128);
    constexpr uint64_t DA = A_TILE >> 4, DH = HALF128 >> 4;
    const uint64_t a_hi = sdesc(smem_u32(w2h), A_LBO, A_SBO) + (uint64_t)(8 * g) * DA;
    const uint64_t a_lo = sdesc(smem_u32(w2l), A_LBO, A_SBO);
    const uint64_t b0 = sdesc_b(smem_u32(Hs));
    const uint32_t d = tmem + TM_F + 128 * g;
#pragma unroll 1
    for (int s = 0; s < 8; ++s) {
        const uint64_t bh = b0 + (uint64_t)(b_kstep_off(128, s) >> 4);
        const uint64_t ah = a_hi + (uint64_t)s * DA;
        mma_f16(d, ah, bh, idesc, 1);
        mma_f16(d, ah, bh + DH, idesc, 1);
        if (g < 2) mma_f16_ts(d, tmem + TM_W2LO + 64 * g + 8 * s, bh, idesc, 1);
        else mma_f16(d, a_lo + (uint64_t)s * DA, bh, idesc, 1);
    }
}

// out = base + (sum over the receiver's edges): receivers in [j0, j1)
// without edges get the base row (the epilogues store base + sum once per
// receiver that has edges).
__device__ __forceinline__ void zero_empty_rows(float* out, const int32_t* row_ptr, int j0, int j1, int w, int lane) {
    for (int j = j0 + w; j < j1; j += NT / 32)
        if (row_ptr[j] == row_ptr[j + 1])
            for (int k = lane; k < 4 * H; k += 32) out[(int64_t)j * 4 * H + k] = 0.0f;
}
__device__ __forceinline__ void copy_empty_rows(float* out, const float* base, const int32_t* row_ptr, int j0, int j1,
                                                int w, int lane) {
    for (int j = j0 + w; j < j1; j += NT / 32)
        if (row_ptr[j] == row_ptr[j + 1])
            for (int k = lane; k < 4 * H; k += 32) out[(int64_t)j * 4 * H + k] = base[(int64_t)j * 4 * H + k];
}

// ------------------------------------------------------- forward kernel
constexpr int FN = 128;                                   // edges per tile
constexpr uint32_t F_HH = 2 * b_block(FN);                // H tile, one half (K = 128)
static_assert(F_HH == HALF128, "GEMM2 B layout");
constexpr uint32_t F_OFF_W1 = 0;
constexpr uint32_t F_OFF_W2H = F_OFF_W1 + W1_BYTES;
constexpr uint32_t F_OFF_H = align1k(F_OFF_W2H + W2_HALF);     // H tile; the E tile shares its start
constexpr uint32_t F_OFF_W2L = align1k(F_OFF_H + 2 * F_HH);
// per-tile edge arrays, two buffers: (u, d), sender, receiver, sender row
// offset, u components, receiver-change bits
constexpr uint32_t F_SB_US = 0;
constexpr uint32_t F_SB_SRC = F_SB_US + FN * 16;
constexpr uint32_t F_SB_RCV = F_SB_SRC + FN * 4;
constexpr uint32_t F_SB_SOFF = F_SB_RCV + FN * 4;
constexpr uint32_t F_SB_UC = F_SB_SOFF + FN * 4;
constexpr uint32_t F_SB_CHG = F_SB_UC + 3 * FN * 4;
constexpr uint32_t F_SB_BYTES = F_SB_CHG + (FN / 32) * 4;
constexpr uint32_t F_OFF_SB = F_OFF_W2L + W2L_BYTES;
constexpr uint32_t F_OFF_B1 = F_OFF_SB + 2 * F_SB_BYTES;
constexpr uint32_t F_OFF_B2 = F_OFF_B1 + H * 4;
constexpr uint32_t F_OFF_BAR = F_OFF_B2 + H3 * 4;
constexpr uint32_t F_OFF_MISC = F_OFF_BAR + 8 * 5;
constexpr uint32_t F_SMEM = align1k(F_OFF_MISC + 16);
static_assert(ET_BYTES <= 2 * F_HH, "E tile fits in the H tile's space");
static_assert(F_SMEM <= 232448, "forward kernel shared memory");

// 16 warps.  Epilogue roles: warp w reads TMEM lane quarter q = w % 4
// (channels / hidden units 32q..32q+31); r = w / 4 selects the edge quarter
// (epilogue 1) or the feature component s, v_x, v_y, v_z (epilogue 2).
__global__ void __launch_bounds__(NT, 1) edge_fwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                            const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + F_OFF_W1;
    unsigned char* w2h = smem + F_OFF_W2H;
    unsigned char* Hs = smem + F_OFF_H;
    unsigned char* Es = smem + F_OFF_H;            // E tile (bulk-copied) lives in the H tile's space
    unsigned char* w2l = smem + F_OFF_W2L;        // resident lo tiles of W2 chunk 2
    float* b1s = reinterpret_cast<float*>(smem + F_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + F_OFF_B2);
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + F_OFF_BAR);
    uint64_t* w2h_bar = mma_bar + 1;
    uint64_t* e_bar = mma_bar + 2;
    uint64_t* g2_bar = mma_bar + 3;                 // GEMM2: one commit per chunk issuer
    uint64_t* never_bar = mma_bar + 4;              // test hook: nothing arrives here
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + F_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + F_OFF_MISC + 4);

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
        mbar_init(mma_bar, 1);
        mbar_init(w2h_bar, 1);
        mbar_init(e_bar, 1);
        mbar_init(g2_bar, 3);
        mbar_init(never_bar, 1);
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

    uint32_t mma_phase = 0, g2_phase = 0;   // GEMM1 / GEMM2 barrier phases
    bool w2h_ready = false;                 // (GEMM2 issuers)
    if (t == 32) load_w2_resident(w2h, w2l, w2g, w2h_bar);

    const int q = w & 3, r = w >> 2;
    const int c = 32 * q + lane;
    const int fidx = r * H + c;                      // this thread's feature element in a [4][H] row
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    load_w2_lo_tmem(lane_base, reinterpret_cast<const uint32_t*>(a.P + a.lo.w2_tm), r, c);
    tmem_st_wait();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    pdl_trigger();   // after the TMEM allocation

    bool aborted = false;
    uint32_t e_phase = 0, e_issued = 0;   // E-tile copies: barrier phase, copies issued (thread 32)
    // GEMM1: z^T = W1 e^T on the bulk-copied E tile, into chunk 0's columns
    auto issue_gemm1 = [&]() {
        if (!mbar_wait(e_bar, e_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 8);
        fence_after_sync();
        constexpr uint32_t idesc = idesc_f16(FN);
#pragma unroll
        for (int s = 0; s < 2; ++s)
#pragma unroll
            for (int pr = 0; pr < 3; ++pr) {
                const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                const uint64_t bd = sdesc(smem_u32(Es + bhl * ET_HALF + s * 4096), 2048, 128);
                mma_f16(tmem + TM_F, ad, bd, idesc, (s | pr) != 0);
            }
        mma_commit(mma_bar);
    };
    bool g1_issued = false;   // GEMM1 of the current tile already issued (at the end of the previous tile)
    for (int p = blockIdx.x; p < a.nparts && !aborted; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        const int ntl = (e1 - e0 + FN - 1) / FN;
        const unsigned char* etiles = a.etile + (size_t)a.etile_base[p] * ET_BYTES;
        copy_empty_rows(a.Xt, a.X, a.row_ptr, j0, j1, w, lane);
        int cur = j0;
        float acc = 0.f, accu = 0.f;   // x * phi and u * phi_v2 parts of the current receiver's sum
        // X of the current receiver (the residual term of Xt), loaded when the
        // receiver starts so that the load is long done when its sum is stored
        float base = a.X[(int64_t)cur * 4 * H + fidx];
        if (ntl > 0) {   // the partition's first tile: edge arrays and E tile
            unsigned char* sb = smem + F_OFF_SB;
            fetch_tile_edges(a, t, FN, e0, min(FN, e1 - e0), reinterpret_cast<float4*>(sb + F_SB_US),
                             reinterpret_cast<int*>(sb + F_SB_SRC), reinterpret_cast<int*>(sb + F_SB_RCV));
            if (t == 32) {
                mbar_expect_tx(e_bar, ET_BYTES);
                bulk_g2s(Es, etiles, ET_BYTES, e_bar);
                ++e_issued;
            }
            cp_async_wait_all();
            __syncthreads();
            if (t < FN)
                tile_prep<FN>(t, min(FN, e1 - e0), j0, reinterpret_cast<int*>(sb + F_SB_SRC),
                              reinterpret_cast<int*>(sb + F_SB_RCV), reinterpret_cast<float4*>(sb + F_SB_US),
                              reinterpret_cast<int*>(sb + F_SB_SOFF), nullptr, reinterpret_cast<float*>(sb + F_SB_UC),
                              reinterpret_cast<uint32_t*>(sb + F_SB_CHG));
            __syncthreads();
        }
        for (int k = 0; k < ntl; ++k) {
            const int t0 = e0 + k * FN, n = min(FN, e1 - t0), buf = k & 1;
            unsigned char* sb = smem + F_OFF_SB + buf * F_SB_BYTES;
            unsigned char* sbn = smem + F_OFF_SB + (buf ^ 1) * F_SB_BYTES;
            const int* rcv_s = reinterpret_cast<const int*>(sb + F_SB_RCV);
            const int* soff = reinterpret_cast<const int*>(sb + F_SB_SOFF);
            const float* uc = reinterpret_cast<const float*>(sb + F_SB_UC);
            const uint32_t* chg = reinterpret_cast<const uint32_t*>(sb + F_SB_CHG);
            if (t == 0 && !g1_issued) issue_gemm1();
            g1_issued = false;
            e_phase ^= 1;
            if (w == 0) __syncwarp();
            // only warp 0 polls the MMA barrier; the others wait at the CTA
            // barrier instead of spinning on shared memory the MMAs read from
            if (w == 0 && (a.stall_test & 1) && k == 0 && !mbar_wait(never_bar, 0, STALL_BUDGET))
                signal_timeout(a, abort_flag, WHERE_STALL_TEST);
            if (w == 0 && !mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 1);
            mma_phase ^= 1;
            fence_before_sync();
            __syncthreads();
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1) -> H tile (split fp16), 32 edges per warp
                const int k = c, col = 32 * r;
                const float bias = b1s[k];
                float z[32];
                tmem_ld32(lane_base + TM_F + col, z);
                tmem_ld_wait();
                const BColumn hc(Hs, F_HH, FN, col, k);
#pragma unroll
                for (int i = 0; i < 32; i += 2) {
                    const float z0 = z[i] + bias, z1 = z[i + 1] + bias;
                    hc.put_pair(i, z0 * fast_sigmoid(z0), z1 * fast_sigmoid(z1));
                }
                // GEMM2 accumulates onto b2[g * 128 + channel]: this warp refills
                // the 32 chunk-0 cells it has just read, and 64 columns of
                // chunks 1 and 2 (warps r = 0, 1: chunk 1; r = 2, 3: chunk 2)
                float bv[16];
                const float b0c = b2s[c], b12 = b2s[(1 + (r >> 1)) * H + c];
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = b0c;
                tmem_st16(lane_base + TM_F + col, bv);
                tmem_st16(lane_base + TM_F + col + 16, bv);
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = b12;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) tmem_st16(lane_base + TM_F + 128 + 64 * r + 16 * kk, bv);
                tmem_st_wait();
            }
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            // epilogue 2's first two 16-edge blocks of sender features are
            // gathered while GEMM2 runs
            float xa[16], xn[16];
            auto gather16 = [&](float (&x)[16], int col) {
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    const int4 so = *reinterpret_cast<const int4*>(soff + col + i);
                    x[i] = col + i < n ? __ldg(a.X + so.x + fidx) : 0.f;
                    x[i + 1] = col + i + 1 < n ? __ldg(a.X + so.y + fidx) : 0.f;
                    x[i + 2] = col + i + 2 < n ? __ldg(a.X + so.z + fidx) : 0.f;
                    x[i + 3] = col + i + 3 < n ? __ldg(a.X + so.w + fidx) : 0.f;
                }
            };
            gather16(xa, 0);
            if (16 < n) gather16(xn, 16);
            if (w < 3 && lane == 0) {   // GEMM2: f^T = W2 h^T, chunk w issued by warp w
                fence_after_sync();
                if (!w2h_ready) {
                    if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) signal_timeout(a, abort_flag, 6);
                    w2h_ready = true;
                }
                issue_gemm2_chunk(w, tmem, w2h, w2l, Hs);
                mma_commit(g2_bar);
            }
            if (w < 3) __syncwarp();   // lanes 1-31 of the issuing warps wait here, not in a spin loop
            // only warp 0 polls the MMA barrier; the others wait at the CTA
            // barrier instead of spinning on shared memory the MMAs read from
            if (w == 0 && !mbar_wait(g2_bar, g2_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 4);
            g2_phase ^= 1;
            fence_before_sync();
            __syncthreads();
            fence_after_sync();
            // ... and the H tile is free: the next tile's E tile and edge arrays
            // arrive while epilogue 2 runs
            const bool more = k + 1 < ntl && !*abort_flag;
            if (more) {
                fetch_tile_edges(a, t, FN, t0 + FN, min(FN, e1 - t0 - FN), reinterpret_cast<float4*>(sbn + F_SB_US),
                                 reinterpret_cast<int*>(sbn + F_SB_SRC), reinterpret_cast<int*>(sbn + F_SB_RCV));
                if (t == 32) {
                    mbar_expect_tx(e_bar, ET_BYTES);
                    bulk_g2s(Es, etiles + (size_t)(k + 1) * ET_BYTES, ET_BYTES, e_bar);
                    ++e_issued;
                }
            }
            if (w == 1) __syncwarp();
            {   // epilogue 2: component r of the message sums, segmented by receiver;
                // 16-edge blocks, the next block's gathers in flight.  Padding
                // edges gather 0 (and have u = 0), so they add nothing.
                const float* ur = uc + (r == 0 ? 0 : (r - 1) * FN);
                const uint32_t f1col = r == 0 ? 128 : 256;
                float* out = a.Xt + fidx;          // Xt = X + message sum (student_model.py:359-385)
                const float* xin = a.X + fidx;
                auto process16 = [&](const float (&x)[16], int col) {
                    float f1[16], f2[16];
                    tmem_ld16(lane_base + f1col + col, f1);
                    if (r != 0) tmem_ld16(lane_base + 384 + col, f2);
                    const uint32_t mask = (chg[col >> 5] >> (col & 31)) & 0xFFFFu;
                    tmem_ld_wait();
                    const float* u = ur + col;
                    if (mask == 0) {
                        if (r == 0) {
#pragma unroll
                            for (int i = 0; i < 16; ++i) acc = fmaf(x[i], f1[i], acc);
                        } else {
#pragma unroll
                            for (int i = 0; i < 16; ++i) {
                                acc = fmaf(x[i], f1[i], acc);
                                accu = fmaf(u[i], f2[i], accu);
                            }
                        }
                    } else {   // a receiver changes in this block: flush its finished sum
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            if (mask & (1u << i)) {
                                out[(int64_t)cur * 4 * H] = base + (acc + accu);
                                cur = rcv_s[col + i];
                                base = xin[(int64_t)cur * 4 * H];
                                acc = 0.f;
                                accu = 0.f;
                            }
                            acc = fmaf(x[i], f1[i], acc);
                            if (r != 0) accu = fmaf(u[i], f2[i], accu);
                        }
                    }
                };
                for (int col = 0; col < n; col += 32) {   // blocks col and col + 16 are in flight
                    process16(xa, col);
                    if (col + 16 >= n) break;
                    if (col + 32 < n) gather16(xa, col + 32);
                    process16(xn, col + 16);
                    if (col + 48 < n) gather16(xn, col + 48);
                }
            }
            // chunk 0 is read by the scalar warps only (r = 0, warps 0-3): once
            // all four are through epilogue 2, the next tile's GEMM1 can write z
            // there while the vector warps finish
            if (more && r == 0) {
                tmem_ld_wait();
                fence_before_sync();
                bar_sync_first(4 * 32);
                if (t == 0) issue_gemm1();
            }
            g1_issued = more;
            cp_async_wait_all();
            fence_before_sync();
            __syncthreads();
            if (*abort_flag) {
                aborted = true;
                break;
            }
            if (more && t < FN)
                tile_prep<FN>(t, min(FN, e1 - t0 - FN), rcv_s[FN - 1], reinterpret_cast<int*>(sbn + F_SB_SRC),
                              reinterpret_cast<int*>(sbn + F_SB_RCV), reinterpret_cast<float4*>(sbn + F_SB_US),
                              reinterpret_cast<int*>(sbn + F_SB_SOFF), nullptr, reinterpret_cast<float*>(sbn + F_SB_UC),
                              reinterpret_cast<uint32_t*>(sbn + F_SB_CHG));
        }
        if (!aborted) a.Xt[(int64_t)cur * 4 * H + fidx] = base + (acc + accu);
    }
    // drain: the resident-weight load, any E-tile copy and a GEMM1 issued
    // for a tile that never ran (abort) must be complete before the CTA exits
    __syncthreads();
    // the last GEMM1 and GEMM2 committed must be complete: a GEMM1 issued for
    // a tile that never ran (abort), or MMAs whose wait timed out.  A wait on
    // the parity of the phase before the current one returns at once, so
    // these also hold when nothing was committed.
    if (t == 0 && !mbar_wait(mma_bar, g1_issued ? mma_phase : (mma_phase ^ 1), WAIT_BUDGET))
        set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 3);
    if (t == 0 && !mbar_wait(g2_bar, g2_phase ^ 1, WAIT_BUDGET))
        set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 5);
    if (t == 32) {
        if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 7);
        // an E-tile copy issued for a tile that never ran (abort) must land first
        if (e_issued > 0 && !mbar_wait(e_bar, (e_issued - 1) & 1, WAIT_BUDGET))
            set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 9);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------- reverse kernel
// 64-edge tiles; E and E' (and then H and H') are stacked as rows 0-63 and
// 64-127 of one 128-row B tile, so every MMA is N = 128: TMEM columns
// [0,64) z^T, [64,128) z'^T, and per chunk g at 128 + 128 g: [0,64) f^T,
// [64,128) f'^T.
constexpr int BN = 64;
constexpr uint32_t B_HH = 2 * b_block(2 * BN);
static_assert(B_HH == HALF128, "GEMM2 B layout");
constexpr uint32_t B_OFF_W1 = 0;
constexpr uint32_t B_OFF_W2H = B_OFF_W1 + W1_BYTES;
constexpr uint32_t B_OFF_H = align1k(B_OFF_W2H + W2_HALF);     // [H; H'] tile; the [E; E'] tile shares its start
constexpr uint32_t B_OFF_W2L = align1k(B_OFF_H + 2 * B_HH);
constexpr uint32_t B_SB_US = 0;
constexpr uint32_t B_SB_SRC = B_SB_US + BN * 16;
constexpr uint32_t B_SB_RCV = B_SB_SRC + BN * 4;
constexpr uint32_t B_SB_SOFF = B_SB_RCV + BN * 4;
constexpr uint32_t B_SB_ROFF = B_SB_SOFF + BN * 4;
constexpr uint32_t B_SB_UC = B_SB_ROFF + BN * 4;
constexpr uint32_t B_SB_CHG = B_SB_UC + 3 * BN * 4;
constexpr uint32_t B_SB_EACC = B_SB_CHG + 16;
constexpr uint32_t B_SB_BYTES = B_SB_EACC + BN * 16;
constexpr uint32_t B_OFF_SB = B_OFF_W2L + W2L_BYTES;
constexpr uint32_t B_OFF_B1 = B_OFF_SB + 2 * B_SB_BYTES;
constexpr uint32_t B_OFF_B2 = B_OFF_B1 + H * 4;
constexpr uint32_t B_OFF_RED = B_OFF_B2 + H3 * 4;
constexpr uint32_t B_OFF_BAR = B_OFF_RED + 16 * BN * 2 * 4;
constexpr uint32_t B_OFF_MISC = B_OFF_BAR + 8 * 5;
constexpr uint32_t B_SMEM = align1k(B_OFF_MISC + 16);
static_assert(ET_BYTES <= 2 * B_HH, "E tile fits in the H tile's space");
static_assert(B_SMEM <= 232448, "reverse kernel shared memory");

__global__ void __launch_bounds__(NT, 1) edge_bwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                            const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + B_OFF_W1;
    unsigned char* w2h = smem + B_OFF_W2H;
    unsigned char* Hs = smem + B_OFF_H;            // [H; H'] hi, then lo
    unsigned char* Es = smem + B_OFF_H;            // [E; E'] tile (bulk-copied), before H is written
    unsigned char* w2l = smem + B_OFF_W2L;        // resident lo tiles of W2 chunk 2
    float* b1s = reinterpret_cast<float*>(smem + B_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + B_OFF_B2);
    float* red = reinterpret_cast<float*>(smem + B_OFF_RED);   // [16 warps][BN][2]
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + B_OFF_BAR);
    uint64_t* w2h_bar = mma_bar + 1;
    uint64_t* e_bar = mma_bar + 2;
    uint64_t* g2_bar = mma_bar + 3;                 // GEMM2: one commit per chunk issuer
    uint64_t* never_bar = mma_bar + 4;              // test hook: nothing arrives here
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + B_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + B_OFF_MISC + 4);

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
        mbar_init(mma_bar, 1);
        mbar_init(w2h_bar, 1);
        mbar_init(e_bar, 1);
        mbar_init(g2_bar, 3);
        mbar_init(never_bar, 1);
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

    uint32_t mma_phase = 0, g2_phase = 0;   // GEMM1 / GEMM2 barrier phases
    bool w2h_ready = false;                 // (GEMM2 issuers)
    if (t == 32) load_w2_resident(w2h, w2l, w2g, w2h_bar);
    const int q = w & 3, r = w >> 2;
    const int c = 32 * q + lane;
    const int fidx = r * H + c;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    load_w2_lo_tmem(lane_base, reinterpret_cast<const uint32_t*>(a.P + a.lo.w2_tm), r, c);
    tmem_st_wait();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    pdl_trigger();   // after the TMEM allocation
    const int rs_idx = reduce_scatter8_index(lane);

    bool aborted = false;
    uint32_t e_phase = 0, e_issued = 0;   // E-tile copies: barrier phase, copies issued (thread 32)
    auto prep = [&](unsigned char* sbx, int nn, int prev) {
        if (t < BN)
            tile_prep<BN>(t, nn, prev, reinterpret_cast<int*>(sbx + B_SB_SRC), reinterpret_cast<int*>(sbx + B_SB_RCV),
                          reinterpret_cast<float4*>(sbx + B_SB_US), reinterpret_cast<int*>(sbx + B_SB_SOFF),
                          reinterpret_cast<int*>(sbx + B_SB_ROFF), reinterpret_cast<float*>(sbx + B_SB_UC),
                          reinterpret_cast<uint32_t*>(sbx + B_SB_CHG));
    };
    for (int p = blockIdx.x; p < a.nparts && !aborted; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        const int ntl = (e1 - e0 + BN - 1) / BN;
        const unsigned char* etiles = a.etile + (size_t)a.etile_base[p] * ET_BYTES;
        if (a.write_nodes) zero_empty_rows(a.xbar, a.row_ptr, j0, j1, w, lane);
        int cur = j0;
        float acc = 0.f;
        if (ntl > 0) {   // the partition's first tile: edge arrays and [E; E'] tile
            unsigned char* sb = smem + B_OFF_SB;
            fetch_tile_edges(a, t, BN, e0, min(BN, e1 - e0), reinterpret_cast<float4*>(sb + B_SB_US),
                             reinterpret_cast<int*>(sb + B_SB_SRC), reinterpret_cast<int*>(sb + B_SB_RCV),
                             a.eacc_init ? nullptr : reinterpret_cast<float4*>(sb + B_SB_EACC));
            if (t == 32) {
                mbar_expect_tx(e_bar, ET_BYTES);
                bulk_g2s(Es, etiles, ET_BYTES, e_bar);
                ++e_issued;
            }
            cp_async_wait_all();
            __syncthreads();
            prep(sb, min(BN, e1 - e0), j0);
            __syncthreads();
        }
        for (int k = 0; k < ntl; ++k) {
            const int t0 = e0 + k * BN, n = min(BN, e1 - t0), buf = k & 1;
            unsigned char* sb = smem + B_OFF_SB + buf * B_SB_BYTES;
            unsigned char* sbn = smem + B_OFF_SB + (buf ^ 1) * B_SB_BYTES;
            const int* rcv_s = reinterpret_cast<const int*>(sb + B_SB_RCV);
            const int* soff = reinterpret_cast<const int*>(sb + B_SB_SOFF);
            const int* roff = reinterpret_cast<const int*>(sb + B_SB_ROFF);
            const float* uc = reinterpret_cast<const float*>(sb + B_SB_UC);
            const uint32_t* chg = reinterpret_cast<const uint32_t*>(sb + B_SB_CHG);
            if (t == 0) {   // [z; z']^T = W1 [e; e']^T on the bulk-copied tile
                if (!mbar_wait(e_bar, e_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 18);
                fence_after_sync();
                constexpr uint32_t idesc = idesc_f16(2 * BN);
#pragma unroll
                for (int s = 0; s < 2; ++s)
#pragma unroll
                    for (int pr = 0; pr < 3; ++pr) {
                        const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                        const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                        const uint64_t bd = sdesc(smem_u32(Es + bhl * ET_HALF + s * 4096), 2048, 128);
                        mma_f16(tmem + TM_Z, ad, bd, idesc, (s | pr) != 0);
                    }
                mma_commit(mma_bar);
            }
            e_phase ^= 1;
            if (w == 0) __syncwarp();
            // only warp 0 polls the MMA barrier; the others wait at the CTA
            // barrier instead of spinning on shared memory the MMAs read from
            if (w == 0 && (a.stall_test & 2) && k == 0 && !mbar_wait(never_bar, 0, STALL_BUDGET))
                signal_timeout(a, abort_flag, WHERE_STALL_TEST);
            if (w == 0 && !mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 11);
            mma_phase ^= 1;
            fence_before_sync();
            __syncthreads();
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1) (rows 0-63), h' = silu'(z + b1) z'
                // (rows 64-127), 16 edges per warp
                const int k = c, col = 16 * r;
                const float bias = b1s[k];
                float z[16], zd[16];
                tmem_ld16(lane_base + TM_Z + col, z);
                tmem_ld16(lane_base + TM_Z + BN + col, zd);
                tmem_ld_wait();
                const BColumn hc(Hs, B_HH, 2 * BN, col, k), hdc(Hs, B_HH, 2 * BN, BN + col, k);
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const float z0 = z[i] + bias, z1 = z[i + 1] + bias;
                    const float s0 = fast_sigmoid(z0), s1 = fast_sigmoid(z1);
                    hc.put_pair(i, z0 * s0, z1 * s1);
                    hdc.put_pair(i, s0 * (1.0f + z0 * (1.0f - s0)) * zd[i], s1 * (1.0f + z1 * (1.0f - s1)) * zd[i + 1]);
                }
                // f = W2 h accumulates onto b2 and f' = W2 h' onto 0 (each chunk:
                // 64 columns f^T, then 64 columns f'^T).  This warp refills the
                // chunk-2 cells it has just read (f then f'), and 64 columns of
                // chunks 0 and 1: r = 0 chunk 0 f, 1 chunk 0 f', 2 chunk 1 f, 3 chunk 1 f'.
                float bv[16];
                const float b2c = b2s[2 * H + c];
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = b2c;
                tmem_st16(lane_base + TM_Z + col, bv);
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = 0.0f;
                tmem_st16(lane_base + TM_Z + BN + col, bv);
                const float b01 = (r & 1) ? 0.0f : b2s[(r >> 1) * H + c];
#pragma unroll
                for (int i = 0; i < 16; ++i) bv[i] = b01;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) tmem_st16(lane_base + TM_F + 64 * r + 16 * kk, bv);
                tmem_st_wait();
            }
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            // epilogue 2's first two 8-edge blocks of gathers are issued while GEMM2 runs
            float tba[8], xba[8], tra[8], tbn[8], xbn[8], trn[8];
            auto gather8 = [&](float (&tb)[8], float (&xb)[8], float (&tr)[8], int col) {
#pragma unroll
                for (int i = 0; i < 8; i += 4) {
                    const int4 so = *reinterpret_cast<const int4*>(soff + col + i);
                    const int4 ro = *reinterpret_cast<const int4*>(roff + col + i);
                    const int sv[4] = {so.x, so.y, so.z, so.w}, rv[4] = {ro.x, ro.y, ro.z, ro.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const bool ok = col + i + k < n;
                        tb[i + k] = ok ? __ldg(a.xtbar + sv[k] + fidx) : 0.f;
                        xb[i + k] = ok ? __ldg(a.X + sv[k] + fidx) : 0.f;
                        tr[i + k] = ok ? __ldg(a.xtbar + rv[k] + fidx) : 0.f;
                    }
                }
            };
            gather8(tba, xba, tra, 0);
            if (8 < n) gather8(tbn, xbn, trn, 8);
            if (w < 3 && lane == 0) {   // [f; f']^T = W2 [h; h']^T, chunk w issued by warp w
                fence_after_sync();
                if (!w2h_ready) {
                    if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) signal_timeout(a, abort_flag, 16);
                    w2h_ready = true;
                }
                issue_gemm2_chunk(w, tmem, w2h, w2l, Hs);
                mma_commit(g2_bar);
            }
            if (w < 3) __syncwarp();   // lanes 1-31 of the issuing warps wait here, not in a spin loop
            // only warp 0 polls the MMA barrier; the others wait at the CTA
            // barrier instead of spinning on shared memory the MMAs read from
            if (w == 0 && !mbar_wait(g2_bar, g2_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 14);
            g2_phase ^= 1;
            fence_before_sync();
            __syncthreads();
            fence_after_sync();
            // the H tile is free too: the next tile's [E; E'] tile and edge
            // arrays arrive while epilogue 2 runs
            const bool more = k + 1 < ntl && !*abort_flag;
            if (more) {
                fetch_tile_edges(a, t, BN, t0 + BN, min(BN, e1 - t0 - BN), reinterpret_cast<float4*>(sbn + B_SB_US),
                                 reinterpret_cast<int*>(sbn + B_SB_SRC), reinterpret_cast<int*>(sbn + B_SB_RCV),
                                 a.eacc_init ? nullptr : reinterpret_cast<float4*>(sbn + B_SB_EACC));
                if (t == 32) {
                    mbar_expect_tx(e_bar, ET_BYTES);
                    bulk_g2s(Es, etiles + (size_t)(k + 1) * ET_BYTES, ET_BYTES, e_bar);
                    ++e_issued;
                }
            }
            if (w == 1) __syncwarp();
            {   // epilogue 2: component r of the node adjoints (gathered from the
                // sender side, summed per receiver) and this component's share
                // of dE/dd, dE/du; 8-edge blocks, the next block's gathers in
                // flight.  Padding edges gather 0, so they add nothing.
                const uint32_t f1col = r == 0 ? 128 : 256, d1col = f1col + BN;
                const float* ur = uc + (r == 0 ? 0 : (r - 1) * BN);
                float* out = a.xbar + fidx;        // gathered adjoint; dE/dXt is added afterwards
                auto process8 = [&](const float (&tb)[8], const float (&xb)[8], const float (&tr)[8], int col) {
                    float f1[8], f2[8], d1[8], d2[8];
                    tmem_ld8(lane_base + f1col + col, f1);   // phi_s or phi_v1 (bias included)
                    tmem_ld8(lane_base + d1col + col, d1);   // its d-derivative
                    if (r != 0) {
                        tmem_ld8(lane_base + 384 + col, f2);       // phi_v2 (bias included)
                        tmem_ld8(lane_base + 384 + BN + col, d2);  // dphi_v2/dd
                    }
                    const uint32_t mask = (chg[col >> 5] >> (col & 31)) & 0xFFu;
                    tmem_ld_wait();
                    if (mask == 0) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) acc = fmaf(tb[i], f1[i], acc);
                    } else {   // a receiver changes in this block: flush its finished sum
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            if (mask & (1u << i)) {
                                if (a.write_nodes) out[(int64_t)cur * 4 * H] = acc;
                                cur = rcv_s[col + i];
                                acc = 0.f;
                            }
                            acc = fmaf(tb[i], f1[i], acc);
                        }
                    }
                    float p0[8], p1[8];
                    if (r == 0) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) p0[i] = (tr[i] * xb[i]) * d1[i];
                    } else {
                        const float* u = ur + col;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            p0[i] = tr[i] * fmaf(xb[i], d1[i], u[i] * d2[i]);
                            p1[i] = tr[i] * f2[i];
                        }
                    }
                    const float s0 = warp_reduce_scatter8(p0, lane);
                    float s1 = 0.f;
                    if (r != 0) s1 = warp_reduce_scatter8(p1, lane);
                    if ((lane & 3) == 0) {
                        float* rr = red + ((size_t)w * BN + col + rs_idx) * 2;
                        rr[0] = s0;
                        rr[1] = s1;
                    }
                };
                for (int col = 0; col < n; col += 16) {   // blocks col and col + 8 are in flight
                    process8(tba, xba, tra, col);
                    if (col + 8 >= n) break;
                    if (col + 16 < n) gather8(tba, xba, tra, col + 16);
                    process8(tbn, xbn, trn, col + 8);
                    if (col + 24 < n) gather8(tbn, xbn, trn, col + 24);
                }
            }
            if (more && t < BN) {   // the next tile's prep, by the two warps that fetched it
                cp_async_wait_all();
                bar_sync_first(BN);
                prep(sbn, min(BN, e1 - t0 - BN), rcv_s[BN - 1]);
            }
            fence_before_sync();
            __syncthreads();
            if (t < n) {
                float dd = 0.f, du[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int ww = 0; ww < 16; ++ww) {
                    const float* rr = red + ((size_t)ww * BN + t) * 2;
                    dd += rr[0];
                    if (ww >= 4) du[(ww >> 2) - 1] += rr[1];
                }
                float4 ea = a.eacc_init ? make_float4(0.f, 0.f, 0.f, 0.f)
                                        : reinterpret_cast<const float4*>(sb + B_SB_EACC)[t];
                ea.x += dd;
                ea.y += du[0];
                ea.z += du[1];
                ea.w += du[2];
                a.eacc[t0 + t] = ea;
            }
            if (*abort_flag) {
                aborted = true;
                break;
            }
        }
        if (!aborted && a.write_nodes) a.xbar[(int64_t)cur * 4 * H + fidx] = acc;
    }
    __syncthreads();
    // after a timed-out wait the MMAs it waited for may still be running: the
    // last GEMM1 and GEMM2 committed must be complete (a wait on the parity of
    // the phase before the current one returns at once, so this also holds
    // when nothing was committed)
    if (t == 0) {
        if (!mbar_wait(mma_bar, mma_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 13);
        if (!mbar_wait(g2_bar, g2_phase ^ 1, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 15);
    }
    if (t == 32) {
        if (!mbar_wait(w2h_bar, 0, WAIT_BUDGET)) set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 17);
        if (e_issued > 0 && !mbar_wait(e_bar, (e_issued - 1) & 1, WAIT_BUDGET))
            set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 19);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------- launchers
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
        attr_err = cudaFuncSetAttribute(edge_fwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "edge_fwd_tc smem attribute");
    const unsigned char* w1 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w1_bf);
    const unsigned char* w2 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w2_bf);
    MLFF_LAUNCH_PDL("edge_fwd_tc", edge_fwd_tc_kernel, tc_grid(a.nparts), NT, F_SMEM, st, a, w1, w2);
    return MLFF_OK;
}

int launch_edge_bwd_tc(const EdgeArgs& a, int layer, cudaStream_t st) {
    (void)layer;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(edge_bwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, B_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "edge_bwd_tc smem attribute");
    const unsigned char* w1 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w1_bf);
    const unsigned char* w2 = reinterpret_cast<const unsigned char*>(a.P + a.lo.w2_bf);
    MLFF_LAUNCH_PDL("edge_bwd_tc", edge_bwd_tc_kernel, tc_grid(a.nparts), NT, B_SMEM, st, a, w1, w2);
    return MLFF_OK;
}

}  // namespace mlff
