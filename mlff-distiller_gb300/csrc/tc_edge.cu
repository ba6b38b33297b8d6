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
//   * W1 (128 x 32) stays in shared memory; W2 (384 x 128) streams through
//     a ring of 8 KB hi/lo slabs filled by cp.async.bulk and recycled by
//     tcgen05.commit on per-slot mbarriers;
//   * every wait is bounded (clock64 budget); on expiry the kernel records
//     MLFF_ERR_TIMEOUT, drains its own copies, frees TMEM and returns.
//
// Forward: 128-edge tiles, TMEM columns [0,128) = z^T, [128,512) = f^T.
// Reverse: 64-edge tiles, TMEM columns [0,64) z^T, [64,128) z'^T,
// [128,320) f^T, [320,512) f'^T (f' = df/dd, forward mode).
#include <cuda_fp16.h>
#include <mutex>
#include "common.cuh"
#include "workspace.h"
#include "edge_common.cuh"
#include "profile.h"
#include "tc_ptx.cuh"

namespace mlff {
using namespace tc;

// ----------------------------------------------------- operand layouts
// A operand (weights): 128 rows x 16 K fp16, K-major, no swizzle:
//   off(m, k) = (k / 8) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2
constexpr uint32_t A_TILE = 4096;
constexpr uint32_t A_LBO = 2048;
constexpr uint32_t A_SBO = 128;
constexpr uint32_t SLAB = 2 * A_TILE;         // hi + lo of one 128 x 16 block
constexpr int W2_SLABS = 24;                  // 3 channel chunks x 8 K-steps, q = g * 8 + s
constexpr uint32_t W1_BYTES = 2 * SLAB;       // 2 K-steps
constexpr int NSLOT = 12;                     // W2 ring depth

__host__ __device__ constexpr uint32_t a_off(int m, int k) {
    return (uint32_t)((k >> 3) * 2048 + (m >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

// B operand (edge rows) with N rows: per K-step two 8-column chunks, the
// second LB = N*16 + 16 bytes after the first (the extra 16 bytes spread
// the epilogue's 2-byte stores over distinct banks).
__host__ __device__ constexpr uint32_t b_lbo(int n) { return (uint32_t)(n * 16 + 16); }
__host__ __device__ constexpr uint32_t b_kstep(int n) { return 2 * b_lbo(n); }
__device__ __forceinline__ uint32_t b_off(int n_rows, int row, int k) {
    return (uint32_t)((k >> 4) * b_kstep(n_rows) + ((k >> 3) & 1) * b_lbo(n_rows) + (row >> 3) * 128 +
                      (row & 7) * 16 + (k & 7) * 2);
}

constexpr uint32_t align1k(uint32_t x) { return (x + 1023u) & ~1023u; }

// ------------------------------------------------------------- packing
// W1 [H][RMAX] -> 2 K-step blocks (hi, lo); W2 [3H][H] -> 24 slabs.
__global__ void pack_tc_kernel(const float* __restrict__ w1, const float* __restrict__ w2,
                               unsigned char* __restrict__ w1_out, unsigned char* __restrict__ w2_out) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * 128 * 16; i += stride) {
        const int s = i / 2048, m = (i / 16) % 128, kk = i % 16;
        __half hi, lo;
        split_f16(w1[m * RMAX + 16 * s + kk], hi, lo);
        *reinterpret_cast<__half*>(w1_out + s * SLAB + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(w1_out + s * SLAB + A_TILE + a_off(m, kk)) = lo;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < W2_SLABS * 128 * 16; i += stride) {
        const int q = i / 2048, m = (i / 16) % 128, kk = i % 16;
        const int g = q / 8, s = q % 8;
        __half hi, lo;
        split_f16(w2[(g * 128 + m) * H + 16 * s + kk], hi, lo);
        *reinterpret_cast<__half*>(w2_out + q * SLAB + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(w2_out + q * SLAB + A_TILE + a_off(m, kk)) = lo;
    }
}

int pack_bf16(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st) {
    for (int l = 0; l < d.n_layers; ++l) {
        const LayerOffsets& L = o.layer[l];
        pack_tc_kernel<<<64, 256, 0, st>>>(out + L.w1, out + L.w2, reinterpret_cast<unsigned char*>(out + L.w1_bf),
                                           reinterpret_cast<unsigned char*>(out + L.w2_bf));
        MLFF_LAUNCH_CHECK("pack_tc");
    }
    return MLFF_OK;
}

// -------------------------------------------------------- shared pieces
constexpr long long WAIT_BUDGET = 1LL << 32;   // ~2 s at 2 GHz

__device__ __forceinline__ void signal_timeout(const EdgeArgs& a, volatile int* abort_flag, int where) {
    set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, where);
    *abort_flag = 1;
}

// Ring producer: fill number p goes to slot p % NSLOT with slab p % 24.
__device__ __forceinline__ bool produce_slab(uint32_t p, unsigned char* ring, const unsigned char* w2,
                                             uint64_t* full, uint64_t* empty) {
    const uint32_t slot = p % NSLOT;
    if (p >= (uint32_t)NSLOT) {
        if (!mbar_wait(&empty[slot], ((p / NSLOT) - 1) & 1, WAIT_BUDGET)) return false;
    }
    mbar_expect_tx(&full[slot], SLAB);
    bulk_g2s(ring + slot * SLAB, w2 + (size_t)(p % W2_SLABS) * SLAB, SLAB, &full[slot]);
    return true;
}

// rbf(d)_r * fc(d) for r in [r0, r0 + 16) (0 beyond R or for padding edges)
__device__ __forceinline__ void rbf16(float d, bool valid, int r0, int R, const float* cent, const float* gam,
                                      float rc, float (&out)[16]) {
    const float fc = cutoff_fn(d, rc);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int r = r0 + i;
        const float diff = d - cent[r];
        out[i] = (valid && r < R) ? expf(-gam[r] * diff * diff) * fc : 0.0f;
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
        const float g = expf(-gam[r] * diff * diff);
        out[i] = (valid && r < R) ? g * (dfc - 2.0f * gam[r] * diff * fc) : 0.0f;
    }
}

// store 16 consecutive K values (one K-step, both 8-column chunks) of one
// row as split fp16 into a B-operand tile (hi half, lo half)
__device__ __forceinline__ void store_row16(unsigned char* tile, uint32_t half_bytes, int n_rows, int row, int s,
                                            const float (&v)[16]) {
    __align__(16) __half hi[16];
    __align__(16) __half lo[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) split_f16(v[i], hi[i], lo[i]);
    const uint32_t o0 = b_off(n_rows, row, 16 * s);
    const uint32_t o1 = b_off(n_rows, row, 16 * s + 8);
    *reinterpret_cast<uint4*>(tile + o0) = *reinterpret_cast<const uint4*>(&hi[0]);
    *reinterpret_cast<uint4*>(tile + o1) = *reinterpret_cast<const uint4*>(&hi[8]);
    *reinterpret_cast<uint4*>(tile + half_bytes + o0) = *reinterpret_cast<const uint4*>(&lo[0]);
    *reinterpret_cast<uint4*>(tile + half_bytes + o1) = *reinterpret_cast<const uint4*>(&lo[8]);
}

// Receiver flush for two of the four feature components (s, v_x, v_y, v_z):
// out[cur] = base[cur] + acc, then out[j] = base[j] for receivers without
// edges up to next.
__device__ __noinline__ void flush2(const float* __restrict__ base, float* __restrict__ out, int c, int comp0,
                                    int comp1, int cur, int next, float acc0, float acc1) {
    const int64_t r0 = (int64_t)cur * 4 * H;
    out[r0 + comp0 * H + c] = base[r0 + comp0 * H + c] + acc0;
    out[r0 + comp1 * H + c] = base[r0 + comp1 * H + c] + acc1;
    for (int j = cur + 1; j < next; ++j) {
        const int64_t rj = (int64_t)j * 4 * H;
        out[rj + comp0 * H + c] = base[rj + comp0 * H + c];
        out[rj + comp1 * H + c] = base[rj + comp1 * H + c];
    }
}

// ------------------------------------------------------- forward kernel
constexpr int FN = 128;                                   // edges per tile
constexpr uint32_t F_EH = 2 * b_kstep(FN);                // E tile, one half (2 K-steps)
constexpr uint32_t F_HH = 8 * b_kstep(FN);                // H tile, one half (8 K-steps)
constexpr uint32_t F_OFF_W1 = 0;
constexpr uint32_t F_OFF_E = F_OFF_W1 + W1_BYTES;
constexpr uint32_t F_OFF_H = align1k(F_OFF_E + 2 * F_EH);
constexpr uint32_t F_OFF_RING = align1k(F_OFF_H + 2 * F_HH);
constexpr uint32_t F_OFF_US = F_OFF_RING + NSLOT * SLAB;
constexpr uint32_t F_OFF_SRC = F_OFF_US + FN * 16;
constexpr uint32_t F_OFF_RCV = F_OFF_SRC + FN * 4;
constexpr uint32_t F_OFF_B1 = F_OFF_RCV + FN * 4;
constexpr uint32_t F_OFF_B2 = F_OFF_B1 + H * 4;
constexpr uint32_t F_OFF_CG = F_OFF_B2 + H3 * 4;
constexpr uint32_t F_OFF_BAR = F_OFF_CG + 2 * RMAX * 4;
constexpr uint32_t F_OFF_MISC = F_OFF_BAR + 8 * (1 + 2 * NSLOT);
constexpr uint32_t F_SMEM = align1k(F_OFF_MISC + 16);
static_assert(F_SMEM <= 232448, "forward kernel shared memory");

__global__ void __launch_bounds__(256, 1) edge_fwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                             const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + F_OFF_W1;
    unsigned char* Es = smem + F_OFF_E;
    unsigned char* Hs = smem + F_OFF_H;
    unsigned char* ring = smem + F_OFF_RING;
    float4* us = reinterpret_cast<float4*>(smem + F_OFF_US);
    int* src_s = reinterpret_cast<int*>(smem + F_OFF_SRC);
    int* rcv_s = reinterpret_cast<int*>(smem + F_OFF_RCV);
    float* b1s = reinterpret_cast<float*>(smem + F_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + F_OFF_B2);
    float* cent = reinterpret_cast<float*>(smem + F_OFF_CG);
    float* gam = cent + RMAX;
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + F_OFF_BAR);
    uint64_t* full = mma_bar + 1;
    uint64_t* empty = full + NSLOT;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + F_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + F_OFF_MISC + 4);
    uint32_t* ccount_s = reinterpret_cast<uint32_t*>(smem + F_OFF_MISC + 8);

    if (a.st->code != 0) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w == 0) {
        tmem_alloc(tslot, 512);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(mma_bar, 1);
        for (int i = 0; i < NSLOT; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_mbar_init();
        *abort_flag = 0;
        *ccount_s = 0;
    }
    for (int i = t; i < (int)(W1_BYTES / 16); i += 256)
        reinterpret_cast<uint4*>(w1s)[i] = reinterpret_cast<const uint4*>(w1g)[i];
    if (t < H) b1s[t] = a.P[a.lo.b1 + t];
    for (int i = t; i < H3; i += 256) b2s[i] = a.P[a.lo.b2 + i];
    if (t < RMAX) {
        cent[t] = a.centers[t];
        gam[t] = a.gamma[t];
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_f16(FN);

    uint32_t mma_phase = 0;
    uint32_t pcount = 0, ccount = 0;   // ring fills (thread 32) / uses (thread 0)
    uint32_t tiles = 0;
    if (t == 32) {
        for (int i = 0; i < NSLOT; ++i) produce_slab(pcount++, ring, w2g, full, empty);
    }

    // epilogue-2 role: lane quarter q (channels 32q..32q+31), components
    const int q = w & 3, role = w >> 2;
    const int c = 32 * q + lane;
    const int comp0 = role == 0 ? 0 : 2, comp1 = role == 0 ? 1 : 3;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);

    bool aborted = false;
    for (int p = blockIdx.x; p < a.nparts && !aborted; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        int cur = j0;
        float acc0 = 0.f, acc1 = 0.f;
        for (int t0 = e0; t0 < e1; t0 += FN) {
            const int n = min(FN, e1 - t0);
            if (t < FN) load_edge(a, t0, t, n, us, src_s, rcv_s);
            __syncthreads();
            {   // E tile: edge row, 16 RBF columns (one K-step) per thread
                const int e = t & (FN - 1), s = t >> 7;
                float v[16];
                rbf16(us[e].w, e < n, 16 * s, a.R, cent, gam, a.cutoff, v);
                store_row16(Es, F_EH, FN, e, s, v);
            }
            fence_async_smem();
            __syncthreads();
            if (t == 0) {   // GEMM1: z^T = W1 e^T
                fence_after_sync();
#pragma unroll
                for (int s = 0; s < 2; ++s)
#pragma unroll
                    for (int pr = 0; pr < 3; ++pr) {
                        const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                        const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                        const uint64_t bd = sdesc(smem_u32(Es + bhl * F_EH + s * b_kstep(FN)), b_lbo(FN), 128);
                        mma_f16(tmem, ad, bd, idesc, (s | pr) != 0);
                    }
                mma_commit(mma_bar);
            }
            if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 1);
            mma_phase ^= 1;
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1) -> H tile (split fp16)
                const int k = 32 * q + lane, half = w >> 2;
                const float bias = b1s[k];
#pragma unroll
                for (int blk = 0; blk < 2; ++blk) {
                    const int col = 64 * half + 32 * blk;
                    float z[32];
                    tmem_ld32(lane_base + col, z);
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        __half hi, lo;
                        split_f16(silu_f(z[i] + bias), hi, lo);
                        const uint32_t off = b_off(FN, col + i, k);
                        *reinterpret_cast<__half*>(Hs + off) = hi;
                        *reinterpret_cast<__half*>(Hs + F_HH + off) = lo;
                    }
                }
            }
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            if (t == 0) {   // GEMM2: f^T = W2 h^T, W2 streamed slab by slab
                fence_after_sync();
                bool ok = true;
                for (int qq = 0; qq < W2_SLABS && ok; ++qq) {
                    const uint32_t slot = ccount % NSLOT;
                    if (!mbar_wait(&full[slot], (ccount / NSLOT) & 1, WAIT_BUDGET)) {
                        signal_timeout(a, abort_flag, 2);
                        ok = false;
                        break;
                    }
                    const int g = qq / 8, s = qq % 8;
#pragma unroll
                    for (int pr = 0; pr < 3; ++pr) {
                        const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                        const uint64_t ad = sdesc(smem_u32(ring + slot * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                        const uint64_t bd = sdesc(smem_u32(Hs + bhl * F_HH + s * b_kstep(FN)), b_lbo(FN), 128);
                        mma_f16(tmem + 128 + 128 * g, ad, bd, idesc, (s | pr) != 0);
                    }
                    mma_commit(&empty[slot]);
                    ++ccount;
                }
                mma_commit(mma_bar);
                *ccount_s = ccount;
            }
            if (t == 32) {
                const uint32_t target = (uint32_t)W2_SLABS * (tiles + 1);
                while (pcount < target) {
                    if (!produce_slab(pcount, ring, w2g, full, empty)) {
                        signal_timeout(a, abort_flag, 3);
                        break;
                    }
                    ++pcount;
                }
            }
            if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 4);
            mma_phase ^= 1;
            fence_after_sync();
            ++tiles;
            if (t == 32 && !*abort_flag) {
                // the ring is idle: prefetch the first slabs of the next tile
                const uint32_t target = (uint32_t)W2_SLABS * tiles + NSLOT;
                while (pcount < target && produce_slab(pcount, ring, w2g, full, empty)) ++pcount;
            }
            {   // epilogue 2: messages, receiver-segmented sums (no atomics)
                const float bs = b2s[c], bv1 = b2s[H + c], bv2 = b2s[2 * H + c];
                for (int blk = 0; blk < FN / 32; ++blk) {
                    const int col = 32 * blk;
                    if (col >= n) break;
                    float fs[32], fv1[32], fv2[32];
                    tmem_ld32(lane_base + 256 + col, fv1);
                    tmem_ld32(lane_base + 384 + col, fv2);
                    if (role == 0) tmem_ld32(lane_base + 128 + col, fs);
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int e = col + i;
                        if (e < n) {
                            const int ra = rcv_s[e];
                            if (ra != cur) {
                                flush2(a.X, a.Xt, c, comp0, comp1, cur, ra, acc0, acc1);
                                acc0 = acc1 = 0.f;
                                cur = ra;
                            }
                            const float* xb = a.X + (int64_t)src_s[e] * 4 * H;
                            const float4 u = us[e];
                            const float p1 = fv1[i] + bv1, p2 = fv2[i] + bv2;
                            if (role == 0) {
                                acc0 = fmaf(xb[c], fs[i] + bs, acc0);
                                acc1 = fmaf(xb[H + c], p1, fmaf(u.x, p2, acc1));
                            } else {
                                acc0 = fmaf(xb[2 * H + c], p1, fmaf(u.y, p2, acc0));
                                acc1 = fmaf(xb[3 * H + c], p1, fmaf(u.z, p2, acc1));
                            }
                        }
                    }
                }
            }
            fence_before_sync();
            __syncthreads();
            if (*abort_flag) {
                aborted = true;
                break;
            }
        }
        if (!aborted) flush2(a.X, a.Xt, c, comp0, comp1, cur, j1, acc0, acc1);
    }
    // drain: every ring fill issued must have landed before the CTA exits
    __syncthreads();
    if (t == 32) {
        const uint32_t used = *ccount_s;
        for (uint32_t f = used; f < pcount; ++f)
            if (!mbar_wait(&full[f % NSLOT], (f / NSLOT) & 1, WAIT_BUDGET)) {
                set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 5);
                break;
            }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------- reverse kernel
constexpr int BN = 64;
constexpr uint32_t B_EH = 2 * b_kstep(BN);
constexpr uint32_t B_HH = 8 * b_kstep(BN);
constexpr uint32_t B_OFF_W1 = 0;
constexpr uint32_t B_OFF_E = B_OFF_W1 + W1_BYTES;          // E then E'
constexpr uint32_t B_OFF_H = align1k(B_OFF_E + 4 * B_EH);   // H then H'
constexpr uint32_t B_OFF_RING = align1k(B_OFF_H + 4 * B_HH);
constexpr uint32_t B_OFF_US = B_OFF_RING + NSLOT * SLAB;
constexpr uint32_t B_OFF_SRC = B_OFF_US + BN * 16;
constexpr uint32_t B_OFF_RCV = B_OFF_SRC + BN * 4;
constexpr uint32_t B_OFF_B1 = B_OFF_RCV + BN * 4;
constexpr uint32_t B_OFF_B2 = B_OFF_B1 + H * 4;
constexpr uint32_t B_OFF_CG = B_OFF_B2 + H3 * 4;
constexpr uint32_t B_OFF_RED = B_OFF_CG + 2 * RMAX * 4;
constexpr uint32_t B_OFF_BAR = B_OFF_RED + 8 * BN * 3 * 4;
constexpr uint32_t B_OFF_MISC = B_OFF_BAR + 8 * (1 + 2 * NSLOT);
constexpr uint32_t B_SMEM = align1k(B_OFF_MISC + 16);
static_assert(B_SMEM <= 232448, "reverse kernel shared memory");

__global__ void __launch_bounds__(256, 1) edge_bwd_tc_kernel(EdgeArgs a, const unsigned char* __restrict__ w1g,
                                                             const unsigned char* __restrict__ w2g) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* w1s = smem + B_OFF_W1;
    unsigned char* Es = smem + B_OFF_E;            // [E hi, E lo, E' hi, E' lo]
    unsigned char* Hs = smem + B_OFF_H;            // [H hi, H lo, H' hi, H' lo]
    unsigned char* ring = smem + B_OFF_RING;
    float4* us = reinterpret_cast<float4*>(smem + B_OFF_US);
    int* src_s = reinterpret_cast<int*>(smem + B_OFF_SRC);
    int* rcv_s = reinterpret_cast<int*>(smem + B_OFF_RCV);
    float* b1s = reinterpret_cast<float*>(smem + B_OFF_B1);
    float* b2s = reinterpret_cast<float*>(smem + B_OFF_B2);
    float* cent = reinterpret_cast<float*>(smem + B_OFF_CG);
    float* gam = cent + RMAX;
    float* red = reinterpret_cast<float*>(smem + B_OFF_RED);   // [8 warps][BN][3]
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + B_OFF_BAR);
    uint64_t* full = mma_bar + 1;
    uint64_t* empty = full + NSLOT;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + B_OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + B_OFF_MISC + 4);
    uint32_t* ccount_s = reinterpret_cast<uint32_t*>(smem + B_OFF_MISC + 8);

    if (a.st->code != 0) return;
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (w == 0) {
        tmem_alloc(tslot, 512);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(mma_bar, 1);
        for (int i = 0; i < NSLOT; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_mbar_init();
        *abort_flag = 0;
        *ccount_s = 0;
    }
    for (int i = t; i < (int)(W1_BYTES / 16); i += 256)
        reinterpret_cast<uint4*>(w1s)[i] = reinterpret_cast<const uint4*>(w1g)[i];
    if (t < H) b1s[t] = a.P[a.lo.b1 + t];
    for (int i = t; i < H3; i += 256) b2s[i] = a.P[a.lo.b2 + i];
    if (t < RMAX) {
        cent[t] = a.centers[t];
        gam[t] = a.gamma[t];
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = idesc_f16(BN);

    uint32_t mma_phase = 0;
    uint32_t pcount = 0, ccount = 0;
    uint32_t tiles = 0;
    if (t == 32) {
        for (int i = 0; i < NSLOT; ++i) produce_slab(pcount++, ring, w2g, full, empty);
    }
    const int q = w & 3, role = w >> 2;
    const int c = 32 * q + lane;
    const int comp0 = role == 0 ? 0 : 2, comp1 = role == 0 ? 1 : 3;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);

    bool aborted = false;
    for (int p = blockIdx.x; p < a.nparts && !aborted; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        int cur = j0;
        float acc0 = 0.f, acc1 = 0.f;
        float ta0, ta1;   // receiver adjoint (dE/dXt) for this thread's two components
        {
            const float* tr = a.xtbar + (int64_t)cur * 4 * H;
            ta0 = tr[comp0 * H + c];
            ta1 = tr[comp1 * H + c];
        }
        for (int t0 = e0; t0 < e1; t0 += BN) {
            const int n = min(BN, e1 - t0);
            if (t < BN) load_edge(a, t0, t, n, us, src_s, rcv_s);
            __syncthreads();
            {   // E (rbf * fc) and E' (its d-derivative) tiles
                const int e = t & (BN - 1), s = (t >> 6) & 1, which = t >> 7;
                float v[16];
                if (which == 0) rbf16(us[e].w, e < n, 16 * s, a.R, cent, gam, a.cutoff, v);
                else rbf16_d(us[e].w, e < n, 16 * s, a.R, cent, gam, a.cutoff, v);
                store_row16(Es + which * 2 * B_EH, B_EH, BN, e, s, v);
            }
            fence_async_smem();
            __syncthreads();
            if (t == 0) {   // z^T = W1 e^T, z'^T = W1 e'^T
                fence_after_sync();
#pragma unroll
                for (int which = 0; which < 2; ++which)
#pragma unroll
                    for (int s = 0; s < 2; ++s)
#pragma unroll
                        for (int pr = 0; pr < 3; ++pr) {
                            const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                            const uint64_t ad = sdesc(smem_u32(w1s + s * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                            const uint64_t bd = sdesc(smem_u32(Es + which * 2 * B_EH + bhl * B_EH + s * b_kstep(BN)),
                                                      b_lbo(BN), 128);
                            mma_f16(tmem + 64 * which, ad, bd, idesc, (s | pr) != 0);
                        }
                mma_commit(mma_bar);
            }
            if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 11);
            mma_phase ^= 1;
            fence_after_sync();
            {   // epilogue 1: h = silu(z + b1), h' = silu'(z + b1) z'
                const int k = 32 * q + lane, col = 32 * (w >> 2);
                const float bias = b1s[k];
                float z[32], zd[32];
                tmem_ld32(lane_base + col, z);
                tmem_ld32(lane_base + 64 + col, zd);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float zz = z[i] + bias;
                    __half hi, lo, dhi, dlo;
                    split_f16(silu_f(zz), hi, lo);
                    split_f16(dsilu_f(zz) * zd[i], dhi, dlo);
                    const uint32_t off = b_off(BN, col + i, k);
                    *reinterpret_cast<__half*>(Hs + off) = hi;
                    *reinterpret_cast<__half*>(Hs + B_HH + off) = lo;
                    *reinterpret_cast<__half*>(Hs + 2 * B_HH + off) = dhi;
                    *reinterpret_cast<__half*>(Hs + 3 * B_HH + off) = dlo;
                }
            }
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            if (t == 0) {   // f^T = W2 h^T and f'^T = W2 h'^T share each W2 slab
                fence_after_sync();
                bool ok = true;
                for (int qq = 0; qq < W2_SLABS && ok; ++qq) {
                    const uint32_t slot = ccount % NSLOT;
                    if (!mbar_wait(&full[slot], (ccount / NSLOT) & 1, WAIT_BUDGET)) {
                        signal_timeout(a, abort_flag, 12);
                        ok = false;
                        break;
                    }
                    const int g = qq / 8, s = qq % 8;
#pragma unroll
                    for (int which = 0; which < 2; ++which)
#pragma unroll
                        for (int pr = 0; pr < 3; ++pr) {
                            const uint32_t ahl = pr == 2 ? 1 : 0, bhl = pr == 1 ? 1 : 0;
                            const uint64_t ad = sdesc(smem_u32(ring + slot * SLAB + ahl * A_TILE), A_LBO, A_SBO);
                            const uint64_t bd = sdesc(smem_u32(Hs + which * 2 * B_HH + bhl * B_HH + s * b_kstep(BN)),
                                                      b_lbo(BN), 128);
                            mma_f16(tmem + 128 + 192 * which + 64 * g, ad, bd, idesc, (s | pr) != 0);
                        }
                    mma_commit(&empty[slot]);
                    ++ccount;
                }
                mma_commit(mma_bar);
                *ccount_s = ccount;
            }
            if (t == 32) {
                const uint32_t target = (uint32_t)W2_SLABS * (tiles + 1);
                while (pcount < target) {
                    if (!produce_slab(pcount, ring, w2g, full, empty)) {
                        signal_timeout(a, abort_flag, 13);
                        break;
                    }
                    ++pcount;
                }
            }
            if (!mbar_wait(mma_bar, mma_phase, WAIT_BUDGET)) signal_timeout(a, abort_flag, 14);
            mma_phase ^= 1;
            fence_after_sync();
            ++tiles;
            if (t == 32 && !*abort_flag) {
                const uint32_t target = (uint32_t)W2_SLABS * tiles + NSLOT;
                while (pcount < target && produce_slab(pcount, ring, w2g, full, empty)) ++pcount;
            }
            {   // epilogue 2: node adjoints (gathered), per-edge dE/dd and dE/du partials
                const float bs = b2s[c], bv1 = b2s[H + c], bv2 = b2s[2 * H + c];
                for (int blk = 0; blk < BN / 16; ++blk) {
                    const int col = 16 * blk;
                    if (col >= n) break;
                    float fs[16], fv1[16], fv2[16], ds[16], dv1[16], dv2[16];
                    tmem_ld16(lane_base + 128 + 64 + col, fv1);
                    tmem_ld16(lane_base + 128 + 128 + col, fv2);
                    tmem_ld16(lane_base + 320 + 64 + col, dv1);
                    tmem_ld16(lane_base + 320 + 128 + col, dv2);
                    if (role == 0) {
                        tmem_ld16(lane_base + 128 + col, fs);
                        tmem_ld16(lane_base + 320 + col, ds);
                    }
                    tmem_ld_wait();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int e = col + i;
                        if (e < n) {
                            const int ra = rcv_s[e];
                            if (ra != cur) {
                                flush2(a.xtbar, a.xbar, c, comp0, comp1, cur, ra, acc0, acc1);
                                acc0 = acc1 = 0.f;
                                cur = ra;
                                const float* tr = a.xtbar + (int64_t)cur * 4 * H;
                                ta0 = tr[comp0 * H + c];
                                ta1 = tr[comp1 * H + c];
                            }
                            const int64_t rb = (int64_t)src_s[e] * 4 * H;
                            const float tb0 = a.xtbar[rb + comp0 * H + c], tb1 = a.xtbar[rb + comp1 * H + c];
                            const float xb0 = a.X[rb + comp0 * H + c], xb1 = a.X[rb + comp1 * H + c];
                            const float4 u = us[e];
                            const float p1 = fv1[i] + bv1, p2 = fv2[i] + bv2;
                            float r0, r1, r2;
                            if (role == 0) {   // components s, v_x
                                acc0 = fmaf(tb0, fs[i] + bs, acc0);
                                acc1 = fmaf(tb1, p1, acc1);
                                r0 = (ta0 * xb0) * ds[i] + (ta1 * xb1) * dv1[i] + (ta1 * u.x) * dv2[i];
                                r1 = ta1 * p2;
                                r2 = 0.f;
                            } else {           // components v_y, v_z
                                acc0 = fmaf(tb0, p1, acc0);
                                acc1 = fmaf(tb1, p1, acc1);
                                r0 = (ta0 * xb0 + ta1 * xb1) * dv1[i] + (ta0 * u.y + ta1 * u.z) * dv2[i];
                                r1 = ta0 * p2;
                                r2 = ta1 * p2;
                            }
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1) {
                                r0 += __shfl_xor_sync(0xffffffffu, r0, o);
                                r1 += __shfl_xor_sync(0xffffffffu, r1, o);
                                r2 += __shfl_xor_sync(0xffffffffu, r2, o);
                            }
                            if (lane == 0) {
                                float* rr = red + ((size_t)w * BN + e) * 3;
                                rr[0] = r0;
                                rr[1] = r1;
                                rr[2] = r2;
                            }
                        }
                    }
                }
            }
            fence_before_sync();
            __syncthreads();
            if (t < n) {
                float dd = 0.f, dux = 0.f, duy = 0.f, duz = 0.f;
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const float* r0p = red + ((size_t)qq * BN + t) * 3;         // role 0 warps
                    const float* r1p = red + ((size_t)(4 + qq) * BN + t) * 3;   // role 1 warps
                    dd += r0p[0] + r1p[0];
                    dux += r0p[1];
                    duy += r1p[1];
                    duz += r1p[2];
                }
                float4 acc = a.eacc[t0 + t];
                acc.x += dd;
                acc.y += dux;
                acc.z += duy;
                acc.w += duz;
                a.eacc[t0 + t] = acc;
            }
            __syncthreads();
            if (*abort_flag) {
                aborted = true;
                break;
            }
        }
        if (!aborted) flush2(a.xtbar, a.xbar, c, comp0, comp1, cur, j1, acc0, acc1);
    }
    __syncthreads();
    if (t == 32) {
        const uint32_t used = *ccount_s;
        for (uint32_t f = used; f < pcount; ++f)
            if (!mbar_wait(&full[f % NSLOT], (f / NSLOT) & 1, WAIT_BUDGET)) {
                set_status(const_cast<Status*>(a.st), MLFF_ERR_TIMEOUT, 15);
                break;
            }
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
    edge_fwd_tc_kernel<<<tc_grid(a.nparts), 256, F_SMEM, st>>>(a, w1, w2);
    MLFF_LAUNCH_CHECK("edge_fwd_tc");
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
    edge_bwd_tc_kernel<<<tc_grid(a.nparts), 256, B_SMEM, st>>>(a, w1, w2);
    MLFF_LAUNCH_CHECK("edge_bwd_tc");
    return MLFF_OK;
}

}  // namespace mlff
