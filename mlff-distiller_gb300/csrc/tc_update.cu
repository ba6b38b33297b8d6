// Tensor-core (tcgen05) per-atom update block (PaiNNUpdate.forward,
// student_model.py:434-470, and its adjoint), the dense per-atom MLP
// Linear(2H, H) - SiLU - Linear(H, 3H) on split-FP16 operands with FP32
// accumulation in TMEM, like the edge filters in tc_edge.cu.
//
// Transposed GEMMs, D[channel][atom] = W[channel][k] X[atom][k]^T: a TMEM
// lane is an output channel, a column an atom, so the epilogue thread that
// owns channel c touches channel c of consecutive atoms -- coalesced rows of
// the [N][4][H] feature arrays.  64-atom tiles (MMA N = 64, so that a
// 3,000-atom system still spreads over 47 SMs), persistent CTAs of 8 warps,
// two per SM (one CTA's epilogues overlap the other's weight stream and MMAs):
// in the epilogues warp w reads TMEM lane quarter w % 4 for atoms
// 32 (w / 4) .. +31; the B tiles are built one atom row per warp (lane l:
// channels 4l..4l+3, coalesced 512-byte rows).
//
// The weights (split-FP16 A-operand tile pairs, 8 KB per 128 x 16 block)
// stream through a ring of bulk copies (5 slots forward, 2 reverse: what
// two CTAs per SM leave of shared memory) in the order the MMAs use
// them: one thread issues the MMAs and commits each slot, another refills
// the slots (during a GEMM, and ahead of the next GEMM while the epilogue
// runs).  The forward accumulators are pre-filled with the bias, so every
// MMA accumulates.  Every wait is bounded (MLFF_ERR_TIMEOUT).
#include <cuda_fp16.h>
#include <mutex>
#include "common.cuh"
#include "workspace.h"
#include "profile.h"
#include "tc_ptx.cuh"
#include "tc_layout.cuh"

namespace mlff {
using namespace tc;

// ------------------------------------------------------------- packing
// pair p of a matrix: hi tile at p * A_PAIR, lo tile at p * A_PAIR + A_TILE;
// element (m, k) of the pair's 128 x 16 block at a_off(m, k).
__global__ void pack_update_tc_kernel(const float* __restrict__ u1, const float* __restrict__ u2,
                                      unsigned char* __restrict__ u1p, unsigned char* __restrict__ u2p,
                                      unsigned char* __restrict__ u2tp, unsigned char* __restrict__ u1tp) {
    const int stride = gridDim.x * blockDim.x;
    auto put = [](unsigned char* dst, int pair, int m, int kk, float v) {
        __half hi, lo;
        split_f16(v, hi, lo);
        *reinterpret_cast<__half*>(dst + pair * A_PAIR + a_off(m, kk)) = hi;
        *reinterpret_cast<__half*>(dst + pair * A_PAIR + A_TILE + a_off(m, kk)) = lo;
    };
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * 128 * 16; i += stride) {
        const int p = i / 2048, m = (i / 16) % 128, kk = i % 16;
        put(u1p, p, m, kk, u1[m * 2 * H + 16 * p + kk]);                       // U1 [H][2H], K-step p
        const int g = p >> 3, s = p & 7;
        put(u1tp, p, m, kk, u1[(16 * s + kk) * 2 * H + g * 128 + m]);          // U1^T [2H][H], chunk g
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 24 * 128 * 16; i += stride) {
        const int p = i / 2048, m = (i / 16) % 128, kk = i % 16;
        const int g = p >> 3, s = p & 7;
        put(u2p, p, m, kk, u2[(g * 128 + m) * H + 16 * s + kk]);               // U2 [3H][H], chunk g
        put(u2tp, p, m, kk, u2[(16 * p + kk) * H + m]);                        // U2^T [H][3H], K-step p
    }
}

int pack_update_tc(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st) {
    for (int l = 0; l < d.n_layers; ++l) {
        const LayerOffsets& L = o.layer[l];
        auto b = [&](int64_t off) { return reinterpret_cast<unsigned char*>(out + off); };
        pack_update_tc_kernel<<<64, 256, 0, st>>>(out + L.u1, out + L.u2, b(L.u1_tc), b(L.u2_tc), b(L.u2t_tc),
                                                  b(L.u1t_tc));
        MLFF_LAUNCH_CHECK("pack_update_tc");
    }
    return MLFF_OK;
}

// ------------------------------------------------------- weight stream
constexpr int UNT = 256;

template <int URING>
struct UStream {
    unsigned char* ring;
    uint64_t* full;
    uint64_t* empty;
    const unsigned char* src[2];   // pair sources of the two GEMMs of a tile
    int npairs[2];
    uint32_t issued;               // producer: pairs copied so far (global count)
    uint32_t consumed;             // consumer: pairs whose copy was seen complete
};

template <int URING>
__device__ __forceinline__ const unsigned char* ustream_src(const UStream<URING>& s, uint32_t P) {
    const uint32_t per = s.npairs[0] + s.npairs[1];
    const uint32_t q = P % per;
    return q < (uint32_t)s.npairs[0] ? s.src[0] + (size_t)q * A_PAIR : s.src[1] + (size_t)(q - s.npairs[0]) * A_PAIR;
}

// producer: copy pairs until `target` (exclusive) are issued; a slot is
// reused once the commit of the pair that used it URING pairs earlier has
// arrived
template <int URING>
__device__ __forceinline__ bool ustream_fill(UStream<URING>& s, uint32_t target) {
    while (s.issued < target) {
        const uint32_t slot = s.issued % URING;
        if (s.issued >= (uint32_t)URING && !mbar_wait(&s.empty[slot], ((s.issued / URING) - 1) & 1, WAIT_BUDGET))
            return false;
        mbar_expect_tx(&s.full[slot], A_PAIR);
        bulk_g2s(s.ring + slot * A_PAIR, ustream_src(s, s.issued), A_PAIR, &s.full[slot]);
        ++s.issued;
    }
    return true;
}

// consumer: one GEMM of a tile.  Pair i of n (global pair P0 + i): D[d_of(i)]
// += A_hi B_hi(i) + A_hi B_lo(i) + A_lo B_hi(i); the first MMA of pair i
// overwrites D instead when fresh(i).
template <int UN, int URING, typename DOf, typename BOf, typename Fresh>
__device__ __forceinline__ bool ustream_gemm(UStream<URING>& s, uint32_t P0, int n, DOf d_of, BOf b_of, uint64_t bhalf,
                                             Fresh fresh) {
    constexpr uint32_t idesc = idesc_f16(UN);
    const uint64_t a0 = sdesc(smem_u32(s.ring), A_LBO, A_SBO);
#pragma unroll 1
    for (int i = 0; i < n; ++i) {
        const uint32_t P = P0 + i;
        const uint32_t slot = P % URING;
        if (!mbar_wait(&s.full[slot], (P / URING) & 1, WAIT_BUDGET)) return false;
        s.consumed = P + 1;
        const uint64_t ahi = a0 + (uint64_t)(slot * A_PAIR >> 4), alo = ahi + (A_TILE >> 4);
        const uint64_t bhi = b_of(i);
        const uint32_t d = d_of(i);
        mma_f16(d, ahi, bhi, idesc, fresh(i) ? 0u : 1u);
        mma_f16(d, ahi, bhi + bhalf, idesc, 1);
        mma_f16(d, alo, bhi, idesc, 1);
        mma_commit(&s.empty[slot]);
    }
    return true;
}

__device__ __forceinline__ void ufill_tmem(uint32_t taddr, float v, int n16) {
    float bv[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) bv[i] = v;
    for (int k = 0; k < n16; ++k) tmem_st16(taddr + 16 * k, bv);
}

// four consecutive K values (k % 4 == 0) of one row as split fp16
__device__ __forceinline__ void store_row4(unsigned char* tile, uint32_t half_bytes, int n_rows, int row, int k,
                                           float4 v) {
    __half2 h0, l0, h1, l1;
    split2(v.x, v.y, h0, l0);
    split2(v.z, v.w, h1, l1);
    const uint32_t o = b_off(n_rows, row, k);
    uint2 hv, lv;
    hv.x = *reinterpret_cast<uint32_t*>(&h0);
    hv.y = *reinterpret_cast<uint32_t*>(&h1);
    lv.x = *reinterpret_cast<uint32_t*>(&l0);
    lv.y = *reinterpret_cast<uint32_t*>(&l1);
    *reinterpret_cast<uint2*>(tile + o) = hv;
    *reinterpret_cast<uint2*>(tile + half_bytes + o) = lv;
}

// One atom's row of a [N][4][H] array (lane: channels 4 lane .. 4 lane + 3
// of each component) in the component-major layout or, with pairs, in the
// pair layout of the edge kernels' gathers (pair_off).
__device__ __forceinline__ void store_atom_row(float* row, int lane, float4 s, float4 x, float4 y, float4 z,
                                               bool pairs) {
    float4* o = reinterpret_cast<float4*>(row);
    if (pairs) {
        o[2 * lane] = make_float4(s.x, x.x, s.y, x.y);
        o[2 * lane + 1] = make_float4(s.z, x.z, s.w, x.w);
        o[64 + 2 * lane] = make_float4(y.x, z.x, y.y, z.y);
        o[64 + 2 * lane + 1] = make_float4(y.z, z.z, y.w, z.w);
    } else {
        o[lane] = s;
        o[32 + lane] = x;
        o[64 + lane] = y;
        o[96 + lane] = z;
    }
}

// Synchronisation helpers shared by both kernels: one thread issues the
// MMAs of a GEMM while the producer keeps the ring full; then the CTA waits
// for the MMAs (warp 0 polls, the others wait at the barrier).
struct UCtl {
    uint64_t* mma_bar;
    volatile int* abort_flag;
    Status* st;
    uint32_t phase;
};

__device__ __forceinline__ void ufail(UCtl& c, int where) {
    set_status(c.st, MLFF_ERR_TIMEOUT, where);
    *c.abort_flag = 1;
}

__device__ __forceinline__ void uwait_mma(UCtl& c, int w, int where) {
    if (w == 0) __syncwarp();
    if (w == 0 && !mbar_wait(c.mma_bar, c.phase, WAIT_BUDGET)) ufail(c, where);
    c.phase ^= 1;
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
}

// ------------------------------------------------------- forward kernel
// smem: B tile [s, |v|] (K = 256: 4 K-blocks; hi half then lo half, 64 KB),
// the H tile (K = 128, 32 KB) aliased into it after GEMM1, the ring (40 KB).
// TMEM: D1 = z (cols 0..UN-1), D2 chunk g = (ds, g1, g2)[g] (UN + UN g).
// UN-atom tiles, UN = 64 or 32 (the autotuner's update tile: small systems
// spread over more SMs with 32); the ring takes what two CTAs per SM leave.
template <int UN>
struct UFwd {
    static constexpr uint32_t BH = 4 * b_block(UN);
    static constexpr uint32_t HH = 2 * b_block(UN);
    // epilogue 2 stages (ds, g1, g2) of 32 atoms, [3][32][H] floats, in the B region
    static constexpr uint32_t T_BYTES = 3 * 32 * H * 4;
    static constexpr uint32_t B_REGION = 2 * BH > T_BYTES ? 2 * BH : T_BYTES;
    static constexpr int RING = UN == 64 ? 5 : 7;
    static constexpr uint32_t OFF_B = 0;
    static constexpr uint32_t OFF_RING = OFF_B + B_REGION;
    static constexpr uint32_t OFF_C = OFF_RING + RING * A_PAIR;      // c1 [H], c2 [3H], mix [9]
    static constexpr uint32_t OFF_BAR = OFF_C + 4 * (H + H3 + 16);
    static constexpr uint32_t OFF_MISC = OFF_BAR + 8 * (1 + 2 * RING);
    static constexpr uint32_t SMEM = align1k(OFF_MISC + 16);
    static constexpr uint32_t TMEM_COLS = 4 * UN;
    static_assert(2 * (SMEM + 1024) <= 228 * 1024, "two update CTAs per SM");
};

template <int UN>
__global__ void __launch_bounds__(UNT, 2) update_fwd_tc_kernel(const float* __restrict__ P, LayerOffsets lo,
                                                               const float* __restrict__ Xt, int32_t n_atoms,
                                                               float* __restrict__ Xout, int out_pairs,
                                                               float* __restrict__ uz, float* __restrict__ ua,
                                                               Status* st) {
    using LF = UFwd<UN>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* Bs = smem + LF::OFF_B;
    float* c1s = reinterpret_cast<float*>(smem + LF::OFF_C);
    float* c2s = c1s + H;
    float* mix = c2s + H3;
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + LF::OFF_BAR);
    uint64_t* full = mma_bar + 1;
    uint64_t* empty = full + LF::RING;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + LF::OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + LF::OFF_MISC + 4);
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const int ntiles = (n_atoms + UN - 1) / UN;
    if (w == 0) {
        tmem_alloc(tslot, LF::TMEM_COLS);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(mma_bar, 1);
        for (int i = 0; i < LF::RING; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_mbar_init();
        *abort_flag = 0;
    }
    for (int i = t; i < H; i += UNT) c1s[i] = P[lo.c1 + i];
    for (int i = t; i < H3; i += UNT) c2s[i] = P[lo.c2 + i];
    if (t < 9) mix[t] = P[lo.mix + t];
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    UStream<LF::RING> ws{smem + LF::OFF_RING, full, empty,
               {reinterpret_cast<const unsigned char*>(P + lo.u1_tc), reinterpret_cast<const unsigned char*>(P + lo.u2_tc)},
               {16, 24}, 0, 0};
    UCtl ctl{mma_bar, abort_flag, st, 0};
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t P_end = (uint32_t)my_tiles * 40;
    const bool producer = t == 32;
    if (producer && !ustream_fill(ws, min((uint32_t)LF::RING, P_end))) ufail(ctl, 20);
    // everything above reads packed weights only and overlaps the previous kernel
    pdl_wait();
    if (t == 0 && st->code != 0) *abort_flag = 1;
    __syncthreads();
    pdl_trigger();
    const int q = w & 3, hh = w >> 2, c = 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t P0 = 0;

    for (int tile = blockIdx.x; tile < ntiles && !*abort_flag; tile += gridDim.x, P0 += 40) {
        const int a0 = tile * UN;
        // accumulators <- bias: D1 c1, D2 chunk g c2[g]
        ufill_tmem(lane_base + (UN / 2) * hh, c1s[c], UN / 32);
#pragma unroll 1
        for (int g = 0; g < 3; ++g) ufill_tmem(lane_base + UN + UN * g + (UN / 2) * hh, c2s[g * H + c], UN / 32);
        // B tile: row = atom, K = [s (128), |v| (128)]; warp w builds rows w, w + 8, ...,
        // two rows per step so that their loads overlap
#pragma unroll 1
        for (int i0 = w; i0 < UN; i0 += 16) {
            float4 r[2][4];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int a = a0 + i0 + 8 * k;
                const float4* x = reinterpret_cast<const float4*>(Xt + (int64_t)(a < n_atoms ? a : 0) * 4 * H);
#pragma unroll
                for (int j = 0; j < 4; ++j) r[k][j] = a < n_atoms ? x[32 * j + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const float4 vx = r[k][1], vy = r[k][2], vz = r[k][3];
                const float4 nv = make_float4(pair_distance(vx.x, vy.x, vz.x), pair_distance(vx.y, vy.y, vz.y),
                                              pair_distance(vx.z, vy.z, vz.z), pair_distance(vx.w, vy.w, vz.w));  // |v| (:437)
                store_row4(Bs, LF::BH, UN, i0 + 8 * k, 4 * lane, r[k][0]);
                store_row4(Bs, LF::BH, UN, i0 + 8 * k, H + 4 * lane, nv);
            }
        }
        tmem_st_wait();
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (t == 0) {   // GEMM1: z^T = U1 [s, |v|]^T, K = 256
            fence_after_sync();
            const uint64_t b0 = sdesc_b(smem_u32(Bs));
            if (!ustream_gemm<UN>(ws, P0, 16, [&](int) { return tmem; },
                              [&](int i) { return b0 + (uint64_t)(b_kstep_off(UN, i) >> 4); }, (uint64_t)(LF::BH >> 4),
                              [](int) { return false; }))
                ufail(ctl, 21);
            mma_commit(mma_bar);
        }
        if (producer && !ustream_fill(ws, min(P0 + 16, P_end))) ufail(ctl, 26);
        uwait_mma(ctl, w, 22);
        // GEMM1 is done, so every slot is free: fetch GEMM2's pairs during epilogue 1
        if (producer && !ustream_fill(ws, min(P0 + 16 + LF::RING, P_end))) ufail(ctl, 27);
        {   // epilogue 1: z -> uz, h = silu(z) -> H tile (aliases the B tile)
            constexpr int NC = UN / 2;   // this warp half's atoms
            const int col = NC * hh;
            float z[NC];
            if constexpr (NC == 32) tmem_ld32(lane_base + col, z);
            else tmem_ld16(lane_base + col, z);
            tmem_ld_wait();
            const BColumn hcol(Bs, LF::HH, UN, col, c);
#pragma unroll
            for (int i = 0; i < NC; i += 2) {
                const int a = a0 + col + i;
                if (a < n_atoms) uz[(int64_t)a * H + c] = z[i];
                if (a + 1 < n_atoms) uz[(int64_t)(a + 1) * H + c] = z[i + 1];
                // accurate exp: per-atom pre-activations reach |z| ~ 20 with
                // trained-like weights
                hcol.put_pair(i, silu_f(z[i]), silu_f(z[i + 1]));
            }
        }
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (t == 0) {   // GEMM2: a^T = U2 h^T, 3 chunks x 8 K-steps
            fence_after_sync();
            const uint64_t b0 = sdesc_b(smem_u32(Bs));
            if (!ustream_gemm<UN>(ws, P0 + 16, 24, [&](int i) { return tmem + UN + UN * (i >> 3); },
                              [&](int i) { return b0 + (uint64_t)(b_kstep_off(UN, i & 7) >> 4); },
                              (uint64_t)(LF::HH >> 4), [](int) { return false; }))
                ufail(ctl, 23);
            mma_commit(mma_bar);
        }
        if (producer && !ustream_fill(ws, min(P0 + 40, P_end))) ufail(ctl, 28);
        uwait_mma(ctl, w, 24);
        // the next tile's GEMM1 pairs arrive while this epilogue and the next build run
        if (producer && !ustream_fill(ws, min(P0 + 40 + LF::RING, P_end))) ufail(ctl, 29);
        {   // epilogue 2: (ds, g1, g2) -> ua; s' = s + ds, v' = v g1 + (M v) g2 (:452-468).
            // The TMEM owner of channel c writes (ds, g1, g2) of 32 atoms to
            // shared memory (the B tile is free), then each warp handles
            // whole atom rows with 128-bit accesses; UN / 32 passes of 32 atoms.
            float* T = reinterpret_cast<float*>(Bs);      // [3][32 atoms][H]
#pragma unroll 1
            for (int pass = 0; pass < UN / 32; ++pass) {
                if (hh == pass) {
#pragma unroll 1
                    for (int g = 0; g < 3; ++g) {
                        float v[32];
                        tmem_ld32(lane_base + UN + UN * g + 32 * pass, v);
                        tmem_ld_wait();
#pragma unroll
                        for (int i = 0; i < 32; ++i) T[(g * 32 + i) * H + c] = v[i];
                    }
                }
                __syncthreads();
#pragma unroll 1
                for (int i0 = w; i0 < 32; i0 += 16) {
                    float4 x[2][4];
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const int a = a0 + 32 * pass + i0 + 8 * k;
                        const float4* xr = reinterpret_cast<const float4*>(Xt + (int64_t)(a < n_atoms ? a : 0) * 4 * H);
#pragma unroll
                        for (int j = 0; j < 4; ++j) x[k][j] = a < n_atoms ? xr[32 * j + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const int i = i0 + 8 * k, a = a0 + 32 * pass + i;
                        if (a >= n_atoms) continue;
                        const float4 ds = reinterpret_cast<const float4*>(T + (0 * 32 + i) * H)[lane];
                        const float4 g1 = reinterpret_cast<const float4*>(T + (1 * 32 + i) * H)[lane];
                        const float4 g2 = reinterpret_cast<const float4*>(T + (2 * 32 + i) * H)[lane];
                        float4* u = reinterpret_cast<float4*>(ua + (int64_t)a * H3);
                        u[lane] = ds;
                        u[32 + lane] = g1;
                        u[64 + lane] = g2;
                        const float4 sv = x[k][0], vx = x[k][1], vy = x[k][2], vz = x[k][3];
                        auto vnew = [&](float px, float py, float pz, float pc, float a1, float a2, int r) {
                            return pc * a1 + (mix[3 * r] * px + mix[3 * r + 1] * py + mix[3 * r + 2] * pz) * a2;
                        };
                        float4 ox, oy, oz;
                        ox.x = vnew(vx.x, vy.x, vz.x, vx.x, g1.x, g2.x, 0);
                        ox.y = vnew(vx.y, vy.y, vz.y, vx.y, g1.y, g2.y, 0);
                        ox.z = vnew(vx.z, vy.z, vz.z, vx.z, g1.z, g2.z, 0);
                        ox.w = vnew(vx.w, vy.w, vz.w, vx.w, g1.w, g2.w, 0);
                        oy.x = vnew(vx.x, vy.x, vz.x, vy.x, g1.x, g2.x, 1);
                        oy.y = vnew(vx.y, vy.y, vz.y, vy.y, g1.y, g2.y, 1);
                        oy.z = vnew(vx.z, vy.z, vz.z, vy.z, g1.z, g2.z, 1);
                        oy.w = vnew(vx.w, vy.w, vz.w, vy.w, g1.w, g2.w, 1);
                        oz.x = vnew(vx.x, vy.x, vz.x, vz.x, g1.x, g2.x, 2);
                        oz.y = vnew(vx.y, vy.y, vz.y, vz.y, g1.y, g2.y, 2);
                        oz.z = vnew(vx.z, vy.z, vz.z, vz.z, g1.z, g2.z, 2);
                        oz.w = vnew(vx.w, vy.w, vz.w, vz.w, g1.w, g2.w, 2);
                        store_atom_row(Xout + (int64_t)a * 4 * H, lane,
                                       make_float4(sv.x + ds.x, sv.y + ds.y, sv.z + ds.z, sv.w + ds.w), ox, oy, oz,
                                       out_pairs != 0);
                    }
                }
                __syncthreads();
            }
        }
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
    }
    // drain: every pair copied must have landed before the CTA exits
    __syncthreads();
    if (producer) {
        // copies still in flight are among the last LF::RING issued (a slot is
        // refilled only after its previous copy was consumed)
        for (uint32_t f = ws.issued > (uint32_t)LF::RING ? ws.issued - LF::RING : 0u; f < ws.issued; ++f)
            if (!mbar_wait(&full[f % LF::RING], (f / LF::RING) & 1, WAIT_BUDGET)) {
                set_status(st, MLFF_ERR_TIMEOUT, 25);
                break;
            }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, LF::TMEM_COLS);
}

// UN-atom tiles, two CTAs per SM: one CTA's epilogues overlap the other's
// weight stream and MMAs
template <int UN>
static int launch_update_fwd_tc_t(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                                  cudaStream_t st) {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(update_fwd_tc_kernel<UN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        UFwd<UN>::SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "update_fwd_tc smem attribute");
    ProfScope prof(PK_UPDATE_FWD, st);
    const int64_t NX = (int64_t)L.N * 4 * H;
    const float* Xt = ws_ptr<float>(ws, L.Xt) + layer * NX;
    float* Xout = ws_ptr<float>(ws, L.X) + (layer + 1) * NX;
    float* uz = ws_ptr<float>(ws, L.uz) + (int64_t)layer * L.N * H;
    float* ua = ws_ptr<float>(ws, L.ua) + (int64_t)layer * L.N * H3;
    const int ntiles = (L.N + UN - 1) / UN;
    const int grid = std::max(1, std::min(ntiles, 2 * num_sms()));
    // the next layer's input in the pair layout of the edge kernels' gathers;
    // the last layer's output (read by the readout) component-major
    const int out_pairs = layer + 1 < L.L ? 1 : 0;
    MLFF_LAUNCH_PDL("update_fwd_tc", update_fwd_tc_kernel<UN>, grid, UNT, UFwd<UN>::SMEM, st, packed, lo, Xt, L.N,
                    Xout, out_pairs, uz, ua, ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

int launch_update_fwd_tc(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                         cudaStream_t st) {
    return L.UT == 32 ? launch_update_fwd_tc_t<32>(packed, lo, L, ws, layer, st)
                      : launch_update_fwd_tc_t<64>(packed, lo, L, ws, layer, st);
}

// ------------------------------------------------------- reverse kernel
// abar = dE/d(ds, g1, g2) [atom][3H] -> zbar = (U2^T abar) silu'(uz) ->
// cb = U1^T zbar = dE/d[s, |v|]; xtbar = (sb + cs, vb + cn v / |v|).
// smem: abar B tile (K = 384: 6 K-blocks, hi then lo, 96 KB), the zbar tile
// (K = 128, 32 KB) aliased into it after GEMM3, the ring (16 KB).
// TMEM: D3 = zbar pre-activation (cols 0..UN-1), D4 = (cs, cn) (UN + UN g).
template <int UN>
struct UBwd {
    static constexpr uint32_t AH = 6 * b_block(UN);
    static constexpr uint32_t ZH = 2 * b_block(UN);
    static constexpr int RING = UN == 64 ? 2 : 7;
    static constexpr uint32_t OFF_B = 0;
    static constexpr uint32_t OFF_RING = OFF_B + 2 * AH;
    static constexpr uint32_t OFF_MIX = OFF_RING + RING * A_PAIR;
    static constexpr uint32_t OFF_BAR = OFF_MIX + 64;
    static constexpr uint32_t OFF_MISC = OFF_BAR + 8 * (1 + 2 * RING);
    static constexpr uint32_t SMEM = align1k(OFF_MISC + 16);
    static constexpr uint32_t TMEM_COLS = UN == 64 ? 256 : 128;   // 3 UN columns, a power of two
    static_assert(2 * (SMEM + 1024) <= 228 * 1024, "two update reverse CTAs per SM");
    static_assert(2 * UN * H * 4 <= 2 * AH, "epilogue 4 stages (cs, cn) of the tile in the abar region");
};

template <int UN>
__global__ void __launch_bounds__(UNT, 2) update_bwd_tc_kernel(const float* __restrict__ P, LayerOffsets lo,
                                                               const float* __restrict__ Xt, const float* __restrict__ uz,
                                                               const float* __restrict__ ua,
                                                               const float* __restrict__ xbo, int32_t n_atoms,
                                                               float* __restrict__ xtbar, Status* st) {
    using LB = UBwd<UN>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* Bs = smem + LB::OFF_B;
    float* mix = reinterpret_cast<float*>(smem + LB::OFF_MIX);
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + LB::OFF_BAR);
    uint64_t* full = mma_bar + 1;
    uint64_t* empty = full + LB::RING;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + LB::OFF_MISC);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + LB::OFF_MISC + 4);
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const int ntiles = (n_atoms + UN - 1) / UN;
    if (w == 0) {
        tmem_alloc(tslot, LB::TMEM_COLS);
        tmem_relinquish();
    }
    if (t == 0) {
        mbar_init(mma_bar, 1);
        for (int i = 0; i < LB::RING; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        fence_mbar_init();
        *abort_flag = 0;
    }
    if (t < 9) mix[t] = P[lo.mix + t];
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    UStream<LB::RING> ws{smem + LB::OFF_RING, full, empty,
               {reinterpret_cast<const unsigned char*>(P + lo.u2t_tc), reinterpret_cast<const unsigned char*>(P + lo.u1t_tc)},
               {24, 16}, 0, 0};
    UCtl ctl{mma_bar, abort_flag, st, 0};
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint32_t P_end = (uint32_t)my_tiles * 40;
    const bool producer = t == 32;
    if (producer && !ustream_fill(ws, min((uint32_t)LB::RING, P_end))) ufail(ctl, 30);
    // everything above reads packed weights only and overlaps the previous kernel
    pdl_wait();
    if (t == 0 && st->code != 0) *abort_flag = 1;
    __syncthreads();
    pdl_trigger();
    const int q = w & 3, hh = w >> 2, c = 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t P0 = 0;

    for (int tile = blockIdx.x; tile < ntiles && !*abort_flag; tile += gridDim.x, P0 += 40) {
        const int a0 = tile * UN;
        // abar tile: row = atom; K = [sb, sum_i xb_i v_i, sum_i xb_i (M v)_i]; warp w builds
        // rows w, w + 8, ..., two rows per step so that their loads overlap
        auto gpart = [&](float b_x, float b_y, float b_z, float v_x, float v_y, float v_z, float& o1, float& o2) {
            o1 = b_x * v_x + b_y * v_y + b_z * v_z;
            o2 = b_x * (mix[0] * v_x + mix[1] * v_y + mix[2] * v_z) + b_y * (mix[3] * v_x + mix[4] * v_y + mix[5] * v_z) +
                 b_z * (mix[6] * v_x + mix[7] * v_y + mix[8] * v_z);
        };
#pragma unroll 1
        for (int i0 = w; i0 < UN; i0 += 16) {
            float4 r[2][7];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const int a = a0 + i0 + 8 * k;
                const int64_t aa = a < n_atoms ? a : 0;
                const float4* xo = reinterpret_cast<const float4*>(xbo + aa * 4 * H);
                const float4* x = reinterpret_cast<const float4*>(Xt + aa * 4 * H);
#pragma unroll
                for (int j = 0; j < 4; ++j) r[k][j] = a < n_atoms ? xo[32 * j + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int j = 1; j < 4; ++j) r[k][3 + j] = a < n_atoms ? x[32 * j + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                const float4 bx = r[k][1], by = r[k][2], bz = r[k][3], vx = r[k][4], vy = r[k][5], vz = r[k][6];
                float4 g1, g2;
                gpart(bx.x, by.x, bz.x, vx.x, vy.x, vz.x, g1.x, g2.x);
                gpart(bx.y, by.y, bz.y, vx.y, vy.y, vz.y, g1.y, g2.y);
                gpart(bx.z, by.z, bz.z, vx.z, vy.z, vz.z, g1.z, g2.z);
                gpart(bx.w, by.w, bz.w, vx.w, vy.w, vz.w, g1.w, g2.w);
                const int i = i0 + 8 * k;
                store_row4(Bs, LB::AH, UN, i, 4 * lane, r[k][0]);
                store_row4(Bs, LB::AH, UN, i, H + 4 * lane, g1);
                store_row4(Bs, LB::AH, UN, i, 2 * H + 4 * lane, g2);
            }
        }
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (t == 0) {   // GEMM3: zbar_pre^T = U2^T abar^T, K = 384
            fence_after_sync();
            const uint64_t b0 = sdesc_b(smem_u32(Bs));
            if (!ustream_gemm<UN>(ws, P0, 24, [&](int) { return tmem; },
                              [&](int i) { return b0 + (uint64_t)(b_kstep_off(UN, i) >> 4); }, (uint64_t)(LB::AH >> 4),
                              [](int i) { return i == 0; }))
                ufail(ctl, 31);
            mma_commit(mma_bar);
        }
        if (producer && !ustream_fill(ws, min(P0 + 24, P_end))) ufail(ctl, 36);
        uwait_mma(ctl, w, 32);
        if (producer && !ustream_fill(ws, min(P0 + 24 + LB::RING, P_end))) ufail(ctl, 37);
        {   // epilogue 3: zbar = D3 silu'(uz) -> zbar tile (aliases the abar tile)
            constexpr int NC = UN / 2;   // this warp half's atoms
            const int col = NC * hh;
            float zb[NC];
            if constexpr (NC == 32) tmem_ld32(lane_base + col, zb);
            else tmem_ld16(lane_base + col, zb);
            float zz[NC];
#pragma unroll
            for (int i = 0; i < NC; ++i) {
                const int a = a0 + col + i;
                zz[i] = a < n_atoms ? uz[(int64_t)a * H + c] : 0.f;
            }
            tmem_ld_wait();
            const BColumn zcol(Bs, LB::ZH, UN, col, c);
#pragma unroll
            for (int i = 0; i < NC; i += 2) zcol.put_pair(i, zb[i] * dsilu_f(zz[i]), zb[i + 1] * dsilu_f(zz[i + 1]));
        }
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (t == 0) {   // GEMM4: cb^T = U1^T zbar^T, 2 chunks x 8 K-steps
            fence_after_sync();
            const uint64_t b0 = sdesc_b(smem_u32(Bs));
            if (!ustream_gemm<UN>(ws, P0 + 24, 16, [&](int i) { return tmem + UN + UN * (i >> 3); },
                              [&](int i) { return b0 + (uint64_t)(b_kstep_off(UN, i & 7) >> 4); },
                              (uint64_t)(LB::ZH >> 4), [](int i) { return (i & 7) == 0; }))
                ufail(ctl, 33);
            mma_commit(mma_bar);
        }
        if (producer && !ustream_fill(ws, min(P0 + 40, P_end))) ufail(ctl, 38);
        uwait_mma(ctl, w, 34);
        if (producer && !ustream_fill(ws, min(P0 + 40 + LB::RING, P_end))) ufail(ctl, 39);
        {   // epilogue 4: xtbar = (sb + cs, xb g1 + M^T xb g2 + cn v / |v|).  The
            // TMEM owner of channel c writes (cs, cn) of its 32 atoms to shared
            // memory (the abar tile is free), then each warp handles whole atom
            // rows with 128-bit accesses.
            float* T = reinterpret_cast<float*>(Bs);      // [2][UN atoms][H]
#pragma unroll 1
            for (int g = 0; g < 2; ++g) {
                constexpr int NC = UN / 2;
                float v[NC];
                if constexpr (NC == 32) tmem_ld32(lane_base + UN + UN * g + NC * hh, v);
                else tmem_ld16(lane_base + UN + UN * g + NC * hh, v);
                tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < NC; ++i) T[(g * UN + NC * hh + i) * H + c] = v[i];
            }
            __syncthreads();
#pragma unroll 1
            for (int i0 = w; i0 < UN; i0 += 16) {
                float4 r[2][9];
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int a = a0 + i0 + 8 * k;
                    const int64_t aa = a < n_atoms ? a : 0;
                    const float4* xo = reinterpret_cast<const float4*>(xbo + aa * 4 * H);
                    const float4* x = reinterpret_cast<const float4*>(Xt + aa * 4 * H);
                    const float4* u = reinterpret_cast<const float4*>(ua + aa * H3);
#pragma unroll
                    for (int j = 0; j < 4; ++j) r[k][j] = xo[32 * j + lane];
#pragma unroll
                    for (int j = 1; j < 4; ++j) r[k][3 + j] = x[32 * j + lane];
                    r[k][7] = u[32 + lane];
                    r[k][8] = u[64 + lane];
                }
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int i = i0 + 8 * k, a = a0 + i;
                    if (a >= n_atoms) continue;
                    const float4 cs = reinterpret_cast<const float4*>(T + i * H)[lane];
                    const float4 cn = reinterpret_cast<const float4*>(T + (UN + i) * H)[lane];
                    const float4 sb = r[k][0], bx = r[k][1], by = r[k][2], bz = r[k][3];
                    const float4 vx = r[k][4], vy = r[k][5], vz = r[k][6], g1 = r[k][7], g2 = r[k][8];
                    float4 ox, oy, oz;
                    auto one = [&](float b_x, float b_y, float b_z, float v_x, float v_y, float v_z, float a1, float a2,
                                   float n_c, float& px, float& py, float& pz) {
                        const float nn = pair_distance(v_x, v_y, v_z);
                        const float sc = nn > 0.0f ? n_c / nn : 0.0f;   // d|v|/dv = v / |v|, 0 at v = 0
                        px = b_x * a1 + (mix[0] * b_x + mix[3] * b_y + mix[6] * b_z) * a2 + sc * v_x;
                        py = b_y * a1 + (mix[1] * b_x + mix[4] * b_y + mix[7] * b_z) * a2 + sc * v_y;
                        pz = b_z * a1 + (mix[2] * b_x + mix[5] * b_y + mix[8] * b_z) * a2 + sc * v_z;
                    };
                    one(bx.x, by.x, bz.x, vx.x, vy.x, vz.x, g1.x, g2.x, cn.x, ox.x, oy.x, oz.x);
                    one(bx.y, by.y, bz.y, vx.y, vy.y, vz.y, g1.y, g2.y, cn.y, ox.y, oy.y, oz.y);
                    one(bx.z, by.z, bz.z, vx.z, vy.z, vz.z, g1.z, g2.z, cn.z, ox.z, oy.z, oz.z);
                    one(bx.w, by.w, bz.w, vx.w, vy.w, vz.w, g1.w, g2.w, cn.w, ox.w, oy.w, oz.w);
                    // dE/dXt in the pair layout the reverse edge kernel gathers from
                    store_atom_row(xtbar + (int64_t)a * 4 * H, lane,
                                   make_float4(sb.x + cs.x, sb.y + cs.y, sb.z + cs.z, sb.w + cs.w), ox, oy, oz, true);
                }
            }
        }
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
    }
    __syncthreads();
    if (producer) {
        // copies still in flight are among the last LB::RING issued (a slot is
        // refilled only after its previous copy was consumed)
        for (uint32_t f = ws.issued > (uint32_t)LB::RING ? ws.issued - LB::RING : 0u; f < ws.issued; ++f)
            if (!mbar_wait(&full[f % LB::RING], (f / LB::RING) & 1, WAIT_BUDGET)) {
                set_status(st, MLFF_ERR_TIMEOUT, 35);
                break;
            }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (w == 0) tmem_dealloc(tmem, LB::TMEM_COLS);
}

template <int UN>
static int launch_update_bwd_tc_t(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                                  const float* xbar_out, float* xtbar, cudaStream_t st) {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(update_bwd_tc_kernel<UN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        UBwd<UN>::SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "update_bwd_tc smem attribute");
    ProfScope prof(PK_UPDATE_BWD, st);
    const int64_t NX = (int64_t)L.N * 4 * H;
    const float* Xt = ws_ptr<float>(ws, L.Xt) + layer * NX;
    const float* uz = ws_ptr<float>(ws, L.uz) + (int64_t)layer * L.N * H;
    const float* ua = ws_ptr<float>(ws, L.ua) + (int64_t)layer * L.N * H3;
    const int ntiles = (L.N + UN - 1) / UN;
    const int grid = std::max(1, std::min(ntiles, 2 * num_sms()));
    MLFF_LAUNCH_PDL("update_bwd_tc", update_bwd_tc_kernel<UN>, grid, UNT, UBwd<UN>::SMEM, st, packed, lo, Xt, uz, ua,
                    xbar_out, L.N, xtbar, ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

int launch_update_bwd_tc(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                         const float* xbar_out, float* xtbar, cudaStream_t st) {
    return L.UT == 32 ? launch_update_bwd_tc_t<32>(packed, lo, L, ws, layer, xbar_out, xtbar, st)
                      : launch_update_bwd_tc_t<64>(packed, lo, L, ws, layer, xbar_out, xtbar, st);
}

}  // namespace mlff
