// Kernels shared by both evaluation paths: weight packing, embedding,
// energy readout (forward + adjoint), per-structure FP64 energy sums, the
// fused per-atom update block (forward + adjoint, FP32 CUDA cores), and the
// force / virial gather from per-edge adjoints.
//
// Reference semantics (src/mlff_distiller/models/student_model.py):
//   embedding            :684
//   PaiNNUpdate.forward   :434-470  (|v| over xyz, MLP on [s, |v|], split
//                                     (ds, g1, g2), v' = v g1 + (M v) g2)
//   energy_head + sum     :599-605, :734-757
//   forces = -dE/dpos     :759-795
#include <cstdio>
#include <mutex>
#include "common.cuh"
#include "workspace.h"
#include "profile.h"

namespace mlff {

// ------------------------------------------------------------ weight pack
PackedOffsets packed_offsets(const mlff_dims& d) {
    PackedOffsets o{};
    int64_t p = 0;
    auto take = [&](int64_t n) {
        int64_t r = p;
        p += (n + 63) & ~int64_t(63);   // 256-byte alignment
        return r;
    };
    o.emb = take((int64_t)d.n_species * H);
    o.centers = take(RMAX);
    o.gamma = take(RMAX);
    o.head_w1t = take(H * 64);
    o.head_w1 = take(64 * H);
    o.head_b1 = take(64);
    o.head_w2t = take(64 * 32);
    o.head_w2 = take(32 * 64);
    o.head_b2 = take(32);
    o.head_w3 = take(32);
    o.head_b3 = take(1);
    for (int l = 0; l < d.n_layers; ++l) {
        LayerOffsets& L = o.layer[l];
        L.w1t = take(RMAX * H);
        L.w1 = take(H * RMAX);
        L.b1 = take(H);
        L.w2t = take(H * H3);
        L.w2 = take(H3 * H);
        L.b2 = take(H3);
        L.mix = take(9);
        L.u1t = take(2 * H * H);
        L.u1 = take(H * 2 * H);
        L.c1 = take(H);
        L.u2t = take(H * H3);
        L.u2 = take(H3 * H);
        L.c2 = take(H3);
        // split-fp16 operand tiles (hi and lo, 2 bytes per value) for the
        // tensor-core filter, W1 (H x RMAX) and W2 (H3 x H), and update MLP,
        // U1 and U2 in both orientations
        L.w1_bf = take(2 * H * RMAX / 2);
        L.w2_bf = take(2 * H3 * H / 2);
        L.w2_tm = take(4 * 32 * H);
        L.u1_tc = take(2 * H * 2 * H / 2);
        L.u2_tc = take(2 * H3 * H / 2);
        L.u2t_tc = take(2 * H3 * H / 2);
        L.u1t_tc = take(2 * H * 2 * H / 2);
        L.w2q_tc = take(2 * H * H / 2);
    }
    o.total = p;
    return o;
}

// dst[r][c] = src[c][r] (src rows x cols, zero-padded to dst_rows x dst_cols)
__global__ void transpose_pad_kernel(const float* __restrict__ src, int rows, int cols,
                                     float* __restrict__ dst, int dst_rows, int dst_cols) {
    // dst is [cols_pad][rows_pad]: dst[c * dst_cols + r] = src[r * cols + c]
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < dst_rows * dst_cols; i += gridDim.x * blockDim.x) {
        int c = i / dst_cols, r = i % dst_cols;
        dst[i] = (c < cols && r < rows) ? src[(int64_t)r * cols + c] : 0.0f;
    }
}

// dst [rows][dst_cols] = src [rows][cols] zero-padded columns
__global__ void copy_pad_kernel(const float* __restrict__ src, int rows, int cols,
                                float* __restrict__ dst, int dst_cols) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows * dst_cols; i += gridDim.x * blockDim.x) {
        int r = i / dst_cols, c = i % dst_cols;
        dst[i] = c < cols ? src[(int64_t)r * cols + c] : 0.0f;
    }
}

__global__ void rbf_pack_kernel(const float* __restrict__ centers, const float* __restrict__ widths, int R,
                                float* __restrict__ c_out, float* __restrict__ g_out) {
    int r = threadIdx.x;
    if (r < RMAX) {
        c_out[r] = r < R ? centers[r] : 0.0f;
        // gamma = 1 / w^2 as the reference computes it (student_model.py:253)
        g_out[r] = r < R ? 1.0f / (widths[r] * widths[r]) : 0.0f;
    }
}

int pack_fp32(const mlff_dims& d, const mlff_params& p, float* out, const PackedOffsets& o, cudaStream_t st) {
    const int R = d.n_rbf;
    auto cp = [&](float* dst, const float* src, int64_t n) -> int {
        MLFF_CUDA(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        return MLFF_OK;
    };
    auto tr = [&](const float* src, int rows, int cols, float* dst, int dst_rows, int dst_cols) -> int {
        // dst holds src^T padded: dst_rows >= cols, dst_cols >= rows
        transpose_pad_kernel<<<128, 256, 0, st>>>(src, rows, cols, dst, dst_rows, dst_cols);
        MLFF_LAUNCH_CHECK("transpose_pad");
        return MLFF_OK;
    };
    int r;
    if ((r = cp(out + o.emb, p.embedding, (int64_t)d.n_species * H))) return r;
    rbf_pack_kernel<<<1, RMAX, 0, st>>>(p.rbf_centers, p.rbf_widths, R, out + o.centers, out + o.gamma);
    MLFF_LAUNCH_CHECK("rbf_pack");
    if ((r = tr(p.head_w1, 64, H, out + o.head_w1t, H, 64))) return r;
    if ((r = cp(out + o.head_w1, p.head_w1, 64 * H))) return r;
    if ((r = cp(out + o.head_b1, p.head_b1, 64))) return r;
    if ((r = tr(p.head_w2, 32, 64, out + o.head_w2t, 64, 32))) return r;
    if ((r = cp(out + o.head_w2, p.head_w2, 32 * 64))) return r;
    if ((r = cp(out + o.head_b2, p.head_b2, 32))) return r;
    if ((r = cp(out + o.head_w3, p.head_w3, 32))) return r;
    if ((r = cp(out + o.head_b3, p.head_b3, 1))) return r;
    for (int l = 0; l < d.n_layers; ++l) {
        const LayerOffsets& L = o.layer[l];
        if ((r = tr(p.filter_w1[l], H, R, out + L.w1t, RMAX, H))) return r;
        copy_pad_kernel<<<64, 256, 0, st>>>(p.filter_w1[l], H, R, out + L.w1, RMAX);
        MLFF_LAUNCH_CHECK("copy_pad");
        if ((r = cp(out + L.b1, p.filter_b1[l], H))) return r;
        if ((r = tr(p.filter_w2[l], H3, H, out + L.w2t, H, H3))) return r;
        if ((r = cp(out + L.w2, p.filter_w2[l], (int64_t)H3 * H))) return r;
        if ((r = cp(out + L.b2, p.filter_b2[l], H3))) return r;
        if ((r = cp(out + L.mix, p.mixing[l], 9))) return r;
        if ((r = tr(p.update_w1[l], H, 2 * H, out + L.u1t, 2 * H, H))) return r;
        if ((r = cp(out + L.u1, p.update_w1[l], (int64_t)H * 2 * H))) return r;
        if ((r = cp(out + L.c1, p.update_b1[l], H))) return r;
        if ((r = tr(p.update_w2[l], H3, H, out + L.u2t, H, H3))) return r;
        if ((r = cp(out + L.u2, p.update_w2[l], (int64_t)H3 * H))) return r;
        if ((r = cp(out + L.c2, p.update_b2[l], H3))) return r;
    }
    return MLFF_OK;
}

// ------------------------------------------------------------- embedding
__global__ void embed_kernel(const float* __restrict__ emb, const int64_t* __restrict__ Z, int32_t n_atoms,
                             int32_t n_species, float* __restrict__ X, int pairs, Status* st) {
    pdl_wait();
    pdl_trigger();
    // X[a] = (emb[Z[a]], 0, 0, 0), component-major or in the pair layout
    const int64_t total = (int64_t)n_atoms * 4 * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = i / (4 * H);
        int q = (int)(i % (4 * H));
        const int comp = pairs ? 2 * (q / (2 * H)) + (q & 1) : q / H;
        const int ch = pairs ? (q % (2 * H)) / 2 : q % H;
        float v = 0.0f;
        if (comp == 0) {
            int64_t z = Z[a];
            if (z < 0 || z >= n_species) {
                set_status(st, MLFF_ERR_INVALID, (int)a);
                z = 0;
            }
            v = emb[z * H + ch];
        }
        X[i] = v;
    }
}

int launch_embed(const mlff_dims& d, const float* packed, const PackedOffsets& po, const mlff_system& sys,
                 const WsLayout& L, void* ws, cudaStream_t st, bool pairs) {
    ProfScope prof(PK_OTHER, st);
    MLFF_LAUNCH_PDL("embed", embed_kernel, 152 * 8, 256, 0, st, packed + po.emb, sys.Z, sys.n_atoms, d.n_species,
                    ws_ptr<float>(ws, L.X), pairs ? 1 : 0, ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

// ---------------------------------------------------------------- readout
// Per atom: E_a = w3 . silu(W2 silu(W1 s + b1) + b2) + b3 and, when
// requested, dE_a/ds written as the adjoint seed (v adjoint = 0).
// One CTA of 256 threads per SM walks groups of RO_ATOMS atoms; the head's
// four weight matrices (80 KB) are staged in shared memory once per CTA with
// independent 128-bit loads, so the dot products read shared memory only.
constexpr int RO_ATOMS = 32;
constexpr int RO_NT = 256;
// the head's weights transposed, rows padded by one float so that both the
// forward (threads along a row) and the backward products (threads along a
// column) read shared memory without bank conflicts; two CTAs per SM
constexpr int RO_W1T_LD = 64 + 1, RO_W2T_LD = 32 + 1;
constexpr int RO_W1T = 0;                       // [H][65]: W1T[i][o] = W1[o][i]
constexpr int RO_W2T = RO_W1T + H * RO_W1T_LD;  // [64][33]
constexpr int RO_S = ((RO_W2T + 64 * RO_W2T_LD) + 3) & ~3;   // [RO_ATOMS][H]     s (16-byte aligned)
constexpr int RO_Z1 = RO_S + RO_ATOMS * H;      // [RO_ATOMS][64]    z1
constexpr int RO_H1 = RO_Z1 + RO_ATOMS * 64;    // [RO_ATOMS][64]    silu(z1)
constexpr int RO_G1 = RO_H1 + RO_ATOMS * 64;    // [RO_ATOMS][64]    dE/dz1
constexpr int RO_Z2 = RO_G1 + RO_ATOMS * 64;    // [RO_ATOMS][32]    z2
constexpr int RO_G2 = RO_Z2 + RO_ATOMS * 32;    // [RO_ATOMS][32]    dE/dz2
constexpr int RO_FLOATS = RO_G2 + RO_ATOMS * 32;
constexpr size_t RO_SMEM = sizeof(float) * RO_FLOATS;

// rows x cols floats into rows of ld floats
__device__ __forceinline__ void ro_stage(float* dst, const float* __restrict__ src, int rows, int cols, int ld) {
    for (int i = threadIdx.x; i < rows * cols; i += RO_NT) dst[(i / cols) * ld + i % cols] = __ldg(src + i);
}

__global__ void __launch_bounds__(RO_NT, 2) readout_kernel(const float* __restrict__ P, PackedOffsets po,
                                                        const float* __restrict__ X, int32_t n_atoms,
                                                        float* __restrict__ e_atom, float* __restrict__ xbar,
                                                        int want_grad, const Status* st) {
    extern __shared__ __align__(16) float ro[];
    const int t = threadIdx.x;
    ro_stage(ro + RO_W1T, P + po.head_w1t, H, 64, RO_W1T_LD);
    ro_stage(ro + RO_W2T, P + po.head_w2t, 64, 32, RO_W2T_LD);
    pdl_wait();   // the weights above overlap the previous kernel
    pdl_trigger();
    if (st->code != 0) return;
    float* S = ro + RO_S;
    float* Z1 = ro + RO_Z1;
    float* H1 = ro + RO_H1;
    float* G1 = ro + RO_G1;
    float* Z2 = ro + RO_Z2;
    float* G2 = ro + RO_G2;
    for (int a0 = blockIdx.x * RO_ATOMS; a0 < n_atoms; a0 += gridDim.x * RO_ATOMS) {
        // s rows of the group (128-bit, one warp per atom row)
        for (int i = t; i < RO_ATOMS * (H / 4); i += RO_NT) {
            const int q = i / (H / 4), k = i % (H / 4), a = a0 + q;
            reinterpret_cast<float4*>(S + q * H)[k] =
                a < n_atoms ? __ldg(reinterpret_cast<const float4*>(X + (int64_t)a * 4 * H) + k)
                            : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        {   // z1 = W1 s + b1: thread -> output o, atoms 8 (t / 64) .. + 8
            const int o = t & 63, q0 = (t >> 6) * 8;
            float acc[8];
            const float b = P[po.head_b1 + o];
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[q] = b;
#pragma unroll 4
            for (int i = 0; i < H; i += 4) {
                const float w0 = ro[RO_W1T + (i + 0) * RO_W1T_LD + o], w1 = ro[RO_W1T + (i + 1) * RO_W1T_LD + o];
                const float w2 = ro[RO_W1T + (i + 2) * RO_W1T_LD + o], w3 = ro[RO_W1T + (i + 3) * RO_W1T_LD + o];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 x = *reinterpret_cast<const float4*>(S + (q0 + q) * H + i);
                    acc[q] = fmaf(w3, x.w, fmaf(w2, x.z, fmaf(w1, x.y, fmaf(w0, x.x, acc[q]))));
                }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                Z1[(q0 + q) * 64 + o] = acc[q];
                H1[(q0 + q) * 64 + o] = silu_f(acc[q]);
            }
        }
        __syncthreads();
        {   // z2 = W2 h1 + b2: thread -> output o, atoms 4 (t / 32) .. + 4
            const int o = t & 31, q0 = (t >> 5) * 4;
            float acc[4];
            const float b = P[po.head_b2 + o];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = b;
#pragma unroll 4
            for (int i = 0; i < 64; i += 4) {
                const float w0 = ro[RO_W2T + (i + 0) * RO_W2T_LD + o], w1 = ro[RO_W2T + (i + 1) * RO_W2T_LD + o];
                const float w2 = ro[RO_W2T + (i + 2) * RO_W2T_LD + o], w3 = ro[RO_W2T + (i + 3) * RO_W2T_LD + o];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 h = *reinterpret_cast<const float4*>(H1 + (q0 + q) * 64 + i);
                    acc[q] = fmaf(w3, h.w, fmaf(w2, h.z, fmaf(w1, h.y, fmaf(w0, h.x, acc[q]))));
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                Z2[(q0 + q) * 32 + o] = acc[q];
                // adjoint seed of the last layer: dE/dz2 = w3 * silu'(z2)
                G2[(q0 + q) * 32 + o] = P[po.head_w3 + o] * dsilu_f(acc[q]);
            }
        }
        __syncthreads();
        {   // E_a = w3 . silu(z2) + b3: warp w -> atoms 4w .. 4w + 3, lanes over the 32 inputs
            const int w = t >> 5, lane = t & 31;
            const float w3 = P[po.head_w3 + lane];
#pragma unroll
            for (int q = 4 * w; q < 4 * w + 4; ++q) {
                float e = w3 * silu_f(Z2[q * 32 + lane]);
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) e += __shfl_xor_sync(0xffffffffu, e, off);
                if (lane == 0 && a0 + q < n_atoms) e_atom[a0 + q] = e + P[po.head_b3];
            }
        }
        if (want_grad) {
            {   // dE/dz1 = (W2^T g2) * silu'(z1): thread -> output o, atoms 8 (t / 64) .. + 8
                const int o = t & 63, q0 = (t >> 6) * 8;
                float acc[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) acc[q] = 0.0f;
#pragma unroll 4
                for (int j = 0; j < 32; ++j) {
                    const float w = ro[RO_W2T + o * RO_W2T_LD + j];   // W2[j][o]
#pragma unroll
                    for (int q = 0; q < 8; ++q) acc[q] = fmaf(w, G2[(q0 + q) * 32 + j], acc[q]);
                }
#pragma unroll
                for (int q = 0; q < 8; ++q) G1[(q0 + q) * 64 + o] = acc[q] * dsilu_f(Z1[(q0 + q) * 64 + o]);
            }
            __syncthreads();
            {   // dE/ds = W1^T g1: thread -> output o, atoms 16 (t / 128) .. + 16
                const int o = t & 127, q0 = (t >> 7) * 16;
                float acc[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc[q] = 0.0f;
#pragma unroll 2
                for (int j = 0; j < 64; j += 4) {
                    const float* wr = ro + RO_W1T + o * RO_W1T_LD + j;   // W1[j .. j + 3][o]
                    const float w0 = wr[0], w1 = wr[1], w2 = wr[2], w3 = wr[3];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const float4 g = *reinterpret_cast<const float4*>(G1 + (q0 + q) * 64 + j);
                        acc[q] = fmaf(w3, g.w, fmaf(w2, g.z, fmaf(w1, g.y, fmaf(w0, g.x, acc[q]))));
                    }
                }
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int a = a0 + q0 + q;
                    if (a < n_atoms) xbar[(int64_t)a * 4 * H + o] = acc[q];
                }
            }
            // the vector part of the seed is zero
            for (int i = t; i < RO_ATOMS * (3 * H / 4); i += RO_NT) {
                const int q = i / (3 * H / 4), k = i % (3 * H / 4), a = a0 + q;
                if (a < n_atoms)
                    reinterpret_cast<float4*>(xbar + (int64_t)a * 4 * H + H)[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncthreads();
    }
}

// FP64 per-structure sums of per-atom energies (fixed-order tree)
__global__ void energy_sum_kernel(const float* __restrict__ e_atom, const int64_t* __restrict__ mol_ptr,
                                  int32_t n_mol, double* __restrict__ energy, const Status* st) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[256];
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        int64_t a0 = mol_ptr[m], a1 = mol_ptr[m + 1];
        double s = 0.0;
        for (int64_t a = a0 + threadIdx.x; a < a1; a += blockDim.x) s += (double)e_atom[a];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) energy[m] = st->code != 0 ? __longlong_as_double(0x7ff8000000000000ULL) : red[0];
        __syncthreads();
    }
}

int launch_readout(const mlff_dims& d, const float* packed, const PackedOffsets& po, const mlff_system& sys,
                   const WsLayout& L, void* ws, const mlff_outputs& out, int want_grad, cudaStream_t st) {
    ProfScope prof(PK_READOUT, st);
    const float* X = ws_ptr<float>(ws, L.X) + (int64_t)d.n_layers * sys.n_atoms * 4 * H;
    float* e_atom = ws_ptr<float>(ws, L.e_atom);
    float* xbar = ws_ptr<float>(ws, L.xbar);  // buffer 0
    const Status* status = ws_ptr<Status>(ws, L.status);
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
        attr_err = cudaFuncSetAttribute(readout_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RO_SMEM);
    });
    if (attr_err != cudaSuccess) return cuda_status(attr_err, "readout smem attribute");
    const int blocks = (int)std::min<int64_t>((sys.n_atoms + RO_ATOMS - 1) / RO_ATOMS, 2 * num_sms());
    MLFF_LAUNCH_PDL("readout", readout_kernel, std::max(blocks, 1), RO_NT, RO_SMEM, st, packed, po, X, sys.n_atoms,
                    e_atom, xbar, want_grad, status);
    MLFF_LAUNCH_PDL("energy_sum", energy_sum_kernel, std::min(std::max(sys.n_mol, 1), 152 * 8), 256, 0, st, e_atom, sys.mol_ptr, sys.n_mol,
                                                                                 out.energy, status);
    if (out.atom_energy)
        MLFF_CUDA(cudaMemcpyAsync(out.atom_energy, e_atom, sizeof(float) * sys.n_atoms, cudaMemcpyDeviceToDevice, st));
    return MLFF_OK;
}

// ------------------------------------------------------------ forces
// g = dE/dr for one directed edge from its accumulated adjoints:
// dE/dd (acc.x) and dE/du (acc.yzw), u = r / (d + 1e-8).
__device__ __forceinline__ float3 edge_grad(float4 acc, float3 r) {
    const float d = pair_distance(r.x, r.y, r.z);
    if (d == 0.0f) return make_float3(0.f, 0.f, 0.f);
    const float inv_d = 1.0f / d;
    const float inv_de = 1.0f / (d + 1e-8f);
    const float ur = acc.y * r.x + acc.z * r.y + acc.w * r.z;
    const float c = ur * inv_d * inv_de * inv_de;
    return make_float3(acc.x * r.x * inv_d + acc.y * inv_de - c * r.x,
                       acc.x * r.y * inv_d + acc.z * inv_de - c * r.y,
                       acc.x * r.z * inv_d + acc.w * inv_de - c * r.z);
}

// One warp per receiver atom: lane l takes edges l, l + 32, ... of the row
// (independent loads across lanes), then a fixed-order shuffle reduction.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void forces_kernel(const float4* __restrict__ pos4, const int32_t* __restrict__ atom_mol,
                              const float* __restrict__ box, const uint8_t* __restrict__ pbc,
                              const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                              const int32_t* __restrict__ rev, const float4* __restrict__ acc,
                              int32_t n_atoms, float* __restrict__ forces, double* __restrict__ vir_atom,
                              VerletFuse vf, const Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    const int lane = threadIdx.x & 31;
    if (vf.step_counter && blockIdx.x == 0 && threadIdx.x == 0) *vf.step_counter += 1;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n_atoms; a += nw) {
        const int m = atom_mol[a];
        Box b;
        b.periodic = (pbc != nullptr && box != nullptr && pbc[m]) ? 1 : 0;
        for (int q = 0; q < 3; ++q) {
            b.L[q] = b.periodic ? box[3 * m + q] : 1.0f;
            b.invL[q] = __fdiv_rn(1.0f, b.L[q]);
        }
        const float4 pa = pos4[a];
        float fx = 0.f, fy = 0.f, fz = 0.f;
        double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = row_ptr[a] + lane; k < row_ptr[a + 1]; k += 32) {
            const int bb = col[k];
            const float3 r = edge_vector(pos4[bb], pa, b);         // sender bb -> receiver a
            const float3 g = edge_grad(acc[k], r);
            const float3 gr = edge_grad(acc[rev[k]], make_float3(-r.x, -r.y, -r.z));
            fx += g.x - gr.x;
            fy += g.y - gr.y;
            fz += g.z - gr.z;
            if (vir_atom) {
                const float gg[3] = {g.x, g.y, g.z}, rr[3] = {r.x, r.y, r.z};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) v[3 * i + j] += (double)gg[i] * (double)rr[j];
            }
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        if (forces && lane == 0) {
            forces[3 * a] = fx;
            forces[3 * a + 1] = fy;
            forces[3 * a + 2] = fz;
        }
        if (vf.vel && lane < 3) {   // the integrator's update of this atom, lane = component
            const double im = vf.inv_mass[a];
            const float f = lane == 0 ? fx : (lane == 1 ? fy : fz);
            const int64_t i = 3 * (int64_t)a + lane;
            const double v = verlet_half_kick(vf.vel[i], f, im, vf.dt);   // closes this step
            if (vf.ke_atom) {
                const double vx = __shfl_sync(0x7u, v, 0), vy = __shfl_sync(0x7u, v, 1), vz = __shfl_sync(0x7u, v, 2);
                if (lane == 0) vf.ke_atom[a] = kinetic_term(vx, vy, vz, im);
            }
            if (vf.open_next) {   // the next step's half kick and drift
                const double vn = verlet_half_kick(v, f, im, vf.dt);
                vf.vel[i] = vn;
                const double p = vf.pos[i] + vf.dt * vn;
                vf.pos[i] = p;
                vf.pos32[i] = (float)p;
            } else {
                vf.vel[i] = v;
            }
        }
        if (vir_atom) {
#pragma unroll
            for (int i = 0; i < 9; ++i) v[i] = warp_sum_d(v[i]);
            if (lane == 0)
                for (int i = 0; i < 9; ++i) vir_atom[(int64_t)9 * a + i] = v[i];
        }
    }
}

__global__ void virial_sum_kernel(const double* __restrict__ vir_atom, const int64_t* __restrict__ mol_ptr,
                                  int32_t n_mol, double* __restrict__ virial, const Status* st) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[9][128];
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int64_t a = mol_ptr[m] + threadIdx.x; a < mol_ptr[m + 1]; a += blockDim.x)
            for (int i = 0; i < 9; ++i) s[i] += vir_atom[9 * a + i];
        for (int i = 0; i < 9; ++i) red[i][threadIdx.x] = s[i];
        __syncthreads();
        for (int o = 64; o > 0; o >>= 1) {
            if (threadIdx.x < o)
                for (int i = 0; i < 9; ++i) red[i][threadIdx.x] += red[i][threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x < 9) virial[9 * m + threadIdx.x] = st->code != 0 ? 0.0 : red[threadIdx.x][0];
        __syncthreads();
    }
}

int launch_forces(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws,
                  const mlff_outputs& out, cudaStream_t st, const VerletFuse* vf) {
    (void)d;
    ProfScope prof(PK_FORCES, st);
    const Status* status = ws_ptr<Status>(ws, L.status);
    // per-atom virial scratch reuses the second adjoint buffer (free by now)
    double* vir_atom = out.virial ? reinterpret_cast<double*>(ws_ptr<float>(ws, L.xbar) + (int64_t)sys.n_atoms * 4 * H)
                                  : nullptr;
    int blocks = (int)std::min<int64_t>((sys.n_atoms + 3) / 4, 152 * 16);   // 4 atoms (warps) per block
    MLFF_LAUNCH_PDL("forces", forces_kernel, std::max(blocks, 1), 128, 0, st, 
        ws_ptr<float4>(ws, L.pos4), ws_ptr<int32_t>(ws, L.atom_mol), sys.box, sys.pbc,
        ws_ptr<int32_t>(ws, L.row_ptr), ws_ptr<int32_t>(ws, L.col), ws_ptr<int32_t>(ws, L.rev),
        ws_ptr<float4>(ws, L.edge_acc), sys.n_atoms, out.forces, vir_atom, vf ? *vf : VerletFuse{}, status);
    if (out.virial) {
        MLFF_LAUNCH_PDL("virial_sum", virial_sum_kernel, std::min(std::max(sys.n_mol, 1), 152 * 8), 128, 0, st, vir_atom, sys.mol_ptr, sys.n_mol,
                                                                                      out.virial, status);
    }
    return MLFF_OK;
}

// ------------------------------------------------------- update (fused)
// One block of 128 threads handles UPD_ATOMS atoms at a time.  Thread c owns
// channel c.  Saves the pre-activation z (uz) and the MLP output (ua) for
// the adjoint.
constexpr int UPD_ATOMS = 16;

__global__ void __launch_bounds__(128) update_fwd_kernel(const float* __restrict__ P, LayerOffsets lo,
                                                         const float* __restrict__ Xt, int32_t n_atoms,
                                                         float* __restrict__ Xout, float* __restrict__ uz,
                                                         float* __restrict__ ua, const Status* st) {
    __shared__ float comb[UPD_ATOMS][2 * H];
    __shared__ float hsm[UPD_ATOMS][H];
    __shared__ float mix[9];
    if (st->code != 0) return;
    const int c = threadIdx.x;
    if (c < 9) mix[c] = P[lo.mix + c];
    const float* U1t = P + lo.u1t;   // [2H][H]
    const float* U2t = P + lo.u2t;   // [H][3H]
    for (int a0 = blockIdx.x * UPD_ATOMS; a0 < n_atoms; a0 += gridDim.x * UPD_ATOMS) {
        float sv[UPD_ATOMS], vx[UPD_ATOMS], vy[UPD_ATOMS], vz[UPD_ATOMS];
#pragma unroll
        for (int q = 0; q < UPD_ATOMS; ++q) {
            int a = a0 + q;
            if (a < n_atoms) {
                const float* x = Xt + (int64_t)a * 4 * H;
                sv[q] = x[c]; vx[q] = x[H + c]; vy[q] = x[2 * H + c]; vz[q] = x[3 * H + c];
            } else {
                sv[q] = vx[q] = vy[q] = vz[q] = 0.0f;
            }
            comb[q][c] = sv[q];
            comb[q][H + c] = pair_distance(vx[q], vy[q], vz[q]);   // |v| over xyz (student_model.py:437)
        }
        __syncthreads();
        {
            float acc[UPD_ATOMS];
            const float bias = P[lo.c1 + c];
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) acc[q] = bias;
            for (int i = 0; i < 2 * H; i += 4) {
                float w0 = U1t[(i + 0) * H + c], w1 = U1t[(i + 1) * H + c];
                float w2 = U1t[(i + 2) * H + c], w3 = U1t[(i + 3) * H + c];
#pragma unroll
                for (int q = 0; q < UPD_ATOMS; ++q) {
                    float4 x = *reinterpret_cast<const float4*>(&comb[q][i]);
                    acc[q] = fmaf(w0, x.x, acc[q]);
                    acc[q] = fmaf(w1, x.y, acc[q]);
                    acc[q] = fmaf(w2, x.z, acc[q]);
                    acc[q] = fmaf(w3, x.w, acc[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) {
                int a = a0 + q;
                if (a < n_atoms) uz[(int64_t)a * H + c] = acc[q];
                hsm[q][c] = silu_f(acc[q]);
            }
        }
        __syncthreads();
        float o[3][UPD_ATOMS];
#pragma unroll
        for (int g = 0; g < 3; ++g) {
            const float bias = P[lo.c2 + g * H + c];
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) o[g][q] = bias;
        }
        for (int k = 0; k < H; k += 4) {
            float w[3][4];
#pragma unroll
            for (int g = 0; g < 3; ++g)
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) w[g][kk] = U2t[(k + kk) * H3 + g * H + c];
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) {
                float4 h = *reinterpret_cast<const float4*>(&hsm[q][k]);
#pragma unroll
                for (int g = 0; g < 3; ++g) {
                    o[g][q] = fmaf(w[g][0], h.x, o[g][q]);
                    o[g][q] = fmaf(w[g][1], h.y, o[g][q]);
                    o[g][q] = fmaf(w[g][2], h.z, o[g][q]);
                    o[g][q] = fmaf(w[g][3], h.w, o[g][q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < UPD_ATOMS; ++q) {
            int a = a0 + q;
            if (a >= n_atoms) continue;
            float* uo = ua + (int64_t)a * H3;
            uo[c] = o[0][q];
            uo[H + c] = o[1][q];
            uo[2 * H + c] = o[2][q];
            // s' = s + ds ; v' = v g1 + (M v) g2  (student_model.py:452-468)
            const float v3[3] = {vx[q], vy[q], vz[q]};
            float* xo = Xout + (int64_t)a * 4 * H;
            xo[c] = sv[q] + o[0][q];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                float mv = mix[3 * i] * v3[0] + mix[3 * i + 1] * v3[1] + mix[3 * i + 2] * v3[2];
                xo[(1 + i) * H + c] = v3[i] * o[1][q] + mv * o[2][q];
            }
        }
        __syncthreads();
    }
}

// Adjoint of the update block: from dE/dX' (xbar_out) to dE/dXt (xtbar).
__global__ void __launch_bounds__(128) update_bwd_kernel(const float* __restrict__ P, LayerOffsets lo,
                                                         const float* __restrict__ Xt, const float* __restrict__ uz,
                                                         const float* __restrict__ ua,
                                                         const float* __restrict__ xbar_out, int32_t n_atoms,
                                                         float* __restrict__ xtbar, const Status* st) {
    __shared__ float abar[UPD_ATOMS][H3];
    __shared__ float zbar[UPD_ATOMS][H];
    __shared__ float mix[9];
    if (st->code != 0) return;
    const int c = threadIdx.x;
    if (c < 9) mix[c] = P[lo.mix + c];
    __syncthreads();
    const float* U2 = P + lo.u2;   // [3H][H]
    const float* U1 = P + lo.u1;   // [H][2H]
    for (int a0 = blockIdx.x * UPD_ATOMS; a0 < n_atoms; a0 += gridDim.x * UPD_ATOMS) {
        float sb[UPD_ATOMS], vb[3][UPD_ATOMS], vt[3][UPD_ATOMS];
#pragma unroll
        for (int q = 0; q < UPD_ATOMS; ++q) {
            int a = a0 + q;
            float xv[3] = {0, 0, 0}, xb[3] = {0, 0, 0}, g1 = 0, g2 = 0, sbo = 0;
            if (a < n_atoms) {
                const float* x = Xt + (int64_t)a * 4 * H;
                const float* xo = xbar_out + (int64_t)a * 4 * H;
                const float* u = ua + (int64_t)a * H3;
                sbo = xo[c];
#pragma unroll
                for (int i = 0; i < 3; ++i) { xv[i] = x[(1 + i) * H + c]; xb[i] = xo[(1 + i) * H + c]; }
                g1 = u[H + c];
                g2 = u[2 * H + c];
            }
            float mv[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) mv[i] = mix[3 * i] * xv[0] + mix[3 * i + 1] * xv[1] + mix[3 * i + 2] * xv[2];
            abar[q][c] = sbo;
            abar[q][H + c] = xb[0] * xv[0] + xb[1] * xv[1] + xb[2] * xv[2];
            abar[q][2 * H + c] = xb[0] * mv[0] + xb[1] * mv[1] + xb[2] * mv[2];
            sb[q] = sbo;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                // dv_i = xb_i g1 + sum_j M[j][i] xb_j g2
                vb[i][q] = xb[i] * g1 + (mix[i] * xb[0] + mix[3 + i] * xb[1] + mix[6 + i] * xb[2]) * g2;
                vt[i][q] = xv[i];
            }
        }
        __syncthreads();
        {
            float acc[UPD_ATOMS];
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) acc[q] = 0.0f;
            for (int j = 0; j < H3; j += 4) {
                float w0 = U2[(j + 0) * H + c], w1 = U2[(j + 1) * H + c];
                float w2 = U2[(j + 2) * H + c], w3 = U2[(j + 3) * H + c];
#pragma unroll
                for (int q = 0; q < UPD_ATOMS; ++q) {
                    float4 x = *reinterpret_cast<const float4*>(&abar[q][j]);
                    acc[q] = fmaf(w0, x.x, acc[q]);
                    acc[q] = fmaf(w1, x.y, acc[q]);
                    acc[q] = fmaf(w2, x.z, acc[q]);
                    acc[q] = fmaf(w3, x.w, acc[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) {
                int a = a0 + q;
                float z = a < n_atoms ? uz[(int64_t)a * H + c] : 0.0f;
                zbar[q][c] = acc[q] * dsilu_f(z);
            }
        }
        __syncthreads();
        float cs[UPD_ATOMS], cn[UPD_ATOMS];
#pragma unroll
        for (int q = 0; q < UPD_ATOMS; ++q) { cs[q] = 0.0f; cn[q] = 0.0f; }
        for (int k = 0; k < H; k += 4) {
            float ws_[4], wn[4];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                ws_[kk] = U1[(k + kk) * 2 * H + c];
                wn[kk] = U1[(k + kk) * 2 * H + H + c];
            }
#pragma unroll
            for (int q = 0; q < UPD_ATOMS; ++q) {
                float4 z = *reinterpret_cast<const float4*>(&zbar[q][k]);
                cs[q] = fmaf(ws_[0], z.x, cs[q]); cn[q] = fmaf(wn[0], z.x, cn[q]);
                cs[q] = fmaf(ws_[1], z.y, cs[q]); cn[q] = fmaf(wn[1], z.y, cn[q]);
                cs[q] = fmaf(ws_[2], z.z, cs[q]); cn[q] = fmaf(wn[2], z.z, cn[q]);
                cs[q] = fmaf(ws_[3], z.w, cs[q]); cn[q] = fmaf(wn[3], z.w, cn[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < UPD_ATOMS; ++q) {
            int a = a0 + q;
            if (a >= n_atoms) continue;
            float n = pair_distance(vt[0][q], vt[1][q], vt[2][q]);
            float sc = n > 0.0f ? cn[q] / n : 0.0f;     // d|v|/dv = v/|v|, 0 at v = 0
            float* o = xtbar + (int64_t)a * 4 * H;
            o[c] = sb[q] + cs[q];
#pragma unroll
            for (int i = 0; i < 3; ++i) o[(1 + i) * H + c] = vb[i][q] + sc * vt[i][q];
        }
        __syncthreads();
    }
}

int launch_update_fwd(const mlff_dims& d, const float* packed, const LayerOffsets& lo, const WsLayout& L,
                      void* ws, int layer, cudaStream_t st) {
    (void)d;
    ProfScope prof(PK_UPDATE_FWD, st);
    const int64_t NX = (int64_t)L.N * 4 * H;
    const float* Xt = ws_ptr<float>(ws, L.Xt) + layer * NX;
    float* Xout = ws_ptr<float>(ws, L.X) + (layer + 1) * NX;
    float* uz = ws_ptr<float>(ws, L.uz) + (int64_t)layer * L.N * H;
    float* ua = ws_ptr<float>(ws, L.ua) + (int64_t)layer * L.N * H3;
    int blocks = (int)std::min<int64_t>((L.N + UPD_ATOMS - 1) / UPD_ATOMS, 152 * 4);
    update_fwd_kernel<<<std::max(blocks, 1), 128, 0, st>>>(packed, lo, Xt, L.N, Xout, uz, ua,
                                                           ws_ptr<Status>(ws, L.status));
    MLFF_LAUNCH_CHECK("update_fwd");
    return MLFF_OK;
}

int launch_update_bwd(const mlff_dims& d, const float* packed, const LayerOffsets& lo, const WsLayout& L,
                      void* ws, int layer, const float* xbar_out, float* xtbar, cudaStream_t st) {
    (void)d;
    ProfScope prof(PK_UPDATE_BWD, st);
    const int64_t NX = (int64_t)L.N * 4 * H;
    const float* Xt = ws_ptr<float>(ws, L.Xt) + layer * NX;
    const float* uz = ws_ptr<float>(ws, L.uz) + (int64_t)layer * L.N * H;
    const float* ua = ws_ptr<float>(ws, L.ua) + (int64_t)layer * L.N * H3;
    int blocks = (int)std::min<int64_t>((L.N + UPD_ATOMS - 1) / UPD_ATOMS, 152 * 4);
    update_bwd_kernel<<<std::max(blocks, 1), 128, 0, st>>>(packed, lo, Xt, uz, ua, xbar_out, L.N, xtbar,
                                                           ws_ptr<Status>(ws, L.status));
    MLFF_LAUNCH_CHECK("update_bwd");
    return MLFF_OK;
}

}  // namespace mlff
