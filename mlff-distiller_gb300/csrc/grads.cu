// Parameter gradients of sum_b w_b E_b for training (the parameter part of
// loss.backward() in Trainer.train_epoch, training/trainer.py:288-393, for
// the energy term of ForceFieldLoss, training/losses.py:106-246).
//
// They hang off the plain FP32 path's reverse pass (plain.cu), which keeps
// every per-op intermediate the reductions need: the readout adjoint is
// scaled per structure by w_b, and at each layer the weight gradients are
// reductions over atoms or edges of an adjoint times a forward activation:
//   filter   dW2 = sum_e fbar_e (x) silu(z_e)   db2 = sum_e fbar_e
//            dW1 = sum_e zbar_e (x) rbf_e        db1 = sum_e zbar_e
//   update   dU2 = sum_a abar_a (x) silu(uz_a)  dc2 = sum_a abar_a
//            dU1 = sum_a zbar_a (x) [s, |v|]_a   dc1 = sum_a zbar_a
//            dM_ij = sum_a,c xbar'_{v_i,c} g2_c v_{j,c}
//   readout  the three Linear layers of energy_head, per atom
//   embedding dEmb[z] = sum_{a: Z_a = z} dE/ds_a of the layer-0 input.
// Every reduction here adds in a fixed order (fixed row splits, partial
// sums written to a scratch buffer and added in split order); the inputs
// come from the plain path, whose message scatter-adds are float atomics.
//
// The same reductions over Dual scalars (the plain path's tangent pass,
// dual.cuh) give the derivative of grad_theta E along positions moved by
// -G and cells strained by S; their tangent part is added to the gradient
// outputs: sum_i G_i . dF_i/dtheta + sum_b S_b : dW_b/dtheta, the parameter
// gradient of a force / stress loss with dL/dF = G, dL/dW = S (the
// second-order term of loss.backward() through forces and strain
// derivatives taken with create_graph=True).
#include "common.cuh"
#include "dual.cuh"
#include "workspace.h"
#include "profile.h"

namespace mlff {

// ------------------------------------------------ generic A^T B reduction
// partial[split][m][k] = sum over rows n of split: A[n][m] * op(B[n][k]),
// op = identity (BOP 0), silu (BOP 1) or 1 (BOP 2: column sums of A, K = 1).
// 32 x 32 output tile per block, 2 x 2 per thread, rows staged 32 at a time.
template <int BOP, class T>
__global__ void __launch_bounds__(256) wgrad_partial_kernel(const T* __restrict__ A, int lda,
                                                            const T* __restrict__ B, int ldb, int M, int K,
                                                            int64_t n_static, const int32_t* __restrict__ n_dev,
                                                            T* __restrict__ partial, const Status* st) {
    __shared__ T As[32][33];
    __shared__ T Bs[32][33];
    if (st->code != 0) return;
    const int64_t n = n_dev ? (int64_t)(*n_dev) : n_static;
    const int tiles_k = (K + 31) / 32;
    const int m0 = (blockIdx.x / tiles_k) * 32, k0 = (blockIdx.x % tiles_k) * 32;
    const int split = blockIdx.y;
    const int64_t per = (n + GRAD_SPLIT - 1) / GRAD_SPLIT;
    const int64_t r0 = split * per, r1 = min(n, r0 + per);
    const int t = threadIdx.x, tm = t >> 4, tk = t & 15;
    T acc[2][2] = {{T{}, T{}}, {T{}, T{}}};
    for (int64_t n0 = r0; n0 < r1; n0 += 32) {
        for (int i = t; i < 32 * 32; i += 256) {
            const int rr = i >> 5, cc = i & 31;
            const int64_t row = n0 + rr;
            const bool okr = row < r1;
            As[rr][cc] = (okr && m0 + cc < M) ? A[row * lda + m0 + cc] : T{};
            T b = T{};
            if (okr && k0 + cc < K) {
                if (BOP == 2) b = tone<T>();
                else {
                    b = B[row * ldb + k0 + cc];
                    if (BOP == 1) b = tsilu(b);
                }
            }
            Bs[rr][cc] = b;
        }
        __syncthreads();
#pragma unroll 8
        for (int i = 0; i < 32; ++i) {
            const T a0 = As[i][2 * tm], a1 = As[i][2 * tm + 1];
            const T b0 = Bs[i][2 * tk], b1 = Bs[i][2 * tk + 1];
            acc[0][0] = tfma(a0, b0, acc[0][0]);
            acc[0][1] = tfma(a0, b1, acc[0][1]);
            acc[1][0] = tfma(a1, b0, acc[1][0]);
            acc[1][1] = tfma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    T* out = partial + (int64_t)split * M * K;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int m = m0 + 2 * tm + i, k = k0 + 2 * tk + j;
            if (m < M && k < K) out[(int64_t)m * K + k] = acc[i][j];
        }
}

// float: out = the sum; Dual: out += the tangent of the sum
__device__ __forceinline__ void grad_store(float* out, float s) { *out = s; }
__device__ __forceinline__ void grad_store(float* out, Dual s) { *out += s.t; }

template <class T>
__global__ void wgrad_reduce_kernel(const T* __restrict__ partial, int64_t MK, float* __restrict__ out,
                                    const Status* st) {
    if (st->code != 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < MK; i += (int64_t)gridDim.x * blockDim.x) {
        T s = T{};
        for (int sp = 0; sp < GRAD_SPLIT; ++sp) s = s + partial[(int64_t)sp * MK + i];
        grad_store(out + i, s);
    }
}

// out[M][K] = sum_n A[n][m] op(B[n][k]) (out NULL: nothing to do)
template <int BOP, class T>
static int wgrad(const T* A, int lda, const T* B, int ldb, int M, int K, int64_t n, const int32_t* n_dev,
                 float* out, const WsLayout& L, void* ws, cudaStream_t st) {
    if (!out) return MLFF_OK;
    T* part = ws_ptr<T>(ws, L.gpart);
    const Status* status = ws_ptr<Status>(ws, L.status);
    dim3 grid(((M + 31) / 32) * ((K + 31) / 32), GRAD_SPLIT);
    wgrad_partial_kernel<BOP, T><<<grid, 256, 0, st>>>(A, lda, B, ldb, M, K, n, n_dev, part, status);
    MLFF_LAUNCH_CHECK("wgrad_partial");
    const int64_t MK = (int64_t)M * K;
    wgrad_reduce_kernel<T><<<(int)std::min<int64_t>((MK + 255) / 256, 152 * 4), 256, 0, st>>>(part, MK, out, status);
    MLFF_LAUNCH_CHECK("wgrad_reduce");
    return MLFF_OK;
}

// ------------------------------------------------------------- readout
// Per atom (one thread per hidden unit, RO_G atoms per block): recompute
// z1 = W1 s + b1, z2 = W2 silu(z1) + b2 and the adjoints for the seed
// w = w_b of the atom's structure: ebar = w, a2bar = w w3 silu'(z2),
// a1bar = (W2^T a2bar) silu'(z1); store h1, a1bar, h2, a2bar, ebar.
// float: scale the unit-seed adjoint dE_a/ds (xbar, written by the readout)
// by w.  Dual (w NULL: unit seed): write the adjoint xbar = (W1^T a1bar, 0).
constexpr int RO_G = 8;
template <class T>
__global__ void __launch_bounds__(128) readout_grad_kernel(const float* __restrict__ P, PackedOffsets po,
                                                           const T* __restrict__ X, const int32_t* __restrict__ atom_mol,
                                                           const double* __restrict__ w, int32_t n_atoms,
                                                           T* __restrict__ ghead, T* __restrict__ xbar,
                                                           const Status* st) {
    constexpr bool DUAL = is_dual_v<T>;
    __shared__ T s_in[RO_G][H];
    __shared__ T z1[RO_G][64];
    __shared__ T z2[RO_G][32];
    __shared__ T g2[RO_G][32];
    __shared__ T g1[DUAL ? RO_G : 1][64];
    if (st->code != 0) return;
    const int t = threadIdx.x;
    auto weight = [&](int a) -> float { return w ? (float)w[atom_mol[a]] : 1.0f; };
    for (int a0 = blockIdx.x * RO_G; a0 < n_atoms; a0 += gridDim.x * RO_G) {
        for (int q = 0; q < RO_G; ++q) {
            const int a = a0 + q;
            s_in[q][t] = a < n_atoms ? X[(int64_t)a * 4 * H + t] : T{};
        }
        __syncthreads();
        if (t < 64) {
            for (int q = 0; q < RO_G; ++q) {
                T acc = tmake<T>(P[po.head_b1 + t], 0.0f);
                for (int i = 0; i < H; ++i) acc = tfma(P[po.head_w1t + i * 64 + t], s_in[q][i], acc);
                z1[q][t] = acc;
            }
        }
        __syncthreads();
        if (t < 32) {
            for (int q = 0; q < RO_G; ++q) {
                T acc = tmake<T>(P[po.head_b2 + t], 0.0f);
                for (int i = 0; i < 64; ++i) acc = tfma(P[po.head_w2t + i * 32 + t], tsilu(z1[q][i]), acc);
                z2[q][t] = acc;
                const int a = a0 + q;
                const float wq = a < n_atoms ? weight(a) : 0.f;
                g2[q][t] = wq * P[po.head_w3 + t] * tdsilu(acc);
            }
        }
        __syncthreads();
        for (int q = 0; q < RO_G; ++q) {
            const int a = a0 + q;
            if (a >= n_atoms) continue;
            T* gh = ghead + (int64_t)a * 193;
            if (t < 64) {
                T acc = T{};
                for (int j = 0; j < 32; ++j) acc = tfma(P[po.head_w2 + j * 64 + t], g2[q][j], acc);
                gh[t] = tsilu(z1[q][t]);
                const T a1 = acc * tdsilu(z1[q][t]);
                gh[64 + t] = a1;
                if constexpr (DUAL) g1[q][t] = a1;
            } else if (t < 96) {
                gh[128 + (t - 64)] = tsilu(z2[q][t - 64]);
                gh[160 + (t - 64)] = g2[q][t - 64];
            } else if (t == 96) {
                gh[192] = tmake<T>(weight(a), 0.0f);
            }
            if constexpr (!DUAL) {
                const float wq = weight(a);
                xbar[(int64_t)a * 4 * H + t] *= wq;
            }
        }
        if constexpr (DUAL) {
            __syncthreads();
            for (int q = 0; q < RO_G; ++q) {
                const int a = a0 + q;
                if (a >= n_atoms) continue;
                T acc = T{};
                for (int j = 0; j < 64; ++j) acc = tfma(P[po.head_w1 + j * H + t], g1[q][j], acc);
                T* xb = xbar + (int64_t)a * 4 * H;
                xb[t] = acc;
                xb[H + t] = T{};
                xb[2 * H + t] = T{};
                xb[3 * H + t] = T{};
            }
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------- embedding
// dEmb[z][c] = sum over atoms of species z of xbar0[a][c] (s part), in atom
// order; one block per species.
template <class T>
__global__ void embed_grad_kernel(const int64_t* __restrict__ Z, const T* __restrict__ xbar0, int32_t n_atoms,
                                  int32_t n_species, float* __restrict__ out, const Status* st) {
    if (st->code != 0) return;
    for (int z = blockIdx.x; z < n_species; z += gridDim.x) {
        T acc = T{};
        for (int a = 0; a < n_atoms; ++a)
            if (Z[a] == z) acc = acc + xbar0[(int64_t)a * 4 * H + threadIdx.x];
        grad_store(out + (int64_t)z * H + threadIdx.x, acc);
    }
}

// -------------------------------------------------------------- mixing
// v' = v g1 + (M v) g2 (student_model.py:452-468): dM_ij = sum_a,c
// xbar'_{v_i}[a][c] g2[a][c] v_j[a][c]; per-block partials, then a
// fixed-order sum.
template <class T>
__global__ void __launch_bounds__(256) mix_grad_partial_kernel(const T* __restrict__ Xt,
                                                               const T* __restrict__ ua,
                                                               const T* __restrict__ xbo, int32_t n_atoms,
                                                               T* __restrict__ part, const Status* st) {
    __shared__ T red[9][256];
    if (st->code != 0) return;
    T acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = T{};
    const int64_t total = (int64_t)n_atoms * H;
    for (int64_t i = blockIdx.x * 256 + threadIdx.x; i < total; i += (int64_t)gridDim.x * 256) {
        const int64_t a = i / H;
        const int c = (int)(i % H);
        const T g2 = ua[a * H3 + 2 * H + c];
        const T* x = Xt + a * 4 * H;
        const T* xb = xbo + a * 4 * H;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int j = 0; j < 3; ++j) acc[3 * r + j] = tfma(xb[(1 + r) * H + c] * g2, x[(1 + j) * H + c], acc[3 * r + j]);
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
#pragma unroll
            for (int k = 0; k < 9; ++k) red[k][threadIdx.x] = red[k][threadIdx.x] + red[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 9) part[blockIdx.x * 9 + threadIdx.x] = red[threadIdx.x][0];
}

template <class T>
__global__ void mix_grad_reduce_kernel(const T* __restrict__ part, float* __restrict__ out, const Status* st) {
    if (st->code != 0) return;
    if (threadIdx.x < 9) {
        T s = T{};
        for (int b = 0; b < GRAD_MIX_BLOCKS; ++b) s = s + part[b * 9 + threadIdx.x];
        grad_store(out + threadIdx.x, s);
    }
}

// ------------------------------------------------------------ launchers
template <class T>
int grad_readout(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
                 const WsLayout& L, void* ws, const double* w, const mlff_grads& g, cudaStream_t st) {
    ProfScope prof(PK_OTHER, st);
    const int N = sys.n_atoms;
    const T* XL = ws_ptr<T>(ws, L.X) + (int64_t)d.n_layers * N * 4 * H;
    T* gh = ws_ptr<T>(ws, L.ghead);
    T* xbar0 = ws_ptr<T>(ws, L.xbar);
    const Status* status = ws_ptr<Status>(ws, L.status);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((N + RO_G - 1) / RO_G, 152 * 8));
    readout_grad_kernel<T><<<blocks, 128, 0, st>>>(P, po, XL, ws_ptr<int32_t>(ws, L.atom_mol), w, N, gh, xbar0,
                                                   status);
    MLFF_LAUNCH_CHECK("readout_grad");
    int r;
    // energy_head.0: [64][128] = sum a1bar (x) s ; energy_head.2: [32][64] = sum a2bar (x) h1 ; .4: [1][32]
    if ((r = wgrad<0, T>(gh + 64, 193, XL, 4 * H, 64, H, N, nullptr, g.head_w1, L, ws, st))) return r;
    if ((r = wgrad<2, T>(gh + 64, 193, nullptr, 0, 64, 1, N, nullptr, g.head_b1, L, ws, st))) return r;
    if ((r = wgrad<0, T>(gh + 160, 193, gh, 193, 32, 64, N, nullptr, g.head_w2, L, ws, st))) return r;
    if ((r = wgrad<2, T>(gh + 160, 193, nullptr, 0, 32, 1, N, nullptr, g.head_b2, L, ws, st))) return r;
    if ((r = wgrad<0, T>(gh + 192, 193, gh + 128, 193, 1, 32, N, nullptr, g.head_w3, L, ws, st))) return r;
    return wgrad<2, T>(gh + 192, 193, nullptr, 0, 1, 1, N, nullptr, g.head_b3, L, ws, st);
}

// after the update reverse prologue: abar = dE/d(ds, g1, g2) [N][3H]
template <class T>
int grad_update_out(const WsLayout& L, void* ws, int l, const T* xbo, const mlff_grads& g, cudaStream_t st) {
    ProfScope prof(PK_OTHER, st);
    const int N = L.N;
    const T* abar = ws_ptr<T>(ws, L.abar);
    const T* uz = ws_ptr<T>(ws, L.uz) + (int64_t)l * N * H;
    const T* ua = ws_ptr<T>(ws, L.ua) + (int64_t)l * N * H3;
    const T* Xt = ws_ptr<T>(ws, L.Xt) + (int64_t)l * N * 4 * H;
    int r;
    if ((r = wgrad<1, T>(abar, H3, uz, H, H3, H, N, nullptr, g.update_w2[l], L, ws, st))) return r;
    if ((r = wgrad<2, T>(abar, H3, nullptr, 0, H3, 1, N, nullptr, g.update_b2[l], L, ws, st))) return r;
    if (g.mixing[l]) {
        const Status* status = ws_ptr<Status>(ws, L.status);
        T* part = ws_ptr<T>(ws, L.gmix);
        mix_grad_partial_kernel<T><<<GRAD_MIX_BLOCKS, 256, 0, st>>>(Xt, ua, xbo, N, part, status);
        MLFF_LAUNCH_CHECK("mix_grad");
        mix_grad_reduce_kernel<T><<<1, 32, 0, st>>>(part, g.mixing[l], status);
        MLFF_LAUNCH_CHECK("mix_grad_reduce");
    }
    return MLFF_OK;
}

// after zbar_u = (abar U2) silu'(uz) is in uh [N][H]; comb_l = [s, |v|] of Xt_l in gcomb
template <class T>
int grad_update_in(const WsLayout& L, void* ws, int l, const T* zbar_u, const T* comb_l, const mlff_grads& g,
                   cudaStream_t st) {
    ProfScope prof(PK_OTHER, st);
    const int N = L.N;
    int r;
    if ((r = wgrad<0, T>(zbar_u, H, comb_l, 2 * H, H, 2 * H, N, nullptr, g.update_w1[l], L, ws, st))) return r;
    return wgrad<2, T>(zbar_u, H, nullptr, 0, H, 1, N, nullptr, g.update_b1[l], L, ws, st);
}

// after the message reverse: fbar [cap][3H]; z of layer l in fz
template <class T>
int grad_filter_out(const WsLayout& L, void* ws, int l, const int32_t* E_dev, const mlff_grads& g, cudaStream_t st) {
    ProfScope prof(PK_OTHER, st);
    const T* fbar = ws_ptr<T>(ws, L.fbar);
    const T* z = ws_ptr<T>(ws, L.fz) + (int64_t)l * L.cap * H;
    int r;
    if ((r = wgrad<1, T>(fbar, H3, z, H, H3, H, L.cap, E_dev, g.filter_w2[l], L, ws, st))) return r;
    return wgrad<2, T>(fbar, H3, nullptr, 0, H3, 1, L.cap, E_dev, g.filter_b2[l], L, ws, st);
}

// after zbar_f = (fbar W2) silu'(z) is in fh [cap][H]
template <class T>
int grad_filter_in(const mlff_dims& d, const WsLayout& L, void* ws, int l, const int32_t* E_dev, const mlff_grads& g,
                   cudaStream_t st) {
    ProfScope prof(PK_OTHER, st);
    const T* zbar = ws_ptr<T>(ws, L.fh);
    const T* erbf = ws_ptr<T>(ws, L.erbf);
    int r;
    if ((r = wgrad<0, T>(zbar, H, erbf, RMAX, H, d.n_rbf, L.cap, E_dev, g.filter_w1[l], L, ws, st))) return r;
    return wgrad<2, T>(zbar, H, nullptr, 0, H, 1, L.cap, E_dev, g.filter_b1[l], L, ws, st);
}

template <class T>
int grad_embedding(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws, const T* xbar0,
                   const mlff_grads& g, cudaStream_t st) {
    if (!g.embedding) return MLFF_OK;
    ProfScope prof(PK_OTHER, st);
    embed_grad_kernel<T><<<std::min(d.n_species, 152 * 4), H, 0, st>>>(sys.Z, xbar0, sys.n_atoms, d.n_species,
                                                                        g.embedding, ws_ptr<Status>(ws, L.status));
    MLFF_LAUNCH_CHECK("embed_grad");
    return MLFF_OK;
}

#define MLFF_GRAD_INSTANTIATE(T)                                                                                    \
    template int grad_readout<T>(const mlff_dims&, const float*, const PackedOffsets&, const mlff_system&,          \
                                 const WsLayout&, void*, const double*, const mlff_grads&, cudaStream_t);          \
    template int grad_update_out<T>(const WsLayout&, void*, int, const T*, const mlff_grads&, cudaStream_t);       \
    template int grad_update_in<T>(const WsLayout&, void*, int, const T*, const T*, const mlff_grads&,              \
                                   cudaStream_t);                                                                  \
    template int grad_filter_out<T>(const WsLayout&, void*, int, const int32_t*, const mlff_grads&, cudaStream_t); \
    template int grad_filter_in<T>(const mlff_dims&, const WsLayout&, void*, int, const int32_t*,                  \
                                   const mlff_grads&, cudaStream_t);                                               \
    template int grad_embedding<T>(const mlff_dims&, const mlff_system&, const WsLayout&, void*, const T*,         \
                                   const mlff_grads&, cudaStream_t);
MLFF_GRAD_INSTANTIATE(float)
MLFF_GRAD_INSTANTIATE(Dual)
#undef MLFF_GRAD_INSTANTIATE

}  // namespace mlff
