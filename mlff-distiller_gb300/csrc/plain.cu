// Plain FP32 path: one kernel per operation of the reference's graph
// (src/mlff_distiller/models/student_model.py:706-757), with per-edge
// tensors materialised in HBM and messages scattered with atomics, the way
// index_add_ runs on a GPU.  Forces come from a hand-written reverse pass
// over the same operations (no autograd).  This is the FP32 CUDA-core
// comparator for the fused tensor-core path.
//
// The kernels are templates over the scalar type T: float is the plain
// path; Dual (dual.cuh) runs the same graph on (value, tangent) pairs for
// the force-matching term of the training loss, where the tangent is the
// derivative along a direction G of the atom positions.
#include "common.cuh"
#include "dual.cuh"
#include "workspace.h"
#include "profile.h"

namespace mlff {

constexpr float PI_F = 3.14159265358979f;

// ------------------------------------------------------------- geometry
// u = r / (d + 1e-8), d = |r| (:709-715); e = rbf(d) * fc(d) (:718-722) and
// de/dd for the reverse pass.  Dual: the edge vector's tangent is
// -(pos_t[b] - pos_t[a]) (positions moved along -G, G = pos_t [N][3],
// optional; F = -dE/dpos) plus S_m r for a strain direction S_m [B][3][3]
// (optional; positions and image shifts scale with the cell, so every
// edge vector r becomes (I + eps S_m) r).
template <class T>
__global__ void pl_geom_kernel(const float4* __restrict__ pos4, const float* __restrict__ pos_t,
                               const double* __restrict__ strain_t,
                               const int32_t* __restrict__ atom_mol,
                               const float* __restrict__ box, const uint8_t* __restrict__ pbc,
                               const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                               const int32_t* __restrict__ erecv, int32_t n_atoms,
                               const float* __restrict__ centers, const float* __restrict__ gamma,
                               int R, float cutoff, Vec4<T>* __restrict__ geo, T* __restrict__ erbf,
                               T* __restrict__ erbf_d, const Status* st) {
    if (st->code != 0) return;
    const int32_t E = row_ptr[n_atoms];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
        const int a = erecv[k], b = col[k];
        const int m = atom_mol[a];
        Box bx;
        bx.periodic = (pbc != nullptr && box != nullptr && pbc[m]) ? 1 : 0;
        for (int q = 0; q < 3; ++q) {
            bx.L[q] = bx.periodic ? box[3 * m + q] : 1.0f;
            bx.invL[q] = __fdiv_rn(1.0f, bx.L[q]);
        }
        const float3 r0 = edge_vector(pos4[b], pos4[a], bx);
        float tx = 0.0f, ty = 0.0f, tz = 0.0f;
        if (is_dual_v<T> && pos_t) {
            // a position direction leaves the image shift alone: r' = -(G_b - G_a)
            tx = pos_t[3 * a] - pos_t[3 * b];
            ty = pos_t[3 * a + 1] - pos_t[3 * b + 1];
            tz = pos_t[3 * a + 2] - pos_t[3 * b + 2];
        }
        if (is_dual_v<T> && strain_t) {
            const double* S = strain_t + 9 * m;
            tx += (float)(S[0] * r0.x + S[1] * r0.y + S[2] * r0.z);
            ty += (float)(S[3] * r0.x + S[4] * r0.y + S[5] * r0.z);
            tz += (float)(S[6] * r0.x + S[7] * r0.y + S[8] * r0.z);
        }
        const T rx = tmake<T>(r0.x, tx), ry = tmake<T>(r0.y, ty), rz = tmake<T>(r0.z, tz);
        const T d = tdist(rx, ry, rz);
        const T inv = 1.0f / (d + 1e-8f);
        geo[k] = tvec4(rx * inv, ry * inv, rz * inv, d);
        const T arg = PI_F * d / cutoff;
        const bool inside = tval(d) < cutoff;
        const T fc = inside ? 0.5f * (tcos(arg) + 1.0f) : T{};
        const T dfc = inside ? -0.5f * (PI_F / cutoff) * tsin(arg) : T{};
        T* e = erbf + (int64_t)k * RMAX;
        T* ed = erbf_d + (int64_t)k * RMAX;
        for (int q = 0; q < RMAX; ++q) {
            if (q < R) {
                const T diff = d - centers[q];
                const T g = texp(-gamma[q] * diff * diff);
                e[q] = g * fc;
                ed[q] = g * (dfc - 2.0f * gamma[q] * diff * fc);
            } else {
                e[q] = T{};
                ed[q] = T{};
            }
        }
    }
}

// ---------------------------------------------------------------- SGEMM
// C[M][N] = A[M][K] * B[K][N] (row-major, contiguous) with an epilogue:
//   0: C = acc + bias
//   1: C = acc + bias, C2 = silu(C)
//   2: C = acc * silu'(Z)          (Z same shape as C)
// M may be a device value (edge count) read through m_dev.  B and bias are
// weights (float); A, C, C2 and Z have the scalar type T.
constexpr int SG_BM = 64, SG_BN = 64, SG_BK = 16;

template <int MODE, class T>
__global__ void __launch_bounds__(256) sgemm_kernel(const T* __restrict__ A, const float* __restrict__ B,
                                                    const float* __restrict__ bias, T* __restrict__ C,
                                                    T* __restrict__ C2, const T* __restrict__ Z,
                                                    int64_t M_static, const int32_t* __restrict__ m_dev,
                                                    int N, int K, const Status* st) {
    __shared__ T As[SG_BK][SG_BM + 4];
    __shared__ float Bs[SG_BK][SG_BN];
    if (st->code != 0) return;
    const int64_t M = m_dev ? (int64_t)(*m_dev) : M_static;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int n_tiles = (N + SG_BN - 1) / SG_BN;
    const int64_t m_tiles = (M + SG_BM - 1) / SG_BM;
    for (int64_t tile = blockIdx.x; tile < m_tiles * n_tiles; tile += gridDim.x) {
        const int64_t m0 = (tile / n_tiles) * SG_BM;
        const int n0 = (int)(tile % n_tiles) * SG_BN;
        T acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = T{};
        for (int k0 = 0; k0 < K; k0 += SG_BK) {
            // A tile: 64 x 16 -> 256 threads x 4
            for (int i = threadIdx.x; i < SG_BM * SG_BK; i += 256) {
                int r = i / SG_BK, kk = i % SG_BK;
                int64_t gm = m0 + r;
                As[kk][r] = (gm < M && k0 + kk < K) ? A[gm * K + k0 + kk] : T{};
            }
            for (int i = threadIdx.x; i < SG_BK * SG_BN; i += 256) {
                int kk = i / SG_BN, c = i % SG_BN;
                int gn = n0 + c;
                Bs[kk][c] = (gn < N && k0 + kk < K) ? B[(int64_t)(k0 + kk) * N + gn] : 0.0f;
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < SG_BK; ++kk) {
                T a[4];
                float b[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = tfma(a[i], b[j], acc[i][j]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t gm = m0 + ty * 4 + i;
            if (gm >= M) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int gn = n0 + tx * 4 + j;
                if (gn >= N) continue;
                const int64_t idx = gm * N + gn;
                T v = acc[i][j];
                if (MODE == 0 || MODE == 1) v = v + (bias ? bias[gn] : 0.0f);
                if (MODE == 2) v = v * tdsilu(Z[idx]);
                C[idx] = v;
                if (MODE == 1) C2[idx] = tsilu(v);
            }
        }
    }
}

// M sizes the grid; when m_dev is given the kernel reads the actual row
// count there (M is then the capacity bound).
template <int MODE, class T>
static int sgemm(const T* A, const float* B, const float* bias, T* C, T* C2, const T* Z,
                 int64_t M, const int32_t* m_dev, int N, int K, const Status* st, cudaStream_t s) {
    const int64_t tiles = ((M + SG_BM - 1) / SG_BM) * ((N + SG_BN - 1) / SG_BN);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, 152 * 8));
    ProfScope prof(PK_PLAIN_GEMM, s);
    sgemm_kernel<MODE, T><<<blocks, 256, 0, s>>>(A, B, bias, C, C2, Z, M, m_dev, N, K, st);
    MLFF_LAUNCH_CHECK("sgemm");
    return MLFF_OK;
}

// ------------------------------------------------------------- message
// Xt[a] = X[a] + sum over receiver a's edges (index_add_, :359-385) of
// X[src] * phi, in edge order: one block per receiver row (the edges are
// receiver-sorted), thread c = channel, so the sums are deterministic.
template <class T>
__global__ void __launch_bounds__(128) pl_message_kernel(const T* __restrict__ X, const T* __restrict__ F,
                                                         const Vec4<T>* __restrict__ geo,
                                                         const int32_t* __restrict__ col,
                                                         const int32_t* __restrict__ row_ptr, int32_t n_atoms,
                                                         T* __restrict__ Xt, const Status* st) {
    if (st->code != 0) return;
    const int c = threadIdx.x;
    for (int a = blockIdx.x; a < n_atoms; a += gridDim.x) {
        const T* xa = X + (int64_t)a * 4 * H;
        T s = xa[c], v0 = xa[H + c], v1 = xa[2 * H + c], v2 = xa[3 * H + c];
        const int k1 = row_ptr[a + 1];
        for (int k = row_ptr[a]; k < k1; ++k) {
            const T* xs = X + (int64_t)col[k] * 4 * H;
            const T* f = F + (int64_t)k * H3;
            const Vec4<T> g = geo[k];
            const T f1 = f[H + c], f2 = f[2 * H + c];
            s = s + xs[c] * f[c];
            v0 = v0 + (xs[H + c] * f1 + g.x * f2);
            v1 = v1 + (xs[2 * H + c] * f1 + g.y * f2);
            v2 = v2 + (xs[3 * H + c] * f1 + g.z * f2);
        }
        T* xt = Xt + (int64_t)a * 4 * H;
        xt[c] = s;
        xt[H + c] = v0;
        xt[2 * H + c] = v1;
        xt[3 * H + c] = v2;
    }
}

// Node adjoints of the message step: dE/dX[b] = dE/dXt[b] + sum over the
// edges k with sender b of (dE/dXt[a].s phi_s(k), dE/dXt[a].v phi_v1(k)),
// a the receiver of k.  Gathered from b's own receiver row instead of
// scattered from the senders: the edge k' = (a -> b) of that row is the
// reverse of k and has the same filter (the same distance, bit for bit), so
// the sum runs over b's row in order -- one block per atom, thread c =
// channel, deterministic.
template <class T>
__global__ void __launch_bounds__(128) pl_message_bwd_nodes_kernel(const T* __restrict__ F,
                                                                   const int32_t* __restrict__ col,
                                                                   const int32_t* __restrict__ row_ptr,
                                                                   int32_t n_atoms, const T* __restrict__ xtbar,
                                                                   T* __restrict__ xbar, const Status* st) {
    if (st->code != 0) return;
    const int c = threadIdx.x;
    for (int b = blockIdx.x; b < n_atoms; b += gridDim.x) {
        const T* tb = xtbar + (int64_t)b * 4 * H;
        T s = tb[c], v0 = tb[H + c], v1 = tb[2 * H + c], v2 = tb[3 * H + c];
        const int k1 = row_ptr[b + 1];
        for (int k = row_ptr[b]; k < k1; ++k) {
            const T* ta = xtbar + (int64_t)col[k] * 4 * H;
            const T* f = F + (int64_t)k * H3;
            const T f1 = f[H + c];
            s = s + ta[c] * f[c];
            v0 = v0 + ta[H + c] * f1;
            v1 = v1 + ta[2 * H + c] * f1;
            v2 = v2 + ta[3 * H + c] * f1;
        }
        T* ob = xbar + (int64_t)b * 4 * H;
        ob[c] = s;
        ob[H + c] = v0;
        ob[2 * H + c] = v1;
        ob[3 * H + c] = v2;
    }
}

// ------------------------------------------------------------- update
template <class T>
__global__ void pl_update_pre_kernel(const T* __restrict__ Xt, int32_t n_atoms, T* __restrict__ comb,
                                     const Status* st) {
    if (st->code != 0) return;
    const int64_t total = (int64_t)n_atoms * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = i / H;
        const int c = (int)(i % H);
        const T* x = Xt + a * 4 * H;
        comb[a * 2 * H + c] = x[c];
        comb[a * 2 * H + H + c] = tdist(x[H + c], x[2 * H + c], x[3 * H + c]);
    }
}

template <class T>
__global__ void pl_update_post_kernel(const T* __restrict__ Xt, const T* __restrict__ ua,
                                      const float* __restrict__ mix_g, int32_t n_atoms, T* __restrict__ Xo,
                                      const Status* st) {
    if (st->code != 0) return;
    float mix[9];
    for (int q = 0; q < 9; ++q) mix[q] = mix_g[q];
    const int64_t total = (int64_t)n_atoms * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = i / H;
        const int c = (int)(i % H);
        const T* x = Xt + a * 4 * H;
        const T* u = ua + a * H3;
        T* o = Xo + a * 4 * H;
        const T v[3] = {x[H + c], x[2 * H + c], x[3 * H + c]};
        o[c] = x[c] + u[c];
        for (int q = 0; q < 3; ++q) {
            const T mv = mix[3 * q] * v[0] + mix[3 * q + 1] * v[1] + mix[3 * q + 2] * v[2];
            o[(1 + q) * H + c] = v[q] * u[H + c] + mv * u[2 * H + c];
        }
    }
}

// reverse of the gates and mixing: abar (dE/d(ds,g1,g2)) and the direct
// parts of dE/dXt
template <class T>
__global__ void pl_update_bwd_pre_kernel(const T* __restrict__ Xt, const T* __restrict__ ua,
                                         const float* __restrict__ mix_g, const T* __restrict__ xbo,
                                         int32_t n_atoms, T* __restrict__ abar, T* __restrict__ xtbar,
                                         const Status* st) {
    if (st->code != 0) return;
    float mix[9];
    for (int q = 0; q < 9; ++q) mix[q] = mix_g[q];
    const int64_t total = (int64_t)n_atoms * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = i / H;
        const int c = (int)(i % H);
        const T* x = Xt + a * 4 * H;
        const T* u = ua + a * H3;
        const T* xb = xbo + a * 4 * H;
        const T v[3] = {x[H + c], x[2 * H + c], x[3 * H + c]};
        const T vb[3] = {xb[H + c], xb[2 * H + c], xb[3 * H + c]};
        T mv[3];
        for (int q = 0; q < 3; ++q) mv[q] = mix[3 * q] * v[0] + mix[3 * q + 1] * v[1] + mix[3 * q + 2] * v[2];
        abar[a * H3 + c] = xb[c];
        abar[a * H3 + H + c] = vb[0] * v[0] + vb[1] * v[1] + vb[2] * v[2];
        abar[a * H3 + 2 * H + c] = vb[0] * mv[0] + vb[1] * mv[1] + vb[2] * mv[2];
        T* o = xtbar + a * 4 * H;
        o[c] = xb[c];
        const T g1 = u[H + c], g2 = u[2 * H + c];
        for (int q = 0; q < 3; ++q)
            o[(1 + q) * H + c] = vb[q] * g1 + (mix[q] * vb[0] + mix[3 + q] * vb[1] + mix[6 + q] * vb[2]) * g2;
    }
}

// xtbar += d[s,|v|] terms: cb = dE/d(comb) [N][2H]
template <class T>
__global__ void pl_update_bwd_post_kernel(const T* __restrict__ Xt, const T* __restrict__ cb,
                                          int32_t n_atoms, T* __restrict__ xtbar, const Status* st) {
    if (st->code != 0) return;
    const int64_t total = (int64_t)n_atoms * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = i / H;
        const int c = (int)(i % H);
        const T* x = Xt + a * 4 * H;
        T* o = xtbar + a * 4 * H;
        o[c] = o[c] + cb[a * 2 * H + c];
        const T v[3] = {x[H + c], x[2 * H + c], x[3 * H + c]};
        const T n = tdist(v[0], v[1], v[2]);
        const T sc = tval(n) > 0.0f ? cb[a * 2 * H + H + c] / n : T{};
        for (int q = 0; q < 3; ++q) o[(1 + q) * H + c] = o[(1 + q) * H + c] + sc * v[q];
    }
}

// ---------------------------------------------------- message reverse
// Per edge k (sender b -> receiver a), channel c:
//   fbar[k] = (xtb_a.s * x_b.s, sum_i xtb_a.v_i * x_b.v_i, sum_i xtb_a.v_i * u_i)
//   dE/du_k += sum_c xtb_a.v * phi_v2                    (block reduction)
// (the node adjoints xbar_b: pl_message_bwd_nodes_kernel)
// The dE/du accumulation feeds the forces only; the Dual instantiation
// (parameter gradients of the force loss) leaves it out.
constexpr int MB_EDGES = 8;
template <class T>
__global__ void __launch_bounds__(128) pl_message_bwd_kernel(const T* __restrict__ X, const T* __restrict__ F,
                                                             const Vec4<T>* __restrict__ geo,
                                                             const int32_t* __restrict__ col,
                                                             const int32_t* __restrict__ erecv,
                                                             const int32_t* __restrict__ E_dev,
                                                             const T* __restrict__ xtbar, T* __restrict__ fbar,
                                                             float4* __restrict__ eacc, const Status* st) {
    __shared__ float red[4][MB_EDGES][3];
    if (st->code != 0) return;
    const int c = threadIdx.x, lane = c & 31, w = c >> 5;
    const int64_t E = *E_dev;
    for (int64_t k0 = (int64_t)blockIdx.x * MB_EDGES; k0 < E; k0 += (int64_t)gridDim.x * MB_EDGES) {
        float pu[MB_EDGES][3];
#pragma unroll
        for (int q = 0; q < MB_EDGES; ++q) {
            const int64_t k = k0 + q;
            pu[q][0] = pu[q][1] = pu[q][2] = 0.0f;
            if (k >= E) continue;
            const int a = erecv[k], b = col[k];
            const T* xb = X + (int64_t)b * 4 * H;
            const T* ta = xtbar + (int64_t)a * 4 * H;
            const T* f = F + k * H3;
            const Vec4<T> g = geo[k];
            const T tas = ta[c], tv0 = ta[H + c], tv1 = ta[2 * H + c], tv2 = ta[3 * H + c];
            T* fb = fbar + k * H3;
            fb[c] = tas * xb[c];
            fb[H + c] = tv0 * xb[H + c] + tv1 * xb[2 * H + c] + tv2 * xb[3 * H + c];
            fb[2 * H + c] = tv0 * g.x + tv1 * g.y + tv2 * g.z;
            if constexpr (!is_dual_v<T>) {
                const T f2 = f[2 * H + c];
                pu[q][0] = tv0 * f2;
                pu[q][1] = tv1 * f2;
                pu[q][2] = tv2 * f2;
            }
        }
        if constexpr (!is_dual_v<T>) {
#pragma unroll
            for (int q = 0; q < MB_EDGES; ++q)
#pragma unroll
                for (int x = 0; x < 3; ++x) {
                    float v = pu[q][x];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) red[w][q][x] = v;
                }
            __syncthreads();
            if (c < MB_EDGES) {
                const int64_t k = k0 + c;
                if (k < E) {
                    float4 acc = eacc[k];
                    acc.y += red[0][c][0] + red[1][c][0] + red[2][c][0] + red[3][c][0];
                    acc.z += red[0][c][1] + red[1][c][1] + red[2][c][1] + red[3][c][1];
                    acc.w += red[0][c][2] + red[1][c][2] + red[2][c][2] + red[3][c][2];
                    eacc[k] = acc;
                }
            }
            __syncthreads();
        }
    }
}

// dE/dd_k += sum_r ebar[k][r] * de_r/dd
__global__ void pl_dd_kernel(const float* __restrict__ ebar, const float* __restrict__ erbf_d,
                             const int32_t* __restrict__ E_dev, float4* __restrict__ eacc, const Status* st) {
    if (st->code != 0) return;
    const int64_t E = *E_dev;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < E; k += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int r = 0; r < RMAX; ++r) s += ebar[k * RMAX + r] * erbf_d[k * RMAX + r];
        eacc[k].x += s;
    }
}

template <class T>
__global__ void copy_kernel(const T* __restrict__ src, T* __restrict__ dst, int64_t n, const Status* st) {
    if (st->code != 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// Dual layer-0 input: X = ((emb[Z], 0), 0, 0, 0) -- the embedding does not
// depend on the positions.
__global__ void pl_embed_dual_kernel(const float* __restrict__ emb, const int64_t* __restrict__ Z, int32_t n_atoms,
                                     int32_t n_species, Dual* __restrict__ X, Status* st) {
    if (st->code != 0) return;
    const int64_t total = (int64_t)n_atoms * 4 * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = i / (4 * H);
        const int q = (int)(i % (4 * H));
        float v = 0.0f;
        if (q < H) {
            int64_t z = Z[a];
            if (z < 0 || z >= n_species) {
                set_status(st, MLFF_ERR_INVALID, (int)a);
                z = 0;
            }
            v = emb[z * H + q];
        }
        X[i] = Dual{v, 0.0f};
    }
}

// One pass of the plain path over scalars T.  float: energies, the
// reverse pass for forces (and, with grad, the parameter gradients of
// sum_b w_b E_b).  Dual (grad required; pos_t the position direction G
// and / or strain_t the strain direction S): the same graph with unit
// seeds along (-G, S); the weight-gradient reductions add the tangent of
// grad_theta E, i.e. sum_i G_i . dF_i/dtheta + sum_b S_b : dW_b/dtheta.
template <class T>
static int run_plain_t(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
                       const WsLayout& L, void* ws, const mlff_outputs& out, cudaStream_t st, const GradCtx* grad,
                       const float* pos_t, const double* strain_t, const VerletFuse* vf = nullptr) {
    constexpr bool DUAL = is_dual_v<T>;
    const int N = sys.n_atoms;
    const int64_t NX = (int64_t)N * 4 * H;
    const int64_t cap = L.cap;
    const Status* status = ws_ptr<Status>(ws, L.status);
    const int32_t* row_ptr = ws_ptr<int32_t>(ws, L.row_ptr);
    const int32_t* E_dev = row_ptr + N;
    Vec4<T>* geo = ws_ptr<Vec4<T>>(ws, L.geo);
    T* erbf = ws_ptr<T>(ws, L.erbf);
    T* erbf_d = ws_ptr<T>(ws, L.erbf_d);
    T* X = ws_ptr<T>(ws, L.X);
    T* Xt = ws_ptr<T>(ws, L.Xt);
    T* uz = ws_ptr<T>(ws, L.uz);
    T* ua = ws_ptr<T>(ws, L.ua);
    T* fz = ws_ptr<T>(ws, L.fz);
    T* ff = ws_ptr<T>(ws, L.ff);
    T* fh = ws_ptr<T>(ws, L.fh);
    T* fbar = ws_ptr<T>(ws, L.fbar);
    T* comb = ws_ptr<T>(ws, L.comb);
    T* uh = ws_ptr<T>(ws, L.uh);
    T* abar = ws_ptr<T>(ws, L.abar);
    T* xbar0 = ws_ptr<T>(ws, L.xbar);
    T* xbar1 = xbar0 + NX;
    float4* eacc = ws_ptr<float4>(ws, L.edge_acc);
    const int eblocks = 152 * 8;
    const int nblocks = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)N * H + 255) / 256, 152 * 8));
    const int rblocks = std::max(1, std::min(N, 152 * 16));   // receiver-row kernels: one block per atom
    int r;
    if (DUAL && (!grad || (!pos_t && !strain_t))) {
        set_error("the tangent pass needs gradient outputs and a position or strain direction");
        return MLFF_ERR_INVALID;
    }

    {
        ProfScope prof(PK_PLAIN_EDGE, st);
        pl_geom_kernel<T><<<eblocks, 256, 0, st>>>(ws_ptr<float4>(ws, L.pos4), pos_t, strain_t,
                                                   ws_ptr<int32_t>(ws, L.atom_mol),
                                                   sys.box, sys.pbc, row_ptr, ws_ptr<int32_t>(ws, L.col),
                                                   ws_ptr<int32_t>(ws, L.erecv), N, P + po.centers, P + po.gamma,
                                                   d.n_rbf, d.cutoff, geo, erbf, erbf_d, status);
        MLFF_LAUNCH_CHECK("pl_geom");
    }
    if constexpr (DUAL) {
        ProfScope prof(PK_OTHER, st);
        pl_embed_dual_kernel<<<152 * 8, 256, 0, st>>>(P + po.emb, sys.Z, N, d.n_species, X,
                                                      ws_ptr<Status>(ws, L.status));
        MLFF_LAUNCH_CHECK("pl_embed_dual");
    } else {
        if ((r = launch_embed(d, P, po, sys, L, ws, st))) return r;
    }

    for (int l = 0; l < d.n_layers; ++l) {
        const LayerOffsets& lo = po.layer[l];
        T* zl = fz + (int64_t)l * cap * H;
        T* fl = ff + (int64_t)l * cap * H3;
        // filter: z = e W1^T + b1, h = silu(z), f = h W2^T + b2  (:350)
        if ((r = sgemm<1>(erbf, P + lo.w1t, P + lo.b1, zl, fh, (const T*)nullptr, cap, E_dev, H, RMAX, status, st)))
            return r;
        if ((r = sgemm<0>(fh, P + lo.w2t, P + lo.b2, fl, (T*)nullptr, (const T*)nullptr, cap, E_dev, H3, H, status,
                          st))) return r;
        {
            ProfScope prof(PK_PLAIN_EDGE, st);
            pl_message_kernel<T><<<rblocks, 128, 0, st>>>(X + l * NX, fl, geo, ws_ptr<int32_t>(ws, L.col),
                                                          ws_ptr<int32_t>(ws, L.row_ptr), N, Xt + l * NX, status);
            MLFF_LAUNCH_CHECK("pl_message");
        }
        // update (:434-470)
        {
            ProfScope prof(PK_UPDATE_FWD, st);
            pl_update_pre_kernel<T><<<nblocks, 256, 0, st>>>(Xt + l * NX, N, comb, status);
            MLFF_LAUNCH_CHECK("pl_update_pre");
        }
        if ((r = sgemm<1>(comb, P + lo.u1t, P + lo.c1, uz + (int64_t)l * N * H, uh, (const T*)nullptr, N, nullptr, H,
                          2 * H, status, st))) return r;
        if ((r = sgemm<0>(uh, P + lo.u2t, P + lo.c2, ua + (int64_t)l * N * H3, (T*)nullptr, (const T*)nullptr, N,
                          nullptr, H3, H, status, st))) return r;
        {
            ProfScope prof(PK_UPDATE_FWD, st);
            pl_update_post_kernel<T><<<nblocks, 256, 0, st>>>(Xt + l * NX, ua + (int64_t)l * N * H3, P + lo.mix, N,
                                                              X + (l + 1) * NX, status);
            MLFF_LAUNCH_CHECK("pl_update_post");
        }
    }
    if constexpr (DUAL) {
        // unit seeds: the head's adjoint of sum_b E_b and its tangent
        if ((r = grad_readout<T>(d, P, po, sys, L, ws, nullptr, grad->g, st))) return r;
    } else {
        const bool want_grad = out.forces != nullptr || out.virial != nullptr || grad != nullptr;
        if ((r = launch_readout(d, P, po, sys, L, ws, out, want_grad ? 1 : 0, st))) return r;
        if (!want_grad) return MLFF_OK;
        // training: head gradients, and the adjoint seeded with dL/dE_b
        if (grad && (r = grad_readout<T>(d, P, po, sys, L, ws, grad->w, grad->g, st))) return r;
        MLFF_CUDA(cudaMemsetAsync(eacc, 0, sizeof(float4) * cap, st));
        prof_launch(PK_OTHER);   // the memset above
    }

    T* xbo = xbar0;   // dE/dX^(l+1)
    T* xtb = xbar1;   // dE/dXt^(l)
    for (int l = d.n_layers - 1; l >= 0; --l) {
        const LayerOffsets& lo = po.layer[l];
        // update reverse
        {
            ProfScope prof(PK_UPDATE_BWD, st);
            pl_update_bwd_pre_kernel<T><<<nblocks, 256, 0, st>>>(Xt + l * NX, ua + (int64_t)l * N * H3, P + lo.mix,
                                                                 xbo, N, abar, xtb, status);
            MLFF_LAUNCH_CHECK("pl_update_bwd_pre");
        }
        if (grad && (r = grad_update_out<T>(L, ws, l, xbo, grad->g, st))) return r;
        if ((r = sgemm<2>((const T*)abar, P + lo.u2, nullptr, uh, (T*)nullptr, (const T*)(uz + (int64_t)l * N * H), N,
                          nullptr, H, H3, status, st))) return r;
        if (grad) {
            T* gcomb = ws_ptr<T>(ws, L.gcomb);
            pl_update_pre_kernel<T><<<nblocks, 256, 0, st>>>(Xt + l * NX, N, gcomb, status);
            MLFF_LAUNCH_CHECK("pl_update_pre");
            if ((r = grad_update_in<T>(L, ws, l, uh, gcomb, grad->g, st))) return r;
        }
        if ((r = sgemm<0>((const T*)uh, P + lo.u1, nullptr, comb, (T*)nullptr, (const T*)nullptr, N, nullptr, 2 * H, H,
                          status, st))) return r;
        {
            ProfScope prof(PK_UPDATE_BWD, st);
            pl_update_bwd_post_kernel<T><<<nblocks, 256, 0, st>>>(Xt + l * NX, comb, N, xtb, status);
            MLFF_LAUNCH_CHECK("pl_update_bwd_post");
        }
        // message reverse: dE/dX^(l) = xtb + scatter; fbar; dE/du
        {
            ProfScope prof(PK_PLAIN_EDGE, st);
            pl_message_bwd_nodes_kernel<T><<<rblocks, 128, 0, st>>>(ff + (int64_t)l * cap * H3,
                                                                    ws_ptr<int32_t>(ws, L.col),
                                                                    ws_ptr<int32_t>(ws, L.row_ptr), N, xtb, xbo,
                                                                    status);
            MLFF_LAUNCH_CHECK("pl_message_bwd_nodes");
            pl_message_bwd_kernel<T><<<eblocks, 128, 0, st>>>(X + l * NX, ff + (int64_t)l * cap * H3, geo,
                                                              ws_ptr<int32_t>(ws, L.col), ws_ptr<int32_t>(ws, L.erecv),
                                                              E_dev, xtb, fbar, DUAL ? nullptr : eacc, status);
            MLFF_LAUNCH_CHECK("pl_message_bwd");
        }
        if (grad && (r = grad_filter_out<T>(L, ws, l, E_dev, grad->g, st))) return r;
        // filter reverse: hbar = fbar W2, zbar = hbar silu'(z), ebar = zbar W1
        if ((r = sgemm<2>((const T*)fbar, P + lo.w2, nullptr, fh, (T*)nullptr, (const T*)(fz + (int64_t)l * cap * H),
                          cap, E_dev, H, H3, status, st))) return r;
        if (grad && (r = grad_filter_in<T>(d, L, ws, l, E_dev, grad->g, st))) return r;
        if constexpr (!DUAL) {
            // dE/dd for the forces (the parameter gradients stop at the filter input)
            if ((r = sgemm<0>((const T*)fh, P + lo.w1, nullptr, fbar, (T*)nullptr, (const T*)nullptr, cap, E_dev, RMAX,
                              H, status, st))) return r;
            ProfScope prof(PK_PLAIN_EDGE, st);
            pl_dd_kernel<<<eblocks, 256, 0, st>>>(fbar, erbf_d, E_dev, eacc, status);
            MLFF_LAUNCH_CHECK("pl_dd");
        }
    }
    if (grad && (r = grad_embedding<T>(d, sys, L, ws, xbo, grad->g, st))) return r;
    if constexpr (DUAL) return MLFF_OK;
    if (!out.forces && !out.virial) return MLFF_OK;
    return launch_forces(d, sys, L, ws, out, st, vf);
}

// Float32 C[M][N] = A[M][K] B[K][N] (+ bias) for the per-module entry points
// (modules.cu): mode 0 C = acc + bias; 1 also C2 = silu(C); 2 C = acc *
// silu'(Z).
int plain_sgemm(int mode, const float* A, const float* B, const float* bias, float* C, float* C2, const float* Z,
                int64_t M, int N, int K, const Status* st, cudaStream_t s) {
    if (mode == 0) return sgemm<0, float>(A, B, bias, C, C2, Z, M, nullptr, N, K, st, s);
    if (mode == 1) return sgemm<1, float>(A, B, bias, C, C2, Z, M, nullptr, N, K, st, s);
    return sgemm<2, float>(A, B, bias, C, C2, Z, M, nullptr, N, K, st, s);
}

int run_plain(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
              const WsLayout& L, void* ws, const mlff_outputs& out, cudaStream_t st, const GradCtx* grad,
              const VerletFuse* vf) {
    return run_plain_t<float>(d, P, po, sys, L, ws, out, st, grad, nullptr, nullptr, vf);
}

int run_plain_tangent(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
                      const WsLayout& L, void* ws, cudaStream_t st, const GradCtx& grad, const float* pos_t,
                      const double* strain_t) {
    mlff_outputs none{};
    return run_plain_t<Dual>(d, P, po, sys, L, ws, none, st, &grad, pos_t, strain_t);
}

}  // namespace mlff
