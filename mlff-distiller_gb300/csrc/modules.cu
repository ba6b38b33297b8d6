// Per-module entry points: the reference's PaiNNMessage and PaiNNUpdate
// blocks (src/mlff_distiller/models/student_model.py:297-470) evaluated on
// their own, for any hidden width and any number of radial basis functions,
// with their reverse passes (input and parameter gradients).
//
// These serve callers that use the blocks outside StudentForceField (the
// reference's unit tests build a PaiNNInteraction of width 64 and call it
// directly).  They follow the reference's per-op graph in FP32 -- filter
// GEMMs on the plain path's SGEMM, messages scattered with float atomics as
// index_add_ does on a GPU -- and are not the fused hot path.  Edge indices
// come from the caller: an out-of-range index is reported through the
// status word (MLFF_ERR_INVALID, the edge's position) and every later kernel
// of the call returns without work, so nothing is read or written out of
// bounds (the outputs then hold the residual copies only).
#include "common.cuh"
#include "workspace.h"

namespace mlff {

int plain_sgemm(int mode, const float* A, const float* B, const float* bias, float* C, float* C2, const float* Z,
                int64_t M, int N, int K, const Status* st, cudaStream_t s);

namespace {

constexpr int MOD_BLOCKS_MAX = 152 * 8;

inline int grid_for(int64_t n, int threads = 256) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, MOD_BLOCKS_MAX));
}

// Byte layout of a module workspace: a status word, then float arrays.
struct ModLayout {
    size_t st = 0;
    size_t a[16] = {};
    size_t total = 0;
};
inline ModLayout mod_layout(const int64_t* sizes, int n) {
    ModLayout L;
    size_t p = 0;
    auto take = [&](size_t bytes) {
        size_t r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    L.st = take(sizeof(Status));
    for (int i = 0; i < n; ++i) L.a[i] = take(sizeof(float) * (size_t)sizes[i]);
    L.total = p;
    return L;
}

// message workspace: w1t [R][H], w2t [H][3H], z, h [E][H], f [E][3H];
// reverse pass: gf [E][3H], gz [E][H], gfT [3H][E], gzT [H][E]
inline ModLayout msg_layout(int64_t H, int64_t R, int64_t E, bool bwd) {
    const int64_t s[9] = {R * H, H * 3 * H, E * H, E * H, E * 3 * H, E * 3 * H, E * H, 3 * H * E, H * E};
    return mod_layout(s, bwd ? 9 : 5);
}
// update workspace: u1t [2H][H], u2t [H][3H], comb [N][2H], z, h [N][H],
// a [N][3H]; reverse pass: ga [N][3H], gz [N][H], gcomb [N][2H], gaT [3H][N],
// gzT [H][N], gmix [MIX_BLOCKS][9]
constexpr int MIX_BLOCKS = 256;
inline ModLayout upd_layout(int64_t H, int64_t N, bool bwd) {
    const int64_t s[12] = {2 * H * H, H * 3 * H, N * 2 * H, N * H, N * H, N * 3 * H,
                           N * 3 * H, N * H, N * 2 * H, 3 * H * N, H * N, MIX_BLOCKS * 9};
    return mod_layout(s, bwd ? 12 : 6);
}

template <typename T>
inline T* at(void* ws, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

// out[c][r] = in[r][c]
__global__ void mod_transpose_kernel(const float* __restrict__ in, float* __restrict__ out, int64_t rows, int64_t cols,
                                     const Status* st) {
    if (st->code != 0) return;
    const int64_t n = rows * cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / cols, c = i % cols;
        out[c * rows + r] = in[i];
    }
}

// sums over rows: out[c] = sum_r in[r][c] (fixed order)
__global__ void mod_colsum_kernel(const float* __restrict__ in, float* __restrict__ out, int64_t rows, int cols,
                                  const Status* st) {
    if (st->code != 0) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int64_t r = 0; r < rows; ++r) s += in[r * cols + c];
        out[c] = s;
    }
}

__global__ void mod_check_edges_kernel(const int64_t* __restrict__ ei, int64_t E, int32_t N, Status* st) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = ei[e], d = ei[E + e];
        if (s < 0 || s >= N || d < 0 || d >= N) set_status(st, MLFF_ERR_INVALID, (int)std::min<int64_t>(e, INT32_MAX));
    }
}

// scalar_out[dst] += s[src] * phi_s;  vector_out[dst][i] += v[src][i] * phi_v1
// + u[i] * phi_v2   (index_add_, student_model.py:359-385), thread per (edge, channel)
__global__ void msg_scatter_kernel(const float* __restrict__ s, const float* __restrict__ v,
                                   const int64_t* __restrict__ ei, const float* __restrict__ evec,
                                   const float* __restrict__ f, int64_t E, int H, float* __restrict__ s_out,
                                   float* __restrict__ v_out, const Status* st) {
    if (st->code != 0) return;
    const int64_t n = E * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / H;
        const int k = (int)(i % H);
        const int64_t b = ei[e], a = ei[E + e];
        const float* fe = f + e * 3 * H;
        const float fs = fe[k], f1 = fe[H + k], f2 = fe[2 * H + k];
        atomicAdd(s_out + a * H + k, s[b * H + k] * fs);
#pragma unroll
        for (int q = 0; q < 3; ++q)
            atomicAdd(v_out + (a * 3 + q) * H + k, v[(b * 3 + q) * H + k] * f1 + evec[e * 3 + q] * f2);
    }
}

// reverse of the scatter: filter adjoint gf [E][3H], and the gathered
// adjoints of the sender features (grad_s, grad_v hold the residual part)
__global__ void msg_scatter_bwd_kernel(const float* __restrict__ s, const float* __restrict__ v,
                                       const int64_t* __restrict__ ei, const float* __restrict__ evec,
                                       const float* __restrict__ f, const float* __restrict__ gs,
                                       const float* __restrict__ gv, int64_t E, int H, float* __restrict__ gf,
                                       float* __restrict__ grad_s, float* __restrict__ grad_v, const Status* st) {
    if (st->code != 0) return;
    const int64_t n = E * H;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / H;
        const int k = (int)(i % H);
        const int64_t b = ei[e], a = ei[E + e];
        const float* fe = f + e * 3 * H;
        const float gsa = gs[a * H + k];
        float g1 = 0.f, g2 = 0.f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float gva = gv[(a * 3 + q) * H + k];
            g1 = fmaf(gva, v[(b * 3 + q) * H + k], g1);
            g2 = fmaf(gva, evec[e * 3 + q], g2);
            atomicAdd(grad_v + (b * 3 + q) * H + k, gva * fe[H + k]);
        }
        float* g = gf + e * 3 * H;
        g[k] = gsa * s[b * H + k];
        g[H + k] = g1;
        g[2 * H + k] = g2;
        atomicAdd(grad_s + b * H + k, gsa * fe[k]);
    }
}

// grad_u[e][q] = sum_k gv[dst][q][k] phi_v2[e][k]
__global__ void msg_evec_bwd_kernel(const int64_t* __restrict__ ei, const float* __restrict__ f,
                                    const float* __restrict__ gv, int64_t E, int H, float* __restrict__ gu,
                                    const Status* st) {
    if (st->code != 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E * 3; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = i / 3;
        const int q = (int)(i % 3);
        const int64_t a = ei[E + e];
        const float* f2 = f + e * 3 * H + 2 * H;
        const float* g = gv + (a * 3 + q) * H;
        float acc = 0.f;
        for (int k = 0; k < H; ++k) acc = fmaf(g[k], f2[k], acc);
        gu[i] = acc;
    }
}

// comb = [s, |v|] (norm over xyz, student_model.py:437-440)
__global__ void upd_comb_kernel(const float* __restrict__ s, const float* __restrict__ v, int64_t N, int H,
                                float* __restrict__ comb, const Status* st) {
    if (st->code != 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * H; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / H;
        const int k = (int)(i % H);
        const float x = v[(n * 3) * H + k], y = v[(n * 3 + 1) * H + k], z = v[(n * 3 + 2) * H + k];
        comb[n * 2 * H + k] = s[i];
        comb[n * 2 * H + H + k] = sqrtf(x * x + y * y + z * z);
    }
}

// s_out = s + a_s;  v_out = v g1 + (M v) g2, M over xyz (:452-468)
__global__ void upd_finish_kernel(const float* __restrict__ s, const float* __restrict__ v,
                                  const float* __restrict__ a, const float* __restrict__ mix, int64_t N, int H,
                                  float* __restrict__ s_out, float* __restrict__ v_out, const Status* st) {
    if (st->code != 0) return;
    float M[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) M[j] = mix[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * H; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / H;
        const int k = (int)(i % H);
        const float* an = a + n * 3 * H;
        s_out[i] = s[i] + an[k];
        const float g1 = an[H + k], g2 = an[2 * H + k];
        float vv[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) vv[q] = v[(n * 3 + q) * H + k];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float mixed = M[3 * q] * vv[0] + M[3 * q + 1] * vv[1] + M[3 * q + 2] * vv[2];
            v_out[(n * 3 + q) * H + k] = vv[q] * g1 + mixed * g2;
        }
    }
}

// reverse of upd_finish: ga [N][3H]; grad_s = gs; grad_v (direct part)
__global__ void upd_finish_bwd_kernel(const float* __restrict__ v, const float* __restrict__ a,
                                      const float* __restrict__ mix, const float* __restrict__ gs,
                                      const float* __restrict__ gv, int64_t N, int H, float* __restrict__ ga,
                                      float* __restrict__ grad_s, float* __restrict__ grad_v, const Status* st) {
    if (st->code != 0) return;
    float M[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) M[j] = mix[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * H; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / H;
        const int k = (int)(i % H);
        const float* an = a + n * 3 * H;
        const float g1 = an[H + k], g2 = an[2 * H + k];
        float vv[3], gg[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            vv[q] = v[(n * 3 + q) * H + k];
            gg[q] = gv[(n * 3 + q) * H + k];
        }
        float dg1 = 0.f, dg2 = 0.f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float mixed = M[3 * q] * vv[0] + M[3 * q + 1] * vv[1] + M[3 * q + 2] * vv[2];
            dg1 = fmaf(gg[q], vv[q], dg1);
            dg2 = fmaf(gg[q], mixed, dg2);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j)
            grad_v[(n * 3 + j) * H + k] = gg[j] * g1 + g2 * (M[j] * gg[0] + M[3 + j] * gg[1] + M[6 + j] * gg[2]);
        grad_s[i] = gs[i];
        float* g = ga + n * 3 * H;
        g[k] = gs[i];
        g[H + k] = dg1;
        g[2 * H + k] = dg2;
    }
}

// adds the combined-input adjoint: grad_s += gcomb[:, :H]; grad_v += gcomb[:,
// H:] v / |v| (0 where |v| = 0, the subgradient torch.norm uses)
__global__ void upd_comb_bwd_kernel(const float* __restrict__ v, const float* __restrict__ comb,
                                    const float* __restrict__ gcomb, int64_t N, int H, float* __restrict__ grad_s,
                                    float* __restrict__ grad_v, const Status* st) {
    if (st->code != 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * H; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / H;
        const int k = (int)(i % H);
        grad_s[i] += gcomb[n * 2 * H + k];
        const float nrm = comb[n * 2 * H + H + k];
        if (nrm > 0.f) {
            const float sc = gcomb[n * 2 * H + H + k] / nrm;
#pragma unroll
            for (int q = 0; q < 3; ++q) grad_v[(n * 3 + q) * H + k] += sc * v[(n * 3 + q) * H + k];
        }
    }
}

// grad_M[q][j] = sum_{n,k} gv[n][q][k] g2[n][k] v[n][j][k]: per-block partials, fixed order
__global__ void __launch_bounds__(256) upd_mix_bwd_kernel(const float* __restrict__ v, const float* __restrict__ a,
                                                          const float* __restrict__ gv, int64_t N, int H,
                                                          float* __restrict__ part, const Status* st) {
    __shared__ float red[9][256];
    if (st->code != 0) return;
    float acc[9] = {};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * H; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = i / H;
        const int k = (int)(i % H);
        const float g2 = a[n * 3 * H + 2 * H + k];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float gq = gv[(n * 3 + q) * H + k] * g2;
#pragma unroll
            for (int j = 0; j < 3; ++j) acc[3 * q + j] = fmaf(gq, v[(n * 3 + j) * H + k], acc[3 * q + j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 9; ++j) red[j][threadIdx.x] = acc[j];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
#pragma unroll
            for (int j = 0; j < 9; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 9) part[blockIdx.x * 9 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void upd_mix_sum_kernel(const float* __restrict__ part, int blocks, float* __restrict__ out,
                                   const Status* st) {
    if (st->code != 0) return;
    if (threadIdx.x < 9) {
        float s = 0.f;
        for (int b = 0; b < blocks; ++b) s += part[b * 9 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

int check_mod(int32_t H, int32_t R, int64_t rows) {
    if (H < 1 || H > 4096 || R < 0 || R > 4096 || rows < 0) {
        set_error("module shape outside limits (hidden %d, n_rbf %d, rows %lld)", H, R, (long long)rows);
        return MLFF_ERR_INVALID;
    }
    return MLFF_OK;
}

#define MOD_LAUNCH(kernel, n, st, ...)                                              \
    do {                                                                            \
        kernel<<<grid_for(n), 256, 0, st>>>(__VA_ARGS__);                           \
        MLFF_LAUNCH_CHECK(#kernel);                                                 \
    } while (0)

}  // namespace
}  // namespace mlff

using namespace mlff;

extern "C" {

size_t mlff_painn_message_workspace_size(int32_t hidden, int32_t n_rbf, int64_t n_edges, int32_t with_backward) {
    if (check_mod(hidden, n_rbf, n_edges)) return 0;
    return msg_layout(hidden, n_rbf, n_edges, with_backward != 0).total;
}

int mlff_painn_message(int32_t hidden, int32_t n_rbf, int32_t n_atoms, int64_t n_edges, const float* scalar,
                       const float* vector, const int64_t* edge_index, const float* edge_rbf,
                       const float* edge_vector, const float* w1, const float* b1, const float* w2, const float* b2,
                       float* scalar_out, float* vector_out, int32_t* status, void* workspace,
                       size_t workspace_bytes, mlff_stream_t stream) {
    int r = check_mod(hidden, n_rbf, n_edges);
    if (r) return r;
    if (n_atoms < 1 || !scalar || !vector || !w1 || !b1 || !w2 || !b2 || !scalar_out || !vector_out || !status ||
        !workspace || (n_edges > 0 && (!edge_index || !edge_rbf || !edge_vector))) {
        set_error("painn_message: missing argument");
        return MLFF_ERR_INVALID;
    }
    const int64_t H = hidden, R = n_rbf, E = n_edges, N = n_atoms;
    const ModLayout L = msg_layout(H, R, E, false);
    if (workspace_bytes < L.total) {
        set_error("workspace %zu bytes < %zu needed", workspace_bytes, L.total);
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Status* sw = at<Status>(workspace, L.st);
    MLFF_CUDA(cudaMemsetAsync(sw, 0, sizeof(Status), st));
    MLFF_CUDA(cudaMemcpyAsync(scalar_out, scalar, sizeof(float) * N * H, cudaMemcpyDeviceToDevice, st));
    MLFF_CUDA(cudaMemcpyAsync(vector_out, vector, sizeof(float) * N * 3 * H, cudaMemcpyDeviceToDevice, st));
    if (E > 0) {
        float *w1t = at<float>(workspace, L.a[0]), *w2t = at<float>(workspace, L.a[1]);
        float *z = at<float>(workspace, L.a[2]), *h = at<float>(workspace, L.a[3]), *f = at<float>(workspace, L.a[4]);
        MOD_LAUNCH(mod_check_edges_kernel, E, st, edge_index, E, n_atoms, sw);
        MOD_LAUNCH(mod_transpose_kernel, H * R, st, w1, w1t, H, R, sw);
        MOD_LAUNCH(mod_transpose_kernel, 3 * H * H, st, w2, w2t, 3 * H, H, sw);
        // filter = Linear(R, H) - SiLU - Linear(H, 3H)  (:318-322, :350)
        if ((r = plain_sgemm(1, edge_rbf, w1t, b1, z, h, nullptr, E, (int)H, (int)R, sw, st))) return r;
        if ((r = plain_sgemm(0, h, w2t, b2, f, nullptr, nullptr, E, (int)(3 * H), (int)H, sw, st))) return r;
        MOD_LAUNCH(msg_scatter_kernel, E * H, st, scalar, vector, edge_index, edge_vector, f, E, (int)H, scalar_out,
                   vector_out, sw);
    }
    MLFF_CUDA(cudaMemcpyAsync(status, sw, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
    return MLFF_OK;
}

int mlff_painn_message_backward(int32_t hidden, int32_t n_rbf, int32_t n_atoms, int64_t n_edges, const float* scalar,
                                const float* vector, const int64_t* edge_index, const float* edge_rbf,
                                const float* edge_vector, const float* w1, const float* b1, const float* w2,
                                const float* b2, const float* grad_scalar_out, const float* grad_vector_out,
                                float* grad_scalar, float* grad_vector, float* grad_rbf, float* grad_edge_vector,
                                float* grad_w1, float* grad_b1, float* grad_w2, float* grad_b2, int32_t* status,
                                void* workspace, size_t workspace_bytes, mlff_stream_t stream) {
    int r = check_mod(hidden, n_rbf, n_edges);
    if (r) return r;
    if (n_atoms < 1 || !scalar || !vector || !w1 || !b1 || !w2 || !b2 || !grad_scalar_out || !grad_vector_out ||
        !grad_scalar || !grad_vector || !grad_w1 || !grad_b1 || !grad_w2 || !grad_b2 || !status || !workspace ||
        (n_edges > 0 && (!edge_index || !edge_rbf || !edge_vector || !grad_rbf || !grad_edge_vector))) {
        set_error("painn_message_backward: missing argument");
        return MLFF_ERR_INVALID;
    }
    const int64_t H = hidden, R = n_rbf, E = n_edges, N = n_atoms;
    const ModLayout L = msg_layout(H, R, E, true);
    if (workspace_bytes < L.total) {
        set_error("workspace %zu bytes < %zu needed (with_backward)", workspace_bytes, L.total);
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Status* sw = at<Status>(workspace, L.st);
    MLFF_CUDA(cudaMemsetAsync(sw, 0, sizeof(Status), st));
    // residual part of the feature adjoints
    MLFF_CUDA(cudaMemcpyAsync(grad_scalar, grad_scalar_out, sizeof(float) * N * H, cudaMemcpyDeviceToDevice, st));
    MLFF_CUDA(cudaMemcpyAsync(grad_vector, grad_vector_out, sizeof(float) * N * 3 * H, cudaMemcpyDeviceToDevice, st));
    if (E == 0) {
        MLFF_CUDA(cudaMemsetAsync(grad_w1, 0, sizeof(float) * H * R, st));
        MLFF_CUDA(cudaMemsetAsync(grad_b1, 0, sizeof(float) * H, st));
        MLFF_CUDA(cudaMemsetAsync(grad_w2, 0, sizeof(float) * 3 * H * H, st));
        MLFF_CUDA(cudaMemsetAsync(grad_b2, 0, sizeof(float) * 3 * H, st));
        MLFF_CUDA(cudaMemcpyAsync(status, sw, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
        return MLFF_OK;
    }
    float *w1t = at<float>(workspace, L.a[0]), *w2t = at<float>(workspace, L.a[1]);
    float *z = at<float>(workspace, L.a[2]), *h = at<float>(workspace, L.a[3]), *f = at<float>(workspace, L.a[4]);
    float *gf = at<float>(workspace, L.a[5]), *gz = at<float>(workspace, L.a[6]);
    float *gfT = at<float>(workspace, L.a[7]), *gzT = at<float>(workspace, L.a[8]);
    MOD_LAUNCH(mod_check_edges_kernel, E, st, edge_index, E, n_atoms, sw);
    // the filter of the forward pass, recomputed (no activation is kept between the calls)
    MOD_LAUNCH(mod_transpose_kernel, H * R, st, w1, w1t, H, R, sw);
    MOD_LAUNCH(mod_transpose_kernel, 3 * H * H, st, w2, w2t, 3 * H, H, sw);
    if ((r = plain_sgemm(1, edge_rbf, w1t, b1, z, h, nullptr, E, (int)H, (int)R, sw, st))) return r;
    if ((r = plain_sgemm(0, h, w2t, b2, f, nullptr, nullptr, E, (int)(3 * H), (int)H, sw, st))) return r;
    // filter adjoint and the gathered feature adjoints; unit-vector adjoint
    MOD_LAUNCH(msg_scatter_bwd_kernel, E * H, st, scalar, vector, edge_index, edge_vector, f, grad_scalar_out,
               grad_vector_out, E, (int)H, gf, grad_scalar, grad_vector, sw);
    MOD_LAUNCH(msg_evec_bwd_kernel, E * 3, st, edge_index, f, grad_vector_out, E, (int)H, grad_edge_vector, sw);
    // through the filter MLP: gz = (gf W2) silu'(z), grad_rbf = gz W1
    if ((r = plain_sgemm(2, gf, w2, nullptr, gz, nullptr, z, E, (int)H, (int)(3 * H), sw, st))) return r;
    if ((r = plain_sgemm(0, gz, w1, nullptr, grad_rbf, nullptr, nullptr, E, (int)R, (int)H, sw, st))) return r;
    // parameter gradients: W2 = gf^T h, W1 = gz^T rbf, biases = column sums
    MOD_LAUNCH(mod_transpose_kernel, E * 3 * H, st, gf, gfT, E, 3 * H, sw);
    MOD_LAUNCH(mod_transpose_kernel, E * H, st, gz, gzT, E, H, sw);
    if ((r = plain_sgemm(0, gfT, h, nullptr, grad_w2, nullptr, nullptr, 3 * H, (int)H, (int)E, sw, st))) return r;
    if ((r = plain_sgemm(0, gzT, edge_rbf, nullptr, grad_w1, nullptr, nullptr, H, (int)R, (int)E, sw, st))) return r;
    MOD_LAUNCH(mod_colsum_kernel, 3 * H, st, gf, grad_b2, E, (int)(3 * H), sw);
    MOD_LAUNCH(mod_colsum_kernel, H, st, gz, grad_b1, E, (int)H, sw);
    MLFF_CUDA(cudaMemcpyAsync(status, sw, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
    return MLFF_OK;
}

size_t mlff_painn_update_workspace_size(int32_t hidden, int32_t n_atoms, int32_t with_backward) {
    if (check_mod(hidden, 0, n_atoms)) return 0;
    return upd_layout(hidden, n_atoms, with_backward != 0).total;
}

int mlff_painn_update(int32_t hidden, int32_t n_atoms, const float* scalar, const float* vector, const float* w1,
                      const float* b1, const float* w2, const float* b2, const float* mixing, float* scalar_out,
                      float* vector_out, void* workspace, size_t workspace_bytes, mlff_stream_t stream) {
    int r = check_mod(hidden, 0, n_atoms);
    if (r) return r;
    if (n_atoms < 1 || !scalar || !vector || !w1 || !b1 || !w2 || !b2 || !mixing || !scalar_out || !vector_out ||
        !workspace) {
        set_error("painn_update: missing argument");
        return MLFF_ERR_INVALID;
    }
    const int64_t H = hidden, N = n_atoms;
    const ModLayout L = upd_layout(H, N, false);
    if (workspace_bytes < L.total) {
        set_error("workspace %zu bytes < %zu needed", workspace_bytes, L.total);
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Status* sw = at<Status>(workspace, L.st);
    MLFF_CUDA(cudaMemsetAsync(sw, 0, sizeof(Status), st));
    float *u1t = at<float>(workspace, L.a[0]), *u2t = at<float>(workspace, L.a[1]);
    float *comb = at<float>(workspace, L.a[2]), *z = at<float>(workspace, L.a[3]);
    float *h = at<float>(workspace, L.a[4]), *a = at<float>(workspace, L.a[5]);
    MOD_LAUNCH(mod_transpose_kernel, 2 * H * H, st, w1, u1t, H, 2 * H, sw);
    MOD_LAUNCH(mod_transpose_kernel, 3 * H * H, st, w2, u2t, 3 * H, H, sw);
    MOD_LAUNCH(upd_comb_kernel, N * H, st, scalar, vector, N, (int)H, comb, sw);
    // update_mlp = Linear(2H, H) - SiLU - Linear(H, 3H)  (:440-444)
    if ((r = plain_sgemm(1, comb, u1t, b1, z, h, nullptr, N, (int)H, (int)(2 * H), sw, st))) return r;
    if ((r = plain_sgemm(0, h, u2t, b2, a, nullptr, nullptr, N, (int)(3 * H), (int)H, sw, st))) return r;
    MOD_LAUNCH(upd_finish_kernel, N * H, st, scalar, vector, a, mixing, N, (int)H, scalar_out, vector_out, sw);
    return MLFF_OK;
}

int mlff_painn_update_backward(int32_t hidden, int32_t n_atoms, const float* scalar, const float* vector,
                               const float* w1, const float* b1, const float* w2, const float* b2,
                               const float* mixing, const float* grad_scalar_out, const float* grad_vector_out,
                               float* grad_scalar, float* grad_vector, float* grad_w1, float* grad_b1,
                               float* grad_w2, float* grad_b2, float* grad_mixing, void* workspace,
                               size_t workspace_bytes, mlff_stream_t stream) {
    int r = check_mod(hidden, 0, n_atoms);
    if (r) return r;
    if (n_atoms < 1 || !scalar || !vector || !w1 || !b1 || !w2 || !b2 || !mixing || !grad_scalar_out ||
        !grad_vector_out || !grad_scalar || !grad_vector || !grad_w1 || !grad_b1 || !grad_w2 || !grad_b2 ||
        !grad_mixing || !workspace) {
        set_error("painn_update_backward: missing argument");
        return MLFF_ERR_INVALID;
    }
    const int64_t H = hidden, N = n_atoms;
    const ModLayout L = upd_layout(H, N, true);
    if (workspace_bytes < L.total) {
        set_error("workspace %zu bytes < %zu needed (with_backward)", workspace_bytes, L.total);
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Status* sw = at<Status>(workspace, L.st);
    MLFF_CUDA(cudaMemsetAsync(sw, 0, sizeof(Status), st));
    float *u1t = at<float>(workspace, L.a[0]), *u2t = at<float>(workspace, L.a[1]);
    float *comb = at<float>(workspace, L.a[2]), *z = at<float>(workspace, L.a[3]);
    float *h = at<float>(workspace, L.a[4]), *a = at<float>(workspace, L.a[5]);
    float *ga = at<float>(workspace, L.a[6]), *gz = at<float>(workspace, L.a[7]);
    float *gcomb = at<float>(workspace, L.a[8]), *gaT = at<float>(workspace, L.a[9]);
    float *gzT = at<float>(workspace, L.a[10]), *gmix = at<float>(workspace, L.a[11]);
    // the forward pass, recomputed
    MOD_LAUNCH(mod_transpose_kernel, 2 * H * H, st, w1, u1t, H, 2 * H, sw);
    MOD_LAUNCH(mod_transpose_kernel, 3 * H * H, st, w2, u2t, 3 * H, H, sw);
    MOD_LAUNCH(upd_comb_kernel, N * H, st, scalar, vector, N, (int)H, comb, sw);
    if ((r = plain_sgemm(1, comb, u1t, b1, z, h, nullptr, N, (int)H, (int)(2 * H), sw, st))) return r;
    if ((r = plain_sgemm(0, h, u2t, b2, a, nullptr, nullptr, N, (int)(3 * H), (int)H, sw, st))) return r;
    // gates and mixing; through the MLP; the combined input's adjoint
    MOD_LAUNCH(upd_finish_bwd_kernel, N * H, st, vector, a, mixing, grad_scalar_out, grad_vector_out, N, (int)H, ga,
               grad_scalar, grad_vector, sw);
    upd_mix_bwd_kernel<<<MIX_BLOCKS, 256, 0, st>>>(vector, a, grad_vector_out, N, (int)H, gmix, sw);
    MLFF_LAUNCH_CHECK("upd_mix_bwd_kernel");
    upd_mix_sum_kernel<<<1, 32, 0, st>>>(gmix, MIX_BLOCKS, grad_mixing, sw);
    MLFF_LAUNCH_CHECK("upd_mix_sum_kernel");
    if ((r = plain_sgemm(2, ga, w2, nullptr, gz, nullptr, z, N, (int)H, (int)(3 * H), sw, st))) return r;
    if ((r = plain_sgemm(0, gz, w1, nullptr, gcomb, nullptr, nullptr, N, (int)(2 * H), (int)H, sw, st))) return r;
    MOD_LAUNCH(upd_comb_bwd_kernel, N * H, st, vector, comb, gcomb, N, (int)H, grad_scalar, grad_vector, sw);
    // parameter gradients
    MOD_LAUNCH(mod_transpose_kernel, N * 3 * H, st, ga, gaT, N, 3 * H, sw);
    MOD_LAUNCH(mod_transpose_kernel, N * H, st, gz, gzT, N, H, sw);
    if ((r = plain_sgemm(0, gaT, h, nullptr, grad_w2, nullptr, nullptr, 3 * H, (int)H, (int)N, sw, st))) return r;
    if ((r = plain_sgemm(0, gzT, comb, nullptr, grad_w1, nullptr, nullptr, H, (int)(2 * H), (int)N, sw, st))) return r;
    MOD_LAUNCH(mod_colsum_kernel, 3 * H, st, ga, grad_b2, N, (int)(3 * H), sw);
    MOD_LAUNCH(mod_colsum_kernel, H, st, gz, grad_b1, N, (int)H, sw);
    return MLFF_OK;
}

}  // extern "C"
