// Fused edge kernels (receiver-centric, persistent, no atomics).
//
// The neighbour build gives a receiver-sorted CSR; a partition splits the
// receivers into P contiguous ranges of about E/P edges each.  CTA p walks
// its range in tiles of edges and, per tile:
//   1. edge geometry r, d, u and e = rbf(d) * fc(d)          (:706-722)
//   2. filter  f = W2 silu(W1 e + b1) + b2                    (:350)
//   3. messages X_b * phi (+ u * phi_v2) summed over the tile's edges into
//      the running receiver sums, one channel per thread    (:359-385)
// A receiver's sum lives in registers until its last edge has been seen,
// then Xt[a] = X[a] + sum is written once: no atomics, fixed order.
//
// Reverse pass (same tiles, same partition).  With f' = df/dd =
// W2 (silu'(z) * (W1 de/dd)) computed forward-mode next to f, per edge
// b -> a and channel c:
//   dE/dX_a   += dE/dXt_b * (phi_s, phi_v1)   (gather from the sender side,
//                                              exact because f(d_ab) = f(d_ba))
//   dE/dd_k   += sum_c fbar_c f'_c,   fbar = (dXt_a.s X_b.s,
//                                             sum_i dXt_a.v_i X_b.v_i,
//                                             sum_i dXt_a.v_i u_i)
//   dE/du_k   += sum_c dXt_a.v * phi_v2
// so no filter activation is stored and no transposed filter GEMM is needed.
// This file holds the FP32 CUDA-core version of those kernels and the
// driver for the fused path; tc_edge.cu holds the tensor-core version.
#include <atomic>
#include "common.cuh"
#include "workspace.h"
#include "edge_common.cuh"
#include "profile.h"

namespace mlff {

// mlff_debug_stall_test: kernels that time out on purpose (test hook)
std::atomic<int> g_stall_test{0};

constexpr int FT = 32;   // edges per tile, forward
constexpr int BT = 16;   // edges per tile, reverse

__device__ __noinline__ void flush_fwd(const float* __restrict__ X, float* __restrict__ Xt, int c, int cur,
                                       int next, float s, float v0, float v1, float v2) {
    const float* x = X + (int64_t)cur * 4 * H;
    float* o = Xt + (int64_t)cur * 4 * H;
    o[c] = x[c] + s;
    o[H + c] = x[H + c] + v0;
    o[2 * H + c] = x[2 * H + c] + v1;
    o[3 * H + c] = x[3 * H + c] + v2;
    for (int j = cur + 1; j < next; ++j) {
        const float* xj = X + (int64_t)j * 4 * H;
        float* oj = Xt + (int64_t)j * 4 * H;
        oj[c] = xj[c];
        oj[H + c] = xj[H + c];
        oj[2 * H + c] = xj[2 * H + c];
        oj[3 * H + c] = xj[3 * H + c];
    }
}

__global__ void __launch_bounds__(128) edge_fwd_simt_kernel(EdgeArgs a) {
    __shared__ float w1s[H][RMAX + 1];
    __shared__ float b1s[H];
    __shared__ float rbf[FT][RMAX + 1];
    __shared__ __align__(16) float hs[H][FT + 4];
    __shared__ float4 us[FT];
    __shared__ int src_s[FT], rcv_s[FT];
    __shared__ float cent[RMAX], gam[RMAX];
    if (a.st->code != 0) return;
    const int t = threadIdx.x;
    for (int i = t; i < H * RMAX; i += 128) w1s[i / RMAX][i % RMAX] = a.P[a.lo.w1 + i];
    b1s[t] = a.P[a.lo.b1 + t];
    if (t < RMAX) { cent[t] = a.centers[t]; gam[t] = a.gamma[t]; }
    const float* W2T = a.P + a.lo.w2t;
    const float bb0 = a.P[a.lo.b2 + t], bb1 = a.P[a.lo.b2 + H + t], bb2 = a.P[a.lo.b2 + 2 * H + t];
    __syncthreads();
    for (int p = blockIdx.x; p < a.nparts; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        int cur = j0;
        float acc_s = 0.f, acc_v0 = 0.f, acc_v1 = 0.f, acc_v2 = 0.f;
        for (int t0 = e0; t0 < e1; t0 += FT) {
            const int n = min(FT, e1 - t0);
            if (t < FT) load_edge(a, t0, t, n, us, src_s, rcv_s);
            __syncthreads();
            {
                const int e = t & (FT - 1), rg = (t >> 5) * 8;
                const float d = us[e].w;
                const float fc = cutoff_fn(d, a.cutoff);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int r = rg + q;
                    const float diff = d - cent[r];
                    rbf[e][r] = (r < a.R && e < n) ? expf(-gam[r] * diff * diff) * fc : 0.0f;
                }
            }
            __syncthreads();
            {
                const int e = t & (FT - 1), kb = (t >> 5) * 32;
                for (int kk = 0; kk < 32; ++kk) {
                    const int k = kb + kk;
                    float z = b1s[k];
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) z = fmaf(w1s[k][r], rbf[e][r], z);
                    hs[k][e] = silu_f(z);
                }
            }
            __syncthreads();
            float f[3][FT];
#pragma unroll
            for (int e = 0; e < FT; ++e) { f[0][e] = bb0; f[1][e] = bb1; f[2][e] = bb2; }
            for (int k = 0; k < H; ++k) {
                const float w0 = W2T[k * H3 + t], w1 = W2T[k * H3 + H + t], w2 = W2T[k * H3 + 2 * H + t];
#pragma unroll
                for (int e4 = 0; e4 < FT; e4 += 4) {
                    const float4 h = *reinterpret_cast<const float4*>(&hs[k][e4]);
                    f[0][e4] = fmaf(w0, h.x, f[0][e4]); f[0][e4 + 1] = fmaf(w0, h.y, f[0][e4 + 1]);
                    f[0][e4 + 2] = fmaf(w0, h.z, f[0][e4 + 2]); f[0][e4 + 3] = fmaf(w0, h.w, f[0][e4 + 3]);
                    f[1][e4] = fmaf(w1, h.x, f[1][e4]); f[1][e4 + 1] = fmaf(w1, h.y, f[1][e4 + 1]);
                    f[1][e4 + 2] = fmaf(w1, h.z, f[1][e4 + 2]); f[1][e4 + 3] = fmaf(w1, h.w, f[1][e4 + 3]);
                    f[2][e4] = fmaf(w2, h.x, f[2][e4]); f[2][e4 + 1] = fmaf(w2, h.y, f[2][e4 + 1]);
                    f[2][e4 + 2] = fmaf(w2, h.z, f[2][e4 + 2]); f[2][e4 + 3] = fmaf(w2, h.w, f[2][e4 + 3]);
                }
            }
#pragma unroll
            for (int e = 0; e < FT; ++e) {
                if (e < n) {
                    const int ra = rcv_s[e];
                    if (ra != cur) {
                        flush_fwd(a.X, a.Xt, t, cur, ra, acc_s, acc_v0, acc_v1, acc_v2);
                        acc_s = acc_v0 = acc_v1 = acc_v2 = 0.f;
                        cur = ra;
                    }
                    const float* xb = a.X + (int64_t)src_s[e] * 4 * H;
                    const float4 u = us[e];
                    acc_s = fmaf(xb[t], f[0][e], acc_s);
                    acc_v0 = fmaf(xb[H + t], f[1][e], fmaf(u.x, f[2][e], acc_v0));
                    acc_v1 = fmaf(xb[2 * H + t], f[1][e], fmaf(u.y, f[2][e], acc_v1));
                    acc_v2 = fmaf(xb[3 * H + t], f[1][e], fmaf(u.z, f[2][e], acc_v2));
                }
            }
            __syncthreads();
        }
        flush_fwd(a.X, a.Xt, t, cur, j1, acc_s, acc_v0, acc_v1, acc_v2);
    }
}

__device__ __noinline__ void flush_bwd(const float* __restrict__ xtbar, float* __restrict__ xbar, int c, int cur,
                                       int next, float s, float v0, float v1, float v2) {
    const float* x = xtbar + (int64_t)cur * 4 * H;
    float* o = xbar + (int64_t)cur * 4 * H;
    o[c] = x[c] + s;
    o[H + c] = x[H + c] + v0;
    o[2 * H + c] = x[2 * H + c] + v1;
    o[3 * H + c] = x[3 * H + c] + v2;
    for (int j = cur + 1; j < next; ++j) {
        const float* xj = xtbar + (int64_t)j * 4 * H;
        float* oj = xbar + (int64_t)j * 4 * H;
        oj[c] = xj[c];
        oj[H + c] = xj[H + c];
        oj[2 * H + c] = xj[2 * H + c];
        oj[3 * H + c] = xj[3 * H + c];
    }
}

__global__ void __launch_bounds__(128) edge_bwd_simt_kernel(EdgeArgs a) {
    __shared__ float w1s[H][RMAX + 1];
    __shared__ float b1s[H];
    __shared__ float rbf[BT][RMAX + 1];
    __shared__ float rbfd[BT][RMAX + 1];
    __shared__ __align__(16) float hs[H][BT + 4];
    __shared__ __align__(16) float hds[H][BT + 4];
    __shared__ float4 us[BT];
    __shared__ int src_s[BT], rcv_s[BT];
    __shared__ float cent[RMAX], gam[RMAX];
    __shared__ float red[4][BT][4];
    if (a.st->code != 0) return;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int i = t; i < H * RMAX; i += 128) w1s[i / RMAX][i % RMAX] = a.P[a.lo.w1 + i];
    b1s[t] = a.P[a.lo.b1 + t];
    if (t < RMAX) { cent[t] = a.centers[t]; gam[t] = a.gamma[t]; }
    const float* W2T = a.P + a.lo.w2t;
    const float bb0 = a.P[a.lo.b2 + t], bb1 = a.P[a.lo.b2 + H + t], bb2 = a.P[a.lo.b2 + 2 * H + t];
    __syncthreads();
    for (int p = blockIdx.x; p < a.nparts; p += gridDim.x) {
        const int j0 = a.part[p], j1 = a.part[p + 1];
        if (j0 >= j1) continue;
        const int e0 = a.row_ptr[j0], e1 = a.row_ptr[j1];
        int cur = j0;
        float acc_s = 0.f, acc_v0 = 0.f, acc_v1 = 0.f, acc_v2 = 0.f;
        const float* ta = a.xtbar + (int64_t)cur * 4 * H;
        float ta_s = ta[t], ta_v0 = ta[H + t], ta_v1 = ta[2 * H + t], ta_v2 = ta[3 * H + t];
        for (int t0 = e0; t0 < e1; t0 += BT) {
            const int n = min(BT, e1 - t0);
            if (t < BT) load_edge(a, t0, t, n, us, src_s, rcv_s);
            __syncthreads();
            {
                // 128 threads: e = t & 15, r-group of 4
                const int e = t & (BT - 1), rg = (t >> 4) * 4;
                const float d = us[e].w;
                float fc, dfc;
                cutoff_fn_d(d, a.cutoff, fc, dfc);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = rg + q;
                    const float diff = d - cent[r];
                    const float g = expf(-gam[r] * diff * diff);
                    const bool ok = r < a.R && e < n;
                    rbf[e][r] = ok ? g * fc : 0.0f;
                    rbfd[e][r] = ok ? g * (dfc - 2.0f * gam[r] * diff * fc) : 0.0f;
                }
            }
            __syncthreads();
            {
                const int e = t & (BT - 1), kb = (t >> 4) * 16;
                for (int kk = 0; kk < 16; ++kk) {
                    const int k = kb + kk;
                    float z = b1s[k], zd = 0.0f;
#pragma unroll
                    for (int r = 0; r < RMAX; ++r) {
                        z = fmaf(w1s[k][r], rbf[e][r], z);
                        zd = fmaf(w1s[k][r], rbfd[e][r], zd);
                    }
                    hs[k][e] = silu_f(z);
                    hds[k][e] = dsilu_f(z) * zd;
                }
            }
            __syncthreads();
            float f[3][BT], fd[3][BT];
#pragma unroll
            for (int e = 0; e < BT; ++e) {
                f[0][e] = bb0; f[1][e] = bb1; f[2][e] = bb2;
                fd[0][e] = 0.f; fd[1][e] = 0.f; fd[2][e] = 0.f;
            }
            for (int k = 0; k < H; ++k) {
                const float w0 = W2T[k * H3 + t], w1 = W2T[k * H3 + H + t], w2 = W2T[k * H3 + 2 * H + t];
#pragma unroll
                for (int e4 = 0; e4 < BT; e4 += 4) {
                    const float4 h = *reinterpret_cast<const float4*>(&hs[k][e4]);
                    const float4 hd = *reinterpret_cast<const float4*>(&hds[k][e4]);
                    const float hv[4] = {h.x, h.y, h.z, h.w}, hdv[4] = {hd.x, hd.y, hd.z, hd.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        f[0][e4 + q] = fmaf(w0, hv[q], f[0][e4 + q]);
                        f[1][e4 + q] = fmaf(w1, hv[q], f[1][e4 + q]);
                        f[2][e4 + q] = fmaf(w2, hv[q], f[2][e4 + q]);
                        fd[0][e4 + q] = fmaf(w0, hdv[q], fd[0][e4 + q]);
                        fd[1][e4 + q] = fmaf(w1, hdv[q], fd[1][e4 + q]);
                        fd[2][e4 + q] = fmaf(w2, hdv[q], fd[2][e4 + q]);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < BT; ++e) {
                if (e < n) {
                    const int ra = rcv_s[e];
                    if (ra != cur) {
                        flush_bwd(a.xtbar, a.xbar, t, cur, ra, acc_s, acc_v0, acc_v1, acc_v2);
                        acc_s = acc_v0 = acc_v1 = acc_v2 = 0.f;
                        cur = ra;
                        const float* tr = a.xtbar + (int64_t)cur * 4 * H;
                        ta_s = tr[t]; ta_v0 = tr[H + t]; ta_v1 = tr[2 * H + t]; ta_v2 = tr[3 * H + t];
                    }
                    const int sb = src_s[e];
                    const float* tb = a.xtbar + (int64_t)sb * 4 * H;
                    const float* xb = a.X + (int64_t)sb * 4 * H;
                    const float4 u = us[e];
                    acc_s = fmaf(tb[t], f[0][e], acc_s);
                    acc_v0 = fmaf(tb[H + t], f[1][e], acc_v0);
                    acc_v1 = fmaf(tb[2 * H + t], f[1][e], acc_v1);
                    acc_v2 = fmaf(tb[3 * H + t], f[1][e], acc_v2);
                    const float fs = ta_s * xb[t];
                    const float fv1 = ta_v0 * xb[H + t] + ta_v1 * xb[2 * H + t] + ta_v2 * xb[3 * H + t];
                    const float fv2 = ta_v0 * u.x + ta_v1 * u.y + ta_v2 * u.z;
                    float q0 = fs * fd[0][e] + fv1 * fd[1][e] + fv2 * fd[2][e];
                    float q1 = ta_v0 * f[2][e], q2 = ta_v1 * f[2][e], q3 = ta_v2 * f[2][e];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
                        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
                        q2 += __shfl_xor_sync(0xffffffffu, q2, o);
                        q3 += __shfl_xor_sync(0xffffffffu, q3, o);
                    }
                    if (lane == 0) { red[w][e][0] = q0; red[w][e][1] = q1; red[w][e][2] = q2; red[w][e][3] = q3; }
                }
            }
            __syncthreads();
            if (t < n) {
                float4 acc = a.eacc_init ? make_float4(0.f, 0.f, 0.f, 0.f) : a.eacc[t0 + t];
                acc.x += red[0][t][0] + red[1][t][0] + red[2][t][0] + red[3][t][0];
                acc.y += red[0][t][1] + red[1][t][1] + red[2][t][1] + red[3][t][1];
                acc.z += red[0][t][2] + red[1][t][2] + red[2][t][2] + red[3][t][2];
                acc.w += red[0][t][3] + red[1][t][3] + red[2][t][3] + red[3][t][3];
                a.eacc[t0 + t] = acc;
            }
            __syncthreads();
        }
        flush_bwd(a.xtbar, a.xbar, t, cur, j1, acc_s, acc_v0, acc_v1, acc_v2);
    }
}

int launch_edge_fwd_tc(const EdgeArgs& a, int layer, cudaStream_t st);
int launch_edge_bwd_tc(const EdgeArgs& a, int layer, cudaStream_t st);
int launch_vq(const float* P, const LayerOffsets& lo, const float* xtbar, int n_atoms, unsigned char* qs, float* qb,
              Status* st_word, cudaStream_t st);
int launch_etiles(const EdgeArgs& a, int32_t* base, unsigned char* tiles, cudaStream_t st);


__global__ void edge_geom_kernel(EdgeArgs a, float4* __restrict__ geo) {
    pdl_wait();
    pdl_trigger();
    if (a.st->code != 0) return;
    const int n_edges = a.row_ptr[a.n_atoms];
    __shared__ float4 us[256];
    __shared__ int src_s[256], rcv_s[256];
    for (int t0 = blockIdx.x * 256; t0 < n_edges; t0 += gridDim.x * 256) {
        const int n = min(256, n_edges - t0);
        load_edge(a, t0, threadIdx.x, n, us, src_s, rcv_s);
        if ((int)threadIdx.x < n) geo[t0 + threadIdx.x] = us[threadIdx.x];
    }
}

// dst += src over n4 float4 elements (the reverse tensor-core edge kernel
// writes the gathered part of dE/dX only)
int run_tuned(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
              const WsLayout& L, void* ws, const mlff_outputs& out, int path, cudaStream_t st,
              const VerletFuse* vf) {
    const int N = sys.n_atoms;
    const int64_t NX = (int64_t)N * 4 * H;
    int r;
    const bool tc = path == MLFF_PATH_TUNED_TC;
    // the tensor-core path keeps the layer inputs X[0..L-1] and dE/dXt in the
    // pair layout of its edge kernels' gathers
    if ((r = launch_embed(d, P, po, sys, L, ws, st, tc))) return r;
    if ((r = launch_partition(L, ws, st))) return r;
    EdgeArgs a{};
    a.pos4 = ws_ptr<float4>(ws, L.pos4);
    a.atom_mol = ws_ptr<int32_t>(ws, L.atom_mol);
    a.box = sys.box;
    a.pbc = sys.pbc;
    a.row_ptr = ws_ptr<int32_t>(ws, L.row_ptr);
    a.col = ws_ptr<int32_t>(ws, L.col);
    a.erecv = ws_ptr<int32_t>(ws, L.erecv);
    a.part = ws_ptr<int32_t>(ws, L.part);
    a.nparts = L.P;
    a.P = P;
    a.centers = P + po.centers;
    a.gamma = P + po.gamma;
    a.R = d.n_rbf;
    a.cutoff = d.cutoff;
    a.n_atoms = N;
    a.st = ws_ptr<Status>(ws, L.status);
    a.eacc = ws_ptr<float4>(ws, L.edge_acc);
    a.stall_test = g_stall_test.load();
    float* X = ws_ptr<float>(ws, L.X);
    float* Xt = ws_ptr<float>(ws, L.Xt);
    if (tc) {
        float4* geo = ws_ptr<float4>(ws, L.geo);
        ProfScope prof(PK_NEIGHBORS, st);
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((L.cap + 255) / 256, 152 * 8));
        MLFF_LAUNCH_PDL("edge_geom", edge_geom_kernel, blocks, 256, 0, st, a, geo);
        a.geo = geo;
        // [E; E'] tiles (RBF x cutoff and its d-derivative) of every 32 edges,
        // for every layer: the forward kernel reads their E rows, the reverse
        // kernel both
        if ((r = launch_etiles(a, ws_ptr<int32_t>(ws, L.etile_base), ws_ptr<unsigned char>(ws, L.etile), st)))
            return r;
        a.etile = ws_ptr<unsigned char>(ws, L.etile);
        a.etile_base = ws_ptr<int32_t>(ws, L.etile_base);
    }
    for (int l = 0; l < d.n_layers; ++l) {
        a.lo = po.layer[l];
        a.X = X + l * NX;
        a.Xt = Xt + l * NX;
        {
            ProfScope prof(PK_EDGE_FWD, st);
            if (tc) {
                if ((r = launch_edge_fwd_tc(a, l, st))) return r;   // writes Xt = X + messages
            } else {
                edge_fwd_simt_kernel<<<L.P, 128, 0, st>>>(a);
                MLFF_LAUNCH_CHECK("edge_fwd_simt");
            }
        }
        if (tc) r = launch_update_fwd_tc(P, po.layer[l], L, ws, l, st);
        else r = launch_update_fwd(d, P, po.layer[l], L, ws, l, st);
        if (r) return r;
    }
    const bool want_grad = out.forces != nullptr || out.virial != nullptr;
    if ((r = launch_readout(d, P, po, sys, L, ws, out, want_grad ? 1 : 0, st))) return r;
    if (!want_grad) return MLFF_OK;
    float* xbo = ws_ptr<float>(ws, L.xbar);
    float* xtb = xbo + NX;
    for (int l = d.n_layers - 1; l >= 0; --l) {
        if (tc) r = launch_update_bwd_tc(P, po.layer[l], L, ws, l, xbo, xtb, st);
        else r = launch_update_bwd(d, P, po.layer[l], L, ws, l, xbo, xtb, st);
        if (r) return r;
        a.lo = po.layer[l];
        a.X = X + l * NX;
        a.xtbar = xtb;
        a.xbar = xbo;
        a.write_nodes = l > 0 ? 1 : 0;
        a.eacc_init = l == d.n_layers - 1 ? 1 : 0;
        if (tc) {
            ProfScope prof(PK_EDGE_BWD_Q, st);
            a.qs = ws_ptr<unsigned char>(ws, L.qs);
            a.qb = ws_ptr<float>(ws, L.qb);
            if ((r = launch_vq(P, po.layer[l], xtb, L.N, ws_ptr<unsigned char>(ws, L.qs), ws_ptr<float>(ws, L.qb),
                               ws_ptr<Status>(ws, L.status), st)))
                return r;
        }
        {
            ProfScope prof(PK_EDGE_BWD, st);   // the reverse edge kernel alone
            if (tc) {
                if ((r = launch_edge_bwd_tc(a, l, st))) return r;
            } else {
                edge_bwd_simt_kernel<<<L.P, 128, 0, st>>>(a);
                MLFF_LAUNCH_CHECK("edge_bwd_simt");
            }
        }
        // (the tensor-core reverse kernel writes dE/dX = dE/dXt + the gathered part itself)
    }
    return launch_forces(d, sys, L, ws, out, st, vf);
}

}  // namespace mlff
