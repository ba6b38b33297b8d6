// Pieces shared by the fused edge kernels (CUDA-core and tensor-core).
#pragma once
#include "common.cuh"

namespace mlff {

constexpr float PI_FC = 3.14159265358979f;

struct EdgeArgs {
    const float4* pos4;
    const float4* geo;        // optional per-edge (u_x, u_y, u_z, d), computed once per call
    const unsigned char* etile;       // tensor-core path: precomputed E tiles of this pass
    const int32_t* etile_base;        // first tile of each partition
    const int32_t* atom_mol;
    const float* box;
    const uint8_t* pbc;
    const int32_t* row_ptr;
    const int32_t* col;       // sender of each edge
    const int32_t* erecv;     // receiver of each edge
    const int32_t* part;      // receiver partition [nparts + 1]
    int32_t nparts;
    const float* P;           // packed fp32 parameters
    LayerOffsets lo;
    const float* centers;
    const float* gamma;
    int R;
    float cutoff;
    const float* X;           // layer input [N][4][H]
    float* Xt;                // forward: after the message step
    const float* xtbar;       // reverse: dE/dXt
    float* xbar;              // reverse: dE/dX
    float4* eacc;             // reverse: per-edge (dE/dd, dE/du)
    const unsigned char* qs;  // reverse, tensor-core path: per-atom Q rows (split fp16) of the current layer
    const float* qb;          // reverse, tensor-core path: per-atom b2 . dE/dXt_v of the current layer
    int32_t eacc_init;        // reverse: 1 = first layer processed, eacc is written rather than added to
    int32_t write_nodes;      // reverse: also produce dE/dX (unused for the first layer)
    int32_t n_atoms;
    int32_t stall_test;       // tensor-core kernels, test hook: time out at the first main-loop wait
    const Status* st;
};

// 0.5 (cos(pi d / rc) + 1) [d < rc]  (CosineCutoff.forward, student_model.py:284-292)
__device__ __forceinline__ float cutoff_fn(float d, float rc) {
    return d < rc ? 0.5f * (cosf(PI_FC * d / rc) + 1.0f) : 0.0f;
}

__device__ __forceinline__ void cutoff_fn_d(float d, float rc, float& fc, float& dfc) {
    if (d < rc) {
        const float arg = PI_FC * d / rc;
        fc = 0.5f * (cosf(arg) + 1.0f);
        dfc = -0.5f * (PI_FC / rc) * sinf(arg);
    } else {
        fc = 0.0f;
        dfc = 0.0f;
    }
}

// Thread t < n of a tile loads edge t0 + t: (u, d), sender and receiver.
// Padding slots get d = 0 (masked out by the callers through n).
__device__ __forceinline__ void load_edge(const EdgeArgs& a, int t0, int t, int n, float4* us, int* src_s,
                                          int* rcv_s) {
    if (t < n && a.geo) {
        const int k = t0 + t;
        us[t] = a.geo[k];
        src_s[t] = a.col[k];
        rcv_s[t] = a.erecv[k];
    } else if (t < n) {
        const int k = t0 + t;
        const int ra = a.erecv[k], sb = a.col[k];
        const int m = a.atom_mol[ra];
        Box bx;
        bx.periodic = (a.pbc != nullptr && a.box != nullptr && a.pbc[m]) ? 1 : 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            bx.L[q] = bx.periodic ? a.box[3 * m + q] : 1.0f;
            bx.invL[q] = __fdiv_rn(1.0f, bx.L[q]);
        }
        const float3 r = edge_vector(a.pos4[sb], a.pos4[ra], bx);
        const float d = pair_distance(r.x, r.y, r.z);
        const float inv = 1.0f / (d + 1e-8f);
        us[t] = make_float4(r.x * inv, r.y * inv, r.z * inv, d);
        src_s[t] = sb;
        rcv_s[t] = ra;
    } else {
        us[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        src_s[t] = 0;
        rcv_s[t] = -1;
    }
}

// Per-edge geometry for edges [0, n_edges): (u, d) exactly as load_edge
// computes it, once per call instead of once per layer and pass.
__global__ void edge_geom_kernel(EdgeArgs a, float4* __restrict__ geo);

}  // namespace mlff
