// Workspace layout: one caller-owned device buffer carved into the arrays
// the kernels need.  Everything is addressed by byte offsets aligned to 256.
#pragma once
#include <cstddef>
#include <cstdint>
#include "common.cuh"

namespace mlff {

constexpr int GRAD_SPLIT = 64;        // row splits of the weight-gradient reductions
constexpr int GRAD_MIX_BLOCKS = 304;  // blocks of the mixing-matrix gradient

struct WsLayout {
    int32_t N, B, L, P;        // atoms, structures, layers, persistent CTAs
    int32_t UT;                // atoms per tile of the tensor-core update kernels (64 or 32)
    int64_t cap;               // edge capacity
    int64_t ncell_cap;         // cell-code capacity, 8 (N + 27 B) (Morton code spaces of the cell grids)
    size_t status;             // Status
    size_t pos4;               // float4 [N]
    size_t atom_mol;           // int32 [N]
    size_t row_ptr;            // int32 [N+1]
    size_t col;                // int32 [cap]  sender of each edge
    size_t erecv;              // int32 [cap]  receiver of each edge
    size_t rev;                // int32 [cap]  index of the reversed edge
    size_t edge_acc;           // float4 [cap] (dE/dd, dE/du) summed over layers
    size_t scan_tmp;           // int32 [scan_blocks + 1]
    size_t mol_grid;           // int4 [B + 1]  (ncx, ncy, ncz, first cell code); [B].x = codes in use
    size_t mol_box;            // float4 [2 B]  open structures with a cell grid: origin, 1 / cell width
    size_t cell_count;         // int32 [ncell_cap + 1]
    size_t cell_fill;          // int32 [ncell_cap]
    size_t cell_pos;           // float4 [N]  atoms in cell order: x, y, z, atom index (int bits)
    size_t atom_cell;          // int32 [N]
    size_t part;               // int32 [P + 1] receiver partition
    size_t X;                  // float [L+1][N][4][H]  layer inputs (s, v_x, v_y, v_z)
    size_t Xt;                 // float [L][N][4][H]    after the message step
    size_t uz;                 // float [L][N][H]       update MLP pre-activation
    size_t ua;                 // float [L][N][3H]      update MLP output (ds, g1, g2)
    size_t xbar;               // float [2][N][4][H]    adjoints
    size_t e_atom;             // float [N]
    size_t md_pos32;           // float [N][3]  positions the integrator hands to the force call
    size_t md_noise;           // double [N][6] Langevin normals of a step (ASE's scheme: xi, eta)
    // plain path (materialised per-edge tensors, like the reference's graph)
    size_t geo;                // float4 [cap] (u_x, u_y, u_z, d)
    size_t etile_base;         // int32 [P+1] first [E; E'] tile of each partition
    size_t etile;              // [E; E'] tiles: 32 edges, 64 rows (E, then E'), split fp16, 8 KB each
    size_t qs;                 // reverse: per-atom Q rows [N][3][hi, lo][H] fp16 (W2's third chunk^T dE/dXt_v)
    size_t qb;                 // reverse: per-atom b2 . dE/dXt_v [N][3] float
    int64_t n_etile;
    size_t erbf;               // float [cap][RMAX]
    size_t erbf_d;             // float [cap][RMAX]
    size_t fz;                 // float [L][cap][H]
    size_t ff;                 // float [L][cap][3H]
    size_t fh;                 // float [cap][H]
    size_t fbar;               // float [cap][3H]
    size_t comb;               // float [N][2H]
    size_t uh;                 // float [N][H]
    size_t abar;               // float [N][3H]
    // parameter-gradient paths only (float arrays of the plain path hold
    // (value, tangent) pairs, twice the size, on MLFF_PATH_TRAIN_FORCES)
    size_t gcomb;              // float [N][2H]   update-MLP input recomputed per layer
    size_t ghead;              // float [N][193]  readout: h1 (64), a1bar (64), h2 (32), a2bar (32), ebar (1)
    size_t gpart;              // float [GRAD_SPLIT][3H*H] partial weight gradients
    size_t gmix;               // float [GRAD_MIX_BLOCKS][9] partial mixing-matrix gradients
    size_t total;
};

WsLayout ws_layout(const mlff_dims& d, int32_t n_atoms, int32_t n_mol, int64_t cap, int32_t path);

template <typename T>
inline T* ws_ptr(void* ws, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}
template <typename T>
inline const T* ws_ptr(const void* ws, size_t off) {
    return reinterpret_cast<const T*>(static_cast<const char*>(ws) + off);
}

// Buffers of one radius-graph build given as explicit device pointers.
struct NbrBuffers {
    Status* status;
    float4* pos4;           // [N]
    int32_t* atom_mol;      // [N]
    int32_t* row_ptr;       // [N+1]
    int32_t* col;           // [cap]
    int32_t* erecv;         // [cap]
    int32_t* scan_tmp;      // [(max(N+1, ncell_cap+1) + 1023) / 1024 + 2]
    int4* mol_grid;         // [B + 1]
    float4* mol_box;        // [2 B] open structures with a cell grid: origin (then upper corner), 1 / cell width
    int32_t* cell_count;    // [ncell_cap + 1]
    int32_t* cell_fill;     // [ncell_cap]
    float4* cell_pos;       // [N] atoms in cell order (x, y, z, index bits)
    int32_t* atom_cell;     // [N]
    int64_t ncell_cap;      // 8 (N + 27 B): the Morton code spaces of the cell grids
    int64_t cap;            // edge capacity
};

// Kernel launch helpers implemented in the .cu files.
int launch_neighbors_into(const mlff_dims& d, const mlff_system& sys, const NbrBuffers& b, cudaStream_t st);
int launch_neighbors(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws,
                     cudaStream_t st);
// X[0] component-major or (pairs: the tensor-core path) in the pair layout
int launch_embed(const mlff_dims& d, const float* packed, const PackedOffsets& po,
                 const mlff_system& sys, const WsLayout& L, void* ws, cudaStream_t st, bool pairs = false);
int launch_readout(const mlff_dims& d, const float* packed, const PackedOffsets& po,
                   const mlff_system& sys, const WsLayout& L, void* ws, const mlff_outputs& out,
                   int want_grad, cudaStream_t st);
// Velocity-Verlet update fused into the force kernel: with the new force F
// of atom a, the closing half kick v += dt/2 F/m of this step, the atom's
// kinetic energy 1/2 m v^2 (into ke_atom, when given), and, with open_next,
// the next step's opening half kick and drift (v += dt/2 F/m; r += dt v;
// pos32 = (float)r).  step_counter (when given) advances by one.
struct VerletFuse {
    double* vel;
    const double* inv_mass;
    double* pos;
    float* pos32;
    double* ke_atom;
    int64_t* step_counter;
    double dt;
    int open_next;
};
int launch_forces(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws,
                  const mlff_outputs& out, cudaStream_t st, const VerletFuse* vf = nullptr);
// Training: per-structure loss weights dL/dE_b and the gradient outputs.
struct GradCtx {
    const double* w;
    mlff_grads g;
};
int run_plain(const mlff_dims& d, const float* packed, const PackedOffsets& po,
              const mlff_system& sys, const WsLayout& L, void* ws, const mlff_outputs& out,
              cudaStream_t st, const GradCtx* grad = nullptr, const VerletFuse* vf = nullptr);
// Pass of the plain path over (value, tangent) pairs along positions moved
// by -pos_t [N][3] and cells strained by strain_t [B][3][3] (either may be
// NULL): adds the derivative of grad_theta sum_b E_b along that direction
// to every non-NULL gradient in grad.g (grad.w unused), i.e. sum_i G_i .
// dF_i/dtheta + sum_b S_b : dW_b/dtheta.
int run_plain_tangent(const mlff_dims& d, const float* packed, const PackedOffsets& po,
                      const mlff_system& sys, const WsLayout& L, void* ws, cudaStream_t st,
                      const GradCtx& grad, const float* pos_t, const double* strain_t);
// Weight-gradient reductions of the plain path's reverse pass, over float
// or Dual scalars (instantiated in grads.cu).
template <class T>
int grad_readout(const mlff_dims& d, const float* P, const PackedOffsets& po, const mlff_system& sys,
                 const WsLayout& L, void* ws, const double* w, const mlff_grads& g, cudaStream_t st);
template <class T>
int grad_update_out(const WsLayout& L, void* ws, int l, const T* xbo, const mlff_grads& g, cudaStream_t st);
template <class T>
int grad_update_in(const WsLayout& L, void* ws, int l, const T* zbar_u, const T* comb_l,
                   const mlff_grads& g, cudaStream_t st);
template <class T>
int grad_filter_out(const WsLayout& L, void* ws, int l, const int32_t* E_dev, const mlff_grads& g, cudaStream_t st);
template <class T>
int grad_filter_in(const mlff_dims& d, const WsLayout& L, void* ws, int l, const int32_t* E_dev, const mlff_grads& g,
                   cudaStream_t st);
template <class T>
int grad_embedding(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws, const T* xbar0,
                   const mlff_grads& g, cudaStream_t st);
int run_tuned(const mlff_dims& d, const float* packed, const PackedOffsets& po,
              const mlff_system& sys, const WsLayout& L, void* ws, const mlff_outputs& out,
              int path, cudaStream_t st, const VerletFuse* vf = nullptr);
int launch_partition(const WsLayout& L, void* ws, cudaStream_t st);
int launch_scan(int32_t* data, int64_t n, int32_t* tmp, cudaStream_t st);
int launch_update_fwd(const mlff_dims& d, const float* packed, const LayerOffsets& lo,
                      const WsLayout& L, void* ws, int layer, cudaStream_t st);
int launch_update_fwd_tc(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                         cudaStream_t st);
int launch_update_bwd_tc(const float* packed, const LayerOffsets& lo, const WsLayout& L, void* ws, int layer,
                         const float* xbar_out, float* xtbar, cudaStream_t st);
int launch_update_bwd(const mlff_dims& d, const float* packed, const LayerOffsets& lo,
                      const WsLayout& L, void* ws, int layer, const float* xbar_out,
                      float* xtbar, cudaStream_t st);

}  // namespace mlff
