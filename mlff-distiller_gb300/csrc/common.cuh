// Shared definitions for the mlff_gb300 CUDA library (sm_103a).
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include <utility>
#include "../../include/mlff_gb300.h"

namespace mlff {

constexpr int H = 128;        // hidden width (StudentForceField default)
constexpr int H3 = 3 * H;     // filter / update output width
constexpr int RMAX = 32;      // padded number of radial basis functions
constexpr int MAXL = 8;       // maximum number of interaction blocks

// Device status word layout (int32[8], lives in the workspace).
//   [0] status code (MLFF_OK or an MLFF_ERR_* value)
//   [1] edges found by the neighbour build (low 31 bits; saturates)
//   [2] first offending atom / molecule for row or box errors
//   [3] edge count high word (edges >> 31)
struct Status {
    int32_t code;
    int32_t n_edges;
    int32_t where;
    int32_t n_edges_hi;
    int32_t pad[4];
};

__device__ __forceinline__ void set_status(Status* st, int code, int where) {
    if (atomicCAS(&st->code, 0, code) == 0) st->where = where;
}

// Programmatic dependent launch.  A kernel launched by MLFF_LAUNCH_PDL may be
// scheduled while the kernel before it in the stream is still running, as
// soon as that kernel has executed pdl_trigger() in every CTA (or exited).
// Rules every such kernel follows:
//  * pdl_wait() in every thread before it reads or writes any buffer an
//    earlier kernel of the stream touches (the status word included) and
//    before it can return; only packed weights and shared memory come before
//    it, so that the prologue overlaps the previous kernel;
//  * pdl_trigger() only after pdl_wait() and, in kernels that own tensor
//    memory, only after the allocation (a dependent CTA then never holds
//    columns a CTA of this kernel still waits for).
// Both are no-ops in a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ float silu_f(float x) {
    return x / (1.0f + expf(-x));
}
// sigmoid and silu'(z) = s (1 + z (1 - s))
__device__ __forceinline__ float sigmoid_f(float x) { return 1.0f / (1.0f + expf(-x)); }
__device__ __forceinline__ float dsilu_f(float x) {
    float s = sigmoid_f(x);
    return s * (1.0f + x * (1.0f - s));
}

// Pair layout of the tensor-core path's node features and adjoints (the
// layer inputs X[0..L-1] and dE/dXt): per atom, (s, v_x) of channel c at
// floats 2c, 2c + 1 and (v_y, v_z) at 2H + 2c, 2H + 2c + 1, so that a thread
// that owns two components of one channel loads both with one 8-byte
// access.  (The other per-atom arrays keep the component-major layout
// comp * H + c.)
__host__ __device__ constexpr int pair_off(int comp, int c) { return (comp >> 1) * 2 * H + 2 * c + (comp & 1); }

// Velocity-Verlet half kick v + dt/2 F/m in float64 (F is the float32
// force) and the kinetic energy 1/2 m v^2 of one atom; the integrator
// kernels and the force kernel's fused update share these expressions.
__device__ __forceinline__ double verlet_half_kick(double v, float f, double inv_mass, double dt) {
    return v + 0.5 * dt * (double)f * inv_mass;
}
__device__ __forceinline__ double kinetic_term(double vx, double vy, double vz, double inv_mass) {
    return 0.5 * (vx * vx + vy * vy + vz * vz) / inv_mass;
}

// float32 |d| rounded as the reference's torch.norm: x*x rounded, then two
// fused multiply-adds, then a correctly rounded square root.
__device__ __forceinline__ float pair_distance(float dx, float dy, float dz) {
    return __fsqrt_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))));
}

// Minimum image along one periodic axis: k = rint(dx / L) (via the rounded
// reciprocal), dx' = fma(-k, L, dx).  Exactly antisymmetric in dx.
__device__ __forceinline__ float min_image(float dx, float L, float invL) {
    float k = rintf(__fmul_rn(dx, invL));
    return __fmaf_rn(-k, L, dx);
}

struct Box {
    float L[3];
    float invL[3];
    int periodic;
};

// Edge vector r = pos[src] - pos[dst] (+ minimum image) exactly as the
// neighbour build decided it.
__device__ __forceinline__ float3 edge_vector(float4 ps, float4 pd, const Box& b) {
    float dx = __fsub_rn(ps.x, pd.x);
    float dy = __fsub_rn(ps.y, pd.y);
    float dz = __fsub_rn(ps.z, pd.z);
    if (b.periodic) {
        dx = min_image(dx, b.L[0], b.invL[0]);
        dy = min_image(dy, b.L[1], b.invL[1]);
        dz = min_image(dz, b.L[2], b.invL[2]);
    }
    return make_float3(dx, dy, dz);
}

// Packed fp32 parameters (built by mlff_pack_weights from the state_dict).
// All offsets are in floats from the start of the packed blob.
struct LayerOffsets {
    int64_t w1t;    // [RMAX][H]   filter Linear(R->H) weight, transposed, zero padded
    int64_t w1;     // [H][RMAX]   same, original orientation
    int64_t b1;     // [H]
    int64_t w2t;    // [H][H3]     filter Linear(H->3H) weight, transposed
    int64_t w2;     // [H3][H]     original orientation
    int64_t b2;     // [H3]
    int64_t mix;    // [9]
    int64_t u1t;    // [2H][H]     update Linear(2H->H), transposed
    int64_t u1;     // [H][2H]
    int64_t c1;     // [H]
    int64_t u2t;    // [H][H3]     update Linear(H->3H), transposed
    int64_t u2;     // [H3][H]
    int64_t c2;     // [H3]
    int64_t w1_bf;  // split-fp16 hi/lo tiles for the tensor-core filter (bytes offset / 4)
    int64_t w2_bf;
    int64_t w2_tm;  // lo halves of W2 rows [0,2H) as the TMEM image of the filter kernels ([4][32][H] u32)
    int64_t u1_tc;  // split-fp16 A-operand tile pairs of the tensor-core update MLP:
    int64_t u2_tc;  //   U1 [H][2H] and U2 [3H][H] (forward),
    int64_t u2t_tc; //   U2^T [H][3H] and U1^T [2H][H] (reverse)
    int64_t u1t_tc;
    int64_t w2q_tc; // W2 rows [2H,3H) transposed as split-fp16 A tiles (reverse pass: per-atom Q rows)
};

struct PackedOffsets {
    int64_t emb;       // [S][H]
    int64_t centers;   // [RMAX]
    int64_t gamma;     // [RMAX]  1/w^2 (0 for padding)
    int64_t head_w1t;  // [H][64]
    int64_t head_w1;   // [64][H]
    int64_t head_b1;   // [64]
    int64_t head_w2t;  // [64][32]
    int64_t head_w2;   // [32][64]
    int64_t head_b2;   // [32]
    int64_t head_w3;   // [32]
    int64_t head_b3;   // [1]
    LayerOffsets layer[MAXL];
    int64_t total;     // floats
};

PackedOffsets packed_offsets(const mlff_dims& d);

}  // namespace mlff

// ----- error handling shared by the host side of the library -----
namespace mlff {
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);
int num_sms();   // streaming multiprocessors of the current device (cached)
void prof_count_launch();   // profile.cu: one kernel launch of the current kind
}

#define MLFF_CUDA(call)                                                     \
    do {                                                                    \
        cudaError_t _e = (call);                                            \
        if (_e != cudaSuccess) return mlff::cuda_status(_e, #call);         \
    } while (0)

namespace mlff {
bool pdl_enabled();   // programmatic dependent launch (on unless MLFF_PDL=0)
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
}  // namespace mlff

// Launch of a kernel that follows the pdl_wait / pdl_trigger rules, with the
// same accounting and error check as MLFF_LAUNCH_CHECK.
#define MLFF_LAUNCH_PDL(what, kernel, grid, block, smem, st, ...)                      \
    do {                                                                              \
        cudaError_t _e = mlff::launch_pdl(kernel, grid, block, smem, st, __VA_ARGS__); \
        mlff::prof_count_launch();                                                    \
        if (_e != cudaSuccess) return mlff::cuda_status(_e, what);                    \
    } while (0)

// Every kernel launch is followed by this check (it also counts the launch
// for the optional benchmark profile).
#define MLFF_LAUNCH_CHECK(what)                                             \
    do {                                                                    \
        cudaError_t _e = cudaGetLastError();                                \
        mlff::prof_count_launch();                                          \
        if (_e != cudaSuccess) return mlff::cuda_status(_e, what);          \
    } while (0)
