// Velocity-Verlet NVE integrator kernels, float64 state.  One step is
//   v += dt/2 F/m ; r += dt v ; (float32 copy of r) -> F(r) ; v += dt/2 F/m
// which is what ASE's VelocityVerlet does per step when driven by
// NVEMDHarness.run_simulation (src/mlff_distiller/testing/nve_harness.py:
// 173-261; the integrator itself lives in the un-vendored ASE package).
#include "common.cuh"
#include "workspace.h"
#include "profile.h"

namespace mlff {

__global__ void kick_drift_kernel(double* __restrict__ pos, double* __restrict__ vel,
                                  const double* __restrict__ inv_mass, const float* __restrict__ F, double dt,
                                  int32_t n_atoms, float* __restrict__ pos32, const Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n_atoms; i += gridDim.x * blockDim.x) {
        const int a = i / 3;
        const double v = vel[i] + 0.5 * dt * (double)F[i] * inv_mass[a];
        vel[i] = v;
        const double p = pos[i] + dt * v;
        pos[i] = p;
        pos32[i] = (float)p;
    }
}

__global__ void kick_kernel(double* __restrict__ vel, const double* __restrict__ inv_mass,
                            const float* __restrict__ F, double dt, int32_t n_atoms, const Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n_atoms; i += gridDim.x * blockDim.x)
        vel[i] += 0.5 * dt * (double)F[i] * inv_mass[i / 3];
}

// kinetic energy 1/2 m v^2 per structure (fixed-order tree)
__global__ void kinetic_kernel(const double* __restrict__ vel, const double* __restrict__ inv_mass,
                               const int64_t* __restrict__ mol_ptr, int32_t n_mol, double* __restrict__ ke) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[256];
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        double s = 0.0;
        for (int64_t a = mol_ptr[m] + threadIdx.x; a < mol_ptr[m + 1]; a += blockDim.x) {
            const double v2 = vel[3 * a] * vel[3 * a] + vel[3 * a + 1] * vel[3 * a + 1] + vel[3 * a + 2] * vel[3 * a + 2];
            s += 0.5 * v2 / inv_mass[a];
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) ke[m] = red[0];
        __syncthreads();
    }
}

int md_kick_drift(const WsLayout& L, void* ws, mlff_md_state* s, double dt, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((3LL * L.N + 255) / 256, 152 * 8));
    MLFF_LAUNCH_PDL("kick_drift", kick_drift_kernel, blocks, 256, 0, st, s->pos, s->vel, s->inv_mass, s->forces, dt, L.N,
                                              ws_ptr<float>(ws, L.md_pos32), ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

int md_kick(const WsLayout& L, void* ws, mlff_md_state* s, double dt, const int64_t* mol_ptr, int32_t n_mol,
            bool kinetic, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((3LL * L.N + 255) / 256, 152 * 8));
    MLFF_LAUNCH_PDL("kick", kick_kernel, blocks, 256, 0, st, s->vel, s->inv_mass, s->forces, dt, L.N, ws_ptr<Status>(ws, L.status));
    if (kinetic && s->kinetic) {
        MLFF_LAUNCH_PDL("kinetic", kinetic_kernel, std::min(std::max(n_mol, 1), 152 * 8), 256, 0, st, s->vel, s->inv_mass, mol_ptr, n_mol,
                                                                              s->kinetic);
    }
    return MLFF_OK;
}

}  // namespace mlff
