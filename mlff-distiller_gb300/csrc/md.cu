// Velocity-Verlet NVE and Langevin (BAOAB) NVT integrator kernels, float64
// state.  One Verlet step is
//   v += dt/2 F/m ; r += dt v ; (float32 copy of r) -> F(r) ; v += dt/2 F/m
// which is what ASE's VelocityVerlet does per step when driven by
// NVEMDHarness.run_simulation (src/mlff_distiller/testing/nve_harness.py:
// 173-261; the integrator itself lives in the un-vendored ASE package).
#include <algorithm>
#include <cmath>
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

// The closing half kick; it also advances the step counter (when given) that
// the next step's random draws are keyed by.
__global__ void kick_kernel(double* __restrict__ vel, const double* __restrict__ inv_mass,
                            const float* __restrict__ F, double dt, int32_t n_atoms, int64_t* __restrict__ step_counter,
                            const Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    if (step_counter && blockIdx.x == 0 && threadIdx.x == 0) *step_counter += 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n_atoms; i += gridDim.x * blockDim.x)
        vel[i] += 0.5 * dt * (double)F[i] * inv_mass[i / 3];
}

// ------------------------------------------------------------ Langevin
// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11): ten rounds of two
// 32x32->64-bit multiplies on a 4-word counter, the 2-word key bumped by
// the Weyl constants between rounds.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// BAOA of one BAOAB step (Leimkuhler and Matthews, J. Chem. Phys. 138,
// 174102 (2013)): v += dt/2 F/m; r += dt/2 v; v = c1 v + c2 sqrt(kT/m) xi;
// r += dt/2 v.  xi: three standard normals per atom by Box-Muller from one
// Philox block keyed by the seed, counter (step, atom): the draw does not
// depend on the launch shape.  The step number is read from device memory
// so that a captured graph draws new numbers on every replay.
__global__ void langevin_baoa_kernel(double* __restrict__ pos, double* __restrict__ vel,
                                     const double* __restrict__ inv_mass, const float* __restrict__ F, double dt,
                                     double c1, double c2, double kT, uint64_t seed,
                                     const int64_t* __restrict__ step_counter, int32_t n_atoms,
                                     float* __restrict__ pos32, const Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    const uint64_t step = (uint64_t)*step_counter;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n_atoms; a += gridDim.x * blockDim.x) {
        const uint4 x = philox4x32_10(make_uint4((uint32_t)step, (uint32_t)(step >> 32), (uint32_t)a, 0u),
                                      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
        const double u0 = ((double)x.x + 0.5) * 0x1p-32, u1 = ((double)x.y + 0.5) * 0x1p-32;
        const double u2 = ((double)x.z + 0.5) * 0x1p-32, u3 = ((double)x.w + 0.5) * 0x1p-32;
        const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
        double s0, k0, s1, k1;
        sincospi(2.0 * u1, &s0, &k0);
        sincospi(2.0 * u3, &s1, &k1);
        const double xi[3] = {r0 * k0, r0 * s0, r1 * k1};
        const double sig = c2 * sqrt(kT * inv_mass[a]);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int i = 3 * a + d;
            double v = vel[i] + 0.5 * dt * (double)F[i] * inv_mass[a];
            double r = pos[i] + 0.5 * dt * v;
            v = c1 * v + sig * xi[d];
            r += 0.5 * dt * v;
            vel[i] = v;
            pos[i] = r;
            pos32[i] = (float)r;
        }
    }
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

int md_langevin_baoa(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT,
                     uint64_t seed, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    const double c1 = exp(-friction * dt);
    const double c2 = sqrt(std::max(0.0, 1.0 - c1 * c1));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((L.N + 255) / 256, 152 * 8));
    MLFF_LAUNCH_PDL("langevin_baoa", langevin_baoa_kernel, blocks, 256, 0, st, s->pos, s->vel, s->inv_mass, s->forces,
                    dt, c1, c2, kT, seed, s->step_counter, L.N, ws_ptr<float>(ws, L.md_pos32),
                    ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

int md_kick(const WsLayout& L, void* ws, mlff_md_state* s, double dt, const int64_t* mol_ptr, int32_t n_mol,
            bool kinetic, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((3LL * L.N + 255) / 256, 152 * 8));
    MLFF_LAUNCH_PDL("kick", kick_kernel, blocks, 256, 0, st, s->vel, s->inv_mass, s->forces, dt, L.N, s->step_counter,
                    ws_ptr<Status>(ws, L.status));
    if (kinetic && s->kinetic) {
        MLFF_LAUNCH_PDL("kinetic", kinetic_kernel, std::min(std::max(n_mol, 1), 152 * 8), 256, 0, st, s->vel, s->inv_mass, mol_ptr, n_mol,
                                                                              s->kinetic);
    }
    return MLFF_OK;
}

}  // namespace mlff
