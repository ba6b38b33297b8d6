// Velocity-Verlet NVE, Langevin (BAOAB) NVT and Nose-Hoover /
// Parrinello-Rahman NPT integrator kernels, float64 state.  One Verlet step is
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
        const double v = verlet_half_kick(vel[i], F[i], inv_mass[a], dt);
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
        vel[i] = verlet_half_kick(vel[i], F[i], inv_mass[i / 3], dt);
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

// ------------------------------------------------- Langevin, ASE's scheme
// The propagator of Vanden-Eijnden and Ciccotti (Chem. Phys. Lett. 429, 310
// (2006), Eq. 23), the one ASE's Langevin integrates, with ASE's default of
// a fixed centre of mass per structure.  Per step, with gamma the friction,
// sigma = sqrt(2 kT gamma / m) and two standard-normal vectors xi, eta per
// atom:
//   v += c1 F/m - c2 v + c3 xi - c4 eta
//   r += dt v + c5 eta    (then, with fix_com, every atom of a structure is
//                          shifted back by its centre-of-mass change and v
//                          takes that shift / dt: v = (r_new - r - c5 eta)/dt)
//   F = F(r)
//   v += c1 F/m - c2 v + c3 xi - c4 eta;  with fix_com v -= its centre-of-mass velocity
// c1 = dt/2 - dt^2 gamma/8, c2 = gamma dt/2 - gamma^2 dt^2/8,
// c3 = sqrt(dt) sigma/2 - dt^1.5 gamma sigma/8, c5 = dt^1.5 sigma/(2 sqrt 3),
// c4 = gamma c5/2.  The six normals of an atom come from two Philox blocks
// keyed by (seed; step, atom, 1) and (seed; step, atom, 2), Box-Muller on
// consecutive uniform pairs; xi = the first three, eta = the next three.
// The open kernel stores them for the close kernel, which advances the step
// counter (no kernel reads and writes the counter).
struct VecCoef {
    double c1, c2, c3, c4, c5;
};
__device__ __forceinline__ VecCoef vec_coef(double dt, double gamma, double kT, double inv_m) {
    const double sigma = sqrt(2.0 * kT * gamma * inv_m);
    VecCoef c;
    c.c1 = 0.5 * dt - dt * dt * gamma / 8.0;
    c.c2 = 0.5 * gamma * dt - gamma * gamma * dt * dt / 8.0;
    c.c3 = 0.5 * sqrt(dt) * sigma - dt * sqrt(dt) * gamma * sigma / 8.0;
    c.c5 = dt * sqrt(dt) * sigma / (2.0 * sqrt(3.0));
    c.c4 = 0.5 * gamma * c.c5;
    return c;
}
__device__ __forceinline__ void box_muller4(uint4 x, double* n) {
    const double u0 = ((double)x.x + 0.5) * 0x1p-32, u1 = ((double)x.y + 0.5) * 0x1p-32;
    const double u2 = ((double)x.z + 0.5) * 0x1p-32, u3 = ((double)x.w + 0.5) * 0x1p-32;
    const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
    double s0, k0, s1, k1;
    sincospi(2.0 * u1, &s0, &k0);
    sincospi(2.0 * u3, &s1, &k1);
    n[0] = r0 * k0;
    n[1] = r0 * s0;
    n[2] = r1 * k1;
    n[3] = r1 * s1;
}

constexpr int VEC_NT = 256;
// sum of 8 doubles over the block, fixed tree; every thread gets the sums
__device__ __forceinline__ void block_sum8(double (&v)[8], double (*red)[VEC_NT]) {
    const int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < 8; ++j) red[j][t] = v[j];
    __syncthreads();
    for (int o = VEC_NT / 2; o > 0; o >>= 1) {
        if (t < o)
#pragma unroll
            for (int j = 0; j < 8; ++j) red[j][t] += red[j][t + o];
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = red[j][0];
    __syncthreads();
}

// first half of a step and the drift, one block per structure
__global__ void __launch_bounds__(VEC_NT) vec_open_kernel(double* __restrict__ pos, double* __restrict__ vel,
                                                          const double* __restrict__ inv_mass,
                                                          const float* __restrict__ F, double dt, double gamma,
                                                          double kT, uint64_t seed,
                                                          const int64_t* __restrict__ step_counter,
                                                          const int64_t* __restrict__ mol_ptr, int32_t n_mol,
                                                          int32_t fix_com, double* __restrict__ noise,
                                                          float* __restrict__ pos32, const Status* st) {
    __shared__ double red[8][VEC_NT];
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    const uint64_t step = (uint64_t)*step_counter;
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        const int64_t a0 = mol_ptr[m], a1 = mol_ptr[m + 1];
        double acc[8] = {};   // sum m r_old (3), sum m r_new (3), total mass
        for (int64_t a = a0 + threadIdx.x; a < a1; a += VEC_NT) {
            double nz[8];
            box_muller4(philox4x32_10(make_uint4((uint32_t)step, (uint32_t)(step >> 32), (uint32_t)a, 1u), key), nz);
            box_muller4(philox4x32_10(make_uint4((uint32_t)step, (uint32_t)(step >> 32), (uint32_t)a, 2u), key),
                        nz + 4);
#pragma unroll
            for (int j = 0; j < 6; ++j) noise[6 * a + j] = nz[j];
            const double im = inv_mass[a], mass = 1.0 / im;
            const VecCoef c = vec_coef(dt, gamma, kT, im);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int64_t i = 3 * a + d;
                double v = vel[i];
                v += c.c1 * (double)F[i] * im - c.c2 * v + c.c3 * nz[d] - c.c4 * nz[3 + d];
                const double r0 = pos[i], r = r0 + dt * v + c.c5 * nz[3 + d];
                vel[i] = v;
                pos[i] = r;
                acc[d] += mass * r0;
                acc[3 + d] += mass * r;
            }
            acc[6] += mass;
        }
        if (fix_com) {
            block_sum8(acc, red);
            double sh[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) sh[d] = (acc[d] - acc[3 + d]) / acc[6];
            for (int64_t a = a0 + threadIdx.x; a < a1; a += VEC_NT)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int64_t i = 3 * a + d;
                    const double r = pos[i] + sh[d];
                    pos[i] = r;
                    vel[i] += sh[d] / dt;
                    pos32[i] = (float)r;
                }
        } else {
            for (int64_t a = a0 + threadIdx.x; a < a1; a += VEC_NT)
#pragma unroll
                for (int d = 0; d < 3; ++d) pos32[3 * a + d] = (float)pos[3 * a + d];
        }
    }
}

// second half of a step at the new forces, centre-of-mass velocity removed,
// kinetic energy per structure (when ke is given); advances the step counter
__global__ void __launch_bounds__(VEC_NT) vec_close_kernel(double* __restrict__ vel, const double* __restrict__ inv_mass,
                                                           const float* __restrict__ F, double dt, double gamma,
                                                           double kT, const double* __restrict__ noise,
                                                           const int64_t* __restrict__ mol_ptr, int32_t n_mol,
                                                           int32_t fix_com, double* __restrict__ ke,
                                                           int64_t* __restrict__ step_counter, const Status* st) {
    __shared__ double red[8][VEC_NT];
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) *step_counter += 1;
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        const int64_t a0 = mol_ptr[m], a1 = mol_ptr[m + 1];
        double acc[8] = {};   // sum m v (3), total mass, sum m v^2
        for (int64_t a = a0 + threadIdx.x; a < a1; a += VEC_NT) {
            const double im = inv_mass[a], mass = 1.0 / im;
            const VecCoef c = vec_coef(dt, gamma, kT, im);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int64_t i = 3 * a + d;
                double v = vel[i];
                v += c.c1 * (double)F[i] * im - c.c2 * v + c.c3 * noise[6 * a + d] - c.c4 * noise[6 * a + 3 + d];
                vel[i] = v;
                acc[d] += mass * v;
                acc[4] += mass * v * v;
            }
            acc[3] += mass;
        }
        if (fix_com || ke) block_sum8(acc, red);
        if (fix_com) {
            double vc[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) vc[d] = acc[d] / acc[3];
            double k2[8] = {};
            for (int64_t a = a0 + threadIdx.x; a < a1; a += VEC_NT) {
                const double mass = 1.0 / inv_mass[a];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int64_t i = 3 * a + d;
                    const double v = vel[i] - vc[d];
                    vel[i] = v;
                    k2[0] += mass * v * v;
                }
            }
            if (ke) {
                block_sum8(k2, red);
                if (threadIdx.x == 0) ke[m] = 0.5 * k2[0];
            }
        } else if (ke && threadIdx.x == 0) {
            ke[m] = 0.5 * acc[4];
        }
    }
}

int md_vec_open(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT, uint64_t seed,
                int32_t fix_com, const int64_t* mol_ptr, int32_t n_mol, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    MLFF_LAUNCH_PDL("vec_open", vec_open_kernel, std::min(std::max(n_mol, 1), 152 * 8), VEC_NT, 0, st, s->pos,
                    s->vel, s->inv_mass, s->forces, dt, friction, kT, seed, s->step_counter, mol_ptr, n_mol, fix_com,
                    ws_ptr<double>(ws, L.md_noise), ws_ptr<float>(ws, L.md_pos32), ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

int md_vec_close(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT,
                 int32_t fix_com, const int64_t* mol_ptr, int32_t n_mol, double* kinetic, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    MLFF_LAUNCH_PDL("vec_close", vec_close_kernel, std::min(std::max(n_mol, 1), 152 * 8), VEC_NT, 0, st, s->vel,
                    s->inv_mass, s->forces, dt, friction, kT, ws_ptr<double>(ws, L.md_noise), mol_ptr, n_mol,
                    fix_com, kinetic, s->step_counter, ws_ptr<Status>(ws, L.status));
    return MLFF_OK;
}

// kinetic energy 1/2 m v^2 per structure (fixed-order tree), from the
// velocities or, when ke_atom is given, from per-atom terms the force
// kernel's fused Verlet update wrote
__global__ void kinetic_kernel(const double* __restrict__ vel, const double* __restrict__ inv_mass,
                               const double* __restrict__ ke_atom, const int64_t* __restrict__ mol_ptr, int32_t n_mol,
                               double* __restrict__ ke) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[256];
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        double s = 0.0;
        for (int64_t a = mol_ptr[m] + threadIdx.x; a < mol_ptr[m + 1]; a += blockDim.x)
            s += ke_atom ? ke_atom[a] : kinetic_term(vel[3 * a], vel[3 * a + 1], vel[3 * a + 2], inv_mass[a]);
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
        MLFF_LAUNCH_PDL("kinetic", kinetic_kernel, std::min(std::max(n_mol, 1), 152 * 8), 256, 0, st, s->vel,
                        s->inv_mass, (const double*)nullptr, mol_ptr, n_mol, s->kinetic);
    }
    return MLFF_OK;
}

// Per-structure kinetic energy from the per-atom terms of the force kernel's
// fused Verlet update (no separate kick).
int md_kinetic_from_atoms(const double* ke_atom, mlff_md_state* s, const int64_t* mol_ptr, int32_t n_mol,
                          cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    MLFF_LAUNCH_PDL("kinetic", kinetic_kernel, std::min(std::max(n_mol, 1), 152 * 8), 256, 0, st,
                    (const double*)s->vel, (const double*)s->inv_mass, ke_atom, mol_ptr, n_mol, s->kinetic);
    return MLFF_OK;
}


// ----------------------------------------------------------------- NPT
// Isothermal-isobaric dynamics with the equations of motion of ASE's NPT
// (Nose-Hoover thermostat and Parrinello-Rahman barostat, Melchionna,
// Ciccotti and Holian, Mol. Phys. 78, 533 (1993)), for orthorhombic boxes
// (diagonal strain rate eta), per structure:
//   dr/dt = v + eta (r - R0)        R0 = centre of mass
//   dv/dt = F/m - (zeta + eta) v
//   dzeta/dt = (2 K / (g kT) - 1) / ttime^2           g = 3 n
//   deta_a/dt = V / pfactor (P_aa - P_ext),  P_aa = (sum m v_a^2 - W_aa) / V
//   dL_a/dt = eta_a L_a
// with W = dE/d(strain), the virial the force call returns.  These conserve
//   H = E + K + P_ext V + g kT (ttime^2 zeta^2 / 2 + xi) + pfactor |eta|^2 / 2,
// dxi/dt = zeta.  Time-reversible splitting per step: half step of zeta,
// eta (and xi); v scaled by exp(-(zeta + eta) dt/2) and half-kicked; the
// drift solved exactly for constant v (positions relative to the moving
// centre of mass scale by exp(eta dt), boxes too); forces and virial; half
// kick, scaling and half step of the extended variables with the new
// kinetic tensor and virial.  ttime = 0 switches the thermostat off,
// pfactor = 0 the barostat.  One block per structure, fixed-order sums.
constexpr int NPT_NT = 256;

struct NptArgs {
    double* pos;
    double* vel;
    const double* inv_mass;
    const float* F;
    const double* virial;    // [B][9]
    double* box;             // [B][3] float64 master copy
    float* box32;            // [B][3] what the force call reads
    double* zeta;            // [B]
    double* eta;             // [B][3]
    double* xi;              // [B]
    double* kinetic;         // [B] or NULL
    const int64_t* mol_ptr;
    int32_t n_mol;
    double dt, kT, ttime, pfactor, pext;
    float* pos32;
    Status* st;
};

__device__ double npt_block_sum(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = NPT_NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// kinetic tensor diagonal sum m v_a^2 of structure m's atoms [a0, a1)
__device__ void npt_kinetic_diag(const NptArgs& a, int64_t a0, int64_t a1, double* red, double K[3]) {
    double k[3] = {0.0, 0.0, 0.0};
    for (int64_t i = a0 + threadIdx.x; i < a1; i += NPT_NT) {
        const double m = 1.0 / a.inv_mass[i];
#pragma unroll
        for (int d = 0; d < 3; ++d) k[d] += m * a.vel[3 * i + d] * a.vel[3 * i + d];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) K[d] = npt_block_sum(k[d], red);
}

// half step of zeta and eta from the kinetic tensor K and virial W (thread 0)
__device__ void npt_half_extended(const NptArgs& a, int m, const double K[3], double n_atoms) {
    const double* L = a.box + 3 * m;
    const double V = L[0] * L[1] * L[2];
    const double h = 0.5 * a.dt;
    if (a.ttime > 0.0) {
        const double g = 3.0 * n_atoms;
        a.zeta[m] += h * ((K[0] + K[1] + K[2]) / (g * a.kT) - 1.0) / (a.ttime * a.ttime);
    }
    if (a.pfactor > 0.0) {
        const double* W = a.virial + 9 * m;
#pragma unroll
        for (int d = 0; d < 3; ++d) a.eta[3 * m + d] += h * (V / a.pfactor) * ((K[d] - W[4 * d]) / V - a.pext);
    }
}

// exp(x) - 1 over x, 1 at x = 0
__device__ __forceinline__ double expm1_over(double x) { return fabs(x) < 1e-12 ? 1.0 + 0.5 * x : expm1(x) / x; }

// extended half step, thermostat/barostat scaling, half kick, exact drift
__global__ void __launch_bounds__(NPT_NT) npt_open_kernel(NptArgs a) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[NPT_NT];
    __shared__ double sh[8];
    if (a.st->code != 0) return;
    for (int m = blockIdx.x; m < a.n_mol; m += gridDim.x) {
        const int64_t a0 = a.mol_ptr[m], a1 = a.mol_ptr[m + 1];
        double K[3];
        npt_kinetic_diag(a, a0, a1, red, K);
        if (threadIdx.x == 0) {
            npt_half_extended(a, m, K, (double)(a1 - a0));
            a.xi[m] += 0.5 * a.dt * a.zeta[m];
            sh[0] = a.zeta[m];
            sh[1] = a.eta[3 * m];
            sh[2] = a.eta[3 * m + 1];
            sh[3] = a.eta[3 * m + 2];
        }
        __syncthreads();
        const double zeta = sh[0], eta[3] = {sh[1], sh[2], sh[3]};
        double scale[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) scale[d] = exp(-0.5 * a.dt * (zeta + eta[d]));
        // scaled, half-kicked velocities; mass-weighted sums of positions and velocities
        double s[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int64_t i = a0 + threadIdx.x; i < a1; i += NPT_NT) {
            const double m_i = 1.0 / a.inv_mass[i];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double v = a.vel[3 * i + d] * scale[d] + 0.5 * a.dt * (double)a.F[3 * i + d] * a.inv_mass[i];
                a.vel[3 * i + d] = v;
                s[d] += m_i * a.pos[3 * i + d];
                s[3 + d] += m_i * v;
            }
            s[6] += m_i;
        }
        double t[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) t[k] = npt_block_sum(s[k], red);
        const double R0[3] = {t[0] / t[6], t[1] / t[6], t[2] / t[6]};
        const double vc[3] = {t[3] / t[6], t[4] / t[6], t[5] / t[6]};
        double ex[3], ph[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            ex[d] = exp(eta[d] * a.dt);
            ph[d] = a.dt * expm1_over(eta[d] * a.dt);
        }
        // r - R0(t) scales by exp(eta dt) while moving with v - v_com; R0 moves with v_com
        for (int64_t i = a0 + threadIdx.x; i < a1; i += NPT_NT) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double r = R0[d] + vc[d] * a.dt + ex[d] * (a.pos[3 * i + d] - R0[d]) +
                                 (a.vel[3 * i + d] - vc[d]) * ph[d];
                a.pos[3 * i + d] = r;
                a.pos32[3 * i + d] = (float)r;
            }
        }
        if (threadIdx.x < 3) {
            const double Lb = a.box[3 * m + threadIdx.x] * ex[threadIdx.x];
            a.box[3 * m + threadIdx.x] = Lb;
            a.box32[3 * m + threadIdx.x] = (float)Lb;
            // a box that changes by more than 20 % in one step (or stops being finite) means the
            // barostat has run away (pfactor far too small for the system): stop with an error
            if (!(fabs(eta[threadIdx.x] * a.dt) < 0.2) || !isfinite(Lb)) set_status(a.st, MLFF_ERR_BOX, m);
        }
        __syncthreads();
    }
}

// half kick, scaling, extended half step with the new virial; kinetic energy
__global__ void __launch_bounds__(NPT_NT) npt_close_kernel(NptArgs a) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[NPT_NT];
    if (a.st->code != 0) return;
    for (int m = blockIdx.x; m < a.n_mol; m += gridDim.x) {
        const int64_t a0 = a.mol_ptr[m], a1 = a.mol_ptr[m + 1];
        const double zeta = a.zeta[m];
        double scale[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) scale[d] = exp(-0.5 * a.dt * (zeta + a.eta[3 * m + d]));
        for (int64_t i = a0 + threadIdx.x; i < a1; i += NPT_NT) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
                a.vel[3 * i + d] = (a.vel[3 * i + d] + 0.5 * a.dt * (double)a.F[3 * i + d] * a.inv_mass[i]) * scale[d];
        }
        __syncthreads();
        double K[3];
        npt_kinetic_diag(a, a0, a1, red, K);
        if (threadIdx.x == 0) {
            a.xi[m] += 0.5 * a.dt * a.zeta[m];
            npt_half_extended(a, m, K, (double)(a1 - a0));
            if (a.kinetic) a.kinetic[m] = 0.5 * (K[0] + K[1] + K[2]);
        }
        __syncthreads();
    }
}

static NptArgs npt_args(const WsLayout& L, void* ws, const mlff_md_state* s, const mlff_npt_state* n, double dt,
                        double kT, double ttime, double pfactor, double pext, const int64_t* mol_ptr, int32_t n_mol,
                        double* kinetic) {
    NptArgs a;
    a.pos = s->pos; a.vel = s->vel; a.inv_mass = s->inv_mass; a.F = s->forces;
    a.virial = n->virial; a.box = n->box; a.box32 = n->box32; a.zeta = n->zeta; a.eta = n->eta; a.xi = n->xi;
    a.kinetic = kinetic; a.mol_ptr = mol_ptr; a.n_mol = n_mol;
    a.dt = dt; a.kT = kT; a.ttime = ttime; a.pfactor = pfactor; a.pext = pext;
    a.pos32 = ws_ptr<float>(ws, L.md_pos32);
    a.st = ws_ptr<Status>(ws, L.status);
    return a;
}

int md_npt_open(const WsLayout& L, void* ws, const mlff_md_state* s, const mlff_npt_state* n, double dt, double kT,
                double ttime, double pfactor, double pext, const int64_t* mol_ptr, int32_t n_mol, cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    NptArgs a = npt_args(L, ws, s, n, dt, kT, ttime, pfactor, pext, mol_ptr, n_mol, nullptr);
    MLFF_LAUNCH_PDL("npt_open", npt_open_kernel, std::min(std::max(n_mol, 1), 152 * 8), NPT_NT, 0, st, a);
    return MLFF_OK;
}

int md_npt_close(const WsLayout& L, void* ws, const mlff_md_state* s, const mlff_npt_state* n, double dt, double kT,
                 double ttime, double pfactor, double pext, const int64_t* mol_ptr, int32_t n_mol, double* kinetic,
                 cudaStream_t st) {
    ProfScope prof(PK_MD, st);
    NptArgs a = npt_args(L, ws, s, n, dt, kT, ttime, pfactor, pext, mol_ptr, n_mol, kinetic);
    MLFF_LAUNCH_PDL("npt_close", npt_close_kernel, std::min(std::max(n_mol, 1), 152 * 8), NPT_NT, 0, st, a);
    return MLFF_OK;
}

// --------------------------------------------------- energy statistics
// Per-replica NVE statistics of an energy trace, the quantities of the
// reference's energy-conservation report (testing/energy_metrics.py:48-357):
// drift, fluctuations, conservation ratio, kinetic/potential stability,
// linear-fit drift rate, temperature.  One block per replica, every sum a
// fixed-order strided accumulation followed by a fixed tree: the result
// does not depend on the launch and is the same on every run.
constexpr int ES_NT = 256;

__device__ double es_block_sum(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = ES_NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(ES_NT) energy_stats_kernel(const double* __restrict__ epot,
                                                            const double* __restrict__ ekin, int32_t n, int32_t B,
                                                            const int64_t* __restrict__ mol_ptr, double dt_ps,
                                                            double* __restrict__ out) {
    pdl_wait();
    pdl_trigger();
    __shared__ double red[ES_NT];
    for (int b = blockIdx.x; b < B; b += gridDim.x) {
        auto et = [&](int i) { return epot[(int64_t)i * B + b] + ekin[(int64_t)i * B + b]; };
        double se = 0.0, sk = 0.0, sp = 0.0;
        for (int i = threadIdx.x; i < n; i += ES_NT) {
            se += et(i);
            sk += ekin[(int64_t)i * B + b];
            sp += epot[(int64_t)i * B + b];
        }
        const double me = es_block_sum(se, red) / n, mk = es_block_sum(sk, red) / n, mp = es_block_sum(sp, red) / n;
        const double tm = 0.5 * (n - 1) * dt_ps;   // mean sample time
        double see = 0.0, sad = 0.0, skk = 0.0, spp = 0.0, skp = 0.0, stt = 0.0, ste = 0.0, smax = 0.0;
        double emin = 1e300, emax = -1e300;
        const double e0 = et(0);
        for (int i = threadIdx.x; i < n; i += ES_NT) {
            const double e = et(i), de = e - me;
            const double dk = ekin[(int64_t)i * B + b] - mk, dp = epot[(int64_t)i * B + b] - mp;
            const double dt = i * dt_ps - tm;
            see += de * de;
            sad += fabs(de);
            skk += dk * dk;
            spp += dp * dp;
            skp += dk * dp;
            stt += dt * dt;
            ste += dt * de;
            smax = fmax(smax, fabs(e - e0));
            emin = fmin(emin, e);
            emax = fmax(emax, e);
        }
        see = es_block_sum(see, red);
        sad = es_block_sum(sad, red);
        skk = es_block_sum(skk, red);
        spp = es_block_sum(spp, red);
        skp = es_block_sum(skp, red);
        stt = es_block_sum(stt, red);
        ste = es_block_sum(ste, red);
        // maxima and minima by the same fixed tree
        red[threadIdx.x] = smax;
        __syncthreads();
        for (int o = ES_NT / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
            __syncthreads();
        }
        smax = red[0];
        __syncthreads();
        red[threadIdx.x] = emax;
        __syncthreads();
        for (int o = ES_NT / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
            __syncthreads();
        }
        emax = red[0];
        __syncthreads();
        red[threadIdx.x] = emin;
        __syncthreads();
        for (int o = ES_NT / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + o]);
            __syncthreads();
        }
        emin = red[0];
        __syncthreads();
        // residual sum of squares of the linear fit E = a + r t
        const double rate = stt > 0.0 ? ste / stt : 0.0;
        double srr = 0.0;
        for (int i = threadIdx.x; i < n; i += ES_NT) {
            const double res = et(i) - me - rate * (i * dt_ps - tm);
            srr += res * res;
        }
        srr = es_block_sum(srr, red);
        if (threadIdx.x == 0) {
            const double ef = et(n - 1);
            const double sd = sqrt(see / n), sdk = sqrt(skk / n), sdp = sqrt(spp / n);
            const double na = mol_ptr ? (double)(mol_ptr[b + 1] - mol_ptr[b]) : 0.0;
            const double kTconv = na > 0 ? 2.0 / (3.0 * na * 8.617333262e-5) : 0.0;   // K per eV of kinetic energy
            double* o = out + (int64_t)b * 20;
            o[0] = e0;
            o[1] = ef;
            o[2] = fabs(e0) >= 1e-10 ? 100.0 * (ef - e0) / fabs(e0) : 0.0;   // drift %
            o[3] = fabs(e0) >= 1e-10 ? 100.0 * smax / fabs(e0) : 0.0;        // max deviation %
            o[4] = me;
            o[5] = sd;                                                        // std
            o[6] = emax - emin;                                               // range
            o[7] = sad / n;                                                   // mean absolute deviation
            o[8] = fabs(me) >= 1e-10 ? fmax(0.0, 1.0 - sd / fabs(me)) : 1.0;  // conservation ratio
            o[9] = mk;
            o[10] = sdk;
            o[11] = mp;
            o[12] = sdp;
            o[13] = (sdk > 0.0 && sdp > 0.0) ? (skp / n) / (sdk * sdp) : 0.0;  // KE-PE correlation
            o[14] = fabs(mp) > 1e-10 ? mk / fabs(mp) : 0.0;                   // partition ratio
            o[15] = rate;                                                     // drift rate (eV/ps)
            o[16] = see > 1e-10 ? 1.0 - srr / see : 1.0;                      // R^2
            const double st = sqrt(stt / n);
            o[17] = st > 1e-10 ? sqrt(srr / n) / (st * sqrt((double)n)) : 0.0;   // drift-rate standard error
            o[18] = mk * kTconv;                                              // mean temperature (K)
            o[19] = sdk * kTconv;                                             // temperature std (K)
        }
        __syncthreads();
    }
}

int md_energy_stats(const double* epot, const double* ekin, int32_t n, int32_t B, const int64_t* mol_ptr,
                    double dt_ps, double* out, cudaStream_t st) {
    MLFF_LAUNCH_PDL("energy_stats", energy_stats_kernel, std::min(std::max(B, 1), 152 * 8), ES_NT, 0, st, epot,
                    ekin, n, B, mol_ptr, dt_ps, out);
    return MLFF_OK;
}
}  // namespace mlff
