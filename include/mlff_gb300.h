/*
 * mlff_gb300 -- C ABI of the GB300 (sm_103a) energy/force/MD library for a
 * PaiNN-style StudentForceField.
 *
 * The reference (MLFF-Distiller) is pure Python/PyTorch: it has no native
 * FFI.  Each entry point below replaces one Python call on the hot path; the
 * comment names that call (file:line inside the reference project).  The
 * Python package mlff_gb300 binds these with ctypes (mlff_gb300/_lib.py).
 *
 * Conventions
 *  - Every pointer to array data is a DEVICE pointer owned by the caller
 *    (e.g. a torch tensor's data_ptr()) unless the comment says "host".
 *  - The library never allocates device memory: the caller provides the
 *    packed-weight blob and one workspace, sized by the *_size() queries.
 *  - Every call is asynchronous on the given stream (cudaStream_t; NULL =
 *    legacy default stream) and returns an int status; errors found on the
 *    device (edge capacity, bad box) are written to a status word inside the
 *    workspace and read back with mlff_read_status().  Nothing traps, exits
 *    or throws across the ABI.
 *  - Threading: one host thread per workspace at a time (the reference's
 *    calculator is not re-entrant either).
 */
#ifndef MLFF_GB300_H
#define MLFF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *mlff_stream_t; /* same type as cudaStream_t */

/* status codes */
#define MLFF_OK 0
#define MLFF_ERR_INVALID 1     /* bad argument (host-side check) */
#define MLFF_ERR_CAPACITY 2    /* more edges than edge_capacity; read n_edges */
#define MLFF_ERR_CUDA 3        /* CUDA runtime error; see mlff_last_error_string */
#define MLFF_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define MLFF_ERR_UNSUPPORTED 5 /* model shape outside what the kernels implement */
#define MLFF_ERR_BOX 6         /* periodic box edge < 2*cutoff or non-finite */
#define MLFF_ERR_ROW 7         /* one atom has more neighbours than a row holds */
#define MLFF_ERR_WORKSPACE 8   /* workspace or packed blob smaller than required */

/* evaluation paths */
#define MLFF_PATH_PLAIN_FP32 0    /* per-op FP32 kernels (the plain drop-in) */
#define MLFF_PATH_TUNED_TC 1      /* fused edge kernels, tcgen05, split-FP16 operands */
#define MLFF_PATH_TUNED_FP32 2    /* fused edge kernels, FP32 CUDA cores */
#define MLFF_PATH_TRAIN 3         /* plain FP32 path plus parameter gradients (workspace sizing) */
#define MLFF_PATH_TRAIN_FORCES 4  /* plus the force-loss term (workspace sizing; runs as path 0) */

#define MLFF_MAX_LAYERS 8

/* Model shape: StudentForceField(hidden_dim, num_interactions, num_rbf,
 * cutoff, max_z) -- src/mlff_distiller/models/student_model.py:566-575. */
typedef struct {
    int32_t hidden;    /* hidden_dim; the kernels implement 128 */
    int32_t n_rbf;     /* num_rbf, 1..32 */
    int32_t n_layers;  /* num_interactions, 1..8 */
    int32_t n_species; /* max_z + 1 */
    float cutoff;      /* Angstrom */
} mlff_dims;

/* Float32 parameters, one device pointer per state_dict tensor, in the
 * reference's shapes (student_model.py:566-628; keys in the comments). */
typedef struct {
    const float *embedding;   /* embedding.weight [S,H] */
    const float *rbf_centers; /* rbf.centers [R] */
    const float *rbf_widths;  /* rbf.widths [R] */
    const float *filter_w1[MLFF_MAX_LAYERS]; /* interactions.l.message.rbf_to_scalar.0.weight [H,R] */
    const float *filter_b1[MLFF_MAX_LAYERS]; /* ...rbf_to_scalar.0.bias [H] */
    const float *filter_w2[MLFF_MAX_LAYERS]; /* ...rbf_to_scalar.2.weight [3H,H] */
    const float *filter_b2[MLFF_MAX_LAYERS]; /* ...rbf_to_scalar.2.bias [3H] */
    const float *mixing[MLFF_MAX_LAYERS];    /* interactions.l.update.mixing_matrix [3,3] */
    const float *update_w1[MLFF_MAX_LAYERS]; /* ...update.update_mlp.0.weight [H,2H] */
    const float *update_b1[MLFF_MAX_LAYERS]; /* ...update_mlp.0.bias [H] */
    const float *update_w2[MLFF_MAX_LAYERS]; /* ...update_mlp.2.weight [3H,H] */
    const float *update_b2[MLFF_MAX_LAYERS]; /* ...update_mlp.2.bias [3H] */
    const float *head_w1, *head_b1; /* energy_head.0 [H/2,H], [H/2] */
    const float *head_w2, *head_b2; /* energy_head.2 [H/4,H/2], [H/4] */
    const float *head_w3, *head_b3; /* energy_head.4 [1,H/4], [1] */
} mlff_params;

/* Float32 parameter gradients, one device pointer per state_dict tensor
 * (same order and shapes as mlff_params); a NULL entry is skipped. */
typedef struct {
    float *embedding;
    float *rbf_centers; /* not trained (buffers of the reference); left untouched */
    float *rbf_widths;
    float *filter_w1[MLFF_MAX_LAYERS];
    float *filter_b1[MLFF_MAX_LAYERS];
    float *filter_w2[MLFF_MAX_LAYERS];
    float *filter_b2[MLFF_MAX_LAYERS];
    float *mixing[MLFF_MAX_LAYERS];
    float *update_w1[MLFF_MAX_LAYERS];
    float *update_b1[MLFF_MAX_LAYERS];
    float *update_w2[MLFF_MAX_LAYERS];
    float *update_b2[MLFF_MAX_LAYERS];
    float *head_w1, *head_b1;
    float *head_w2, *head_b2;
    float *head_w3, *head_b3;
} mlff_grads;

/* A ragged batch of structures (ase_calculator.py:647-706 _prepare_batch):
 * structure m owns atoms mol_ptr[m] .. mol_ptr[m+1]-1.  Edges never cross
 * structures (student_model.py:94-95).  A periodic structure is an
 * orthorhombic box, periodic on all three axes, edge >= 2*cutoff. */
typedef struct {
    int32_t n_atoms;
    int32_t n_mol;
    const float *pos;       /* [N,3] float32, Angstrom */
    const int64_t *Z;       /* [N] atomic numbers (0..n_species-1) */
    const int64_t *mol_ptr; /* [B+1] */
    const float *box;       /* [B,3] box edge lengths, or NULL (all open) */
    const uint8_t *pbc;     /* [B] 1 = periodic, or NULL (all open) */
} mlff_system;

typedef struct {
    double *energy;      /* [B] per-structure energy (eV), required */
    float *forces;       /* [N,3] -dE/dpos (eV/A), or NULL for energy only */
    double *virial;      /* [B,3,3] dE/d(strain), or NULL */
    float *atom_energy;  /* [N] per-atom energies, or NULL */
} mlff_outputs;

/* Library version, major*10000 + minor*100 + patch. */
int mlff_version(void);

/* Last host-side error message of the calling thread ("" if none). */
const char *mlff_last_error_string(void);

/* Bytes of the packed weight blob for these dims. */
size_t mlff_packed_weights_size(const mlff_dims *dims);

/* Pack float32 state_dict tensors into the kernels' layouts (transposes,
 * zero padding, split-BF16 hi/lo tiles).  Replaces nothing in the reference
 * (its nn.Linear layers read the state_dict directly); call once after
 * StudentForceField.load / load_state_dict (student_model.py:1101-1176). */
int mlff_pack_weights(const mlff_dims *dims, const mlff_params *params, void *packed,
                      size_t packed_bytes, mlff_stream_t stream);

/* Workspace bytes for a batch of n_atoms atoms in n_mol structures with
 * room for edge_capacity directed edges, for the given path. */
size_t mlff_workspace_size(const mlff_dims *dims, int32_t n_atoms, int32_t n_mol,
                           int64_t edge_capacity, int32_t path);

/* Radius graph: replaces radius_graph / radius_graph_native
 * (student_model.py:63-109, 165-191) plus a minimum-image rule for periodic
 * boxes.  Builds a receiver-sorted CSR in the workspace whose rows and
 * columns, read as [row; col], equal the reference's edge_index bit for
 * bit.  On overflow the status word holds MLFF_ERR_CAPACITY and the number
 * of edges needed. */
int mlff_build_neighbors(const mlff_dims *dims, const mlff_system *sys, int64_t edge_capacity,
                         void *workspace, size_t workspace_bytes, mlff_stream_t stream);

/* Copy the CSR built by the last neighbour build out of the workspace:
 * row_ptr [N+1] int32 and col [E] int32 (device), E = row_ptr[N]. */
int mlff_copy_neighbors(const void *workspace, int32_t n_atoms, int32_t n_mol,
                        int64_t edge_capacity, int32_t path, int32_t *row_ptr, int32_t *col,
                        mlff_stream_t stream);

/* Energies, forces (and virial): replaces StudentForceField.forward +
 * torch.autograd.grad in predict_energy_and_forces (student_model.py:634-795)
 * and the batched path of StudentForceFieldCalculator._batch_forward
 * (ase_calculator.py:708-770).  Runs the neighbour build first. */
int mlff_energy_forces(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                       int64_t edge_capacity, int32_t path, const mlff_outputs *out,
                       void *workspace, size_t workspace_bytes, mlff_stream_t stream);

/* Synchronise the stream and read the device status word: code (MLFF_OK or
 * a device-side MLFF_ERR_*), edges found by the last neighbour build, and
 * the first offending atom or structure (or -1).  Host pointers. */
int mlff_read_status(const void *workspace, int32_t *code, int64_t *n_edges, int32_t *where,
                     mlff_stream_t stream);

/* Clear the device status word (asynchronous). */
int mlff_clear_status(void *workspace, mlff_stream_t stream);

/* Velocity-Verlet NVE steps in float64 state: replaces ASE VelocityVerlet
 * driven by NVEMDHarness.run_simulation (testing/nve_harness.py:173-261).
 * Per step: v += dt/2 * F/m; r += dt * v; F = F(r); v += dt/2 * F/m.
 * pos/vel are float64 [N,3] (Angstrom, Angstrom per ASE time unit), forces
 * float32 [N,3] hold F(r) on entry and on exit, inv_mass float64 [N]
 * (1/amu).  energy receives the potential energy per structure after the
 * last step, kinetic (optional) the kinetic energy.  energy_trace and
 * kinetic_trace (optional, [n_steps][n_mol]) receive both after every step
 * -- the per-step record NVEMDHarness._collect_data keeps on the host
 * (nve_harness.py:239-265).  No host synchronisation, so a fixed number of
 * steps can be captured in a CUDA graph once the edge capacity is known to
 * suffice. */
typedef struct {
    double *pos;
    double *vel;
    const double *inv_mass;
    float *forces;
    double *energy;
    double *kinetic;
    double *energy_trace;
    double *kinetic_trace;
    int64_t *step_counter; /* device int64: steps taken; keys the Langevin draws (required
                              by mlff_langevin_steps, optional here); +1 per step */
} mlff_md_state;

int mlff_verlet_steps(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                      int64_t edge_capacity, int32_t path, mlff_md_state *state, double dt,
                      int32_t n_steps, void *workspace, size_t workspace_bytes,
                      mlff_stream_t stream);

/* Langevin (NVT) steps in float64 state, BAOAB splitting (Leimkuhler and
 * Matthews, J. Chem. Phys. 138, 174102 (2013)): per step
 *   v += dt/2 F/m; r += dt/2 v; v = c1 v + sqrt((1 - c1^2) kT/m) xi;
 *   r += dt/2 v; F = F(r); v += dt/2 F/m,   c1 = exp(-friction dt),
 * with xi standard normals drawn by Box-Muller from Philox4x32-10 (Salmon
 * et al., SC'11) keyed by (seed, *step_counter, atom) -- reproducible and
 * independent of launch shape; the counter lives in device memory so a
 * captured graph draws new numbers on every replay.  Replaces ASE's
 * Langevin in the reference's NVT protocol (benchmarks/md_trajectory.py:
 * 400-413).  Units as mlff_verlet_steps: dt and 1/friction in ASE time units
 * (Angstrom sqrt(amu/eV)), kT in eV.  Same state, traces and workspace as
 * mlff_verlet_steps; state->step_counter is required. */
int mlff_langevin_steps(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                        int64_t edge_capacity, int32_t path, mlff_md_state *state, double dt,
                        double friction, double kT, uint64_t seed, int32_t n_steps, void *workspace,
                        size_t workspace_bytes, mlff_stream_t stream);

/* Langevin NVT with the scheme of ASE's Langevin, the reference's NVT
 * protocol (src/mlff_distiller/benchmarks/md_trajectory.py:407-413, ASE
 * Langevin with friction 0.01 and its default fixcm=True): the propagator
 * of Vanden-Eijnden and Ciccotti (Chem. Phys. Lett. 429, 310 (2006),
 * Eq. 23), restated in the library's own kernels.  Same state and
 * arguments as mlff_langevin_steps (friction in inverse ASE time units, kT
 * in eV); fix_com = 1 keeps each structure's centre of mass in place and
 * removes its centre-of-mass velocity every step, as ASE does by default.
 * Six normals per atom and step (Philox4x32-10 keyed by seed and (step,
 * atom, 1 or 2), Box-Muller).  ASE draws from numpy's generator instead,
 * so trajectories agree with ASE's in distribution, not sample by sample.
 * Graph-capturable like mlff_langevin_steps. */
int mlff_langevin_ase_steps(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                            int64_t edge_capacity, int32_t path, mlff_md_state *state, double dt,
                            double friction, double kT, uint64_t seed, int32_t fix_com, int32_t n_steps,
                            void *workspace, size_t workspace_bytes, mlff_stream_t stream);

/* NPT state beyond mlff_md_state, per structure (all device memory):
 * box float64 [B,3] edge lengths and box32 float32 [B,3] (the copy the
 * force call reads; both updated every step), zeta [B] thermostat rate,
 * eta [B,3] diagonal barostat strain rate (1 / ASE time unit), xi [B] the
 * time integral of zeta (for the conserved quantity), virial [B,3,3]
 * dE/d(strain) at the current positions (in and out, like forces). */
typedef struct {
    double *box;
    float *box32;
    double *zeta;
    double *eta;
    double *xi;
    double *virial;
} mlff_npt_state;

/* NPT steps (isothermal-isobaric) with the equations of motion of ASE's NPT
 * (Nose-Hoover thermostat + Parrinello-Rahman barostat, Melchionna et al.,
 * Mol. Phys. 78, 533 (1993)) that the reference's NPT protocol runs
 * (benchmarks/md_trajectory.py:415-424: ttime 25 fs, pfactor 75 fs^2,
 * externalstress 0), for orthorhombic periodic boxes (diagonal strain
 * rate):
 *   dr/dt = v + eta (r - R_com),  dv/dt = F/m - (zeta + eta) v,
 *   dzeta/dt = (2 K / (3 n kT) - 1) / ttime^2,
 *   deta/dt = V / pfactor (diag(sum m v v - W) / V - pressure),
 *   dL/dt = eta L,
 * integrated by a time-reversible splitting (half step of zeta and eta,
 * velocity scaling and half kick, exact drift of positions and box, force
 * and virial, half kick and scaling, half step of zeta and eta).  Conserved:
 *   E + K + pressure V + 3 n kT (ttime^2 zeta^2 / 2 + xi) + pfactor |eta|^2 / 2.
 * ttime = 0 turns the thermostat off, pfactor = 0 the barostat.  Units as
 * mlff_verlet_steps (ttime in ASE time units, pfactor in eV (ASE time)^2 /
 * A^3 -- ASE's pfactor -- pressure in eV/A^3, kT in eV).  sys->pbc must mark
 * every structure periodic; the force call reads npt->box32 (sys->box is
 * ignored).  Traces, workspace and status as mlff_verlet_steps.  Parity with
 * ASE's own discretisation is not claimed (ASE is not vendored). */
int mlff_npt_steps(const mlff_dims *dims, const void *packed, const mlff_system *sys, int64_t edge_capacity,
                   int32_t path, mlff_md_state *state, mlff_npt_state *npt, double dt, double kT, double ttime,
                   double pfactor, double pressure, int32_t n_steps, void *workspace, size_t workspace_bytes,
                   mlff_stream_t stream);

/* Per-replica energy-conservation statistics of an MD energy trace, the
 * report of testing/energy_metrics.py:48-357 (compute_energy_drift,
 * compute_energy_conservation_ratio, compute_energy_fluctuations,
 * compute_kinetic_potential_stability, compute_time_resolved_drift with a
 * linear fit) for every replica at once, on the device.  epot and ekin are
 * [n_samples][n_mol] (eV, e.g. the traces of mlff_verlet_steps with the
 * initial energies prepended), samples dt_ps apart; mol_ptr (optional,
 * [n_mol + 1]) gives atom counts for the temperature.  out [n_mol][20]:
 *  0 E_0, 1 E_final, 2 drift % (relative), 3 max deviation %, 4 mean E,
 *  5 std E, 6 range E, 7 mean |E - mean|, 8 conservation ratio,
 *  9 mean KE, 10 std KE, 11 mean PE, 12 std PE, 13 KE-PE correlation,
 *  14 <KE>/|<PE>|, 15 drift rate eV/ps (linear fit), 16 R^2 of the fit,
 *  17 standard error of the rate, 18 mean T (K), 19 std T (K).
 * Fixed-order reductions: identical results on every run. */
#define MLFF_ENERGY_STATS 20
int mlff_md_energy_stats(const double *epot, const double *ekin, int32_t n_samples, int32_t n_mol,
                         const int64_t *mol_ptr, double dt_ps, double *out, mlff_stream_t stream);

/* Parameter gradients for training: grads <- sum_b w_b dE_b/dtheta for
 * every state_dict tensor, with w (device, double [B]) the derivative of
 * the loss with respect to each structure's energy (the energy term of
 * ForceFieldLoss, training/losses.py:106-246, e.g. w_b = 2 (E_b - E_ref_b)
 * / B for a mean-squared energy error).  Replaces the parameter part of
 * loss.backward() in Trainer.train_epoch (training/trainer.py:288-393) for
 * the energy loss.  Runs the plain FP32 path forward (energies into
 * out->energy) and its hand-written reverse pass with the weight-gradient
 * reductions added; out->forces (optional) receives -sum_b w_b dE_b/dpos.
 * The plain path sums messages and node adjoints per receiver row in edge
 * order and the weight-gradient reductions in a fixed order, so repeated
 * calls give the same bits.
 * Workspace: mlff_workspace_size(..., MLFF_PATH_TRAIN). */
int mlff_param_grads(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                     int64_t edge_capacity, const double *energy_weights, const mlff_grads *grads,
                     const mlff_outputs *out, void *workspace, size_t workspace_bytes,
                     mlff_stream_t stream);

/* Force and stress terms of the training loss: grads += sum_i G_i .
 * dF_i/dtheta + sum_b S_b : dW_b/dtheta for every non-NULL state_dict
 * gradient, with G = force_weights (device, float [N,3], or NULL) the
 * derivative of the loss with respect to the predicted forces F = -dE/dpos
 * (e.g. G = 2 w_F (F - F_ref) / (3N) for the mean-squared force error of
 * ForceFieldLoss, training/losses.py:154-170, weight w_F = 100 in
 * configs/train_student.yaml) and S = virial_weights (device, double
 * [B,3,3], or NULL) the derivative with respect to the strain derivatives
 * W_b = dE_b/d(strain) that mlff_energy_forces returns as the virial (the
 * stress term, :222-234, enters through stress = sym(W) / volume).  This
 * is the second-order part of loss.backward() when forces were taken with
 * torch.autograd.grad(..., create_graph=True) (predict_energy_and_forces,
 * models/student_model.py:759-795, in training mode).  Computed exactly,
 * in forward mode over the reverse pass: the plain FP32 path runs once on
 * (value, derivative) pairs along the direction (positions moved by -G,
 * every edge vector r of structure b strained by S_b r) and the derivative
 * of grad_theta E is added to the gradients.  Call after
 * mlff_param_grads (which writes the energy term) to get the full loss
 * gradient; the grads structure is the same.  Workspace:
 * mlff_workspace_size(..., MLFF_PATH_TRAIN_FORCES), which also serves
 * mlff_param_grads. */
int mlff_param_grads_forces(const mlff_dims *dims, const void *packed, const mlff_system *sys,
                            int64_t edge_capacity, const float *force_weights, const double *virial_weights,
                            const mlff_grads *grads, void *workspace, size_t workspace_bytes,
                            mlff_stream_t stream);

/* Kernel timing for benchmarks (no counterpart in the reference, whose
 * timers wrap whole Python calls: cuda/benchmark_utils.py:147-194).
 * Between begin and end the library brackets its kernel groups with CUDA
 * events on the launching stream and counts its kernel launches.  end
 * synchronises those events and returns, per kind, the summed milliseconds
 * and the number of launches.  Kinds: 0 neighbours, 1 fused edge forward,
 * 2 fused edge reverse, 3 update forward, 4 update reverse, 5 readout,
 * 6 forces, 7 plain-path GEMMs, 8 plain-path edge ops, 9 other, 10 MD
 * integrator, 11 the per-atom Q rows of the tensor-core reverse edge pass.
 * Do not enable while a stream is being captured. */
#define MLFF_PROFILE_KINDS 12
int mlff_profile_begin(void);
int mlff_profile_end(double *ms_by_kind, int64_t *launches_by_kind, int32_t n_kinds);

/* Autotuning (no counterpart in the reference, whose only GPU kernels fix
 * their block sizes by hand).  Two shapes of the tensor-core path are
 * chosen per size bucket (path, ceil(log2 n_atoms), ceil(log2 n_mol)) and
 * kept in a process-wide cache guarded by a mutex; every call of that
 * bucket then uses them:
 *  - the partition factor f (1, 2 or 4): the edge kernels split the
 *    receivers into 2 x SMs x f partitions;
 *  - the update tile (64 or 32 atoms per CTA tile of the update kernels;
 *    32 spreads a small system over more SMs).
 * Results do not depend on either (each receiver's sums run over its edges
 * in order inside one partition; each atom's update is the same sequence of
 * MMAs), and the workspace size does not either.  mlff_autotune times
 * `repeats` calls of mlff_energy_forces per candidate (same arguments; the
 * outputs are overwritten) with CUDA events on the stream: f = 1, 2, 4 with
 * 64-atom update tiles, then the fastest f with 32-atom tiles (kept when at
 * least 1 % faster); it
 * synchronises the stream, caches the fastest shape and writes its f to
 * *chosen (host) and the milliseconds per call of f = 1, 2, 4 (64-atom
 * tiles) to ms_per_candidate (host double [3], or NULL).  Not for use while
 * the stream is being captured.  Other paths: *chosen = 1, nothing timed.
 * _query reads the factor a call of that size would use, _set pins one
 * (0 removes the entry; the bucket's update tile is kept), _query_shape
 * reads both shapes (f, update_atoms) and _set_shape pins both (f = 0
 * removes the entry), _reset empties the cache.  Untuned buckets use f = 1
 * and 64-atom update tiles. */
int mlff_autotune(const mlff_dims *dims, const void *packed, const mlff_system *sys, int64_t edge_capacity,
                  int32_t path, const mlff_outputs *out, void *workspace, size_t workspace_bytes,
                  mlff_stream_t stream, int32_t repeats, int32_t *chosen, double *ms_per_candidate);
int mlff_autotune_query(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t *factor);
int mlff_autotune_set(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t factor);
int mlff_autotune_query_shape(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t *factor, int32_t *update_atoms);
int mlff_autotune_set_shape(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t factor, int32_t update_atoms);
int mlff_autotune_reset(void);

/* Force-accuracy statistics on the device (testing/force_metrics.py:46-384,
 * whose functions take host arrays): pred and ref are double [n_vectors,3]
 * device arrays; stats (double [MLFF_FORCE_STATS], device) receives
 *   0 n, 1-3 sum of squared component errors (x, y, z), 4-6 sum of absolute
 *   component errors, 7 sum of squared magnitude errors, 8 sum of absolute
 *   magnitude errors, 9 sum of |magnitude error| / |ref| over vectors with
 *   |ref| > 1e-6, 10 their count, 11 count of vectors with both magnitudes
 *   > 1e-6, 12 sum of their cosines, 13-17 sums of p, r, p^2, r^2, p r over
 *   all components, 18 largest absolute component error, 19 unused;
 * per_vector (double [n_vectors,4], device, or NULL): per vector the RMSE
 * and MAE over its components, |magnitude error| and the angle in degrees
 * (NaN where a magnitude is <= 1e-6).  Sums are reduced in a fixed order.
 * workspace: mlff_force_stats_workspace_size() bytes, device. */
#define MLFF_FORCE_STATS 20
size_t mlff_force_stats_workspace_size(void);
int mlff_force_stats(const double *pred, const double *ref, int64_t n_vectors, double *stats,
                     double *per_vector, void *workspace, size_t workspace_bytes, mlff_stream_t stream);

/* Per-module blocks, any hidden width H and number of basis functions R:
 * the reference's PaiNNMessage.forward (src/mlff_distiller/models/
 * student_model.py:324-387) and PaiNNUpdate.forward (:418-470) and their
 * reverse passes, for callers that use the blocks outside StudentForceField
 * (the fused path does not call these).  FP32, float-atomic scatter as
 * index_add_ on a GPU.  Layouts as the reference's tensors: scalar [N,H],
 * vector [N,3,H], edge_index int64 [2,E] (row 0 senders, row 1
 * receivers), edge_rbf [E,R], edge_vector [E,3], weights in nn.Linear's
 * [out,in] layout, mixing [3,3].  Outputs must not alias inputs.  Each call
 * needs a caller-owned workspace of *_workspace_size(..., with_backward)
 * bytes (with_backward = 1 for the *_backward calls, which recompute the
 * forward activations).  status (message calls): int32 [4] device; an
 * out-of-range edge index gives MLFF_ERR_INVALID with the edge's position
 * and the call stops after the residual copies. */
size_t mlff_painn_message_workspace_size(int32_t hidden, int32_t n_rbf, int64_t n_edges, int32_t with_backward);
int mlff_painn_message(int32_t hidden, int32_t n_rbf, int32_t n_atoms, int64_t n_edges, const float *scalar,
                       const float *vector, const int64_t *edge_index, const float *edge_rbf,
                       const float *edge_vector, const float *w1, const float *b1, const float *w2,
                       const float *b2, float *scalar_out, float *vector_out, int32_t *status, void *workspace,
                       size_t workspace_bytes, mlff_stream_t stream);
/* grad_* = d(loss)/d(input or parameter) from grad_scalar_out / grad_vector_out */
int mlff_painn_message_backward(int32_t hidden, int32_t n_rbf, int32_t n_atoms, int64_t n_edges,
                                const float *scalar, const float *vector, const int64_t *edge_index,
                                const float *edge_rbf, const float *edge_vector, const float *w1,
                                const float *b1, const float *w2, const float *b2,
                                const float *grad_scalar_out, const float *grad_vector_out, float *grad_scalar,
                                float *grad_vector, float *grad_rbf, float *grad_edge_vector, float *grad_w1,
                                float *grad_b1, float *grad_w2, float *grad_b2, int32_t *status,
                                void *workspace, size_t workspace_bytes, mlff_stream_t stream);
size_t mlff_painn_update_workspace_size(int32_t hidden, int32_t n_atoms, int32_t with_backward);
int mlff_painn_update(int32_t hidden, int32_t n_atoms, const float *scalar, const float *vector,
                      const float *w1, const float *b1, const float *w2, const float *b2, const float *mixing,
                      float *scalar_out, float *vector_out, void *workspace, size_t workspace_bytes,
                      mlff_stream_t stream);
int mlff_painn_update_backward(int32_t hidden, int32_t n_atoms, const float *scalar, const float *vector,
                               const float *w1, const float *b1, const float *w2, const float *b2,
                               const float *mixing, const float *grad_scalar_out, const float *grad_vector_out,
                               float *grad_scalar, float *grad_vector, float *grad_w1, float *grad_b1,
                               float *grad_w2, float *grad_b2, float *grad_mixing, void *workspace,
                               size_t workspace_bytes, mlff_stream_t stream);

/* Test hook for the bounded device waits (no counterpart in the reference;
 * the timeout path replaces a hang where the reference would block).  While
 * bit 0 (forward) or bit 1 (reverse) of `kernels` is set, every CTA of the
 * tensor-core edge kernels launched afterwards also waits, at its first
 * main-loop wait, on an mbarrier that nothing arrives at, for about 65,000
 * cycles; the wait runs out and the kernel takes the path of a real timeout:
 * MLFF_ERR_TIMEOUT with index 99 in the status word, abort flag raised, its
 * own copies and MMAs drained, tensor memory freed, return.  The kernels
 * that follow see the status and do nothing.  0 (the default) turns it off.
 * Kernel arguments are fixed when a CUDA graph is captured: the hook applies
 * to eager calls and to graphs captured while it is set.  Not for use in
 * production. */
int mlff_debug_stall_test(int32_t kernels);

/* Radius graph that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc or hand over a
 * workspace (hosts that own every allocation, allocation-free regions).
 * Same CSR as mlff_build_neighbors (row_ptr [N+1], col [edge_capacity],
 * caller-owned outputs) plus status [4] int32 (code, edges found, first
 * offending index, edges >> 31), all device pointers.  Scratch lives in one
 * file-scope device array of about 13 MB, so sizes are capped: n_atoms <=
 * 16384, n_mol <= 4096, edge_capacity <= 1048576 (MLFF_ERR_INVALID above
 * that).  The first call on a device looks up the array's address; make it
 * before any stream capture.  Calls share the array: calls that overlap on
 * the GPU race. */
#define MLFF_NOALLOC_MAX_ATOMS 16384
#define MLFF_NOALLOC_MAX_MOLS 4096
#define MLFF_NOALLOC_MAX_EDGES 1048576
int mlff_radius_graph_noalloc(const mlff_system *sys, float cutoff, int64_t edge_capacity,
                              int32_t *row_ptr, int32_t *col, int32_t *status, mlff_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MLFF_GB300_H */
