// extern "C" entry points of libmlff_gb300.so (declared in
// include/mlff_gb300.h), workspace layout and host-side validation.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <atomic>
#include "common.cuh"
#include "workspace.h"

namespace mlff {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    return MLFF_ERR_CUDA;
}

bool pdl_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = std::getenv("MLFF_PDL");
        on = (e && e[0] == '0') ? 0 : 1;
    }
    return on == 1;
}

int num_sms() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 152;
    }
    return sms;
}

int persistent_ctas(int32_t path) {
    // Receiver partitions: the CUDA-core fused kernels run 4 CTAs of 128
    // threads per SM; the tensor-core kernels run one CTA per SM with two
    // partitions each (the reverse kernel's two pipelines take one each,
    // the forward kernel walks both as one receiver range), times the
    // partition factor the autotuner chose for the call's size.
    return path == MLFF_PATH_TUNED_TC ? 2 * num_sms() : num_sms() * 4;
}

// ----------------------------------------------------------- autotuning
// Two shapes of the tensor-core path, chosen per size bucket (path,
// ceil(log2 atoms), ceil(log2 structures)) by mlff_autotune and kept in a
// process-wide cache guarded by a mutex:
//  * the receiver partitions per CTA pipeline of the edge kernels (the
//    partition factor; 1, 2 or 4: more, smaller partitions balance uneven
//    rows better at the cost of more partial edge tiles);
//  * the atoms per tile of the update kernels (64 or 32: 32-atom tiles
//    spread a small system over more SMs, 64-atom tiles stream the weights
//    once per 64 atoms).
// Results do not depend on either: every receiver's sums run over its
// edges in order within one partition, and every atom's update is the same
// sequence of MMAs.  The workspace is sized for the largest factor.
constexpr int TUNE_FACTORS[3] = {1, 2, 4};
constexpr int TUNE_FACTOR_MAX = 4;
struct TunedShape {
    int factor;          // partition factor (0: none)
    int update_atoms;    // atoms per update-kernel tile
};
constexpr TunedShape DEFAULT_SHAPE{1, 64};
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, TunedShape> g_tune;
thread_local TunedShape g_tune_override{0, 0};   // set by mlff_autotune while it times a candidate
int ceil_log2(int64_t x) {
    int b = 0;
    while ((int64_t(1) << b) < x) ++b;
    return b;
}
std::tuple<int, int, int> tune_key(int32_t path, int32_t n_atoms, int32_t n_mol) {
    return {path, ceil_log2(std::max(n_atoms, 1)), ceil_log2(std::max(n_mol, 1))};
}
}  // namespace

TunedShape tuned_shape(int32_t path, int32_t n_atoms, int32_t n_mol) {
    if (path != MLFF_PATH_TUNED_TC) return DEFAULT_SHAPE;
    if (g_tune_override.factor) return g_tune_override;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(path, n_atoms, n_mol));
    return it == g_tune.end() ? DEFAULT_SHAPE : it->second;
}

WsLayout ws_layout(const mlff_dims& d, int32_t n_atoms, int32_t n_mol, int64_t cap, int32_t path) {
    WsLayout L{};
    L.N = n_atoms;
    L.B = n_mol;
    L.L = d.n_layers;
    // arrays sized for the largest partition factor, so that tuning never changes the size
    const int64_t P_max = (int64_t)persistent_ctas(path) * (path == MLFF_PATH_TUNED_TC ? TUNE_FACTOR_MAX : 1);
    const TunedShape shape = tuned_shape(path, n_atoms, n_mol);
    L.P = persistent_ctas(path) * shape.factor;
    L.UT = shape.update_atoms;
    L.cap = cap;
    // Morton code spaces of the cell grids: under 8 x max(n_atoms, 27) per structure
    L.ncell_cap = 8LL * ((int64_t)n_atoms + 27LL * n_mol);
    size_t p = 0;
    auto take = [&](size_t bytes) {
        size_t r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    const int64_t N = n_atoms, B = n_mol, Ly = d.n_layers;
    // the tangent pass of the force-loss gradient keeps (value, tangent)
    // pairs in the plain path's float arrays
    const bool dual = path == MLFF_PATH_TRAIN_FORCES;
    const size_t fs = dual ? 2 * sizeof(float) : sizeof(float);
    const int64_t scan_n = std::max<int64_t>(N + 1, L.ncell_cap + 1);
    L.status = take(sizeof(Status));
    L.pos4 = take(sizeof(float4) * N);
    L.atom_mol = take(4 * N);
    L.row_ptr = take(4 * (N + 1));
    L.col = take(4 * cap);
    L.erecv = take(4 * cap);
    L.rev = take(4 * cap);
    L.edge_acc = take(sizeof(float4) * cap);
    L.scan_tmp = take(4 * ((scan_n + 1023) / 1024 + 2));
    L.mol_grid = take(sizeof(int4) * (B + 1));   // + the count of cell codes in use
    L.mol_box = take(sizeof(float4) * 2 * B);
    L.cell_count = take(4 * (L.ncell_cap + 1));
    L.cell_fill = take(4 * L.ncell_cap);
    L.cell_pos = take(sizeof(float4) * N);
    L.atom_cell = take(4 * N);
    L.part = take(4 * (P_max + 1));
    L.X = take(fs * (Ly + 1) * N * 4 * H);
    L.Xt = take(fs * Ly * N * 4 * H);
    L.uz = take(fs * Ly * N * H);
    L.ua = take(fs * Ly * N * H3);
    // two adjoint buffers; the second also holds the per-atom virial (9 doubles)
    L.xbar = take(fs * 2 * N * 4 * H);
    L.e_atom = take(sizeof(float) * N);
    L.md_pos32 = take(sizeof(float) * 3 * N);
    L.md_noise = take(sizeof(double) * 6 * N);
    if (path == MLFF_PATH_TUNED_TC) {
        L.geo = take(sizeof(float4) * cap);
        // at most cap / 32 + one partial tile per partition: sum over partitions of ceil(E_p / 32)
        L.n_etile = cap / 32 + P_max + 1;
        L.etile_base = take(4 * ((size_t)P_max + 1));
        L.etile = take((size_t)L.n_etile * 8192);
        L.qs = take((size_t)N * 3 * 2 * H * 2);
        L.qb = take(sizeof(float) * 3 * N);
    }
    if (path == MLFF_PATH_PLAIN_FP32 || path == MLFF_PATH_TRAIN || dual) {
        L.geo = take(4 * fs * cap);
        L.erbf = take(fs * cap * RMAX);
        L.erbf_d = take(fs * cap * RMAX);
        L.fz = take(fs * Ly * cap * H);
        L.ff = take(fs * Ly * cap * H3);
        L.fh = take(fs * cap * H);
        L.fbar = take(fs * cap * H3);
        L.comb = take(fs * N * 2 * H);
        L.uh = take(fs * N * H);
        L.abar = take(fs * N * H3);
    }
    if (path == MLFF_PATH_TRAIN || dual) {
        L.gcomb = take(fs * N * 2 * H);
        L.ghead = take(fs * N * 193);
        L.gpart = take(fs * GRAD_SPLIT * H3 * H);
        L.gmix = take(fs * GRAD_MIX_BLOCKS * 9);
    }
    L.total = p;
    return L;
}

static int check_dims(const mlff_dims* d) {
    if (!d) { set_error("dims is NULL"); return MLFF_ERR_INVALID; }
    if (d->hidden != H) {
        set_error("hidden=%d: the kernels implement hidden_dim=128", d->hidden);
        return MLFF_ERR_UNSUPPORTED;
    }
    if (d->n_rbf < 1 || d->n_rbf > RMAX) {
        set_error("n_rbf=%d outside 1..%d", d->n_rbf, RMAX);
        return MLFF_ERR_UNSUPPORTED;
    }
    if (d->n_layers < 1 || d->n_layers > MAXL) {
        set_error("n_layers=%d outside 1..%d", d->n_layers, MAXL);
        return MLFF_ERR_UNSUPPORTED;
    }
    if (d->n_species < 1) { set_error("n_species=%d", d->n_species); return MLFF_ERR_INVALID; }
    if (!(d->cutoff > 0.0f)) { set_error("cutoff must be > 0"); return MLFF_ERR_INVALID; }
    return MLFF_OK;
}

static int check_sys(const mlff_system* s, int64_t cap) {
    if (!s) { set_error("system is NULL"); return MLFF_ERR_INVALID; }
    if (s->n_atoms < 1 || s->n_mol < 1) { set_error("empty system (n_atoms=%d n_mol=%d)", s->n_atoms, s->n_mol); return MLFF_ERR_INVALID; }
    if (!s->pos || !s->Z || !s->mol_ptr) { set_error("pos, Z and mol_ptr are required"); return MLFF_ERR_INVALID; }
    if ((s->box == nullptr) != (s->pbc == nullptr)) { set_error("box and pbc must both be given or both be NULL"); return MLFF_ERR_INVALID; }
    if (cap < 0 || cap > INT32_MAX) { set_error("edge_capacity %lld outside 0..2^31-1", (long long)cap); return MLFF_ERR_INVALID; }
    return MLFF_OK;
}

static int check_path(int32_t path) {
    if (path != MLFF_PATH_PLAIN_FP32 && path != MLFF_PATH_TUNED_TC && path != MLFF_PATH_TUNED_FP32 &&
        path != MLFF_PATH_TRAIN && path != MLFF_PATH_TRAIN_FORCES) {
        set_error("unknown path %d", path);
        return MLFF_ERR_INVALID;
    }
    return MLFF_OK;
}

int pack_fp32(const mlff_dims& d, const mlff_params& p, float* out, const PackedOffsets& o, cudaStream_t st);
extern std::atomic<int> g_stall_test;
int pack_bf16(const mlff_dims& d, float* out, const PackedOffsets& o, cudaStream_t st);

}  // namespace mlff

namespace mlff {
// neighbour build + model + reverse pass; leaves the status word alone so
// that an error raised in an earlier MD step stays visible
int energy_forces_impl(const mlff_dims& d, const void* packed, const mlff_system& sys, const WsLayout& L,
                       int32_t path, const mlff_outputs& out, void* ws, cudaStream_t st,
                       const VerletFuse* vf = nullptr) {
    PackedOffsets po = packed_offsets(d);
    int r = launch_neighbors(d, sys, L, ws, st);
    if (r) return r;
    const float* P = static_cast<const float*>(packed);
    if (path == MLFF_PATH_PLAIN_FP32 || path == MLFF_PATH_TRAIN || path == MLFF_PATH_TRAIN_FORCES)
        return run_plain(d, P, po, sys, L, ws, out, st, nullptr, vf);
    return run_tuned(d, P, po, sys, L, ws, out, path, st, vf);
}
int md_kick_drift(const WsLayout& L, void* ws, mlff_md_state* s, double dt, cudaStream_t st);
int md_langevin_baoa(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT,
                     uint64_t seed, cudaStream_t st);
int md_vec_open(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT, uint64_t seed,
                int32_t fix_com, const int64_t* mol_ptr, int32_t n_mol, cudaStream_t st);
int md_vec_close(const WsLayout& L, void* ws, mlff_md_state* s, double dt, double friction, double kT,
                 int32_t fix_com, const int64_t* mol_ptr, int32_t n_mol, double* kinetic, cudaStream_t st);
int md_energy_stats(const double* epot, const double* ekin, int32_t n, int32_t B, const int64_t* mol_ptr,
                    double dt_ps, double* out, cudaStream_t st);
int md_kinetic_from_atoms(const double* ke_atom, mlff_md_state* s, const int64_t* mol_ptr, int32_t n_mol,
                          cudaStream_t st);
int md_kick(const WsLayout& L, void* ws, mlff_md_state* s, double dt, const int64_t* mol_ptr, int32_t n_mol,
            bool kinetic, cudaStream_t st);
int md_npt_open(const WsLayout& L, void* ws, const mlff_md_state* s, const mlff_npt_state* n, double dt, double kT,
                double ttime, double pfactor, double pext, const int64_t* mol_ptr, int32_t n_mol, cudaStream_t st);
int md_npt_close(const WsLayout& L, void* ws, const mlff_md_state* s, const mlff_npt_state* n, double dt, double kT,
                 double ttime, double pfactor, double pext, const int64_t* mol_ptr, int32_t n_mol, double* kinetic,
                 cudaStream_t st);
}  // namespace mlff

using namespace mlff;

extern "C" {

int mlff_version(void) { return 100; }

int mlff_debug_stall_test(int32_t kernels) {
    if (kernels < 0 || kernels > 3) {
        set_error("stall test mask %d outside 0..3", kernels);
        return MLFF_ERR_INVALID;
    }
    g_stall_test.store(kernels);
    return MLFF_OK;
}

const char* mlff_last_error_string(void) { return g_err; }

size_t mlff_packed_weights_size(const mlff_dims* dims) {
    if (check_dims(dims)) return 0;
    return sizeof(float) * (size_t)packed_offsets(*dims).total;
}

int mlff_pack_weights(const mlff_dims* dims, const mlff_params* params, void* packed, size_t packed_bytes,
                      mlff_stream_t stream) {
    int r = check_dims(dims);
    if (r) return r;
    if (!params || !packed) { set_error("params and packed are required"); return MLFF_ERR_INVALID; }
    PackedOffsets o = packed_offsets(*dims);
    if (packed_bytes < sizeof(float) * (size_t)o.total) {
        set_error("packed blob %zu bytes < %zu needed", packed_bytes, sizeof(float) * (size_t)o.total);
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if ((r = pack_fp32(*dims, *params, static_cast<float*>(packed), o, st))) return r;
    return pack_bf16(*dims, static_cast<float*>(packed), o, st);
}

size_t mlff_workspace_size(const mlff_dims* dims, int32_t n_atoms, int32_t n_mol, int64_t edge_capacity,
                           int32_t path) {
    if (check_dims(dims) || check_path(path) || n_atoms < 0 || n_mol < 0 || edge_capacity < 0) return 0;
    return ws_layout(*dims, n_atoms, n_mol, edge_capacity, path).total;
}

static int prepare(const mlff_dims* dims, const mlff_system* sys, int64_t cap, int32_t path, void* ws,
                   size_t ws_bytes, WsLayout& L) {
    int r = check_dims(dims);
    if (r) return r;
    if ((r = check_sys(sys, cap))) return r;
    if ((r = check_path(path))) return r;
    if (!ws) { set_error("workspace is NULL"); return MLFF_ERR_INVALID; }
    L = ws_layout(*dims, sys->n_atoms, sys->n_mol, cap, path);
    if (ws_bytes < L.total) {
        set_error("workspace %zu bytes < %zu needed", ws_bytes, L.total);
        return MLFF_ERR_WORKSPACE;
    }
    return MLFF_OK;
}

int mlff_build_neighbors(const mlff_dims* dims, const mlff_system* sys, int64_t edge_capacity, void* workspace,
                         size_t workspace_bytes, mlff_stream_t stream) {
    WsLayout L;
    int r = prepare(dims, sys, edge_capacity, MLFF_PATH_TUNED_FP32, workspace, workspace_bytes, L);
    if (r) return r;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    return launch_neighbors(*dims, *sys, L, workspace, st);
}

int mlff_copy_neighbors(const void* workspace, int32_t n_atoms, int32_t n_mol, int64_t edge_capacity, int32_t path,
                        int32_t* row_ptr, int32_t* col, mlff_stream_t stream) {
    if (!workspace || !row_ptr || !col) { set_error("workspace, row_ptr and col are required"); return MLFF_ERR_INVALID; }
    mlff_dims d{H, RMAX, 1, 1, 5.0f};
    WsLayout L = ws_layout(d, n_atoms, n_mol, edge_capacity, path);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemcpyAsync(row_ptr, ws_ptr<int32_t>(workspace, L.row_ptr), 4 * ((size_t)n_atoms + 1),
                              cudaMemcpyDeviceToDevice, st));
    MLFF_CUDA(cudaMemcpyAsync(col, ws_ptr<int32_t>(workspace, L.col), 4 * (size_t)edge_capacity,
                              cudaMemcpyDeviceToDevice, st));
    return MLFF_OK;
}


int mlff_energy_forces(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                       int32_t path, const mlff_outputs* out, void* workspace, size_t workspace_bytes,
                       mlff_stream_t stream) {
    WsLayout L;
    int r = prepare(dims, sys, edge_capacity, path, workspace, workspace_bytes, L);
    if (r) return r;
    if (!packed || !out || !out->energy) { set_error("packed weights and out->energy are required"); return MLFF_ERR_INVALID; }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    return energy_forces_impl(*dims, packed, *sys, L, path, *out, workspace, st);
}

// One integrator for both entry points: Verlet (langevin false) or BAOAB.
int mlff_autotune(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                  int32_t path, const mlff_outputs* out, void* workspace, size_t workspace_bytes, mlff_stream_t stream,
                  int32_t repeats, int32_t* chosen, double* ms_per_candidate) {
    if (path != MLFF_PATH_TUNED_TC) {
        if (chosen) *chosen = 1;
        return MLFF_OK;   // the other paths have no tunable shape
    }
    if (repeats < 1 || repeats > 1000) { set_error("repeats %d outside 1..1000", repeats); return MLFF_ERR_INVALID; }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    MLFF_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_status(ce, "cudaEventCreate");
    }
    int r = MLFF_OK;
    // mean milliseconds per call of one candidate shape
    auto time_shape = [&](TunedShape sh, float& ms) {
        g_tune_override = sh;
        r = mlff_energy_forces(dims, packed, sys, edge_capacity, path, out, workspace, workspace_bytes, stream);
        if (r == MLFF_OK && (ce = cudaEventRecord(e0, st)) != cudaSuccess) r = cuda_status(ce, "cudaEventRecord");
        for (int k = 0; k < repeats && r == MLFF_OK; ++k)
            r = mlff_energy_forces(dims, packed, sys, edge_capacity, path, out, workspace, workspace_bytes, stream);
        if (r == MLFF_OK && (ce = cudaEventRecord(e1, st)) != cudaSuccess) r = cuda_status(ce, "cudaEventRecord");
        if (r == MLFF_OK && (ce = cudaEventSynchronize(e1)) != cudaSuccess) r = cuda_status(ce, "cudaEventSynchronize");
        if (r == MLFF_OK && (ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) r = cuda_status(ce, "cudaEventElapsedTime");
        if (r == MLFF_OK) ms /= repeats;
    };
    // the partition factor with 64-atom update tiles, then the winner with 32-atom tiles
    TunedShape best = DEFAULT_SHAPE;
    float best_ms = 0.f;
    for (int i = 0; i < 3 && r == MLFF_OK; ++i) {
        float ms = 0.f;
        time_shape(TunedShape{TUNE_FACTORS[i], 64}, ms);
        if (r == MLFF_OK) {
            if (ms_per_candidate) ms_per_candidate[i] = ms;
            if (i == 0 || ms < best_ms) {
                best_ms = ms;
                best = TunedShape{TUNE_FACTORS[i], 64};
            }
        }
    }
    if (r == MLFF_OK) {   // 32-atom tiles only when clearly faster (timings vary by ~0.5 %)
        float ms = 0.f;
        time_shape(TunedShape{best.factor, 32}, ms);
        if (r == MLFF_OK && ms < 0.99f * best_ms) best.update_atoms = 32;
    }
    g_tune_override = TunedShape{0, 0};
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r) return r;
    // a device error (capacity, box, ...) in the timed calls makes the timings meaningless
    Status s{};
    MLFF_CUDA(cudaMemcpyAsync(&s, workspace, sizeof(Status), cudaMemcpyDeviceToHost, st));
    MLFF_CUDA(cudaStreamSynchronize(st));
    if (s.code != MLFF_OK) {
        set_error("device status %d during autotuning: nothing cached", s.code);
        return s.code;
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[tune_key(path, sys->n_atoms, sys->n_mol)] = best;
    }
    if (chosen) *chosen = best.factor;
    return MLFF_OK;
}

int mlff_autotune_query(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t* factor) {
    if (!factor) { set_error("factor is required"); return MLFF_ERR_INVALID; }
    *factor = tuned_shape(path, n_atoms, n_mol).factor;
    return MLFF_OK;
}

int mlff_autotune_query_shape(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t* factor, int32_t* update_atoms) {
    if (!factor || !update_atoms) { set_error("factor and update_atoms are required"); return MLFF_ERR_INVALID; }
    const TunedShape sh = tuned_shape(path, n_atoms, n_mol);
    *factor = sh.factor;
    *update_atoms = sh.update_atoms;
    return MLFF_OK;
}

int mlff_autotune_set(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t factor) {
    if (factor != 0 && factor != 1 && factor != 2 && factor != 4) {
        set_error("partition factor %d: use 1, 2 or 4 (0 removes the entry)", factor);
        return MLFF_ERR_INVALID;
    }
    if (path != MLFF_PATH_TUNED_TC) { set_error("only the tensor-core path has a tunable shape"); return MLFF_ERR_INVALID; }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const auto key = tune_key(path, n_atoms, n_mol);
    if (factor == 0) {
        g_tune.erase(key);
    } else {
        auto it = g_tune.find(key);   // the bucket's update tile stays as it was
        g_tune[key] = TunedShape{factor, it == g_tune.end() ? DEFAULT_SHAPE.update_atoms : it->second.update_atoms};
    }
    return MLFF_OK;
}

int mlff_autotune_set_shape(int32_t path, int32_t n_atoms, int32_t n_mol, int32_t factor, int32_t update_atoms) {
    if (factor != 0 && factor != 1 && factor != 2 && factor != 4) {
        set_error("partition factor %d: use 1, 2 or 4 (0 removes the entry)", factor);
        return MLFF_ERR_INVALID;
    }
    if (factor != 0 && update_atoms != 32 && update_atoms != 64) {
        set_error("update tile %d atoms: use 32 or 64", update_atoms);
        return MLFF_ERR_INVALID;
    }
    if (path != MLFF_PATH_TUNED_TC) { set_error("only the tensor-core path has a tunable shape"); return MLFF_ERR_INVALID; }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (factor == 0) g_tune.erase(tune_key(path, n_atoms, n_mol));
    else g_tune[tune_key(path, n_atoms, n_mol)] = TunedShape{factor, update_atoms};
    return MLFF_OK;
}

int mlff_autotune_reset(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
    return MLFF_OK;
}

// One integrator for three entry points: scheme 0 velocity Verlet, 1 BAOAB
// Langevin, 2 ASE's Langevin (Vanden-Eijnden-Ciccotti; fix_com as ASE's fixcm).
enum { MD_VERLET = 0, MD_BAOAB = 1, MD_VEC = 2 };
static int md_steps(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                    int32_t path, mlff_md_state* state, double dt, int scheme, double friction, double kT,
                    uint64_t seed, int32_t fix_com, int32_t n_steps, void* workspace, size_t workspace_bytes,
                    mlff_stream_t stream) {
    const bool langevin = scheme != MD_VERLET;
    if (!sys || !state || !state->pos || !state->vel || !state->inv_mass || !state->forces || !state->energy) {
        set_error("system and md state (pos, vel, inv_mass, forces, energy) are required");
        return MLFF_ERR_INVALID;
    }
    if (n_steps < 0 || !(dt > 0.0)) { set_error("n_steps >= 0 and dt > 0 required"); return MLFF_ERR_INVALID; }
    if (langevin && (!state->step_counter || !(friction >= 0.0) || !(kT >= 0.0))) {
        set_error("Langevin steps need state->step_counter, friction >= 0 and kT >= 0");
        return MLFF_ERR_INVALID;
    }
    if (!packed) { set_error("packed weights are required"); return MLFF_ERR_INVALID; }
    mlff_system s2 = *sys;
    WsLayout L;
    {
        // validate with a non-null placeholder position pointer
        s2.pos = reinterpret_cast<const float*>(workspace);
        int r = prepare(dims, &s2, edge_capacity, path, workspace, workspace_bytes, L);
        if (r) return r;
    }
    s2.pos = ws_ptr<float>(workspace, L.md_pos32);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    const int64_t B = sys->n_mol;
    // Velocity Verlet: the force kernel of step s closes step s (half kick,
    // kinetic energy terms) and opens step s + 1 (half kick, drift), so only
    // the first step of a call has a kick-drift launch of its own.  The
    // per-atom kinetic terms go to the per-atom virial scratch's far end
    // (the second adjoint buffer, free once the force kernel runs).
    double* ke_atom = reinterpret_cast<double*>(ws_ptr<float>(workspace, L.xbar) + (int64_t)L.N * 4 * H) +
                      (int64_t)9 * L.N;
    int r;
    for (int s = 0; s < n_steps; ++s) {
        const bool last = s == n_steps - 1;
        mlff_outputs out{state->energy_trace && !last ? state->energy_trace + s * B : state->energy, state->forces,
                         nullptr, nullptr};
        mlff_md_state ks = *state;
        if (state->kinetic_trace) ks.kinetic = state->kinetic_trace + s * B;
        const bool want_ke = (last || state->kinetic_trace) && ks.kinetic;
        if (scheme == MD_VEC) r = md_vec_open(L, workspace, state, dt, friction, kT, seed, fix_com, sys->mol_ptr,
                                              sys->n_mol, st);
        else if (scheme == MD_BAOAB) r = md_langevin_baoa(L, workspace, state, dt, friction, kT, seed, st);
        else r = s == 0 ? md_kick_drift(L, workspace, state, dt, st) : MLFF_OK;
        if (r) return r;
        if (scheme == MD_VERLET) {
            const VerletFuse vf{state->vel, state->inv_mass, state->pos, ws_ptr<float>(workspace, L.md_pos32),
                                want_ke ? ke_atom : nullptr, state->step_counter, dt, last ? 0 : 1};
            if ((r = energy_forces_impl(*dims, packed, s2, L, path, out, workspace, st, &vf))) return r;
            if (want_ke) r = md_kinetic_from_atoms(ke_atom, &ks, sys->mol_ptr, sys->n_mol, st);
        } else {
            if ((r = energy_forces_impl(*dims, packed, s2, L, path, out, workspace, st))) return r;
            if (scheme == MD_VEC)
                r = md_vec_close(L, workspace, &ks, dt, friction, kT, fix_com, sys->mol_ptr, sys->n_mol,
                                 (last || state->kinetic_trace) ? ks.kinetic : nullptr, st);
            else
                r = md_kick(L, workspace, &ks, dt, sys->mol_ptr, sys->n_mol, last || state->kinetic_trace, st);
        }
        if (r) return r;
        if (last) {
            if (state->energy_trace)
                MLFF_CUDA(cudaMemcpyAsync(state->energy_trace + s * B, state->energy, sizeof(double) * B,
                                          cudaMemcpyDeviceToDevice, st));
            if (state->kinetic_trace && state->kinetic)
                MLFF_CUDA(cudaMemcpyAsync(state->kinetic, state->kinetic_trace + s * B, sizeof(double) * B,
                                          cudaMemcpyDeviceToDevice, st));
        }
    }
    return MLFF_OK;
}

int mlff_verlet_steps(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                      int32_t path, mlff_md_state* state, double dt, int32_t n_steps, void* workspace,
                      size_t workspace_bytes, mlff_stream_t stream) {
    return md_steps(dims, packed, sys, edge_capacity, path, state, dt, MD_VERLET, 0.0, 0.0, 0, 0, n_steps, workspace,
                    workspace_bytes, stream);
}

int mlff_langevin_steps(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                        int32_t path, mlff_md_state* state, double dt, double friction, double kT, uint64_t seed,
                        int32_t n_steps, void* workspace, size_t workspace_bytes, mlff_stream_t stream) {
    return md_steps(dims, packed, sys, edge_capacity, path, state, dt, MD_BAOAB, friction, kT, seed, 0, n_steps,
                    workspace, workspace_bytes, stream);
}

int mlff_langevin_ase_steps(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                            int32_t path, mlff_md_state* state, double dt, double friction, double kT, uint64_t seed,
                            int32_t fix_com, int32_t n_steps, void* workspace, size_t workspace_bytes,
                            mlff_stream_t stream) {
    return md_steps(dims, packed, sys, edge_capacity, path, state, dt, MD_VEC, friction, kT, seed, fix_com ? 1 : 0,
                    n_steps, workspace, workspace_bytes, stream);
}

int mlff_npt_steps(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                   int32_t path, mlff_md_state* state, mlff_npt_state* npt, double dt, double kT, double ttime,
                   double pfactor, double pressure, int32_t n_steps, void* workspace, size_t workspace_bytes,
                   mlff_stream_t stream) {
    if (!sys || !state || !state->pos || !state->vel || !state->inv_mass || !state->forces || !state->energy) {
        set_error("system and md state (pos, vel, inv_mass, forces, energy) are required");
        return MLFF_ERR_INVALID;
    }
    if (!npt || !npt->box || !npt->box32 || !npt->zeta || !npt->eta || !npt->xi || !npt->virial || !sys->pbc) {
        set_error("NPT state (box, box32, zeta, eta, xi, virial) and periodic flags are required");
        return MLFF_ERR_INVALID;
    }
    if (n_steps < 0 || !(dt > 0.0) || !(ttime >= 0.0) || !(pfactor >= 0.0) || !(kT >= 0.0) ||
        (ttime > 0.0 && !(kT > 0.0)) || !std::isfinite(pressure)) {
        set_error("NPT needs n_steps >= 0, dt > 0, ttime >= 0, pfactor >= 0, kT > 0 with a thermostat, "
                  "finite pressure");
        return MLFF_ERR_INVALID;
    }
    if (!packed) { set_error("packed weights are required"); return MLFF_ERR_INVALID; }
    mlff_system s2 = *sys;
    s2.box = npt->box32;
    WsLayout L;
    {
        const float* keep = s2.pos;
        s2.pos = reinterpret_cast<const float*>(workspace);   // placeholder for the check
        int r = prepare(dims, &s2, edge_capacity, path, workspace, workspace_bytes, L);
        s2.pos = keep;
        if (r) return r;
    }
    s2.pos = ws_ptr<float>(workspace, L.md_pos32);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    const int64_t B = sys->n_mol;
    int r;
    for (int s = 0; s < n_steps; ++s) {
        const bool last = s == n_steps - 1;
        mlff_outputs out{state->energy_trace && !last ? state->energy_trace + s * B : state->energy, state->forces,
                         npt->virial, nullptr};
        double* ke = state->kinetic_trace ? state->kinetic_trace + s * B : state->kinetic;
        if ((r = md_npt_open(L, workspace, state, npt, dt, kT, ttime, pfactor, pressure, sys->mol_ptr, sys->n_mol, st)))
            return r;
        if ((r = energy_forces_impl(*dims, packed, s2, L, path, out, workspace, st))) return r;
        if ((r = md_npt_close(L, workspace, state, npt, dt, kT, ttime, pfactor, pressure, sys->mol_ptr, sys->n_mol,
                              (last || state->kinetic_trace) ? ke : nullptr, st)))
            return r;
        if (last) {
            if (state->energy_trace)
                MLFF_CUDA(cudaMemcpyAsync(state->energy_trace + s * B, state->energy, sizeof(double) * B,
                                          cudaMemcpyDeviceToDevice, st));
            if (state->kinetic_trace && state->kinetic)
                MLFF_CUDA(cudaMemcpyAsync(state->kinetic, state->kinetic_trace + s * B, sizeof(double) * B,
                                          cudaMemcpyDeviceToDevice, st));
        }
    }
    return MLFF_OK;
}

int mlff_md_energy_stats(const double* epot, const double* ekin, int32_t n_samples, int32_t n_mol,
                         const int64_t* mol_ptr, double dt_ps, double* out, mlff_stream_t stream) {
    if (!epot || !ekin || !out) { set_error("epot, ekin and out are required"); return MLFF_ERR_INVALID; }
    if (n_samples < 1 || n_mol < 1) { set_error("n_samples >= 1 and n_mol >= 1 required"); return MLFF_ERR_INVALID; }
    if (!(dt_ps > 0.0)) { set_error("dt_ps > 0 required"); return MLFF_ERR_INVALID; }
    return md_energy_stats(epot, ekin, n_samples, n_mol, mol_ptr, dt_ps, out, reinterpret_cast<cudaStream_t>(stream));
}

int mlff_param_grads(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                     const double* energy_weights, const mlff_grads* grads, const mlff_outputs* out, void* workspace,
                     size_t workspace_bytes, mlff_stream_t stream) {
    WsLayout L;
    int r = prepare(dims, sys, edge_capacity, MLFF_PATH_TRAIN, workspace, workspace_bytes, L);
    if (r) return r;
    if (!packed || !energy_weights || !grads || !out || !out->energy) {
        set_error("packed weights, energy_weights, grads and out->energy are required");
        return MLFF_ERR_INVALID;
    }
    if (out->virial) { set_error("the training path returns no virial"); return MLFF_ERR_INVALID; }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    if ((r = launch_neighbors(*dims, *sys, L, workspace, st))) return r;
    PackedOffsets po = packed_offsets(*dims);
    GradCtx g{energy_weights, *grads};
    return run_plain(*dims, static_cast<const float*>(packed), po, *sys, L, workspace, *out, st, &g);
}

int mlff_param_grads_forces(const mlff_dims* dims, const void* packed, const mlff_system* sys, int64_t edge_capacity,
                            const float* force_weights, const double* virial_weights, const mlff_grads* grads,
                            void* workspace, size_t workspace_bytes, mlff_stream_t stream) {
    WsLayout L;
    int r = prepare(dims, sys, edge_capacity, MLFF_PATH_TRAIN_FORCES, workspace, workspace_bytes, L);
    if (r) return r;
    if (!packed || (!force_weights && !virial_weights) || !grads) {
        set_error("packed weights, grads and force_weights and / or virial_weights are required");
        return MLFF_ERR_INVALID;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    MLFF_CUDA(cudaMemsetAsync(ws_ptr<Status>(workspace, L.status), 0, sizeof(Status), st));
    if ((r = launch_neighbors(*dims, *sys, L, workspace, st))) return r;
    PackedOffsets po = packed_offsets(*dims);
    GradCtx g{nullptr, *grads};
    return run_plain_tangent(*dims, static_cast<const float*>(packed), po, *sys, L, workspace, st, g, force_weights,
                             virial_weights);
}

int mlff_read_status(const void* workspace, int32_t* code, int64_t* n_edges, int32_t* where, mlff_stream_t stream) {
    if (!workspace) { set_error("workspace is NULL"); return MLFF_ERR_INVALID; }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Status s;
    MLFF_CUDA(cudaMemcpyAsync(&s, workspace, sizeof(Status), cudaMemcpyDeviceToHost, st));
    MLFF_CUDA(cudaStreamSynchronize(st));
    if (code) *code = s.code;
    if (n_edges) *n_edges = ((int64_t)s.n_edges_hi << 31) | (int64_t)(uint32_t)s.n_edges;
    if (where) *where = s.code ? s.where : -1;
    return MLFF_OK;
}

int mlff_clear_status(void* workspace, mlff_stream_t stream) {
    if (!workspace) { set_error("workspace is NULL"); return MLFF_ERR_INVALID; }
    MLFF_CUDA(cudaMemsetAsync(workspace, 0, sizeof(Status), reinterpret_cast<cudaStream_t>(stream)));
    return MLFF_OK;
}

}  // extern "C"
