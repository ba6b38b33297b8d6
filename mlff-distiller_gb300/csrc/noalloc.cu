// Radius graph for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc or hand the library a workspace: a
// host that owns every allocation itself (a memory-budgeted MD engine, an
// FFI caller whose allocator is not CUDA-aware, code running inside a
// region where allocation is forbidden).  mlff_radius_graph_noalloc serves
// them with the same kernels as mlff_build_neighbors, but its scratch
// (atom copies, scan blocks, cell lists, receiver ids, status word) lives in
// one file-scope device array of fixed size instead of a workspace.
//
// Limits: at most NOALLOC_MAX_ATOMS atoms, NOALLOC_MAX_MOLS structures and
// NOALLOC_MAX_EDGES directed edges per call; larger inputs are rejected.
// The array is about 13 MB and stays resident on every device that has
// loaded the library until the process exits.
//
// Every call shares the array and it keeps the last call's contents: the
// entry point clears what must start at zero, and two calls that overlap on
// the GPU (different streams, no ordering between them) race on it.  The
// first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current); make that first call
// before any stream capture.
#include <mutex>
#include "common.cuh"
#include "workspace.h"

namespace mlff {

constexpr int64_t NOALLOC_MAX_ATOMS = 16384;
constexpr int64_t NOALLOC_MAX_MOLS = 4096;
constexpr int64_t NOALLOC_MAX_EDGES = 1 << 20;

namespace {
constexpr int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }
constexpr int64_t kNcellCap = 8 * (NOALLOC_MAX_ATOMS + 27 * NOALLOC_MAX_MOLS);   // Morton code spaces
constexpr int64_t kScanN = kNcellCap + 1;    // >= N + 1
constexpr int64_t kOffStatus = 0;
constexpr int64_t kOffPos4 = align256(kOffStatus + (int64_t)sizeof(Status));
constexpr int64_t kOffAtomMol = align256(kOffPos4 + 16 * NOALLOC_MAX_ATOMS);
constexpr int64_t kOffErecv = align256(kOffAtomMol + 4 * NOALLOC_MAX_ATOMS);
constexpr int64_t kOffScan = align256(kOffErecv + 4 * NOALLOC_MAX_EDGES);
constexpr int64_t kOffGrid = align256(kOffScan + 4 * ((kScanN + 1023) / 1024 + 2));
constexpr int64_t kOffMolBox = align256(kOffGrid + 16 * (NOALLOC_MAX_MOLS + 1));
constexpr int64_t kOffCellCount = align256(kOffMolBox + 16 * 2 * NOALLOC_MAX_MOLS);
constexpr int64_t kOffCellFill = align256(kOffCellCount + 4 * (kNcellCap + 1));
constexpr int64_t kOffCellPos = align256(kOffCellFill + 4 * kNcellCap);
constexpr int64_t kOffAtomCell = align256(kOffCellPos + 16 * NOALLOC_MAX_ATOMS);
constexpr int64_t kScratchBytes = align256(kOffAtomCell + 4 * NOALLOC_MAX_ATOMS);
static_assert(kScratchBytes < 14 * 1024 * 1024, "static scratch must stay modest");
}  // namespace

// The shared scratch of the allocation-free entry point.  In host code this
// name is only a host-side stand-in for the symbol; kernels get its device
// address from scratch_address().
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {
std::mutex g_scratch_mu;
void* g_scratch_dev[256] = {};

// Device address of the scratch array for the current device, looked up
// once per device.
int scratch_address(void** out) {
    int dev = 0;
    MLFF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_error("device ordinal %d out of range", dev);
        return MLFF_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (g_scratch_dev[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return MLFF_OK;
}
}  // namespace

}  // namespace mlff

using namespace mlff;

extern "C" int mlff_radius_graph_noalloc(const mlff_system* sys, float cutoff, int64_t edge_capacity,
                                         int32_t* row_ptr, int32_t* col, int32_t* status,
                                         mlff_stream_t stream) {
    if (!sys || !row_ptr || !col || !status) {
        set_error("system, row_ptr, col and status are required");
        return MLFF_ERR_INVALID;
    }
    if (sys->n_atoms < 1 || sys->n_atoms > NOALLOC_MAX_ATOMS) {
        set_error("n_atoms=%d outside 1..%lld (static scratch limit)", sys->n_atoms, (long long)NOALLOC_MAX_ATOMS);
        return MLFF_ERR_INVALID;
    }
    if (sys->n_mol < 1 || sys->n_mol > NOALLOC_MAX_MOLS) {
        set_error("n_mol=%d outside 1..%lld (static scratch limit)", sys->n_mol, (long long)NOALLOC_MAX_MOLS);
        return MLFF_ERR_INVALID;
    }
    if (edge_capacity < 0 || edge_capacity > NOALLOC_MAX_EDGES) {
        set_error("edge_capacity=%lld outside 0..%lld (static scratch limit)", (long long)edge_capacity,
                  (long long)NOALLOC_MAX_EDGES);
        return MLFF_ERR_INVALID;
    }
    if (!sys->pos || !sys->Z || !sys->mol_ptr || (sys->box == nullptr) != (sys->pbc == nullptr)) {
        set_error("pos, Z, mol_ptr required; box and pbc both given or both NULL");
        return MLFF_ERR_INVALID;
    }
    if (!(cutoff > 0.0f)) {
        set_error("cutoff must be > 0");
        return MLFF_ERR_INVALID;
    }
    void* base = nullptr;
    int r = scratch_address(&base);
    if (r) return r;
    char* s = static_cast<char*>(base);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    NbrBuffers b;
    b.status = reinterpret_cast<Status*>(s + kOffStatus);
    b.pos4 = reinterpret_cast<float4*>(s + kOffPos4);
    b.atom_mol = reinterpret_cast<int32_t*>(s + kOffAtomMol);
    b.row_ptr = row_ptr;
    b.col = col;
    b.erecv = reinterpret_cast<int32_t*>(s + kOffErecv);
    b.scan_tmp = reinterpret_cast<int32_t*>(s + kOffScan);
    b.mol_grid = reinterpret_cast<int4*>(s + kOffGrid);
    b.mol_box = reinterpret_cast<float4*>(s + kOffMolBox);
    b.cell_count = reinterpret_cast<int32_t*>(s + kOffCellCount);
    b.cell_fill = reinterpret_cast<int32_t*>(s + kOffCellFill);
    b.cell_pos = reinterpret_cast<float4*>(s + kOffCellPos);
    b.atom_cell = reinterpret_cast<int32_t*>(s + kOffAtomCell);
    b.ncell_cap = 8LL * ((int64_t)sys->n_atoms + 27LL * sys->n_mol);
    b.cap = edge_capacity;
    // the status word keeps the previous call's value: clear it
    MLFF_CUDA(cudaMemsetAsync(b.status, 0, sizeof(Status), st));
    mlff_dims d{H, 1, 1, 1, cutoff};
    if ((r = launch_neighbors_into(d, *sys, b, st))) return r;
    MLFF_CUDA(cudaMemcpyAsync(status, b.status, 4 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
    return MLFF_OK;
}
