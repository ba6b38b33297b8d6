// Radius graph on the GPU: bit-exact with the reference's
// radius_graph_native (src/mlff_distiller/models/student_model.py:63-109)
// plus an orthorhombic minimum-image rule for periodic boxes.
//
// Output: receiver-sorted CSR.  Row a lists, in ascending order, every atom
// b of the same structure with |pos[b] - pos[a]| <= cutoff (float32, same
// rounding as torch.norm), b != a.  Read as [row; col] this equals the
// reference's edge_index (src-major, then dst) element for element.  In the
// model kernels row a is the receiver of the message b -> a.
//
// Open structures below OPEN_CELL_MIN atoms: every atom pair of the
// structure is tested (one warp per row, warp-ballot compaction keeps the
// ascending order).  Larger open structures get a cell grid over their
// bounding box (cells of width >= 1.001 cutoff, at most 1024 per axis and
// max(n, 27) in all, no wrap).  Periodic boxes: atoms are binned into
// cells of edge >= cutoff.  In both the cells are numbered along a
// Morton (Z-order) curve, and the atoms copied in that order (position and
// atom index in one float4, so a cell's candidates are contiguous and
// neighbouring cells lie close in memory); a row's warp looks up its 27 (or
// fewer, for small grids)
// neighbouring cells in one step -- one cell per lane, a warp scan of their
// sizes -- and walks the concatenated candidates 32 at a time, each lane
// finding its cell by a binary search over the scan; hits are compacted
// with a warp ballot into shared memory and rank-sorted.  The cell grid
// only chooses candidates: every candidate pair goes through the same
// distance decision, and two atoms within the cutoff always sit in the same
// or adjacent cells (clamped, monotone cell indices of width >= cutoff), so
// the edge set is the all-pairs one.
#include "common.cuh"
#include "workspace.h"
#include "profile.h"

namespace mlff {

constexpr int NBR_WARPS = 8;        // warps per block in the row kernels
constexpr int ROW_CAP = 512;        // neighbours one cell-list row can hold
constexpr int OPEN_CELL_MIN = 256;  // open structures with at least this many atoms use a cell grid
constexpr int OPEN_NC_MAX = 1024;   // cells per axis of an open structure's grid
constexpr float OPEN_CELL_MARGIN = 1.001f;   // open cell width / cutoff: covers the float32 cell-index rounding

// ------------------------------------------------------------------ scan
__global__ void scan_local_kernel(int32_t* __restrict__ data, int64_t n, int32_t* __restrict__ sums) {
    pdl_wait();
    pdl_trigger();
    __shared__ int32_t warp_tot[8];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t base = (int64_t)blockIdx.x * 1024 + (int64_t)t * 4;
    int32_t v[4], s = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int64_t idx = base + i;
        v[i] = idx < n ? data[idx] : 0;
        s += v[i];
    }
    int32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t wt = lane < 8 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, wt, o);
            if (lane >= o) wt += y;
        }
        if (lane < 8) warp_tot[lane] = wt;
    }
    __syncthreads();
    int32_t run = x - s + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int64_t idx = base + i;
        if (idx < n) data[idx] = run;
        run += v[i];
    }
    if (t == 255) sums[blockIdx.x] = run;
}

// exclusive scan of sums[0..nb) by one block; sums[nb] receives the total
__global__ void scan_blocks_kernel(int32_t* __restrict__ sums, int64_t nb) {
    pdl_wait();
    pdl_trigger();
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) carry = 0;
    __syncthreads();
    for (int64_t c0 = 0; c0 < nb; c0 += 1024) {
        int64_t idx = c0 + t;
        int32_t v = idx < nb ? sums[idx] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int32_t wt = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int32_t y = __shfl_up_sync(0xffffffffu, wt, o);
                if (lane >= o) wt += y;
            }
            warp_tot[lane] = wt;
        }
        __syncthreads();
        int32_t excl = carry + x - v + (w > 0 ? warp_tot[w - 1] : 0);
        if (idx < nb) sums[idx] = excl;
        __syncthreads();
        if (t == 1023) carry = excl + v;
        __syncthreads();
    }
    if (t == 0) sums[nb] = carry;
}

__global__ void scan_add_kernel(int32_t* __restrict__ data, int64_t n, const int32_t* __restrict__ sums) {
    pdl_wait();
    pdl_trigger();
    const int64_t base = (int64_t)blockIdx.x * 1024;
    const int32_t add = sums[blockIdx.x];
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
        int64_t idx = base + i;
        if (idx < n) data[idx] += add;
    }
}

// One block for small inputs: exclusive scan of data[0..n_in), data[n_in] =
// total, with n_in = n_max or the device-side count *n_dev (at most n_max).
// Each of the 1024 threads owns a contiguous run of ceil(n_in/1024) values
// (read twice: once to sum, once to write).  With st non-NULL the total is
// the edge count: it is recorded in the status word and checked against the
// edge capacity.
constexpr int64_t SCAN1_MAX = 8192;
__global__ void __launch_bounds__(1024) scan_single_kernel(int32_t* __restrict__ data, int64_t n_max,
                                                           const int32_t* __restrict__ n_dev, Status* st,
                                                           int64_t cap) {
    pdl_wait();
    pdl_trigger();
    __shared__ int32_t warp_tot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    // the count of values: n_max, or the smaller device-side count when given
    const int64_t n_in = n_dev ? min((int64_t)max(*n_dev, 0), n_max) : n_max;
    const int64_t per = (n_in + 1023) / 1024;
    const int64_t b0 = min((int64_t)t * per, n_in), b1 = min(b0 + per, n_in);
    int32_t s = 0;
    for (int64_t k = b0; k < b1; ++k) s += data[k];
    int32_t x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t wt = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, wt, o);
            if (lane >= o) wt += y;
        }
        warp_tot[lane] = wt;
    }
    __syncthreads();
    int32_t run = x - s + (w > 0 ? warp_tot[w - 1] : 0);
    for (int64_t k = b0; k < b1; ++k) {
        const int32_t v = data[k];
        data[k] = run;
        run += v;
    }
    if (t == 1023) {
        data[n_in] = run;
        if (st) {
            const int64_t e = (int64_t)(uint32_t)run;
            st->n_edges = (int32_t)(e & 0x7fffffff);
            st->n_edges_hi = (int32_t)(e >> 31);
            if (e > cap) set_status(st, MLFF_ERR_CAPACITY, -1);
        }
    }
}

// In-place exclusive scan of n int32 values; tmp holds ceil(n/1024)+1 ints.
int launch_scan(int32_t* data, int64_t n, int32_t* tmp, cudaStream_t st) {
    if (n <= 0) return MLFF_OK;
    int64_t nb = (n + 1023) / 1024;
    MLFF_LAUNCH_PDL("scan_local", scan_local_kernel, (unsigned)nb, 256, 0, st, data, n, tmp);
    MLFF_LAUNCH_PDL("scan_blocks", scan_blocks_kernel, 1, 1024, 0, st, tmp, nb);
    if (nb > 1) {
        MLFF_LAUNCH_PDL("scan_add", scan_add_kernel, (unsigned)nb, 256, 0, st, data, n, tmp);
    }
    return MLFF_OK;
}

// ------------------------------------------------------------ atom setup
__global__ void prep_atoms_kernel(const float* __restrict__ pos, const int64_t* __restrict__ mol_ptr,
                                  int32_t n_mol, int32_t n_atoms, float4* __restrict__ pos4,
                                  int32_t* __restrict__ atom_mol) {
    pdl_wait();
    pdl_trigger();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_atoms; i += gridDim.x * blockDim.x) {
        pos4[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.0f);
        // last m with mol_ptr[m] <= i
        int lo = 0, hi = n_mol - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (mol_ptr[mid] <= i) lo = mid; else hi = mid - 1;
        }
        atom_mol[i] = lo;
    }
}

// bits of a cell coordinate on an axis with nc cells
__device__ __forceinline__ int cell_bits(int nc) { return nc > 1 ? 32 - __clz(nc - 1) : 0; }

// Morton (Z-order) code of cell (x, y, z) on a grid with bx, by, bz bits per
// axis: the coordinates' bits interleaved from the lowest level up, each axis
// contributing while it still has bits -- a bijection onto [0, 2^(bx+by+bz)).
__device__ __forceinline__ int morton3(int x, int y, int z, int bx, int by, int bz) {
    int code = 0, pos = 0;
    const int nb = max(bx, max(by, bz));
    for (int b = 0; b < nb; ++b) {
        if (b < bz) code |= ((z >> b) & 1) << pos++;
        if (b < by) code |= ((y >> b) & 1) << pos++;
        if (b < bx) code |= ((x >> b) & 1) << pos++;
    }
    return code;
}

__device__ __forceinline__ bool mol_celled_open(const int64_t* mol_ptr, const uint8_t* pbc, const float* box,
                                                int m) {
    const bool per = pbc != nullptr && box != nullptr && pbc[m] != 0;
    return !per && mol_ptr[m + 1] - mol_ptr[m] >= OPEN_CELL_MIN;
}

// Bounding box (lower and upper corner) of every open structure that gets a
// cell grid: one block per structure, fixed-order min / max.
__global__ void __launch_bounds__(256) mol_bbox_kernel(const float4* __restrict__ pos4,
                                                       const int64_t* __restrict__ mol_ptr,
                                                       const uint8_t* __restrict__ pbc, const float* __restrict__ box,
                                                       int32_t n_mol, float4* __restrict__ mol_box) {
    pdl_wait();
    pdl_trigger();
    __shared__ float lo[3][256], hi[3][256];
    const int t = threadIdx.x;
    for (int m = blockIdx.x; m < n_mol; m += gridDim.x) {
        if (!mol_celled_open(mol_ptr, pbc, box, m)) continue;
        float l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t a = mol_ptr[m] + t; a < mol_ptr[m + 1]; a += 256) {
            const float4 p = pos4[a];
            l[0] = fminf(l[0], p.x); l[1] = fminf(l[1], p.y); l[2] = fminf(l[2], p.z);
            h[0] = fmaxf(h[0], p.x); h[1] = fmaxf(h[1], p.y); h[2] = fmaxf(h[2], p.z);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            lo[q][t] = l[q];
            hi[q][t] = h[q];
        }
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (t < o)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    lo[q][t] = fminf(lo[q][t], lo[q][t + o]);
                    hi[q][t] = fmaxf(hi[q][t], hi[q][t + o]);
                }
            __syncthreads();
        }
        if (t == 0) {
            mol_box[2 * m] = make_float4(lo[0][0], lo[1][0], lo[2][0], 0.f);
            mol_box[2 * m + 1] = make_float4(hi[0][0], hi[1][0], hi[2][0], 0.f);
        }
        __syncthreads();
    }
}

// One block: per periodic structure choose the cell grid (cells of edge
// >= cutoff, at most max(n_atoms, 27) cells) and the first cell code (the
// structure's Morton code space is under 8 times its cell count).
// It also zeroes the counters and fill cursors of the codes in use and
// writes their count to grid[n_mol].x.
// Open structures with a cell grid: cells of width max(1.001 cutoff,
// extent / nc) over the bounding box, the cell count limited the same way;
// mol_box[2m + 1] becomes 1 / cell width per axis.
__global__ void mol_grid_kernel(const int64_t* __restrict__ mol_ptr, const float* __restrict__ box,
                                const uint8_t* __restrict__ pbc, int32_t n_mol, float cutoff,
                                int4* __restrict__ grid, float4* __restrict__ mol_box,
                                int32_t* __restrict__ cell_count, int32_t* __restrict__ cell_fill,
                                int64_t ncell_cap, Status* st) {
    pdl_wait();
    pdl_trigger();
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < n_mol; c0 += 1024) {
        int m = c0 + t;
        int ncell = 0, nc[3] = {0, 0, 0};
        if (m < n_mol && pbc != nullptr && box != nullptr && pbc[m]) {
            int n_m = (int)(mol_ptr[m + 1] - mol_ptr[m]);
            bool ok = true;
            for (int a = 0; a < 3; ++a) {
                float L = box[3 * m + a];
                if (!(L >= 2.0f * cutoff) || !isfinite(L)) ok = false;
                else nc[a] = max(1, (int)floorf(L / (cutoff * 1.0001f)));  // cell edge > cutoff with margin
            }
            if (!ok) {
                set_status(st, MLFF_ERR_BOX, m);
                nc[0] = nc[1] = nc[2] = 1;
            }
            int lim = max(n_m, 27);
            // no axis needs more cells than lim; this also keeps the product below 2^63 for huge boxes
            for (int a = 0; a < 3; ++a) nc[a] = min(nc[a], lim);
            while ((long long)nc[0] * nc[1] * nc[2] > lim) {
                int a = (nc[0] >= nc[1] && nc[0] >= nc[2]) ? 0 : (nc[1] >= nc[2] ? 1 : 2);
                nc[a] -= 1;
            }
            // cells are numbered by their Morton code: the code space holds 2^(bits x + y + z)
            ncell = 1 << (cell_bits(nc[0]) + cell_bits(nc[1]) + cell_bits(nc[2]));
        } else if (m < n_mol && mol_celled_open(mol_ptr, pbc, box, m)) {
            const int n_m = (int)(mol_ptr[m + 1] - mol_ptr[m]);
            const float4 lo = mol_box[2 * m], hi = mol_box[2 * m + 1];
            const float ext[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
            const float w0 = cutoff * OPEN_CELL_MARGIN;
            for (int a = 0; a < 3; ++a) {
                // a non-finite extent (inf or NaN positions) gets one cell: every pair is then a candidate
                nc[a] = isfinite(ext[a]) ? (int)fminf(floorf(ext[a] / w0) + 1.0f, (float)OPEN_NC_MAX) : 1;
                nc[a] = max(nc[a], 1);
            }
            const int lim = max(n_m, 27);
            while ((long long)nc[0] * nc[1] * nc[2] > lim) {
                int a = (nc[0] >= nc[1] && nc[0] >= nc[2]) ? 0 : (nc[1] >= nc[2] ? 1 : 2);
                nc[a] -= 1;
            }
            float inv[3];
            for (int a = 0; a < 3; ++a) {
                const float wa = isfinite(ext[a]) ? fmaxf(w0, ext[a] / (float)nc[a] * OPEN_CELL_MARGIN) : 1.0f;
                inv[a] = nc[a] > 1 ? 1.0f / wa : 0.0f;
            }
            mol_box[2 * m + 1] = make_float4(inv[0], inv[1], inv[2], 0.f);
            ncell = 1 << (cell_bits(nc[0]) + cell_bits(nc[1]) + cell_bits(nc[2]));
        }
        int32_t x = ncell;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int32_t wt = warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int32_t y = __shfl_up_sync(0xffffffffu, wt, o);
                if (lane >= o) wt += y;
            }
            warp_tot[lane] = wt;
        }
        __syncthreads();
        int32_t excl = carry + x - ncell + (w > 0 ? warp_tot[w - 1] : 0);
        if (m < n_mol) grid[m] = make_int4(nc[0], nc[1], nc[2], excl);
        __syncthreads();
        if (t == 1023) carry = excl + ncell;
        __syncthreads();
    }
    // the codes in use: [0, carry); zero their counters (and the total slot) and fill cursors
    const int64_t used = min((int64_t)carry, ncell_cap);
    for (int64_t k = t; k <= used; k += blockDim.x) {
        cell_count[k] = 0;
        if (k < used) cell_fill[k] = 0;
    }
    if (t == 0) {
        if (carry > ncell_cap) set_status(st, MLFF_ERR_BOX, -1);
        grid[n_mol] = make_int4((int)used, 0, 0, 0);
    }
}

__device__ __forceinline__ bool mol_periodic(const uint8_t* pbc, const float* box, int m) {
    return pbc != nullptr && box != nullptr && pbc[m] != 0;
}

__device__ __forceinline__ Box load_box(const float* box, const uint8_t* pbc, int m) {
    Box b;
    b.periodic = mol_periodic(pbc, box, m) ? 1 : 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        b.L[a] = b.periodic ? box[3 * m + a] : 1.0f;
        b.invL[a] = __fdiv_rn(1.0f, b.L[a]);
    }
    return b;
}

__device__ __forceinline__ int cell_coord(float x, float L, float invL, int nc) {
    float w = x - L * floorf(x * invL);
    int c = (int)(w * invL * (float)nc);
    return min(max(c, 0), nc - 1);
}
// open structure: cell of coordinate x on a grid starting at lo (no wrap;
// NaN lands in cell 0)
__device__ __forceinline__ int open_cell_coord(float x, float lo, float inv_w, int nc) {
    const float f = (x - lo) * inv_w;
    const int c = f > 0.f ? (int)fminf(f, (float)(nc - 1)) : 0;
    return min(max(c, 0), nc - 1);
}

__global__ void cell_count_kernel(const float4* __restrict__ pos4, const int32_t* __restrict__ atom_mol,
                                  const int64_t* __restrict__ mol_ptr, const float* __restrict__ box,
                                  const uint8_t* __restrict__ pbc, const int4* __restrict__ grid,
                                  const float4* __restrict__ mol_box, int32_t n_atoms,
                                  int32_t* __restrict__ atom_cell, int32_t* __restrict__ cell_count) {
    pdl_wait();
    pdl_trigger();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_atoms; i += gridDim.x * blockDim.x) {
        int m = atom_mol[i];
        const bool open_cells = mol_celled_open(mol_ptr, pbc, box, m);
        if (!mol_periodic(pbc, box, m) && !open_cells) { atom_cell[i] = -1; continue; }
        int4 g = grid[m];
        float4 p = pos4[i];
        int cx, cy, cz;
        if (open_cells) {
            const float4 lo = mol_box[2 * m], iw = mol_box[2 * m + 1];
            cx = open_cell_coord(p.x, lo.x, iw.x, g.x);
            cy = open_cell_coord(p.y, lo.y, iw.y, g.y);
            cz = open_cell_coord(p.z, lo.z, iw.z, g.z);
        } else {
            Box b = load_box(box, pbc, m);
            cx = cell_coord(p.x, b.L[0], b.invL[0], g.x);
            cy = cell_coord(p.y, b.L[1], b.invL[1], g.y);
            cz = cell_coord(p.z, b.L[2], b.invL[2], g.z);
        }
        int c = g.w + morton3(cx, cy, cz, cell_bits(g.x), cell_bits(g.y), cell_bits(g.z));
        atom_cell[i] = c;
        atomicAdd(&cell_count[c], 1);
    }
}

__global__ void cell_fill_kernel(const int32_t* __restrict__ atom_cell, const int32_t* __restrict__ cell_start,
                                 const float4* __restrict__ pos4, int32_t n_atoms, int32_t* __restrict__ cell_fill,
                                 float4* __restrict__ cell_pos) {
    pdl_wait();
    pdl_trigger();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_atoms; i += gridDim.x * blockDim.x) {
        int c = atom_cell[i];
        if (c < 0) continue;
        int slot = atomicAdd(&cell_fill[c], 1);
        const float4 p = pos4[i];
        cell_pos[cell_start[c] + slot] = make_float4(p.x, p.y, p.z, __int_as_float(i));
    }
}

// -------------------------------------------------------------- rows
struct NbrArgs {
    const float4* pos4;
    const int32_t* atom_mol;
    const int64_t* mol_ptr;
    const float* box;
    const uint8_t* pbc;
    const int4* grid;
    const float4* mol_box;
    const int32_t* cell_start;
    const float4* cell_pos;
    int32_t n_atoms;
    float cutoff;
    int64_t cap;
    int32_t* counts;   // count pass: per-row counts; fill pass: row_ptr
    int32_t* col;
    int32_t* erecv;
    Status* st;
};

template <bool FILL>
__global__ void __launch_bounds__(NBR_WARPS * 32) nbr_rows_kernel(NbrArgs a) {
    pdl_wait();
    pdl_trigger();
    __shared__ int32_t sbuf[FILL ? NBR_WARPS : 1][FILL ? ROW_CAP : 1];
    if (FILL && a.st->code != 0) return;
    // the count pass zeroes the entry after the last row: the scan's total lands there
    if (!FILL && blockIdx.x == 0 && threadIdx.x == 0) a.counts[a.n_atoms] = 0;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nwarps = gridDim.x * NBR_WARPS;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int i = blockIdx.x * NBR_WARPS + wib; i < a.n_atoms; i += nwarps) {
        const int m = a.atom_mol[i];
        const float4 pi = a.pos4[i];
        const Box b = load_box(a.box, a.pbc, m);
        int cnt = 0;
        const int base = FILL ? a.counts[i] : 0;
        const bool open_cells = !b.periodic && a.mol_ptr[m + 1] - a.mol_ptr[m] >= OPEN_CELL_MIN;
        if (!b.periodic && !open_cells) {
            const int a0 = (int)a.mol_ptr[m], a1 = (int)a.mol_ptr[m + 1];
            for (int j0 = a0; j0 < a1; j0 += 32) {
                const int j = j0 + lane;
                bool ok = false;
                if (j < a1 && j != i) {
                    float4 pj = a.pos4[j];
                    float3 r = edge_vector(pj, pi, b);
                    ok = pair_distance(r.x, r.y, r.z) <= a.cutoff;
                }
                const unsigned mask = __ballot_sync(0xffffffffu, ok);
                if (FILL && ok) {
                    int64_t p = (int64_t)base + cnt + __popc(mask & lt_mask);
                    a.col[p] = j;
                    a.erecv[p] = i;
                }
                cnt += __popc(mask);
            }
        } else {
            const int4 g = a.grid[m];
            // the row atom's cell, computed as the binning did
            int cc[3];
            if (open_cells) {
                const float4 lo = a.mol_box[2 * m], iw = a.mol_box[2 * m + 1];
                cc[0] = open_cell_coord(pi.x, lo.x, iw.x, g.x);
                cc[1] = open_cell_coord(pi.y, lo.y, iw.y, g.y);
                cc[2] = open_cell_coord(pi.z, lo.z, iw.z, g.z);
            } else {
                cc[0] = cell_coord(pi.x, b.L[0], b.invL[0], g.x);
                cc[1] = cell_coord(pi.y, b.L[1], b.invL[1], g.y);
                cc[2] = cell_coord(pi.z, b.L[2], b.invL[2], g.z);
            }
            const int ncs[3] = {g.x, g.y, g.z};
            const int bits[3] = {cell_bits(g.x), cell_bits(g.y), cell_bits(g.z)};
            bool overflow = false;
            // lane k < 27 looks up neighbour cell (k / 9, k / 3 % 3, k % 3) - 1 (wrapped); on an
            // axis with fewer than 3 cells the offsets 0 .. nc-1 name its cells directly; an open
            // grid does not wrap (cells outside it are skipped)
            int c0 = 0, len = 0;
            if (lane < 27) {
                const int o[3] = {lane / 9, (lane / 3) % 3, lane % 3};
                bool keep = true;
                int q[3];
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) {
                    if (open_cells) {
                        q[ax] = cc[ax] + o[ax] - 1;
                        keep = keep && q[ax] >= 0 && q[ax] < ncs[ax];
                    } else if (ncs[ax] >= 3) {
                        q[ax] = (cc[ax] + o[ax] - 1 + ncs[ax]) % ncs[ax];
                    } else {
                        keep = keep && o[ax] < ncs[ax];
                        q[ax] = o[ax];
                    }
                }
                if (keep) {
                    const int qc = g.w + morton3(q[0], q[1], q[2], bits[0], bits[1], bits[2]);
                    c0 = a.cell_start[qc];
                    len = a.cell_start[qc + 1] - c0;
                }
            }
            int incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int excl = incl - len;
            for (int t = 0; t < total; t += 32) {
                const int c = t + lane;
                // cell of candidate c: the number of lanes whose cells end at or before c
                int k = 0;
#pragma unroll
                for (int bit = 16; bit > 0; bit >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, incl, k + bit - 1);
                    if (v <= c) k += bit;
                }
                const int kb = __shfl_sync(0xffffffffu, c0, k);
                const int ke = __shfl_sync(0xffffffffu, excl, k);
                bool ok = false;
                int j = -1;
                if (c < total) {
                    const float4 pj = a.cell_pos[kb + c - ke];
                    j = __float_as_int(pj.w);
                    if (j != i) {
                        float3 r = edge_vector(pj, pi, b);
                        ok = pair_distance(r.x, r.y, r.z) <= a.cutoff;
                    }
                }
                const unsigned mask = __ballot_sync(0xffffffffu, ok);
                if (FILL) {
                    const int slot = cnt + __popc(mask & lt_mask);
                    if (ok && slot < ROW_CAP) sbuf[wib][slot] = j;
                }
                cnt += __popc(mask);
            }
            if (cnt > ROW_CAP) overflow = true;
            if (FILL) {
                __syncwarp();
                if (overflow) {
                    if (lane == 0) set_status(a.st, MLFF_ERR_ROW, i);
                } else {
                    // rank sort: neighbour indices in a row are distinct
                    for (int k = lane; k < cnt; k += 32) {
                        const int v = sbuf[wib][k];
                        int rank = 0;
                        for (int q2 = 0; q2 < cnt; ++q2) rank += sbuf[wib][q2] < v ? 1 : 0;
                        int64_t p = (int64_t)base + rank;
                        a.col[p] = v;
                        a.erecv[p] = i;
                    }
                }
                __syncwarp();
            }
        }
        if (!FILL && lane == 0) a.counts[i] = cnt;
    }
}

__global__ void check_edges_kernel(const int32_t* __restrict__ row_ptr, int32_t n_atoms, int64_t cap, Status* st) {
    pdl_wait();
    pdl_trigger();
    int64_t e = (int64_t)(uint32_t)row_ptr[n_atoms];
    st->n_edges = (int32_t)(e & 0x7fffffff);
    st->n_edges_hi = (int32_t)(e >> 31);
    if (e > cap) set_status(st, MLFF_ERR_CAPACITY, -1);
}

// rev[k]: position of the reversed edge (row b, col a) for edge k = (row a, col b)
__global__ void rev_kernel(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                           const int32_t* __restrict__ erecv, int32_t n_atoms,
                           int32_t* __restrict__ rev, Status* st) {
    pdl_wait();
    pdl_trigger();
    if (st->code != 0) return;
    const int32_t E = row_ptr[n_atoms];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < E; k += gridDim.x * blockDim.x) {
        const int a = erecv[k], b = col[k];
        int lo = row_ptr[b], hi = row_ptr[b + 1] - 1, found = -1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            int v = col[mid];
            if (v == a) { found = mid; break; }
            if (v < a) lo = mid + 1; else hi = mid - 1;
        }
        if (found < 0) set_status(st, MLFF_ERR_INVALID, k);
        rev[k] = found < 0 ? k : found;
    }
}

// receiver partition for the persistent edge kernels: part[p] is the first
// receiver whose row starts at or after p*E/P
__global__ void partition_kernel(const int32_t* __restrict__ row_ptr, int32_t n_atoms, int32_t P,
                                 int32_t* __restrict__ part) {
    pdl_wait();
    pdl_trigger();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > P) return;
    const int64_t E = row_ptr[n_atoms];
    if (p == 0) { part[0] = 0; return; }
    if (p == P) { part[P] = n_atoms; return; }
    const int64_t target = (E * p + P - 1) / P;
    int lo = 0, hi = n_atoms;   // first a with row_ptr[a] >= target
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (row_ptr[mid] >= target) hi = mid; else lo = mid + 1;
    }
    part[p] = lo;
}

int launch_partition(const WsLayout& L, void* ws, cudaStream_t st) {
    ProfScope prof(PK_NEIGHBORS, st);
    MLFF_LAUNCH_PDL("partition", partition_kernel, (L.P + 1 + 255) / 256, 256, 0, st, ws_ptr<int32_t>(ws, L.row_ptr), L.N, L.P,
                                                            ws_ptr<int32_t>(ws, L.part));
    return MLFF_OK;
}

// Exclusive scan of data[0..n_in) with the total written to data[n_in]
// (which must hold 0 for the multi-block form); with st the total is the
// edge count, recorded and checked against cap.  With n_dev the count is
// read on the device (at most n_in) and one block scans it.
static int scan_with_total(int32_t* data, int64_t n_in, int32_t* tmp, Status* st, int64_t cap, cudaStream_t s,
                           const int32_t* n_dev = nullptr) {
    if (n_in + 1 <= SCAN1_MAX || n_dev) {
        MLFF_LAUNCH_PDL("scan_single", scan_single_kernel, 1, 1024, 0, s, data, n_in, n_dev, st, cap);
        return MLFF_OK;
    }
    int r = launch_scan(data, n_in + 1, tmp, s);
    if (r) return r;
    if (st) MLFF_LAUNCH_PDL("check_edges", check_edges_kernel, 1, 1, 0, s, data, (int32_t)n_in, cap, st);
    return MLFF_OK;
}

// Radius graph into explicit buffers: atom copies, cell lists (periodic
// structures), row counts, their scan (row_ptr) and the rank-sorted rows.
int launch_neighbors_into(const mlff_dims& d, const mlff_system& sys, const NbrBuffers& b, cudaStream_t st) {
    const int N = sys.n_atoms;
    const bool any_pbc = sys.pbc != nullptr && sys.box != nullptr;
    // an open structure of OPEN_CELL_MIN atoms or more needs at least that many atoms in all
    const bool any_open_cells = N >= OPEN_CELL_MIN;
    const int tb = 256;
    const int gb = (int)std::max<int64_t>(1, std::min<int64_t>((N + tb - 1) / tb, 152 * 16));
    MLFF_LAUNCH_PDL("prep_atoms", prep_atoms_kernel, gb, tb, 0, st, sys.pos, sys.mol_ptr, sys.n_mol, N, b.pos4,
                    b.atom_mol);
    if (any_pbc || any_open_cells) {
        if (any_open_cells) {
            const int mb = std::max(1, std::min(sys.n_mol, 152 * 8));
            MLFF_LAUNCH_PDL("mol_bbox", mol_bbox_kernel, mb, 256, 0, st, b.pos4, sys.mol_ptr, sys.pbc, sys.box,
                            sys.n_mol, b.mol_box);
        }
        MLFF_LAUNCH_PDL("mol_grid", mol_grid_kernel, 1, 1024, 0, st, sys.mol_ptr, sys.box, sys.pbc, sys.n_mol, d.cutoff,
                        b.mol_grid, b.mol_box, b.cell_count, b.cell_fill, b.ncell_cap, b.status);
        MLFF_LAUNCH_PDL("cell_count", cell_count_kernel, gb, tb, 0, st, b.pos4, b.atom_mol, sys.mol_ptr, sys.box,
                        sys.pbc, b.mol_grid, b.mol_box, N, b.atom_cell, b.cell_count);
        // the cell codes in use (grid[n_mol].x, at most ncell_cap), scanned by one block
        int r = scan_with_total(b.cell_count, b.ncell_cap, b.scan_tmp, nullptr, 0, st,
                                reinterpret_cast<const int32_t*>(b.mol_grid + sys.n_mol));
        if (r) return r;
        MLFF_LAUNCH_PDL("cell_fill", cell_fill_kernel, gb, tb, 0, st, b.atom_cell, b.cell_count, b.pos4, N, b.cell_fill,
                        b.cell_pos);
    }
    NbrArgs a;
    a.pos4 = b.pos4; a.atom_mol = b.atom_mol; a.mol_ptr = sys.mol_ptr; a.box = sys.box; a.pbc = sys.pbc;
    a.grid = b.mol_grid; a.mol_box = b.mol_box; a.cell_start = b.cell_count; a.cell_pos = b.cell_pos;
    a.n_atoms = N; a.cutoff = d.cutoff; a.cap = b.cap; a.counts = b.row_ptr;
    a.col = b.col; a.erecv = b.erecv; a.st = b.status;
    const int rows_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((N + NBR_WARPS - 1) / NBR_WARPS, 152 * 32));
    MLFF_LAUNCH_PDL("nbr_count", nbr_rows_kernel<false>, rows_blocks, NBR_WARPS * 32, 0, st, a);
    int r = scan_with_total(b.row_ptr, N, b.scan_tmp, b.status, b.cap, st);
    if (r) return r;
    MLFF_LAUNCH_PDL("nbr_fill", nbr_rows_kernel<true>, rows_blocks, NBR_WARPS * 32, 0, st, a);
    return MLFF_OK;
}

int launch_neighbors(const mlff_dims& d, const mlff_system& sys, const WsLayout& L, void* ws,
                     cudaStream_t st) {
    ProfScope prof(PK_NEIGHBORS, st);
    NbrBuffers b;
    b.status = ws_ptr<Status>(ws, L.status);
    b.pos4 = ws_ptr<float4>(ws, L.pos4);
    b.atom_mol = ws_ptr<int32_t>(ws, L.atom_mol);
    b.row_ptr = ws_ptr<int32_t>(ws, L.row_ptr);
    b.col = ws_ptr<int32_t>(ws, L.col);
    b.erecv = ws_ptr<int32_t>(ws, L.erecv);
    b.scan_tmp = ws_ptr<int32_t>(ws, L.scan_tmp);
    b.mol_grid = ws_ptr<int4>(ws, L.mol_grid);
    b.mol_box = ws_ptr<float4>(ws, L.mol_box);
    b.cell_count = ws_ptr<int32_t>(ws, L.cell_count);
    b.cell_fill = ws_ptr<int32_t>(ws, L.cell_fill);
    b.cell_pos = ws_ptr<float4>(ws, L.cell_pos);
    b.atom_cell = ws_ptr<int32_t>(ws, L.atom_cell);
    b.ncell_cap = L.ncell_cap;
    b.cap = L.cap;
    int r = launch_neighbors_into(d, sys, b, st);
    if (r) return r;
    const int eb = (int)std::min<int64_t>((L.cap + 255) / 256, 152 * 16);
    MLFF_LAUNCH_PDL("rev", rev_kernel, std::max(eb, 1), 256, 0, st, b.row_ptr, b.col, b.erecv, sys.n_atoms,
                    ws_ptr<int32_t>(ws, L.rev), b.status);
    return MLFF_OK;
}

}  // namespace mlff
