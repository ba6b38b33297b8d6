// Force-accuracy statistics on the device (the reference's
// testing/force_metrics.py:46-384 computed over predicted and reference
// force vectors without copying them to the host).  One pass over the
// vectors gives the sums every metric needs, reduced in a fixed order (the
// result does not depend on timing), and optionally the per-vector errors
// (RMSE and MAE over the three components, magnitude error, angle).
#include <cmath>
#include "common.cuh"
#include "profile.h"

namespace mlff {

constexpr int FS_NT = 256;
constexpr int FS_BLOCKS = 256;
constexpr int FS_N = MLFF_FORCE_STATS;   // quantities, see the header
constexpr double FS_MIN_MAG = 1e-6;      // force_metrics.py: magnitudes below this have no direction

__device__ __forceinline__ void fs_accumulate(const double* p, const double* r, double* acc, double* per_vec,
                                              int64_t i) {
    double d2 = 0.0, da = 0.0, pm2 = 0.0, rm2 = 0.0, dot = 0.0;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double d = p[q] - r[q];
        acc[1 + q] += d * d;
        acc[4 + q] += fabs(d);
        d2 += d * d;
        da += fabs(d);
        pm2 += p[q] * p[q];
        rm2 += r[q] * r[q];
        dot += p[q] * r[q];
        acc[13] += p[q];
        acc[14] += r[q];
        acc[15] += p[q] * p[q];
        acc[16] += r[q] * r[q];
        acc[17] += p[q] * r[q];
        acc[18] = fmax(acc[18], fabs(d));
    }
    const double pm = sqrt(pm2), rm = sqrt(rm2), dm = pm - rm;
    acc[0] += 1.0;
    acc[7] += dm * dm;
    acc[8] += fabs(dm);
    if (rm > FS_MIN_MAG) {
        acc[9] += fabs(dm) / rm;
        acc[10] += 1.0;
    }
    double ang = NAN;
    if (pm > FS_MIN_MAG && rm > FS_MIN_MAG) {
        const double c = dot / (pm * rm);
        acc[11] += 1.0;
        acc[12] += c;
        ang = acos(fmin(1.0, fmax(-1.0, c))) * (180.0 / 3.14159265358979323846);
    }
    if (per_vec) {
        double* o = per_vec + 4 * i;
        o[0] = sqrt(d2 / 3.0);
        o[1] = da / 3.0;
        o[2] = fabs(dm);
        o[3] = ang;
    }
}

// block b takes vectors b, b + FS_BLOCKS, ... (fixed assignment); partial
// sums of its threads combined in a fixed tree
__global__ void __launch_bounds__(FS_NT) force_stats_kernel(const double* __restrict__ pred,
                                                            const double* __restrict__ ref, int64_t n,
                                                            double* __restrict__ part, double* __restrict__ per_vec) {
    __shared__ double red[FS_N][FS_NT];
    double acc[FS_N];
#pragma unroll
    for (int j = 0; j < FS_N; ++j) acc[j] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)FS_NT + threadIdx.x; i < n; i += (int64_t)FS_BLOCKS * FS_NT)
        fs_accumulate(pred + 3 * i, ref + 3 * i, acc, per_vec, i);
#pragma unroll
    for (int j = 0; j < FS_N; ++j) red[j][threadIdx.x] = acc[j];
    __syncthreads();
    for (int o = FS_NT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
#pragma unroll
            for (int j = 0; j < FS_N; ++j)
                red[j][threadIdx.x] = j == 18 ? fmax(red[j][threadIdx.x], red[j][threadIdx.x + o])
                                              : red[j][threadIdx.x] + red[j][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < FS_N) part[blockIdx.x * FS_N + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void force_stats_sum_kernel(const double* __restrict__ part, double* __restrict__ out) {
    const int j = threadIdx.x;
    if (j >= FS_N) return;
    double s = 0.0;
    for (int b = 0; b < FS_BLOCKS; ++b) s = j == 18 ? fmax(s, part[b * FS_N + j]) : s + part[b * FS_N + j];
    out[j] = s;
}

}  // namespace mlff

using namespace mlff;

extern "C" {

size_t mlff_force_stats_workspace_size(void) { return sizeof(double) * FS_BLOCKS * FS_N; }

int mlff_force_stats(const double* pred, const double* ref, int64_t n_vectors, double* stats, double* per_vector,
                     void* workspace, size_t workspace_bytes, mlff_stream_t stream) {
    if (!pred || !ref || !stats || !workspace || n_vectors < 0) {
        set_error("force_stats: pred, ref, stats and workspace are required, n_vectors >= 0");
        return MLFF_ERR_INVALID;
    }
    if (workspace_bytes < mlff_force_stats_workspace_size()) {
        set_error("workspace %zu bytes < %zu needed", workspace_bytes, mlff_force_stats_workspace_size());
        return MLFF_ERR_WORKSPACE;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    double* part = static_cast<double*>(workspace);
    force_stats_kernel<<<FS_BLOCKS, FS_NT, 0, st>>>(pred, ref, n_vectors, part, per_vector);
    MLFF_LAUNCH_CHECK("force_stats");
    force_stats_sum_kernel<<<1, 32, 0, st>>>(part, stats);
    MLFF_LAUNCH_CHECK("force_stats_sum");
    return MLFF_OK;
}

}  // extern "C"
