// Optional kernel timing for benchmarks: while enabled, launch sites
// bracket kernel groups with CUDA events on the launching stream and count
// launches.  Disabled (the default) it costs one branch per launch site.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mlff {

enum ProfKind {
    PK_NEIGHBORS = 0,
    PK_EDGE_FWD = 1,
    PK_EDGE_BWD = 2,
    PK_UPDATE_FWD = 3,
    PK_UPDATE_BWD = 4,
    PK_READOUT = 5,
    PK_FORCES = 6,
    PK_PLAIN_GEMM = 7,
    PK_PLAIN_EDGE = 8,
    PK_OTHER = 9,
    PK_MD = 10,
    PK_EDGE_BWD_Q = 11,   // per-atom Q rows of the reverse tensor-core edge kernel
    PK_COUNT = 12
};

bool prof_enabled();
void prof_launch(int kind, int n = 1);      // count kernel launches

struct ProfScope {
    int kind;
    int prev_kind;
    cudaStream_t st;
    int slot;
    ProfScope(int kind, cudaStream_t st);
    ~ProfScope();
};

}  // namespace mlff
