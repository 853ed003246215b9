// Deterministic sort-based mass assignment (sorted.cu), used by mas.cu for
// PYL_STRATEGY_SORTED.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace pyl {

// dims^3 <= 2^32 cells and fewer than 2^32 particles.
bool sorted_supported(long long n, int dims);

// Workspace bytes of the sorted strategy (keys, values, digit histograms,
// per-cell runs, positions in sorted order).
size_t sorted_workspace_bytes(long long n, int dims);

// Deposits n particles into grid (and the half-cell-shifted grid2 when non-null).
// fold: add to the existing grid values in a fixed order (MA); otherwise add
// scale * (cell sum) to the grid (scale from *scale_d when non-null).
int launch_sorted(int mas, const float *pos, const float *w, long long n, float *grid, float *grid2, int dims,
                  float inv, float halfcell, void *workspace, float scale_h, const float *scale_d, bool fold,
                  cudaStream_t st);

}  // namespace pyl
