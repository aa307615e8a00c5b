// sort.cuh -- device layout of the per-cell sort arrays (sort.cu).
#pragma once
#include <cuda_runtime.h>

namespace sphgpu {

// One non-empty cell of the tree.
struct SortCell {
  long long off;   // first entry of its 13 arrays (axis j at off + j * (count + 1))
  int first;       // first particle (cell-sorted order)
  int count;
  int progeny[8];  // SortCell index of each child, -1 where none
};

struct SortTree {
  const SortCell* cells;
  const int* leaves;     // SortCell indices of the leaves
  int nleaves;
  const int* g_of_s;     // cell-sorted index -> store index
  const double* xd;      // positions, store order
  float* d;              // keys
  int* i;                // indices within the cell
};

// Leaf sorts, then the merges of the split cells of each depth, deepest
// first (split_by_depth[k]: SortCell indices of the split cells of depth k).
cudaError_t launch_hydro_sort(const SortTree& t, const int* const* split_by_depth,
                              const int* n_by_depth, int max_depth, int flags,
                              cudaStream_t s);

}  // namespace sphgpu
