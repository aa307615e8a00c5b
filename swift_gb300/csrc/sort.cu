// sort.cu -- the per-cell sort arrays of runner_do_hydro_sort
// (runner_sort.c:203-463) for the whole tree, on the device.
//
// For every non-empty cell and every requested axis j of the 13 (bit j of
// flags) the cell holds count + 1 entries {d, i}: d = (float)(x . axis_j)
// of the cell's particles in their cell-sorted order, i their index in the
// cell, ascending in d, then a sentinel {FLT_MAX, 0}.  Ties keep the order
// the reference's algorithms leave them in, so the algorithms are the
// reference's: leaves are sorted by its quicksort (explicit stack, middle
// pivot, selection sort below 16 elements), and a split cell merges its
// progeny's arrays with its 8-way merge (strict comparisons), deepest cells
// first.  One thread handles one (cell, axis) array.  The key is evaluated
// with explicitly rounded double operations in the reference's order, then
// rounded to float, so it is bit-identical to the reference's.
#include <cuda_runtime.h>

#include <cfloat>

#include "sort.cuh"

namespace sphgpu {

namespace {

// Unit vectors of the 13 sort axes: the decimal literals of the reference's
// table (sort_part.h:42-57).
#define SORT_S3 5.773502691896258e-01
#define SORT_S2 7.071067811865475e-01
__constant__ double c_axis[13][3] = {
    {SORT_S3, SORT_S3, SORT_S3},   {SORT_S2, SORT_S2, 0.0},   {SORT_S3, SORT_S3, -SORT_S3},
    {SORT_S2, 0.0, SORT_S2},       {1.0, 0.0, 0.0},           {SORT_S2, 0.0, -SORT_S2},
    {SORT_S3, -SORT_S3, SORT_S3},  {SORT_S2, -SORT_S2, 0.0},  {SORT_S3, -SORT_S3, -SORT_S3},
    {0.0, SORT_S2, SORT_S2},       {0.0, 1.0, 0.0},           {0.0, SORT_S2, -SORT_S2},
    {0.0, 0.0, 1.0}};

__device__ void quicksort(float* d, int* id, int n) {
  int lo_s[64], hi_s[64];
  int q = 0;
  lo_s[0] = 0;
  hi_s[0] = n - 1;
  while (q >= 0) {
    const int lo = lo_s[q], hi = hi_s[q];
    q--;
    if (hi - lo < 15) {
      for (int i = lo; i < hi; i++) {
        int imin = i;
        for (int j = i + 1; j <= hi; j++)
          if (d[j] < d[imin]) imin = j;
        if (imin != i) {
          const float td = d[imin];
          const int ti = id[imin];
          d[imin] = d[i];
          id[imin] = id[i];
          d[i] = td;
          id[i] = ti;
        }
      }
    } else {
      const float pivot = d[(lo + hi) / 2];
      int i = lo, j = hi;
      while (i <= j) {
        while (d[i] < pivot) i++;
        while (d[j] > pivot) j--;
        if (i <= j) {
          if (i < j) {
            const float td = d[i];
            const int ti = id[i];
            d[i] = d[j];
            id[i] = id[j];
            d[j] = td;
            id[j] = ti;
          }
          i++;
          j--;
        }
      }
      // the larger part goes on the stack first, as in the reference
      if (j > (lo + hi) / 2) {
        if (lo < j) { q++; lo_s[q] = lo; hi_s[q] = j; }
        if (i < hi) { q++; lo_s[q] = i; hi_s[q] = hi; }
      } else {
        if (i < hi) { q++; lo_s[q] = i; hi_s[q] = hi; }
        if (lo < j) { q++; lo_s[q] = lo; hi_s[q] = j; }
      }
    }
  }
}

__global__ void sort_leaves(SortTree t, int flags) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= 13LL * t.nleaves) return;
  const int axis = (int)(tid % 13);
  if (!(flags & (1 << axis))) return;
  const SortCell c = t.cells[t.leaves[tid / 13]];
  float* d = t.d + c.off + (long long)axis * (c.count + 1);
  int* id = t.i + c.off + (long long)axis * (c.count + 1);
  const double a0 = c_axis[axis][0], a1 = c_axis[axis][1], a2 = c_axis[axis][2];
  for (int k = 0; k < c.count; k++) {
    const int g = t.g_of_s[c.first + k];
    const double* x = t.xd + 3 * (size_t)g;
    const double dd = __dadd_rn(__dadd_rn(__dmul_rn(x[0], a0), __dmul_rn(x[1], a1)),
                                __dmul_rn(x[2], a2));
    d[k] = __double2float_rn(dd);
    id[k] = k;
  }
  d[c.count] = FLT_MAX;
  id[c.count] = 0;
  quicksort(d, id, c.count);
}

__global__ void sort_merge(SortTree t, const int* __restrict__ split_cells, int n, int flags) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= 13LL * n) return;
  const int axis = (int)(tid % 13);
  if (!(flags & (1 << axis))) return;
  const SortCell c = t.cells[split_cells[tid / 13]];
  int off[8];
  off[0] = 0;
  for (int k = 1; k < 8; k++)
    off[k] = off[k - 1] + (c.progeny[k - 1] >= 0 ? t.cells[c.progeny[k - 1]].count : 0);
  long long fing[8];
  float buff[8];
  int inds[8];
  for (int k = 0; k < 8; k++) {
    inds[k] = k;
    fing[k] = -1;
    buff[k] = FLT_MAX;
    if (c.progeny[k] >= 0) {
      const SortCell p = t.cells[c.progeny[k]];
      if (p.count > 0) {
        fing[k] = p.off + (long long)axis * (p.count + 1);
        buff[k] = t.d[fing[k]];
      }
    }
  }
  for (int i = 0; i < 7; i++)
    for (int k = i + 1; k < 8; k++)
      if (buff[inds[k]] < buff[inds[i]]) {
        const int tmp = inds[i];
        inds[i] = inds[k];
        inds[k] = tmp;
      }
  float* d = t.d + c.off + (long long)axis * (c.count + 1);
  int* id = t.i + c.off + (long long)axis * (c.count + 1);
  for (int ind = 0; ind < c.count; ind++) {
    const int s = inds[0];
    d[ind] = buff[s];
    id[ind] = t.i[fing[s]] + off[s];
    fing[s] += 1;
    buff[s] = t.d[fing[s]];  // the progeny's sentinel once it is used up
    for (int k = 1; k < 8 && buff[inds[k]] < buff[inds[k - 1]]; k++) {
      const int tmp = inds[k - 1];
      inds[k - 1] = inds[k];
      inds[k] = tmp;
    }
  }
  d[c.count] = FLT_MAX;
  id[c.count] = 0;
}

int blocks_for(long long n) { return (int)((n + 127) / 128); }

}  // namespace

cudaError_t launch_hydro_sort(const SortTree& t, const int* const* split_by_depth,
                              const int* n_by_depth, int max_depth, int flags,
                              cudaStream_t s) {
  if (t.nleaves > 0) {
    sort_leaves<<<blocks_for(13LL * t.nleaves), 128, 0, s>>>(t, flags);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  for (int dep = max_depth; dep >= 0; dep--) {
    if (n_by_depth[dep] == 0) continue;
    sort_merge<<<blocks_for(13LL * n_by_depth[dep]), 128, 0, s>>>(t, split_by_depth[dep],
                                                                    n_by_depth[dep], flags);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace sphgpu
