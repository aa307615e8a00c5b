// drift.cu -- a space's particles moved without a rebuild.
//
// Between two rebuilds the reference keeps every particle in the cell the
// rebuild gave it and tracks how far it has moved since (cell_drift.c:330-382:
// x_diff, dx_max_part = sqrtf of the largest squared motion, h_max); the
// recursions add dx_max_part to their cut-off (cell.h:934-1010) and a pair of
// neighbouring top-level cells needs a rebuild once
//   kernel_gamma max(h_max_i, h_max_j) + dx_max_part_i + dx_max_part_j > dmin
// (cell_need_rebuild_for_hydro_pair, cell.h:1237).  Here the motion is
// measured against the rebuild's positions in one step (x_rebuild - x_new
// rounded to FP32 per component), every operation rounded on its own.
#include <algorithm>

#include "devplan.cuh"
#include "device_sms.h"
#include "sph_kernels.cuh"

namespace sphgpu {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kRun = 8;  // particles per run of a j-block (the host build's kSubBlock)

int grid_for(long long n) {
  return (int)std::max(1LL, std::min((n + 255) / 256, 8LL * sm_count()));
}

int leaf_blocks(int nleaves) {
  return std::max(1, std::min((nleaves + 7) / 8, 16 * sm_count()));
}

__global__ void drift_reset(unsigned* dxn, unsigned* hmx, int ncells) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
    dxn[c] = 0u;
    hmx[c] = 0u;
  }
}

// One warp per leaf: the leaf's largest squared motion and largest new h,
// then an atomic maximum into every ancestor (dx_max as sqrtf of the leaf's
// largest square: the maximum over progeny of the same root, cell_drift.c:222).
__global__ void __launch_bounds__(256) drift_cells_k(DPTree t, const int32_t* __restrict__ perm,
                                                     const double* __restrict__ xn,
                                                     const double* __restrict__ xr,
                                                     const float* __restrict__ hn,
                                                     unsigned* dxn, unsigned* hmx) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  for (int l = warp; l < t.nleaves; l += nwarps) {
    const int L = t.leaf_cell[l];
    const int first = t.cell[L].first, count = t.cell[L].count;
    unsigned d2 = 0u, hm = 0u;
    for (int i = first + lane; i < first + count; i += 32) {
      const size_t k = (size_t)perm[i];
      const float ax = (float)(xr[3 * k] - xn[3 * k]);
      const float ay = (float)(xr[3 * k + 1] - xn[3 * k + 1]);
      const float az = (float)(xr[3 * k + 2] - xn[3 * k + 2]);
      const float dx2 = __fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az));
      d2 = max(d2, __float_as_uint(dx2));
      hm = max(hm, __float_as_uint(hn[k]));
    }
    d2 = __reduce_max_sync(kFull, d2);
    hm = __reduce_max_sync(kFull, hm);
    if (lane == 0) {
      const unsigned dx = __float_as_uint(sqrtf(__uint_as_float(d2)));
      for (int c = L; c >= 0; c = t.cell[c].parent) {
        atomicMax(&dxn[c], dx);
        atomicMax(&hmx[c], hm);
      }
    }
  }
}

__global__ void drift_check_k(DPTree t, const unsigned* __restrict__ dxn,
                              const unsigned* __restrict__ hmx, int ntasks, int* flag) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ntasks; q += gridDim.x * blockDim.x) {
    const int2 tk = t.task[q];
    if (tk.y < 0) continue;
    const float hm = fmaxf(__uint_as_float(hmx[tk.x]), __uint_as_float(hmx[tk.y]));
    const float r = __fadd_rn(__fadd_rn(__fmul_rn(SPH_KG, hm), __uint_as_float(dxn[tk.x])),
                              __uint_as_float(dxn[tk.y]));
    if (r > t.cell[tk.y].dmin) atomicExch(flag, 1);
  }
}

__global__ void drift_commit_k(DevParticles P, double* __restrict__ xd, int8_t* __restrict__ dh0,
                               const int32_t* __restrict__ perm,
                               const double* __restrict__ xn, const float* __restrict__ hn,
                               const int32_t* __restrict__ top_of,
                               const double* __restrict__ top_loc,
                               const LeafInfo* __restrict__ leaves) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
    const size_t k = (size_t)perm[i];
    const int t = top_of[i];
    double x[3];
    float4 q;
    for (int d = 0; d < 3; d++) {
      x[d] = xn[3 * k + d];
      xd[3 * (size_t)i + d] = x[d];
    }
    q.x = __double2float_rn(x[0] - top_loc[3 * t + 0]);
    q.y = __double2float_rn(x[1] - top_loc[3 * t + 1]);
    q.z = __double2float_rn(x[2] - top_loc[3 * t + 2]);
    const float h = hn[k];
    q.w = h;
    P.posh[i] = q;
    P.h0[i] = h;
    // cell_set_part_h_depth (cell.h:1787) on the leaf chain: depth_h keeps
    // its value when h is above every level; the step's starting depth (the
    // host's h_depth_of) is 0 there
    const LeafInfo* L = &leaves[P.leaf_of[i]];
    int dnow = P.depth_h[i], d0 = 0;
    if (h < L->hmin[0]) {
      dnow = d0 = L->depth[0];
    } else {
      for (int lev = 0; lev < L->nlevels; lev++)
        if (h >= L->hmin[lev] && h < L->hmax[lev]) {
          dnow = d0 = L->depth[lev];
          break;
        }
    }
    P.depth_h[i] = (int8_t)dnow;
    dh0[i] = (int8_t)d0;
  }
}

__global__ void block_boxes_k(const int2* __restrict__ fc, const float4* __restrict__ posh,
                              float4* lo, float4* hi, float4* slo, float4* shi, int nblocks) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += gridDim.x * blockDim.x) {
    const int2 r = fc[b];
    float3 l = make_float3(3.4e38f, 3.4e38f, 3.4e38f), h = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
    for (int q = 0; q < 4; q++) {
      float3 sl = make_float3(3.4e38f, 3.4e38f, 3.4e38f),
             sh = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
      const int k0 = r.x + q * kRun, k1 = min(r.x + r.y, k0 + kRun);
      for (int k = k0; k < k1; k++) {
        const float4 p = posh[k];
        sl = make_float3(fminf(sl.x, p.x), fminf(sl.y, p.y), fminf(sl.z, p.z));
        sh = make_float3(fmaxf(sh.x, p.x), fmaxf(sh.y, p.y), fmaxf(sh.z, p.z));
      }
      slo[4 * b + q] = make_float4(sl.x, sl.y, sl.z, 0.f);
      shi[4 * b + q] = make_float4(sh.x, sh.y, sh.z, 0.f);
      l = make_float3(fminf(l.x, sl.x), fminf(l.y, sl.y), fminf(l.z, sl.z));
      h = make_float3(fmaxf(h.x, sh.x), fmaxf(h.y, sh.y), fmaxf(h.z, sh.z));
    }
    // .w of lo is the force's block radius (block_hmax), kept
    const float w = lo[b].w;
    lo[b] = make_float4(l.x, l.y, l.z, w);
    hi[b] = make_float4(h.x, h.y, h.z, 0.f);
  }
}

}  // namespace

cudaError_t launch_drift_cells(const DPTree& t, const int32_t* perm, const double* x_new,
                               const double* x_rebuild, const float* h_new, unsigned* dxn,
                               unsigned* hmx, cudaStream_t st) {
  drift_reset<<<grid_for(t.ncells), 256, 0, st>>>(dxn, hmx, t.ncells);
  drift_cells_k<<<leaf_blocks(t.nleaves), 256, 0, st>>>(t, perm, x_new, x_rebuild, h_new, dxn,
                                                        hmx);
  return cudaGetLastError();
}

cudaError_t launch_drift_check(const DPTree& t, const unsigned* dxn, const unsigned* hmx,
                               int* flag, cudaStream_t st) {
  drift_check_k<<<grid_for(t.ntasks), 256, 0, st>>>(t, dxn, hmx, t.ntasks, flag);
  return cudaGetLastError();
}

cudaError_t launch_drift_commit(const DevParticles& P, double* xd, int8_t* depth_h0,
                                const int32_t* perm, const double* x_new, const float* h_new,
                                const int32_t* top_of, const double* top_loc,
                                const LeafInfo* leaves, cudaStream_t st) {
  drift_commit_k<<<grid_for(P.n), 256, 0, st>>>(P, xd, depth_h0, perm, x_new, h_new, top_of,
                                                top_loc, leaves);
  return cudaGetLastError();
}

cudaError_t launch_block_boxes(const int2* fc, const float4* posh, float4* lo, float4* hi,
                               float4* sub_lo, float4* sub_hi, int nblocks, cudaStream_t st) {
  block_boxes_k<<<grid_for(nblocks), 256, 0, st>>>(fc, posh, lo, hi, sub_lo, sub_hi, nblocks);
  return cudaGetLastError();
}

}  // namespace sphgpu
