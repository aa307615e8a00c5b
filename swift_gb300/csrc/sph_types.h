// sph_types.h -- data layout shared by the host planner (space.cpp) and the
// sm_103a kernels (sph_kernels.cu).
//
// Particles live in HBM as structure-of-arrays in the cell-sorted order of
// the reference's space build (every cell, at every tree level, is one
// contiguous index range).  Positions are kept in FP64 for the exact
// neighbour predicate and, for the arithmetic, as FP32 offsets from the
// particle's top-level cell corner (the reference's cell-relative frames,
// runner_doiact_functions_hydro.h:1327-1346).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define SPH_HD __host__ __device__
#else
#define SPH_HD
#endif

namespace sphgpu {

// Scheme constants, evaluated the way kernel_hydro.h / dimension.h /
// adiabatic_index.h evaluate them (float products, double divisions).
#define SPH_KG ((float)(1.936492))
#define SPH_KCONST ((float)(21. * 0.31830988618379067154 / 2.))
#define SPH_KG_INV ((float)(1. / SPH_KG))
#define SPH_KG2 ((float)(SPH_KG * SPH_KG))
#define SPH_KG_INV_DIM ((float)(1. / (SPH_KG * SPH_KG * SPH_KG)))
#define SPH_KG_INV_DIM1 ((float)(1. / (SPH_KG * SPH_KG * SPH_KG * SPH_KG)))
#define SPH_KROOT ((float)(1.f) * SPH_KCONST * SPH_KG_INV_DIM)
#define SPH_HDIM 3.f
#define SPH_HDIM_INV 0.3333333333f
#define SPH_GAMMA 1.66666666666666667f
#define SPH_GAMMA_M1 0.66666666666666667f
#define SPH_VISC_BETA 3.0f

// box_wrap(x, 0, dim) of the rebuild (periodic.h:34-40,
// space_cell_index.c:113-116): one period back into the box.
SPH_HD inline double wrap_periodic(double x, double dim) {
  return x < 0.0 ? x + dim : (x >= dim ? x - dim : x);
}

// Top-level cell of a wrapped position (space_cell_index.c:126-128,
// cell_getid cell.h:532): (int)(pos * (1 / width)) per axis.  A position
// within rounding of the upper face can give cdim, which the reference
// would index past its grid with; it is kept in the last cell here.
SPH_HD inline int top_cell_index(const double pos[3], const double iw[3], const int cdim[3]) {
  int c[3];
  for (int d = 0; d < 3; d++) {
    c[d] = (int)(pos[d] * iw[d]);
    if (c[d] >= cdim[d]) c[d] = cdim[d] - 1;
  }
  return c[2] + cdim[2] * (c[1] + cdim[1] * c[0]);
}

// Kinds of reference evaluation frame.  The neighbour predicate r^2 < H^2
// must be evaluated in the same frame, with the same roundings, as the
// reference loop that owns the pair, or borderline pairs flip.
enum FrameKind : int8_t {
  FRAME_PAIR_CELLREL = 0,  // DOPAIR1/DOPAIR2: (float)(x_u - O_u) - (float)(x_p - O_p)
  FRAME_SELF_DBL = 1,      // DOSELF1/DOSELF2: (float)(x_u - x_p) in double
  FRAME_SELF_CELLREL = 2,  // DOSELF_SUBSET:   (float)(x - c.loc) differences
  FRAME_PAIR_ABS = 3,      // DOPAIR_SUBSET:   (float)((x_u - shift) - x_p)
};

// One partner cell of a leaf in a gather list: the particles of the leaf
// that pass the depth filter interact with every particle of the partner
// range, in the given frame.
struct Entry {
  int32_t first, count;       // partner particle range
  int32_t bfirst, bcount;     // partner j-block range
  int8_t kind;                // FrameKind
  int8_t min_depth, max_depth;
  int8_t pad0;
  float fdx, fdy, fdz;        // fast frame: partner top-cell origin (+periodic
                              // shift) minus the leaf's top-cell origin
  double ou[3];               // exact frame origin of the updated particle
                              // (PAIR_CELLREL / SELF_CELLREL) or the shift
                              // applied to it (PAIR_ABS)
  double op[3];               // exact frame origin of the partner particle
};
static_assert(sizeof(Entry) == 80, "Entry layout");

// j-block: up to kJBlock consecutive particles of one leaf (spatially
// sorted), with their bounding box in the top-cell frame; the gather culls
// whole blocks against each particle's search sphere.
#define SPH_NUM_TIME_BINS 56  // timeline.h:36
#define SPH_JBLOCK 16  // default j-block depth (the autotuner tries 8, 16, 32)

// Per-leaf geometry needed on the device by the ghost (cell_set_part_h_depth,
// cell.h:1787): the (h_min_allowed, h_max_allowed, depth) chain from the
// leaf up to its top cell.
#define SPH_MAX_DEPTH 24
struct LeafInfo {
  int32_t first, count;
  int32_t top;
  int32_t nlevels;            // chain length (leaf first)
  float hmin[SPH_MAX_DEPTH];
  float hmax[SPH_MAX_DEPTH];
  int8_t depth[SPH_MAX_DEPTH];
};

}  // namespace sphgpu
