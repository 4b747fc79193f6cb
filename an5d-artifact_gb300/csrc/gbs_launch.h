// Host-side launch descriptions and the per-(stencil, type, mode) launcher
// tables that the instantiation units export to the engine.
#pragma once
#include <cuda_runtime.h>

namespace gbs {

// One launch of the 2-D family (see kernel2d.cuh for the decomposition).
struct Launch2D {
  const void *src;
  void *dst;
  int *err;
  long long pitch;
  int d0, d1, shift, b, wout, nstrips, nblocks, sl;
  const double *coef;
  double div, eps;
  bool div_proven;    // the one-correction quotient is exact for every float input
  void *stash;        // not null: level l < b also stores its interior cells to
                      // stash + (l-1)*stash_stride elements (the states between)
  long long stash_stride;
};

// One launch of the 3-D family (see kernel3d.cuh).
struct Launch3D {
  const void *src;
  void *dst;
  int *err;
  long long pitch;    // elements per padded k-row
  int d0, d1, d2, shift, b;
  int jout, wk;       // valid rows (j) and columns (k) per tile
  int ntk, ntj, nblocks, sl;
  const double *coef;
  double div;
  bool div_proven;
};

using Launch2DFn = cudaError_t (*)(const Launch2D &, cudaStream_t);
// resident warps per SM of a 2-D launcher (occupancy), 0 on error
using Occupancy2DFn = int (*)();
using Launch3DFn = cudaError_t (*)(const Launch3D &, cudaStream_t);
// resident CTAs per SM of a 3-D launcher (occupancy), 0 on error
using Occupancy3DFn = int (*)();

// Launchers of one (stencil, element type, fp mode), indexed by the fused
// degree b (nullptr where none is built).
constexpr int kMaxB = 16;
// warps per CTA of the 2-D kernels (each warp streams its own work items)
constexpr int kWarpsPerCta2D = 4;
// largest degree of the 2-D FMA-mode kernels built in stash mode (the
// adjoint's chunk recompute, which keeps every intermediate state)
constexpr int kMaxStashB = 4;
// 3-D block shapes per degree: variant v of the tile kernel has kTileWarps[v]
// warps (tile rows = warps x rows per warp)
constexpr int kVar3 = 2;
constexpr int kTileWarps[kVar3] = {16, 8};
struct Picks {
  int maxb;
  Launch2DFn l2[kMaxB + 1];
  Launch2DFn l2s[kMaxB + 1];    // stash-mode 2-D launchers (FMA mode, low degrees; else null)
  Occupancy2DFn o2[kMaxB + 1];
  Launch3DFn l3[kMaxB + 1][kVar3];
  Occupancy3DFn o3[kMaxB + 1][kVar3];
  int tj3[kMaxB + 1][kVar3];    // tile rows of the 3-D launcher (0: variant not built)
  int jout3[kMaxB + 1][kVar3];  // valid (output) rows of its tile
  int wk3[kMaxB + 1][kVar3];    // valid (output) columns of its tile
  int tile3[kMaxB + 1];         // 1: the tensor-map tile kernel (no column window checks needed)
};

// Encodes the tensor map of one time plane of a 3-D grid for the tile kernel:
// a {pitch, d1, d0}-element tensor at `plane` (16-byte aligned), rows of
// pitch*esize bytes, copied in boxes of bx x by x 1 elements (zero fill
// outside). `map` points at a CUtensorMap (64-byte aligned storage).
cudaError_t encode_plane_map(void *map, const void *plane, int esize, long long pitch, int d1, int d0, int bx,
                             int by);

}  // namespace gbs
