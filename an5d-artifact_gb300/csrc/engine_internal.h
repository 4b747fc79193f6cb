// Engine internals shared by the host-side translation units.
#pragma once
#include <cstdarg>
#include <cstddef>
#include <vector>

#include "../../include/gbstencil.h"
#include "gbs_launch.h"
#include "stencil_defs.h"
#include "stencil_table.cuh"

namespace gbs {

// Device layout of a two-plane grid (see gbs_layout in gbstencil.h).
struct Layout {
  int dim, rad, V;
  size_t esize;
  int dims[3];          // dimsize per axis
  long long shift;      // element offset of column 0
  long long pitch;      // elements per padded innermost row
  long long rows;       // rows per plane
  long long plane;      // elements per plane
  size_t bytes;         // both planes
};

struct Geometry2D {
  int b, wout, nstrips, nblocks, sl;
};

struct Geometry3D {
  int b, tj, jout, wk, ntk, ntj, nblocks, sl;
  int tile;  // the tensor-map tile kernel (its copies are bounds-checked by the hardware)
};
// Tile shape of the 3-D launcher of degree b: computed rows, valid rows and
// valid columns per tile, and whether it is the tensor-map tile kernel.
struct Tile3DShape {
  int tj, jout, wk, tile;
};
Tile3DShape tile_shape_3d(int sid, int dtype, int fma, int b, int variant);
// block-shape variant of the 3-D launcher of degree b for d: the one whose
// tile rows equal d->bs1, else the tuning table's, else variant 0; -1 (and
// an error recorded) when d->bs1 names no built shape
int variant_3d(const gbs_desc *d, int b);
Geometry3D geometry3d(const Layout &L, int b, const Tile3DShape &ts, int sl_req, long long resident_ctas);
gbs_status validate3d(const Layout &L, const Geometry3D &g);
long long resident_ctas_3d(int sid, int dtype, int fma, int b, int variant);

gbs_status fail(gbs_status st, const char *fmt, ...);
gbs_status cuda_fail(cudaError_t e, const char *what);
const gbs_stencil_def_t *stencil_def(int sid);
gbs_status check_desc(const gbs_desc *d);
Layout make_layout(const gbs_desc *d);
std::vector<int> split_steps(int T, int bt);
// resident_warps: warps the GPU holds at once for this kernel (0 = unknown)
Geometry2D geometry2d(const Layout &L, int b, int sl_req, long long resident_warps);
long long resident_warps_2d(int sid, int dtype, int fma, int b);
gbs_status validate2d(const Layout &L, const Geometry2D &g);
gbs_status error_word(int **out);
gbs_status run_loop(const gbs_desc *d, const Layout &L, void *dev_A, cudaStream_t stream, int *err);
gbs_status launch_block(const gbs_desc *d, const Layout &L, const double *coef, double div, double eps, int sl,
                        int b, const void *src, void *dst, cudaStream_t stream, int *err);
// launch_block that also stores the states after 1 .. b-1 steps (interior
// cells) to the planes stash, stash + plane, ... (2-D grids only; stash may
// be null)
gbs_status launch_block_stash(const gbs_desc *d, const Layout &L, const double *coef, double div, double eps, int sl,
                              int b, const void *src, void *dst, void *stash, cudaStream_t stream, int *err);
int max_bt(int sid, int dtype, int fma);
// the tuning table's (bt, sl) for d's stencil, dtype, mode and size class
bool tuned_lookup(const gbs_desc *d, int *bt, int *sl, int *bs1 = nullptr);
bool div_proven_exact(double d);

}  // namespace gbs
