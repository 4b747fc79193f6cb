// gbstencil engine: the C ABI of include/gbstencil.h.
//
// Replaces the AN5D-generated host sequencer of every benchmark
// (compiled/<prec>/<cfg>_host.cu:10-566: cudaMalloc, H2D of both planes, a
// loop of ceil(T/bt) launches with parity-correcting remainder launches, D2H,
// cudaFree) with a planner that picks the fused degree and tiling per grid,
// a launch sequence whose final plane is T%2 by construction, host-side
// validation of every address range a launch touches, and status codes in
// place of asserts.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbstencil.h"
#include "engine_internal.h"
#include "stencil_defs.h"

namespace gbs {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

gbs_status fail(gbs_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

gbs_status cuda_fail(cudaError_t e, const char *what) {
  // leave no non-sticky error behind for the caller's next CUDA call
  (void)cudaGetLastError();
  if (e == cudaErrorMemoryAllocation)
    return fail(GBS_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
  return fail(GBS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// launcher registry (the instantiation units)
// ---------------------------------------------------------------------------
#define GBS_DECL(id, S)                 \
  Picks picks_##id##_f_e();             \
  Picks picks_##id##_f_m();             \
  Picks picks_##id##_d_e();             \
  Picks picks_##id##_d_m();
GBS_FOR_EACH_STENCIL(GBS_DECL)
#undef GBS_DECL

static const Picks &picks(int sid, int dtype, int fma) {
  static std::once_flag once;
  static Picks table[kNumStencils][2][2];
  std::call_once(once, [] {
#define GBS_FILL(id, S)                     \
  table[id][0][0] = picks_##id##_f_e();     \
  table[id][0][1] = picks_##id##_f_m();     \
  table[id][1][0] = picks_##id##_d_e();     \
  table[id][1][1] = picks_##id##_d_m();
    GBS_FOR_EACH_STENCIL(GBS_FILL)
#undef GBS_FILL
  });
  return table[sid][dtype][fma];
}

int max_bt(int sid, int dtype, int fma) { return picks(sid, dtype, fma).maxb; }

// ---------------------------------------------------------------------------
// descriptors and layout
// ---------------------------------------------------------------------------
const gbs_stencil_def_t *stencil_def(int sid) {
  if (sid < 0 || sid >= GBS_NUM_STENCILS) return nullptr;
  return &gbs_stencil_defs[sid];
}

gbs_status check_desc(const gbs_desc *d) {
  if (!d) return fail(GBS_ERR_INVALID, "descriptor is NULL");
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  if (!s) return fail(GBS_ERR_INVALID, "unknown stencil id %d", d->stencil);
  if (d->dtype != GBS_F32 && d->dtype != GBS_F64)
    return fail(GBS_ERR_INVALID, "dtype must be GBS_F32 or GBS_F64 (got %d)", d->dtype);
  if (d->fp_mode != GBS_FP_EXACT && d->fp_mode != GBS_FP_FMA)
    return fail(GBS_ERR_INVALID, "fp_mode must be GBS_FP_EXACT or GBS_FP_FMA (got %d)", d->fp_mode);
  for (int a = 0; a < s->dim; ++a)
    if (d->n[a] < 1 || d->n[a] > (1 << 24))
      return fail(GBS_ERR_INVALID, "interior extent n[%d]=%d out of range [1, 2^24]", a, d->n[a]);
  if (d->timestep < 0) return fail(GBS_ERR_INVALID, "timestep must be >= 0 (got %d)", d->timestep);
  if (d->bt < 0 || d->sl < 0 || d->bs1 < 0 || d->bs2 < 0)
    return fail(GBS_ERR_INVALID, "bt/bs1/bs2/sl must be >= 0");
  const int V = d->dtype == GBS_F64 ? 2 : 4;
  if (d->bs2 != 0 && d->bs2 != 32 * V)
    return fail(GBS_ERR_UNSUPPORTED, "bs2 (tile columns) must be 0 or %d for this element type", 32 * V);
  if (s->dim == 2 && d->bs1 != 0 && d->bs1 != kWarpsPerCta2D)
    return fail(GBS_ERR_UNSUPPORTED, "bs1 (warps per CTA) of a 2-D grid must be 0 or %d", kWarpsPerCta2D);
  return GBS_OK;
}

size_t elem_size(int dtype) { return dtype == GBS_F64 ? 8 : 4; }

Layout make_layout(const gbs_desc *d) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  Layout L{};
  L.dim = s->dim;
  L.rad = s->rad;
  L.esize = elem_size(d->dtype);
  L.V = (int)(16 / L.esize);
  for (int a = 0; a < 3; ++a) L.dims[a] = a < s->dim ? d->n[a] + 2 * s->rad : 1;
  const int inner = L.dims[s->dim - 1];
  // column c at element shift + c; the first interior column is 16-byte aligned
  L.shift = (L.V - s->rad % L.V) % L.V;
  // every 32*V-element window starting at an aligned element < shift + inner
  // must fit in the row
  const long long need = (long long)L.shift + inner + 32 * L.V;
  const long long align = 128 / (long long)L.esize;
  L.pitch = (need + align - 1) / align * align;
  L.rows = s->dim == 2 ? (long long)L.dims[0] : (long long)L.dims[0] * L.dims[1];
  L.plane = L.rows * L.pitch;
  L.bytes = 2ull * (size_t)L.plane * L.esize;
  return L;
}

// ---------------------------------------------------------------------------
// planning
// ---------------------------------------------------------------------------
static int default_bt(const gbs_desc *d) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const int mx = max_bt(d->stencil, d->dtype, d->fp_mode);
  if (d->dtype == GBS_F64) return 1;
  int bt = 1;
  if (s->dim == 3) {
    bt = (s->rad == 1 && s->fpp <= 60) ? 2 : 1;
  } else if (s->dim == 2) {
    if (s->kind == 1) bt = 1;
    else if (s->fpp <= 20) bt = s->rad == 1 ? 4 : 2;
    else if (s->fpp <= 40) bt = 2;
    else bt = 1;
  }
  return std::max(1, std::min(bt, mx));
}

// bt and sl of the time loop for d: the caller's values, else the tuning
// table's choice for this size, else the fixed rule above (sl 0: one wave)
static void resolve_bt_sl(const gbs_desc *d, int *bt, int *sl) {
  int tb = 0, ts = 0;
  const bool tuned = (d->bt <= 0 || d->sl <= 0) && tuned_lookup(d, &tb, &ts);
  *bt = d->bt > 0 ? d->bt : (tuned ? tb : default_bt(d));
  *sl = d->sl > 0 ? d->sl : (tuned && tb == *bt ? ts : 0);
}

// ---------------------------------------------------------------------------
// tensor maps (cuTensorMapEncodeTiled, reached through the runtime's driver
// entry point so that the library needs no link against libcuda)
// ---------------------------------------------------------------------------
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    (void)cudaGetLastError();
  });
  return fn;
}

cudaError_t encode_plane_map(void *map, const void *plane, int esize, long long pitch, int d1, int d0, int bx,
                             int by) {
  EncodeTiledFn fn = encode_tiled_fn();
  if (!fn) return cudaErrorNotSupported;
  if (reinterpret_cast<uintptr_t>(plane) % 16 != 0 || (pitch * esize) % 16 != 0) return cudaErrorInvalidValue;
  const cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)d1, (cuuint64_t)d0};
  const cuuint64_t strides[2] = {(cuuint64_t)pitch * esize, (cuuint64_t)pitch * esize * (cuuint64_t)d1};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(static_cast<CUtensorMap *>(map),
                        esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                        const_cast<void *>(plane), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Divisors for which the exhaustive self-test (every float input, see
// gbs_check_division) shows the one-correction quotient equal to IEEE
// division: the artifact's 118 and 159. The GPU test suite re-proves this.
bool div_proven_exact(double d) { return d == 118.0 || d == 159.0; }

// splits T steps into n launches of at most bt steps with n == T (mod 2), so
// that launch j reads plane j%2 and the result lands in plane T%2.
std::vector<int> split_steps(int T, int bt) {
  std::vector<int> out;
  if (T <= 0) return out;
  int n = (T + bt - 1) / bt;
  if ((n - T) % 2 != 0) ++n;
  const int q = T / n, rem = T % n;
  for (int j = 0; j < n; ++j) out.push_back(q + (j < rem ? 1 : 0));
  return out;
}

static int sm_count() {
  static int n = -1;
  if (n < 0) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
      n = v;
    else
      n = 152;  // GB300
  }
  return n;
}

long long resident_warps_2d(int sid, int dtype, int fma, int b) {
  static std::mutex mu;
  static int cache[kNumStencils][2][2][kMaxB + 1];
  std::lock_guard<std::mutex> lk(mu);
  int &c = cache[sid][dtype][fma][b];
  if (c == 0) {
    const Picks &pk = picks(sid, dtype, fma);
    int w = (b <= kMaxB && pk.o2[b]) ? pk.o2[b]() : 0;
    c = w > 0 ? w : 16;
  }
  return (long long)c * sm_count();
}

Geometry2D geometry2d(const Layout &L, int b, int sl_req, long long resident) {
  Geometry2D g{};
  const int R = L.rad, V = L.V;
  g.b = b;
  // window starts are 16-byte aligned, so the strip can start up to V-1
  // columns inside it
  g.wout = ((32 * V - 2 * b * R - (V - 1)) / V) * V;
  const int ni = L.dims[0] - 2 * R, nj = L.dims[1] - 2 * R;
  g.nstrips = g.wout > 0 ? (nj + g.wout - 1) / g.wout : 1;
  int sl = sl_req;
  if (sl <= 0) {
    // one full wave of resident warps, each streaming one block; blocks at
    // least 4*b*r rows long so that the stream overlap stays small
    if (resident <= 0) resident = 152LL * 16;
    long long nb = std::max<long long>(1, resident / std::max(1, g.nstrips));
    sl = (int)((ni + nb - 1) / nb);
    sl = std::max(sl, std::max(8, 4 * b * R));
  }
  g.sl = std::min(sl, ni);
  g.nblocks = (ni + g.sl - 1) / g.sl;
  return g;
}

long long resident_ctas_3d(int sid, int dtype, int fma, int b, int v) {
  static std::mutex mu;
  static int cache[kNumStencils][2][2][kMaxB + 1][kVar3];
  std::lock_guard<std::mutex> lk(mu);
  if (b < 1 || b > kMaxB || v < 0 || v >= kVar3) return sm_count();
  int &c = cache[sid][dtype][fma][b][v];
  if (c == 0) {
    const Picks &pk = picks(sid, dtype, fma);
    int n = pk.o3[b][v] ? pk.o3[b][v]() : 0;
    c = n > 0 ? n : 1;
  }
  return (long long)c * sm_count();
}

Tile3DShape tile_shape_3d(int sid, int dtype, int fma, int b, int v) {
  const Picks &pk = picks(sid, dtype, fma);
  Tile3DShape t{};
  if (b >= 1 && b <= kMaxB && v >= 0 && v < kVar3 && pk.tj3[b][v] > 0) {
    t.tj = pk.tj3[b][v];
    t.jout = pk.jout3[b][v];
    t.wk = pk.wk3[b][v];
    t.tile = pk.tile3[b];
  }
  return t;
}

int variant_3d(const gbs_desc *d, int b) {
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const Picks &pk = picks(d->stencil, d->dtype, fma);
  if (b < 1 || b > kMaxB) return -1;
  int want = d->bs1;
  if (want <= 0) {
    int tb = 0, ts = 0, tr = 0;
    if (tuned_lookup(d, &tb, &ts, &tr) && tb == b) want = tr;
  }
  if (want > 0) {
    for (int v = 0; v < kVar3; ++v)
      if (pk.tj3[b][v] == want) return v;
    if (d->bs1 > 0) {
      fail(GBS_ERR_UNSUPPORTED, "no 3-D tile of %d rows at degree %d (built: %d, %d)", d->bs1, b, pk.tj3[b][0],
           pk.tj3[b][1]);
      return -1;
    }
  }
  return 0;
}

// Tiles of the launcher's shape (rows x one 32*V-column window); the number
// of stream blocks is chosen to fill whole waves of resident CTAs while
// keeping the 2*b*r-plane stream overlap small.
Geometry3D geometry3d(const Layout &L, int b, const Tile3DShape &ts, int sl_req, long long resident) {
  Geometry3D g{};
  const int R = L.rad;
  g.b = b;
  g.tj = ts.tj;
  g.jout = ts.jout;
  g.wk = ts.wk;
  g.tile = ts.tile;
  const int ni = L.dims[0] - 2 * R, nj = L.dims[1] - 2 * R, nk = L.dims[2] - 2 * R;
  g.ntk = g.wk > 0 ? (nk + g.wk - 1) / g.wk : 1;
  g.ntj = g.jout > 0 ? (nj + g.jout - 1) / g.jout : 1;
  const long long tiles = (long long)g.ntk * g.ntj;
  int sl = sl_req;
  if (sl <= 0) {
    if (resident <= 0) resident = sm_count();
    double best = 1e30;
    for (int nb = 1; nb <= std::min(ni, 256); ++nb) {
      const int cand = (ni + nb - 1) / nb;
      const long long ctas = tiles * ((ni + cand - 1) / cand);
      const double waves = std::ceil((double)ctas / resident);
      // time ~ waves * (planes streamed per CTA)
      const double cost = waves * (cand + 2.0 * b * R + (b - 1));
      if (cost < best - 1e-9) {
        best = cost;
        sl = cand;
      }
    }
  }
  g.sl = std::max(1, std::min(sl, ni));
  g.nblocks = (ni + g.sl - 1) / g.sl;
  return g;
}

gbs_status validate3d(const Layout &L, const Geometry3D &g) {
  const int R = L.rad, V = L.V, ROW = 32 * V;
  if (g.tj <= 0) return fail(GBS_ERR_UNSUPPORTED, "no 3-D kernel of degree %d", g.b);
  if (g.jout <= 0 || g.wk <= 0)
    return fail(GBS_ERR_UNSUPPORTED, "fused degree %d leaves no output cells in a %d-row tile (r=%d)", g.b,
                g.tj, R);
  if ((L.pitch * (long long)L.esize) % 16 != 0) return fail(GBS_ERR_INVALID, "internal: pitch alignment");
  if ((L.shift + R) % V != 0) return fail(GBS_ERR_INVALID, "internal: first interior column not aligned");
  if (g.wk % V != 0) return fail(GBS_ERR_INVALID, "internal: tile width not a whole number of vectors");
  // the tile kernel's plane copies are tensor-map boxes: the hardware fills
  // what lies outside the plane, and its halo loads are guarded per lane
  if (g.tile) return GBS_OK;
  for (int t = 0; t < g.ntk; ++t) {
    const int cs = R + t * g.wk;
    const int ce = std::min(cs + g.wk, L.dims[2] - R);
    const long long ws = ((std::max(0, cs - g.b * R) + L.shift) / V) * (long long)V;
    const int need_hi = std::min(L.dims[2], ce + g.b * R);
    if (ws < 0 || ws + ROW > L.pitch || need_hi + L.shift > ws + ROW)
      return fail(GBS_ERR_INVALID, "internal: 3-D column window %d out of range", t);
  }
  return GBS_OK;
}

// Every address range a 2-D launch touches, checked against the buffer.
gbs_status validate2d(const Layout &L, const Geometry2D &g) {
  const int R = L.rad, V = L.V, ROW = 32 * V;
  if (g.wout <= 0) return fail(GBS_ERR_UNSUPPORTED, "fused degree %d leaves no output columns", g.b);
  if (L.shift % 1 != 0 || (L.pitch * (long long)L.esize) % 16 != 0)
    return fail(GBS_ERR_INVALID, "internal: row pitch not 16-byte aligned");
  for (int s = 0; s < g.nstrips; ++s) {
    const int cs = R + s * g.wout;
    const int ce = std::min(cs + g.wout, L.dims[1] - R);
    const int need_lo = std::max(0, cs - g.b * R);
    const int need_hi = std::min(L.dims[1], ce + g.b * R);
    const long long ws = ((need_lo + L.shift) / V) * (long long)V;
    if (ws < 0 || ws + ROW > L.pitch)
      return fail(GBS_ERR_INVALID, "internal: strip %d window [%lld,%lld) outside row of %lld", s, ws,
                  ws + ROW, L.pitch);
    if (need_hi + L.shift > ws + ROW)
      return fail(GBS_ERR_INVALID, "internal: strip %d window misses columns", s);
    if ((ws * (long long)L.esize) % 16 != 0) return fail(GBS_ERR_INVALID, "internal: unaligned window");
  }
  return GBS_OK;
}

}  // namespace gbs

using namespace gbs;

// ---------------------------------------------------------------------------
// device state: error word, cached buffer, stream
// ---------------------------------------------------------------------------
namespace {
// Dense rows <-> the engine layout's padded rows, on the device: row r of
// `rows` rows of `words` 32-bit words. A host copy of a dense grid into a
// dense device buffer is one contiguous transfer (full link speed); the
// strided layout change then runs at HBM speed instead of as one copy
// descriptor per row.
__global__ void repitch_kernel(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, long long rows,
                               int words, long long src_stride, long long dst_stride) {
  for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
    const uint32_t *a = src + r * src_stride;
    uint32_t *b = dst + r * dst_stride;
    for (int c = threadIdx.x; c < words; c += blockDim.x) b[c] = a[c];
  }
}

cudaError_t repitch(const void *src, void *dst, long long rows, size_t row_bytes, size_t src_pitch_bytes,
                    size_t dst_pitch_bytes, cudaStream_t s) {
  const long long blocks = std::min<long long>(rows, 152LL * 16);
  repitch_kernel<<<(unsigned)std::max<long long>(1, blocks), 256, 0, s>>>(
      static_cast<const uint32_t *>(src), static_cast<uint32_t *>(dst), rows, (int)(row_bytes / 4),
      (long long)(src_pitch_bytes / 4), (long long)(dst_pitch_bytes / 4));
  return cudaGetLastError();
}

struct DeviceState {
  int *err = nullptr;          // error word of the kernels (device)
  void *buf = nullptr;         // gbs_run's cached grid buffer
  size_t buf_bytes = 0;
  void *dense = nullptr;       // gbs_run's cached staging buffer (the host grid's dense layout)
  size_t dense_bytes = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};
std::mutex g_mu;
DeviceState g_dev[64];

gbs_status device_state(DeviceState **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(GBS_ERR_NODEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_NODEVICE, "device ordinal %d unsupported", dev);
  DeviceState &s = g_dev[dev];
  if (!s.err) {
    if ((e = cudaMalloc(&s.err, sizeof(int))) != cudaSuccess) return cuda_fail(e, "cudaMalloc(error word)");
    if ((e = cudaMemset(s.err, 0, sizeof(int))) != cudaSuccess) return cuda_fail(e, "cudaMemset");
  }
  *out = &s;
  return GBS_OK;
}
}  // namespace

namespace gbs {
gbs_status error_word(int **out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState *s;
  gbs_status st = device_state(&s);
  if (st != GBS_OK) return st;
  *out = s->err;
  return GBS_OK;
}

// Enqueues the whole time loop of `d` on `stream` for a buffer in layout L.
gbs_status run_loop(const gbs_desc *d, const Layout &L, void *dev_A, cudaStream_t stream, int *err) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const Picks &pk = picks(d->stencil, d->dtype, fma);
  if (pk.maxb == 0)
    return fail(GBS_ERR_UNSUPPORTED, "no kernels built for %s dtype=%d fp_mode=%d", s->name, d->dtype,
                d->fp_mode);
  int bt = 0, sl = 0;
  resolve_bt_sl(d, &bt, &sl);
  if (bt > pk.maxb)
    return fail(GBS_ERR_UNSUPPORTED, "bt=%d exceeds the largest fused degree built for %s (%d)", bt,
                s->name, pk.maxb);
  // coefficients
  std::vector<double> coef(s->nterms > 0 ? s->nterms : 1);
  if (s->kind == 1) {
    coef[0] = d->coef ? (d->dtype == GBS_F64 ? ((const double *)d->coef)[0] : ((const float *)d->coef)[0])
                      : (double)s->numerator;
  } else {
    for (int t = 0; t < s->nterms; ++t)
      coef[t] = d->coef ? (d->dtype == GBS_F64 ? ((const double *)d->coef)[t] : ((const float *)d->coef)[t])
                        : (double)s->terms[t].coef;
  }
  const double div = d->divisor != 0.0 ? d->divisor : (double)s->divisor;
  const double eps = d->eps != 0.0 ? d->eps : (double)s->eps;
  if (s->divisor && div == 0.0) return fail(GBS_ERR_INVALID, "divisor must be nonzero");

  const std::vector<int> steps = split_steps(d->timestep, bt);
  char *base = static_cast<char *>(dev_A);
  const size_t plane_bytes = (size_t)L.plane * L.esize;
  for (size_t j = 0; j < steps.size(); ++j) {
    gbs_status st = launch_block(d, L, coef.data(), div, eps, sl, steps[j], base + (j % 2) * plane_bytes,
                                 base + ((j + 1) % 2) * plane_bytes, stream, err);
    if (st != GBS_OK) return st;
  }
  return GBS_OK;
}

// One launch of b fused steps from plane src to plane dst (layout L; the
// interior of dst is written, its halo never): coefficients as the source
// writes them, divisor and eps resolved, sl 0 = one wave.
gbs_status launch_block(const gbs_desc *d, const Layout &L, const double *coef, double div, double eps, int sl,
                        int b, const void *src, void *dst, cudaStream_t stream, int *err) {
  return launch_block_stash(d, L, coef, div, eps, sl, b, src, dst, nullptr, stream, err);
}

gbs_status launch_block_stash(const gbs_desc *d, const Layout &L, const double *coef, double div, double eps, int sl,
                              int b, const void *src, void *dst, void *stash, cudaStream_t stream, int *err) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  if (stash && s->dim != 2) return fail(GBS_ERR_UNSUPPORTED, "stashed launches take 2-D grids");
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const Picks &pk = picks(d->stencil, d->dtype, fma);
  if (b < 1 || b > pk.maxb)
    return fail(GBS_ERR_UNSUPPORTED, "no kernel of degree %d built for %s", b, s->name);
  {
    if (s->dim == 2) {
      Geometry2D g = geometry2d(L, b, sl, resident_warps_2d(d->stencil, d->dtype, fma, b));
      gbs_status st = validate2d(L, g);
      if (st != GBS_OK) return st;
      Launch2D a{};
      a.src = src;
      a.dst = dst;
      a.err = err;
      a.pitch = L.pitch;
      a.d0 = L.dims[0];
      a.d1 = L.dims[1];
      a.shift = L.shift;
      a.b = b;
      a.wout = g.wout;
      a.nstrips = g.nstrips;
      a.nblocks = g.nblocks;
      a.sl = g.sl;
      a.coef = coef;
      a.div = div;
      a.eps = eps;
      a.div_proven = d->dtype == GBS_F32 && div_proven_exact(div);
      a.stash = stash;
      a.stash_stride = L.plane;
      Launch2DFn fn = stash ? pk.l2s[b] : pk.l2[b];
      if (!fn) return fail(GBS_ERR_UNSUPPORTED, "no 2-D kernel%s for b=%d", stash ? " in stash mode" : "", b);
      cudaError_t e = fn(a, stream);
      if (e != cudaSuccess) return cuda_fail(e, "2-D stencil launch");
    } else {
      const int v = variant_3d(d, b);
      if (v < 0) return GBS_ERR_UNSUPPORTED;
      Geometry3D g = geometry3d(L, b, tile_shape_3d(d->stencil, d->dtype, fma, b, v), sl,
                                 resident_ctas_3d(d->stencil, d->dtype, fma, b, v));
      gbs_status st = validate3d(L, g);
      if (st != GBS_OK) return st;
      Launch3D a{};
      a.src = src;
      a.dst = dst;
      a.err = err;
      a.pitch = L.pitch;
      a.d0 = L.dims[0];
      a.d1 = L.dims[1];
      a.d2 = L.dims[2];
      a.shift = (int)L.shift;
      a.b = b;
      a.jout = g.jout;
      a.wk = g.wk;
      a.ntk = g.ntk;
      a.ntj = g.ntj;
      a.nblocks = g.nblocks;
      a.sl = g.sl;
      a.coef = coef;
      a.div = div;
      a.div_proven = d->dtype == GBS_F32 && div_proven_exact(div);
      if (!pk.l3[b][v]) return fail(GBS_ERR_UNSUPPORTED, "no 3-D kernel for b=%d", b);
      cudaError_t e = pk.l3[b][v](a, stream);
      if (e != cudaSuccess) return cuda_fail(e, "3-D stencil launch");
    }
  }
  return GBS_OK;
}
}  // namespace gbs

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int gbs_num_stencils(void) { return GBS_NUM_STENCILS; }

const char *gbs_stencil_name(int id) {
  const gbs_stencil_def_t *s = stencil_def(id);
  return s ? s->name : nullptr;
}

int gbs_stencil_id(const char *name) {
  if (!name) return -1;
  for (int i = 0; i < GBS_NUM_STENCILS; ++i)
    if (std::strcmp(gbs_stencil_defs[i].name, name) == 0) return i;
  return -1;
}

gbs_status gbs_stencil_info(int id, int *dim, int *rad, int *nterms, int *fpp) {
  const gbs_stencil_def_t *s = stencil_def(id);
  if (!s) return fail(GBS_ERR_INVALID, "unknown stencil id %d", id);
  if (dim) *dim = s->dim;
  if (rad) *rad = s->rad;
  if (nterms) *nterms = s->kind == 1 ? 1 : s->nterms;
  if (fpp) *fpp = s->fpp;
  return GBS_OK;
}

const char *gbs_last_error(void) { return g_last_error.c_str(); }

gbs_status gbs_get_layout(const gbs_desc *d, gbs_layout *out) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!out) return fail(GBS_ERR_INVALID, "out is NULL");
  const Layout L = make_layout(d);
  out->pitch = (size_t)L.pitch;
  out->shift = (size_t)L.shift;
  out->rows = (size_t)L.rows;
  out->plane = (size_t)L.plane;
  out->bytes = L.bytes;
  for (int a = 0; a < 3; ++a) out->dimsize[a] = L.dims[a];
  out->dim = L.dim;
  out->rad = L.rad;
  return GBS_OK;
}

gbs_status gbs_plan(const gbs_desc *d, gbs_plan_info *out) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!out) return fail(GBS_ERR_INVALID, "out is NULL");
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const Layout L = make_layout(d);
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const int mx = max_bt(d->stencil, d->dtype, fma);
  if (mx == 0) return fail(GBS_ERR_UNSUPPORTED, "no kernels built for %s", s->name);
  int bt = 0, sl = 0;
  resolve_bt_sl(d, &bt, &sl);
  if (bt > mx) return fail(GBS_ERR_UNSUPPORTED, "bt=%d exceeds the largest fused degree built (%d)", bt, mx);
  std::memset(out, 0, sizeof *out);
  out->bt = bt;
  out->launches = (int)split_steps(d->timestep, bt).size();
  if (s->dim == 2) {
    Geometry2D g = geometry2d(L, bt, sl, resident_warps_2d(d->stencil, d->dtype, fma, bt));
    st = validate2d(L, g);
    if (st != GBS_OK) return st;
    out->bs1 = kWarpsPerCta2D;
    out->bs2 = 32 * L.V;
    out->sl = g.sl;
    out->ctas = (g.nstrips * g.nblocks + 3) / 4;
    out->valid_w = g.wout;
    const double cols = 32.0 * L.V, rows = g.sl + 2.0 * bt * L.rad;
    out->redundancy = (cols * rows) / ((double)g.wout * g.sl);
  } else {
    const int v = variant_3d(d, bt);
    if (v < 0) return GBS_ERR_UNSUPPORTED;
    Geometry3D g = geometry3d(L, bt, tile_shape_3d(d->stencil, d->dtype, fma, bt, v), sl,
                                 resident_ctas_3d(d->stencil, d->dtype, fma, bt, v));
    st = validate3d(L, g);
    if (st != GBS_OK) return st;
    out->bs1 = g.tj;
    out->bs2 = 32 * L.V;
    out->sl = g.sl;
    out->ctas = g.ntk * g.ntj * g.nblocks;
    out->valid_w = g.wk;
    out->redundancy = (32.0 * L.V * g.tj * (g.sl + 2.0 * bt * L.rad)) / ((double)g.wk * g.jout * g.sl);
    out->bs1 = g.tj;
  }
  return GBS_OK;
}

gbs_status gbs_upload(const gbs_desc *d, const void *host_A, void *dev_A, void *stream) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!host_A || !dev_A) return fail(GBS_ERR_INVALID, "NULL buffer");
  const Layout L = make_layout(d);
  const size_t w = (size_t)L.dims[L.dim - 1] * L.esize;
  const size_t nrows = 2 * (size_t)L.rows;
  cudaError_t e = cudaMemcpy2DAsync(static_cast<char *>(dev_A) + L.shift * L.esize, L.pitch * L.esize,
                                    host_A, w, w, nrows, cudaMemcpyHostToDevice, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "upload");
  return GBS_OK;
}

gbs_status gbs_download(const gbs_desc *d, const void *dev_A, void *host_A, void *stream) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!host_A || !dev_A) return fail(GBS_ERR_INVALID, "NULL buffer");
  const Layout L = make_layout(d);
  const size_t w = (size_t)L.dims[L.dim - 1] * L.esize;
  const size_t nrows = 2 * (size_t)L.rows;
  cudaError_t e = cudaMemcpy2DAsync(host_A, w, static_cast<const char *>(dev_A) + L.shift * L.esize,
                                    L.pitch * L.esize, w, nrows, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "download");
  return GBS_OK;
}

gbs_status gbs_sync(void *stream) {
  int *err = nullptr;
  gbs_status st = error_word(&err);
  if (st != GBS_OK) return st;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
  int h = 0;
  e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read error word");
  if (h != 0) {
    cudaMemset(err, 0, sizeof(int));
    return fail(GBS_ERR_TIMEOUT, "a device-side wait gave up (error bits 0x%x)", h);
  }
  return GBS_OK;
}

gbs_status gbs_run_device(const gbs_desc *d, void *dev_A, void *stream) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!dev_A) return fail(GBS_ERR_INVALID, "dev_A is NULL");
  if (reinterpret_cast<uintptr_t>(dev_A) % 128 != 0)
    return fail(GBS_ERR_INVALID, "dev_A must be 128-byte aligned");
  int *err = nullptr;
  st = error_word(&err);
  if (st != GBS_OK) return st;
  const Layout L = make_layout(d);
  return run_loop(d, L, dev_A, (cudaStream_t)stream, err);
}

gbs_status gbs_run(const gbs_desc *d, void *host_A, double *ms_out) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!host_A) return fail(GBS_ERR_INVALID, "host_A is NULL");
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState *s;
  st = device_state(&s);
  if (st != GBS_OK) return st;
  cudaError_t e;
  if (!s->stream) {
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&s->ev0)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&s->ev1)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  }
  const Layout L = make_layout(d);
  if (s->buf_bytes < L.bytes) {
    if (s->buf) cudaFree(s->buf);
    s->buf = nullptr;
    s->buf_bytes = 0;
    if ((e = cudaMalloc(&s->buf, L.bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(grid)");
    s->buf_bytes = L.bytes;
    // margins are never part of a result but are read by edge windows
    if ((e = cudaMemset(s->buf, 0, L.bytes)) != cudaSuccess) return cuda_fail(e, "cudaMemset(grid)");
  }
  // host grid -> dense staging buffer (one contiguous copy) -> engine layout
  const size_t row_bytes = (size_t)L.dims[L.dim - 1] * L.esize;
  const long long nrows = 2 * (long long)L.rows;
  const size_t dense_bytes = row_bytes * (size_t)nrows;
  if (s->dense_bytes < dense_bytes) {
    if (s->dense) cudaFree(s->dense);
    s->dense = nullptr;
    s->dense_bytes = 0;
    if ((e = cudaMalloc(&s->dense, dense_bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(staging)");
    s->dense_bytes = dense_bytes;
  }
  char *padded = static_cast<char *>(s->buf) + L.shift * L.esize;
  const size_t pitch_bytes = (size_t)L.pitch * L.esize;
  if ((e = cudaMemcpyAsync(s->dense, host_A, dense_bytes, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
    return cuda_fail(e, "upload");
  if ((e = repitch(s->dense, padded, nrows, row_bytes, row_bytes, pitch_bytes, s->stream)) != cudaSuccess)
    return cuda_fail(e, "upload (layout)");
  if ((e = cudaEventRecord(s->ev0, s->stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
  st = run_loop(d, L, s->buf, s->stream, s->err);
  if (st != GBS_OK) {
    cudaStreamSynchronize(s->stream);
    return st;
  }
  if ((e = cudaEventRecord(s->ev1, s->stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
  if ((e = repitch(padded, s->dense, nrows, row_bytes, pitch_bytes, row_bytes, s->stream)) != cudaSuccess)
    return cuda_fail(e, "download (layout)");
  if ((e = cudaMemcpyAsync(host_A, s->dense, dense_bytes, cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
    return cuda_fail(e, "download");
  {
    // gbs_sync takes the lock through error_word(); read the word directly
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "stream synchronize");
    int h = 0;
    if ((e = cudaMemcpy(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
      return cuda_fail(e, "read error word");
    if (h != 0) {
      cudaMemset(s->err, 0, sizeof(int));
      return fail(GBS_ERR_TIMEOUT, "a device-side wait gave up (error bits 0x%x)", h);
    }
  }
  if (ms_out) {
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, s->ev0, s->ev1)) != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
    *ms_out = ms;
  }
  return GBS_OK;
}

void gbs_release_cache(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &s : g_dev) {
    if (s.buf) cudaFree(s.buf);
    if (s.dense) cudaFree(s.dense);
    s.buf = nullptr;
    s.buf_bytes = 0;
    s.dense = nullptr;
    s.dense_bytes = 0;
  }
}

}  // extern "C"
