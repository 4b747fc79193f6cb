// Batched persistent launch: many independent 2-D grids of uneven sizes,
// radii and step counts advanced by ONE kernel launch, replayed from a CUDA
// graph.
//
// Work items are (grid, time block, strip, stream block): one warp runs the
// same temporally-blocked pipeline as the single-grid kernel
// (warp_item2d) on one item. The host orders the items by time block;
// persistent CTAs take groups of consecutive items in that order from an
// atomic counter. An item of time block k of grid g starts once its stream
// block and the two beside it have finished g's earlier blocks (completion
// counters per stream block, or one per grid in the run without
// allocation, reaching the item's `need`). The order (by time block) makes
// this deadlock-free: every item an item waits on was taken earlier by a
// running CTA that never waits on a later item. Waits are bounded (the
// error word is set and the CTA stops). The layered schedule runs the same
// items as one kernel node per time block instead, with no waits.
//
// Memory ordering: a finishing item's lanes fence their stores, then lane 0
// increments its block's counter; a starting item's lane 0 reads the
// counters with acquire semantics and issues a proxy fence before its bulk
// copies (an async-proxy read) touch the data. Loads outside the bulk copies
// bypass L1.
//
// Built twice: -DGBS_FMA=0 (exact mode) and -DGBS_FMA=1.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "engine_internal.h"
#include "kernel2d.cuh"

#ifndef GBS_FMA
#error "GBS_FMA must be defined"
#endif

namespace gbs {
namespace batchdetail {
constexpr int kMaxTerms = 81;

struct GridDev {
  float *base;          // two-plane buffer (engine layout)
  long long pitch, plane;
  int d0, d1, shift, sid;
  int sl, nblocks;
  // completion counters of the grid: done[cbase .. cbase + ccount); one per
  // stream block (an item waits for its own block and the two beside it),
  // or one for the whole grid (an item waits for every earlier item of it)
  int cbase, ccount;
  float coef[kMaxTerms];
  float div, rdiv, eps;
  int divmode;
};

struct Item {
  int grid, k, b, strip, blk, need, pad0, pad1;
};
}  // namespace batchdetail
using batchdetail::GridDev;
using batchdetail::Item;

namespace {
constexpr bool kFma = GBS_FMA != 0;
constexpr int kWpc = kWpc2D, kStages = kStages2D;
// CTAs per SM the batched kernels are built for. The layered kernel takes 4
// (at most 128 registers a thread, 16 warps an SM; every variant but
// star2d3r at degree 2 fits without spilling): 2.92x the per-grid launches
// on the 512-grid mix against 2.76x at 3 CTAs (168 registers, of which the
// heaviest variants use 154-164 and so set them for all). The persistent
// kernel keeps 3: at 4 its warps stalled more on instruction fetch (more
// variants resident per SM) and it was 1% slower.
constexpr int kLayerCtas = 4, kPersistentCtas = 3;

// The stencils a batch may mix and the fused degree used for each (the full
// blocks; remainders run at degree 1). Measured on the 512-grid mix
// (layered): radius 1 at 4 -> 6 and radius 2 at 2 -> 3 gave +1.7%; radius 3
// direct (star2d3r) at 1 instead of 2 lost 2.7%. box2d2r (25 terms, FP32
// bound from degree 2) stays at 2, where it does not spill.
template <class S> constexpr int batch_degree() {
  if (S::kKind == KIND_GRADIENT) return 1;
  if (S::kRad == 1) return 6;
  if (S::kRad == 2) return S::kTerms > 13 ? 2 : 3;
  if (S::kRad == 3) return S::kAssoc ? 1 : 2;
  return 1;
}

struct Args {
  const GridDev *grids;
  const Item *items;
  int nitems;
  unsigned *next;       // groups of kWpc items taken (persistent)
  unsigned *done;       // completed items per counter (GridDev::cbase)
  int *err;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// bytes of the per-warp shared-memory slot that holds an item's parameters
constexpr int kParamSlot = 512;
static_assert(sizeof(Params2D<float, batchdetail::kMaxTerms>) <= kParamSlot, "parameter slot too small");

// One (stencil, degree) variant per function, not inlined: each variant gets
// its own register allocation (inlining all of them into the dispatcher
// forces a local-memory frame onto every variant's loop) and the call costs
// once per item. The parameters (with up to 81 coefficients) are staged in
// shared memory: a per-thread copy would sit on the local-memory stack.
// Everything else comes by value (time block k, strip, stream block, the
// warp's copy count) and the new copy count is the return value, ~0u when a
// bounded wait gave up: a reference into the caller's frame would place
// that frame in local memory.
template <class S, int B>
__device__ __noinline__ unsigned run_item(const GridDev *gp, int k, int strip, int blk, float *ring,
                                          uint64_t *bars, unsigned load_base, int *err, unsigned char *slot) {
  const GridDev &g = *gp;
  auto &p = *reinterpret_cast<Params2D<float, S::kTerms> *>(slot);
  const int lane = threadIdx.x & 31;
  for (int t = lane; t < S::kTerms; t += 32) p.coef[t] = g.coef[t];
  if (lane == 0) {
    p.src = g.base + (long long)(k % 2) * g.plane;
    p.dst = g.base + (long long)((k + 1) % 2) * g.plane;
    p.err = err;
    p.pitch = g.pitch;
    p.d0 = g.d0;
    p.d1 = g.d1;
    p.shift = g.shift;
    p.b = B;
    p.wout = ((128 - 2 * B * S::kRad - 3) / 4) * 4;
    p.nstrips = 0;
    p.nblocks = g.nblocks;
    p.sl = g.sl;
    p.div = g.div;
    p.rdiv = g.rdiv;
    p.eps = g.eps;
    p.divmode = g.divmode;
    p.stash = nullptr;
    p.stash_stride = 0;
  }
  __syncwarp();
  bool ok;
  if constexpr (S::kTerms <= 25) {
    // small parameter sets ride in registers for the whole item
    const Params2D<float, S::kTerms> pl = p;
    ok = warp_item2d<S, float, B, kFma, kStages>(pl, strip, blk, ring, bars, load_base);
  } else {
    ok = warp_item2d<S, float, B, kFma, kStages>(p, strip, blk, ring, bars, load_base);
  }
  __syncwarp();  // the slot is rewritten by the next item
  return ok ? load_base : ~0u;
}

template <class S>
__device__ __forceinline__ bool dispatch_b(const GridDev &g, const Item &it, float *ring, uint64_t *bars,
                                           unsigned &load_base, int *err, unsigned char *slot) {
  constexpr int BS = batch_degree<S>();
  unsigned next = ~0u;
  if (it.b == BS) next = run_item<S, BS>(&g, it.k, it.strip, it.blk, ring, bars, load_base, err, slot);
  if constexpr (BS != 1) {
    if (it.b == 1) next = run_item<S, 1>(&g, it.k, it.strip, it.blk, ring, bars, load_base, err, slot);
  }
  if (next == ~0u) return false;
  load_base = next;
  return true;
}

__device__ __forceinline__ bool dispatch(const GridDev &g, const Item &it, float *ring, uint64_t *bars,
                                         unsigned &load_base, int *err, unsigned char *slot) {
  switch (g.sid) {
#define GBS_CASE(id, S)                                                  \
  case id:                                                               \
    if constexpr (S::kDim == 2)                                          \
      return dispatch_b<S>(g, it, ring, bars, load_base, err, slot);     \
    else                                                                 \
      return false;
    GBS_FOR_EACH_STENCIL(GBS_CASE)
#undef GBS_CASE
    default:
      return false;
  }
}

// One work item on one warp: wait (bounded) until the stream blocks it
// reads have finished the grid's earlier time blocks, run it, count it done.
// False when a wait gave up (the error word says which).
__device__ __forceinline__ bool persistent_item(const Args &a, unsigned idx, float *ring, uint64_t *bars,
                                                unsigned &load_base, unsigned char *slot) {
  const int lane = threadIdx.x & 31;
  const Item it = a.items[idx];
  bool ok = true;
  const GridDev &g = a.grids[it.grid];
  // the counter this item completes, and the ones it waits on: the stream
  // blocks it reads (b*r rows at most past its own, less than one block)
  // and whose readers its writes must follow
  const int cown = g.cbase + (g.ccount > 1 ? it.blk : 0);
  if (lane == 0 && it.need > 0) {
    const unsigned long long t0 = global_ns();
    const int lo = g.ccount > 1 ? max(0, it.blk - 1) : 0;
    const int hi = g.ccount > 1 ? min(g.ccount - 1, it.blk + 1) : 0;
    for (int c = lo; c <= hi && ok; ++c) {
      unsigned spins = 0;
      while (ld_acquire(&a.done[g.cbase + c]) < (unsigned)it.need) {
        if (++spins > 64) {
          __nanosleep(200);
          if (global_ns() - t0 > kWaitLimitNs) {
            atomicOr(a.err, ERR_DEP_TIMEOUT);
            ok = false;
            break;
          }
        }
      }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");
  }
  if (!__all_sync(0xffffffffu, ok)) return false;
  __syncwarp();
  if (!dispatch(g, it, ring, bars, load_base, a.err, slot)) {
    if (lane == 0) atomicOr(a.err, ERR_WAIT_TIMEOUT);
    return false;
  }
  __threadfence();
  __syncwarp();
  if (lane == 0) atomicAdd(&a.done[cown], 1u);
  return true;
}

// Persistent: each CTA takes groups of kWpc consecutive items from an
// atomic counter, warp w running item group * kWpc + w, the way the layered
// schedule's CTAs run consecutive items. Neighbouring items are the same
// stencil and degree (consecutive strips of one stream block), so the CTAs
// resident on an SM mostly run one kernel variant and share its code in the
// instruction cache; warps that took items one at a time mixed variants on
// every SM and stalled on instruction fetch. Groups are taken in order and
// an item waits only on earlier items, whose groups were taken by running
// CTAs: progress does not need every CTA resident.
__global__ void __launch_bounds__(kWpc * 32, kPersistentCtas) batch2d_kernel(const __grid_constant__ Args a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ unsigned s_group;
  __shared__ int s_stop;
  float *ring;
  uint64_t *bars;
  warp_ring2d<float, kWpc, kStages>(smem_raw, ring, bars);
  unsigned char *slot = smem_raw + (size_t)kWpc * kStages * (128 * sizeof(float) + sizeof(uint64_t)) +
                        (size_t)(threadIdx.x >> 5) * kParamSlot;
  unsigned load_base = 0;
  if (threadIdx.x == 0) s_stop = 0;
  while (true) {
    if (threadIdx.x == 0) s_group = atomicAdd(a.next, 1u);
    __syncthreads();
    const unsigned first = s_group * (unsigned)kWpc;
    const bool stop = s_stop != 0 || first >= (unsigned)a.nitems;
    __syncthreads();  // s_group and s_stop are read before they are written again
    if (stop) break;
    const unsigned idx = first + (threadIdx.x >> 5);
    if (idx < (unsigned)a.nitems && !persistent_item(a, idx, ring, bars, load_base, slot) &&
        (threadIdx.x & 31) == 0)
      s_stop = 1;
  }
}

// One time block of every grid: warp w runs item first + w. Kernel
// boundaries order the blocks, so nothing here waits.
__global__ void __launch_bounds__(kWpc * 32, kLayerCtas) batch_layer_kernel(const __grid_constant__ Args a, int first,
                                                                   int count) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const long long gw = (long long)blockIdx.x * kWpc + (threadIdx.x >> 5);
  if (gw >= count) return;
  float *ring;
  uint64_t *bars;
  warp_ring2d<float, kWpc, kStages>(smem_raw, ring, bars);
  unsigned char *slot = smem_raw + (size_t)kWpc * kStages * (128 * sizeof(float) + sizeof(uint64_t)) +
                        (size_t)(threadIdx.x >> 5) * kParamSlot;
  unsigned load_base = 0;
  const Item it = a.items[first + gw];
  if (!dispatch(a.grids[it.grid], it, ring, bars, load_base, a.err, slot) && (threadIdx.x & 31) == 0)
    atomicOr(a.err, ERR_WAIT_TIMEOUT);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int family_degree(int sid) {
  switch (sid) {
#define GBS_DEG(id, S) \
  case id:             \
    return S::kDim == 2 ? batch_degree<S>() : 0;
    GBS_FOR_EACH_STENCIL(GBS_DEG)
#undef GBS_DEG
    default:
      return 0;
  }
}

// time blocks of T steps: blocks of degree bs plus single steps, with as
// many blocks as T has parity (launch k reads plane k%2)
std::vector<int> batch_blocks(int T, int bs) {
  std::vector<int> out;
  if (T <= 0) return out;
  int n = T / bs, r = T - n * bs;
  if (((n + r) - T) % 2 != 0) {  // only possible for even bs
    if (n > 0) {
      --n;
      r += bs;
    }
  }
  for (int i = 0; i < n; ++i) out.push_back(bs);
  for (int i = 0; i < r; ++i) out.push_back(1);
  return out;
}
}  // namespace
}  // namespace gbs

using namespace gbs;

struct gbs_batch {
  gbs::batchdetail::GridDev *d_grids = nullptr;
  gbs::batchdetail::Item *d_items = nullptr;
  unsigned *d_counters = nullptr;  // [0] next, [1..] done per stream block of every grid
  int ncounters = 0;
  int ngrids = 0, nitems = 0, ctas = 0;
  long long cells = 0;             // sum over grids of interior cells * timestep
  size_t smem = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches_plain = 0;          // what per-grid plain launches would need
  long long hbm_bytes = 0;         // algorithmic: each fused launch reads and writes the interior once
  int mode = 0, kernels = 0;
};

#define GBS_BATCH_FN(name) GBS_BATCH_FN2(name, GBS_FMA)
#define GBS_BATCH_FN2(name, m) GBS_BATCH_FN3(name, m)
#define GBS_BATCH_FN3(name, m) name##_##m

extern "C++" gbs_status GBS_BATCH_FN(gbs_batch_build)(const gbs_batch_grid *grids, int ngrids, int mode,
                                                       gbs_batch **out) {
  if (!grids || ngrids <= 0 || !out) return fail(GBS_ERR_INVALID, "batch: no grids");
  std::vector<GridDev> gd(ngrids);
  std::vector<std::vector<int>> blocks(ngrids);
  long long cells = 0;
  for (int g = 0; g < ngrids; ++g) {
    const gbs_batch_grid &bg = grids[g];
    const gbs_stencil_def_t *s = stencil_def(bg.stencil);
    if (!s) return fail(GBS_ERR_INVALID, "batch grid %d: unknown stencil %d", g, bg.stencil);
    if (s->dim != 2)
      return fail(GBS_ERR_UNSUPPORTED, "batch grid %d: the work-item schedules take 2-D grids (use GBS_BATCH_STREAMS)",
                  g);
    if (bg.n[0] < 1 || bg.n[1] < 1 || bg.timestep < 0 || !bg.dev_A)
      return fail(GBS_ERR_INVALID, "batch grid %d: bad extent, timestep or buffer", g);
    if (reinterpret_cast<uintptr_t>(bg.dev_A) % 128 != 0)
      return fail(GBS_ERR_INVALID, "batch grid %d: buffer not 128-byte aligned", g);
    gbs_desc d{};
    d.stencil = bg.stencil;
    d.dtype = GBS_F32;
    d.n[0] = bg.n[0];
    d.n[1] = bg.n[1];
    d.n[2] = 1;
    d.timestep = bg.timestep;
    d.fp_mode = kFma ? GBS_FP_FMA : GBS_FP_EXACT;
    const Layout L = make_layout(&d);
    GridDev &x = gd[g];
    std::memset(&x, 0, sizeof x);
    x.base = static_cast<float *>(bg.dev_A);
    x.pitch = L.pitch;
    x.plane = L.plane;
    x.d0 = L.dims[0];
    x.d1 = L.dims[1];
    x.shift = (int)L.shift;
    x.sid = bg.stencil;
    const int ni = L.dims[0] - 2 * s->rad;
    // stream blocks long enough to amortise an item's start (dependency
    // check, first copies), short enough that a time block's items finish
    // together. Measured on the 512-grid mix: layered 64 / 96 / 128 / 256
    // rows gave 3.00 / 3.01 / 2.98 / 2.47x the per-grid launches, persistent
    // 2.65x at 64 rows and 2.71x at 128.
    x.sl = std::min(ni, mode == GBS_BATCH_LAYERED ? 96 : 128);
    x.nblocks = (ni + x.sl - 1) / x.sl;
    const double div = bg.divisor != 0.0 ? bg.divisor : (double)s->divisor;
    const bool fold = kFma && s->divisor;
    const int nt = s->kind == 1 ? 1 : s->nterms;
    for (int t = 0; t < nt; ++t) {
      double c = bg.coef ? (double)((const float *)bg.coef)[t]
                         : (s->kind == 1 ? (double)s->numerator : (double)s->terms[t].coef);
      x.coef[t] = fold ? (float)(c / div) : (float)c;
    }
    x.div = (float)div;
    x.rdiv = div_reciprocal<float>(div);
    x.eps = (float)s->eps;
    x.divmode = !s->divisor || fold ? 0 : (div_proven_exact(div) ? 2 : 1);
    blocks[g] = batch_blocks(bg.timestep, family_degree(bg.stencil));
    cells += (long long)bg.n[0] * bg.n[1] * bg.timestep;
    // validate every strip window of every degree used
    for (int b : blocks[g]) {
      Geometry2D geo = geometry2d(L, b, x.sl, 0);
      gbs_status st = validate2d(L, geo);
      if (st != GBS_OK) return st;
    }
  }
  // one completion counter per stream block of every grid
  int ncounters = 0;
  for (int g = 0; g < ngrids; ++g) {
    gd[g].cbase = ncounters;
    gd[g].ccount = gd[g].nblocks;
    ncounters += gd[g].nblocks;
  }
  // Items ordered by time block, then stencil, then grid: every grid's
  // blocks stay in order (each item's dependencies come earlier in the
  // list), all grids advance together (the critical path is the longest
  // grid's chain of blocks, not a sum over groups), and warps taking
  // neighbouring items run the same kernel variant (one instruction-cache
  // working set). An item waits until its stream block and the two beside
  // it have finished every earlier time block: `need` counts the items of
  // one stream block in the grid's earlier time blocks.
  std::vector<Item> items;
  std::vector<int> done_before(ngrids, 0);
  size_t kmax = 0;
  for (auto &b : blocks) kmax = std::max(kmax, b.size());
  std::vector<int> layer_start;
  for (size_t k = 0; k < kmax; ++k)
  for (int sid = 0; sid < GBS_NUM_STENCILS; ++sid) {
    if (sid == 0) layer_start.push_back((int)items.size());
    for (int g = 0; g < ngrids; ++g) {
      if (grids[g].stencil != sid || k >= blocks[g].size()) continue;
      const int b = blocks[g][k];
      const gbs_stencil_def_t *s = stencil_def(grids[g].stencil);
      const int wout = ((128 - 2 * b * s->rad - 3) / 4) * 4;
      const int nj = gd[g].d1 - 2 * s->rad;
      const int nstrips = (nj + wout - 1) / wout;
      const int need = done_before[g];
      for (int blk = 0; blk < gd[g].nblocks; ++blk)
        for (int st = 0; st < nstrips; ++st) items.push_back(Item{g, (int)k, b, st, blk, need, 0, 0});
      done_before[g] += nstrips;
    }
  }
  auto *h = new gbs_batch();
  h->ngrids = ngrids;
  h->ncounters = ncounters;
  h->nitems = (int)items.size();
  h->cells = cells;
  for (auto &b : blocks) h->launches_plain += (int)b.size();
  for (int g = 0; g < ngrids; ++g)
    h->hbm_bytes += 2LL * (long long)blocks[g].size() * grids[g].n[0] * grids[g].n[1] * (long long)sizeof(float);
  cudaError_t e;
  if ((e = cudaMalloc(&h->d_grids, sizeof(GridDev) * ngrids)) != cudaSuccess ||
      (e = cudaMalloc(&h->d_items, sizeof(Item) * std::max<size_t>(1, items.size()))) != cudaSuccess ||
      (e = cudaMalloc(&h->d_counters, sizeof(unsigned) * (ncounters + 1))) != cudaSuccess) {
    gbs_batch_destroy(h);
    return cuda_fail(e, "batch: cudaMalloc");
  }
  cudaMemcpy(h->d_grids, gd.data(), sizeof(GridDev) * ngrids, cudaMemcpyHostToDevice);
  if (!items.empty()) cudaMemcpy(h->d_items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice);
  int *err = nullptr;
  gbs_status st = error_word(&err);
  if (st != GBS_OK) {
    gbs_batch_destroy(h);
    return st;
  }
  h->smem = (size_t)kWpc * kStages * (128 * sizeof(float) + sizeof(uint64_t)) + (size_t)kWpc * kParamSlot;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch2d_kernel, kWpc * 32, h->smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  (void)cudaGetLastError();
  // every CTA resident at once (persistent), never more CTAs than warps of work
  h->ctas = std::max(1, std::min(per_sm * sms, (h->nitems + kWpc - 1) / kWpc));

  Args a{};
  a.grids = h->d_grids;
  a.items = h->d_items;
  a.nitems = h->nitems;
  a.next = h->d_counters;
  a.done = h->d_counters + 1;
  a.err = err;
  // capture: reset the counters, then the persistent kernel
  cudaStream_t cs;
  if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) {
    gbs_batch_destroy(h);
    return cuda_fail(e, "batch: stream");
  }
  layer_start.push_back((int)items.size());
  h->mode = mode;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    if (mode == GBS_BATCH_LAYERED) {
      for (size_t k = 0; k + 1 < layer_start.size(); ++k) {
        const int first = layer_start[k], count = layer_start[k + 1] - first;
        if (count <= 0) continue;
        batch_layer_kernel<<<(count + kWpc - 1) / kWpc, kWpc * 32, h->smem, cs>>>(a, first, count);
        ++h->kernels;
      }
    } else {
      cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned) * (ncounters + 1), cs);
      batch2d_kernel<<<h->ctas, kWpc * 32, h->smem, cs>>>(a);
      h->kernels = 1;
    }
    e = cudaStreamEndCapture(cs, &h->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&h->exec, h->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    gbs_batch_destroy(h);
    return cuda_fail(e, "batch: graph capture");
  }
  *out = h;
  return GBS_OK;
}

// ---------------------------------------------------------------------------
// Batched run without allocation, for callers that may not allocate device
// memory. Its scratch (grid table, work list, counters, error word) lives in
// a static device array of this unit, its host staging in static host
// arrays: nothing is allocated per call, on the device or the host.
// ---------------------------------------------------------------------------
namespace gbs {
namespace noalloc {
namespace {  // one copy per unit (exact and FMA mode each have their own)
constexpr int kMaxGrids = GBS_NOALLOC_MAX_GRIDS;
constexpr int kMaxItems = GBS_NOALLOC_MAX_ITEMS;

struct Scratch {
  GridDev grids[kMaxGrids];
  Item items[kMaxItems];
  unsigned counters[kMaxGrids + 1];  // [0] next item, [1 + g] items of grid g done
  int err;                           // error bits of the kernel
};

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char scratch[sizeof(Scratch)];

std::mutex mu;                       // one call at a time: one staging area
GridDev h_grids[kMaxGrids];
Item h_items[kMaxItems];
void *dev_scratch[64];               // address of `scratch` per device

// Time blocks of grid g: `full` blocks of degree bs, then single steps, with
// as many blocks as T has parity (the same split as batch_blocks).
void split_blocks(int T, int bs, int &full, int &single) {
  full = T > 0 ? T / bs : 0;
  single = T > 0 ? T - full * bs : 0;
  if (T > 0 && ((full + single) - T) % 2 != 0 && full > 0) {
    --full;
    single += bs;
  }
}

gbs_status run(const gbs_batch_grid *grids, int ngrids, cudaStream_t stream) {
  if (!grids || ngrids <= 0) return fail(GBS_ERR_INVALID, "batch (no allocation): no grids");
  {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess) {
      (void)cudaGetLastError();
      cap = cudaStreamCaptureStatusNone;
    }
    if (cap != cudaStreamCaptureStatusNone)
      return fail(GBS_ERR_INVALID, "batch (no allocation): the call synchronises its stream and cannot be captured");
  }
  if (ngrids > kMaxGrids)
    return fail(GBS_ERR_INVALID, "batch (no allocation): %d grids, at most %d fit its static scratch", ngrids,
                kMaxGrids);
  std::lock_guard<std::mutex> lk(mu);
  int kmax = 0;
  for (int g = 0; g < ngrids; ++g) {
    const gbs_batch_grid &bg = grids[g];
    const gbs_stencil_def_t *s = stencil_def(bg.stencil);
    if (!s) return fail(GBS_ERR_INVALID, "batch grid %d: unknown stencil %d", g, bg.stencil);
    if (s->dim != 2) return fail(GBS_ERR_UNSUPPORTED, "batch grid %d: the run without allocation takes 2-D grids", g);
    if (bg.n[0] < 1 || bg.n[1] < 1 || bg.timestep < 0 || !bg.dev_A)
      return fail(GBS_ERR_INVALID, "batch grid %d: bad extent, timestep or buffer", g);
    if (reinterpret_cast<uintptr_t>(bg.dev_A) % 128 != 0)
      return fail(GBS_ERR_INVALID, "batch grid %d: buffer not 128-byte aligned", g);
    gbs_desc d{};
    d.stencil = bg.stencil;
    d.dtype = GBS_F32;
    d.n[0] = bg.n[0];
    d.n[1] = bg.n[1];
    d.n[2] = 1;
    d.timestep = bg.timestep;
    d.fp_mode = kFma ? GBS_FP_FMA : GBS_FP_EXACT;
    const Layout L = make_layout(&d);
    GridDev &x = h_grids[g];
    std::memset(&x, 0, sizeof x);
    x.base = static_cast<float *>(bg.dev_A);
    x.pitch = L.pitch;
    x.plane = L.plane;
    x.d0 = L.dims[0];
    x.d1 = L.dims[1];
    x.shift = (int)L.shift;
    x.sid = bg.stencil;
    const int ni = L.dims[0] - 2 * s->rad;
    x.sl = std::min(ni, 128);
    x.nblocks = (ni + x.sl - 1) / x.sl;
    x.cbase = g;  // one counter per grid: the scratch holds ngrids + 1
    x.ccount = 1;
    const double div = bg.divisor != 0.0 ? bg.divisor : (double)s->divisor;
    const bool fold = kFma && s->divisor;
    const int nt = s->kind == 1 ? 1 : s->nterms;
    for (int t = 0; t < nt; ++t) {
      const double c = bg.coef ? (double)((const float *)bg.coef)[t]
                               : (s->kind == 1 ? (double)s->numerator : (double)s->terms[t].coef);
      x.coef[t] = fold ? (float)(c / div) : (float)c;
    }
    x.div = (float)div;
    x.rdiv = div_reciprocal<float>(div);
    x.eps = (float)s->eps;
    x.divmode = !s->divisor || fold ? 0 : (div_proven_exact(div) ? 2 : 1);
    int full, single;
    split_blocks(bg.timestep, family_degree(bg.stencil), full, single);
    kmax = std::max(kmax, full + single);
    for (int b : {family_degree(bg.stencil), 1}) {
      gbs_status st = validate2d(L, geometry2d(L, b, x.sl, 0));
      if (st != GBS_OK) return st;
    }
  }
  // work items in time-block order, as the planned batch orders them
  int nitems = 0;
  int done_before[kMaxGrids] = {0};
  for (int k = 0; k < kmax; ++k)
    for (int sid = 0; sid < GBS_NUM_STENCILS; ++sid)
      for (int g = 0; g < ngrids; ++g) {
        if (grids[g].stencil != sid) continue;
        const int bs = family_degree(sid);
        int full, single;
        split_blocks(grids[g].timestep, bs, full, single);
        if (k >= full + single) continue;
        const int b = k < full ? bs : 1;
        const gbs_stencil_def_t *s = stencil_def(sid);
        const int wout = ((128 - 2 * b * s->rad - 3) / 4) * 4;
        const int nstrips = (h_grids[g].d1 - 2 * s->rad + wout - 1) / wout;
        const int count = nstrips * h_grids[g].nblocks;
        if (nitems + count > kMaxItems)
          return fail(GBS_ERR_INVALID,
                      "batch (no allocation): more than %d work items do not fit its static scratch "
                      "(use gbs_batch_plan for larger batches)",
                      kMaxItems);
        for (int blk = 0; blk < h_grids[g].nblocks; ++blk)
          for (int st = 0; st < nstrips; ++st) h_items[nitems++] = Item{g, k, b, st, blk, done_before[g], 0, 0};
        done_before[g] += count;
      }
  if (nitems == 0) return GBS_OK;

  // set-up, once per device, with that device current: the device address
  // of the static scratch (its name in host code is only a stand-in)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "batch (no allocation): cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_NODEVICE, "device ordinal %d unsupported", dev);
  if (!dev_scratch[dev]) {
    void *ptr = nullptr;
    if ((e = cudaGetSymbolAddress(&ptr, scratch)) != cudaSuccess)
      return cuda_fail(e, "batch (no allocation): cudaGetSymbolAddress");
    dev_scratch[dev] = ptr;
  }
  Scratch *sc = static_cast<Scratch *>(dev_scratch[dev]);

  // stage the tables, clear the counters and the error word
  if ((e = cudaMemcpyAsync(sc->grids, h_grids, sizeof(GridDev) * ngrids, cudaMemcpyHostToDevice, stream)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(sc->items, h_items, sizeof(Item) * nitems, cudaMemcpyHostToDevice, stream)) !=
          cudaSuccess ||
      (e = cudaMemsetAsync(sc->counters, 0, sizeof(unsigned) * (ngrids + 1), stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(&sc->err, 0, sizeof(int), stream)) != cudaSuccess)
    return cuda_fail(e, "batch (no allocation): staging");
  Args a{};
  a.grids = sc->grids;
  a.items = sc->items;
  a.nitems = nitems;
  a.next = sc->counters;
  a.done = sc->counters + 1;
  a.err = &sc->err;
  const size_t smem = (size_t)kWpc * kStages * (128 * sizeof(float) + sizeof(uint64_t)) + (size_t)kWpc * kParamSlot;
  int per_sm = 0, sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch2d_kernel, kWpc * 32, smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  (void)cudaGetLastError();
  const int ctas = std::max(1, std::min(per_sm * std::max(sms, 1), (nitems + kWpc - 1) / kWpc));
  batch2d_kernel<<<ctas, kWpc * 32, smem, stream>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "batch (no allocation): launch");
  // wait, and turn the kernel's error bits into a status
  int herr = 0;
  if ((e = cudaMemcpyAsync(&herr, &sc->err, sizeof(int), cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(stream)) != cudaSuccess)
    return cuda_fail(e, "batch (no allocation): completion");
  if (herr) return fail(GBS_ERR_TIMEOUT, "batch (no allocation): a device-side wait gave up (bits 0x%x)", herr);
  return GBS_OK;
}
}  // namespace
}  // namespace noalloc
}  // namespace gbs

extern "C++" gbs_status GBS_BATCH_FN(gbs_batch_run_noalloc)(const gbs_batch_grid *grids, int ngrids,
                                                             cudaStream_t stream) {
  return gbs::noalloc::run(grids, ngrids, stream);
}

#if GBS_FMA
// The C ABI entry points live in the FMA unit; they dispatch on fp_mode.
extern "C++" gbs_status gbs_batch_build_0(const gbs_batch_grid *, int, int, gbs_batch **);
extern "C++" gbs_status gbs_batch_run_noalloc_0(const gbs_batch_grid *, int, cudaStream_t);

namespace gbs {
namespace {
// GBS_BATCH_STREAMS: each grid's own time loop (the engine's plain kernels at
// the tuned degree) captured as a chain of kernel nodes; the chains are
// spread over kStreams capture streams (branches of the graph), heaviest
// first onto the least loaded one, so independent grids run side by side.
// One graph launch. GBS_BATCH_BRANCHES (environment, 1..64) overrides
// kStreams; GBS_BATCH_SHARE=1 sizes each grid's stream length for a
// branch's share of the GPU instead of a whole wave.
constexpr int kStreams = 16;
constexpr int kMaxStreams = 64;

int branches() {
  const char *e = std::getenv("GBS_BATCH_BRANCHES");
  const int n = e ? std::atoi(e) : kStreams;
  return n >= 1 && n <= kMaxStreams ? n : kStreams;
}

gbs_status build_streams(const gbs_batch_grid *grids, int ngrids, int dtype, int fp_mode, gbs_batch **out) {
  if (!grids || ngrids <= 0) return fail(GBS_ERR_INVALID, "batch: no grids");
  const int nbr = branches();
  std::vector<gbs_desc> ds(ngrids);
  std::vector<double> work(ngrids);
  long long cells = 0, hbm = 0;
  int launches = 0;
  for (int g = 0; g < ngrids; ++g) {
    const gbs_batch_grid &bg = grids[g];
    const gbs_stencil_def_t *s = stencil_def(bg.stencil);
    if (!s) return fail(GBS_ERR_INVALID, "batch grid %d: unknown stencil %d", g, bg.stencil);
    if (bg.n[0] < 1 || bg.n[1] < 1 || (s->dim == 3 && bg.n[2] < 1) || bg.timestep < 0 || !bg.dev_A)
      return fail(GBS_ERR_INVALID, "batch grid %d: bad extent, timestep or buffer", g);
    if (reinterpret_cast<uintptr_t>(bg.dev_A) % 128 != 0)
      return fail(GBS_ERR_INVALID, "batch grid %d: buffer not 128-byte aligned", g);
    gbs_desc &d = ds[g];
    d = gbs_desc{};
    d.stencil = bg.stencil;
    d.dtype = dtype;
    d.n[0] = bg.n[0];
    d.n[1] = bg.n[1];
    d.n[2] = s->dim == 3 ? bg.n[2] : 1;
    d.timestep = bg.timestep;
    d.fp_mode = fp_mode;
    d.coef = bg.coef;
    d.divisor = bg.divisor;
    gbs_status st = check_desc(&d);
    if (st != GBS_OK) return st;
    gbs_plan_info pi;
    if ((st = gbs_plan(&d, &pi)) != GBS_OK) return st;
    // GBS_BATCH_SHARE=1: stream length for this grid's share of one wave
    // (default: the single-grid choice, one whole wave per kernel, which
    // measured faster on GB300: 254 vs 220 GCells/s at 16 branches)
    d.bt = pi.bt;
    const char *share_env = std::getenv("GBS_BATCH_SHARE");
    if (s->dim == 2 && d.sl == 0 && share_env && share_env[0] == '1') {
      const Layout L = make_layout(&d);
      const int fma = fp_mode == GBS_FP_FMA ? 1 : 0;
      const long long share = std::max<long long>(1, resident_warps_2d(d.stencil, dtype, fma, pi.bt) / nbr);
      d.sl = geometry2d(L, pi.bt, 0, share).sl;
      if ((st = gbs_plan(&d, &pi)) != GBS_OK) return st;
    }
    launches += pi.launches;
    const long long area = (long long)d.n[0] * d.n[1] * (s->dim == 3 ? d.n[2] : 1);
    cells += area * bg.timestep;
    hbm += 2LL * pi.launches * area * (dtype == GBS_F64 ? 8 : 4);
    work[g] = (double)area * bg.timestep;
  }
  int *err = nullptr;
  gbs_status st = error_word(&err);
  if (st != GBS_OK) return st;
  std::vector<int> order(ngrids);
  for (int g = 0; g < ngrids; ++g) order[g] = g;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  auto *h = new gbs_batch();
  h->ngrids = ngrids;
  h->cells = cells;
  h->launches_plain = launches;
  h->hbm_bytes = hbm;
  h->mode = GBS_BATCH_STREAMS;
  cudaStream_t cs = nullptr, side[kMaxStreams] = {};
  cudaEvent_t fork = nullptr, join[kMaxStreams] = {};
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  for (int k = 0; k < nbr && e == cudaSuccess; ++k) e = cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
  for (int k = 0; k < nbr && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming);
  auto release = [&]() {
    for (int k = 0; k < kMaxStreams; ++k) {
      if (join[k]) cudaEventDestroy(join[k]);
      if (side[k]) cudaStreamDestroy(side[k]);
    }
    if (fork) cudaEventDestroy(fork);
    if (cs) cudaStreamDestroy(cs);
  };
  if (e != cudaSuccess) {
    release();
    delete h;
    return cuda_fail(e, "batch: streams");
  }
  st = GBS_OK;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaEventRecord(fork, cs);
    for (int k = 0; k < nbr; ++k) cudaStreamWaitEvent(side[k], fork, 0);
    double load[kMaxStreams] = {};
    for (int g : order) {
      const int k = (int)(std::min_element(load, load + nbr) - load);
      load[k] += work[g];
      const Layout L = make_layout(&ds[g]);
      st = run_loop(&ds[g], L, grids[g].dev_A, side[k], err);
      if (st != GBS_OK) break;
    }
    for (int k = 0; k < nbr; ++k) {
      cudaEventRecord(join[k], side[k]);
      cudaStreamWaitEvent(cs, join[k], 0);
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cs, &graph);
    h->graph = graph;
  }
  if (st == GBS_OK && e == cudaSuccess) e = cudaGraphInstantiate(&h->exec, h->graph, 0);
  release();
  if (st != GBS_OK || e != cudaSuccess) {
    gbs_batch_destroy(h);
    return st != GBS_OK ? st : cuda_fail(e, "batch: graph capture");
  }
  h->kernels = launches;
  h->nitems = launches;
  *out = h;
  return GBS_OK;
}
}  // namespace
}  // namespace gbs

extern "C" {
gbs_status gbs_batch_plan(const gbs_batch_grid *grids, int ngrids, int dtype, int fp_mode, int mode,
                          gbs_batch **out) {
  if (mode != GBS_BATCH_PERSISTENT && mode != GBS_BATCH_LAYERED && mode != GBS_BATCH_STREAMS)
    return fail(GBS_ERR_INVALID, "bad batch mode");
  if (dtype != GBS_F32 && dtype != GBS_F64) return fail(GBS_ERR_INVALID, "bad dtype");
  if (dtype != GBS_F32 && mode != GBS_BATCH_STREAMS)
    return fail(GBS_ERR_UNSUPPORTED, "the work-item schedules take GBS_F32 grids (use GBS_BATCH_STREAMS)");
  if (fp_mode != GBS_FP_EXACT && fp_mode != GBS_FP_FMA) return fail(GBS_ERR_INVALID, "bad fp_mode");
  if (!out) return fail(GBS_ERR_INVALID, "out is NULL");
  gbs_batch *h = nullptr;
  gbs_status st;
  if (mode == GBS_BATCH_STREAMS) st = build_streams(grids, ngrids, dtype, fp_mode, &h);
  else st = fp_mode == GBS_FP_FMA ? gbs_batch_build_1(grids, ngrids, mode, &h)
                                  : gbs_batch_build_0(grids, ngrids, mode, &h);
  *out = h;
  return st;
}

gbs_status gbs_batch_run(gbs_batch *plan, void *stream) {
  auto *h = plan;
  if (!h || !h->exec) return fail(GBS_ERR_INVALID, "batch plan is NULL");
  cudaError_t e = cudaGraphLaunch(h->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "batch: graph launch");
  return GBS_OK;
}

gbs_status gbs_batch_info(const gbs_batch *plan, gbs_batch_stats *out) {
  auto *h = plan;
  if (!h || !out) return fail(GBS_ERR_INVALID, "NULL argument");
  out->grids = h->ngrids;
  out->items = h->nitems;
  out->ctas = h->ctas;
  out->cell_updates = h->cells;
  out->plain_launches = h->launches_plain;
  out->kernels = h->kernels;
  out->mode = h->mode;
  out->hbm_bytes = h->hbm_bytes;
  return GBS_OK;
}

gbs_status gbs_batch_run_noalloc(const gbs_batch_grid *grids, int ngrids, int fp_mode, void *stream) {
  if (fp_mode == GBS_FP_FMA) return gbs_batch_run_noalloc_1(grids, ngrids, (cudaStream_t)stream);
  if (fp_mode == GBS_FP_EXACT) return gbs_batch_run_noalloc_0(grids, ngrids, (cudaStream_t)stream);
  return fail(GBS_ERR_INVALID, "bad fp_mode");
}

void gbs_batch_destroy(gbs_batch *plan) {
  auto *h = plan;
  if (!h) return;
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->d_grids) cudaFree(h->d_grids);
  if (h->d_items) cudaFree(h->d_items);
  if (h->d_counters) cudaFree(h->d_counters);
  delete h;
}
}  // extern "C"
#endif
