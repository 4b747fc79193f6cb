// 2-D temporally-blocked stencil kernel family (sm_103a).
//
// Replaces the AN5D-generated 2-D kernels kernel0_<b> (e.g.
// compiled/float/star2d1r-256-10-256_kernel.cu:4..3488) and computes what
// the artifact's scop loop computes (star2d1r.c:14-24 and the other 2-D
// sources): b Jacobi steps of A[(t+1)%2][i][j] = f(A[t%2][neighbourhood]) on
// the interior, the halo held fixed.
//
// Work decomposition. One WARP is the unit of work; warps never wait on each
// other. A warp owns a strip of output columns [cs, ce) (wout wide) and a
// block of output rows [i0, i1) (sl long). It streams level-0 rows
// i0-b*r .. i1-1+b*r through a per-warp ring of NSTAGE shared-memory row
// buffers filled by bulk-async (TMA) copies, one 32*V-element window row per
// copy (V = 16 bytes / element size, 512 bytes per copy). Lane l holds window
// elements [l*V, l*V+V).
//
// Per fused time level l (1..b) the warp keeps a (2r+1)-row register window.
// At pipeline step p (level-0 row p arrives) level l produces row p - l*r,
// which feeds level l+1 in the same step; level b's row p - b*r is stored if
// it lies in [i0, i1). Row neighbours at other column offsets come from the
// neighbouring lanes by shuffles. The window's edge lanes (b*r columns at
// each side) lose accuracy level by level; they are the overlap that
// neighbouring strips compute for real (overlapped tiling), so no warp ever
// needs another warp's result.
//
// Two evaluation forms, chosen per stencil by the tap-table generator:
//  * direct: the window holds the input rows; each output is one chain over
//    the terms in source order. Used for stars, gradient2d and star2d4r.
//  * assoc:  the window holds partial sums of the 2r+1 outputs in flight;
//    each arriving row adds its terms to every output it touches. Used for
//    stencils whose source groups the terms by ascending row (the boxes,
//    j2d9pt-gol), where the partial sums are built in exactly the source
//    order, so both forms give the same bits.
//
// Halo cells (rows/columns within r of the grid edge) carry their input
// value through every level, like the reference's untouched halo.
#pragma once
#include "gbs_device.cuh"
#include "gbs_launch.h"
#include "stencil_table.cuh"

namespace gbs {

template <typename T, int NT> struct Params2D {
  const T *src;        // plane read (row 0, element 0 of the padded row)
  T *dst;              // plane written
  int *err;            // error word (bounded waits)
  long long pitch;     // elements per padded row
  int d0, d1;          // dimsize: rows, columns (interior + 2r)
  int shift;           // column c is stored at element shift + c
  int b;               // time levels fused in this launch (the kernel's B)
  int wout;            // output columns per strip (multiple of V)
  int nstrips, nblocks, sl;
  T coef[NT];
  T div, rdiv, eps;    // divisor, RN(1/divisor), gradient epsilon
  int divmode;         // 0: no division (folded into coef), 1: checked, 2: proven fast path
  T *stash;            // stash-mode kernels: level l < b also stores its interior cells to
  long long stash_stride;  // stash + (l-1)*stash_stride (the states between)
};

// y / div as the params ask (see div_by / div_by_fast)
template <typename T, int NT>
__device__ __forceinline__ T apply_div(T y, const Params2D<T, NT> &p) {
  if constexpr (sizeof(T) == 4) {
    if (p.divmode == 2) return div_by_fast(y, p.div, p.rdiv);
  }
  if (p.divmode == 0) return y;
  return div_by(y, p.div, p.rdiv);
}

// Compile-time facts about a stencil's term list.
template <class ST, int V> struct Tap2 {
  static constexpr int R = ST::kRad;
  static constexpr int NT = ST::kTerms;
  // does some term read row offset di at element x (x relative to the lane's
  // first element, x in [-R, V+R))?
  __host__ __device__ static constexpr bool need(int di, int x) {
    if (ST::kKind == KIND_GRADIENT && di == 0 && x >= 0 && x < V) return true;
    for (int t = 0; t < NT; ++t)
      if (ST::kOff[t][0] == di) {
        const int e = x - ST::kOff[t][1];
        if (e >= 0 && e < V) return true;
      }
    return false;
  }
  __host__ __device__ static constexpr bool row_has_dj(int di) {
    for (int t = 0; t < NT; ++t)
      if (ST::kOff[t][0] == di && ST::kOff[t][1] != 0) return true;
    if (ST::kKind == KIND_GRADIENT) return false;
    return false;
  }
};

// ext[R + x] = row element x, x in [-R, V+R), for the x some term needs.
template <class ST, int V, int DI, typename T>
__device__ __forceinline__ void extend_row(T (&ext)[V + 2 * ST::kRad], const T (&row)[V]) {
  constexpr int R = ST::kRad;
  static_for<V + 2 * R>([&](auto XI) {
    constexpr int x = decltype(XI)::value - R;
    if constexpr (Tap2<ST, V>::need(DI, x)) ext[R + x] = row_elem<V, x>(row);
  });
}


// One fused time level: the level-(l) row x arrives, the level-(l+1) row q
// leaves in x. CAREFUL handles halo rows and columns (grid edges);
// otherwise the caller guarantees that every row and column is interior.
// Level-0 rows a warp's ring keeps after they arrive: the assoc form carries
// halo cells of row q (up to b*r rows back) from the ring; the direct form
// carries them from its register window.
template <class ST, int B> constexpr int ring_keep2d() { return ST::kAssoc ? B * ST::kRad : 0; }

// Where an assoc-form level finds the fixed halo values of row q: the warp's
// ring, which still holds level-0 row q (load index q - pstart). Reading
// them there costs a shared-memory load instead of a memory round trip in
// every step of a warp at the grid's edge.
template <typename T, int NSTAGE> struct CarryRing {
  const T *ring;        // the warp's ring + lane * V
  unsigned base;        // the item's first load index on the ring
  int pstart;           // row of load index 0
  int nrows;            // rows loaded by the item
  __device__ __forceinline__ const T *row(int q) const {
    const int n = q - pstart;
    return (n >= 0 && n < nrows) ? ring + (size_t)((base + (unsigned)n) % NSTAGE) * (32 * (16 / sizeof(T)))
                                 : nullptr;
  }
};

template <class ST, typename T, bool FMA, bool UNR, bool CAREFUL, int PH, int V, int NSTAGE>
__device__ __forceinline__ void level2d(T (&win)[2 * ST::kRad + 1][V], T (&x)[V], int q, bool edge,
                                        int col0, const CarryRing<T, NSTAGE> &carry,
                                        const Params2D<T, ST::kTerms> &p) {
  constexpr int R = ST::kRad;
  constexpr int W = 2 * R + 1;
  using A = Arith<T>;
  T y[V];
  bool halo_row = false;
  if constexpr (CAREFUL) halo_row = (q < R) || (q >= p.d0 - R);
  if constexpr (!ST::kAssoc) {
#pragma unroll
    for (int e = 0; e < V; ++e) win[wslot<UNR, W>(PH, 2 * R)][e] = x[e];
    constexpr int cslot = wslot<UNR, W>(PH, R);
    if (CAREFUL && halo_row) {
#pragma unroll
      for (int e = 0; e < V; ++e) y[e] = win[cslot][e];
    } else {
      if constexpr (ST::kKind == KIND_GRADIENT) {
        T ext[V + 2 * R];
        extend_row<ST, V, 0>(ext, win[cslot]);
        static_for<V>([&](auto EI) {
          constexpr int e = decltype(EI)::value;
          T nb[ST::kTerms];
          static_for<ST::kTerms>([&](auto TI) {
            constexpr int t = decltype(TI)::value;
            constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
            if constexpr (di == 0) nb[t] = ext[R + e + dj];
            else nb[t] = win[wslot<UNR, W>(PH, R + di)][e];
          });
          y[e] = gradient_update<T, ST::kTerms, FMA>(win[cslot][e], nb, p.eps, p.coef[0]);
        });
      } else {
        // the direct form serves stencils whose off-centre rows are read at
        // the centre column only (stars, star2d4r): one extended row
        T ext[V + 2 * R];
        extend_row<ST, V, 0>(ext, win[cslot]);
        static_for<ST::kTerms>([&](auto TI) {
          constexpr int t = decltype(TI)::value;
          constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
          static_assert(di == 0 || dj == 0, "direct 2-D form expects off-centre rows at dj == 0");
          constexpr int slot = wslot<UNR, W>(PH, R + di);
          static_for<V>([&](auto EI) {
            constexpr int e = decltype(EI)::value;
            T a;
            if constexpr (dj == 0) a = win[slot][e];
            else a = ext[R + e + dj];
            if constexpr (t == 0) y[e] = A::mul(p.coef[t], a);
            else y[e] = term_next<T, FMA>(y[e], p.coef[t], a);
          });
        });
        if constexpr (ST::kHasDiv && !FMA) {  // FMA mode: folded into the coefficients
#pragma unroll
          for (int e = 0; e < V; ++e) y[e] = apply_div(y[e], p);
        }
      }
      if (CAREFUL && edge) {
#pragma unroll
        for (int e = 0; e < V; ++e)
          if (col0 + e < R || col0 + e >= p.d1 - R) y[e] = win[cslot][e];
      }
    }
  } else {
    // assoc: the arriving row m = q + R adds its terms to outputs q..q+2R
    T ext[V + 2 * R];
    static_for<V + 2 * R>([&](auto XI) {
      constexpr int xx = decltype(XI)::value - R;
      constexpr bool any = [] {
        for (int di = -R; di <= R; ++di)
          if (Tap2<ST, V>::need(di, xx)) return true;
        return false;
      }();
      if constexpr (any) ext[R + xx] = row_elem<V, xx>(x);
    });
    static_for<ST::kTerms>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
      constexpr int slot = wslot<UNR, W>(PH, R - di);
      static_for<V>([&](auto EI) {
        constexpr int e = decltype(EI)::value;
        const T a = ext[R + e + dj];
        if constexpr (t == 0) win[slot][e] = A::mul(p.coef[t], a);
        else win[slot][e] = term_next<T, FMA>(win[slot][e], p.coef[t], a);
      });
    });
    constexpr int oslot = wslot<UNR, W>(PH, 0);
#pragma unroll
    for (int e = 0; e < V; ++e) y[e] = win[oslot][e];
    if constexpr (ST::kHasDiv && !FMA) {  // FMA mode: folded into the coefficients
#pragma unroll
      for (int e = 0; e < V; ++e) y[e] = apply_div(y[e], p);
    }
    if constexpr (CAREFUL) {
      if (halo_row || edge) {
        const T *c = (q >= 0 && q < p.d0) ? carry.row(q) : nullptr;
        if (c) {
          T cv[V];
          ld_vec<T, V>(cv, c);
#pragma unroll
          for (int e = 0; e < V; ++e)
            if (halo_row || col0 + e < R || col0 + e >= p.d1 - R) y[e] = cv[e];
        }
      }
    }
  }
  if constexpr (!UNR) {
#pragma unroll
    for (int j = 0; j < 2 * R; ++j)
#pragma unroll
      for (int e = 0; e < V; ++e) win[j][e] = win[j + 1][e];
  }
#pragma unroll
  for (int e = 0; e < V; ++e) x[e] = y[e];
}

// One work item of a warp: output columns [cs, ce) of strip `strip` and
// output rows [i0, i1) of stream block `blk`, advanced by B levels from p.src
// into p.dst. `ring`/`bars` are the warp's NSTAGE row buffers and their
// mbarriers (initialised by the caller); `load_base` counts the copies this
// warp has issued on them so far, so that items can follow each other on the
// same barriers. Returns false when a bounded wait gave up (p.err is set and
// the copies in flight have been drained).
// STASH: the intermediate levels also store their rows (the states after 1
// .. B-1 steps) in the item's output rows and columns, where every level is
// valid, to p.stash; a separate instantiation, so that the plain kernels
// carry none of it.
template <class ST, typename T, int B, bool FMA, int NSTAGE, bool STASH = false>
__device__ __forceinline__ bool warp_item2d(const Params2D<T, ST::kTerms> &p, int strip, int blk, T *ring,
                                            uint64_t *bars, unsigned &load_base) {
  constexpr int V = 16 / sizeof(T);
  constexpr int R = ST::kRad;
  constexpr int W = 2 * R + 1;
  constexpr bool UNR = (R <= 2);
  constexpr int NPH = UNR ? W : 1;
  constexpr int ROW = 32 * V;
  constexpr unsigned ROW_BYTES = ROW * sizeof(T);
  const int lane = threadIdx.x & 31;

  // ---- columns (column space c; offset space c + shift) ----
  const int cs = R + strip * p.wout;
  const int ce = min(cs + p.wout, p.d1 - R);
  const int need_lo = max(0, cs - B * R);
  const int ws = ((need_lo + p.shift) / V) * V;
  const int col0 = ws - p.shift + lane * V;  // column of this lane's element 0
  const bool edge = (ws - p.shift < R) || (ws - p.shift + ROW > p.d1 - R);
  const bool store_all = (col0 >= cs && col0 + V <= ce);

  // ---- rows ----
  const int i0 = R + blk * p.sl;
  const int i1 = min(i0 + p.sl, p.d0 - R);
  const int pstart = max(0, i0 - B * R);
  const int pend = min(p.d0, i1 + B * R);  // rows loaded: [pstart, pend)
  const int plast = i1 - 1 + B * R;        // last pipeline step
  const int nload = pend - pstart;

  const T *src_win = p.src + ws;
  T *dst_lane = p.dst + ws + lane * V;
  const long long pitch = p.pitch;
  const unsigned base = load_base;
  constexpr int KEEP = ring_keep2d<ST, B>();
  static_assert(KEEP + 2 <= NSTAGE, "the ring must keep b*r rows and still prefetch");
  const CarryRing<T, NSTAGE> carry{ring + lane * V, base, pstart, nload};

  if (lane == 0) {
#pragma unroll 1
    for (int n = 0; n < NSTAGE && n < nload; ++n) {
      const unsigned s = (base + n) % NSTAGE;
      mbar_arrive_expect_tx(&bars[s], ROW_BYTES);
      bulk_g2s(ring + s * ROW, src_win + (long long)(pstart + n) * p.pitch, ROW_BYTES, &bars[s]);
    }
  }
  __syncwarp();

  T win[B][W][V];
#pragma unroll
  for (int l = 0; l < B; ++l)
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
      for (int e = 0; e < V; ++e) win[l][w][e] = T(0);

  int consumed = 0;  // loads consumed so far (for the drain on timeout)
  bool ok = true;

  // One pipeline step at row pp with phase PH. CAREFUL steps handle the
  // stream ends, halo rows and edge columns; the others assume none occur.
  auto step = [&](auto PHI, auto CAREI, int pp) GBS_INL {
    constexpr int ph = decltype(PHI)::value;
    constexpr bool careful = decltype(CAREI)::value;
    T x[V];
    if (!careful || pp < pend) {
      const int n = pp - pstart;
      const unsigned gn = base + n;
      const unsigned s = gn % NSTAGE;
      // every lane waits; the decision to give up is warp-uniform
      const bool got = mbar_wait(&bars[s], (gn / NSTAGE) & 1u, nullptr, 0);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) atomicOr(p.err, ERR_WAIT_TIMEOUT);
        ok = false;
        return;
      }
      ld_vec<T, V>(x, ring + s * ROW + lane * V);
      consumed = n + 1;
    } else {
#pragma unroll
      for (int e = 0; e < V; ++e) x[e] = T(0);
    }
    static_for<B>([&](auto LI) {
      constexpr int l = decltype(LI)::value;
      level2d<ST, T, FMA, UNR, careful, ph, V, NSTAGE>(win[l], x, pp - (l + 1) * R, edge, col0, carry, p);
      if constexpr (STASH && l + 1 < B) {
        const int ql = pp - (l + 1) * R;
        if (ql >= i0 && ql < i1) {
          T *d = p.stash + (long long)l * p.stash_stride + ws + lane * V + (long long)ql * pitch;
          if (store_all) {
            st_vec_global<T, V>(d, x);
          } else {
#pragma unroll
            for (int e = 0; e < V; ++e)
              if (col0 + e >= cs && col0 + e < ce) st_global(d + e, x[e]);
          }
        }
      }
    });
    const int q = pp - B * R;
    if (q >= i0 && q < i1) {
      T *d = dst_lane + (long long)q * pitch;
      if (store_all) {
        st_vec_global<T, V>(d, x);
      } else {
#pragma unroll
        for (int e = 0; e < V; ++e)
          if (col0 + e >= cs && col0 + e < ce) st_global(d + e, x[e]);
      }
    }
    // the row KEEP steps back is no longer needed: refill its stage
    const int nf = pp - pstart - KEEP;
    if (nf >= 0 && nf + NSTAGE < nload) {
      __syncwarp();
      if (lane == 0) {
        const unsigned sf = (base + nf) % NSTAGE;
        mbar_arrive_expect_tx(&bars[sf], ROW_BYTES);
        bulk_g2s(ring + sf * ROW, src_win + (long long)(pstart + nf + NSTAGE) * pitch, ROW_BYTES, &bars[sf]);
      }
    }
  };

  // steps [lo, hi) in whole groups of NPH phases, starting at a group boundary
  auto run = [&](int lo, int hi, auto CAREI) GBS_INL {
#pragma unroll 1
    for (int pb = lo; pb < hi && ok; pb += NPH) {
      static_for<NPH>([&](auto PHI) {
        const int pp = pb + decltype(PHI)::value;
        if (!ok || (decltype(CAREI)::value && pp >= hi)) return;
        step(PHI, CAREI, pp);
      });
    }
  };
  const int steps = plast + 1 - pstart;
  if (edge) {
    run(pstart, plast + 1, IC<1>());
  } else {
    // rows whose levels all lie in the interior and that are loaded
    const int mid_lo = max(pstart, (B + 1) * R);
    const int mid_hi = min(plast + 1, p.d0);
    int a = pstart + (mid_lo - pstart + NPH - 1) / NPH * NPH;
    int z = pstart + max(0, mid_hi - pstart) / NPH * NPH;
    if (a > z) a = z = pstart + steps;  // no interior stretch: all careful
    run(pstart, min(a, plast + 1), IC<1>());
    if (a < z) run(a, z, IC<0>());
    if (z < plast + 1) run(z, plast + 1, IC<1>());
  }

  if (!ok) {
    if (lane == 0) {
      // Timed out: wait (bounded) for the copies still in flight into this
      // warp's ring before the CTA may exit and release its shared memory.
      const int issued = min(nload, max(NSTAGE, consumed + NSTAGE - KEEP));
      for (int n = consumed; n < issued; ++n) {
        const unsigned gn = base + n;
        if (!mbar_wait(&bars[gn % NSTAGE], (gn / NSTAGE) & 1u, p.err, ERR_DRAIN_TIMEOUT)) break;
      }
    }
    return false;
  }
  load_base = base + nload;
  return true;
}

// The warp's ring and barriers inside the CTA's dynamic shared memory.
template <typename T, int WPC, int NSTAGE>
__device__ __forceinline__ void warp_ring2d(unsigned char *smem_raw, T *&ring, uint64_t *&bars) {
  constexpr int ROW = 32 * (16 / sizeof(T));
  const int wid = threadIdx.x >> 5;
  ring = reinterpret_cast<T *>(smem_raw) + (size_t)wid * NSTAGE * ROW;
  bars = reinterpret_cast<uint64_t *>(smem_raw + (size_t)WPC * NSTAGE * ROW * sizeof(T)) + wid * NSTAGE;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncwarp();
}

template <class ST, typename T, int B, bool FMA, int WPC, int NSTAGE, bool STASH = false>
__global__ void __launch_bounds__(WPC * 32, gbs_min_ctas(WPC * 32))
    stencil2d_kernel(const __grid_constant__ Params2D<T, ST::kTerms> p) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const long long gw = (long long)blockIdx.x * WPC + (threadIdx.x >> 5);
  if (gw >= (long long)p.nstrips * p.nblocks) return;
  T *ring;
  uint64_t *bars;
  warp_ring2d<T, WPC, NSTAGE>(smem_raw, ring, bars);
  unsigned load_base = 0;
  warp_item2d<ST, T, B, FMA, NSTAGE, STASH>(p, (int)(gw % p.nstrips), (int)(gw / p.nstrips), ring, bars,
                                            load_base);
}

constexpr int kWpc2D = kWarpsPerCta2D, kStages2D = 16;

template <class ST, typename T, int B, bool FMA>
int occupancy2d() {
  constexpr int V = 16 / sizeof(T);
  const size_t smem = (size_t)kWpc2D * kStages2D * (32 * V * sizeof(T) + sizeof(uint64_t));
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stencil2d_kernel<ST, T, B, FMA, kWpc2D, kStages2D>,
                                                    kWpc2D * 32, smem) != cudaSuccess)
    return 0;
  return nb * kWpc2D;
}

template <class ST, typename T, int B, bool FMA, bool STASH = false>
cudaError_t launch2d(const Launch2D &a, cudaStream_t stream) {
  constexpr int WPC = kWpc2D, NSTAGE = kStages2D;
  constexpr int V = 16 / sizeof(T);
  Params2D<T, ST::kTerms> p;
  p.src = static_cast<const T *>(a.src);
  p.dst = static_cast<T *>(a.dst);
  p.err = a.err;
  p.pitch = a.pitch;
  p.d0 = a.d0;
  p.d1 = a.d1;
  p.shift = a.shift;
  p.b = a.b;
  p.wout = a.wout;
  p.nstrips = a.nstrips;
  p.nblocks = a.nblocks;
  p.sl = a.sl;
  // FMA mode is tolerance-bound: a divisor (nonzero, checked by the planner)
  // is folded into the coefficients, and the kernel has no division at all
  const bool fold = FMA && ST::kHasDiv;
  for (int t = 0; t < ST::kTerms; ++t) p.coef[t] = fold ? (T)(a.coef[t] / a.div) : (T)a.coef[t];
  p.divmode = !ST::kHasDiv || fold ? 0 : (a.div_proven ? 2 : 1);
  p.div = (T)a.div;
  p.rdiv = div_reciprocal<T>(a.div);
  p.eps = (T)a.eps;
  p.stash = static_cast<T *>(a.stash);
  p.stash_stride = a.stash_stride;
  if (STASH != (a.stash != nullptr)) return cudaErrorInvalidValue;
  const size_t smem = (size_t)WPC * NSTAGE * (32 * V * sizeof(T) + sizeof(uint64_t));
  const long long warps = (long long)a.nstrips * a.nblocks;
  const long long grid = (warps + WPC - 1) / WPC;
  stencil2d_kernel<ST, T, B, FMA, WPC, NSTAGE, STASH><<<(unsigned)grid, WPC * 32, smem, stream>>>(p);
  return cudaGetLastError();
}

}  // namespace gbs
