// 3-D temporally-blocked stencil kernel family (sm_103a): the one-row-per-warp
// kernel used for exact mode and for the boxes of more than 125 terms (FMA
// mode otherwise runs the tensor-map tiles of kernel3d_tile.cuh), and the
// launchers of both.
//
// Replaces the AN5D-generated 3-D kernels (e.g.
// compiled/float/box3d1r-32x32-3-128_kernel.cu:4,284,509) and computes what
// the artifact's 3-D scop loops compute (star3d2r.c:15-29, box3d1r.c:15-50,
// ...): B Jacobi steps of A[(t+1)%2][i][j][k] = f(A[t%2][neighbourhood]) on
// the interior, the halo held fixed.
//
// Work decomposition. A CTA owns a tile of TJ rows (j) by one 32*V-element
// window of columns (k) and streams the outermost axis i over a block of sl
// output planes. Warp w owns tile row w; lane l owns window elements
// [l*V, l*V+V). Each warp bulk-copies its own row of every level-0 plane into
// a CTA-wide ring of NS stage buffers; a stage's mbarrier completes when all
// TJ rows have landed. The valid output region of a tile is its centre:
// B*r rows and columns are overlap at each side, recomputed by the
// neighbouring tiles (overlapped tiling), as the artifact's kernels do.
//
// Fused levels are skewed by one step: at step s level 1 consumes level-0
// plane s, level l consumes the plane level l-1 wrote at step s-1, and one
// __syncthreads per step publishes every level's output plane. Levels
// 1..B-1 write their planes to shared-memory rings; level B stores to HBM.
// In-plane neighbours come from shared memory (j) and from lane shuffles
// (k); the i-direction lives in registers:
//  * assoc form (any stencil in FMA mode; grouped stencils in exact mode):
//    partial sums of the 2r+1 output planes in flight; the arriving plane
//    adds its terms to each;
//  * direct form (exact mode, stencils whose terms are not grouped by plane,
//    the stars): a register window of the centre column over 2r+1 planes,
//    the centre plane's in-plane neighbours read r steps after it arrived,
//    so each output is one chain in source order.
// Halo cells carry their input value through every level.
#pragma once
#include "gbs_device.cuh"
#include "gbs_launch.h"
#include "stencil_table.cuh"

namespace gbs {

template <typename T, int NT> struct Params3D {
  const T *src;
  T *dst;
  int *err;
  long long pitch;      // elements per padded k-row
  int d0, d1, d2;       // dimsize per axis
  int shift;            // column k at element shift + k
  int jout, wk;         // valid rows / columns per tile
  int ntk, ntj, nblocks, sl;
  T coef[NT];
  T div, rdiv;
  int divmode;          // 0 none (folded), 1 checked, 2 proven fast path
};

template <typename T, int NT>
__device__ __forceinline__ T apply_div3(T y, const Params3D<T, NT> &p) {
  if constexpr (sizeof(T) == 4) {
    if (p.divmode == 2) return div_by_fast(y, p.div, p.rdiv);
  }
  if (p.divmode == 0) return y;
  return div_by(y, p.div, p.rdiv);
}

// Compile-time facts about a 3-D stencil's terms.
template <class ST, int V> struct Tap3 {
  static constexpr int R = ST::kRad;
  static constexpr int NT = ST::kTerms;
  // does a term at plane offset di read row offset dj?
  __host__ __device__ static constexpr bool row_used(int di, int dj) {
    for (int t = 0; t < NT; ++t)
      if (ST::kOff[t][0] == di && ST::kOff[t][1] == dj) return true;
    return false;
  }
  // does a term at plane offset di (any, if di > R) and row offset dj read
  // element x of the lane-extended row?
  __host__ __device__ static constexpr bool need(int di, int dj, int x) {
    for (int t = 0; t < NT; ++t)
      if ((di > R || ST::kOff[t][0] == di) && ST::kOff[t][1] == dj) {
        const int e = x - ST::kOff[t][2];
        if (e >= 0 && e < V) return true;
      }
    return false;
  }
  __host__ __device__ static constexpr bool row_used_any(int dj) {
    for (int t = 0; t < NT; ++t)
      if (ST::kOff[t][1] == dj) return true;
    return false;
  }
};

template <class ST, bool FMA> struct Form3 {
  static constexpr bool kAssoc = FMA || ST::kGrouped;
};

// Order in which the assoc form applies the terms of an arriving plane. Each
// output receives, step by step, one plane-offset group of terms in this
// order; exact mode keeps the source order (the stencils it uses the assoc
// form for list their terms grouped by ascending plane offset, so every
// output's sum is the source's left-to-right sum), FMA mode sorts by row
// offset so that each row of the arriving plane is loaded once.
template <class ST, bool FMA> struct Order3 {
  static constexpr int NT = ST::kTerms;
  struct Arr { int v[NT]; };
  static constexpr Arr make() {
    Arr a{};
    for (int t = 0; t < NT; ++t) a.v[t] = t;
    if (FMA) {  // stable insertion sort by row offset
      for (int i = 1; i < NT; ++i) {
        int x = a.v[i], k = i - 1;
        while (k >= 0 && ST::kOff[a.v[k]][1] > ST::kOff[x][1]) { a.v[k + 1] = a.v[k]; --k; }
        a.v[k + 1] = x;
      }
    }
    return a;
  }
  static constexpr Arr idx = make();
  static constexpr int min_di() {
    int m = 1 << 20;
    for (int t = 0; t < NT; ++t) m = ST::kOff[t][0] < m ? ST::kOff[t][0] : m;
    return m;
  }
  // the position (in this order) of the term that starts every output's sum
  static constexpr int init_pos() {
    for (int u = 0; u < NT; ++u)
      if (ST::kOff[idx.v[u]][0] == min_di()) return u;
    return 0;
  }
  // row offset of the term at position u (or a sentinel before the first)
  static constexpr int dj_at(int u) { return u < 0 ? (1 << 20) : ST::kOff[idx.v[u]][1]; }
};

template <class ST, typename T, bool FMA>
struct Smem3 {
  static constexpr int R = ST::kRad;
  static constexpr bool kAssoc = Form3<ST, FMA>::kAssoc;
  // level-0 stages: the arriving plane (+ the centre plane r back, direct)
  // plus two planes of prefetch
  static constexpr int NS = kAssoc ? 4 : R + 3;
  // ring depth of an intermediate level
  static constexpr int DEP = kAssoc ? 2 : R + 2;
  static constexpr int V = 16 / sizeof(T);
  static constexpr int ROW = 32 * V;
  static constexpr size_t plane_bytes(int tj) { return (size_t)(tj + 2 * R) * ROW * sizeof(T); }
  static constexpr size_t bytes(int tj, int b) {
    return plane_bytes(tj) * (NS + (size_t)(b - 1) * DEP) + NS * sizeof(uint64_t);
  }
};

template <class ST, typename T, int B, bool FMA, int TJ>
__global__ void __launch_bounds__(TJ * 32, gbs_min_ctas(TJ * 32))
    stencil3d_kernel(const __grid_constant__ Params3D<T, ST::kTerms> p) {
  using SM = Smem3<ST, T, FMA>;
  constexpr int V = SM::V;
  constexpr int R = ST::kRad;
  constexpr int W = 2 * R + 1;
  constexpr int ROW = SM::ROW;
  constexpr unsigned ROW_BYTES = ROW * sizeof(T);
  constexpr int NS = SM::NS, DEP = SM::DEP;
  constexpr bool ASSOC = SM::kAssoc;
  constexpr int RD = ASSOC ? 0 : R;  // planes a level-0 stage is kept after it arrives
  constexpr int PLANE = (TJ + 2 * R) * ROW;  // elements of one smem plane
  using A = Arith<T>;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  T *ring0 = reinterpret_cast<T *>(smem_raw);
  T *rings = ring0 + (size_t)NS * PLANE;  // level l (1..B-1) at rings + (l-1)*DEP*PLANE
  uint64_t *bars = reinterpret_cast<uint64_t *>(rings + (size_t)(B - 1) * DEP * PLANE);

  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  int bid = blockIdx.x;
  const int tk = bid % p.ntk;
  bid /= p.ntk;
  const int tj = bid % p.ntj;
  const int blk = bid / p.ntj;

  // columns k
  const int cs = R + tk * p.wk;
  const int ce = min(cs + p.wk, p.d2 - R);
  const int ws = ((max(0, cs - B * R) + p.shift) / V) * V;
  const int col0 = ws - p.shift + lane * V;
  const bool kedge = (ws - p.shift < R) || (ws - p.shift + ROW > p.d2 - R);
  // rows j
  const int js = R + tj * p.jout;
  const int je = min(js + p.jout, p.d1 - R);
  const int j = js - B * R + w;  // this warp's row
  const bool jvalid = (j >= 0 && j < p.d1);
  const bool jhalo = (j < R || j >= p.d1 - R);
  const bool jstore = (j >= js && j < je);
  // planes i
  const int i0 = R + blk * p.sl;
  const int i1 = min(i0 + p.sl, p.d0 - R);
  const int pstart = max(0, i0 - B * R);
  const int pend = min(p.d0, i1 + B * R);
  const int slast = i1 - 1 + (B - 1) + B * R;

  const T *src_row = p.src + ((long long)j * p.pitch + ws);  // + plane * d1 * pitch
  const long long plane_stride = (long long)p.d1 * p.pitch;
  T *dst_lane = p.dst + ((long long)j * p.pitch + ws + lane * V);

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], TJ);
    fence_mbar_init();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int plane) GBS_INL {  // lane 0 of every warp: this warp's row of `plane`
    const int n = plane - pstart;
    const int s = n % NS;
    T *dstp = ring0 + (size_t)s * PLANE + (size_t)(w + R) * ROW;
    if (jvalid) {
      mbar_arrive_expect_tx(&bars[s], ROW_BYTES);
      bulk_g2s(dstp, src_row + plane * plane_stride, ROW_BYTES, &bars[s]);
    } else {
      mbar_arrive(&bars[s]);
    }
  };
  if (lane == 0)
    for (int pl = pstart; pl < pend && pl < pstart + NS; ++pl) issue(pl);

  // register state per level: window (direct) or partial sums (assoc)
  T acc[B][W][V];
#pragma unroll
  for (int l = 0; l < B; ++l)
#pragma unroll
    for (int a = 0; a < W; ++a)
#pragma unroll
      for (int e = 0; e < V; ++e) acc[l][a][e] = T(0);

  bool ok = true;
  int waited = pstart;  // planes whose stage this thread has waited on

  // waits (bounded) for level-0 plane pl; the give-up decision is CTA-uniform
  // and the call is the step's barrier
  auto wait_plane = [&](int pl) GBS_INL -> bool {
    bool got = true;
    if (pl < pend) {
      const int n = pl - pstart;
      got = mbar_wait(&bars[n % NS], (unsigned)(n / NS) & 1u, nullptr, 0);
    }
    if (!__syncthreads_and(got)) {
      if (threadIdx.x == 0) atomicOr(p.err, ERR_WAIT_TIMEOUT);
      return false;
    }
    if (pl < pend) waited = pl + 1;
    return true;
  };
  ok = wait_plane(pstart);

#pragma unroll 1
  for (int s = pstart; ok && s <= slast; ++s) {
    // refill the stage freed by the previous step
    if (lane == 0 && s > pstart) {
      const int pf = s - 1 - RD + NS;
      if (pf >= pstart + NS && pf < pend) issue(pf);
    }

    static_for<B>([&](auto LI) {
      constexpr int l = decltype(LI)::value;  // computes level l+1
      const int m = s - l * (R + 1);          // arriving plane of level l
      const int q = m - R;                    // output plane of level l+1
      // buffers of level l's planes: arriving plane m and (direct) centre plane q
      const T *in_m;
      const T *in_q;
      if constexpr (l == 0) {
        in_m = ring0 + (size_t)(((m - pstart) % NS + NS) % NS) * PLANE;
        in_q = ring0 + (size_t)(((q - pstart) % NS + NS) % NS) * PLANE;
      } else {
        const T *rl = rings + (size_t)(l - 1) * DEP * PLANE;
        in_m = rl + (size_t)(((s - 1) % DEP + DEP) % DEP) * PLANE;
        in_q = rl + (size_t)(((s - 1 - R) % DEP + DEP) % DEP) * PLANE;
      }
      const bool qhalo = (q < R || q >= p.d0 - R);
      T y[V];
      if constexpr (ASSOC) {
        // the arriving plane adds its terms to outputs m-R .. m+R, in the
        // order Order3 fixes; the lane-extended row of the current row
        // offset is reloaded when the offset changes
        using OR = Order3<ST, FMA>;
        T ext[V + 2 * R];
        static_for<ST::kTerms>([&](auto UI) {
          constexpr int u = decltype(UI)::value;
          constexpr int t = OR::idx.v[u];
          constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
          if constexpr (OR::dj_at(u - 1) != dj) {
            T row[V];
            ld_vec<T, V>(row, in_m + (size_t)(w + R + dj) * ROW + lane * V);
            static_for<V + 2 * R>([&](auto XI) {
              constexpr int xx = decltype(XI)::value - R;
              if constexpr (Tap3<ST, V>::need(R + 1, dj, xx)) ext[R + xx] = row_elem<V, xx>(row);
            });
          }
          // output m - di sits at logical position R - di (0 = completes now)
          constexpr int slot = R - di;
          static_for<V>([&](auto EI) {
            constexpr int e = decltype(EI)::value;
            const T a = ext[R + e + dk];
            if constexpr (u == OR::init_pos()) acc[l][slot][e] = A::mul(p.coef[t], a);
            else acc[l][slot][e] = term_next<T, FMA>(acc[l][slot][e], p.coef[t], a);
          });
        });
#pragma unroll
        for (int e = 0; e < V; ++e) {
          if constexpr (ST::kHasDiv && !FMA) y[e] = apply_div3(acc[l][0][e], p);
          else y[e] = acc[l][0][e];
        }
        if (qhalo || jhalo || kedge) {
          if (q >= 0 && q < p.d0 && jvalid) {
            T c[V];
            ld_vec_global<T, V>(c, src_row + q * plane_stride + lane * V);
            if (qhalo || jhalo) {
#pragma unroll
              for (int e = 0; e < V; ++e) y[e] = c[e];
            } else {
#pragma unroll
              for (int e = 0; e < V; ++e)
                if (col0 + e < R || col0 + e >= p.d2 - R) y[e] = c[e];
            }
          }
        }
        // shift the partial sums: position a+1 becomes a
#pragma unroll
        for (int a = 0; a < 2 * R; ++a)
#pragma unroll
          for (int e = 0; e < V; ++e) acc[l][a][e] = acc[l][a + 1][e];
      } else {
        // direct: push the arriving centre column, evaluate the centre plane q
        ld_vec<T, V>(acc[l][2 * R], in_m + (size_t)(w + R) * ROW + lane * V);
        if (qhalo || jhalo) {
#pragma unroll
          for (int e = 0; e < V; ++e) y[e] = acc[l][R][e];
        } else {
          T ext[W][V + 2 * R];  // in-plane rows of plane q, lane-extended
          static_for<W>([&](auto DJI) {
            constexpr int dj = decltype(DJI)::value - R;
            if constexpr (Tap3<ST, V>::row_used(0, dj)) {
              T row[V];
              if constexpr (dj == 0) {
#pragma unroll
                for (int e = 0; e < V; ++e) row[e] = acc[l][R][e];
              } else {
                ld_vec<T, V>(row, in_q + (size_t)(w + R + dj) * ROW + lane * V);
              }
              static_for<V + 2 * R>([&](auto XI) {
                constexpr int xx = decltype(XI)::value - R;
                if constexpr (Tap3<ST, V>::need(0, dj, xx)) ext[dj + R][R + xx] = row_elem<V, xx>(row);
              });
            }
          });
          static_for<ST::kTerms>([&](auto TI) {
            constexpr int t = decltype(TI)::value;
            constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
            static_assert(di == 0 || (dj == 0 && dk == 0), "direct 3-D form expects a star");
            static_for<V>([&](auto EI) {
              constexpr int e = decltype(EI)::value;
              T a;
              if constexpr (di != 0) a = acc[l][R + di][e];
              else a = ext[dj + R][R + e + dk];
              if constexpr (t == 0) y[e] = A::mul(p.coef[t], a);
              else y[e] = term_next<T, FMA>(y[e], p.coef[t], a);
            });
          });
          if constexpr (ST::kHasDiv && !FMA) {
#pragma unroll
            for (int e = 0; e < V; ++e) y[e] = apply_div3(y[e], p);
          }
          if (kedge) {
#pragma unroll
            for (int e = 0; e < V; ++e)
              if (col0 + e < R || col0 + e >= p.d2 - R) y[e] = acc[l][R][e];
          }
        }
#pragma unroll
        for (int a = 0; a < 2 * R; ++a)
#pragma unroll
          for (int e = 0; e < V; ++e) acc[l][a][e] = acc[l][a + 1][e];
      }

      if constexpr (l + 1 < B) {
        T *out = rings + (size_t)l * DEP * PLANE + (size_t)(s % DEP) * PLANE;
        st_vec<T, V>(out + (size_t)(w + R) * ROW + lane * V, y);
      } else {
        if (q >= i0 && q < i1 && jstore) {
          T *d = dst_lane + q * plane_stride;
          if (col0 >= cs && col0 + V <= ce) {
            st_vec<T, V>(d, y);
          } else {
#pragma unroll
            for (int e = 0; e < V; ++e)
              if (col0 + e >= cs && col0 + e < ce) d[e] = y[e];
          }
        }
      }
    });
    ok = wait_plane(s + 1);
  }

  if (!ok && lane == 0) {
    // Timed out: wait (bounded) for this warp's copies still in flight.
    const int last = min(pend, waited + NS);
    for (int pl = waited; pl < last; ++pl) {
      const int n = pl - pstart;
      if (!mbar_wait(&bars[n % NS], (unsigned)(n / NS) & 1u, p.err, ERR_DRAIN_TIMEOUT)) break;
    }
  }
}

}  // namespace gbs

#include "kernel3d_tile.cuh"

namespace gbs {

// rows per warp of the FMA variant: as many as the partial sums allow in
// the 128 registers a 512-thread CTA may use
template <class ST, typename T, int B>
constexpr int rows_per_warp() {
  constexpr int W = 2 * ST::kRad + 1;
  constexpr int regs_per_cell = sizeof(T) / 4;  // 32-bit registers per value
  constexpr int V = 16 / sizeof(T);
  // stencils with many terms keep more temporaries live per row
  constexpr int budget = ST::kTerms > 30 ? 24 : 96;
  if (B * W * 4 * V * regs_per_cell <= budget) return 4;
  if (B * W * 2 * V * regs_per_cell <= budget) return 2;
  return 1;
}
constexpr int kNw3D = 16;

constexpr int kTj3D = 32;

// The tile kernel (tensor-map copies, exact output coverage) serves FMA mode
// except for the large boxes, whose hundreds of terms per row make its
// per-row unrolling too big to inline; they (and exact mode) use the
// one-row kernel.
template <class ST, bool FMA>
constexpr bool use_tile3d() { return FMA && ST::kTerms <= 125; }

// level-0 stages of the tile kernel: four, or three where four do not fit
template <class ST, typename T, int B, int NW>
constexpr int tile_stages3d() {
  return Tile3<ST, T, B, NW, rows_per_warp<ST, T, B>(), 4>::bytes() <= 227u * 1024u ? 4 : 3;
}
template <class ST, typename T, int B, int NW = kNw3D>
using TileOf = Tile3<ST, T, B, NW, rows_per_warp<ST, T, B>(), tile_stages3d<ST, T, B, NW>()>;

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
constexpr int tile_rows3d() {
  return use_tile3d<ST, FMA>() ? TileOf<ST, T, B, NW>::TJ : kTj3D;
}

// valid rows and columns per tile of the launcher for (ST, T, B, FMA)
template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
constexpr int tile_jout3d() {
  return use_tile3d<ST, FMA>() ? TileOf<ST, T, B, NW>::JOUT : kTj3D - 2 * B * ST::kRad;
}
template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
constexpr int tile_wk3d() {
  constexpr int V = 16 / sizeof(T);
  return use_tile3d<ST, FMA>() ? TileOf<ST, T, B, NW>::WK : (32 * V - 2 * B * ST::kRad - (V - 1)) / V * V;
}

// Double at degree 1 runs the tile as a decoupled pipeline (one producer
// warp more): the FP64 pipe bounds it, and the per-plane barrier of the tile
// kernel idles that pipe while the last warps of a plane drain. (Float at
// degree 1 is bound by HBM; with the extra warp its registers would spill.)
template <class ST, typename T, int B, bool FMA>
constexpr bool use_stream3d() { return use_tile3d<ST, FMA>() && B == 1 && sizeof(T) == 8; }

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
constexpr size_t smem_bytes3d() {
  if constexpr (use_stream3d<ST, T, B, FMA>()) {
    using G = TileOf<ST, T, B, NW>;
    return Stream3<ST, T, NW, rows_per_warp<ST, T, B>(), G::NS>::bytes();
  } else if constexpr (use_tile3d<ST, FMA>()) {
    return TileOf<ST, T, B, NW>::bytes();
  } else {
    return Smem3<ST, T, FMA>::bytes(kTj3D, B);
  }
}

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
auto kernel3d_ptr() {
  if constexpr (use_stream3d<ST, T, B, FMA>()) {
    using G = TileOf<ST, T, B, NW>;
    return stencil3d_stream_kernel<ST, T, NW, rows_per_warp<ST, T, B>(), G::NS>;
  } else if constexpr (use_tile3d<ST, FMA>()) {
    using G = TileOf<ST, T, B, NW>;
    return stencil3d_tile_kernel<ST, T, B, NW, rows_per_warp<ST, T, B>(), G::NS>;
  } else {
    return stencil3d_kernel<ST, T, B, FMA, kTj3D>;
  }
}

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
constexpr int threads3d() {
  return use_tile3d<ST, FMA>() ? (use_stream3d<ST, T, B, FMA>() ? NW + 1 : NW) * 32 : kTj3D * 32;
}

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
cudaError_t launch3d(const Launch3D &a, cudaStream_t stream) {
  constexpr int NT = threads3d<ST, T, B, FMA, NW>();
  auto kern = kernel3d_ptr<ST, T, B, FMA, NW>();
  const size_t smem = smem_bytes3d<ST, T, B, FMA, NW>();
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return e;
    }
    attr_set = true;
  }
  const bool fold = FMA && ST::kHasDiv;  // the divisor is nonzero (checked by the planner)
  const long long grid = (long long)a.ntk * a.ntj * a.nblocks;
  if constexpr (use_tile3d<ST, FMA>()) {
    using G = TileOf<ST, T, B, NW>;
    Params3T<T, ST::kTerms> p;
    cudaError_t e = encode_plane_map(&p.tmap, a.src, (int)sizeof(T), a.pitch, a.d1, a.d0, G::BX, G::BY);
    if (e != cudaSuccess) return e;
    p.src = static_cast<const T *>(a.src);
    p.dst = static_cast<T *>(a.dst);
    p.err = a.err;
    p.pitch = a.pitch;
    p.d0 = a.d0;
    p.d1 = a.d1;
    p.d2 = a.d2;
    p.shift = a.shift;
    p.jout = a.jout;
    p.wk = a.wk;
    p.ntk = a.ntk;
    p.ntj = a.ntj;
    p.nblocks = a.nblocks;
    p.sl = a.sl;
    for (int t = 0; t < ST::kTerms; ++t) p.coef[t] = fold ? (T)(a.coef[t] / a.div) : (T)a.coef[t];
    kern<<<(unsigned)grid, NT, smem, stream>>>(p);
  } else {
    Params3D<T, ST::kTerms> p;
    p.src = static_cast<const T *>(a.src);
    p.dst = static_cast<T *>(a.dst);
    p.err = a.err;
    p.pitch = a.pitch;
    p.d0 = a.d0;
    p.d1 = a.d1;
    p.d2 = a.d2;
    p.shift = a.shift;
    p.jout = a.jout;
    p.wk = a.wk;
    p.ntk = a.ntk;
    p.ntj = a.ntj;
    p.nblocks = a.nblocks;
    p.sl = a.sl;
    for (int t = 0; t < ST::kTerms; ++t) p.coef[t] = fold ? (T)(a.coef[t] / a.div) : (T)a.coef[t];
    p.divmode = !ST::kHasDiv || fold ? 0 : (a.div_proven ? 2 : 1);
    p.div = (T)a.div;
    p.rdiv = div_reciprocal<T>(a.div);
    kern<<<(unsigned)grid, NT, smem, stream>>>(p);
  }
  return cudaGetLastError();
}

template <class ST, typename T, int B, bool FMA, int NW = kNw3D>
int occupancy3d() {
  constexpr int NT = threads3d<ST, T, B, FMA, NW>();
  auto kern = kernel3d_ptr<ST, T, B, FMA, NW>();
  const size_t smem = smem_bytes3d<ST, T, B, FMA, NW>();
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, NT, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return nb;
}

}  // namespace gbs
