// Adjoint (reverse-mode gradient) of the stencil time loop.
//
// No counterpart in the artifact: it differentiates the time loop that
// kernel_stencil runs. For u_{t+1} = F(u_t) on the interior (halo fixed)
// and a loss L(u_T) whose gradient lam_T = dL/du_T the caller supplies, it
// returns dL/du_0 (interior and halo) and, on request, dL/dc_k for the
// coefficients as the source writes them (before any divisor).
//
// Linear stencils, u_{t+1}(x) = sum_k c_k u_t(x + o_k) / d:
//  * lam_t(y) = sum_k c_k/d lam_{t+1}(y - o_k) on the interior, zero on the
//    halo. Every offset set in the catalogue is symmetric (o in the set iff
//    -o is), so this is the forward stencil with each coefficient moved to
//    the mirrored offset: the engine's own kernels run it (FMA mode), one
//    launch per step from one lam plane to the other.
//  * a halo cell h feeds every step: dL/du_0(h) = sum_t sum_k c_k/d
//    lam_{t+1}(h - o_k), accumulated by a kernel over the halo cells only.
//  * dL/dc_k = sum_t sum_x lam_{t+1}(x) u_t(x + o_k) / d needs the forward
//    states: only then are they recomputed (below), and a streaming kernel
//    accumulates the products per thread and reduces them per CTA into a
//    partial buffer (no atomics; summed in double at the end).
// gradient2d, u_{t+1} = u + c q, q = (eps + s)^{-1/2}, s = sum_n (u - u_{x+n})^2:
//    the linearised update, dF(x)/du(x) = 1 - c q^3 sum_n d_n(x),
//    dF(x)/du(x+n) = c q^3 d_n(x), dF(x)/dc = q(x), evaluated on u_t: a
//    pre-pass stores q and sum_n d_n per cell, a gather kernel applies the
//    transposed Jacobian.
//
// Checkpointing: gbs_adjoint_forward advances the grid and saves u_t every
// C steps into the caller's workspace. When the states are needed,
// gbs_adjoint_backward walks the chunks backwards and recomputes a chunk's C
// states from its checkpoint with the forward engine (one launch per step,
// each into its own stash slot), then runs the chunk's adjoint steps. With
// fewer than 2C stash slots (a smaller memory budget) each chunk is
// reversed by the binomial (revolve) schedule instead: a recursion that
// advances from the newest stored state into a free slot, reverses the
// right part with one slot fewer and then the left part, which is the
// fewest forward steps any schedule with that many slots can take (Griewank
// and Walther, ACM TOMS 26(1), 2000, Algorithm 799).
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <cstring>
#include <vector>

#include "engine_internal.h"
#include "gbs_device.cuh"

namespace gbs {
namespace {

constexpr int kAdjThreads = 256;
constexpr int kMaxCoefGrad = 32;  // coefficient gradients for stencils of at most this many terms
constexpr int kCoefBlocks = 1024;  // CTAs of the coefficient kernel (one partial row each)

struct AdjGeom {
  long long pitch, plane;  // elements
  int d0, d1, d2, dim, shift, rad;
  int rows, last;          // rows per plane (d0 or d0*d1), cells per row
  long long cells;         // d0*d1*d2
};

__device__ __forceinline__ long long cell_off(const AdjGeom &g, int i, int j, int k) {
  return g.dim == 2 ? (long long)i * g.pitch + g.shift + j
                    : ((long long)i * g.d1 + j) * g.pitch + g.shift + k;
}

// (i, j) of row r; for 2-D rows j = 0 and the column is the second index
__device__ __forceinline__ void row_ij(const AdjGeom &g, int r, int &i, int &j) {
  if (g.dim == 2) {
    i = r;
    j = 0;
  } else {
    i = r / g.d1;
    j = r - i * g.d1;
  }
}

__device__ __forceinline__ bool row_interior(const AdjGeom &g, int i, int j) {
  const int R = g.rad;
  return i >= R && i < g.d0 - R && (g.dim == 2 || (j >= R && j < g.d1 - R));
}

// value of plane p at (i, j, c) (c the innermost index; 2-D: (i, c)); 0 off the grid
template <typename T>
__device__ __forceinline__ T ldz(const T *p, const AdjGeom &g, int i, int j, int c) {
  if (i < 0 || i >= g.d0 || c < 0 || c >= g.last) return T(0);
  if (g.dim == 2) return p[(long long)i * g.pitch + g.shift + c];
  if (j < 0 || j >= g.d1) return T(0);
  return p[((long long)i * g.d1 + j) * g.pitch + g.shift + c];
}

template <typename T, int NT> struct LinCoef {
  T c[NT];  // c_k / d
};

// Halo cells, enumerated without touching the interior:
//  A: the 2R edge columns of every interior row, one thread per cell;
//  B: every cell of the all-halo rows, one warp per 32-column segment.
// All-halo rows: 2-D rows i < R or i >= d0 - R; 3-D the planes i < R or
// i >= d0 - R (every row j), then the rows j < R or j >= d1 - R of each
// interior plane.
struct HaloPlan {
  long long na;      // A cells, rounded up to whole warps
  long long rows_b;  // all-halo rows
  int nseg;          // 32-column segments per row
};

__host__ __device__ inline HaloPlan halo_plan(const AdjGeom &g) {
  HaloPlan h{};
  const int R = g.rad;
  const long long inner_rows = g.dim == 2 ? (long long)(g.d0 - 2 * R) : (long long)(g.d0 - 2 * R) * (g.d1 - 2 * R);
  h.na = (inner_rows * 2 * R + 31) / 32 * 32;
  h.rows_b = (long long)g.rows - inner_rows;
  h.nseg = (g.last + 31) / 32;
  return h;
}

// halo cell number tid of the enumeration above: (i, j, c); false past the end
__device__ __forceinline__ bool halo_cell(const AdjGeom &g, const HaloPlan &hp, long long tid, int &i, int &j,
                                          int &c) {
  const int R = g.rad;
  j = 0;
  if (tid < hp.na) {
    const long long row = tid / (2 * R);
    const int e = (int)(tid - row * 2 * R);
    if (g.dim == 2) {
      if (row >= g.d0 - 2 * R) return false;
      i = R + (int)row;
    } else {
      const int w1 = g.d1 - 2 * R;
      if (row >= (long long)(g.d0 - 2 * R) * w1) return false;
      i = R + (int)(row / w1);
      j = R + (int)(row - (long long)(i - R) * w1);
    }
    c = e < R ? e : g.last - 2 * R + e;
    return true;
  }
  const long long b = tid - hp.na;
  const long long wrow = (b >> 5) / hp.nseg;
  const int seg = (int)((b >> 5) - wrow * hp.nseg);
  if (wrow >= hp.rows_b) return false;
  c = seg * 32 + (int)(b & 31);
  if (c >= g.last) return false;
  if (g.dim == 2) {
    i = wrow < R ? (int)wrow : g.d0 - 2 * R + (int)wrow;
  } else {
    const long long full = 2LL * R * g.d1;  // rows of the all-halo planes
    if (wrow < full) {
      const int p = (int)(wrow / g.d1);
      i = p < R ? p : g.d0 - 2 * R + p;
      j = (int)(wrow - (long long)p * g.d1);
    } else {
      const long long q = wrow - full;
      i = R + (int)(q / (2 * R));
      const int jj = (int)(q - (long long)(i - R) * 2 * R);
      j = jj < R ? jj : g.d1 - 2 * R + jj;
    }
  }
  return true;
}

// hg(h) += sum_k c_k/d lam(h - o_k) at halo cell h
template <class ST, typename T>
__device__ __forceinline__ void halo_update(const AdjGeom &g, const T *lam, T *hg, const LinCoef<T, ST::kTerms> &cf,
                                            int i, int j, int c) {
  T acc = T(0);
  static_for<ST::kTerms>([&](auto TI) {
    constexpr int t = decltype(TI)::value;
    constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
    // 2-D offsets are (row, column); 3-D (plane, row, column)
    const T l = ST::kDim == 2 ? ldz(lam, g, i - di, 0, c - dj) : ldz(lam, g, i - di, j - dj, c - dk);
    acc = fma(cf.c[t], l, acc);
  });
  const long long o = (ST::kDim == 2 ? (long long)i * g.pitch : ((long long)i * g.d1 + j) * g.pitch) + g.shift + c;
  hg[o] += acc;
}

// hg(h) += sum_k c_k/d lam(h - o_k) for every halo cell h
template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) halo_kernel(const __grid_constant__ AdjGeom g, const T *lam, T *hg,
                                                           const __grid_constant__ LinCoef<T, ST::kTerms> cf) {
  const HaloPlan hp = halo_plan(g);
  int i, j, c;
  if (halo_cell(g, hp, (long long)blockIdx.x * kAdjThreads + threadIdx.x, i, j, c))
    halo_update<ST, T>(g, lam, hg, cf, i, j, c);
}

// part[blockIdx.x][k] += sum over interior x of lam(x) u(x + o_k) / d.
// Work units of one warp: (interior row, 128-column segment), four
// independent columns per lane in flight; products summed per thread in T,
// reduced per CTA in double.
template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) coef_kernel(const __grid_constant__ AdjGeom g, const T *lam, const T *u,
                                                           double *part, T inv_div) {
  constexpr int NT = ST::kTerms;
  constexpr int SEG = 128;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int R = g.rad;
  const int width = g.last - 2 * R;
  const long long nseg = (width + SEG - 1) / SEG;
  const long long units = (long long)g.rows * nseg;
  const long long nwarps = ((long long)gridDim.x * kAdjThreads) >> 5;
  T acc[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) acc[t] = T(0);
  for (long long un = ((long long)blockIdx.x * kAdjThreads + threadIdx.x) >> 5; un < units; un += nwarps) {
    const int r = (int)(un / nseg), seg = (int)(un - (long long)r * nseg);
    int i, j;
    row_ij(g, r, i, j);
    if (!row_interior(g, i, j)) continue;
    const long long row = (ST::kDim == 2 ? (long long)i * g.pitch : ((long long)i * g.d1 + j) * g.pitch) + g.shift;
    const int c0 = R + seg * SEG + lane;
    T l[SEG / 32];
    bool in[SEG / 32];
#pragma unroll
    for (int q = 0; q < SEG / 32; ++q) {
      const int c = c0 + 32 * q;
      in[q] = c < g.last - R;
      l[q] = in[q] ? lam[row + c] : T(0);
    }
    static_for<NT>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
      const long long o = ST::kDim == 2 ? (long long)di * g.pitch + dj : ((long long)di * g.d1 + dj) * g.pitch + dk;
#pragma unroll
      for (int q = 0; q < SEG / 32; ++q)
        if (in[q]) acc[t] = fma(l[q], u[row + c0 + 32 * q + o], acc[t]);
    });
  }
  __shared__ double red[kAdjThreads / 32][NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    T v = acc[t];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if (lane == 0) red[w][t] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x < NT) {
    double s = 0.0;
#pragma unroll
    for (int ww = 0; ww < kAdjThreads / 32; ++ww) s += red[ww][threadIdx.x];
    part[(size_t)blockIdx.x * NT + threadIdx.x] += s * (double)inv_div;
  }
}

// The elements of one row that a segment's end lanes cannot take from a
// neighbouring lane: left[x + R] for x in [-R, 0) (lanes within R/V of the
// warp's start) and right[x - V] for x in [V, V + R) (lanes within R/V of
// its end), relative to the lane's first column; loaded once, when the row
// enters the lane's register window, instead of once per term and use.
template <typename T, int V, int R> struct RowEdges {
  T left[R], right[R];
};
template <typename T, int V, int R>
__device__ __forceinline__ void load_edges(RowEdges<T, V, R> &ed, const T *p, long long rowbase, int lane) {
  static_for<R>([&](auto XI) {
    constexpr int x = -1 - decltype(XI)::value;  // -1 .. -R
    constexpr int dl = (-x + V - 1) / V;
    if (lane < dl) ed.left[x + R] = p[rowbase + x];
  });
  static_for<R>([&](auto XI) {
    constexpr int x = V + decltype(XI)::value;   // V .. V+R-1
    constexpr int dl = x / V;
    if (lane >= 32 - dl) ed.right[x - V] = p[rowbase + x];
  });
}
// Element x (relative to the lane's first column, x in [-R, V+R)) of the row
// at window position P: from the lane's own vector, from a lane up to R/V
// away, or, for the lanes whose source lane lies outside the warp, from the
// row's cached edges
template <int V, int R, int P, int X, typename T, int NWIN>
__device__ __forceinline__ T row_value_cached(const T (&rows)[NWIN][V], const RowEdges<T, V, R> (&ed)[NWIN],
                                              int lane) {
  T v = row_elem<V, X>(rows[P]);
  if constexpr (X < 0) {
    constexpr int dl = (-X + V - 1) / V;
    if (lane < dl) v = ed[P].left[X + R];
  } else if constexpr (X >= V) {
    constexpr int dl = X / V;
    if (lane >= 32 - dl) v = ed[P].right[X - V];
  }
  return v;
}

// rows of lam (and u) the adjoint step loads per batch: one memory latency
// per batch of output rows instead of one per row. The window holds 2R + K
// rows of each array, so the batch shrinks with the radius and for double
// (radius 1 float at K = 4 takes 116 registers with the coefficient
// products; larger windows spill).
template <typename T, int R>
constexpr int adj_batch() {
  if (sizeof(T) == 4) return R == 1 ? 4 : (R == 2 ? 2 : 1);
  return R == 1 ? 2 : 1;
}

// 2-D linear adjoint step, fused: lam_out(y) = sum_k c_k/d lam(y - o_k) on
// the interior (lam is zero on the halo; lam_out's halo is never written),
// with WANT_COEF the products lam(y) u(y + o_k) / d summed per thread and
// reduced per CTA into part[blockIdx.x][k], and hg(h) += the transposed sum
// at every halo cell h. One launch per step instead of the transposed engine
// step, the halo kernel and the product kernel: 2-D grids are small enough
// that a step is bound by kernel latency. The first `interior_blocks` CTAs
// take work units of one 32*V-column segment by `rows` interior rows: each
// lane streams its aligned 16-byte vector of V columns down the rows,
// keeping the rows of lam (and of u) that the next batch of output rows
// needs in registers, so that every row is loaded once per unit and the
// loads of a batch of rows are in flight together (a unit of a few rows per
// warp is otherwise a chain of dependent memory latencies); in-row
// neighbours come from the lanes up to R/V away (the warp's edge lanes load
// theirs). The CTAs after them take the halo cells (one thread each).
template <class ST, typename T, bool WANT_COEF>
__global__ void __launch_bounds__(kAdjThreads) adj2d_kernel(const __grid_constant__ AdjGeom g,
                                                            const T *__restrict__ lam, const T *__restrict__ u,
                                                            T *__restrict__ lam_out, T *__restrict__ hg,
                                                            double *__restrict__ part,
                                                            const __grid_constant__ LinCoef<T, ST::kTerms> cf,
                                                            T inv_div, int interior_blocks, int rows) {
  constexpr int NT = ST::kTerms;
  constexpr int NP = WANT_COEF ? NT : 1;
  constexpr int V = 16 / sizeof(T);
  constexpr int R = ST::kRad;
  constexpr int SEG = 32 * V;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if ((int)blockIdx.x >= interior_blocks) {
    const HaloPlan hp = halo_plan(g);
    int i, j, c;
    if (halo_cell(g, hp, (long long)(blockIdx.x - interior_blocks) * kAdjThreads + threadIdx.x, i, j, c))
      halo_update<ST, T>(g, lam, hg, cf, i, j, c);
    return;
  }
  T acc[NP];
#pragma unroll
  for (int t = 0; t < NP; ++t) acc[t] = T(0);
  const int width = g.last - 2 * R;
  const int nseg = (width + SEG - 1) / SEG;
  const int ni = g.d0 - 2 * R;
  const int nblk = (ni + rows - 1) / rows;
  const long long units = (long long)nblk * nseg;
  const long long nwarps = (long long)interior_blocks * (kAdjThreads / 32);
  for (long long un = (long long)blockIdx.x * (kAdjThreads / 32) + w; un < units; un += nwarps) {
    const int blk = (int)(un / nseg), seg = (int)(un - (long long)blk * nseg);
    const int ia = R + blk * rows, ib = min(ia + rows, g.d0 - R);  // output rows [ia, ib)
    const int c0 = R + seg * SEG + lane * V;        // the lane's first column; 16-byte aligned
    const int nvalid = min(V, g.last - R - c0);     // columns of the group inside the interior
    const long long col = (long long)g.shift + c0;
    // windows of rows i-R .. i+R+K-1 (position p holds row i-R+p), refilled
    // K rows at a time: the K new rows of lam (and u) are loaded together
    constexpr int K = adj_batch<T, R>();
    constexpr int NWIN = 2 * R + K;
    T lw[NWIN][V], uw[WANT_COEF ? NWIN : 1][V];
    RowEdges<T, V, R> le[NWIN], ue[WANT_COEF ? NWIN : 1];  // the segment-end elements of each row
    static_for<2 * R>([&](auto PI) {
      constexpr int pp = decltype(PI)::value;  // rows ia-R .. ia+R-1
      const long long rb = (long long)(ia - R + pp) * g.pitch + col;
      ld_vec<T, V>(lw[pp], lam + rb);
      load_edges<T, V, R>(le[pp], lam, rb, lane);
      if constexpr (WANT_COEF) {
        ld_vec<T, V>(uw[pp], u + rb);
        load_edges<T, V, R>(ue[pp], u, rb, lane);
      }
    });
#pragma unroll 1
    for (int i = ia; i < ib; i += K) {
      // load rows i+R .. i+R+K-1 (those below ib+R; the rest are not read)
      static_for<K>([&](auto KI) {
        constexpr int kk = decltype(KI)::value;
        if (i + kk < ib) {
          const long long rb = (long long)(i + R + kk) * g.pitch + col;
          ld_vec<T, V>(lw[2 * R + kk], lam + rb);
          load_edges<T, V, R>(le[2 * R + kk], lam, rb, lane);
          if constexpr (WANT_COEF) {
            ld_vec<T, V>(uw[2 * R + kk], u + rb);
            load_edges<T, V, R>(ue[2 * R + kk], u, rb, lane);
          }
        }
      });
      static_for<K>([&](auto KI) {
        constexpr int kk = decltype(KI)::value;  // output row i+kk: window positions kk .. kk+2R
        if (i + kk < ib) {
          const long long base = (long long)(i + kk) * g.pitch + col;
          T sv[V];
#pragma unroll
          for (int e = 0; e < V; ++e) sv[e] = T(0);
          static_for<NT>([&](auto TI) {
            constexpr int t = decltype(TI)::value;
            constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
            static_for<V>([&](auto EI) {
              constexpr int e = decltype(EI)::value;
              sv[e] = fma(cf.c[t], row_value_cached<V, R, kk + R - di, e - dj>(lw, le, lane), sv[e]);
            });
          });
          if constexpr (WANT_COEF) {
            static_for<NT>([&](auto TI) {
              constexpr int t = decltype(TI)::value;
              constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
              static_for<V>([&](auto EI) {
                constexpr int e = decltype(EI)::value;
                const T uv = row_value_cached<V, R, kk + R + di, e + dj>(uw, ue, lane);
                if (e < nvalid) acc[t] = fma(lw[kk + R][e], uv, acc[t]);
              });
            });
          }
          if (nvalid == V) {
            st_vec<T, V>(lam_out + base, sv);
          } else {
#pragma unroll
            for (int e = 0; e < V; ++e)
              if (e < nvalid) lam_out[base + e] = sv[e];
          }
        }
      });
      // slide by K: rows i+K-R .. i+K+R-1 to positions 0 .. 2R-1
      static_for<2 * R>([&](auto PI) {
        constexpr int pp = decltype(PI)::value;
#pragma unroll
        for (int e = 0; e < V; ++e) {
          lw[pp][e] = lw[pp + K][e];
          if constexpr (WANT_COEF) uw[pp][e] = uw[pp + K][e];
        }
        le[pp] = le[pp + K];
        if constexpr (WANT_COEF) ue[pp] = ue[pp + K];
      });
    }
  }
  if constexpr (WANT_COEF) {
    __shared__ double red[kAdjThreads / 32][NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      T v = acc[t];
#pragma unroll
      for (int sh = 16; sh > 0; sh >>= 1) v += __shfl_down_sync(0xffffffffu, v, sh);
      if (lane == 0) red[w][t] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < NT) {
      double sum = 0.0;
#pragma unroll
      for (int ww = 0; ww < kAdjThreads / 32; ++ww) sum += red[ww][threadIdx.x];
      part[(size_t)blockIdx.x * NT + threadIdx.x] += sum * (double)inv_div;
    }
  }
}

// gradient2d pre-pass: for interior x, q(x) = (eps + s(x))^{-1/2} and
// sd(x) = sum_n d_n(x), d_n = u(x) - u(x + n), from u_t (s formed as the
// forward step forms it)
template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) grad_pre_kernel(const __grid_constant__ AdjGeom g, const T *u, T *qp,
                                                               T *sdp, T eps) {
  const long long cidx = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  if (cidx >= g.cells) return;
  const int i = (int)(cidx / g.d1), j = (int)(cidx - (long long)(cidx / g.d1) * g.d1);
  const int R = g.rad;
  if (!(i >= R && i < g.d0 - R && j >= R && j < g.d1 - R)) return;
  using A = Arith<T>;
  const long long o = cell_off(g, i, j, 0);
  const T ux = u[o];
  T s = eps;
  double sd = 0.0;
  static_for<ST::kTerms>([&](auto TI) {
    constexpr int t = decltype(TI)::value;
    const T d = A::sub(ux, u[cell_off(g, i + ST::kOff[t][0], j + ST::kOff[t][1], 0)]);
    s = A::add(s, A::mul(d, d));
    sd += (double)d;
  });
  // Newton-Raphson for 1/sqrt(s) from a single-precision estimate (two
  // steps: relative error 2^-22 -> 2^-44 -> double precision)
  const double sv = (double)s;
  double y;
  if (sv >= 1e-30 && sv <= 1e30) {
    y = (double)rsqrtf((float)s);
    double h = fma(-sv * y, y, 1.0);
    y = fma(0.5 * y, h, y);
    h = fma(-sv * y, y, 1.0);
    y = fma(0.5 * y, h, y);
  } else {
    y = 1.0 / sqrt(sv);
  }
  qp[o] = (T)y;
  sdp[o] = (T)sd;
}

// gradient2d adjoint step (transposed linearised Jacobian) and dL/dnum partials
template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) grad_adj_kernel(const __grid_constant__ AdjGeom g, const T *u,
                                                               const T *qp, const T *sdp, const T *lam_next,
                                                               T *lam_prev, T *hg, double *part, T num,
                                                               int want_coef) {
  const long long cidx = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  const int R = g.rad;
  double pnum = 0.0;
  if (cidx < g.cells) {
    const int i = (int)(cidx / g.d1), j = (int)(cidx - (long long)(cidx / g.d1) * g.d1);
    auto inter = [&](int a, int b) GBS_INL { return a >= R && a < g.d0 - R && b >= R && b < g.d1 - R; };
    const long long o = cell_off(g, i, j, 0);
    const bool yin = inter(i, j);
    T acc = T(0);
    if (yin) {
      const T q = qp[o], ly = lam_next[o];
      acc = ly * (T(1) - num * q * q * q * sdp[o]);
      pnum = (double)(ly * q);
    }
    const T uy = u[o];
    static_for<ST::kTerms>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      const int a = i - ST::kOff[t][0], b = j - ST::kOff[t][1];  // x with x + n = y
      if (a >= 0 && a < g.d0 && b >= 0 && b < g.d1 && inter(a, b)) {
        const long long ox = cell_off(g, a, b, 0);
        const T qx = qp[ox];
        acc = fma(lam_next[ox] * num * qx * qx * qx, u[ox] - uy, acc);
      }
    });
    if (yin) {
      lam_prev[o] = acc;
    } else {
      hg[o] += acc;
      lam_prev[o] = T(0);
    }
  }
  if (want_coef) {
    __shared__ double red[kAdjThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double v = pnum;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
#pragma unroll
      for (int ww = 0; ww < kAdjThreads / 32; ++ww) s += red[ww];
      part[blockIdx.x] += s;
    }
  }
}

// zero the halo of a plane (lam_T's halo carries no gradient)
template <typename T>
__global__ void zero_halo_kernel(T *x, AdjGeom g) {
  const long long c = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  if (c >= g.cells) return;
  int i, j, k = 0;
  if (g.dim == 2) {
    i = (int)(c / g.d1);
    j = (int)(c % g.d1);
  } else {
    i = (int)(c / ((long long)g.d1 * g.d2));
    const long long r = c % ((long long)g.d1 * g.d2);
    j = (int)(r / g.d2);
    k = (int)(r % g.d2);
  }
  const int R = g.rad;
  const bool interior = i >= R && i < g.d0 - R && j >= R && j < g.d1 - R && (g.dim == 2 || (k >= R && k < g.d2 - R));
  if (!interior) x[cell_off(g, i, j, k)] = T(0);
}

// grad_u0 = lam_0 on the interior, the accumulated halo gradient on the halo
template <typename T>
__global__ void combine_kernel(const T *lam0, const T *hg, T *out, AdjGeom g) {
  const long long c = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  if (c >= g.cells) return;
  int i, j, k = 0;
  if (g.dim == 2) {
    i = (int)(c / g.d1);
    j = (int)(c % g.d1);
  } else {
    i = (int)(c / ((long long)g.d1 * g.d2));
    const long long r = c % ((long long)g.d1 * g.d2);
    j = (int)(r / g.d2);
    k = (int)(r % g.d2);
  }
  const int R = g.rad;
  const bool interior = i >= R && i < g.d0 - R && j >= R && j < g.d1 - R && (g.dim == 2 || (k >= R && k < g.d2 - R));
  const long long o = cell_off(g, i, j, k);
  out[o] = interior ? lam0[o] : hg[o];
}

__global__ void sum_parts_kernel(const double *part, int nblocks, int nt, double *out) {
  const int t = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += part[(size_t)b * nt + t];
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[t] = red[0];
}

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
struct Workspace {
  int ncp, C, nblocks, nt;
  int slots;            // stash planes: 2C (two chunk buffers) or fewer (revolve)
  bool revolve;         // chunks reversed by the binomial schedule
  size_t plane_bytes;
  size_t off_cp, off_stash, off_lam, off_hg, off_q, off_sd, off_part, total;
};

// The stash holds two chunk buffers of C planes when slots >= 2C; with fewer
// slots it holds `slots` snapshot planes plus two work planes of the
// binomial schedule.
Workspace workspace_of(const gbs_desc *d, const Layout &L, int C, int slots) {
  Workspace w{};
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  w.C = C;
  w.ncp = (d->timestep + C - 1) / C;
  if (w.ncp < 1) w.ncp = 1;
  w.revolve = slots < 2 * C;
  w.slots = w.revolve ? slots : 2 * C;
  w.plane_bytes = (size_t)L.plane * L.esize;
  const long long cells = (long long)L.dims[0] * L.dims[1] * L.dims[2];
  const bool grad = s->kind == 1;
  w.nblocks = grad ? (int)((cells + kAdjThreads - 1) / kAdjThreads) : kCoefBlocks;
  w.nt = grad ? 1 : std::min(s->nterms, kMaxCoefGrad);
  w.off_cp = 0;
  w.off_stash = w.off_cp + (size_t)w.ncp * w.plane_bytes;
  w.off_lam = w.off_stash + (size_t)(w.revolve ? w.slots + 2 : 2 * C) * w.plane_bytes;
  w.off_hg = w.off_lam + 2 * w.plane_bytes;
  w.off_q = w.off_hg + w.plane_bytes;
  w.off_sd = w.off_q + (grad ? w.plane_bytes : 0);
  w.off_part = w.off_sd + (grad ? w.plane_bytes : 0);
  w.total = w.off_part + (size_t)w.nblocks * w.nt * sizeof(double) + 256;
  return w;
}

AdjGeom geom_of(const Layout &L) {
  AdjGeom g{};
  g.pitch = L.pitch;
  g.plane = L.plane;
  g.d0 = L.dims[0];
  g.d1 = L.dims[1];
  g.d2 = L.dims[2];
  g.dim = L.dim;
  g.shift = (int)L.shift;
  g.rad = L.rad;
  g.rows = (int)L.rows;
  g.last = L.dims[L.dim - 1];
  g.cells = (long long)L.dims[0] * L.dims[1] * L.dims[2];
  return g;
}

// coefficients of the forward update as the source writes them, divisor and eps
void forward_coefficients(const gbs_desc *d, std::vector<double> &coef, double &div, double &eps) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const int nt = s->kind == 1 ? 1 : s->nterms;
  coef.assign(nt, 0.0);
  for (int t = 0; t < nt; ++t) {
    double c;
    if (d->coef) c = d->dtype == GBS_F64 ? ((const double *)d->coef)[t] : ((const float *)d->coef)[t];
    else c = s->kind == 1 ? (double)s->numerator : (double)s->terms[t].coef;
    coef[t] = c;
  }
  div = d->divisor != 0.0 ? d->divisor : (double)s->divisor;
  eps = d->eps != 0.0 ? d->eps : (double)s->eps;
}

// the forward coefficient of the mirrored offset, per term (linear stencils)
bool transposed_coefficients(const gbs_stencil_def_t *s, const std::vector<double> &coef, std::vector<double> &out) {
  out.assign(s->nterms, 0.0);
  for (int t = 0; t < s->nterms; ++t) {
    int m = -1;
    for (int u = 0; u < s->nterms; ++u)
      if (s->terms[u].di == -s->terms[t].di && s->terms[u].dj == -s->terms[t].dj &&
          s->terms[u].dk == -s->terms[t].dk)
        m = u;
    if (m < 0) return false;
    out[t] = coef[m];
  }
  return true;
}

// kernels of one stencil and dtype
struct AdjKernels {
  cudaError_t (*fused2d)(const AdjGeom &, const void *, const void *, void *, void *, double *,
                         const std::vector<double> &, double, bool, cudaStream_t);
  cudaError_t (*halo)(const AdjGeom &, const void *, void *, const std::vector<double> &, double, cudaStream_t);
  cudaError_t (*coef)(const AdjGeom &, const void *, const void *, double *, double, cudaStream_t);
  cudaError_t (*grad)(const AdjGeom &, const void *, void *, void *, const void *, void *, void *, double *, double,
                      double, bool, cudaStream_t);
};

// CTAs of a grid-stride kernel: one wave of resident CTAs (at most
// kCoefBlocks, the rows of the partial-sum table), so that no partial second
// wave repeats the per-CTA latency
template <class K>
int one_wave(K kernel) {
  int nb = 0, dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kAdjThreads, 0) != cudaSuccess || nb <= 0) {
    (void)cudaGetLastError();
    return kCoefBlocks;
  }
  return std::max(1, std::min(kCoefBlocks, nb * sms));
}

// one_wave(kernel) on the current device, computed once per (device
// ordinal, kernel): kernels of the same signature (the variants with and
// without products, stencils with as many terms) differ in registers and so
// in resident CTAs, and a process may drive GPUs with different SM counts
template <class K>
int wave_cached(K kernel) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return one_wave(kernel);
  }
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(dev, reinterpret_cast<const void *>(kernel));
  auto it = cache.find(key);
  if (it == cache.end()) it = cache.emplace(key, one_wave(kernel)).first;
  return it->second;
}

// one thread per halo cell of the interior rows, one warp per segment of an all-halo row
unsigned halo_grid(const AdjGeom &g) {
  const HaloPlan h = halo_plan(g);
  const long long threads = h.na + h.rows_b * h.nseg * 32;
  return (unsigned)std::max<long long>(1, (threads + kAdjThreads - 1) / kAdjThreads);
}

template <class ST, typename T>
cudaError_t run_halo(const AdjGeom &g, const void *lam, void *hg, const std::vector<double> &coef, double div,
                     cudaStream_t s) {
  if constexpr (ST::kKind == KIND_GRADIENT) {
    return cudaErrorInvalidValue;
  } else {
    LinCoef<T, ST::kTerms> cf;
    const double dv = ST::kHasDiv ? div : 1.0;
    for (int t = 0; t < ST::kTerms; ++t) cf.c[t] = (T)(coef[t] / dv);
    halo_kernel<ST, T><<<halo_grid(g), kAdjThreads, 0, s>>>(g, static_cast<const T *>(lam), static_cast<T *>(hg), cf);
    return cudaGetLastError();
  }
}

template <class ST, typename T>
cudaError_t run_fused2d(const AdjGeom &g, const void *lam, const void *u, void *lam_out, void *hg, double *part,
                        const std::vector<double> &coef, double div, bool want_coef, cudaStream_t s) {
  if constexpr (ST::kKind == KIND_GRADIENT || ST::kDim != 2 || ST::kTerms > kMaxCoefGrad) {
    return cudaErrorInvalidValue;
  } else {
    LinCoef<T, ST::kTerms> cf;
    const double dv = ST::kHasDiv ? div : 1.0;
    for (int t = 0; t < ST::kTerms; ++t) cf.c[t] = (T)(coef[t] / dv);
    const T inv = (T)(1.0 / dv);
    const HaloPlan hp = halo_plan(g);
    const long long halo_threads = hp.na + hp.rows_b * hp.nseg * 32;
    const unsigned halo_blocks = (unsigned)((halo_threads + kAdjThreads - 1) / kAdjThreads);
    const int wave_c = wave_cached(adj2d_kernel<ST, T, true>);
    const int wave_n = wave_cached(adj2d_kernel<ST, T, false>);
    // rows per work unit: about one unit per resident warp, at least 4 rows
    // so that the 2R rows each unit loads to fill its window stay a minor cost
    constexpr int SEG = 32 * (16 / sizeof(T));
    const long long nseg = (g.last - 2 * ST::kRad + SEG - 1) / SEG;
    const int ni = g.d0 - 2 * ST::kRad;
    auto rows_for = [&](int wave) {
      const long long warps = (long long)wave * (kAdjThreads / 32);
      const long long per = (ni * nseg + warps - 1) / std::max(1LL, warps);
      return (int)std::max<long long>(4, std::min<long long>(ni, per));
    };
    if (want_coef)
      adj2d_kernel<ST, T, true><<<wave_c + halo_blocks, kAdjThreads, 0, s>>>(
          g, static_cast<const T *>(lam), static_cast<const T *>(u), static_cast<T *>(lam_out), static_cast<T *>(hg),
          part, cf, inv, wave_c, rows_for(wave_c));
    else
      adj2d_kernel<ST, T, false><<<wave_n + halo_blocks, kAdjThreads, 0, s>>>(
          g, static_cast<const T *>(lam), static_cast<const T *>(u), static_cast<T *>(lam_out), static_cast<T *>(hg),
          part, cf, inv, wave_n, rows_for(wave_n));
    return cudaGetLastError();
  }
}

template <class ST, typename T>
cudaError_t run_coef(const AdjGeom &g, const void *lam, const void *u, double *part, double div, cudaStream_t s) {
  if constexpr (ST::kKind == KIND_GRADIENT || ST::kTerms > kMaxCoefGrad) {
    return cudaErrorInvalidValue;
  } else {
    const double dv = ST::kHasDiv ? div : 1.0;
    const int wave = wave_cached(coef_kernel<ST, T>);
    coef_kernel<ST, T><<<wave, kAdjThreads, 0, s>>>(g, static_cast<const T *>(lam), static_cast<const T *>(u), part,
                                                    (T)(1.0 / dv));
    return cudaGetLastError();
  }
}

template <class ST, typename T>
cudaError_t run_grad(const AdjGeom &g, const void *u, void *q, void *sd, const void *lam_next, void *lam_prev,
                     void *hg, double *part, double num, double eps, bool want_coef, cudaStream_t s) {
  if constexpr (ST::kKind != KIND_GRADIENT) {
    return cudaErrorInvalidValue;
  } else {
    const unsigned blocks = (unsigned)((g.cells + kAdjThreads - 1) / kAdjThreads);
    grad_pre_kernel<ST, T><<<blocks, kAdjThreads, 0, s>>>(g, static_cast<const T *>(u), static_cast<T *>(q),
                                                          static_cast<T *>(sd), (T)eps);
    grad_adj_kernel<ST, T><<<blocks, kAdjThreads, 0, s>>>(
        g, static_cast<const T *>(u), static_cast<const T *>(q), static_cast<const T *>(sd),
        static_cast<const T *>(lam_next), static_cast<T *>(lam_prev), static_cast<T *>(hg), part, (T)num,
        want_coef ? 1 : 0);
    return cudaGetLastError();
  }
}

AdjKernels adj_kernels(int sid, int dtype) {
  switch (sid) {
#define GBS_ADJ(id, S)                                                                            \
  case id:                                                                                         \
    return dtype == GBS_F64                                                                       \
               ? AdjKernels{&run_fused2d<S, double>, &run_halo<S, double>, &run_coef<S, double>,      \
                            &run_grad<S, double>}                                                       \
               : AdjKernels{&run_fused2d<S, float>, &run_halo<S, float>, &run_coef<S, float>, &run_grad<S, float>};
    GBS_FOR_EACH_STENCIL(GBS_ADJ)
#undef GBS_ADJ
    default:
      return AdjKernels{nullptr, nullptr, nullptr, nullptr};
  }
}

// ---------------------------------------------------------------------------
// binomial (revolve) schedule
// ---------------------------------------------------------------------------
// beta(s, r) = (s + r)! / (s! r!): the most steps s snapshots reverse with
// every step advanced at most r times (saturating)
long long revolve_beta(int s, int r) {
  long long v = 1;
  for (int i = 1; i <= s; ++i) {
    v = v * (r + i) / i;
    if (v > (1LL << 40)) return 1LL << 40;
  }
  return v;
}

// Where to place the next snapshot when reversing l >= 2 steps from a stored
// state with k >= 1 free snapshot slots (k + 1 stored states in all): r is
// the least number of advances per step with beta(k+1, r) >= l. The split
// m = l - beta(k, r-1), kept within [1, min(l-1, beta(k+1, r-1))], leaves
// the right part (l - m steps, from the new snapshot, k - 1 slots left) as
// long as r - 1 advances per step allow and the left part (m steps, k
// slots) no longer than r - 1 advances allow; the total is then
// r*l - beta(k+2, r-1) forward steps, the minimum (checked against an
// exhaustive search over every split by the tests).
int revolve_split(int l, int k) {
  int r = 1;
  while (revolve_beta(k + 1, r) < l) ++r;
  long long m = l - revolve_beta(k, r - 1);
  if (m < 1) m = 1;
  const long long hi = std::min<long long>(l - 1, revolve_beta(k + 1, r - 1));
  return (int)std::max(1LL, std::min(m, hi));
}

// forward steps the schedule takes to reverse l steps with s free slots, and
// the most slots it holds at once
void revolve_count(int l, int s, long long *steps, int *peak, int depth = 0) {
  if (depth > *peak) *peak = depth;
  if (l <= 1) return;
  if (s == 0) {
    *steps += (long long)l * (l - 1) / 2;
    return;
  }
  const int m = revolve_split(l, s);
  *steps += m;
  revolve_count(l - m, s - 1, steps, peak, depth + 1);
  revolve_count(m, s, steps, peak, depth);
}

gbs_status check_adjoint_args(const gbs_desc *d, int C, const void *ws) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (C < 1) return fail(GBS_ERR_INVALID, "checkpoint interval must be >= 1");
  if (!ws) return fail(GBS_ERR_INVALID, "workspace is NULL");
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0) return fail(GBS_ERR_INVALID, "workspace must be 256-byte aligned");
  return GBS_OK;
}

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, what);   \
  } while (0)

// Branch streams of the batched entry points, per device: work forked from
// the caller's stream (an event), spread over the branches, joined back.
constexpr int kBranches = 16;
struct Branches {
  cudaStream_t s[kBranches] = {};
  cudaEvent_t fork = nullptr, join[kBranches] = {};
};
std::mutex g_branch_mu;  // held while a batched call enqueues (one set of events per device)
Branches g_branches[64];

gbs_status device_branches(Branches **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(GBS_ERR_NODEVICE, "device ordinal %d unsupported", dev);
  Branches &b = g_branches[dev];
  if (!b.fork) {
    for (int k = 0; k < kBranches && e == cudaSuccess; ++k) {
      e = cudaStreamCreateWithFlags(&b.s[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.join[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint batch: branch streams");
  }
  *out = &b;
  return GBS_OK;
}

// Runs run(i, branch_stream) for i < n on the branches (instance i on branch
// i % kBranches), ordered after the work already on `stream`, and makes
// `stream` wait for all of it.
template <class F>
gbs_status on_branches(int n, cudaStream_t stream, F run) {
  std::lock_guard<std::mutex> lk(g_branch_mu);
  Branches *b = nullptr;
  gbs_status st = device_branches(&b);
  if (st != GBS_OK) return st;
  const int used = std::min(n, kBranches);
  CK(cudaEventRecord(b->fork, stream), "adjoint batch: fork");
  for (int k = 0; k < used; ++k) CK(cudaStreamWaitEvent(b->s[k], b->fork, 0), "adjoint batch: fork");
  for (int i = 0; i < n && st == GBS_OK; ++i) st = run(i, b->s[i % kBranches]);
  // join even after a failure, so that `stream` never runs ahead of work already enqueued
  for (int k = 0; k < used; ++k) {
    cudaEventRecord(b->join[k], b->s[k]);
    cudaStreamWaitEvent(stream, b->join[k], 0);
  }
  return st;
}

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" {

gbs_status gbs_adjoint_workspace(const gbs_desc *d, int checkpoint_every, size_t *bytes) {
  return gbs_adjoint_workspace_slots(d, checkpoint_every, 2 * std::max(1, checkpoint_every), bytes);
}

gbs_status gbs_adjoint_workspace_slots(const gbs_desc *d, int checkpoint_every, int slots, size_t *bytes) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (checkpoint_every < 1 || !bytes) return fail(GBS_ERR_INVALID, "bad checkpoint interval or NULL bytes");
  if (slots < 0) return fail(GBS_ERR_INVALID, "slots must be >= 0");
  const Layout L = make_layout(d);
  *bytes = workspace_of(d, L, checkpoint_every, slots).total;
  return GBS_OK;
}

gbs_status gbs_revolve_cost(int steps, int slots, long long *forward_steps, int *peak_slots) {
  if (steps < 0 || slots < 0 || !forward_steps) return fail(GBS_ERR_INVALID, "bad revolve arguments");
  long long n = 0;
  int peak = 0;
  revolve_count(steps, slots, &n, &peak);
  *forward_steps = n;
  if (peak_slots) *peak_slots = peak;
  return GBS_OK;
}

gbs_status gbs_adjoint_plan_budget(const gbs_desc *d, size_t budget_bytes, int *checkpoint_every, int *slots,
                                   size_t *bytes) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!checkpoint_every || !slots) return fail(GBS_ERR_INVALID, "NULL output");
  const Layout L = make_layout(d);
  const int T = std::max(1, d->timestep);
  // every checkpoint interval C, every slot count: the fewest recomputed
  // forward steps whose workspace fits (ties: the smaller workspace)
  long long best_cost = -1;
  size_t best_bytes = 0;
  int best_c = 0, best_s = 0;
  for (int C = 1; C <= T; ++C) {
    const int ncp = (T + C - 1) / C;
    const Workspace w0 = workspace_of(d, L, C, 0);
    if (w0.total > budget_bytes) continue;
    // slots that still fit: revolve below 2C, the double stash at 2C
    const long long room = (long long)((budget_bytes - w0.total) / w0.plane_bytes);
    int s = (int)std::min<long long>(room, 2LL * C);
    long long cost;
    if (s >= 2 * C) {
      cost = (long long)T - ncp;  // each chunk recomputed once (its states after the checkpoint)
    } else {
      cost = 0;
      for (int j = 0; j < ncp; ++j) {
        long long n = 0;
        int peak = 0;
        revolve_count(std::min(C, T - j * C), s, &n, &peak);
        cost += n;
      }
    }
    const size_t b = workspace_of(d, L, C, s).total;
    if (b > budget_bytes) continue;
    if (best_cost < 0 || cost < best_cost || (cost == best_cost && b < best_bytes)) {
      best_cost = cost;
      best_bytes = b;
      best_c = C;
      best_s = s;
    }
  }
  if (best_cost < 0) return fail(GBS_ERR_NOMEM, "no checkpoint schedule fits %zu bytes", budget_bytes);
  *checkpoint_every = best_c;
  *slots = best_s;
  if (bytes) *bytes = best_bytes;
  return GBS_OK;
}

gbs_status gbs_adjoint_forward(const gbs_desc *d, void *dev_A, int checkpoint_every, void *workspace,
                               void *stream) {
  gbs_status st = check_adjoint_args(d, checkpoint_every, workspace);
  if (st != GBS_OK) return st;
  if (!dev_A) return fail(GBS_ERR_INVALID, "dev_A is NULL");
  int *err = nullptr;
  if ((st = error_word(&err)) != GBS_OK) return st;
  const Layout L = make_layout(d);
  const Workspace w = workspace_of(d, L, checkpoint_every, 2 * checkpoint_every);
  char *ws = static_cast<char *>(workspace);
  char *A = static_cast<char *>(dev_A);
  cudaStream_t s = (cudaStream_t)stream;
  for (int j = 0; j < w.ncp; ++j) {
    const int t0 = j * w.C;
    const int c = std::min(w.C, d->timestep - t0);
    CK(cudaMemcpyAsync(ws + w.off_cp + (size_t)j * w.plane_bytes, A, w.plane_bytes, cudaMemcpyDeviceToDevice, s),
       "adjoint: checkpoint");
    if (c <= 0) break;
    gbs_desc dc = *d;
    dc.timestep = c;
    if ((st = run_loop(&dc, L, dev_A, s, err)) != GBS_OK) return st;
    if (c % 2) CK(cudaMemcpyAsync(A, A + w.plane_bytes, w.plane_bytes, cudaMemcpyDeviceToDevice, s), "adjoint: plane");
  }
  // u_T in both planes
  CK(cudaMemcpyAsync(A + w.plane_bytes, A, w.plane_bytes, cudaMemcpyDeviceToDevice, s), "adjoint: plane");
  return GBS_OK;
}

gbs_status gbs_adjoint_backward(const gbs_desc *d, const void *dev_lamT, void *dev_grad_u0, double *dev_coef_grad,
                                int checkpoint_every, void *workspace, void *stream) {
  return gbs_adjoint_backward_slots(d, dev_lamT, dev_grad_u0, dev_coef_grad, checkpoint_every,
                                    2 * std::max(1, checkpoint_every), workspace, stream);
}

gbs_status gbs_adjoint_backward_slots(const gbs_desc *d, const void *dev_lamT, void *dev_grad_u0,
                                      double *dev_coef_grad, int checkpoint_every, int slots, void *workspace,
                                      void *stream) {
  gbs_status st = check_adjoint_args(d, checkpoint_every, workspace);
  if (st != GBS_OK) return st;
  if (slots < 0) return fail(GBS_ERR_INVALID, "slots must be >= 0");
  if (!dev_lamT || !dev_grad_u0) return fail(GBS_ERR_INVALID, "NULL lam_T or grad_u0");
  const gbs_stencil_def_t *sd = stencil_def(d->stencil);
  const bool gradient = sd->kind == 1;
  if (dev_coef_grad && !gradient && sd->nterms > kMaxCoefGrad)
    return fail(GBS_ERR_UNSUPPORTED, "coefficient gradients need at most %d terms", kMaxCoefGrad);
  int *err = nullptr;
  if ((st = error_word(&err)) != GBS_OK) return st;
  const Layout L = make_layout(d);
  const Workspace w = workspace_of(d, L, checkpoint_every, slots);
  const AdjGeom g = geom_of(L);
  char *ws = static_cast<char *>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  const AdjKernels K = adj_kernels(d->stencil, d->dtype);
  const unsigned blocks = (unsigned)((g.cells + kAdjThreads - 1) / kAdjThreads);
  char *stash = ws + w.off_stash;
  char *lam[2] = {ws + w.off_lam, ws + w.off_lam + w.plane_bytes};
  char *hg = ws + w.off_hg;
  double *part = reinterpret_cast<double *>(ws + w.off_part);

  std::vector<double> coef, coefT;
  double div = 0.0, eps = 0.0;
  forward_coefficients(d, coef, div, eps);
  if (sd->divisor && div == 0.0) return fail(GBS_ERR_INVALID, "divisor must be nonzero");
  if (!gradient && !transposed_coefficients(sd, coef, coefT))
    return fail(GBS_ERR_UNSUPPORTED, "%s has an asymmetric offset set", sd->name);
  gbs_desc dT = *d;  // the transposed step: the forward kernels, FMA mode
  dT.fp_mode = GBS_FP_FMA;

  CK(cudaMemcpyAsync(lam[0], dev_lamT, w.plane_bytes, cudaMemcpyDeviceToDevice, s), "adjoint: lam_T");
  if (d->dtype == GBS_F64) zero_halo_kernel<double><<<blocks, kAdjThreads, 0, s>>>((double *)lam[0], g);
  else zero_halo_kernel<float><<<blocks, kAdjThreads, 0, s>>>((float *)lam[0], g);
  CK(cudaMemsetAsync(lam[1], 0, w.plane_bytes, s), "adjoint: memset");
  CK(cudaMemsetAsync(hg, 0, w.plane_bytes, s), "adjoint: memset");
  CK(cudaMemsetAsync(part, 0, (size_t)w.nblocks * w.nt * sizeof(double), s), "adjoint: memset");
  int cur = 0;
  // one adjoint step lam[cur] (= lam_{t+1}) -> lam[cur ^ 1] (= lam_t) on state u_t
  auto step = [&](const char *u) -> gbs_status {
    if (gradient) {
      CK(K.grad(g, u, ws + w.off_q, ws + w.off_sd, lam[cur], lam[cur ^ 1], hg, part, coef[0], eps,
                dev_coef_grad != nullptr, s),
         "adjoint: gradient2d step");
    } else if (g.dim == 2 && sd->nterms <= kMaxCoefGrad) {
      CK(K.fused2d(g, lam[cur], u, lam[cur ^ 1], hg, part, coef, div, dev_coef_grad != nullptr, s),
         "adjoint: fused 2-D step");
    } else {
      CK(K.halo(g, lam[cur], hg, coef, div, s), "adjoint: halo");
      if (dev_coef_grad) CK(K.coef(g, lam[cur], u, part, div, s), "adjoint: coefficients");
      gbs_status r = launch_block(&dT, L, coefT.data(), div, eps, 0, 1, lam[cur], lam[cur ^ 1], s, err);
      if (r != GBS_OK) return r;
    }
    cur ^= 1;
    return GBS_OK;
  };

  if (!gradient && !dev_coef_grad) {
    // no forward state enters: T transposed steps from lam_T
    for (int t = d->timestep - 1; t >= 0; --t)
      if ((st = step(nullptr)) != GBS_OK) return st;
  } else if (w.revolve) {
    // Each chunk reversed by the binomial schedule over `slots` snapshot
    // planes and two work planes, all on `s`. The halo of every stash plane
    // is the fixed boundary (copied once; launches never write it).
    for (int k = 0; k < w.slots + 2; ++k)
      CK(cudaMemcpyAsync(stash + (size_t)k * w.plane_bytes, ws + w.off_cp, w.plane_bytes, cudaMemcpyDeviceToDevice,
                         s),
         "adjoint: stash");
    char *work0 = stash + (size_t)w.slots * w.plane_bytes;  // ping-pong partner of an advance
    char *work1 = work0 + w.plane_bytes;                     // target of a recompute without slots
    gbs_plan_info pi{};
    {
      gbs_desc dp = *d;
      dp.timestep = std::max(1, w.C);
      if ((st = gbs_plan(&dp, &pi)) != GBS_OK) return st;
    }
    const int bfwd = std::max(1, pi.bt);
    // advance k >= 1 steps from plane src into plane dst (dst != work0)
    auto advance = [&](const char *src, char *dst, int k) -> gbs_status {
      const std::vector<int> blocks_k = split_steps(k, bfwd);
      const int n = (int)blocks_k.size();
      const char *from = src;
      for (int j = 0; j < n; ++j) {
        char *to = ((n - 1 - j) % 2 == 0) ? dst : work0;
        gbs_status r = launch_block(d, L, coef.data(), div, eps, 0, blocks_k[j], from, to, s, err);
        if (r != GBS_OK) return r;
        from = to;
      }
      return GBS_OK;
    };
    // reverse steps [a, b) given u_a in plane ua, with `nfree` snapshot slots
    // free from index `top` on
    std::function<gbs_status(int, int, const char *, int)> reverse = [&](int a, int b, const char *ua,
                                                                         int top) -> gbs_status {
      const int l = b - a, nfree = w.slots - top;
      if (l <= 0) return GBS_OK;
      if (l == 1) return step(ua);
      if (nfree == 0) {
        for (int t = b - 1; t > a; --t) {
          gbs_status r = advance(ua, work1, t - a);
          if (r == GBS_OK) r = step(work1);
          if (r != GBS_OK) return r;
        }
        return step(ua);
      }
      const int m = revolve_split(l, nfree);
      char *snap = stash + (size_t)top * w.plane_bytes;
      gbs_status r = advance(ua, snap, m);
      if (r == GBS_OK) r = reverse(a + m, b, snap, top + 1);
      if (r == GBS_OK) r = reverse(a, a + m, ua, top);
      return r;
    };
    for (int j = w.ncp - 1; j >= 0 && st == GBS_OK; --j) {
      const int t0 = j * w.C;
      const int c = std::min(w.C, d->timestep - t0);
      st = reverse(t0, t0 + c, ws + w.off_cp + (size_t)j * w.plane_bytes, 0);
    }
    if (st != GBS_OK) return st;
  } else {
    // Two stash buffers: while the adjoint steps of chunk j run on `s`, a
    // second stream recomputes the states of chunk j-1 into the other
    // buffer. Events order it: a buffer is refilled only after the adjoint
    // steps that read it (freed), and read only after its refill (ready).
    const size_t buf_bytes = (size_t)w.C * w.plane_bytes;
    cudaStream_t s2 = nullptr;
    cudaEvent_t setup = nullptr, done2 = nullptr, ready[2] = {}, freed[2] = {};
    auto release = [&]() {
      for (int b = 0; b < 2; ++b) {
        if (ready[b]) cudaEventDestroy(ready[b]);
        if (freed[b]) cudaEventDestroy(freed[b]);
      }
      if (setup) cudaEventDestroy(setup);
      if (done2) cudaEventDestroy(done2);
      if (s2) cudaStreamDestroy(s2);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&setup, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done2, cudaEventDisableTiming);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
      e = cudaEventCreateWithFlags(&ready[b], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&freed[b], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      release();
      return cuda_fail(e, "adjoint: streams");
    }
    // the halo of every stash slot of both buffers: the fixed boundary (never rewritten)
    for (int k = 0; k < 2 * w.C; ++k) {
      e = cudaMemcpyAsync(stash + (size_t)k * w.plane_bytes, ws + w.off_cp, w.plane_bytes, cudaMemcpyDeviceToDevice,
                          s);
      if (e != cudaSuccess) {
        release();
        return cuda_fail(e, "adjoint: stash");
      }
    }
    cudaEventRecord(setup, s);
    cudaStreamWaitEvent(s2, setup, 0);
    // recompute degree: 2-D grids in FMA mode use the forward's fused degree
    // (at most the largest stash-mode degree), each launch also storing its
    // intermediate states; otherwise one step per launch
    int bre = 1;
    if (g.dim == 2 && d->fp_mode == GBS_FP_FMA) {
      gbs_desc dp = *d;
      dp.timestep = std::max(1, w.C);
      gbs_plan_info pi{};
      if ((st = gbs_plan(&dp, &pi)) != GBS_OK) {
        release();
        return st;
      }
      bre = std::max(1, std::min(pi.bt, kMaxStashB));
    }
    // recompute u_{t0} .. u_{t0+c-1} of chunk j into buffer j % 2 on s2
    auto recompute = [&](int j) -> gbs_status {
      const int b = j & 1;
      char *buf = stash + (size_t)b * buf_bytes;
      const int c = std::min(w.C, d->timestep - j * w.C);
      cudaStreamWaitEvent(s2, freed[b], 0);  // no-op before the buffer's first use
      cudaError_t ce = cudaMemcpyAsync(buf, ws + w.off_cp + (size_t)j * w.plane_bytes, w.plane_bytes,
                                       cudaMemcpyDeviceToDevice, s2);
      if (ce != cudaSuccess) return cuda_fail(ce, "adjoint: restore");
      for (int k = 1; k < c;) {
        // one launch of bb steps from slot k-1: slots k .. k+bb-1
        const int bb = std::min(bre, c - k);
        gbs_status r = launch_block_stash(d, L, coef.data(), div, eps, 0, bb, buf + (size_t)(k - 1) * w.plane_bytes,
                                          buf + (size_t)(k - 1 + bb) * w.plane_bytes,
                                          bb > 1 ? buf + (size_t)k * w.plane_bytes : nullptr, s2, err);
        if (r != GBS_OK) return r;
        k += bb;
      }
      cudaEventRecord(ready[b], s2);
      return GBS_OK;
    };
    st = recompute(w.ncp - 1);
    for (int j = w.ncp - 1; j >= 0 && st == GBS_OK; --j) {
      const int b = j & 1;
      const int c = std::min(w.C, d->timestep - j * w.C);
      if (j > 0 && (st = recompute(j - 1)) != GBS_OK) break;  // overlaps the steps below
      cudaStreamWaitEvent(s, ready[b], 0);
      // lam_{t+1} -> lam_t for t = t0+c-1 .. t0
      char *buf = stash + (size_t)b * buf_bytes;
      for (int k = c - 1; k >= 0 && st == GBS_OK; --k) st = step(buf + (size_t)k * w.plane_bytes);
      cudaEventRecord(freed[b], s);
    }
    // every piece of s2's work is ordered before s (the last ready event); join anyway
    cudaEventRecord(done2, s2);
    cudaStreamWaitEvent(s, done2, 0);
    release();
    if (st != GBS_OK) return st;
  }
  if (d->dtype == GBS_F64)
    combine_kernel<double><<<blocks, kAdjThreads, 0, s>>>((const double *)lam[cur], (const double *)hg,
                                                         (double *)dev_grad_u0, g);
  else
    combine_kernel<float><<<blocks, kAdjThreads, 0, s>>>((const float *)lam[cur], (const float *)hg,
                                                        (float *)dev_grad_u0, g);
  if (dev_coef_grad) sum_parts_kernel<<<w.nt, 256, 0, s>>>(part, w.nblocks, w.nt, dev_coef_grad);
  CK(cudaGetLastError(), "adjoint: combine");
  return GBS_OK;
}

gbs_status gbs_adjoint_forward_batch(const gbs_desc *descs, int n, void *const *dev_A, int checkpoint_every,
                                     void *const *workspaces, void *stream) {
  if (!descs || n < 1 || !dev_A || !workspaces) return fail(GBS_ERR_INVALID, "adjoint batch: no instances");
  for (int i = 0; i < n; ++i) {
    gbs_status st = check_adjoint_args(&descs[i], checkpoint_every, workspaces[i]);
    if (st != GBS_OK) return st;
    if (!dev_A[i]) return fail(GBS_ERR_INVALID, "adjoint batch: instance %d has no grid", i);
  }
  return on_branches(n, (cudaStream_t)stream, [&](int i, cudaStream_t bs) {
    return gbs_adjoint_forward(&descs[i], dev_A[i], checkpoint_every, workspaces[i], bs);
  });
}

gbs_status gbs_adjoint_backward_batch(const gbs_desc *descs, int n, const void *const *dev_lamT,
                                      void *const *dev_grad_u0, double *const *dev_coef_grad, int checkpoint_every,
                                      void *const *workspaces, void *stream) {
  if (!descs || n < 1 || !dev_lamT || !dev_grad_u0 || !workspaces)
    return fail(GBS_ERR_INVALID, "adjoint batch: no instances");
  for (int i = 0; i < n; ++i) {
    gbs_status st = check_adjoint_args(&descs[i], checkpoint_every, workspaces[i]);
    if (st != GBS_OK) return st;
    if (!dev_lamT[i] || !dev_grad_u0[i]) return fail(GBS_ERR_INVALID, "adjoint batch: instance %d lacks a plane", i);
  }
  return on_branches(n, (cudaStream_t)stream, [&](int i, cudaStream_t bs) {
    return gbs_adjoint_backward(&descs[i], dev_lamT[i], dev_grad_u0[i], dev_coef_grad ? dev_coef_grad[i] : nullptr,
                                checkpoint_every, workspaces[i], bs);
  });
}

}  // extern "C"
