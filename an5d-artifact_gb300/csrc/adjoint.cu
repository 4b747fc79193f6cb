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
// each into its own stash slot), then runs the chunk's adjoint steps.
#include <cuda_runtime.h>

#include <algorithm>
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

// Element x (relative to the lane's first column, x in [-R, V+R)) of row
// offset D of a plane whose 2R+1 row vectors the lane holds: from its own
// vector or from a lane up to R/V away; lanes whose source lane lies outside
// the warp load the element.
template <int V, int R, int D, int X, typename T>
__device__ __forceinline__ T row_value(const T *p, const T (&rows)[2 * R + 1][V], long long base, long long pitch,
                                       int lane) {
  T v = row_elem<V, X>(rows[D + R]);
  if constexpr (X < 0) {
    constexpr int dl = (-X + V - 1) / V;
    if (lane < dl) v = p[base + (long long)D * pitch + X];
  } else if constexpr (X >= V) {
    constexpr int dl = X / V;
    if (lane >= 32 - dl) v = p[base + (long long)D * pitch + X];
  }
  return v;
}

// 2-D linear adjoint step, fused: lam_out(y) = sum_k c_k/d lam(y - o_k) on
// the interior (lam is zero on the halo; lam_out's halo is never written),
// with WANT_COEF the products lam(y) u(y + o_k) / d summed per thread and
// reduced per CTA into part[blockIdx.x][k], and hg(h) += the transposed sum
// at every halo cell h. One launch per step instead of the transposed engine
// step, the halo kernel and the product kernel: 2-D grids are small enough
// that a step is bound by kernel latency. The first `interior_blocks` CTAs
// take (interior row, 32*V-column) units: each lane one aligned 16-byte
// vector of V columns per row offset, the in-row neighbours from the
// lanes up to R/V away (the warp's edge lanes load theirs); the CTAs after
// them take the halo cells (one thread each).
template <class ST, typename T, bool WANT_COEF>
__global__ void __launch_bounds__(kAdjThreads) adj2d_kernel(const __grid_constant__ AdjGeom g,
                                                            const T *__restrict__ lam, const T *__restrict__ u,
                                                            T *__restrict__ lam_out, T *__restrict__ hg,
                                                            double *__restrict__ part,
                                                            const __grid_constant__ LinCoef<T, ST::kTerms> cf,
                                                            T inv_div, int interior_blocks) {
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
  const long long units = (long long)(g.d0 - 2 * R) * nseg;
  const long long nwarps = (long long)interior_blocks * (kAdjThreads / 32);
  for (long long un = (long long)blockIdx.x * (kAdjThreads / 32) + w; un < units; un += nwarps) {
    const int ii = (int)(un / nseg), seg = (int)(un - (long long)ii * nseg);
    const int i = R + ii;
    const int c0 = R + seg * SEG + lane * V;        // the lane's first column; 16-byte aligned
    const int nvalid = min(V, g.last - R - c0);     // columns of the group inside the interior
    const long long base = (long long)i * g.pitch + g.shift + c0;
    // the 2R+1 row vectors of the unit, each loaded once
    T lrow[2 * R + 1][V];
    static_for<2 * R + 1>([&](auto DI) {
      constexpr int d = decltype(DI)::value - R;
      ld_vec<T, V>(lrow[d + R], lam + base + (long long)d * g.pitch);
    });
    T sv[V];
#pragma unroll
    for (int e = 0; e < V; ++e) sv[e] = T(0);
    static_for<NT>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
      static_for<V>([&](auto EI) {
        constexpr int e = decltype(EI)::value;
        sv[e] = fma(cf.c[t], row_value<V, R, -di, e - dj>(lam, lrow, base, g.pitch, lane), sv[e]);
      });
    });
    if constexpr (WANT_COEF) {
      T urow[2 * R + 1][V];
      static_for<2 * R + 1>([&](auto DI) {
        constexpr int d = decltype(DI)::value - R;
        ld_vec<T, V>(urow[d + R], u + base + (long long)d * g.pitch);
      });
      static_for<NT>([&](auto TI) {
        constexpr int t = decltype(TI)::value;
        constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1];
        static_for<V>([&](auto EI) {
          constexpr int e = decltype(EI)::value;
          const T uv = row_value<V, R, di, e + dj>(u, urow, base, g.pitch, lane);
          if (e < nvalid) acc[t] = fma(lrow[R][e], uv, acc[t]);
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
    auto inter = [&](int a, int b) { return a >= R && a < g.d0 - R && b >= R && b < g.d1 - R; };
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
  size_t plane_bytes;
  size_t off_cp, off_stash, off_lam, off_hg, off_q, off_sd, off_part, total;
};

Workspace workspace_of(const gbs_desc *d, const Layout &L, int C) {
  Workspace w{};
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  w.C = C;
  w.ncp = (d->timestep + C - 1) / C;
  if (w.ncp < 1) w.ncp = 1;
  w.plane_bytes = (size_t)L.plane * L.esize;
  const long long cells = (long long)L.dims[0] * L.dims[1] * L.dims[2];
  const bool grad = s->kind == 1;
  w.nblocks = grad ? (int)((cells + kAdjThreads - 1) / kAdjThreads) : kCoefBlocks;
  w.nt = grad ? 1 : std::min(s->nterms, kMaxCoefGrad);
  w.off_cp = 0;
  w.off_stash = w.off_cp + (size_t)w.ncp * w.plane_bytes;
  w.off_lam = w.off_stash + 2 * (size_t)C * w.plane_bytes;  // two stash buffers
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

// one_wave(kernel) for the current device, computed once per device ordinal
// (a process may drive GPUs with different SM counts)
template <class K>
int wave_cached(K kernel) {
  static std::mutex mu;
  static int cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    (void)cudaGetLastError();
    return one_wave(kernel);
  }
  std::lock_guard<std::mutex> lk(mu);
  if (cache[dev] == 0) cache[dev] = one_wave(kernel);
  return cache[dev];
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
    if (want_coef)
      adj2d_kernel<ST, T, true><<<wave_c + halo_blocks, kAdjThreads, 0, s>>>(
          g, static_cast<const T *>(lam), static_cast<const T *>(u), static_cast<T *>(lam_out), static_cast<T *>(hg),
          part, cf, inv, wave_c);
    else
      adj2d_kernel<ST, T, false><<<wave_n + halo_blocks, kAdjThreads, 0, s>>>(
          g, static_cast<const T *>(lam), static_cast<const T *>(u), static_cast<T *>(lam_out), static_cast<T *>(hg),
          part, cf, inv, wave_n);
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

}  // namespace
}  // namespace gbs

using namespace gbs;

extern "C" {

gbs_status gbs_adjoint_workspace(const gbs_desc *d, int checkpoint_every, size_t *bytes) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (checkpoint_every < 1 || !bytes) return fail(GBS_ERR_INVALID, "bad checkpoint interval or NULL bytes");
  const Layout L = make_layout(d);
  *bytes = workspace_of(d, L, checkpoint_every).total;
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
  const Workspace w = workspace_of(d, L, checkpoint_every);
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
  gbs_status st = check_adjoint_args(d, checkpoint_every, workspace);
  if (st != GBS_OK) return st;
  if (!dev_lamT || !dev_grad_u0) return fail(GBS_ERR_INVALID, "NULL lam_T or grad_u0");
  const gbs_stencil_def_t *sd = stencil_def(d->stencil);
  const bool gradient = sd->kind == 1;
  if (dev_coef_grad && !gradient && sd->nterms > kMaxCoefGrad)
    return fail(GBS_ERR_UNSUPPORTED, "coefficient gradients need at most %d terms", kMaxCoefGrad);
  int *err = nullptr;
  if ((st = error_word(&err)) != GBS_OK) return st;
  const Layout L = make_layout(d);
  const Workspace w = workspace_of(d, L, checkpoint_every);
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
    // recompute u_{t0} .. u_{t0+c-1} of chunk j into buffer j % 2 on s2
    auto recompute = [&](int j) -> gbs_status {
      const int b = j & 1;
      char *buf = stash + (size_t)b * buf_bytes;
      const int c = std::min(w.C, d->timestep - j * w.C);
      cudaStreamWaitEvent(s2, freed[b], 0);  // no-op before the buffer's first use
      cudaError_t ce = cudaMemcpyAsync(buf, ws + w.off_cp + (size_t)j * w.plane_bytes, w.plane_bytes,
                                       cudaMemcpyDeviceToDevice, s2);
      if (ce != cudaSuccess) return cuda_fail(ce, "adjoint: restore");
      for (int k = 1; k < c; ++k) {
        gbs_status r = launch_block(d, L, coef.data(), div, eps, 0, 1, buf + (size_t)(k - 1) * w.plane_bytes,
                                    buf + (size_t)k * w.plane_bytes, s2, err);
        if (r != GBS_OK) return r;
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

}  // extern "C"
