// Adjoint (reverse-mode gradient) of the stencil time loop.
//
// No counterpart in the artifact: it differentiates the time loop that
// kernel_stencil runs. For u_{t+1} = F(u_t) on the interior (halo fixed)
// and a loss L(u_T) whose gradient lam_T = dL/du_T the caller supplies, it
// returns dL/du_0 (interior and halo) and, for linear stencils, dL/dc_k for
// the coefficients as the source writes them (before any divisor).
//
// Checkpointing: gbs_adjoint_forward advances the grid and saves u_t every
// C steps into the caller's workspace; gbs_adjoint_backward walks the chunks
// backwards, recomputes a chunk's C states from its checkpoint with the
// forward engine itself (consecutive stash slots form the two-plane buffer
// of a one-step launch), then runs the adjoint step kernel C times.
//
// Adjoint step (lam_{t+1} -> lam_t), with lam zero on the halo:
//  * linear: lam_t(y) = sum_k c_k/d * lam_{t+1}(y - o_k) (the transposed
//    stencil); at halo cells the same sum accumulates into the halo
//    gradient, since a halo value feeds every step; dL/dc_k gains
//    sum_x lam_{t+1}(x) u_t(x + o_k) / d, reduced per CTA into a partial
//    buffer (no atomics; summed at the end in double).
//  * gradient2d (u + c/sqrt(eps + s), s = sum_n (u - u_{x+n})^2): the
//    linearised update, dF(x)/du(x) = 1 - c g(x) sum_n d_n(x),
//    dF(x)/du(x+n) = c g(x) d_n(x), g = (eps + s)^{-3/2}, evaluated on u_t;
//    dF(x)/dc = (eps + s)^{-1/2}.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "engine_internal.h"
#include "gbs_device.cuh"

namespace gbs {
namespace {

constexpr int kAdjThreads = 256;
constexpr int kMaxCoefGrad = 32;  // coefficient gradients for stencils of at most this many terms

struct AdjGeom {
  long long pitch, plane;  // elements
  int d0, d1, d2, dim, shift, rad;
  long long cells;         // d0*d1*d2
};

__device__ __forceinline__ long long cell_off(const AdjGeom &g, int i, int j, int k) {
  return g.dim == 2 ? (long long)i * g.pitch + g.shift + j
                    : ((long long)i * g.d1 + j) * g.pitch + g.shift + k;
}

template <typename T, int NT> struct AdjParams {
  AdjGeom g;
  const T *u;          // u_t (one plane)
  const T *lam_next;   // lam_{t+1}, zero on the halo
  T *lam_prev;         // lam_t (interior written, halo zero)
  T *halo_grad;        // dL/d(halo), accumulated
  double *coef_part;   // [gridDim.x][NT] partial sums, accumulated
  T coef[NT];          // c_k / divisor
  T inv_div;           // 1 / divisor (1 without)
  int want_coef;
};

template <typename T>
__device__ __forceinline__ T ldz(const T *p, const AdjGeom &g, int i, int j, int k) {
  if (i < 0 || i >= g.d0 || j < 0 || j >= g.d1 || (g.dim == 3 && (k < 0 || k >= g.d2))) return T(0);
  return p[cell_off(g, i, j, k)];
}

template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) adjoint_linear_kernel(const __grid_constant__ AdjParams<T, ST::kTerms> p) {
  constexpr int NT = ST::kTerms;
  constexpr int NP = NT <= kMaxCoefGrad ? NT : 1;
  const AdjGeom &g = p.g;
  const long long c = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  T part[NP];
#pragma unroll
  for (int t = 0; t < NP; ++t) part[t] = T(0);
  if (c < g.cells) {
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
    const bool interior = i >= R && i < g.d0 - R && j >= R && j < g.d1 - R &&
                          (g.dim == 2 || (k >= R && k < g.d2 - R));
    T acc = T(0);
    static_for<NT>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
      acc = fma(p.coef[t], ldz(p.lam_next, g, i - di, j - dj, k - dk), acc);
    });
    const long long o = cell_off(g, i, j, k);
    if (interior) {
      p.lam_prev[o] = acc;
      if (p.want_coef && NT <= kMaxCoefGrad) {
        const T l = p.lam_next[o];
        static_for<NP>([&](auto TI) {
          constexpr int t = decltype(TI)::value;
          constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
          part[t] = l * p.u[cell_off(g, i + di, j + dj, k + dk)] * p.inv_div;
        });
      }
    } else {
      p.halo_grad[o] += acc;
      p.lam_prev[o] = T(0);
    }
  }
  if (NT <= kMaxCoefGrad && p.want_coef) {
    // CTA sums of the NT products, added to this CTA's partial slot
    __shared__ T red[kAdjThreads / 32][NP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < NP; ++t) {
      T v = part[t];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
      if (lane == 0) red[w][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < NP) {
      double s = 0.0;
#pragma unroll
      for (int ww = 0; ww < kAdjThreads / 32; ++ww) s += (double)red[ww][threadIdx.x];
      p.coef_part[(size_t)blockIdx.x * NP + threadIdx.x] += s;
    }
  }
}

// gradient2d: linearised adjoint (2-D, radius 1)
template <class ST, typename T>
__global__ void __launch_bounds__(kAdjThreads) adjoint_gradient_kernel(const __grid_constant__ AdjParams<T, ST::kTerms> p, T eps, T num) {
  const AdjGeom &g = p.g;
  const long long c = (long long)blockIdx.x * kAdjThreads + threadIdx.x;
  const int R = g.rad;
  auto inter = [&](int a, int b) { return a >= R && a < g.d0 - R && b >= R && b < g.d1 - R; };
  // q(x) = (eps + s(x))^{-1/2} and sum_n d_n(x) for an interior cell x, in double
  auto qfac = [&](int a, int b, double &sum_d) -> double {
    const double ux = (double)p.u[cell_off(g, a, b, 0)];
    double s = 0.0;
    sum_d = 0.0;
    static_for<ST::kTerms>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      const double dn = ux - (double)p.u[cell_off(g, a + ST::kOff[t][0], b + ST::kOff[t][1], 0)];
      s = fma(dn, dn, s);
      sum_d += dn;
    });
    return 1.0 / sqrt((double)eps + s);
  };
  double pnum = 0.0;  // d u_{t+1}(y) / d num = q(y), weighted by lam_{t+1}(y)
  if (c < g.cells) {
    const int i = (int)(c / g.d1), j = (int)(c % g.d1);
    double acc = 0.0;
    const bool yin = inter(i, j);
    if (yin) {
      double sd;
      const double qy = qfac(i, j, sd);
      const double ly = (double)p.lam_next[cell_off(g, i, j, 0)];
      acc = ly * (1.0 - (double)num * qy * qy * qy * sd);
      pnum = ly * qy;
    }
    const double uy = (double)p.u[cell_off(g, i, j, 0)];
    static_for<ST::kTerms>([&](auto TI) {
      constexpr int t = decltype(TI)::value;
      const int a = i - ST::kOff[t][0], b = j - ST::kOff[t][1];  // x with x + n = y
      if (a >= 0 && a < g.d0 && b >= 0 && b < g.d1 && inter(a, b)) {
        double sd;
        const double qx = qfac(a, b, sd);
        const double dn = (double)p.u[cell_off(g, a, b, 0)] - uy;
        acc += (double)p.lam_next[cell_off(g, a, b, 0)] * (double)num * qx * qx * qx * dn;
      }
    });
    const long long o = cell_off(g, i, j, 0);
    if (yin) {
      p.lam_prev[o] = (T)acc;
    } else {
      p.halo_grad[o] += (T)acc;
      p.lam_prev[o] = T(0);
    }
  }
  if (p.want_coef) {
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
      p.coef_part[blockIdx.x] += s;
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
  size_t off_cp, off_stash, off_lam, off_hg, off_part, total;
};

Workspace workspace_of(const gbs_desc *d, const Layout &L, int C) {
  Workspace w{};
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  w.C = C;
  w.ncp = (d->timestep + C - 1) / C;
  if (w.ncp < 1) w.ncp = 1;
  w.plane_bytes = (size_t)L.plane * L.esize;
  const long long cells = (long long)L.dims[0] * L.dims[1] * L.dims[2];
  w.nblocks = (int)((cells + kAdjThreads - 1) / kAdjThreads);
  w.nt = s->kind == 1 ? 1 : std::min(s->nterms, kMaxCoefGrad);
  w.off_cp = 0;
  w.off_stash = w.off_cp + (size_t)w.ncp * w.plane_bytes;
  w.off_lam = w.off_stash + (size_t)C * w.plane_bytes;
  w.off_hg = w.off_lam + 2 * w.plane_bytes;
  w.off_part = w.off_hg + w.plane_bytes;
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
  g.cells = (long long)L.dims[0] * L.dims[1] * L.dims[2];
  return g;
}

template <class ST, typename T>
cudaError_t adjoint_step(const gbs_desc *d, const Layout &L, const void *u, const void *lam_next, void *lam_prev,
                         void *hg, double *part, bool want_coef, cudaStream_t stream) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  AdjParams<T, ST::kTerms> p;
  p.g = geom_of(L);
  p.u = static_cast<const T *>(u);
  p.lam_next = static_cast<const T *>(lam_next);
  p.lam_prev = static_cast<T *>(lam_prev);
  p.halo_grad = static_cast<T *>(hg);
  p.coef_part = part;
  const double div = d->divisor != 0.0 ? d->divisor : (double)s->divisor;
  const double dv = s->divisor ? div : 1.0;
  for (int t = 0; t < ST::kTerms; ++t) {
    double c;
    if (s->kind == 1) c = d->coef ? (d->dtype == GBS_F64 ? ((const double *)d->coef)[0] : ((const float *)d->coef)[0])
                                  : (double)s->numerator;
    else c = d->coef ? (d->dtype == GBS_F64 ? ((const double *)d->coef)[t] : ((const float *)d->coef)[t])
                     : (double)s->terms[t].coef;
    p.coef[t] = (T)(s->kind == 1 ? c : c / dv);
  }
  p.inv_div = (T)(1.0 / dv);
  p.want_coef = want_coef ? 1 : 0;
  const unsigned blocks = (unsigned)((p.g.cells + kAdjThreads - 1) / kAdjThreads);
  if constexpr (ST::kKind == KIND_GRADIENT) {
    const T eps = (T)(d->eps != 0.0 ? d->eps : (double)s->eps);
    adjoint_gradient_kernel<ST, T><<<blocks, kAdjThreads, 0, stream>>>(p, eps, p.coef[0]);
  } else {
    adjoint_linear_kernel<ST, T><<<blocks, kAdjThreads, 0, stream>>>(p);
  }
  return cudaGetLastError();
}

using AdjStepFn = cudaError_t (*)(const gbs_desc *, const Layout &, const void *, const void *, void *, void *,
                                  double *, bool, cudaStream_t);

AdjStepFn adj_step_fn(int sid, int dtype) {
  switch (sid) {
#define GBS_ADJ(id, S) \
  case id:             \
    return dtype == GBS_F64 ? &adjoint_step<S, double> : &adjoint_step<S, float>;
    GBS_FOR_EACH_STENCIL(GBS_ADJ)
#undef GBS_ADJ
    default:
      return nullptr;
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
  if (dev_coef_grad && sd->kind != 1 && sd->nterms > kMaxCoefGrad)
    return fail(GBS_ERR_UNSUPPORTED, "coefficient gradients need at most %d terms", kMaxCoefGrad);
  int *err = nullptr;
  if ((st = error_word(&err)) != GBS_OK) return st;
  const Layout L = make_layout(d);
  const Workspace w = workspace_of(d, L, checkpoint_every);
  const AdjGeom g = geom_of(L);
  char *ws = static_cast<char *>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  AdjStepFn step = adj_step_fn(d->stencil, d->dtype);
  const unsigned blocks = (unsigned)((g.cells + kAdjThreads - 1) / kAdjThreads);
  char *stash = ws + w.off_stash;
  char *lam[2] = {ws + w.off_lam, ws + w.off_lam + w.plane_bytes};
  char *hg = ws + w.off_hg;
  double *part = reinterpret_cast<double *>(ws + w.off_part);

  CK(cudaMemcpyAsync(lam[0], dev_lamT, w.plane_bytes, cudaMemcpyDeviceToDevice, s), "adjoint: lam_T");
  if (d->dtype == GBS_F64) zero_halo_kernel<double><<<blocks, kAdjThreads, 0, s>>>((double *)lam[0], g);
  else zero_halo_kernel<float><<<blocks, kAdjThreads, 0, s>>>((float *)lam[0], g);
  CK(cudaMemsetAsync(lam[1], 0, w.plane_bytes, s), "adjoint: memset");
  CK(cudaMemsetAsync(hg, 0, w.plane_bytes, s), "adjoint: memset");
  CK(cudaMemsetAsync(part, 0, (size_t)w.nblocks * w.nt * sizeof(double), s), "adjoint: memset");
  // the halo of every stash slot: the fixed boundary (never rewritten)
  for (int k = 0; k < w.C; ++k)
    CK(cudaMemcpyAsync(stash + (size_t)k * w.plane_bytes, ws + w.off_cp, w.plane_bytes, cudaMemcpyDeviceToDevice, s),
       "adjoint: stash");
  int cur = 0;
  gbs_desc d1 = *d;
  d1.timestep = 1;
  d1.bt = 1;
  d1.sl = 0;
  for (int j = w.ncp - 1; j >= 0; --j) {
    const int t0 = j * w.C;
    const int c = std::min(w.C, d->timestep - t0);
    if (c <= 0) continue;
    // recompute u_{t0} .. u_{t0+c-1} into the stash
    CK(cudaMemcpyAsync(stash, ws + w.off_cp + (size_t)j * w.plane_bytes, w.plane_bytes, cudaMemcpyDeviceToDevice, s),
       "adjoint: restore");
    for (int k = 1; k < c; ++k)
      if ((st = run_loop(&d1, L, stash + (size_t)(k - 1) * w.plane_bytes, s, err)) != GBS_OK) return st;
    // lam_{t+1} -> lam_t for t = t0+c-1 .. t0
    for (int k = c - 1; k >= 0; --k) {
      CK(step(d, L, stash + (size_t)k * w.plane_bytes, lam[cur], lam[cur ^ 1], hg, part, dev_coef_grad != nullptr, s),
         "adjoint: step");
      cur ^= 1;
    }
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
