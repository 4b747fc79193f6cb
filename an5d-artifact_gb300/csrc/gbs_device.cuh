// Device-side building blocks shared by the stencil kernels: bulk-async
// (TMA) copies with mbarrier completion, bounded waits, lane shuffles,
// 16-byte vector access and the two floating-point evaluation modes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

namespace gbs {

// Error bits a kernel ORs into the launch's error word.
enum : int {
  ERR_WAIT_TIMEOUT = 1,   // an mbarrier wait exceeded its time limit
  ERR_DRAIN_TIMEOUT = 2,  // draining in-flight copies after a timeout gave up
  ERR_DEP_TIMEOUT = 4,    // a dependency wait (batched scheduler) gave up
};

// Wall-clock limit of every spin-wait, in nanoseconds (about one second).
constexpr unsigned long long kWaitLimitNs = 1000ull * 1000ull * 1000ull;

template <int N> using IC = std::integral_constant<int, N>;

// Compile-time loop: f(IC<0>), ..., f(IC<N-1>).
template <int N, class F, int... Is>
__device__ __forceinline__ void static_for_impl(F &&f, std::integer_sequence<int, Is...>) {
  (f(IC<Is>()), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
  static_for_impl<N>(std::forward<F>(f), std::make_integer_sequence<int, N>());
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- mbarrier ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of `bar` to complete, for at most kWaitLimitNs.
// Returns false (and sets `code` in *err) when the limit is reached.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, int *err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (true) {
#pragma unroll 1
    for (int i = 0; i < 64; ++i)
      if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitLimitNs) {
      if (err) atomicOr(err, code);
      return false;
    }
  }
}

// ---- bulk async copies (TMA, non-tensor form) --------------------------------
// global -> shared, completion counted in bytes on `bar`. Both addresses must
// be 16-byte aligned and `bytes` a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---- tensor-map (TMA tiled) loads -------------------------------------------
__device__ __forceinline__ void tma_load_4d(void *dst, const void *tmap, int c0, int c1, int c2,
                                            int c3, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const void *tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

// ---- vectors of V elements (16 bytes) ----------------------------------------
template <typename T, int V> struct alignas(16) Vec { T v[V]; };

template <typename T, int V>
__device__ __forceinline__ void ld_vec(T (&x)[V], const T *p) {
  const Vec<T, V> t = *reinterpret_cast<const Vec<T, V> *>(p);
#pragma unroll
  for (int e = 0; e < V; ++e) x[e] = t.v[e];
}
template <typename T, int V>
__device__ __forceinline__ void ld_vec_global(T (&x)[V], const T *p) {
  Vec<T, V> t;
  if constexpr (sizeof(T) * V == 16) {
    if constexpr (std::is_same<T, float>::value) {
      float4 f = __ldg(reinterpret_cast<const float4 *>(p));
      t.v[0] = f.x; t.v[1] = f.y; t.v[2] = f.z; t.v[3] = f.w;
    } else {
      double2 f = __ldg(reinterpret_cast<const double2 *>(p));
      t.v[0] = f.x; t.v[1] = f.y;
    }
  } else {
    t = *reinterpret_cast<const Vec<T, V> *>(p);
  }
#pragma unroll
  for (int e = 0; e < V; ++e) x[e] = t.v[e];
}
template <typename T, int V>
__device__ __forceinline__ void st_vec(T *p, const T (&x)[V]) {
  Vec<T, V> t;
#pragma unroll
  for (int e = 0; e < V; ++e) t.v[e] = x[e];
  *reinterpret_cast<Vec<T, V> *>(p) = t;
}

// ---- lane shuffles -----------------------------------------------------------
template <typename T>
__device__ __forceinline__ T shfl_up(T v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }

// Value at element x (x in [-R, V+R)) of a row whose lane-local part is
// row[0..V): x < 0 or x >= V come from the lanes to the left/right.
template <int V, int X, typename T>
__device__ __forceinline__ T row_elem(const T (&row)[V]) {
  if constexpr (X >= 0 && X < V) {
    return row[X];
  } else if constexpr (X < 0) {
    constexpr int dl = (-X + V - 1) / V;  // lanes to the left
    constexpr int m = X + dl * V;         // element index in that lane
    return shfl_up(row[m], dl);
  } else {
    constexpr int dl = X / V;             // lanes to the right
    constexpr int m = X - dl * V;
    return shfl_down(row[m], dl);
  }
}

// ---- arithmetic modes ---------------------------------------------------------
// Exact mode: products and sums rounded separately (never contracted).
// FMA mode: acc + c*a as one fused operation.
template <typename T> struct Arith;
template <> struct Arith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct Arith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

// acc = first ? c*a : acc + c*a   in the requested mode
template <typename T, bool FMA>
__device__ __forceinline__ T term(bool first, T acc, T c, T a) {
  using A = Arith<T>;
  if (first) return A::mul(c, a);
  if constexpr (FMA) return A::fma(c, a, acc);
  else return A::add(acc, A::mul(c, a));
}
template <typename T, bool FMA>
__device__ __forceinline__ T term_first(T c, T a) { return Arith<T>::mul(c, a); }
template <typename T, bool FMA>
__device__ __forceinline__ T term_next(T acc, T c, T a) {
  using A = Arith<T>;
  if constexpr (FMA) return A::fma(c, a, acc);
  else return A::add(acc, A::mul(c, a));
}

// gradient2d.c:17-21: u + num / sqrt(eps + sum_n (u - u_n)^2). In exact mode
// the squares are summed in T and, as C evaluates `1.0f / sqrt(x)`, the root,
// the quotient and the final sum are taken in double before rounding to T.
// In FMA mode the squares are fused and a T-precision IEEE root and quotient
// are used.
template <typename T, bool FMA, int NN>
__device__ __forceinline__ T gradient_update(T u, const T (&nb)[NN], T eps, T num) {
  using A = Arith<T>;
  T s = eps;
#pragma unroll
  for (int n = 0; n < NN; ++n) {
    const T d = A::sub(u, nb[n]);
    if constexpr (FMA) s = A::fma(d, d, s);
    else s = A::add(s, A::mul(d, d));
  }
  if constexpr (!FMA || std::is_same<T, double>::value) {
    const double q = __ddiv_rn((double)num, __dsqrt_rn((double)s));
    const double r = __dadd_rn((double)u, q);
    if constexpr (std::is_same<T, float>::value) return __double2float_rn(r);
    else return r;
  } else {
    return A::add(u, A::div(num, __fsqrt_rn(s)));
  }
}

}  // namespace gbs
