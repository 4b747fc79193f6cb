// Device-side building blocks shared by the stencil kernels: bulk-async
// (TMA) copies with mbarrier completion, bounded waits, lane shuffles,
// 16-byte vector access and the two floating-point evaluation modes.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

// Register cap of a build variant (0: none). A kernel of `threads` threads
// asks for at least 65536 / (threads * cap) resident CTAs per SM, which
// limits it to about `cap` registers per thread.
#ifndef GBS_REGCAP
#define GBS_REGCAP 0
#endif
constexpr int gbs_min_ctas(int threads) {
  return GBS_REGCAP > 0 && 65536 / (threads * GBS_REGCAP) > 1 ? 65536 / (threads * GBS_REGCAP) : 1;
}

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

// Forces a lambda inline. A lambda the compiler keeps as a call (it did so
// for the row loop of a kernel variant inside the batched dispatcher) has
// its captured locals, the register windows among them, in local memory.
#define GBS_INL __attribute__((always_inline))

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
    // cached in L2 only: a batched launch rewrites grids it reads
    if constexpr (std::is_same<T, float>::value) {
      float4 f = __ldcg(reinterpret_cast<const float4 *>(p));
      t.v[0] = f.x; t.v[1] = f.y; t.v[2] = f.z; t.v[3] = f.w;
    } else {
      double2 f = __ldcg(reinterpret_cast<const double2 *>(p));
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
// 16-byte store to global memory, marked as such so that the compiler knows
// it cannot alias shared memory.
template <typename T, int V>
__device__ __forceinline__ void st_vec_global(T *p, const T (&x)[V]) {
  static_assert(sizeof(T) * V == 16, "16-byte vectors only");
  if constexpr (std::is_same<T, float>::value) __stcg(reinterpret_cast<float4 *>(p), make_float4(x[0], x[1], x[2], x[3]));
  else __stcg(reinterpret_cast<double2 *>(p), make_double2(x[0], x[1]));
}
template <typename T>
__device__ __forceinline__ void st_global(T *p, T v) { __stcg(p, v); }

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

// Window slots: with UNR the loop over pipeline steps is unrolled W times and
// the logical window position j (0 = oldest row/plane) of phase ph lives in
// slot (ph + 1 + j) % W, so the window rotates by renaming; without UNR
// (to keep the code small) slot == j and the window shifts by moves.
template <bool UNR, int W>
__host__ __device__ constexpr int wslot(int ph, int j) { return UNR ? (ph + 1 + j) % W : j; }

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

// acc + c*a in the requested mode (the first term of a sum is c*a alone)
template <typename T, bool FMA>
__device__ __forceinline__ T term_next(T acc, T c, T a) {
  using A = Arith<T>;
  if constexpr (FMA) return A::fma(c, a, acc);
  else return A::add(acc, A::mul(c, a));
}

// gradient2d.c:17-21: u + num / sqrt(eps + sum_n (u - u_n)^2), evaluated as
// C evaluates it: the differences and squares summed in T, each rounded, then
// (since `1.0f / sqrt(x)` calls the double sqrt) the root, the quotient and
// the final sum in double, rounded once to T (exact mode). Both modes form
// the sum of squares this way: the update amplifies rounding where
// neighbours agree, so even fusing the squares drifts past the 1e-5 parity
// bound within ten steps. FMA mode (FAST) replaces the double root and
// quotient, which run on the FP64 pipe at 1/64 of the FP32 rate.
template <typename T, int NN, bool FAST = false>
__device__ __forceinline__ T gradient_update(T u, const T (&nb)[NN], T eps, T num) {
  using A = Arith<T>;
  T s = eps;
#pragma unroll
  for (int n = 0; n < NN; ++n) {
    const T d = A::sub(u, nb[n]);
    s = A::add(s, A::mul(d, d));
  }
  if constexpr (FAST && std::is_same<T, float>::value) {
    // FMA mode, float, all on the FP32 pipe. q = num / sqrt(s) as an
    // unevaluated pair qh + ql: y0 = RN(1/sqrt(s)), then one Newton
    // correction 1/sqrt(s) ~ y0 (1 + e/2) whose residual e = 1 - s y0^2 is
    // formed exactly with FMA (s y0 = p + pe). u + qh + ql is then rounded
    // once through Knuth's TwoSum, like exact mode's single rounding of the
    // double sum (they differ only within ~2^-20 ulp of a rounding midpoint).
    const float y0 = __frsqrt_rn(s);
    const float p = __fmul_rn(s, y0);
    const float pe = __fmaf_rn(s, y0, -p);
    float e = __fmaf_rn(-p, y0, 1.0f);
    e = __fmaf_rn(-pe, y0, e);
    const float qh = __fmul_rn(num, y0);
    const float qe = __fmaf_rn(num, y0, -qh);
    const float ql = __fmaf_rn(qh, __fmul_rn(0.5f, e), qe);
    const float t = __fadd_rn(u, qh);
    const float bv = __fsub_rn(t, u);
    const float err = __fadd_rn(__fsub_rn(u, __fsub_rn(t, bv)), __fsub_rn(qh, bv));
    return __fadd_rn(t, __fadd_rn(err, ql));
  } else if constexpr (FAST) {
    // FMA mode, double: Newton-Raphson iteration for 1/sqrt(s),
    // y <- y + y (1 - s y^2) / 2, from a single-precision estimate (relative
    // error about 2^-22); each step squares the error, so two steps reach
    // double precision with five FP64 operations instead of a division and
    // a square root. Outside the guarded range: division and square root.
    if (s >= 1e-30 && s <= 1e30) {
      double y = (double)rsqrtf((float)s);
      double h = fma(-s * y, y, 1.0);
      y = fma(0.5 * y, h, y);
      h = fma(-s * y, y, 1.0);
      y = fma(0.5 * y, h, y);
      return u + num * y;
    }
    return u + num / sqrt(s);
  } else {
    const double q = __ddiv_rn((double)num, __dsqrt_rn((double)s));
    const double r = __dadd_rn((double)u, q);
    if constexpr (std::is_same<T, float>::value) return __double2float_rn(r);
    else return r;
  }
}

// x / d, correctly rounded, for a divisor d known in advance with y =
// RN(1/d) (y == 0 marks a divisor outside [2^-16, 2^16] (float) or
// [2^-50, 2^50] (double): IEEE division only). A reciprocal product with one
// FMA correction (Markstein's scheme) gives q1; q1 is returned only when the
// exact remainder r1 = x - q1*d shows that x/d lies strictly between the two
// rounding midpoints around q1, which makes q1 = RN(x/d). In the guarded
// range r1 is exact (the remainder of a faithful quotient is representable)
// and so are the midpoint bounds |d|*ulp/2 (power-of-two scalings); outside
// it, or when the test fails (x/d within an ulp fraction of a midpoint), the
// IEEE division is used. gbs_check_division compares this with IEEE division.
__device__ __forceinline__ float div_by(float x, float d, float y) {
  if (y != 0.0f) {
    const float q0 = __fmul_rn(x, y);
    const float r = __fmaf_rn(-q0, d, x);
    const float q1 = __fmaf_rn(r, y, q0);
    const float a = fabsf(q1);
    if (a >= 0x1p-80f && a <= 0x1p+100f) {
      const float r1 = __fmaf_rn(-q1, d, x);
      const int ab = __float_as_int(a);
      const float u = __int_as_float((ab & 0x7f800000) - (23 << 23));  // ulp(q1)
      const bool pow2 = (ab & 0x007fffff) == 0;
      // offset of x/d from q1, times |d|, signed positive away from zero
      const float om = ((d < 0.0f) != (q1 < 0.0f)) ? -r1 : r1;
      const float ad = fabsf(d);
      const float lim = (om >= 0.0f || !pow2) ? __fmul_rn(ad, __fmul_rn(u, 0.5f))
                                              : __fmul_rn(ad, __fmul_rn(u, 0.25f));
      if (fabsf(om) < lim) return q1;
    }
  }
  if (x == 0.0f && y != 0.0f) return __fmul_rn(x, y);
  return __fdiv_rn(x, d);
}
__device__ __forceinline__ double div_by(double x, double d, double y) {
  if (y != 0.0) {
    const double q0 = __dmul_rn(x, y);
    const double r = __fma_rn(-q0, d, x);
    const double q1 = __fma_rn(r, y, q0);
    const double a = fabs(q1);
    if (a >= 0x1p-900 && a <= 0x1p+900) {
      const double r1 = __fma_rn(-q1, d, x);
      const long long ab = __double_as_longlong(a);
      const double u = __longlong_as_double((ab & 0x7ff0000000000000ll) - (52ll << 52));
      const bool pow2 = (ab & 0x000fffffffffffffll) == 0;
      const double om = ((d < 0.0) != (q1 < 0.0)) ? -r1 : r1;
      const double ad = fabs(d);
      const double lim = (om >= 0.0 || !pow2) ? __dmul_rn(ad, __dmul_rn(u, 0.5))
                                              : __dmul_rn(ad, __dmul_rn(u, 0.25));
      if (fabs(om) < lim) return q1;
    }
  }
  if (x == 0.0 && y != 0.0) return __dmul_rn(x, y);
  return __ddiv_rn(x, d);
}

// x / d without the remainder test, for divisors for which the one-correction
// quotient is exact on every input: the engine whitelists such divisors only
// when the exhaustive float self-test (gbs_check_division with check=0)
// proves it for that divisor, as it does for the artifact's 118 and 159.
__device__ __forceinline__ float div_by_fast(float x, float d, float y) {
  const float q0 = __fmul_rn(x, y);
  const float r = __fmaf_rn(-q0, d, x);
  const float q1 = __fmaf_rn(r, y, q0);
  const float a = fabsf(q1);
  if (a >= 0x1p-125f && a <= 0x1p+126f) return q1;
  if (x == 0.0f) return __fmul_rn(x, y);
  return __fdiv_rn(x, d);
}

// RN(1/d) for div_by, or 0 when d is outside the range div_by's test covers.
template <typename T> inline T div_reciprocal(double d) {
  const double lo = sizeof(T) == 4 ? 0x1p-16 : 0x1p-50, hi = sizeof(T) == 4 ? 0x1p+16 : 0x1p+50;
  const double ad = d < 0 ? -d : d;
  if (!(ad >= lo && ad <= hi)) return (T)0;
  volatile T one = (T)1;
  return one / (T)d;
}

}  // namespace gbs
