// Instantiates the kernel family for one (stencil, element type, fp mode).
// Compiled once per combination with -DGBS_SID=<table id> -DGBS_T=<float|
// double> -DGBS_FMA=<0|1> -DGBS_PICK=<exported name>, so that the build can
// run the many units in parallel.
#include "gbs_launch.h"
#include "kernel2d.cuh"

#if !defined(GBS_SID) || !defined(GBS_T) || !defined(GBS_FMA) || !defined(GBS_PICK)
#error "GBS_SID, GBS_T, GBS_FMA and GBS_PICK must be defined"
#endif

namespace gbs {
namespace {
using S = typename StencilById<GBS_SID>::type;
using T = GBS_T;
constexpr bool kFma = GBS_FMA != 0;

// Fused-degree classes worth instantiating. A b-level strip loses 2*b*r of
// its 32*V columns to overlap, and stencils with many terms are FP-bound
// before temporal blocking pays; FP64 on GB300 is FP-bound already at b=1.
constexpr int max_class() {
  if (S::kDim == 2) {
    if (sizeof(T) == 8) return 2;
    if (S::kKind == KIND_GRADIENT) return kFma ? 8 : 2;
    if (S::kAssoc) return S::kRad == 1 ? 8 : (S::kRad == 2 ? 4 : 2);
    return S::kRad <= 2 ? 8 : 4;
  }
  return 1;
}

template <int B> void add2(Picks &p) {
  if constexpr (S::kDim == 2 && B <= max_class()) {
    p.cls[p.ncls] = B;
    p.l2[p.ncls] = &launch2d<S, T, B, kFma>;
    p.l3[p.ncls] = nullptr;
    p.smem3[p.ncls] = 0;
    ++p.ncls;
  }
}
}  // namespace

Picks GBS_PICK() {
  Picks p{};
  add2<1>(p);
  add2<2>(p);
  add2<4>(p);
  add2<8>(p);
  return p;
}
}  // namespace gbs
