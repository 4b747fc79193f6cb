// Instantiates the kernel family for one (stencil, element type, fp mode).
// Compiled once per combination with -DGBS_SID=<table id> -DGBS_T=<float|
// double> -DGBS_FMA=<0|1> -DGBS_PICK=<exported name>, so that the build can
// run the many units in parallel.
#include "gbs_launch.h"
#include "kernel2d.cuh"
#include "kernel3d.cuh"

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
// shared memory and tile rows of the 3-D launcher of degree b (run time b)
template <int... Bs>
constexpr size_t smem_pick(int b, std::integer_sequence<int, Bs...>) {
  size_t r = 0;
  ((r = (Bs + 1 == b) ? smem_bytes3d<S, T, Bs + 1, kFma>() : r), ...);
  return r;
}
template <int... Bs>
constexpr int jout_pick(int b, std::integer_sequence<int, Bs...>) {
  int r = 0;
  ((r = (Bs + 1 == b) ? tile_jout3d<S, T, Bs + 1, kFma>() : r), ...);
  return r;
}
template <int... Bs>
constexpr int wk_pick(int b, std::integer_sequence<int, Bs...>) {
  int r = 0;
  ((r = (Bs + 1 == b) ? tile_wk3d<S, T, Bs + 1, kFma>() : r), ...);
  return r;
}
constexpr int kMax3D = 8;  // largest 3-D degree considered
constexpr size_t smem_bytes3d_b(int b) { return smem_pick(b, std::make_integer_sequence<int, kMax3D>()); }
constexpr int jout_b(int b) { return jout_pick(b, std::make_integer_sequence<int, kMax3D>()); }
constexpr int wk_b(int b) { return wk_pick(b, std::make_integer_sequence<int, kMax3D>()); }

// Exact mode spends two FP instructions per term, so its best degree is
// lower; it keeps degrees up to 4. In 3-D a tile loses 2*(b-1)*r of its rows
// and (b-1)*r of its columns to overlap, and FP64 is compute-bound from b=1;
// FMA mode still builds every degree up to 8 whose tile fits and keeps
// outputs, so that the whole degree range can be measured.
constexpr int max_class() {
  if (!kFma && !S::kExact) return 0;  // no exact form (3d125pt: float group sums combined in double)
  if (S::kDim == 2) {
    if (sizeof(T) == 8) return 2;
    if (S::kKind == KIND_GRADIENT) return 2;  // FP64 root and quotient
    const int cap = kFma ? 8 : 4;
    if (S::kAssoc) return S::kRad == 1 ? cap : (S::kRad == 2 ? 4 : 2);
    return S::kRad <= 2 ? cap : 4;
  }
  if (S::kRad >= 3) return 1;
  int b = kFma ? kMax3D : (sizeof(T) == 8 ? 2 : (S::kRad == 1 ? 4 : 3));
  // the level rings must fit the 227 KB of shared memory a CTA may use, and
  // the tile must keep output rows and columns after the overlap
  while (b > 1 && (smem_bytes3d_b(b) > 227u * 1024u || jout_b(b) <= 0 || wk_b(b) <= 0)) --b;
  return b;
}

// block-shape variant V of the 3-D launcher of degree B, when its tile keeps
// outputs and fits in shared memory
template <int B, int V> void add_variant3(Picks &p) {
  constexpr int NW = kTileWarps[V];
  if constexpr (tile_jout3d<S, T, B, kFma, NW>() > 0 && tile_wk3d<S, T, B, kFma, NW>() > 0 &&
                smem_bytes3d<S, T, B, kFma, NW>() <= 227u * 1024u) {
    p.l3[B][V] = &launch3d<S, T, B, kFma, NW>;
    p.o3[B][V] = &occupancy3d<S, T, B, kFma, NW>;
    p.tj3[B][V] = tile_rows3d<S, T, B, kFma, NW>();
    p.jout3[B][V] = tile_jout3d<S, T, B, kFma, NW>();
    p.wk3[B][V] = tile_wk3d<S, T, B, kFma, NW>();
  }
}

template <int B> void add(Picks &p) {
  if constexpr (B <= max_class()) {
    if constexpr (S::kDim == 2) {
      p.l2[B] = &launch2d<S, T, B, kFma>;
      p.o2[B] = &occupancy2d<S, T, B, kFma>;
      if constexpr (kFma && B >= 2 && B <= kMaxStashB) p.l2s[B] = &launch2d<S, T, B, kFma, true>;
    } else {
      add_variant3<B, 0>(p);
      if constexpr (use_tile3d<S, kFma>()) add_variant3<B, 1>(p);
      p.tile3[B] = use_tile3d<S, kFma>() ? 1 : 0;
    }
    p.maxb = B;
  }
}
template <int... Bs> void add_all(Picks &p, std::integer_sequence<int, Bs...>) { (add<Bs + 1>(p), ...); }
}  // namespace

Picks GBS_PICK() {
  Picks p{};
  add_all(p, std::make_integer_sequence<int, kMaxB>());
  return p;
}
}  // namespace gbs
