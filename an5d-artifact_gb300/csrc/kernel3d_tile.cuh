// 3-D temporally-blocked stencil kernel, FMA mode: tensor-map (TMA) tiles.
//
// Replaces the AN5D-generated 3-D kernels (e.g.
// compiled/float/box3d1r-32x32-3-128_kernel.cu:4,284,509) for the FMA
// evaluation mode and computes what the artifact's 3-D scop loops compute
// (star3d2r.c:15-29, box3d1r.c:15-50, ...): B Jacobi steps of
// A[(t+1)%2][i][j][k] = f(A[t%2][neighbourhood]) on the interior, the halo
// held fixed.
//
// Work decomposition. A CTA owns a tile of TJ = NW*H rows (j) by ROW = 32*V
// columns (k) and streams the outermost axis i over a block of sl output
// planes. Warp w computes rows w*H .. w*H+H-1 of the tile; lane l computes
// columns l*V .. l*V+V-1 (V = 16 bytes / element size). Every level
// computes the whole TJ x ROW tile, so after B levels the valid outputs are
// the centre (TJ - 2(B-1)r) x (ROW - 2(B-1)r, rounded to whole vectors): at
// B = 1 every computed cell is an output and nothing is recomputed.
//
// Level-0 planes arrive by one tensor-map copy per plane
// (cp.async.bulk.tensor.3d, issued by one thread): a box of TJ + 2r rows by
// ROW + 2*PADE columns (the tile plus its halo, PADE = r rounded up to a
// vector), completed on an mbarrier, into a ring of NS stages. Rows or
// columns outside the grid arrive as zeros; they feed only cells that are
// outside the valid region. Fused levels are skewed by one step: at step s
// level 1 consumes level-0 plane s, level l+1 the plane level l wrote at
// step s-1, and one __syncthreads per step publishes every level's output
// plane. Levels 1..B-1 write their planes to shared-memory rings of the same
// row layout; level B stores its valid cells to HBM. In-row neighbours come
// from the neighbouring 16-byte vectors of the same shared-memory row; the
// i-direction lives in registers as the partial sums of the 2r+1 output
// planes in flight, to which each arriving plane adds its terms.
// Intermediate levels give their halo cells the fixed halo value, read from
// HBM one step ahead.
//
// stencil3d_stream_kernel is the degree-1 form for double: one producer warp
// more issues the tensor-map copies into the NS stages, each stage guarded by
// a "full" mbarrier (the copy) and an "empty" one (one arrival per consumer
// warp), so consumer warps run without a CTA barrier per plane; the FP64 pipe
// bounds it, and a barrier left that pipe idle while the last warps of a
// plane drained.
#pragma once
#include <cuda.h>

#include "gbs_device.cuh"
#include "gbs_launch.h"
#include "stencil_table.cuh"

namespace gbs {

// Kernel parameters: the tensor map of the source plane plus the plain ones.
template <typename T, int NT> struct Params3T {
  CUtensorMap tmap;      // source plane: {pitch, d1, d0} elements, box {BX, BY, 1}
  const T *src;
  T *dst;
  int *err;
  long long pitch;       // elements per padded k-row
  int d0, d1, d2;        // dimsize per axis
  int shift;             // column k at element shift + k
  int jout, wk;          // valid rows / columns per tile
  int ntk, ntj, nblocks, sl;
  T coef[NT];
};

// 3-D tensor copy of one box into shared memory, completion on `bar`. The
// innermost coordinate x must be a multiple of 16 bytes / element size.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

template <class ST, typename T, int B, int NW, int H, int NSTAGE>
struct Tile3 {
  static constexpr int R = ST::kRad;
  static constexpr int W = 2 * R + 1;
  static constexpr int V = 16 / sizeof(T);
  static constexpr int ROW = 32 * V;                        // computed columns
  static constexpr int PADV = (R + V - 1) / V;              // halo vectors per side
  static constexpr int PADE = PADV * V;                     // halo elements per side
  static constexpr int BX = ROW + 2 * PADE;                 // elements per shared row
  static constexpr int TJ = NW * H;                         // computed rows
  static constexpr int BY = TJ + 2 * R;                     // rows per shared plane
  static constexpr int NS = NSTAGE;                         // level-0 stages
  static constexpr int DEP = 2;                             // stages per intermediate level
  static constexpr size_t BOX_BYTES = (size_t)BX * BY * sizeof(T);
  static constexpr size_t PLANE = (BOX_BYTES + 127) / 128 * 128;
  static constexpr size_t bytes() { return PLANE * (NS + (size_t)(B - 1) * DEP) + NS * sizeof(uint64_t); }
  // first valid column of the window, a whole number of vectors
  static constexpr int OFF = ((B - 1) * R + V - 1) / V * V;
  // valid columns per window
  static constexpr int WK = (ROW - (B - 1) * R - OFF) / V * V;
  static constexpr int JOUT = TJ - 2 * (B - 1) * R;
  static constexpr bool UNR = W * ST::kTerms * H * V <= 4000;
  static constexpr int NPH = UNR ? W : 1;
  static constexpr bool valid() { return BX <= 256 && BY <= 256 && WK > 0 && JOUT > 0; }
};

// Which elements x (relative to a lane's element 0, x in [-R, V+R)) of the
// arriving plane's row RHO (relative to a warp's first row) some term reads
// for one of the warp's H output rows.
template <class ST, int RHO, int H, int V> struct RowNeed {
  static constexpr bool used() {
    for (int t = 0; t < ST::kTerms; ++t) {
      const int hh = RHO - ST::kOff[t][1];
      if (hh >= 0 && hh < H) return true;
    }
    return false;
  }
  static constexpr bool at(int x) {
    for (int t = 0; t < ST::kTerms; ++t) {
      const int hh = RHO - ST::kOff[t][1];
      const int e = x - ST::kOff[t][2];
      if (hh >= 0 && hh < H && e >= 0 && e < V) return true;
    }
    return false;
  }
};

// ext[R + x] = element x of the lane's part of a shared row (x in [-R, V+R)),
// for the x that Need::at selects; rowp points at the lane's element 0. The
// elements come from the lane's own 16-byte vector and from the neighbouring
// vectors of the same row (the row carries PADE halo elements at each end).
template <typename T, int V, int R, class Need>
__device__ __forceinline__ void load_ext(T (&ext)[V + 2 * R], const T *rowp) {
  constexpr int PADV = (R + V - 1) / V;
  static_for<2 * PADV + 1>([&](auto VI) {
    constexpr int vi = decltype(VI)::value - PADV;  // vector offset from the lane's own
    constexpr bool any = [] {
      for (int e = 0; e < V; ++e) {
        const int x = vi * V + e;
        if (x >= -R && x < V + R && Need::at(x)) return true;
      }
      return false;
    }();
    if constexpr (any) {
      T v[V];
      ld_vec<T, V>(v, rowp + vi * V);
      static_for<V>([&](auto EI) {
        constexpr int x = vi * V + decltype(EI)::value;
        if constexpr (x >= -R && x < V + R && Need::at(x)) ext[R + x] = v[decltype(EI)::value];
      });
    }
  });
}

template <class ST, typename T, int B, int NW, int H, int NSTAGE>
__global__ void __launch_bounds__(NW * 32, gbs_min_ctas(NW * 32))
    stencil3d_tile_kernel(const __grid_constant__ Params3T<T, ST::kTerms> p) {
  using G = Tile3<ST, T, B, NW, H, NSTAGE>;
  static_assert(G::valid(), "a tensor-map box is at most 256 elements per axis, and the tile needs outputs");
  constexpr int V = G::V, R = G::R, W = G::W, ROW = G::ROW, BX = G::BX, PADE = G::PADE;
  constexpr int NS = G::NS, DEP = G::DEP, NPH = G::NPH;
  constexpr size_t PLANE = G::PLANE;
  constexpr bool UNR = G::UNR;
  using A = Arith<T>;
  using OR = Order3<ST, true>;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *ring0 = smem_raw;
  unsigned char *rings = smem_raw + NS * PLANE;
  uint64_t *bars = reinterpret_cast<uint64_t *>(rings + (size_t)(B - 1) * DEP * PLANE);

  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  int bid = blockIdx.x;
  const int tk = bid % p.ntk;
  bid /= p.ntk;
  const int tj = bid % p.ntj;
  const int blk = bid / p.ntj;

  // columns k: outputs [cs, ce); the window's column 0 is grid column ws - shift
  const int cs = R + tk * p.wk;
  const int ce = min(cs + p.wk, p.d2 - R);
  const int ws = p.shift + cs - G::OFF;  // element index, a multiple of V
  const int col0 = ws - p.shift + lane * V;
  const bool kedge = (ws - p.shift < R) || (ws - p.shift + ROW > p.d2 - R);
  const bool store_all = (col0 >= cs && col0 + V <= ce);
  // rows j: outputs [js, je); the tile's computed rows start at jt
  const int js = R + tj * p.jout;
  const int je = min(js + p.jout, p.d1 - R);
  const int jt = js - (B - 1) * R;
  const int j0 = jt + w * H;  // this warp's first row
  // planes i
  const int i0 = R + blk * p.sl;
  const int i1 = min(i0 + p.sl, p.d0 - R);
  const int pstart = max(0, i0 - B * R);
  const int pend = min(p.d0, i1 + B * R);
  const int slast = i1 - 1 + (B - 1) + B * R;
  const long long plane_stride = (long long)p.d1 * p.pitch;
  bool warp_jhalo = false;
#pragma unroll
  for (int h = 0; h < H; ++h) warp_jhalo |= (j0 + h < R || j0 + h >= p.d1 - R);

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  // thread 0: the whole box of level-0 plane `plane` into its stage
  int issued = pstart;  // thread 0: one past the last plane issued
  auto issue = [&](int plane) GBS_INL {
    const int st = (plane - pstart) % NS;
    mbar_arrive_expect_tx(&bars[st], (unsigned)G::BOX_BYTES);
    tma_load_3d(ring0 + (size_t)st * PLANE, &p.tmap, ws - PADE, jt - R, plane, &bars[st]);
    issued = plane + 1;
  };
  if (threadIdx.x == 0)
    for (int pl = pstart; pl < pend && pl < pstart + NS; ++pl) issue(pl);

  T acc[B][W][H][V];
  static_for<B>([&](auto LI) {
    static_for<W>([&](auto AI) {
      static_for<H>([&](auto HI) {
        static_for<V>([&](auto EI) {
          acc[decltype(LI)::value][decltype(AI)::value][decltype(HI)::value][decltype(EI)::value] = T(0);
        });
      });
    });
  });
  // fixed-halo values of the next step's output plane, per intermediate level
  constexpr int BC = B > 1 ? B - 1 : 1;
  T cr[BC][H][V];
  bool crv[BC];
#pragma unroll
  for (int l = 0; l < BC; ++l) crv[l] = false;
  // lanes whose window elements lie inside the padded row (the leftmost
  // window of a high degree starts left of the row)
  const bool lane_in_row = (ws + lane * V >= 0) && (ws + lane * V + V <= p.pitch);

  bool ok = true;
  int waited = pstart;
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
  // loads the fixed halo values level l needs at step s (output plane q)
  auto fetch_carry = [&](auto LI, int s) GBS_INL {
    constexpr int l = decltype(LI)::value;
    const int q = s - l * (R + 1) - R;
    const bool need = (q >= 0 && q < p.d0) && (q < R || q >= p.d0 - R || warp_jhalo || kedge);
    crv[l] = need;
    if (need && lane_in_row) {
      static_for<H>([&](auto HI) {
        constexpr int h = decltype(HI)::value;
        const int jr = j0 + h;
        if (jr >= 0 && jr < p.d1)
          ld_vec_global<T, V>(cr[l][h], p.src + q * plane_stride + (long long)jr * p.pitch + ws + lane * V);
      });
    }
  };

  auto step = [&](auto PHI, int s) GBS_INL {
    constexpr int ph = decltype(PHI)::value;
    if (threadIdx.x == 0 && s > pstart) {
      const int pf = s - 1 + NS;  // the stage of plane s-1 is free since the last barrier
      if (pf < pend) issue(pf);
    }
    static_for<B>([&](auto LI) {
      constexpr int l = decltype(LI)::value;
      const int m = s - l * (R + 1);
      const int q = m - R;
      const T *in_m;
      if constexpr (l == 0)
        in_m = reinterpret_cast<const T *>(ring0 + (size_t)((m - pstart) % NS) * PLANE);
      else
        in_m = reinterpret_cast<const T *>(rings + (size_t)(l - 1) * DEP * PLANE +
                                           (size_t)(((s - 1) % DEP + DEP) % DEP) * PLANE);
      // rows rho = -R .. H+R-1 relative to the warp's first row
      static_for<H + 2 * R>([&](auto RI) {
        constexpr int rho = decltype(RI)::value - R;
        using Need = RowNeed<ST, rho, H, V>;
        if constexpr (Need::used()) {
          T ext[V + 2 * R];
          load_ext<T, V, R, Need>(ext, in_m + (size_t)(w * H + R + rho) * BX + PADE + lane * V);
          static_for<ST::kTerms>([&](auto UI) {
            constexpr int u = decltype(UI)::value;
            constexpr int t = OR::idx.v[u];
            constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
            constexpr int h = rho - dj;
            if constexpr (h >= 0 && h < H) {
              constexpr int slot = wslot<UNR, W>(ph, R - di);
              static_for<V>([&](auto EI) {
                constexpr int e = decltype(EI)::value;
                const T a = ext[R + e + dk];
                if constexpr (u == OR::init_pos()) acc[l][slot][h][e] = A::mul(p.coef[t], a);
                else acc[l][slot][h][e] = A::fma(p.coef[t], a, acc[l][slot][h][e]);
              });
            }
          });
        }
      });
      constexpr int oslot = wslot<UNR, W>(ph, 0);
      if constexpr (l + 1 < B) {
        // intermediate level: fixed values into its halo cells, publish the plane
        T *out = reinterpret_cast<T *>(rings + (size_t)l * DEP * PLANE + (size_t)(s % DEP) * PLANE);
        static_for<H>([&](auto HI) {
          constexpr int h = decltype(HI)::value;
          T y[V];
          static_for<V>([&](auto EI) { y[decltype(EI)::value] = acc[l][oslot][h][decltype(EI)::value]; });
          if (crv[l]) {
            const int jr = j0 + h;
            const bool rowhalo = (q < R || q >= p.d0 - R || jr < R || jr >= p.d1 - R);
            static_for<V>([&](auto EI) {
              constexpr int e = decltype(EI)::value;
              if (rowhalo || col0 + e < R || col0 + e >= p.d2 - R) y[e] = cr[l][h][e];
            });
          }
          st_vec<T, V>(out + (size_t)(w * H + R + h) * BX + PADE + lane * V, y);
        });
        fetch_carry(LI, s + 1);
      } else {
        if (q >= i0 && q < i1) {
          static_for<H>([&](auto HI) {
            constexpr int h = decltype(HI)::value;
            const int jr = j0 + h;
            if (jr >= js && jr < je) {
              T *d = p.dst + q * plane_stride + (long long)jr * p.pitch + ws + lane * V;
              if (store_all) {
                st_vec_global<T, V>(d, acc[l][oslot][h]);
              } else {
                static_for<V>([&](auto EI) {
                  constexpr int e = decltype(EI)::value;
                  if (col0 + e >= cs && col0 + e < ce) st_global(d + e, acc[l][oslot][h][e]);
                });
              }
            }
          });
        }
      }
      if constexpr (!UNR) {
        static_for<2 * R>([&](auto AI) {
          constexpr int a = decltype(AI)::value;
          static_for<H>([&](auto HI) {
            static_for<V>([&](auto EI) {
              acc[l][a][decltype(HI)::value][decltype(EI)::value] =
                  acc[l][a + 1][decltype(HI)::value][decltype(EI)::value];
            });
          });
        });
      }
    });
    ok = wait_plane(s + 1);
  };

  if constexpr (B > 1) {
    static_for<B - 1>([&](auto LI) { fetch_carry(LI, pstart); });
  }
  ok = wait_plane(pstart);
#pragma unroll 1
  for (int sb = pstart; ok && sb <= slast; sb += NPH) {
    static_for<NPH>([&](auto PHI) {
      const int s = sb + decltype(PHI)::value;
      if (!ok || s > slast) return;
      step(PHI, s);
    });
  }

  if (!ok && threadIdx.x == 0) {
    // Timed out: wait (bounded) for the copies still in flight before the
    // CTA exits and its shared memory is reassigned.
    for (int pl = waited; pl < issued; ++pl) {
      const int n = pl - pstart;
      if (!mbar_wait(&bars[n % NS], (unsigned)(n / NS) & 1u, p.err, ERR_DRAIN_TIMEOUT)) break;
    }
  }
}

// ---------------------------------------------------------------------------
// Degree 1: the same tile, as a decoupled pipeline. With no intermediate
// level, the only thing the tile kernel's per-plane __syncthreads protects
// is the reuse of a ring stage, and that barrier makes every warp wait for
// the slowest before the next plane (on the FP64 pipe, whose throughput is
// the bound, the pipe then idles while the last warps drain). Here one extra
// warp is the producer: for each plane it waits (bounded) on the stage's
// "empty" mbarrier, on which every consumer warp arrives once it has read
// the plane, then issues the tensor copy whose bytes complete the stage's
// "full" mbarrier. Consumer warps wait (bounded) on "full" only, so they run
// up to NS-1 planes apart and the pipe always has work. Every wait is
// bounded; a consumer that gives up stops, and the producer, which then
// finds its stage never released, gives up too and waits (bounded) for its
// copies in flight before the CTA exits.
// ---------------------------------------------------------------------------
template <class ST, typename T, int NW, int H, int NSTAGE>
struct Stream3 {
  using G = Tile3<ST, T, 1, NW, H, NSTAGE>;
  static constexpr size_t bytes() { return G::PLANE * G::NS + 2 * G::NS * sizeof(uint64_t); }
};

template <class ST, typename T, int NW, int H, int NSTAGE>
__global__ void __launch_bounds__((NW + 1) * 32, gbs_min_ctas((NW + 1) * 32))
    stencil3d_stream_kernel(const __grid_constant__ Params3T<T, ST::kTerms> p) {
  using G = Tile3<ST, T, 1, NW, H, NSTAGE>;
  static_assert(G::valid(), "a tensor-map box is at most 256 elements per axis, and the tile needs outputs");
  constexpr int V = G::V, R = G::R, W = G::W, BX = G::BX, PADE = G::PADE;
  constexpr int NS = G::NS, NPH = G::NPH;
  constexpr size_t PLANE = G::PLANE;
  constexpr bool UNR = G::UNR;
  using OR = Order3<ST, true>;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *ring0 = smem_raw;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + NS * PLANE);
  uint64_t *empty = full + NS;

  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  int bid = blockIdx.x;
  const int tk = bid % p.ntk;
  bid /= p.ntk;
  const int tj = bid % p.ntj;
  const int blk = bid / p.ntj;

  const int cs = R + tk * p.wk;
  const int ce = min(cs + p.wk, p.d2 - R);
  const int ws = p.shift + cs;  // element index of the window's column 0 (a multiple of V)
  const int col0 = ws - p.shift + lane * V;
  const bool store_all = (col0 >= cs && col0 + V <= ce);
  const int js = R + tj * p.jout;
  const int je = min(js + p.jout, p.d1 - R);
  const int j0 = js + w * H;
  const int i0 = R + blk * p.sl;
  const int i1 = min(i0 + p.sl, p.d0 - R);
  const int pstart = max(0, i0 - R);
  const int pend = min(p.d0, i1 + R);
  const int slast = i1 - 1 + R;
  const long long plane_stride = (long long)p.d1 * p.pitch;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NW);
    }
    fence_mbar_init();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  if (w == NW) {
    // producer warp: lane 0 issues every plane of the block
    if (lane == 0) {
      int issued = pstart;
      for (int pl = pstart; pl < pend; ++pl) {
        const int n = pl - pstart;
        const int st = n % NS;
        // the stage's previous plane (n - NS) must have been read by every consumer
        if (n >= NS && !mbar_wait(&empty[st], (unsigned)((n / NS) - 1) & 1u, p.err, ERR_WAIT_TIMEOUT)) break;
        mbar_arrive_expect_tx(&full[st], (unsigned)G::BOX_BYTES);
        tma_load_3d(ring0 + (size_t)st * PLANE, &p.tmap, ws - PADE, js - R, pl, &full[st]);
        issued = pl + 1;
      }
      // the last copy of each stage has landed before the CTA may exit
      for (int n = max(0, issued - pstart - NS); n < issued - pstart; ++n)
        if (!mbar_wait(&full[n % NS], (unsigned)(n / NS) & 1u, p.err, ERR_DRAIN_TIMEOUT)) break;
    }
    return;
  }

  T acc[W][H][V];
  static_for<W>([&](auto AI) {
    static_for<H>([&](auto HI) {
      static_for<V>([&](auto EI) { acc[decltype(AI)::value][decltype(HI)::value][decltype(EI)::value] = T(0); });
    });
  });

  bool ok = true;
  auto step = [&](auto PHI, int s) GBS_INL {
    constexpr int ph = decltype(PHI)::value;
    const int n = s - pstart;
    const int st = n % NS;
    if (s < pend) {
      const bool got = mbar_wait(&full[st], (unsigned)(n / NS) & 1u, nullptr, 0);
      if (!__all_sync(0xffffffffu, got)) {
        if (lane == 0) atomicOr(p.err, ERR_WAIT_TIMEOUT);
        ok = false;
        return;
      }
    }
    // past the block's last plane the stage holds an older plane: its terms
    // reach only outputs that are not stored
    const T *in_m = reinterpret_cast<const T *>(ring0 + (size_t)st * PLANE);
    const int q = s - R;
    static_for<H + 2 * R>([&](auto RI) {
      constexpr int rho = decltype(RI)::value - R;
      using Need = RowNeed<ST, rho, H, V>;
      if constexpr (Need::used()) {
        T ext[V + 2 * R];
        load_ext<T, V, R, Need>(ext, in_m + (size_t)(w * H + R + rho) * BX + PADE + lane * V);
        static_for<ST::kTerms>([&](auto UI) {
          constexpr int u = decltype(UI)::value;
          constexpr int t = OR::idx.v[u];
          constexpr int di = ST::kOff[t][0], dj = ST::kOff[t][1], dk = ST::kOff[t][2];
          constexpr int h = rho - dj;
          if constexpr (h >= 0 && h < H) {
            constexpr int slot = wslot<UNR, W>(ph, R - di);
            static_for<V>([&](auto EI) {
              constexpr int e = decltype(EI)::value;
              const T a = ext[R + e + dk];
              if constexpr (u == OR::init_pos()) acc[slot][h][e] = Arith<T>::mul(p.coef[t], a);
              else acc[slot][h][e] = Arith<T>::fma(p.coef[t], a, acc[slot][h][e]);
            });
          }
        });
      }
    });
    // every lane of the warp has read the plane: release the stage
    __syncwarp();
    if (s < pend && lane == 0) mbar_arrive(&empty[st]);
    constexpr int oslot = wslot<UNR, W>(ph, 0);
    if (q >= i0 && q < i1) {
      static_for<H>([&](auto HI) {
        constexpr int h = decltype(HI)::value;
        const int jr = j0 + h;
        if (jr >= js && jr < je) {
          T *d = p.dst + q * plane_stride + (long long)jr * p.pitch + ws + lane * V;
          if (store_all) {
            st_vec_global<T, V>(d, acc[oslot][h]);
          } else {
            static_for<V>([&](auto EI) {
              constexpr int e = decltype(EI)::value;
              if (col0 + e >= cs && col0 + e < ce) st_global(d + e, acc[oslot][h][e]);
            });
          }
        }
      });
    }
    if constexpr (!UNR) {
      static_for<2 * R>([&](auto AI) {
        constexpr int a = decltype(AI)::value;
        static_for<H>([&](auto HI) {
          static_for<V>([&](auto EI) {
            acc[a][decltype(HI)::value][decltype(EI)::value] = acc[a + 1][decltype(HI)::value][decltype(EI)::value];
          });
        });
      });
    }
  };

#pragma unroll 1
  for (int sb = pstart; ok && sb <= slast; sb += NPH) {
    static_for<NPH>([&](auto PHI) {
      const int s = sb + decltype(PHI)::value;
      if (!ok || s > slast) return;
      step(PHI, s);
    });
  }
}

}  // namespace gbs
