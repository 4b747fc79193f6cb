// Autotuner: chooses (bt, sl, bs1) per (stencil, dtype, fp mode, grid size
// class); bs1 is the 3-D tile's rows (the block shape), 0 in 2-D.
//
// Replaces the artifact's offline performance model (Model_V100.xlsm, sheets
// Formula / Macro, whose top configuration per stencil is listed in
// compiled/v100_float.csv:1-105 as bS1,bS2,bT,sl). That model takes
// max(compute, global-memory, shared-memory time) per candidate from peak
// rates. Here a model of the same kind ranks the candidates:
//   per cell update: max(2*S / (bt * B_hbm), redundancy(bt, sl) * fpp / P_fp)
//   plus one launch gap per bt steps,
// with B_hbm from the device's memory clock and bus width and P_fp measured
// by gbs_measure_fp_peak. The model only prunes: every surviving candidate is
// then timed on the device (CUDA events, a scratch grid of the same size) and
// the fastest one is recorded in the engine's tuning table. The time loop
// (gbs_run, gbs_run_device, gbs_plan) resolves bt = 0 / sl = 0 through that
// table; sizes without an entry use the nearest size class of the same
// stencil, dtype and mode, else the engine's fixed rule.
//
// Table file: one entry per line, '#' starts a comment:
//   <stencil> <f32|f64> <exact|fma> <size class> <bt> <sl> [<bs1>] <ms per step>
// where the size class is floor(log2(interior cells)) and bs1 (3-D tile
// rows; 0 or absent: the launcher's default shape) is optional.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "engine_internal.h"

namespace gbs {
namespace {

struct Entry {
  int sid, dtype, fma, cls, bt, sl;
  double ms;
  int bs1;
};

std::mutex g_mu;
std::vector<Entry> g_table;
bool g_env_loaded = false;

int size_class(const gbs_desc *d) {
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  double cells = 1.0;
  for (int a = 0; a < s->dim; ++a) cells *= (double)d->n[a];
  return cells >= 1.0 ? (int)std::floor(std::log2(cells)) : 0;
}

gbs_status load_locked(const char *path) {
  FILE *f = std::fopen(path, "r");
  if (!f) return fail(GBS_ERR_INVALID, "cannot open tuning table %s", path);
  std::vector<Entry> add;
  char line[512];
  int lineno = 0;
  while (std::fgets(line, sizeof line, f)) {
    ++lineno;
    char *hash = std::strchr(line, '#');
    if (hash) *hash = 0;
    char name[64], dt[8], mode[8];
    Entry e{};
    double f7 = 0.0, f8 = 0.0;
    const int k = std::sscanf(line, "%63s %7s %7s %d %d %d %lf %lf", name, dt, mode, &e.cls, &e.bt, &e.sl, &f7, &f8);
    if (k <= 0) continue;
    if (k == 7) {
      e.ms = f7;
    } else if (k == 8 && f7 == (double)(int)f7 && f7 >= 0) {
      e.bs1 = (int)f7;
      e.ms = f8;
    } else {
      std::fclose(f);
      return fail(GBS_ERR_INVALID, "%s:%d: expected 7 or 8 fields", path, lineno);
    }
    e.sid = gbs_stencil_id(name);
    e.dtype = !std::strcmp(dt, "f32") ? GBS_F32 : !std::strcmp(dt, "f64") ? GBS_F64 : -1;
    e.fma = !std::strcmp(mode, "fma") ? 1 : !std::strcmp(mode, "exact") ? 0 : -1;
    if (e.sid < 0 || e.dtype < 0 || e.fma < 0 || e.bt < 1 || e.sl < 0) {
      std::fclose(f);
      return fail(GBS_ERR_INVALID, "%s:%d: bad entry", path, lineno);
    }
    add.push_back(e);
  }
  std::fclose(f);
  for (const Entry &e : add) {
    auto it = std::find_if(g_table.begin(), g_table.end(), [&](const Entry &x) {
      return x.sid == e.sid && x.dtype == e.dtype && x.fma == e.fma && x.cls == e.cls;
    });
    if (it != g_table.end()) *it = e;
    else g_table.push_back(e);
  }
  return GBS_OK;
}

void env_load_locked() {
  if (g_env_loaded) return;
  g_env_loaded = true;
  if (const char *p = std::getenv("GBS_TUNING")) {
    if (*p) load_locked(p);  // a bad file leaves the table as it was
  }
}

void record_locked(const Entry &e) {
  auto it = std::find_if(g_table.begin(), g_table.end(), [&](const Entry &x) {
    return x.sid == e.sid && x.dtype == e.dtype && x.fma == e.fma && x.cls == e.cls;
  });
  if (it != g_table.end()) *it = e;
  else g_table.push_back(e);
}

double hbm_bytes_per_s() {
  int dev = 0, clk_khz = 0, bus_bits = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 8e12;
  if (cudaDeviceGetAttribute(&clk_khz, cudaDevAttrMemoryClockRate, dev) != cudaSuccess || clk_khz <= 0 ||
      cudaDeviceGetAttribute(&bus_bits, cudaDevAttrGlobalMemoryBusWidth, dev) != cudaSuccess || bus_bits <= 0) {
    cudaGetLastError();
    return 8e12;
  }
  return 2.0 * clk_khz * 1e3 * bus_bits / 8.0;
}

double fp_flops_per_s(int dtype) {
  static double cached[2] = {0.0, 0.0};
  const int k = dtype == GBS_F64 ? 1 : 0;
  if (cached[k] <= 0.0) {
    double g = 0.0;
    if (gbs_measure_fp_peak(dtype, &g) == GBS_OK && g > 0.0) cached[k] = g * 1e9;
    else return dtype == GBS_F64 ? 1.2e12 : 7.5e13;
  }
  return cached[k];
}

// redundancy (computed cells / useful cells) of (bt, sl, bs1) for d, as
// gbs_plan reports it; < 0 if the geometry is invalid
double redundancy(const gbs_desc *d, int bt, int sl, int bs1) {
  gbs_desc c = *d;
  c.bt = bt;
  c.sl = sl;
  c.bs1 = bs1;
  gbs_plan_info pi;
  if (gbs_plan(&c, &pi) != GBS_OK) return -1.0;
  return pi.redundancy;
}

}  // namespace

// The table's choice for d, if any (bt = 0 otherwise); used by the run path.
bool tuned_lookup(const gbs_desc *d, int *bt, int *sl, int *bs1) {
  std::lock_guard<std::mutex> lk(g_mu);
  env_load_locked();
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const int cls = size_class(d);
  const int mx = max_bt(d->stencil, d->dtype, fma);
  const Entry *best = nullptr;
  for (const Entry &e : g_table) {
    if (e.sid != d->stencil || e.dtype != d->dtype || e.fma != fma || e.bt > mx) continue;
    if (!best || std::abs(e.cls - cls) < std::abs(best->cls - cls)) best = &e;
  }
  if (!best || std::abs(best->cls - cls) > 3) return false;
  *bt = best->bt;
  *sl = best->cls == cls ? best->sl : 0;  // stream length only for the exact size class
  if (bs1) *bs1 = best->bs1;
  return true;
}

}  // namespace gbs

using namespace gbs;

extern "C" {

gbs_status gbs_tune_load(const char *path) {
  if (!path) return fail(GBS_ERR_INVALID, "path is NULL");
  std::lock_guard<std::mutex> lk(g_mu);
  g_env_loaded = true;
  return load_locked(path);
}

gbs_status gbs_tune_save(const char *path) {
  if (!path) return fail(GBS_ERR_INVALID, "path is NULL");
  std::lock_guard<std::mutex> lk(g_mu);
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(GBS_ERR_INVALID, "cannot write %s", path);
  std::fprintf(f, "# stencil dtype mode size_class bt sl bs1 ms_per_step\n");
  std::vector<Entry> t = g_table;
  std::sort(t.begin(), t.end(), [](const Entry &a, const Entry &b) {
    return std::make_tuple(a.sid, a.dtype, a.fma, a.cls) < std::make_tuple(b.sid, b.dtype, b.fma, b.cls);
  });
  for (const Entry &e : t)
    std::fprintf(f, "%s %s %s %d %d %d %d %.6g\n", gbs_stencil_name(e.sid), e.dtype == GBS_F64 ? "f64" : "f32",
                 e.fma ? "fma" : "exact", e.cls, e.bt, e.sl, e.bs1, e.ms);
  std::fclose(f);
  return GBS_OK;
}

void gbs_tune_clear(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_table.clear();
  g_env_loaded = true;
}

int gbs_tune_entries(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  env_load_locked();
  return (int)g_table.size();
}

gbs_status gbs_tune_set(const gbs_desc *d, int bt, int sl, double ms_per_step) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const int mx = max_bt(d->stencil, d->dtype, fma);
  if (bt < 1 || bt > mx) return fail(GBS_ERR_INVALID, "bt=%d outside 1..%d", bt, mx);
  if (sl < 0) return fail(GBS_ERR_INVALID, "sl < 0");
  if (stencil_def(d->stencil)->dim == 3 && d->bs1 > 0) {
    gbs_desc t = *d;
    t.bt = bt;
    if (variant_3d(&t, bt) < 0) return GBS_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  env_load_locked();
  record_locked(Entry{d->stencil, d->dtype, fma, size_class(d), bt, sl, ms_per_step, std::max(0, d->bs1)});
  return GBS_OK;
}

gbs_status gbs_tune_lookup(const gbs_desc *d, int *bt, int *sl) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!bt || !sl) return fail(GBS_ERR_INVALID, "NULL output");
  *bt = 0;
  *sl = 0;
  tuned_lookup(d, bt, sl, nullptr);
  return GBS_OK;
}

gbs_status gbs_tune_model(const gbs_desc *d, double *ms_per_step) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (!ms_per_step) return fail(GBS_ERR_INVALID, "NULL output");
  gbs_plan_info pi;
  if ((st = gbs_plan(d, &pi)) != GBS_OK) return st;
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const Layout L = make_layout(d);
  double cells = 1.0;
  for (int a = 0; a < s->dim; ++a) cells *= (double)d->n[a];
  const double per_cell = std::max(2.0 * (double)L.esize / (pi.bt * hbm_bytes_per_s()),
                                   pi.redundancy * s->fpp / fp_flops_per_s(d->dtype));
  *ms_per_step = (cells * per_cell + 3e-6 / pi.bt) * 1e3;
  return GBS_OK;
}

gbs_status gbs_tune(const gbs_desc *d, gbs_tune_candidate *cands, int max_cands, int *ncands) {
  gbs_status st = check_desc(d);
  if (st != GBS_OK) return st;
  if (max_cands < 0 || (max_cands > 0 && !cands)) return fail(GBS_ERR_INVALID, "bad candidate buffer");
  const gbs_stencil_def_t *s = stencil_def(d->stencil);
  const int fma = d->fp_mode == GBS_FP_FMA ? 1 : 0;
  const int mx = max_bt(d->stencil, d->dtype, fma);
  if (mx == 0) return fail(GBS_ERR_UNSUPPORTED, "no kernels built for %s", s->name);
  const Layout L = make_layout(d);
  double cells = 1.0;
  for (int a = 0; a < s->dim; ++a) cells *= (double)d->n[a];
  const double B = hbm_bytes_per_s(), P = fp_flops_per_s(d->dtype);
  const double S = (double)L.esize;
  const double launch_gap_s = 3e-6;

  // candidates and their model times
  std::vector<gbs_tune_candidate> cs;
  const int sls2[] = {0, 64, 128, 256, 512};
  const int sls3[] = {0, 32, 64, 128};
  const int *sls = s->dim == 2 ? sls2 : sls3;
  const int nsl = s->dim == 2 ? 5 : 4;
  const int axis0 = d->n[0];
  for (int bt = 1; bt <= mx; ++bt) {
    // block shapes: the 3-D launcher's built tile heights, else the one shape
    std::vector<int> shapes{0};
    if (s->dim == 3) {
      shapes.clear();
      for (int v = 0; v < kVar3; ++v) {
        const Tile3DShape ts = tile_shape_3d(d->stencil, d->dtype, fma, bt, v);
        if (ts.tj > 0) shapes.push_back(ts.tj);
      }
    }
    for (int bs1 : shapes) {
      for (int k = 0; k < nsl; ++k) {
        if (sls[k] != 0 && sls[k] >= axis0) continue;
        const double red = redundancy(d, bt, sls[k], bs1);
        if (red <= 0.0) continue;
        const double per_cell = std::max(2.0 * S / (bt * B), red * s->fpp / P);
        gbs_tune_candidate c{};
        c.bt = bt;
        c.sl = sls[k];
        c.bs1 = bs1;
        c.redundancy = red;
        c.model_ms_per_step = (cells * per_cell + launch_gap_s / bt) * 1e3;
        c.ms_per_step = -1.0;
        cs.push_back(c);
      }
    }
  }
  if (cs.empty()) return fail(GBS_ERR_UNSUPPORTED, "no valid (bt, sl) for %s at this size", s->name);
  double best_model = 1e300;
  for (const auto &c : cs) best_model = std::min(best_model, c.model_ms_per_step);

  // an earlier entry for this key must not steer the candidates' sl = 0
  {
    std::lock_guard<std::mutex> lk(g_mu);
    env_load_locked();
    const int cls = size_class(d);
    g_table.erase(std::remove_if(g_table.begin(), g_table.end(),
                                 [&](const Entry &x) {
                                   return x.sid == d->stencil && x.dtype == d->dtype && x.fma == fma &&
                                          x.cls == cls;
                                 }),
                  g_table.end());
  }
  // time every candidate the model keeps (within 4x of the best prediction)
  int *err = nullptr;
  if ((st = error_word(&err)) != GBS_OK) return st;
  void *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, L.bytes);
  if (e != cudaSuccess) return cuda_fail(e, "tune: scratch grid");
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (stream) cudaStreamDestroy(stream);
    cudaFree(buf);
  };
  if ((e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess ||
      (e = cudaMemsetAsync(buf, 0x3f, L.bytes, stream)) != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "tune: set-up");
  }
  for (auto &c : cs) {
    if (c.model_ms_per_step > 4.0 * best_model) continue;
    gbs_desc t = *d;
    t.bt = c.bt;
    t.sl = c.sl;
    t.bs1 = c.bs1;
    // full-degree launches only: T a multiple of 2*bt, about 4 ms of work
    const int reps = (int)std::min(64.0, std::max(1.0, std::ceil(4.0 / (c.model_ms_per_step * 2 * c.bt))));
    t.timestep = 2 * c.bt;
    if ((st = run_loop(&t, L, buf, stream, err)) != GBS_OK) {  // warm-up
      cleanup();
      return st;
    }
    t.timestep = 2 * c.bt * reps;
    double best = 1e300;
    for (int r = 0; r < 2; ++r) {
      cudaEventRecord(e0, stream);
      if ((st = run_loop(&t, L, buf, stream, err)) != GBS_OK) {
        cleanup();
        return st;
      }
      cudaEventRecord(e1, stream);
      if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
        cleanup();
        return cuda_fail(e, "tune: timing");
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, (double)ms / t.timestep);
    }
    c.ms_per_step = best;
  }
  int host_err = 0;
  e = cudaMemcpy(&host_err, err, sizeof host_err, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "tune: error word");
  if (host_err) {
    cudaMemset(err, 0, sizeof(int));
    return fail(GBS_ERR_TIMEOUT, "tune: device-side wait gave up (code %d)", host_err);
  }

  std::sort(cs.begin(), cs.end(), [](const gbs_tune_candidate &a, const gbs_tune_candidate &b) {
    const double x = a.ms_per_step < 0 ? 1e300 : a.ms_per_step, y = b.ms_per_step < 0 ? 1e300 : b.ms_per_step;
    return x != y ? x < y : a.model_ms_per_step < b.model_ms_per_step;
  });
  {
    std::lock_guard<std::mutex> lk(g_mu);
    env_load_locked();
    record_locked(Entry{d->stencil, d->dtype, fma, size_class(d), cs[0].bt, cs[0].sl, cs[0].ms_per_step,
                        cs[0].bs1});
  }
  if (ncands) *ncands = (int)cs.size();
  for (int i = 0; i < max_cands && i < (int)cs.size(); ++i) cands[i] = cs[i];
  return GBS_OK;
}

}  // extern "C"
