/* Exercises the engine's C ABI from C, the way the artifact's benchmarks
 * call it (kernel_stencil -> gbs_run, common.h:42), without any Python
 * between the caller and libgbstencil.so.
 *
 *   capi_from_c <stencil> <float|double> <n> <T> <exact|fma> <bt> <in.bin> <want.bin>
 *
 * in.bin holds the dense two-plane grid A[2][d0][d1]([d2]) (d = n + 2r) and
 * want.bin the CPU oracle's result of the same time loop. The program runs
 * the loop twice: through gbs_run on a host copy of the grid (the drop-in
 * entry point) and through gbs_get_layout / gbs_upload / gbs_run_device /
 * gbs_sync / gbs_download on a device buffer it allocates itself. It checks
 * plane T%2 of both against want.bin (exact mode: bit for bit; fma mode:
 * normwise max|a-b|/max|b| within 1e-5 float / 1e-12 double), checks that
 * the halo of both planes is untouched, that a bad descriptor returns
 * GBS_ERR_INVALID with a message, and exits 0 only if every check holds. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime.h>

#include "gbstencil.h"

static void *read_file(const char *path, size_t bytes) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  void *p = malloc(bytes);
  size_t got = p ? fread(p, 1, bytes, f) : 0;
  fclose(f);
  if (got != bytes) {
    free(p);
    return NULL;
  }
  return p;
}

static double value(const void *A, int f64, size_t i) {
  return f64 ? ((const double *)A)[i] : (double)((const float *)A)[i];
}

/* 0 when plane t of `got` matches `want` within the mode's bound and the
 * halo of both planes equals `init` */
static int check(const char *what, const void *got, const void *want, const void *init, int f64, int exact,
                 const int *d, int dim, int r, int T) {
  size_t area = 1;
  for (int a = 0; a < dim; ++a) area *= (size_t)d[a];
  const size_t es = f64 ? 8 : 4;
  const size_t off = (size_t)(T % 2) * area;
  double num = 0.0, den = 0.0;
  size_t halo_bad = 0;
  for (size_t i = 0; i < area; ++i) {
    size_t rem = i;
    int halo = 0;
    for (int a = dim - 1; a >= 0; --a) {
      const int c = (int)(rem % (size_t)d[a]);
      rem /= (size_t)d[a];
      if (c < r || c >= d[a] - r) halo = 1;
    }
    if (halo) {
      for (int p = 0; p < 2; ++p)
        if (memcmp((const char *)got + (p * area + i) * es, (const char *)init + (p * area + i) * es, es) != 0)
          ++halo_bad;
    }
    const double a = value(got, f64, off + i), b = value(want, f64, off + i);
    if (exact && memcmp((const char *)got + (off + i) * es, (const char *)want + (off + i) * es, es) != 0)
      num = fmax(num, fabs(a - b) + 1e-300);
    if (!exact) num = fmax(num, fabs(a - b));
    den = fmax(den, fabs(b));
  }
  const double err = num / (den > 0 ? den : 1.0);
  const double tol = exact ? 0.0 : (f64 ? 1e-12 : 1e-5);
  const int ok = halo_bad == 0 && (exact ? num == 0.0 : err <= tol);
  printf("%s: %s normwise error %.3e (bound %.0e), halo cells changed %zu\n", what, ok ? "ok" : "FAIL", err, tol,
         halo_bad);
  return ok ? 0 : 1;
}

int main(int argc, char **argv) {
  if (argc != 9) {
    fprintf(stderr, "usage: %s stencil float|double n T exact|fma bt in.bin want.bin\n", argv[0]);
    return 2;
  }
  gbs_desc d;
  memset(&d, 0, sizeof d);
  d.stencil = gbs_stencil_id(argv[1]);
  if (d.stencil < 0) {
    fprintf(stderr, "unknown stencil %s\n", argv[1]);
    return 2;
  }
  const int f64 = strcmp(argv[2], "double") == 0;
  d.dtype = f64 ? GBS_F64 : GBS_F32;
  const int n = atoi(argv[3]);
  d.timestep = atoi(argv[4]);
  const int exact = strcmp(argv[5], "exact") == 0;
  d.fp_mode = exact ? GBS_FP_EXACT : GBS_FP_FMA;
  d.bt = atoi(argv[6]);
  int dim = 0, rad = 0, nterms = 0, fpp = 0;
  if (gbs_stencil_info(d.stencil, &dim, &rad, &nterms, &fpp) != GBS_OK) return 2;
  int dims[3] = {1, 1, 1};
  size_t area = 1;
  for (int a = 0; a < dim; ++a) {
    d.n[a] = n;
    dims[a] = n + 2 * rad;
    area *= (size_t)dims[a];
  }
  const size_t bytes = 2 * area * (f64 ? 8 : 4);
  void *init = read_file(argv[7], bytes), *want = read_file(argv[8], bytes);
  if (!init || !want) {
    fprintf(stderr, "cannot read %zu bytes from the input files\n", bytes);
    return 2;
  }
  int fails = 0;

  /* 1. the drop-in: host grid in, host grid out, device milliseconds back */
  void *A = malloc(bytes);
  memcpy(A, init, bytes);
  double ms = -1.0;
  gbs_status st = gbs_run(&d, A, &ms);
  if (st != GBS_OK) {
    printf("gbs_run: FAIL status %d: %s\n", (int)st, gbs_last_error());
    return 1;
  }
  fails += check("gbs_run", A, want, init, f64, exact, dims, dim, rad, d.timestep);
  if (!(ms >= 0.0)) {
    printf("gbs_run: FAIL device time %f\n", ms);
    ++fails;
  }

  /* 2. the device path on a buffer the caller owns */
  gbs_layout L;
  if ((st = gbs_get_layout(&d, &L)) != GBS_OK) {
    printf("gbs_get_layout: FAIL %s\n", gbs_last_error());
    return 1;
  }
  void *dev = NULL;
  cudaStream_t stream = NULL;
  if (cudaMalloc(&dev, L.bytes) != cudaSuccess || cudaMemset(dev, 0, L.bytes) != cudaSuccess ||
      cudaStreamCreate(&stream) != cudaSuccess) {
    printf("cuda set-up: FAIL\n");
    return 1;
  }
  memset(A, 0, bytes);
  if ((st = gbs_upload(&d, init, dev, stream)) != GBS_OK || (st = gbs_run_device(&d, dev, stream)) != GBS_OK ||
      (st = gbs_download(&d, dev, A, stream)) != GBS_OK || (st = gbs_sync(stream)) != GBS_OK) {
    printf("device path: FAIL status %d: %s\n", (int)st, gbs_last_error());
    return 1;
  }
  fails += check("gbs_run_device", A, want, init, f64, exact, dims, dim, rad, d.timestep);
  cudaFree(dev);
  cudaStreamDestroy(stream);

  /* 3. a bad descriptor is a status, not an abort */
  gbs_desc bad = d;
  bad.timestep = -1;
  st = gbs_run(&bad, A, NULL);
  if (st != GBS_ERR_INVALID || gbs_last_error()[0] == '\0') {
    printf("bad descriptor: FAIL status %d\n", (int)st);
    ++fails;
  } else {
    printf("bad descriptor: ok (%s)\n", gbs_last_error());
  }
  free(A);
  free(init);
  free(want);
  return fails ? 1 : 0;
}
