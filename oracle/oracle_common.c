/* TEST INFRASTRUCTURE ONLY: grid initialisation and dispatch for the CPU
 * oracle (see oracle_stencils.c). Used by the parity tests and the timed CPU
 * baseline; never by the engine.
 *
 * oracle_init_grid_<t> restates init_grid (common.h:44-56): every cell of
 * both time planes, halo included, is set to 1000 * rand_r(&seed) / RAND_MAX
 * evaluated in the element type, with seed = flat index + compsize. */
#include <stdlib.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef void (*oracle_fn_f)(float *, const int *, int, const float *, float, float);
typedef void (*oracle_fn_d)(double *, const int *, int, const double *, double, double);
typedef void (*oracle_fn_q)(long double *, const int *, int, const long double *, long double, long double);
extern const oracle_fn_f oracle_table_f[];
extern const oracle_fn_d oracle_table_d[];
extern const oracle_fn_q oracle_table_q[];

#define DEFINE_INIT(T, t)                                                    \
  void oracle_init_grid_##t(T *A, int compsize, int dim, int rad)            \
  {                                                                          \
    size_t area = 1, side = (size_t)compsize + 2 * (size_t)rad;              \
    for (int d = 0; d < dim; d++) area *= side;                              \
    _Pragma("omp parallel for")                                              \
    for (size_t i = 0; i < area; i++) {                                      \
      unsigned int seed = (unsigned int)(i + (size_t)compsize);              \
      T v = (T)1000 * (T)rand_r(&seed);                                      \
      A[i] = v / (T)RAND_MAX;                                                \
      A[area + i] = A[i];                                                    \
    }                                                                        \
  }
DEFINE_INIT(float, f)
DEFINE_INIT(double, d)

void oracle_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* tcode: 0 float, 1 double, 2 long double. coef holds nterms values of the
 * element type (the gradient form takes its numerator in coef[0]). */
void oracle_run(int sid, int tcode, void *A, const int *n, int timestep,
                const void *coef, double divisor, double eps)
{
  if (tcode == 0)
    oracle_table_f[sid]((float *)A, n, timestep, (const float *)coef,
                        (float)divisor, (float)eps);
  else if (tcode == 1)
    oracle_table_d[sid]((double *)A, n, timestep, (const double *)coef,
                        divisor, eps);
  else
    oracle_table_q[sid]((long double *)A, n, timestep,
                        (const long double *)coef, (long double)divisor,
                        (long double)eps);
}
