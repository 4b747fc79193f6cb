/* Generated by oracle/gen_oracle.py from the stencil tap table.
 * TEST INFRASTRUCTURE ONLY: the CPU oracle for the CUDA engine's
 * parity tests and the timed CPU baseline. Do not edit by hand. */
#include <math.h>

void oracle_star2d1r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j];
  }
}

void oracle_star2d1r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j];
  }
}

void oracle_star2d1r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j];
  }
}

void oracle_star2d2r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j];
  }
}

void oracle_star2d2r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j];
  }
}

void oracle_star2d2r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j];
  }
}

void oracle_star2d3r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j]
            + coef[1] * A[t%2][i-2][j]
            + coef[2] * A[t%2][i-1][j]
            + coef[3] * A[t%2][i][j-3]
            + coef[4] * A[t%2][i][j-2]
            + coef[5] * A[t%2][i][j-1]
            + coef[6] * A[t%2][i][j]
            + coef[7] * A[t%2][i][j+1]
            + coef[8] * A[t%2][i][j+2]
            + coef[9] * A[t%2][i][j+3]
            + coef[10] * A[t%2][i+1][j]
            + coef[11] * A[t%2][i+2][j]
            + coef[12] * A[t%2][i+3][j];
  }
}

void oracle_star2d3r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j]
            + coef[1] * A[t%2][i-2][j]
            + coef[2] * A[t%2][i-1][j]
            + coef[3] * A[t%2][i][j-3]
            + coef[4] * A[t%2][i][j-2]
            + coef[5] * A[t%2][i][j-1]
            + coef[6] * A[t%2][i][j]
            + coef[7] * A[t%2][i][j+1]
            + coef[8] * A[t%2][i][j+2]
            + coef[9] * A[t%2][i][j+3]
            + coef[10] * A[t%2][i+1][j]
            + coef[11] * A[t%2][i+2][j]
            + coef[12] * A[t%2][i+3][j];
  }
}

void oracle_star2d3r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j]
            + coef[1] * A[t%2][i-2][j]
            + coef[2] * A[t%2][i-1][j]
            + coef[3] * A[t%2][i][j-3]
            + coef[4] * A[t%2][i][j-2]
            + coef[5] * A[t%2][i][j-1]
            + coef[6] * A[t%2][i][j]
            + coef[7] * A[t%2][i][j+1]
            + coef[8] * A[t%2][i][j+2]
            + coef[9] * A[t%2][i][j+3]
            + coef[10] * A[t%2][i+1][j]
            + coef[11] * A[t%2][i+2][j]
            + coef[12] * A[t%2][i+3][j];
  }
}

void oracle_star2d4r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j]
            + coef[1] * A[t%2][i-3][j]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-1][j]
            + coef[4] * A[t%2][i][j-4]
            + coef[5] * A[t%2][i][j-3]
            + coef[6] * A[t%2][i][j-2]
            + coef[7] * A[t%2][i][j-1]
            + coef[8] * A[t%2][i][j]
            + coef[9] * A[t%2][i][j+1]
            + coef[10] * A[t%2][i][j+2]
            + coef[11] * A[t%2][i][j+3]
            + coef[12] * A[t%2][i][j+4]
            + coef[13] * A[t%2][i+1][j]
            + coef[14] * A[t%2][i+2][j]
            + coef[15] * A[t%2][i+3][j]
            + coef[16] * A[t%2][i-4][j];
  }
}

void oracle_star2d4r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j]
            + coef[1] * A[t%2][i-3][j]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-1][j]
            + coef[4] * A[t%2][i][j-4]
            + coef[5] * A[t%2][i][j-3]
            + coef[6] * A[t%2][i][j-2]
            + coef[7] * A[t%2][i][j-1]
            + coef[8] * A[t%2][i][j]
            + coef[9] * A[t%2][i][j+1]
            + coef[10] * A[t%2][i][j+2]
            + coef[11] * A[t%2][i][j+3]
            + coef[12] * A[t%2][i][j+4]
            + coef[13] * A[t%2][i+1][j]
            + coef[14] * A[t%2][i+2][j]
            + coef[15] * A[t%2][i+3][j]
            + coef[16] * A[t%2][i-4][j];
  }
}

void oracle_star2d4r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j]
            + coef[1] * A[t%2][i-3][j]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-1][j]
            + coef[4] * A[t%2][i][j-4]
            + coef[5] * A[t%2][i][j-3]
            + coef[6] * A[t%2][i][j-2]
            + coef[7] * A[t%2][i][j-1]
            + coef[8] * A[t%2][i][j]
            + coef[9] * A[t%2][i][j+1]
            + coef[10] * A[t%2][i][j+2]
            + coef[11] * A[t%2][i][j+3]
            + coef[12] * A[t%2][i][j+4]
            + coef[13] * A[t%2][i+1][j]
            + coef[14] * A[t%2][i+2][j]
            + coef[15] * A[t%2][i+3][j]
            + coef[16] * A[t%2][i-4][j];
  }
}

void oracle_box2d1r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1];
  }
}

void oracle_box2d1r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1];
  }
}

void oracle_box2d1r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1];
  }
}

void oracle_box2d2r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j-2]
            + coef[1] * A[t%2][i-2][j-1]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-2][j+1]
            + coef[4] * A[t%2][i-2][j+2]
            + coef[5] * A[t%2][i-1][j-2]
            + coef[6] * A[t%2][i-1][j-1]
            + coef[7] * A[t%2][i-1][j]
            + coef[8] * A[t%2][i-1][j+1]
            + coef[9] * A[t%2][i-1][j+2]
            + coef[10] * A[t%2][i][j-2]
            + coef[11] * A[t%2][i][j-1]
            + coef[12] * A[t%2][i][j]
            + coef[13] * A[t%2][i][j+1]
            + coef[14] * A[t%2][i][j+2]
            + coef[15] * A[t%2][i+1][j-2]
            + coef[16] * A[t%2][i+1][j-1]
            + coef[17] * A[t%2][i+1][j]
            + coef[18] * A[t%2][i+1][j+1]
            + coef[19] * A[t%2][i+1][j+2]
            + coef[20] * A[t%2][i+2][j-2]
            + coef[21] * A[t%2][i+2][j-1]
            + coef[22] * A[t%2][i+2][j]
            + coef[23] * A[t%2][i+2][j+1]
            + coef[24] * A[t%2][i+2][j+2];
  }
}

void oracle_box2d2r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j-2]
            + coef[1] * A[t%2][i-2][j-1]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-2][j+1]
            + coef[4] * A[t%2][i-2][j+2]
            + coef[5] * A[t%2][i-1][j-2]
            + coef[6] * A[t%2][i-1][j-1]
            + coef[7] * A[t%2][i-1][j]
            + coef[8] * A[t%2][i-1][j+1]
            + coef[9] * A[t%2][i-1][j+2]
            + coef[10] * A[t%2][i][j-2]
            + coef[11] * A[t%2][i][j-1]
            + coef[12] * A[t%2][i][j]
            + coef[13] * A[t%2][i][j+1]
            + coef[14] * A[t%2][i][j+2]
            + coef[15] * A[t%2][i+1][j-2]
            + coef[16] * A[t%2][i+1][j-1]
            + coef[17] * A[t%2][i+1][j]
            + coef[18] * A[t%2][i+1][j+1]
            + coef[19] * A[t%2][i+1][j+2]
            + coef[20] * A[t%2][i+2][j-2]
            + coef[21] * A[t%2][i+2][j-1]
            + coef[22] * A[t%2][i+2][j]
            + coef[23] * A[t%2][i+2][j+1]
            + coef[24] * A[t%2][i+2][j+2];
  }
}

void oracle_box2d2r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-2][j-2]
            + coef[1] * A[t%2][i-2][j-1]
            + coef[2] * A[t%2][i-2][j]
            + coef[3] * A[t%2][i-2][j+1]
            + coef[4] * A[t%2][i-2][j+2]
            + coef[5] * A[t%2][i-1][j-2]
            + coef[6] * A[t%2][i-1][j-1]
            + coef[7] * A[t%2][i-1][j]
            + coef[8] * A[t%2][i-1][j+1]
            + coef[9] * A[t%2][i-1][j+2]
            + coef[10] * A[t%2][i][j-2]
            + coef[11] * A[t%2][i][j-1]
            + coef[12] * A[t%2][i][j]
            + coef[13] * A[t%2][i][j+1]
            + coef[14] * A[t%2][i][j+2]
            + coef[15] * A[t%2][i+1][j-2]
            + coef[16] * A[t%2][i+1][j-1]
            + coef[17] * A[t%2][i+1][j]
            + coef[18] * A[t%2][i+1][j+1]
            + coef[19] * A[t%2][i+1][j+2]
            + coef[20] * A[t%2][i+2][j-2]
            + coef[21] * A[t%2][i+2][j-1]
            + coef[22] * A[t%2][i+2][j]
            + coef[23] * A[t%2][i+2][j+1]
            + coef[24] * A[t%2][i+2][j+2];
  }
}

void oracle_box2d3r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j-3]
            + coef[1] * A[t%2][i-3][j-2]
            + coef[2] * A[t%2][i-3][j-1]
            + coef[3] * A[t%2][i-3][j]
            + coef[4] * A[t%2][i-3][j+1]
            + coef[5] * A[t%2][i-3][j+2]
            + coef[6] * A[t%2][i-3][j+3]
            + coef[7] * A[t%2][i-2][j-3]
            + coef[8] * A[t%2][i-2][j-2]
            + coef[9] * A[t%2][i-2][j-1]
            + coef[10] * A[t%2][i-2][j]
            + coef[11] * A[t%2][i-2][j+1]
            + coef[12] * A[t%2][i-2][j+2]
            + coef[13] * A[t%2][i-2][j+3]
            + coef[14] * A[t%2][i-1][j-3]
            + coef[15] * A[t%2][i-1][j-2]
            + coef[16] * A[t%2][i-1][j-1]
            + coef[17] * A[t%2][i-1][j]
            + coef[18] * A[t%2][i-1][j+1]
            + coef[19] * A[t%2][i-1][j+2]
            + coef[20] * A[t%2][i-1][j+3]
            + coef[21] * A[t%2][i][j-3]
            + coef[22] * A[t%2][i][j-2]
            + coef[23] * A[t%2][i][j-1]
            + coef[24] * A[t%2][i][j]
            + coef[25] * A[t%2][i][j+1]
            + coef[26] * A[t%2][i][j+2]
            + coef[27] * A[t%2][i][j+3]
            + coef[28] * A[t%2][i+1][j-3]
            + coef[29] * A[t%2][i+1][j-2]
            + coef[30] * A[t%2][i+1][j-1]
            + coef[31] * A[t%2][i+1][j]
            + coef[32] * A[t%2][i+1][j+1]
            + coef[33] * A[t%2][i+1][j+2]
            + coef[34] * A[t%2][i+1][j+3]
            + coef[35] * A[t%2][i+2][j-3]
            + coef[36] * A[t%2][i+2][j-2]
            + coef[37] * A[t%2][i+2][j-1]
            + coef[38] * A[t%2][i+2][j]
            + coef[39] * A[t%2][i+2][j+1]
            + coef[40] * A[t%2][i+2][j+2]
            + coef[41] * A[t%2][i+2][j+3]
            + coef[42] * A[t%2][i+3][j-3]
            + coef[43] * A[t%2][i+3][j-2]
            + coef[44] * A[t%2][i+3][j-1]
            + coef[45] * A[t%2][i+3][j]
            + coef[46] * A[t%2][i+3][j+1]
            + coef[47] * A[t%2][i+3][j+2]
            + coef[48] * A[t%2][i+3][j+3];
  }
}

void oracle_box2d3r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j-3]
            + coef[1] * A[t%2][i-3][j-2]
            + coef[2] * A[t%2][i-3][j-1]
            + coef[3] * A[t%2][i-3][j]
            + coef[4] * A[t%2][i-3][j+1]
            + coef[5] * A[t%2][i-3][j+2]
            + coef[6] * A[t%2][i-3][j+3]
            + coef[7] * A[t%2][i-2][j-3]
            + coef[8] * A[t%2][i-2][j-2]
            + coef[9] * A[t%2][i-2][j-1]
            + coef[10] * A[t%2][i-2][j]
            + coef[11] * A[t%2][i-2][j+1]
            + coef[12] * A[t%2][i-2][j+2]
            + coef[13] * A[t%2][i-2][j+3]
            + coef[14] * A[t%2][i-1][j-3]
            + coef[15] * A[t%2][i-1][j-2]
            + coef[16] * A[t%2][i-1][j-1]
            + coef[17] * A[t%2][i-1][j]
            + coef[18] * A[t%2][i-1][j+1]
            + coef[19] * A[t%2][i-1][j+2]
            + coef[20] * A[t%2][i-1][j+3]
            + coef[21] * A[t%2][i][j-3]
            + coef[22] * A[t%2][i][j-2]
            + coef[23] * A[t%2][i][j-1]
            + coef[24] * A[t%2][i][j]
            + coef[25] * A[t%2][i][j+1]
            + coef[26] * A[t%2][i][j+2]
            + coef[27] * A[t%2][i][j+3]
            + coef[28] * A[t%2][i+1][j-3]
            + coef[29] * A[t%2][i+1][j-2]
            + coef[30] * A[t%2][i+1][j-1]
            + coef[31] * A[t%2][i+1][j]
            + coef[32] * A[t%2][i+1][j+1]
            + coef[33] * A[t%2][i+1][j+2]
            + coef[34] * A[t%2][i+1][j+3]
            + coef[35] * A[t%2][i+2][j-3]
            + coef[36] * A[t%2][i+2][j-2]
            + coef[37] * A[t%2][i+2][j-1]
            + coef[38] * A[t%2][i+2][j]
            + coef[39] * A[t%2][i+2][j+1]
            + coef[40] * A[t%2][i+2][j+2]
            + coef[41] * A[t%2][i+2][j+3]
            + coef[42] * A[t%2][i+3][j-3]
            + coef[43] * A[t%2][i+3][j-2]
            + coef[44] * A[t%2][i+3][j-1]
            + coef[45] * A[t%2][i+3][j]
            + coef[46] * A[t%2][i+3][j+1]
            + coef[47] * A[t%2][i+3][j+2]
            + coef[48] * A[t%2][i+3][j+3];
  }
}

void oracle_box2d3r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-3][j-3]
            + coef[1] * A[t%2][i-3][j-2]
            + coef[2] * A[t%2][i-3][j-1]
            + coef[3] * A[t%2][i-3][j]
            + coef[4] * A[t%2][i-3][j+1]
            + coef[5] * A[t%2][i-3][j+2]
            + coef[6] * A[t%2][i-3][j+3]
            + coef[7] * A[t%2][i-2][j-3]
            + coef[8] * A[t%2][i-2][j-2]
            + coef[9] * A[t%2][i-2][j-1]
            + coef[10] * A[t%2][i-2][j]
            + coef[11] * A[t%2][i-2][j+1]
            + coef[12] * A[t%2][i-2][j+2]
            + coef[13] * A[t%2][i-2][j+3]
            + coef[14] * A[t%2][i-1][j-3]
            + coef[15] * A[t%2][i-1][j-2]
            + coef[16] * A[t%2][i-1][j-1]
            + coef[17] * A[t%2][i-1][j]
            + coef[18] * A[t%2][i-1][j+1]
            + coef[19] * A[t%2][i-1][j+2]
            + coef[20] * A[t%2][i-1][j+3]
            + coef[21] * A[t%2][i][j-3]
            + coef[22] * A[t%2][i][j-2]
            + coef[23] * A[t%2][i][j-1]
            + coef[24] * A[t%2][i][j]
            + coef[25] * A[t%2][i][j+1]
            + coef[26] * A[t%2][i][j+2]
            + coef[27] * A[t%2][i][j+3]
            + coef[28] * A[t%2][i+1][j-3]
            + coef[29] * A[t%2][i+1][j-2]
            + coef[30] * A[t%2][i+1][j-1]
            + coef[31] * A[t%2][i+1][j]
            + coef[32] * A[t%2][i+1][j+1]
            + coef[33] * A[t%2][i+1][j+2]
            + coef[34] * A[t%2][i+1][j+3]
            + coef[35] * A[t%2][i+2][j-3]
            + coef[36] * A[t%2][i+2][j-2]
            + coef[37] * A[t%2][i+2][j-1]
            + coef[38] * A[t%2][i+2][j]
            + coef[39] * A[t%2][i+2][j+1]
            + coef[40] * A[t%2][i+2][j+2]
            + coef[41] * A[t%2][i+2][j+3]
            + coef[42] * A[t%2][i+3][j-3]
            + coef[43] * A[t%2][i+3][j-2]
            + coef[44] * A[t%2][i+3][j-1]
            + coef[45] * A[t%2][i+3][j]
            + coef[46] * A[t%2][i+3][j+1]
            + coef[47] * A[t%2][i+3][j+2]
            + coef[48] * A[t%2][i+3][j+3];
  }
}

void oracle_box2d4r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j-4]
            + coef[1] * A[t%2][i-4][j-3]
            + coef[2] * A[t%2][i-4][j-2]
            + coef[3] * A[t%2][i-4][j-1]
            + coef[4] * A[t%2][i-4][j]
            + coef[5] * A[t%2][i-4][j+1]
            + coef[6] * A[t%2][i-4][j+2]
            + coef[7] * A[t%2][i-4][j+3]
            + coef[8] * A[t%2][i-4][j+4]
            + coef[9] * A[t%2][i-3][j-4]
            + coef[10] * A[t%2][i-3][j-3]
            + coef[11] * A[t%2][i-3][j-2]
            + coef[12] * A[t%2][i-3][j-1]
            + coef[13] * A[t%2][i-3][j]
            + coef[14] * A[t%2][i-3][j+1]
            + coef[15] * A[t%2][i-3][j+2]
            + coef[16] * A[t%2][i-3][j+3]
            + coef[17] * A[t%2][i-3][j+4]
            + coef[18] * A[t%2][i-2][j-4]
            + coef[19] * A[t%2][i-2][j-3]
            + coef[20] * A[t%2][i-2][j-2]
            + coef[21] * A[t%2][i-2][j-1]
            + coef[22] * A[t%2][i-2][j]
            + coef[23] * A[t%2][i-2][j+1]
            + coef[24] * A[t%2][i-2][j+2]
            + coef[25] * A[t%2][i-2][j+3]
            + coef[26] * A[t%2][i-2][j+4]
            + coef[27] * A[t%2][i-1][j-4]
            + coef[28] * A[t%2][i-1][j-3]
            + coef[29] * A[t%2][i-1][j-2]
            + coef[30] * A[t%2][i-1][j-1]
            + coef[31] * A[t%2][i-1][j]
            + coef[32] * A[t%2][i-1][j+1]
            + coef[33] * A[t%2][i-1][j+2]
            + coef[34] * A[t%2][i-1][j+3]
            + coef[35] * A[t%2][i-1][j+4]
            + coef[36] * A[t%2][i][j-4]
            + coef[37] * A[t%2][i][j-3]
            + coef[38] * A[t%2][i][j-2]
            + coef[39] * A[t%2][i][j-1]
            + coef[40] * A[t%2][i][j]
            + coef[41] * A[t%2][i][j+1]
            + coef[42] * A[t%2][i][j+2]
            + coef[43] * A[t%2][i][j+3]
            + coef[44] * A[t%2][i][j+4]
            + coef[45] * A[t%2][i+1][j-4]
            + coef[46] * A[t%2][i+1][j-3]
            + coef[47] * A[t%2][i+1][j-2]
            + coef[48] * A[t%2][i+1][j-1]
            + coef[49] * A[t%2][i+1][j]
            + coef[50] * A[t%2][i+1][j+1]
            + coef[51] * A[t%2][i+1][j+2]
            + coef[52] * A[t%2][i+1][j+3]
            + coef[53] * A[t%2][i+1][j+4]
            + coef[54] * A[t%2][i+2][j-4]
            + coef[55] * A[t%2][i+2][j-3]
            + coef[56] * A[t%2][i+2][j-2]
            + coef[57] * A[t%2][i+2][j-1]
            + coef[58] * A[t%2][i+2][j]
            + coef[59] * A[t%2][i+2][j+1]
            + coef[60] * A[t%2][i+2][j+2]
            + coef[61] * A[t%2][i+2][j+3]
            + coef[62] * A[t%2][i+2][j+4]
            + coef[63] * A[t%2][i+3][j-4]
            + coef[64] * A[t%2][i+3][j-3]
            + coef[65] * A[t%2][i+3][j-2]
            + coef[66] * A[t%2][i+3][j-1]
            + coef[67] * A[t%2][i+3][j]
            + coef[68] * A[t%2][i+3][j+1]
            + coef[69] * A[t%2][i+3][j+2]
            + coef[70] * A[t%2][i+3][j+3]
            + coef[71] * A[t%2][i+3][j+4]
            + coef[72] * A[t%2][i+4][j-4]
            + coef[73] * A[t%2][i+4][j-3]
            + coef[74] * A[t%2][i+4][j-2]
            + coef[75] * A[t%2][i+4][j-1]
            + coef[76] * A[t%2][i+4][j]
            + coef[77] * A[t%2][i+4][j+1]
            + coef[78] * A[t%2][i+4][j+2]
            + coef[79] * A[t%2][i+4][j+3]
            + coef[80] * A[t%2][i+4][j+4];
  }
}

void oracle_box2d4r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j-4]
            + coef[1] * A[t%2][i-4][j-3]
            + coef[2] * A[t%2][i-4][j-2]
            + coef[3] * A[t%2][i-4][j-1]
            + coef[4] * A[t%2][i-4][j]
            + coef[5] * A[t%2][i-4][j+1]
            + coef[6] * A[t%2][i-4][j+2]
            + coef[7] * A[t%2][i-4][j+3]
            + coef[8] * A[t%2][i-4][j+4]
            + coef[9] * A[t%2][i-3][j-4]
            + coef[10] * A[t%2][i-3][j-3]
            + coef[11] * A[t%2][i-3][j-2]
            + coef[12] * A[t%2][i-3][j-1]
            + coef[13] * A[t%2][i-3][j]
            + coef[14] * A[t%2][i-3][j+1]
            + coef[15] * A[t%2][i-3][j+2]
            + coef[16] * A[t%2][i-3][j+3]
            + coef[17] * A[t%2][i-3][j+4]
            + coef[18] * A[t%2][i-2][j-4]
            + coef[19] * A[t%2][i-2][j-3]
            + coef[20] * A[t%2][i-2][j-2]
            + coef[21] * A[t%2][i-2][j-1]
            + coef[22] * A[t%2][i-2][j]
            + coef[23] * A[t%2][i-2][j+1]
            + coef[24] * A[t%2][i-2][j+2]
            + coef[25] * A[t%2][i-2][j+3]
            + coef[26] * A[t%2][i-2][j+4]
            + coef[27] * A[t%2][i-1][j-4]
            + coef[28] * A[t%2][i-1][j-3]
            + coef[29] * A[t%2][i-1][j-2]
            + coef[30] * A[t%2][i-1][j-1]
            + coef[31] * A[t%2][i-1][j]
            + coef[32] * A[t%2][i-1][j+1]
            + coef[33] * A[t%2][i-1][j+2]
            + coef[34] * A[t%2][i-1][j+3]
            + coef[35] * A[t%2][i-1][j+4]
            + coef[36] * A[t%2][i][j-4]
            + coef[37] * A[t%2][i][j-3]
            + coef[38] * A[t%2][i][j-2]
            + coef[39] * A[t%2][i][j-1]
            + coef[40] * A[t%2][i][j]
            + coef[41] * A[t%2][i][j+1]
            + coef[42] * A[t%2][i][j+2]
            + coef[43] * A[t%2][i][j+3]
            + coef[44] * A[t%2][i][j+4]
            + coef[45] * A[t%2][i+1][j-4]
            + coef[46] * A[t%2][i+1][j-3]
            + coef[47] * A[t%2][i+1][j-2]
            + coef[48] * A[t%2][i+1][j-1]
            + coef[49] * A[t%2][i+1][j]
            + coef[50] * A[t%2][i+1][j+1]
            + coef[51] * A[t%2][i+1][j+2]
            + coef[52] * A[t%2][i+1][j+3]
            + coef[53] * A[t%2][i+1][j+4]
            + coef[54] * A[t%2][i+2][j-4]
            + coef[55] * A[t%2][i+2][j-3]
            + coef[56] * A[t%2][i+2][j-2]
            + coef[57] * A[t%2][i+2][j-1]
            + coef[58] * A[t%2][i+2][j]
            + coef[59] * A[t%2][i+2][j+1]
            + coef[60] * A[t%2][i+2][j+2]
            + coef[61] * A[t%2][i+2][j+3]
            + coef[62] * A[t%2][i+2][j+4]
            + coef[63] * A[t%2][i+3][j-4]
            + coef[64] * A[t%2][i+3][j-3]
            + coef[65] * A[t%2][i+3][j-2]
            + coef[66] * A[t%2][i+3][j-1]
            + coef[67] * A[t%2][i+3][j]
            + coef[68] * A[t%2][i+3][j+1]
            + coef[69] * A[t%2][i+3][j+2]
            + coef[70] * A[t%2][i+3][j+3]
            + coef[71] * A[t%2][i+3][j+4]
            + coef[72] * A[t%2][i+4][j-4]
            + coef[73] * A[t%2][i+4][j-3]
            + coef[74] * A[t%2][i+4][j-2]
            + coef[75] * A[t%2][i+4][j-1]
            + coef[76] * A[t%2][i+4][j]
            + coef[77] * A[t%2][i+4][j+1]
            + coef[78] * A[t%2][i+4][j+2]
            + coef[79] * A[t%2][i+4][j+3]
            + coef[80] * A[t%2][i+4][j+4];
  }
}

void oracle_box2d4r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
          A[(t+1)%2][i][j] =
            coef[0] * A[t%2][i-4][j-4]
            + coef[1] * A[t%2][i-4][j-3]
            + coef[2] * A[t%2][i-4][j-2]
            + coef[3] * A[t%2][i-4][j-1]
            + coef[4] * A[t%2][i-4][j]
            + coef[5] * A[t%2][i-4][j+1]
            + coef[6] * A[t%2][i-4][j+2]
            + coef[7] * A[t%2][i-4][j+3]
            + coef[8] * A[t%2][i-4][j+4]
            + coef[9] * A[t%2][i-3][j-4]
            + coef[10] * A[t%2][i-3][j-3]
            + coef[11] * A[t%2][i-3][j-2]
            + coef[12] * A[t%2][i-3][j-1]
            + coef[13] * A[t%2][i-3][j]
            + coef[14] * A[t%2][i-3][j+1]
            + coef[15] * A[t%2][i-3][j+2]
            + coef[16] * A[t%2][i-3][j+3]
            + coef[17] * A[t%2][i-3][j+4]
            + coef[18] * A[t%2][i-2][j-4]
            + coef[19] * A[t%2][i-2][j-3]
            + coef[20] * A[t%2][i-2][j-2]
            + coef[21] * A[t%2][i-2][j-1]
            + coef[22] * A[t%2][i-2][j]
            + coef[23] * A[t%2][i-2][j+1]
            + coef[24] * A[t%2][i-2][j+2]
            + coef[25] * A[t%2][i-2][j+3]
            + coef[26] * A[t%2][i-2][j+4]
            + coef[27] * A[t%2][i-1][j-4]
            + coef[28] * A[t%2][i-1][j-3]
            + coef[29] * A[t%2][i-1][j-2]
            + coef[30] * A[t%2][i-1][j-1]
            + coef[31] * A[t%2][i-1][j]
            + coef[32] * A[t%2][i-1][j+1]
            + coef[33] * A[t%2][i-1][j+2]
            + coef[34] * A[t%2][i-1][j+3]
            + coef[35] * A[t%2][i-1][j+4]
            + coef[36] * A[t%2][i][j-4]
            + coef[37] * A[t%2][i][j-3]
            + coef[38] * A[t%2][i][j-2]
            + coef[39] * A[t%2][i][j-1]
            + coef[40] * A[t%2][i][j]
            + coef[41] * A[t%2][i][j+1]
            + coef[42] * A[t%2][i][j+2]
            + coef[43] * A[t%2][i][j+3]
            + coef[44] * A[t%2][i][j+4]
            + coef[45] * A[t%2][i+1][j-4]
            + coef[46] * A[t%2][i+1][j-3]
            + coef[47] * A[t%2][i+1][j-2]
            + coef[48] * A[t%2][i+1][j-1]
            + coef[49] * A[t%2][i+1][j]
            + coef[50] * A[t%2][i+1][j+1]
            + coef[51] * A[t%2][i+1][j+2]
            + coef[52] * A[t%2][i+1][j+3]
            + coef[53] * A[t%2][i+1][j+4]
            + coef[54] * A[t%2][i+2][j-4]
            + coef[55] * A[t%2][i+2][j-3]
            + coef[56] * A[t%2][i+2][j-2]
            + coef[57] * A[t%2][i+2][j-1]
            + coef[58] * A[t%2][i+2][j]
            + coef[59] * A[t%2][i+2][j+1]
            + coef[60] * A[t%2][i+2][j+2]
            + coef[61] * A[t%2][i+2][j+3]
            + coef[62] * A[t%2][i+2][j+4]
            + coef[63] * A[t%2][i+3][j-4]
            + coef[64] * A[t%2][i+3][j-3]
            + coef[65] * A[t%2][i+3][j-2]
            + coef[66] * A[t%2][i+3][j-1]
            + coef[67] * A[t%2][i+3][j]
            + coef[68] * A[t%2][i+3][j+1]
            + coef[69] * A[t%2][i+3][j+2]
            + coef[70] * A[t%2][i+3][j+3]
            + coef[71] * A[t%2][i+3][j+4]
            + coef[72] * A[t%2][i+4][j-4]
            + coef[73] * A[t%2][i+4][j-3]
            + coef[74] * A[t%2][i+4][j-2]
            + coef[75] * A[t%2][i+4][j-1]
            + coef[76] * A[t%2][i+4][j]
            + coef[77] * A[t%2][i+4][j+1]
            + coef[78] * A[t%2][i+4][j+2]
            + coef[79] * A[t%2][i+4][j+3]
            + coef[80] * A[t%2][i+4][j+4];
  }
}

void oracle_j2d5pt_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j]) / divisor;
  }
}

void oracle_j2d5pt_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j]) / divisor;
  }
}

void oracle_j2d5pt_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j]
            + coef[1] * A[t%2][i][j-1]
            + coef[2] * A[t%2][i][j]
            + coef[3] * A[t%2][i][j+1]
            + coef[4] * A[t%2][i+1][j]) / divisor;
  }
}

void oracle_j2d9pt_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j]) / divisor;
  }
}

void oracle_j2d9pt_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j]) / divisor;
  }
}

void oracle_j2d9pt_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-2][j]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i][j-2]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i][j+2]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+2][j]) / divisor;
  }
}

void oracle_j2d9pt_gol_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1]) / divisor;
  }
}

void oracle_j2d9pt_gol_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1]) / divisor;
  }
}

void oracle_j2d9pt_gol_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
          A[(t+1)%2][i][j] =
            (coef[0] * A[t%2][i-1][j-1]
            + coef[1] * A[t%2][i-1][j]
            + coef[2] * A[t%2][i-1][j+1]
            + coef[3] * A[t%2][i][j-1]
            + coef[4] * A[t%2][i][j]
            + coef[5] * A[t%2][i][j+1]
            + coef[6] * A[t%2][i+1][j-1]
            + coef[7] * A[t%2][i+1][j]
            + coef[8] * A[t%2][i+1][j+1]) / divisor;
  }
}

void oracle_gradient2d_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  float (*A)[d0][d1] = (float (*)[d0][d1])A1;
  const double numer = (double)coef[0];
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++) {
        const float s = eps + (A[t%2][i][j] - A[t%2][i-1][j]) * (A[t%2][i][j] - A[t%2][i-1][j]) +
                 (A[t%2][i][j] - A[t%2][i+1][j]) * (A[t%2][i][j] - A[t%2][i+1][j]) +
                 (A[t%2][i][j] - A[t%2][i][j+1]) * (A[t%2][i][j] - A[t%2][i][j+1]) +
                 (A[t%2][i][j] - A[t%2][i][j-1]) * (A[t%2][i][j] - A[t%2][i][j-1]);
        A[(t+1)%2][i][j] = (float)((double)A[t%2][i][j] + numer / sqrt((double)s));
      }
  }
}

void oracle_gradient2d_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  double (*A)[d0][d1] = (double (*)[d0][d1])A1;
  const double numer = (double)coef[0];
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++) {
        const double s = eps + (A[t%2][i][j] - A[t%2][i-1][j]) * (A[t%2][i][j] - A[t%2][i-1][j]) +
                 (A[t%2][i][j] - A[t%2][i+1][j]) * (A[t%2][i][j] - A[t%2][i+1][j]) +
                 (A[t%2][i][j] - A[t%2][i][j+1]) * (A[t%2][i][j] - A[t%2][i][j+1]) +
                 (A[t%2][i][j] - A[t%2][i][j-1]) * (A[t%2][i][j] - A[t%2][i][j-1]);
        A[(t+1)%2][i][j] = (double)((double)A[t%2][i][j] + numer / sqrt((double)s));
      }
  }
}

void oracle_gradient2d_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2;
  long double (*A)[d0][d1] = (long double (*)[d0][d1])A1;
  const long double numer = (long double)coef[0];
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++) {
        const long double s = eps + (A[t%2][i][j] - A[t%2][i-1][j]) * (A[t%2][i][j] - A[t%2][i-1][j]) +
                 (A[t%2][i][j] - A[t%2][i+1][j]) * (A[t%2][i][j] - A[t%2][i+1][j]) +
                 (A[t%2][i][j] - A[t%2][i][j+1]) * (A[t%2][i][j] - A[t%2][i][j+1]) +
                 (A[t%2][i][j] - A[t%2][i][j-1]) * (A[t%2][i][j] - A[t%2][i][j-1]);
        A[(t+1)%2][i][j] = (long double)((long double)A[t%2][i][j] + numer / sqrtl((long double)s));
      }
  }
}

void oracle_star3d1r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1];
  }
}

void oracle_star3d1r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1];
  }
}

void oracle_star3d1r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1];
  }
}

void oracle_star3d2r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1]
            + coef[7] * A[t%2][i-2][j][k]
            + coef[8] * A[t%2][i+2][j][k]
            + coef[9] * A[t%2][i][j-2][k]
            + coef[10] * A[t%2][i][j+2][k]
            + coef[11] * A[t%2][i][j][k-2]
            + coef[12] * A[t%2][i][j][k+2];
  }
}

void oracle_star3d2r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1]
            + coef[7] * A[t%2][i-2][j][k]
            + coef[8] * A[t%2][i+2][j][k]
            + coef[9] * A[t%2][i][j-2][k]
            + coef[10] * A[t%2][i][j+2][k]
            + coef[11] * A[t%2][i][j][k-2]
            + coef[12] * A[t%2][i][j][k+2];
  }
}

void oracle_star3d2r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i-1][j][k]
            + coef[2] * A[t%2][i+1][j][k]
            + coef[3] * A[t%2][i][j-1][k]
            + coef[4] * A[t%2][i][j+1][k]
            + coef[5] * A[t%2][i][j][k-1]
            + coef[6] * A[t%2][i][j][k+1]
            + coef[7] * A[t%2][i-2][j][k]
            + coef[8] * A[t%2][i+2][j][k]
            + coef[9] * A[t%2][i][j-2][k]
            + coef[10] * A[t%2][i][j+2][k]
            + coef[11] * A[t%2][i][j][k-2]
            + coef[12] * A[t%2][i][j][k+2];
  }
}

void oracle_star3d3r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-3]
            + coef[2] * A[t%2][i][j][k-2]
            + coef[3] * A[t%2][i][j][k-1]
            + coef[4] * A[t%2][i][j][k+1]
            + coef[5] * A[t%2][i][j][k+2]
            + coef[6] * A[t%2][i][j][k+3]
            + coef[7] * A[t%2][i-1][j][k]
            + coef[8] * A[t%2][i+1][j][k]
            + coef[9] * A[t%2][i][j-1][k]
            + coef[10] * A[t%2][i][j+1][k]
            + coef[11] * A[t%2][i-2][j][k]
            + coef[12] * A[t%2][i+2][j][k]
            + coef[13] * A[t%2][i][j-2][k]
            + coef[14] * A[t%2][i][j+2][k]
            + coef[15] * A[t%2][i-3][j][k]
            + coef[16] * A[t%2][i+3][j][k]
            + coef[17] * A[t%2][i][j-3][k]
            + coef[18] * A[t%2][i][j+3][k];
  }
}

void oracle_star3d3r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-3]
            + coef[2] * A[t%2][i][j][k-2]
            + coef[3] * A[t%2][i][j][k-1]
            + coef[4] * A[t%2][i][j][k+1]
            + coef[5] * A[t%2][i][j][k+2]
            + coef[6] * A[t%2][i][j][k+3]
            + coef[7] * A[t%2][i-1][j][k]
            + coef[8] * A[t%2][i+1][j][k]
            + coef[9] * A[t%2][i][j-1][k]
            + coef[10] * A[t%2][i][j+1][k]
            + coef[11] * A[t%2][i-2][j][k]
            + coef[12] * A[t%2][i+2][j][k]
            + coef[13] * A[t%2][i][j-2][k]
            + coef[14] * A[t%2][i][j+2][k]
            + coef[15] * A[t%2][i-3][j][k]
            + coef[16] * A[t%2][i+3][j][k]
            + coef[17] * A[t%2][i][j-3][k]
            + coef[18] * A[t%2][i][j+3][k];
  }
}

void oracle_star3d3r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-3]
            + coef[2] * A[t%2][i][j][k-2]
            + coef[3] * A[t%2][i][j][k-1]
            + coef[4] * A[t%2][i][j][k+1]
            + coef[5] * A[t%2][i][j][k+2]
            + coef[6] * A[t%2][i][j][k+3]
            + coef[7] * A[t%2][i-1][j][k]
            + coef[8] * A[t%2][i+1][j][k]
            + coef[9] * A[t%2][i][j-1][k]
            + coef[10] * A[t%2][i][j+1][k]
            + coef[11] * A[t%2][i-2][j][k]
            + coef[12] * A[t%2][i+2][j][k]
            + coef[13] * A[t%2][i][j-2][k]
            + coef[14] * A[t%2][i][j+2][k]
            + coef[15] * A[t%2][i-3][j][k]
            + coef[16] * A[t%2][i+3][j][k]
            + coef[17] * A[t%2][i][j-3][k]
            + coef[18] * A[t%2][i][j+3][k];
  }
}

void oracle_star3d4r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-4]
            + coef[2] * A[t%2][i][j][k-3]
            + coef[3] * A[t%2][i][j][k-2]
            + coef[4] * A[t%2][i][j][k-1]
            + coef[5] * A[t%2][i][j][k+1]
            + coef[6] * A[t%2][i][j][k+2]
            + coef[7] * A[t%2][i][j][k+3]
            + coef[8] * A[t%2][i][j][k+4]
            + coef[9] * A[t%2][i-1][j][k]
            + coef[10] * A[t%2][i+1][j][k]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j+1][k]
            + coef[13] * A[t%2][i-2][j][k]
            + coef[14] * A[t%2][i+2][j][k]
            + coef[15] * A[t%2][i][j-2][k]
            + coef[16] * A[t%2][i][j+2][k]
            + coef[17] * A[t%2][i-3][j][k]
            + coef[18] * A[t%2][i+3][j][k]
            + coef[19] * A[t%2][i][j-3][k]
            + coef[20] * A[t%2][i][j+3][k]
            + coef[21] * A[t%2][i-4][j][k]
            + coef[22] * A[t%2][i+4][j][k]
            + coef[23] * A[t%2][i][j-4][k]
            + coef[24] * A[t%2][i][j+4][k];
  }
}

void oracle_star3d4r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-4]
            + coef[2] * A[t%2][i][j][k-3]
            + coef[3] * A[t%2][i][j][k-2]
            + coef[4] * A[t%2][i][j][k-1]
            + coef[5] * A[t%2][i][j][k+1]
            + coef[6] * A[t%2][i][j][k+2]
            + coef[7] * A[t%2][i][j][k+3]
            + coef[8] * A[t%2][i][j][k+4]
            + coef[9] * A[t%2][i-1][j][k]
            + coef[10] * A[t%2][i+1][j][k]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j+1][k]
            + coef[13] * A[t%2][i-2][j][k]
            + coef[14] * A[t%2][i+2][j][k]
            + coef[15] * A[t%2][i][j-2][k]
            + coef[16] * A[t%2][i][j+2][k]
            + coef[17] * A[t%2][i-3][j][k]
            + coef[18] * A[t%2][i+3][j][k]
            + coef[19] * A[t%2][i][j-3][k]
            + coef[20] * A[t%2][i][j+3][k]
            + coef[21] * A[t%2][i-4][j][k]
            + coef[22] * A[t%2][i+4][j][k]
            + coef[23] * A[t%2][i][j-4][k]
            + coef[24] * A[t%2][i][j+4][k];
  }
}

void oracle_star3d4r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i][j][k]
            + coef[1] * A[t%2][i][j][k-4]
            + coef[2] * A[t%2][i][j][k-3]
            + coef[3] * A[t%2][i][j][k-2]
            + coef[4] * A[t%2][i][j][k-1]
            + coef[5] * A[t%2][i][j][k+1]
            + coef[6] * A[t%2][i][j][k+2]
            + coef[7] * A[t%2][i][j][k+3]
            + coef[8] * A[t%2][i][j][k+4]
            + coef[9] * A[t%2][i-1][j][k]
            + coef[10] * A[t%2][i+1][j][k]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j+1][k]
            + coef[13] * A[t%2][i-2][j][k]
            + coef[14] * A[t%2][i+2][j][k]
            + coef[15] * A[t%2][i][j-2][k]
            + coef[16] * A[t%2][i][j+2][k]
            + coef[17] * A[t%2][i-3][j][k]
            + coef[18] * A[t%2][i+3][j][k]
            + coef[19] * A[t%2][i][j-3][k]
            + coef[20] * A[t%2][i][j+3][k]
            + coef[21] * A[t%2][i-4][j][k]
            + coef[22] * A[t%2][i+4][j][k]
            + coef[23] * A[t%2][i][j-4][k]
            + coef[24] * A[t%2][i][j+4][k];
  }
}

void oracle_box3d1r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1];
  }
}

void oracle_box3d1r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1];
  }
}

void oracle_box3d1r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1];
  }
}

void oracle_box3d2r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-2][j][k]
            + coef[1] * A[t%2][i-2][j-2][k-2]
            + coef[2] * A[t%2][i-2][j-2][k-1]
            + coef[3] * A[t%2][i-2][j-2][k]
            + coef[4] * A[t%2][i-2][j-2][k+1]
            + coef[5] * A[t%2][i-2][j-2][k+2]
            + coef[6] * A[t%2][i-2][j-1][k-2]
            + coef[7] * A[t%2][i-2][j-1][k-1]
            + coef[8] * A[t%2][i-2][j-1][k]
            + coef[9] * A[t%2][i-2][j-1][k+1]
            + coef[10] * A[t%2][i-2][j-1][k+2]
            + coef[11] * A[t%2][i-2][j][k-2]
            + coef[12] * A[t%2][i-2][j][k-1]
            + coef[13] * A[t%2][i-2][j][k+1]
            + coef[14] * A[t%2][i-2][j][k+2]
            + coef[15] * A[t%2][i-2][j+1][k-2]
            + coef[16] * A[t%2][i-2][j+1][k-1]
            + coef[17] * A[t%2][i-2][j+1][k]
            + coef[18] * A[t%2][i-2][j+1][k+1]
            + coef[19] * A[t%2][i-2][j+1][k+2]
            + coef[20] * A[t%2][i-2][j+2][k-2]
            + coef[21] * A[t%2][i-2][j+2][k-1]
            + coef[22] * A[t%2][i-2][j+2][k]
            + coef[23] * A[t%2][i-2][j+2][k+1]
            + coef[24] * A[t%2][i-2][j+2][k+2]
            + coef[25] * A[t%2][i-1][j][k]
            + coef[26] * A[t%2][i-1][j-2][k-2]
            + coef[27] * A[t%2][i-1][j-2][k-1]
            + coef[28] * A[t%2][i-1][j-2][k]
            + coef[29] * A[t%2][i-1][j-2][k+1]
            + coef[30] * A[t%2][i-1][j-2][k+2]
            + coef[31] * A[t%2][i-1][j-1][k-2]
            + coef[32] * A[t%2][i-1][j-1][k-1]
            + coef[33] * A[t%2][i-1][j-1][k]
            + coef[34] * A[t%2][i-1][j-1][k+1]
            + coef[35] * A[t%2][i-1][j-1][k+2]
            + coef[36] * A[t%2][i-1][j][k-2]
            + coef[37] * A[t%2][i-1][j][k-1]
            + coef[38] * A[t%2][i-1][j][k+1]
            + coef[39] * A[t%2][i-1][j][k+2]
            + coef[40] * A[t%2][i-1][j+1][k-2]
            + coef[41] * A[t%2][i-1][j+1][k-1]
            + coef[42] * A[t%2][i-1][j+1][k]
            + coef[43] * A[t%2][i-1][j+1][k+1]
            + coef[44] * A[t%2][i-1][j+1][k+2]
            + coef[45] * A[t%2][i-1][j+2][k-2]
            + coef[46] * A[t%2][i-1][j+2][k-1]
            + coef[47] * A[t%2][i-1][j+2][k]
            + coef[48] * A[t%2][i-1][j+2][k+1]
            + coef[49] * A[t%2][i-1][j+2][k+2]
            + coef[50] * A[t%2][i][j][k]
            + coef[51] * A[t%2][i][j-2][k-2]
            + coef[52] * A[t%2][i][j-2][k-1]
            + coef[53] * A[t%2][i][j-2][k]
            + coef[54] * A[t%2][i][j-2][k+1]
            + coef[55] * A[t%2][i][j-2][k+2]
            + coef[56] * A[t%2][i][j-1][k-2]
            + coef[57] * A[t%2][i][j-1][k-1]
            + coef[58] * A[t%2][i][j-1][k]
            + coef[59] * A[t%2][i][j-1][k+1]
            + coef[60] * A[t%2][i][j-1][k+2]
            + coef[61] * A[t%2][i][j][k-2]
            + coef[62] * A[t%2][i][j][k-1]
            + coef[63] * A[t%2][i][j][k+1]
            + coef[64] * A[t%2][i][j][k+2]
            + coef[65] * A[t%2][i][j+1][k-2]
            + coef[66] * A[t%2][i][j+1][k-1]
            + coef[67] * A[t%2][i][j+1][k]
            + coef[68] * A[t%2][i][j+1][k+1]
            + coef[69] * A[t%2][i][j+1][k+2]
            + coef[70] * A[t%2][i][j+2][k-2]
            + coef[71] * A[t%2][i][j+2][k-1]
            + coef[72] * A[t%2][i][j+2][k]
            + coef[73] * A[t%2][i][j+2][k+1]
            + coef[74] * A[t%2][i][j+2][k+2]
            + coef[75] * A[t%2][i+1][j][k]
            + coef[76] * A[t%2][i+1][j-2][k-2]
            + coef[77] * A[t%2][i+1][j-2][k-1]
            + coef[78] * A[t%2][i+1][j-2][k]
            + coef[79] * A[t%2][i+1][j-2][k+1]
            + coef[80] * A[t%2][i+1][j-2][k+2]
            + coef[81] * A[t%2][i+1][j-1][k-2]
            + coef[82] * A[t%2][i+1][j-1][k-1]
            + coef[83] * A[t%2][i+1][j-1][k]
            + coef[84] * A[t%2][i+1][j-1][k+1]
            + coef[85] * A[t%2][i+1][j-1][k+2]
            + coef[86] * A[t%2][i+1][j][k-2]
            + coef[87] * A[t%2][i+1][j][k-1]
            + coef[88] * A[t%2][i+1][j][k+1]
            + coef[89] * A[t%2][i+1][j][k+2]
            + coef[90] * A[t%2][i+1][j+1][k-2]
            + coef[91] * A[t%2][i+1][j+1][k-1]
            + coef[92] * A[t%2][i+1][j+1][k]
            + coef[93] * A[t%2][i+1][j+1][k+1]
            + coef[94] * A[t%2][i+1][j+1][k+2]
            + coef[95] * A[t%2][i+1][j+2][k-2]
            + coef[96] * A[t%2][i+1][j+2][k-1]
            + coef[97] * A[t%2][i+1][j+2][k]
            + coef[98] * A[t%2][i+1][j+2][k+1]
            + coef[99] * A[t%2][i+1][j+2][k+2]
            + coef[100] * A[t%2][i+2][j][k]
            + coef[101] * A[t%2][i+2][j-2][k-2]
            + coef[102] * A[t%2][i+2][j-2][k-1]
            + coef[103] * A[t%2][i+2][j-2][k]
            + coef[104] * A[t%2][i+2][j-2][k+1]
            + coef[105] * A[t%2][i+2][j-2][k+2]
            + coef[106] * A[t%2][i+2][j-1][k-2]
            + coef[107] * A[t%2][i+2][j-1][k-1]
            + coef[108] * A[t%2][i+2][j-1][k]
            + coef[109] * A[t%2][i+2][j-1][k+1]
            + coef[110] * A[t%2][i+2][j-1][k+2]
            + coef[111] * A[t%2][i+2][j][k-2]
            + coef[112] * A[t%2][i+2][j][k-1]
            + coef[113] * A[t%2][i+2][j][k+1]
            + coef[114] * A[t%2][i+2][j][k+2]
            + coef[115] * A[t%2][i+2][j+1][k-2]
            + coef[116] * A[t%2][i+2][j+1][k-1]
            + coef[117] * A[t%2][i+2][j+1][k]
            + coef[118] * A[t%2][i+2][j+1][k+1]
            + coef[119] * A[t%2][i+2][j+1][k+2]
            + coef[120] * A[t%2][i+2][j+2][k-2]
            + coef[121] * A[t%2][i+2][j+2][k-1]
            + coef[122] * A[t%2][i+2][j+2][k]
            + coef[123] * A[t%2][i+2][j+2][k+1]
            + coef[124] * A[t%2][i+2][j+2][k+2];
  }
}

void oracle_box3d2r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-2][j][k]
            + coef[1] * A[t%2][i-2][j-2][k-2]
            + coef[2] * A[t%2][i-2][j-2][k-1]
            + coef[3] * A[t%2][i-2][j-2][k]
            + coef[4] * A[t%2][i-2][j-2][k+1]
            + coef[5] * A[t%2][i-2][j-2][k+2]
            + coef[6] * A[t%2][i-2][j-1][k-2]
            + coef[7] * A[t%2][i-2][j-1][k-1]
            + coef[8] * A[t%2][i-2][j-1][k]
            + coef[9] * A[t%2][i-2][j-1][k+1]
            + coef[10] * A[t%2][i-2][j-1][k+2]
            + coef[11] * A[t%2][i-2][j][k-2]
            + coef[12] * A[t%2][i-2][j][k-1]
            + coef[13] * A[t%2][i-2][j][k+1]
            + coef[14] * A[t%2][i-2][j][k+2]
            + coef[15] * A[t%2][i-2][j+1][k-2]
            + coef[16] * A[t%2][i-2][j+1][k-1]
            + coef[17] * A[t%2][i-2][j+1][k]
            + coef[18] * A[t%2][i-2][j+1][k+1]
            + coef[19] * A[t%2][i-2][j+1][k+2]
            + coef[20] * A[t%2][i-2][j+2][k-2]
            + coef[21] * A[t%2][i-2][j+2][k-1]
            + coef[22] * A[t%2][i-2][j+2][k]
            + coef[23] * A[t%2][i-2][j+2][k+1]
            + coef[24] * A[t%2][i-2][j+2][k+2]
            + coef[25] * A[t%2][i-1][j][k]
            + coef[26] * A[t%2][i-1][j-2][k-2]
            + coef[27] * A[t%2][i-1][j-2][k-1]
            + coef[28] * A[t%2][i-1][j-2][k]
            + coef[29] * A[t%2][i-1][j-2][k+1]
            + coef[30] * A[t%2][i-1][j-2][k+2]
            + coef[31] * A[t%2][i-1][j-1][k-2]
            + coef[32] * A[t%2][i-1][j-1][k-1]
            + coef[33] * A[t%2][i-1][j-1][k]
            + coef[34] * A[t%2][i-1][j-1][k+1]
            + coef[35] * A[t%2][i-1][j-1][k+2]
            + coef[36] * A[t%2][i-1][j][k-2]
            + coef[37] * A[t%2][i-1][j][k-1]
            + coef[38] * A[t%2][i-1][j][k+1]
            + coef[39] * A[t%2][i-1][j][k+2]
            + coef[40] * A[t%2][i-1][j+1][k-2]
            + coef[41] * A[t%2][i-1][j+1][k-1]
            + coef[42] * A[t%2][i-1][j+1][k]
            + coef[43] * A[t%2][i-1][j+1][k+1]
            + coef[44] * A[t%2][i-1][j+1][k+2]
            + coef[45] * A[t%2][i-1][j+2][k-2]
            + coef[46] * A[t%2][i-1][j+2][k-1]
            + coef[47] * A[t%2][i-1][j+2][k]
            + coef[48] * A[t%2][i-1][j+2][k+1]
            + coef[49] * A[t%2][i-1][j+2][k+2]
            + coef[50] * A[t%2][i][j][k]
            + coef[51] * A[t%2][i][j-2][k-2]
            + coef[52] * A[t%2][i][j-2][k-1]
            + coef[53] * A[t%2][i][j-2][k]
            + coef[54] * A[t%2][i][j-2][k+1]
            + coef[55] * A[t%2][i][j-2][k+2]
            + coef[56] * A[t%2][i][j-1][k-2]
            + coef[57] * A[t%2][i][j-1][k-1]
            + coef[58] * A[t%2][i][j-1][k]
            + coef[59] * A[t%2][i][j-1][k+1]
            + coef[60] * A[t%2][i][j-1][k+2]
            + coef[61] * A[t%2][i][j][k-2]
            + coef[62] * A[t%2][i][j][k-1]
            + coef[63] * A[t%2][i][j][k+1]
            + coef[64] * A[t%2][i][j][k+2]
            + coef[65] * A[t%2][i][j+1][k-2]
            + coef[66] * A[t%2][i][j+1][k-1]
            + coef[67] * A[t%2][i][j+1][k]
            + coef[68] * A[t%2][i][j+1][k+1]
            + coef[69] * A[t%2][i][j+1][k+2]
            + coef[70] * A[t%2][i][j+2][k-2]
            + coef[71] * A[t%2][i][j+2][k-1]
            + coef[72] * A[t%2][i][j+2][k]
            + coef[73] * A[t%2][i][j+2][k+1]
            + coef[74] * A[t%2][i][j+2][k+2]
            + coef[75] * A[t%2][i+1][j][k]
            + coef[76] * A[t%2][i+1][j-2][k-2]
            + coef[77] * A[t%2][i+1][j-2][k-1]
            + coef[78] * A[t%2][i+1][j-2][k]
            + coef[79] * A[t%2][i+1][j-2][k+1]
            + coef[80] * A[t%2][i+1][j-2][k+2]
            + coef[81] * A[t%2][i+1][j-1][k-2]
            + coef[82] * A[t%2][i+1][j-1][k-1]
            + coef[83] * A[t%2][i+1][j-1][k]
            + coef[84] * A[t%2][i+1][j-1][k+1]
            + coef[85] * A[t%2][i+1][j-1][k+2]
            + coef[86] * A[t%2][i+1][j][k-2]
            + coef[87] * A[t%2][i+1][j][k-1]
            + coef[88] * A[t%2][i+1][j][k+1]
            + coef[89] * A[t%2][i+1][j][k+2]
            + coef[90] * A[t%2][i+1][j+1][k-2]
            + coef[91] * A[t%2][i+1][j+1][k-1]
            + coef[92] * A[t%2][i+1][j+1][k]
            + coef[93] * A[t%2][i+1][j+1][k+1]
            + coef[94] * A[t%2][i+1][j+1][k+2]
            + coef[95] * A[t%2][i+1][j+2][k-2]
            + coef[96] * A[t%2][i+1][j+2][k-1]
            + coef[97] * A[t%2][i+1][j+2][k]
            + coef[98] * A[t%2][i+1][j+2][k+1]
            + coef[99] * A[t%2][i+1][j+2][k+2]
            + coef[100] * A[t%2][i+2][j][k]
            + coef[101] * A[t%2][i+2][j-2][k-2]
            + coef[102] * A[t%2][i+2][j-2][k-1]
            + coef[103] * A[t%2][i+2][j-2][k]
            + coef[104] * A[t%2][i+2][j-2][k+1]
            + coef[105] * A[t%2][i+2][j-2][k+2]
            + coef[106] * A[t%2][i+2][j-1][k-2]
            + coef[107] * A[t%2][i+2][j-1][k-1]
            + coef[108] * A[t%2][i+2][j-1][k]
            + coef[109] * A[t%2][i+2][j-1][k+1]
            + coef[110] * A[t%2][i+2][j-1][k+2]
            + coef[111] * A[t%2][i+2][j][k-2]
            + coef[112] * A[t%2][i+2][j][k-1]
            + coef[113] * A[t%2][i+2][j][k+1]
            + coef[114] * A[t%2][i+2][j][k+2]
            + coef[115] * A[t%2][i+2][j+1][k-2]
            + coef[116] * A[t%2][i+2][j+1][k-1]
            + coef[117] * A[t%2][i+2][j+1][k]
            + coef[118] * A[t%2][i+2][j+1][k+1]
            + coef[119] * A[t%2][i+2][j+1][k+2]
            + coef[120] * A[t%2][i+2][j+2][k-2]
            + coef[121] * A[t%2][i+2][j+2][k-1]
            + coef[122] * A[t%2][i+2][j+2][k]
            + coef[123] * A[t%2][i+2][j+2][k+1]
            + coef[124] * A[t%2][i+2][j+2][k+2];
  }
}

void oracle_box3d2r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-2][j][k]
            + coef[1] * A[t%2][i-2][j-2][k-2]
            + coef[2] * A[t%2][i-2][j-2][k-1]
            + coef[3] * A[t%2][i-2][j-2][k]
            + coef[4] * A[t%2][i-2][j-2][k+1]
            + coef[5] * A[t%2][i-2][j-2][k+2]
            + coef[6] * A[t%2][i-2][j-1][k-2]
            + coef[7] * A[t%2][i-2][j-1][k-1]
            + coef[8] * A[t%2][i-2][j-1][k]
            + coef[9] * A[t%2][i-2][j-1][k+1]
            + coef[10] * A[t%2][i-2][j-1][k+2]
            + coef[11] * A[t%2][i-2][j][k-2]
            + coef[12] * A[t%2][i-2][j][k-1]
            + coef[13] * A[t%2][i-2][j][k+1]
            + coef[14] * A[t%2][i-2][j][k+2]
            + coef[15] * A[t%2][i-2][j+1][k-2]
            + coef[16] * A[t%2][i-2][j+1][k-1]
            + coef[17] * A[t%2][i-2][j+1][k]
            + coef[18] * A[t%2][i-2][j+1][k+1]
            + coef[19] * A[t%2][i-2][j+1][k+2]
            + coef[20] * A[t%2][i-2][j+2][k-2]
            + coef[21] * A[t%2][i-2][j+2][k-1]
            + coef[22] * A[t%2][i-2][j+2][k]
            + coef[23] * A[t%2][i-2][j+2][k+1]
            + coef[24] * A[t%2][i-2][j+2][k+2]
            + coef[25] * A[t%2][i-1][j][k]
            + coef[26] * A[t%2][i-1][j-2][k-2]
            + coef[27] * A[t%2][i-1][j-2][k-1]
            + coef[28] * A[t%2][i-1][j-2][k]
            + coef[29] * A[t%2][i-1][j-2][k+1]
            + coef[30] * A[t%2][i-1][j-2][k+2]
            + coef[31] * A[t%2][i-1][j-1][k-2]
            + coef[32] * A[t%2][i-1][j-1][k-1]
            + coef[33] * A[t%2][i-1][j-1][k]
            + coef[34] * A[t%2][i-1][j-1][k+1]
            + coef[35] * A[t%2][i-1][j-1][k+2]
            + coef[36] * A[t%2][i-1][j][k-2]
            + coef[37] * A[t%2][i-1][j][k-1]
            + coef[38] * A[t%2][i-1][j][k+1]
            + coef[39] * A[t%2][i-1][j][k+2]
            + coef[40] * A[t%2][i-1][j+1][k-2]
            + coef[41] * A[t%2][i-1][j+1][k-1]
            + coef[42] * A[t%2][i-1][j+1][k]
            + coef[43] * A[t%2][i-1][j+1][k+1]
            + coef[44] * A[t%2][i-1][j+1][k+2]
            + coef[45] * A[t%2][i-1][j+2][k-2]
            + coef[46] * A[t%2][i-1][j+2][k-1]
            + coef[47] * A[t%2][i-1][j+2][k]
            + coef[48] * A[t%2][i-1][j+2][k+1]
            + coef[49] * A[t%2][i-1][j+2][k+2]
            + coef[50] * A[t%2][i][j][k]
            + coef[51] * A[t%2][i][j-2][k-2]
            + coef[52] * A[t%2][i][j-2][k-1]
            + coef[53] * A[t%2][i][j-2][k]
            + coef[54] * A[t%2][i][j-2][k+1]
            + coef[55] * A[t%2][i][j-2][k+2]
            + coef[56] * A[t%2][i][j-1][k-2]
            + coef[57] * A[t%2][i][j-1][k-1]
            + coef[58] * A[t%2][i][j-1][k]
            + coef[59] * A[t%2][i][j-1][k+1]
            + coef[60] * A[t%2][i][j-1][k+2]
            + coef[61] * A[t%2][i][j][k-2]
            + coef[62] * A[t%2][i][j][k-1]
            + coef[63] * A[t%2][i][j][k+1]
            + coef[64] * A[t%2][i][j][k+2]
            + coef[65] * A[t%2][i][j+1][k-2]
            + coef[66] * A[t%2][i][j+1][k-1]
            + coef[67] * A[t%2][i][j+1][k]
            + coef[68] * A[t%2][i][j+1][k+1]
            + coef[69] * A[t%2][i][j+1][k+2]
            + coef[70] * A[t%2][i][j+2][k-2]
            + coef[71] * A[t%2][i][j+2][k-1]
            + coef[72] * A[t%2][i][j+2][k]
            + coef[73] * A[t%2][i][j+2][k+1]
            + coef[74] * A[t%2][i][j+2][k+2]
            + coef[75] * A[t%2][i+1][j][k]
            + coef[76] * A[t%2][i+1][j-2][k-2]
            + coef[77] * A[t%2][i+1][j-2][k-1]
            + coef[78] * A[t%2][i+1][j-2][k]
            + coef[79] * A[t%2][i+1][j-2][k+1]
            + coef[80] * A[t%2][i+1][j-2][k+2]
            + coef[81] * A[t%2][i+1][j-1][k-2]
            + coef[82] * A[t%2][i+1][j-1][k-1]
            + coef[83] * A[t%2][i+1][j-1][k]
            + coef[84] * A[t%2][i+1][j-1][k+1]
            + coef[85] * A[t%2][i+1][j-1][k+2]
            + coef[86] * A[t%2][i+1][j][k-2]
            + coef[87] * A[t%2][i+1][j][k-1]
            + coef[88] * A[t%2][i+1][j][k+1]
            + coef[89] * A[t%2][i+1][j][k+2]
            + coef[90] * A[t%2][i+1][j+1][k-2]
            + coef[91] * A[t%2][i+1][j+1][k-1]
            + coef[92] * A[t%2][i+1][j+1][k]
            + coef[93] * A[t%2][i+1][j+1][k+1]
            + coef[94] * A[t%2][i+1][j+1][k+2]
            + coef[95] * A[t%2][i+1][j+2][k-2]
            + coef[96] * A[t%2][i+1][j+2][k-1]
            + coef[97] * A[t%2][i+1][j+2][k]
            + coef[98] * A[t%2][i+1][j+2][k+1]
            + coef[99] * A[t%2][i+1][j+2][k+2]
            + coef[100] * A[t%2][i+2][j][k]
            + coef[101] * A[t%2][i+2][j-2][k-2]
            + coef[102] * A[t%2][i+2][j-2][k-1]
            + coef[103] * A[t%2][i+2][j-2][k]
            + coef[104] * A[t%2][i+2][j-2][k+1]
            + coef[105] * A[t%2][i+2][j-2][k+2]
            + coef[106] * A[t%2][i+2][j-1][k-2]
            + coef[107] * A[t%2][i+2][j-1][k-1]
            + coef[108] * A[t%2][i+2][j-1][k]
            + coef[109] * A[t%2][i+2][j-1][k+1]
            + coef[110] * A[t%2][i+2][j-1][k+2]
            + coef[111] * A[t%2][i+2][j][k-2]
            + coef[112] * A[t%2][i+2][j][k-1]
            + coef[113] * A[t%2][i+2][j][k+1]
            + coef[114] * A[t%2][i+2][j][k+2]
            + coef[115] * A[t%2][i+2][j+1][k-2]
            + coef[116] * A[t%2][i+2][j+1][k-1]
            + coef[117] * A[t%2][i+2][j+1][k]
            + coef[118] * A[t%2][i+2][j+1][k+1]
            + coef[119] * A[t%2][i+2][j+1][k+2]
            + coef[120] * A[t%2][i+2][j+2][k-2]
            + coef[121] * A[t%2][i+2][j+2][k-1]
            + coef[122] * A[t%2][i+2][j+2][k]
            + coef[123] * A[t%2][i+2][j+2][k+1]
            + coef[124] * A[t%2][i+2][j+2][k+2];
  }
}

void oracle_box3d3r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-3][j][k]
            + coef[1] * A[t%2][i-3][j-3][k-3]
            + coef[2] * A[t%2][i-3][j-3][k-2]
            + coef[3] * A[t%2][i-3][j-3][k-1]
            + coef[4] * A[t%2][i-3][j-3][k]
            + coef[5] * A[t%2][i-3][j-3][k+1]
            + coef[6] * A[t%2][i-3][j-3][k+2]
            + coef[7] * A[t%2][i-3][j-3][k+3]
            + coef[8] * A[t%2][i-3][j-2][k-3]
            + coef[9] * A[t%2][i-3][j-2][k-2]
            + coef[10] * A[t%2][i-3][j-2][k-1]
            + coef[11] * A[t%2][i-3][j-2][k]
            + coef[12] * A[t%2][i-3][j-2][k+1]
            + coef[13] * A[t%2][i-3][j-2][k+2]
            + coef[14] * A[t%2][i-3][j-2][k+3]
            + coef[15] * A[t%2][i-3][j-1][k-3]
            + coef[16] * A[t%2][i-3][j-1][k-2]
            + coef[17] * A[t%2][i-3][j-1][k-1]
            + coef[18] * A[t%2][i-3][j-1][k]
            + coef[19] * A[t%2][i-3][j-1][k+1]
            + coef[20] * A[t%2][i-3][j-1][k+2]
            + coef[21] * A[t%2][i-3][j-1][k+3]
            + coef[22] * A[t%2][i-3][j][k-3]
            + coef[23] * A[t%2][i-3][j][k-2]
            + coef[24] * A[t%2][i-3][j][k-1]
            + coef[25] * A[t%2][i-3][j][k+1]
            + coef[26] * A[t%2][i-3][j][k+2]
            + coef[27] * A[t%2][i-3][j][k+3]
            + coef[28] * A[t%2][i-3][j+1][k-3]
            + coef[29] * A[t%2][i-3][j+1][k-2]
            + coef[30] * A[t%2][i-3][j+1][k-1]
            + coef[31] * A[t%2][i-3][j+1][k]
            + coef[32] * A[t%2][i-3][j+1][k+1]
            + coef[33] * A[t%2][i-3][j+1][k+2]
            + coef[34] * A[t%2][i-3][j+1][k+3]
            + coef[35] * A[t%2][i-3][j+2][k-3]
            + coef[36] * A[t%2][i-3][j+2][k-2]
            + coef[37] * A[t%2][i-3][j+2][k-1]
            + coef[38] * A[t%2][i-3][j+2][k]
            + coef[39] * A[t%2][i-3][j+2][k+1]
            + coef[40] * A[t%2][i-3][j+2][k+2]
            + coef[41] * A[t%2][i-3][j+2][k+3]
            + coef[42] * A[t%2][i-3][j+3][k-3]
            + coef[43] * A[t%2][i-3][j+3][k-2]
            + coef[44] * A[t%2][i-3][j+3][k-1]
            + coef[45] * A[t%2][i-3][j+3][k]
            + coef[46] * A[t%2][i-3][j+3][k+1]
            + coef[47] * A[t%2][i-3][j+3][k+2]
            + coef[48] * A[t%2][i-3][j+3][k+3]
            + coef[49] * A[t%2][i-2][j][k]
            + coef[50] * A[t%2][i-2][j-3][k-3]
            + coef[51] * A[t%2][i-2][j-3][k-2]
            + coef[52] * A[t%2][i-2][j-3][k-1]
            + coef[53] * A[t%2][i-2][j-3][k]
            + coef[54] * A[t%2][i-2][j-3][k+1]
            + coef[55] * A[t%2][i-2][j-3][k+2]
            + coef[56] * A[t%2][i-2][j-3][k+3]
            + coef[57] * A[t%2][i-2][j-2][k-3]
            + coef[58] * A[t%2][i-2][j-2][k-2]
            + coef[59] * A[t%2][i-2][j-2][k-1]
            + coef[60] * A[t%2][i-2][j-2][k]
            + coef[61] * A[t%2][i-2][j-2][k+1]
            + coef[62] * A[t%2][i-2][j-2][k+2]
            + coef[63] * A[t%2][i-2][j-2][k+3]
            + coef[64] * A[t%2][i-2][j-1][k-3]
            + coef[65] * A[t%2][i-2][j-1][k-2]
            + coef[66] * A[t%2][i-2][j-1][k-1]
            + coef[67] * A[t%2][i-2][j-1][k]
            + coef[68] * A[t%2][i-2][j-1][k+1]
            + coef[69] * A[t%2][i-2][j-1][k+2]
            + coef[70] * A[t%2][i-2][j-1][k+3]
            + coef[71] * A[t%2][i-2][j][k-3]
            + coef[72] * A[t%2][i-2][j][k-2]
            + coef[73] * A[t%2][i-2][j][k-1]
            + coef[74] * A[t%2][i-2][j][k+1]
            + coef[75] * A[t%2][i-2][j][k+2]
            + coef[76] * A[t%2][i-2][j][k+3]
            + coef[77] * A[t%2][i-2][j+1][k-3]
            + coef[78] * A[t%2][i-2][j+1][k-2]
            + coef[79] * A[t%2][i-2][j+1][k-1]
            + coef[80] * A[t%2][i-2][j+1][k]
            + coef[81] * A[t%2][i-2][j+1][k+1]
            + coef[82] * A[t%2][i-2][j+1][k+2]
            + coef[83] * A[t%2][i-2][j+1][k+3]
            + coef[84] * A[t%2][i-2][j+2][k-3]
            + coef[85] * A[t%2][i-2][j+2][k-2]
            + coef[86] * A[t%2][i-2][j+2][k-1]
            + coef[87] * A[t%2][i-2][j+2][k]
            + coef[88] * A[t%2][i-2][j+2][k+1]
            + coef[89] * A[t%2][i-2][j+2][k+2]
            + coef[90] * A[t%2][i-2][j+2][k+3]
            + coef[91] * A[t%2][i-2][j+3][k-3]
            + coef[92] * A[t%2][i-2][j+3][k-2]
            + coef[93] * A[t%2][i-2][j+3][k-1]
            + coef[94] * A[t%2][i-2][j+3][k]
            + coef[95] * A[t%2][i-2][j+3][k+1]
            + coef[96] * A[t%2][i-2][j+3][k+2]
            + coef[97] * A[t%2][i-2][j+3][k+3]
            + coef[98] * A[t%2][i-1][j][k]
            + coef[99] * A[t%2][i-1][j-3][k-3]
            + coef[100] * A[t%2][i-1][j-3][k-2]
            + coef[101] * A[t%2][i-1][j-3][k-1]
            + coef[102] * A[t%2][i-1][j-3][k]
            + coef[103] * A[t%2][i-1][j-3][k+1]
            + coef[104] * A[t%2][i-1][j-3][k+2]
            + coef[105] * A[t%2][i-1][j-3][k+3]
            + coef[106] * A[t%2][i-1][j-2][k-3]
            + coef[107] * A[t%2][i-1][j-2][k-2]
            + coef[108] * A[t%2][i-1][j-2][k-1]
            + coef[109] * A[t%2][i-1][j-2][k]
            + coef[110] * A[t%2][i-1][j-2][k+1]
            + coef[111] * A[t%2][i-1][j-2][k+2]
            + coef[112] * A[t%2][i-1][j-2][k+3]
            + coef[113] * A[t%2][i-1][j-1][k-3]
            + coef[114] * A[t%2][i-1][j-1][k-2]
            + coef[115] * A[t%2][i-1][j-1][k-1]
            + coef[116] * A[t%2][i-1][j-1][k]
            + coef[117] * A[t%2][i-1][j-1][k+1]
            + coef[118] * A[t%2][i-1][j-1][k+2]
            + coef[119] * A[t%2][i-1][j-1][k+3]
            + coef[120] * A[t%2][i-1][j][k-3]
            + coef[121] * A[t%2][i-1][j][k-2]
            + coef[122] * A[t%2][i-1][j][k-1]
            + coef[123] * A[t%2][i-1][j][k+1]
            + coef[124] * A[t%2][i-1][j][k+2]
            + coef[125] * A[t%2][i-1][j][k+3]
            + coef[126] * A[t%2][i-1][j+1][k-3]
            + coef[127] * A[t%2][i-1][j+1][k-2]
            + coef[128] * A[t%2][i-1][j+1][k-1]
            + coef[129] * A[t%2][i-1][j+1][k]
            + coef[130] * A[t%2][i-1][j+1][k+1]
            + coef[131] * A[t%2][i-1][j+1][k+2]
            + coef[132] * A[t%2][i-1][j+1][k+3]
            + coef[133] * A[t%2][i-1][j+2][k-3]
            + coef[134] * A[t%2][i-1][j+2][k-2]
            + coef[135] * A[t%2][i-1][j+2][k-1]
            + coef[136] * A[t%2][i-1][j+2][k]
            + coef[137] * A[t%2][i-1][j+2][k+1]
            + coef[138] * A[t%2][i-1][j+2][k+2]
            + coef[139] * A[t%2][i-1][j+2][k+3]
            + coef[140] * A[t%2][i-1][j+3][k-3]
            + coef[141] * A[t%2][i-1][j+3][k-2]
            + coef[142] * A[t%2][i-1][j+3][k-1]
            + coef[143] * A[t%2][i-1][j+3][k]
            + coef[144] * A[t%2][i-1][j+3][k+1]
            + coef[145] * A[t%2][i-1][j+3][k+2]
            + coef[146] * A[t%2][i-1][j+3][k+3]
            + coef[147] * A[t%2][i][j][k]
            + coef[148] * A[t%2][i][j-3][k-3]
            + coef[149] * A[t%2][i][j-3][k-2]
            + coef[150] * A[t%2][i][j-3][k-1]
            + coef[151] * A[t%2][i][j-3][k]
            + coef[152] * A[t%2][i][j-3][k+1]
            + coef[153] * A[t%2][i][j-3][k+2]
            + coef[154] * A[t%2][i][j-3][k+3]
            + coef[155] * A[t%2][i][j-2][k-3]
            + coef[156] * A[t%2][i][j-2][k-2]
            + coef[157] * A[t%2][i][j-2][k-1]
            + coef[158] * A[t%2][i][j-2][k]
            + coef[159] * A[t%2][i][j-2][k+1]
            + coef[160] * A[t%2][i][j-2][k+2]
            + coef[161] * A[t%2][i][j-2][k+3]
            + coef[162] * A[t%2][i][j-1][k-3]
            + coef[163] * A[t%2][i][j-1][k-2]
            + coef[164] * A[t%2][i][j-1][k-1]
            + coef[165] * A[t%2][i][j-1][k]
            + coef[166] * A[t%2][i][j-1][k+1]
            + coef[167] * A[t%2][i][j-1][k+2]
            + coef[168] * A[t%2][i][j-1][k+3]
            + coef[169] * A[t%2][i][j][k-3]
            + coef[170] * A[t%2][i][j][k-2]
            + coef[171] * A[t%2][i][j][k-1]
            + coef[172] * A[t%2][i][j][k+1]
            + coef[173] * A[t%2][i][j][k+2]
            + coef[174] * A[t%2][i][j][k+3]
            + coef[175] * A[t%2][i][j+1][k-3]
            + coef[176] * A[t%2][i][j+1][k-2]
            + coef[177] * A[t%2][i][j+1][k-1]
            + coef[178] * A[t%2][i][j+1][k]
            + coef[179] * A[t%2][i][j+1][k+1]
            + coef[180] * A[t%2][i][j+1][k+2]
            + coef[181] * A[t%2][i][j+1][k+3]
            + coef[182] * A[t%2][i][j+2][k-3]
            + coef[183] * A[t%2][i][j+2][k-2]
            + coef[184] * A[t%2][i][j+2][k-1]
            + coef[185] * A[t%2][i][j+2][k]
            + coef[186] * A[t%2][i][j+2][k+1]
            + coef[187] * A[t%2][i][j+2][k+2]
            + coef[188] * A[t%2][i][j+2][k+3]
            + coef[189] * A[t%2][i][j+3][k-3]
            + coef[190] * A[t%2][i][j+3][k-2]
            + coef[191] * A[t%2][i][j+3][k-1]
            + coef[192] * A[t%2][i][j+3][k]
            + coef[193] * A[t%2][i][j+3][k+1]
            + coef[194] * A[t%2][i][j+3][k+2]
            + coef[195] * A[t%2][i][j+3][k+3]
            + coef[196] * A[t%2][i+1][j][k]
            + coef[197] * A[t%2][i+1][j-3][k-3]
            + coef[198] * A[t%2][i+1][j-3][k-2]
            + coef[199] * A[t%2][i+1][j-3][k-1]
            + coef[200] * A[t%2][i+1][j-3][k]
            + coef[201] * A[t%2][i+1][j-3][k+1]
            + coef[202] * A[t%2][i+1][j-3][k+2]
            + coef[203] * A[t%2][i+1][j-3][k+3]
            + coef[204] * A[t%2][i+1][j-2][k-3]
            + coef[205] * A[t%2][i+1][j-2][k-2]
            + coef[206] * A[t%2][i+1][j-2][k-1]
            + coef[207] * A[t%2][i+1][j-2][k]
            + coef[208] * A[t%2][i+1][j-2][k+1]
            + coef[209] * A[t%2][i+1][j-2][k+2]
            + coef[210] * A[t%2][i+1][j-2][k+3]
            + coef[211] * A[t%2][i+1][j-1][k-3]
            + coef[212] * A[t%2][i+1][j-1][k-2]
            + coef[213] * A[t%2][i+1][j-1][k-1]
            + coef[214] * A[t%2][i+1][j-1][k]
            + coef[215] * A[t%2][i+1][j-1][k+1]
            + coef[216] * A[t%2][i+1][j-1][k+2]
            + coef[217] * A[t%2][i+1][j-1][k+3]
            + coef[218] * A[t%2][i+1][j][k-3]
            + coef[219] * A[t%2][i+1][j][k-2]
            + coef[220] * A[t%2][i+1][j][k-1]
            + coef[221] * A[t%2][i+1][j][k+1]
            + coef[222] * A[t%2][i+1][j][k+2]
            + coef[223] * A[t%2][i+1][j][k+3]
            + coef[224] * A[t%2][i+1][j+1][k-3]
            + coef[225] * A[t%2][i+1][j+1][k-2]
            + coef[226] * A[t%2][i+1][j+1][k-1]
            + coef[227] * A[t%2][i+1][j+1][k]
            + coef[228] * A[t%2][i+1][j+1][k+1]
            + coef[229] * A[t%2][i+1][j+1][k+2]
            + coef[230] * A[t%2][i+1][j+1][k+3]
            + coef[231] * A[t%2][i+1][j+2][k-3]
            + coef[232] * A[t%2][i+1][j+2][k-2]
            + coef[233] * A[t%2][i+1][j+2][k-1]
            + coef[234] * A[t%2][i+1][j+2][k]
            + coef[235] * A[t%2][i+1][j+2][k+1]
            + coef[236] * A[t%2][i+1][j+2][k+2]
            + coef[237] * A[t%2][i+1][j+2][k+3]
            + coef[238] * A[t%2][i+1][j+3][k-3]
            + coef[239] * A[t%2][i+1][j+3][k-2]
            + coef[240] * A[t%2][i+1][j+3][k-1]
            + coef[241] * A[t%2][i+1][j+3][k]
            + coef[242] * A[t%2][i+1][j+3][k+1]
            + coef[243] * A[t%2][i+1][j+3][k+2]
            + coef[244] * A[t%2][i+1][j+3][k+3]
            + coef[245] * A[t%2][i+2][j][k]
            + coef[246] * A[t%2][i+2][j-3][k-3]
            + coef[247] * A[t%2][i+2][j-3][k-2]
            + coef[248] * A[t%2][i+2][j-3][k-1]
            + coef[249] * A[t%2][i+2][j-3][k]
            + coef[250] * A[t%2][i+2][j-3][k+1]
            + coef[251] * A[t%2][i+2][j-3][k+2]
            + coef[252] * A[t%2][i+2][j-3][k+3]
            + coef[253] * A[t%2][i+2][j-2][k-3]
            + coef[254] * A[t%2][i+2][j-2][k-2]
            + coef[255] * A[t%2][i+2][j-2][k-1]
            + coef[256] * A[t%2][i+2][j-2][k]
            + coef[257] * A[t%2][i+2][j-2][k+1]
            + coef[258] * A[t%2][i+2][j-2][k+2]
            + coef[259] * A[t%2][i+2][j-2][k+3]
            + coef[260] * A[t%2][i+2][j-1][k-3]
            + coef[261] * A[t%2][i+2][j-1][k-2]
            + coef[262] * A[t%2][i+2][j-1][k-1]
            + coef[263] * A[t%2][i+2][j-1][k]
            + coef[264] * A[t%2][i+2][j-1][k+1]
            + coef[265] * A[t%2][i+2][j-1][k+2]
            + coef[266] * A[t%2][i+2][j-1][k+3]
            + coef[267] * A[t%2][i+2][j][k-3]
            + coef[268] * A[t%2][i+2][j][k-2]
            + coef[269] * A[t%2][i+2][j][k-1]
            + coef[270] * A[t%2][i+2][j][k+1]
            + coef[271] * A[t%2][i+2][j][k+2]
            + coef[272] * A[t%2][i+2][j][k+3]
            + coef[273] * A[t%2][i+2][j+1][k-3]
            + coef[274] * A[t%2][i+2][j+1][k-2]
            + coef[275] * A[t%2][i+2][j+1][k-1]
            + coef[276] * A[t%2][i+2][j+1][k]
            + coef[277] * A[t%2][i+2][j+1][k+1]
            + coef[278] * A[t%2][i+2][j+1][k+2]
            + coef[279] * A[t%2][i+2][j+1][k+3]
            + coef[280] * A[t%2][i+2][j+2][k-3]
            + coef[281] * A[t%2][i+2][j+2][k-2]
            + coef[282] * A[t%2][i+2][j+2][k-1]
            + coef[283] * A[t%2][i+2][j+2][k]
            + coef[284] * A[t%2][i+2][j+2][k+1]
            + coef[285] * A[t%2][i+2][j+2][k+2]
            + coef[286] * A[t%2][i+2][j+2][k+3]
            + coef[287] * A[t%2][i+2][j+3][k-3]
            + coef[288] * A[t%2][i+2][j+3][k-2]
            + coef[289] * A[t%2][i+2][j+3][k-1]
            + coef[290] * A[t%2][i+2][j+3][k]
            + coef[291] * A[t%2][i+2][j+3][k+1]
            + coef[292] * A[t%2][i+2][j+3][k+2]
            + coef[293] * A[t%2][i+2][j+3][k+3]
            + coef[294] * A[t%2][i+3][j][k]
            + coef[295] * A[t%2][i+3][j-3][k-3]
            + coef[296] * A[t%2][i+3][j-3][k-2]
            + coef[297] * A[t%2][i+3][j-3][k-1]
            + coef[298] * A[t%2][i+3][j-3][k]
            + coef[299] * A[t%2][i+3][j-3][k+1]
            + coef[300] * A[t%2][i+3][j-3][k+2]
            + coef[301] * A[t%2][i+3][j-3][k+3]
            + coef[302] * A[t%2][i+3][j-2][k-3]
            + coef[303] * A[t%2][i+3][j-2][k-2]
            + coef[304] * A[t%2][i+3][j-2][k-1]
            + coef[305] * A[t%2][i+3][j-2][k]
            + coef[306] * A[t%2][i+3][j-2][k+1]
            + coef[307] * A[t%2][i+3][j-2][k+2]
            + coef[308] * A[t%2][i+3][j-2][k+3]
            + coef[309] * A[t%2][i+3][j-1][k-3]
            + coef[310] * A[t%2][i+3][j-1][k-2]
            + coef[311] * A[t%2][i+3][j-1][k-1]
            + coef[312] * A[t%2][i+3][j-1][k]
            + coef[313] * A[t%2][i+3][j-1][k+1]
            + coef[314] * A[t%2][i+3][j-1][k+2]
            + coef[315] * A[t%2][i+3][j-1][k+3]
            + coef[316] * A[t%2][i+3][j][k-3]
            + coef[317] * A[t%2][i+3][j][k-2]
            + coef[318] * A[t%2][i+3][j][k-1]
            + coef[319] * A[t%2][i+3][j][k+1]
            + coef[320] * A[t%2][i+3][j][k+2]
            + coef[321] * A[t%2][i+3][j][k+3]
            + coef[322] * A[t%2][i+3][j+1][k-3]
            + coef[323] * A[t%2][i+3][j+1][k-2]
            + coef[324] * A[t%2][i+3][j+1][k-1]
            + coef[325] * A[t%2][i+3][j+1][k]
            + coef[326] * A[t%2][i+3][j+1][k+1]
            + coef[327] * A[t%2][i+3][j+1][k+2]
            + coef[328] * A[t%2][i+3][j+1][k+3]
            + coef[329] * A[t%2][i+3][j+2][k-3]
            + coef[330] * A[t%2][i+3][j+2][k-2]
            + coef[331] * A[t%2][i+3][j+2][k-1]
            + coef[332] * A[t%2][i+3][j+2][k]
            + coef[333] * A[t%2][i+3][j+2][k+1]
            + coef[334] * A[t%2][i+3][j+2][k+2]
            + coef[335] * A[t%2][i+3][j+2][k+3]
            + coef[336] * A[t%2][i+3][j+3][k-3]
            + coef[337] * A[t%2][i+3][j+3][k-2]
            + coef[338] * A[t%2][i+3][j+3][k-1]
            + coef[339] * A[t%2][i+3][j+3][k]
            + coef[340] * A[t%2][i+3][j+3][k+1]
            + coef[341] * A[t%2][i+3][j+3][k+2]
            + coef[342] * A[t%2][i+3][j+3][k+3];
  }
}

void oracle_box3d3r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-3][j][k]
            + coef[1] * A[t%2][i-3][j-3][k-3]
            + coef[2] * A[t%2][i-3][j-3][k-2]
            + coef[3] * A[t%2][i-3][j-3][k-1]
            + coef[4] * A[t%2][i-3][j-3][k]
            + coef[5] * A[t%2][i-3][j-3][k+1]
            + coef[6] * A[t%2][i-3][j-3][k+2]
            + coef[7] * A[t%2][i-3][j-3][k+3]
            + coef[8] * A[t%2][i-3][j-2][k-3]
            + coef[9] * A[t%2][i-3][j-2][k-2]
            + coef[10] * A[t%2][i-3][j-2][k-1]
            + coef[11] * A[t%2][i-3][j-2][k]
            + coef[12] * A[t%2][i-3][j-2][k+1]
            + coef[13] * A[t%2][i-3][j-2][k+2]
            + coef[14] * A[t%2][i-3][j-2][k+3]
            + coef[15] * A[t%2][i-3][j-1][k-3]
            + coef[16] * A[t%2][i-3][j-1][k-2]
            + coef[17] * A[t%2][i-3][j-1][k-1]
            + coef[18] * A[t%2][i-3][j-1][k]
            + coef[19] * A[t%2][i-3][j-1][k+1]
            + coef[20] * A[t%2][i-3][j-1][k+2]
            + coef[21] * A[t%2][i-3][j-1][k+3]
            + coef[22] * A[t%2][i-3][j][k-3]
            + coef[23] * A[t%2][i-3][j][k-2]
            + coef[24] * A[t%2][i-3][j][k-1]
            + coef[25] * A[t%2][i-3][j][k+1]
            + coef[26] * A[t%2][i-3][j][k+2]
            + coef[27] * A[t%2][i-3][j][k+3]
            + coef[28] * A[t%2][i-3][j+1][k-3]
            + coef[29] * A[t%2][i-3][j+1][k-2]
            + coef[30] * A[t%2][i-3][j+1][k-1]
            + coef[31] * A[t%2][i-3][j+1][k]
            + coef[32] * A[t%2][i-3][j+1][k+1]
            + coef[33] * A[t%2][i-3][j+1][k+2]
            + coef[34] * A[t%2][i-3][j+1][k+3]
            + coef[35] * A[t%2][i-3][j+2][k-3]
            + coef[36] * A[t%2][i-3][j+2][k-2]
            + coef[37] * A[t%2][i-3][j+2][k-1]
            + coef[38] * A[t%2][i-3][j+2][k]
            + coef[39] * A[t%2][i-3][j+2][k+1]
            + coef[40] * A[t%2][i-3][j+2][k+2]
            + coef[41] * A[t%2][i-3][j+2][k+3]
            + coef[42] * A[t%2][i-3][j+3][k-3]
            + coef[43] * A[t%2][i-3][j+3][k-2]
            + coef[44] * A[t%2][i-3][j+3][k-1]
            + coef[45] * A[t%2][i-3][j+3][k]
            + coef[46] * A[t%2][i-3][j+3][k+1]
            + coef[47] * A[t%2][i-3][j+3][k+2]
            + coef[48] * A[t%2][i-3][j+3][k+3]
            + coef[49] * A[t%2][i-2][j][k]
            + coef[50] * A[t%2][i-2][j-3][k-3]
            + coef[51] * A[t%2][i-2][j-3][k-2]
            + coef[52] * A[t%2][i-2][j-3][k-1]
            + coef[53] * A[t%2][i-2][j-3][k]
            + coef[54] * A[t%2][i-2][j-3][k+1]
            + coef[55] * A[t%2][i-2][j-3][k+2]
            + coef[56] * A[t%2][i-2][j-3][k+3]
            + coef[57] * A[t%2][i-2][j-2][k-3]
            + coef[58] * A[t%2][i-2][j-2][k-2]
            + coef[59] * A[t%2][i-2][j-2][k-1]
            + coef[60] * A[t%2][i-2][j-2][k]
            + coef[61] * A[t%2][i-2][j-2][k+1]
            + coef[62] * A[t%2][i-2][j-2][k+2]
            + coef[63] * A[t%2][i-2][j-2][k+3]
            + coef[64] * A[t%2][i-2][j-1][k-3]
            + coef[65] * A[t%2][i-2][j-1][k-2]
            + coef[66] * A[t%2][i-2][j-1][k-1]
            + coef[67] * A[t%2][i-2][j-1][k]
            + coef[68] * A[t%2][i-2][j-1][k+1]
            + coef[69] * A[t%2][i-2][j-1][k+2]
            + coef[70] * A[t%2][i-2][j-1][k+3]
            + coef[71] * A[t%2][i-2][j][k-3]
            + coef[72] * A[t%2][i-2][j][k-2]
            + coef[73] * A[t%2][i-2][j][k-1]
            + coef[74] * A[t%2][i-2][j][k+1]
            + coef[75] * A[t%2][i-2][j][k+2]
            + coef[76] * A[t%2][i-2][j][k+3]
            + coef[77] * A[t%2][i-2][j+1][k-3]
            + coef[78] * A[t%2][i-2][j+1][k-2]
            + coef[79] * A[t%2][i-2][j+1][k-1]
            + coef[80] * A[t%2][i-2][j+1][k]
            + coef[81] * A[t%2][i-2][j+1][k+1]
            + coef[82] * A[t%2][i-2][j+1][k+2]
            + coef[83] * A[t%2][i-2][j+1][k+3]
            + coef[84] * A[t%2][i-2][j+2][k-3]
            + coef[85] * A[t%2][i-2][j+2][k-2]
            + coef[86] * A[t%2][i-2][j+2][k-1]
            + coef[87] * A[t%2][i-2][j+2][k]
            + coef[88] * A[t%2][i-2][j+2][k+1]
            + coef[89] * A[t%2][i-2][j+2][k+2]
            + coef[90] * A[t%2][i-2][j+2][k+3]
            + coef[91] * A[t%2][i-2][j+3][k-3]
            + coef[92] * A[t%2][i-2][j+3][k-2]
            + coef[93] * A[t%2][i-2][j+3][k-1]
            + coef[94] * A[t%2][i-2][j+3][k]
            + coef[95] * A[t%2][i-2][j+3][k+1]
            + coef[96] * A[t%2][i-2][j+3][k+2]
            + coef[97] * A[t%2][i-2][j+3][k+3]
            + coef[98] * A[t%2][i-1][j][k]
            + coef[99] * A[t%2][i-1][j-3][k-3]
            + coef[100] * A[t%2][i-1][j-3][k-2]
            + coef[101] * A[t%2][i-1][j-3][k-1]
            + coef[102] * A[t%2][i-1][j-3][k]
            + coef[103] * A[t%2][i-1][j-3][k+1]
            + coef[104] * A[t%2][i-1][j-3][k+2]
            + coef[105] * A[t%2][i-1][j-3][k+3]
            + coef[106] * A[t%2][i-1][j-2][k-3]
            + coef[107] * A[t%2][i-1][j-2][k-2]
            + coef[108] * A[t%2][i-1][j-2][k-1]
            + coef[109] * A[t%2][i-1][j-2][k]
            + coef[110] * A[t%2][i-1][j-2][k+1]
            + coef[111] * A[t%2][i-1][j-2][k+2]
            + coef[112] * A[t%2][i-1][j-2][k+3]
            + coef[113] * A[t%2][i-1][j-1][k-3]
            + coef[114] * A[t%2][i-1][j-1][k-2]
            + coef[115] * A[t%2][i-1][j-1][k-1]
            + coef[116] * A[t%2][i-1][j-1][k]
            + coef[117] * A[t%2][i-1][j-1][k+1]
            + coef[118] * A[t%2][i-1][j-1][k+2]
            + coef[119] * A[t%2][i-1][j-1][k+3]
            + coef[120] * A[t%2][i-1][j][k-3]
            + coef[121] * A[t%2][i-1][j][k-2]
            + coef[122] * A[t%2][i-1][j][k-1]
            + coef[123] * A[t%2][i-1][j][k+1]
            + coef[124] * A[t%2][i-1][j][k+2]
            + coef[125] * A[t%2][i-1][j][k+3]
            + coef[126] * A[t%2][i-1][j+1][k-3]
            + coef[127] * A[t%2][i-1][j+1][k-2]
            + coef[128] * A[t%2][i-1][j+1][k-1]
            + coef[129] * A[t%2][i-1][j+1][k]
            + coef[130] * A[t%2][i-1][j+1][k+1]
            + coef[131] * A[t%2][i-1][j+1][k+2]
            + coef[132] * A[t%2][i-1][j+1][k+3]
            + coef[133] * A[t%2][i-1][j+2][k-3]
            + coef[134] * A[t%2][i-1][j+2][k-2]
            + coef[135] * A[t%2][i-1][j+2][k-1]
            + coef[136] * A[t%2][i-1][j+2][k]
            + coef[137] * A[t%2][i-1][j+2][k+1]
            + coef[138] * A[t%2][i-1][j+2][k+2]
            + coef[139] * A[t%2][i-1][j+2][k+3]
            + coef[140] * A[t%2][i-1][j+3][k-3]
            + coef[141] * A[t%2][i-1][j+3][k-2]
            + coef[142] * A[t%2][i-1][j+3][k-1]
            + coef[143] * A[t%2][i-1][j+3][k]
            + coef[144] * A[t%2][i-1][j+3][k+1]
            + coef[145] * A[t%2][i-1][j+3][k+2]
            + coef[146] * A[t%2][i-1][j+3][k+3]
            + coef[147] * A[t%2][i][j][k]
            + coef[148] * A[t%2][i][j-3][k-3]
            + coef[149] * A[t%2][i][j-3][k-2]
            + coef[150] * A[t%2][i][j-3][k-1]
            + coef[151] * A[t%2][i][j-3][k]
            + coef[152] * A[t%2][i][j-3][k+1]
            + coef[153] * A[t%2][i][j-3][k+2]
            + coef[154] * A[t%2][i][j-3][k+3]
            + coef[155] * A[t%2][i][j-2][k-3]
            + coef[156] * A[t%2][i][j-2][k-2]
            + coef[157] * A[t%2][i][j-2][k-1]
            + coef[158] * A[t%2][i][j-2][k]
            + coef[159] * A[t%2][i][j-2][k+1]
            + coef[160] * A[t%2][i][j-2][k+2]
            + coef[161] * A[t%2][i][j-2][k+3]
            + coef[162] * A[t%2][i][j-1][k-3]
            + coef[163] * A[t%2][i][j-1][k-2]
            + coef[164] * A[t%2][i][j-1][k-1]
            + coef[165] * A[t%2][i][j-1][k]
            + coef[166] * A[t%2][i][j-1][k+1]
            + coef[167] * A[t%2][i][j-1][k+2]
            + coef[168] * A[t%2][i][j-1][k+3]
            + coef[169] * A[t%2][i][j][k-3]
            + coef[170] * A[t%2][i][j][k-2]
            + coef[171] * A[t%2][i][j][k-1]
            + coef[172] * A[t%2][i][j][k+1]
            + coef[173] * A[t%2][i][j][k+2]
            + coef[174] * A[t%2][i][j][k+3]
            + coef[175] * A[t%2][i][j+1][k-3]
            + coef[176] * A[t%2][i][j+1][k-2]
            + coef[177] * A[t%2][i][j+1][k-1]
            + coef[178] * A[t%2][i][j+1][k]
            + coef[179] * A[t%2][i][j+1][k+1]
            + coef[180] * A[t%2][i][j+1][k+2]
            + coef[181] * A[t%2][i][j+1][k+3]
            + coef[182] * A[t%2][i][j+2][k-3]
            + coef[183] * A[t%2][i][j+2][k-2]
            + coef[184] * A[t%2][i][j+2][k-1]
            + coef[185] * A[t%2][i][j+2][k]
            + coef[186] * A[t%2][i][j+2][k+1]
            + coef[187] * A[t%2][i][j+2][k+2]
            + coef[188] * A[t%2][i][j+2][k+3]
            + coef[189] * A[t%2][i][j+3][k-3]
            + coef[190] * A[t%2][i][j+3][k-2]
            + coef[191] * A[t%2][i][j+3][k-1]
            + coef[192] * A[t%2][i][j+3][k]
            + coef[193] * A[t%2][i][j+3][k+1]
            + coef[194] * A[t%2][i][j+3][k+2]
            + coef[195] * A[t%2][i][j+3][k+3]
            + coef[196] * A[t%2][i+1][j][k]
            + coef[197] * A[t%2][i+1][j-3][k-3]
            + coef[198] * A[t%2][i+1][j-3][k-2]
            + coef[199] * A[t%2][i+1][j-3][k-1]
            + coef[200] * A[t%2][i+1][j-3][k]
            + coef[201] * A[t%2][i+1][j-3][k+1]
            + coef[202] * A[t%2][i+1][j-3][k+2]
            + coef[203] * A[t%2][i+1][j-3][k+3]
            + coef[204] * A[t%2][i+1][j-2][k-3]
            + coef[205] * A[t%2][i+1][j-2][k-2]
            + coef[206] * A[t%2][i+1][j-2][k-1]
            + coef[207] * A[t%2][i+1][j-2][k]
            + coef[208] * A[t%2][i+1][j-2][k+1]
            + coef[209] * A[t%2][i+1][j-2][k+2]
            + coef[210] * A[t%2][i+1][j-2][k+3]
            + coef[211] * A[t%2][i+1][j-1][k-3]
            + coef[212] * A[t%2][i+1][j-1][k-2]
            + coef[213] * A[t%2][i+1][j-1][k-1]
            + coef[214] * A[t%2][i+1][j-1][k]
            + coef[215] * A[t%2][i+1][j-1][k+1]
            + coef[216] * A[t%2][i+1][j-1][k+2]
            + coef[217] * A[t%2][i+1][j-1][k+3]
            + coef[218] * A[t%2][i+1][j][k-3]
            + coef[219] * A[t%2][i+1][j][k-2]
            + coef[220] * A[t%2][i+1][j][k-1]
            + coef[221] * A[t%2][i+1][j][k+1]
            + coef[222] * A[t%2][i+1][j][k+2]
            + coef[223] * A[t%2][i+1][j][k+3]
            + coef[224] * A[t%2][i+1][j+1][k-3]
            + coef[225] * A[t%2][i+1][j+1][k-2]
            + coef[226] * A[t%2][i+1][j+1][k-1]
            + coef[227] * A[t%2][i+1][j+1][k]
            + coef[228] * A[t%2][i+1][j+1][k+1]
            + coef[229] * A[t%2][i+1][j+1][k+2]
            + coef[230] * A[t%2][i+1][j+1][k+3]
            + coef[231] * A[t%2][i+1][j+2][k-3]
            + coef[232] * A[t%2][i+1][j+2][k-2]
            + coef[233] * A[t%2][i+1][j+2][k-1]
            + coef[234] * A[t%2][i+1][j+2][k]
            + coef[235] * A[t%2][i+1][j+2][k+1]
            + coef[236] * A[t%2][i+1][j+2][k+2]
            + coef[237] * A[t%2][i+1][j+2][k+3]
            + coef[238] * A[t%2][i+1][j+3][k-3]
            + coef[239] * A[t%2][i+1][j+3][k-2]
            + coef[240] * A[t%2][i+1][j+3][k-1]
            + coef[241] * A[t%2][i+1][j+3][k]
            + coef[242] * A[t%2][i+1][j+3][k+1]
            + coef[243] * A[t%2][i+1][j+3][k+2]
            + coef[244] * A[t%2][i+1][j+3][k+3]
            + coef[245] * A[t%2][i+2][j][k]
            + coef[246] * A[t%2][i+2][j-3][k-3]
            + coef[247] * A[t%2][i+2][j-3][k-2]
            + coef[248] * A[t%2][i+2][j-3][k-1]
            + coef[249] * A[t%2][i+2][j-3][k]
            + coef[250] * A[t%2][i+2][j-3][k+1]
            + coef[251] * A[t%2][i+2][j-3][k+2]
            + coef[252] * A[t%2][i+2][j-3][k+3]
            + coef[253] * A[t%2][i+2][j-2][k-3]
            + coef[254] * A[t%2][i+2][j-2][k-2]
            + coef[255] * A[t%2][i+2][j-2][k-1]
            + coef[256] * A[t%2][i+2][j-2][k]
            + coef[257] * A[t%2][i+2][j-2][k+1]
            + coef[258] * A[t%2][i+2][j-2][k+2]
            + coef[259] * A[t%2][i+2][j-2][k+3]
            + coef[260] * A[t%2][i+2][j-1][k-3]
            + coef[261] * A[t%2][i+2][j-1][k-2]
            + coef[262] * A[t%2][i+2][j-1][k-1]
            + coef[263] * A[t%2][i+2][j-1][k]
            + coef[264] * A[t%2][i+2][j-1][k+1]
            + coef[265] * A[t%2][i+2][j-1][k+2]
            + coef[266] * A[t%2][i+2][j-1][k+3]
            + coef[267] * A[t%2][i+2][j][k-3]
            + coef[268] * A[t%2][i+2][j][k-2]
            + coef[269] * A[t%2][i+2][j][k-1]
            + coef[270] * A[t%2][i+2][j][k+1]
            + coef[271] * A[t%2][i+2][j][k+2]
            + coef[272] * A[t%2][i+2][j][k+3]
            + coef[273] * A[t%2][i+2][j+1][k-3]
            + coef[274] * A[t%2][i+2][j+1][k-2]
            + coef[275] * A[t%2][i+2][j+1][k-1]
            + coef[276] * A[t%2][i+2][j+1][k]
            + coef[277] * A[t%2][i+2][j+1][k+1]
            + coef[278] * A[t%2][i+2][j+1][k+2]
            + coef[279] * A[t%2][i+2][j+1][k+3]
            + coef[280] * A[t%2][i+2][j+2][k-3]
            + coef[281] * A[t%2][i+2][j+2][k-2]
            + coef[282] * A[t%2][i+2][j+2][k-1]
            + coef[283] * A[t%2][i+2][j+2][k]
            + coef[284] * A[t%2][i+2][j+2][k+1]
            + coef[285] * A[t%2][i+2][j+2][k+2]
            + coef[286] * A[t%2][i+2][j+2][k+3]
            + coef[287] * A[t%2][i+2][j+3][k-3]
            + coef[288] * A[t%2][i+2][j+3][k-2]
            + coef[289] * A[t%2][i+2][j+3][k-1]
            + coef[290] * A[t%2][i+2][j+3][k]
            + coef[291] * A[t%2][i+2][j+3][k+1]
            + coef[292] * A[t%2][i+2][j+3][k+2]
            + coef[293] * A[t%2][i+2][j+3][k+3]
            + coef[294] * A[t%2][i+3][j][k]
            + coef[295] * A[t%2][i+3][j-3][k-3]
            + coef[296] * A[t%2][i+3][j-3][k-2]
            + coef[297] * A[t%2][i+3][j-3][k-1]
            + coef[298] * A[t%2][i+3][j-3][k]
            + coef[299] * A[t%2][i+3][j-3][k+1]
            + coef[300] * A[t%2][i+3][j-3][k+2]
            + coef[301] * A[t%2][i+3][j-3][k+3]
            + coef[302] * A[t%2][i+3][j-2][k-3]
            + coef[303] * A[t%2][i+3][j-2][k-2]
            + coef[304] * A[t%2][i+3][j-2][k-1]
            + coef[305] * A[t%2][i+3][j-2][k]
            + coef[306] * A[t%2][i+3][j-2][k+1]
            + coef[307] * A[t%2][i+3][j-2][k+2]
            + coef[308] * A[t%2][i+3][j-2][k+3]
            + coef[309] * A[t%2][i+3][j-1][k-3]
            + coef[310] * A[t%2][i+3][j-1][k-2]
            + coef[311] * A[t%2][i+3][j-1][k-1]
            + coef[312] * A[t%2][i+3][j-1][k]
            + coef[313] * A[t%2][i+3][j-1][k+1]
            + coef[314] * A[t%2][i+3][j-1][k+2]
            + coef[315] * A[t%2][i+3][j-1][k+3]
            + coef[316] * A[t%2][i+3][j][k-3]
            + coef[317] * A[t%2][i+3][j][k-2]
            + coef[318] * A[t%2][i+3][j][k-1]
            + coef[319] * A[t%2][i+3][j][k+1]
            + coef[320] * A[t%2][i+3][j][k+2]
            + coef[321] * A[t%2][i+3][j][k+3]
            + coef[322] * A[t%2][i+3][j+1][k-3]
            + coef[323] * A[t%2][i+3][j+1][k-2]
            + coef[324] * A[t%2][i+3][j+1][k-1]
            + coef[325] * A[t%2][i+3][j+1][k]
            + coef[326] * A[t%2][i+3][j+1][k+1]
            + coef[327] * A[t%2][i+3][j+1][k+2]
            + coef[328] * A[t%2][i+3][j+1][k+3]
            + coef[329] * A[t%2][i+3][j+2][k-3]
            + coef[330] * A[t%2][i+3][j+2][k-2]
            + coef[331] * A[t%2][i+3][j+2][k-1]
            + coef[332] * A[t%2][i+3][j+2][k]
            + coef[333] * A[t%2][i+3][j+2][k+1]
            + coef[334] * A[t%2][i+3][j+2][k+2]
            + coef[335] * A[t%2][i+3][j+2][k+3]
            + coef[336] * A[t%2][i+3][j+3][k-3]
            + coef[337] * A[t%2][i+3][j+3][k-2]
            + coef[338] * A[t%2][i+3][j+3][k-1]
            + coef[339] * A[t%2][i+3][j+3][k]
            + coef[340] * A[t%2][i+3][j+3][k+1]
            + coef[341] * A[t%2][i+3][j+3][k+2]
            + coef[342] * A[t%2][i+3][j+3][k+3];
  }
}

void oracle_box3d3r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 6, d1 = n[1] + 6, d2 = n[2] + 6;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 3; i < d0 - 3; i++)
      for (long j = 3; j < d1 - 3; j++)
        for (long k = 3; k < d2 - 3; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-3][j][k]
            + coef[1] * A[t%2][i-3][j-3][k-3]
            + coef[2] * A[t%2][i-3][j-3][k-2]
            + coef[3] * A[t%2][i-3][j-3][k-1]
            + coef[4] * A[t%2][i-3][j-3][k]
            + coef[5] * A[t%2][i-3][j-3][k+1]
            + coef[6] * A[t%2][i-3][j-3][k+2]
            + coef[7] * A[t%2][i-3][j-3][k+3]
            + coef[8] * A[t%2][i-3][j-2][k-3]
            + coef[9] * A[t%2][i-3][j-2][k-2]
            + coef[10] * A[t%2][i-3][j-2][k-1]
            + coef[11] * A[t%2][i-3][j-2][k]
            + coef[12] * A[t%2][i-3][j-2][k+1]
            + coef[13] * A[t%2][i-3][j-2][k+2]
            + coef[14] * A[t%2][i-3][j-2][k+3]
            + coef[15] * A[t%2][i-3][j-1][k-3]
            + coef[16] * A[t%2][i-3][j-1][k-2]
            + coef[17] * A[t%2][i-3][j-1][k-1]
            + coef[18] * A[t%2][i-3][j-1][k]
            + coef[19] * A[t%2][i-3][j-1][k+1]
            + coef[20] * A[t%2][i-3][j-1][k+2]
            + coef[21] * A[t%2][i-3][j-1][k+3]
            + coef[22] * A[t%2][i-3][j][k-3]
            + coef[23] * A[t%2][i-3][j][k-2]
            + coef[24] * A[t%2][i-3][j][k-1]
            + coef[25] * A[t%2][i-3][j][k+1]
            + coef[26] * A[t%2][i-3][j][k+2]
            + coef[27] * A[t%2][i-3][j][k+3]
            + coef[28] * A[t%2][i-3][j+1][k-3]
            + coef[29] * A[t%2][i-3][j+1][k-2]
            + coef[30] * A[t%2][i-3][j+1][k-1]
            + coef[31] * A[t%2][i-3][j+1][k]
            + coef[32] * A[t%2][i-3][j+1][k+1]
            + coef[33] * A[t%2][i-3][j+1][k+2]
            + coef[34] * A[t%2][i-3][j+1][k+3]
            + coef[35] * A[t%2][i-3][j+2][k-3]
            + coef[36] * A[t%2][i-3][j+2][k-2]
            + coef[37] * A[t%2][i-3][j+2][k-1]
            + coef[38] * A[t%2][i-3][j+2][k]
            + coef[39] * A[t%2][i-3][j+2][k+1]
            + coef[40] * A[t%2][i-3][j+2][k+2]
            + coef[41] * A[t%2][i-3][j+2][k+3]
            + coef[42] * A[t%2][i-3][j+3][k-3]
            + coef[43] * A[t%2][i-3][j+3][k-2]
            + coef[44] * A[t%2][i-3][j+3][k-1]
            + coef[45] * A[t%2][i-3][j+3][k]
            + coef[46] * A[t%2][i-3][j+3][k+1]
            + coef[47] * A[t%2][i-3][j+3][k+2]
            + coef[48] * A[t%2][i-3][j+3][k+3]
            + coef[49] * A[t%2][i-2][j][k]
            + coef[50] * A[t%2][i-2][j-3][k-3]
            + coef[51] * A[t%2][i-2][j-3][k-2]
            + coef[52] * A[t%2][i-2][j-3][k-1]
            + coef[53] * A[t%2][i-2][j-3][k]
            + coef[54] * A[t%2][i-2][j-3][k+1]
            + coef[55] * A[t%2][i-2][j-3][k+2]
            + coef[56] * A[t%2][i-2][j-3][k+3]
            + coef[57] * A[t%2][i-2][j-2][k-3]
            + coef[58] * A[t%2][i-2][j-2][k-2]
            + coef[59] * A[t%2][i-2][j-2][k-1]
            + coef[60] * A[t%2][i-2][j-2][k]
            + coef[61] * A[t%2][i-2][j-2][k+1]
            + coef[62] * A[t%2][i-2][j-2][k+2]
            + coef[63] * A[t%2][i-2][j-2][k+3]
            + coef[64] * A[t%2][i-2][j-1][k-3]
            + coef[65] * A[t%2][i-2][j-1][k-2]
            + coef[66] * A[t%2][i-2][j-1][k-1]
            + coef[67] * A[t%2][i-2][j-1][k]
            + coef[68] * A[t%2][i-2][j-1][k+1]
            + coef[69] * A[t%2][i-2][j-1][k+2]
            + coef[70] * A[t%2][i-2][j-1][k+3]
            + coef[71] * A[t%2][i-2][j][k-3]
            + coef[72] * A[t%2][i-2][j][k-2]
            + coef[73] * A[t%2][i-2][j][k-1]
            + coef[74] * A[t%2][i-2][j][k+1]
            + coef[75] * A[t%2][i-2][j][k+2]
            + coef[76] * A[t%2][i-2][j][k+3]
            + coef[77] * A[t%2][i-2][j+1][k-3]
            + coef[78] * A[t%2][i-2][j+1][k-2]
            + coef[79] * A[t%2][i-2][j+1][k-1]
            + coef[80] * A[t%2][i-2][j+1][k]
            + coef[81] * A[t%2][i-2][j+1][k+1]
            + coef[82] * A[t%2][i-2][j+1][k+2]
            + coef[83] * A[t%2][i-2][j+1][k+3]
            + coef[84] * A[t%2][i-2][j+2][k-3]
            + coef[85] * A[t%2][i-2][j+2][k-2]
            + coef[86] * A[t%2][i-2][j+2][k-1]
            + coef[87] * A[t%2][i-2][j+2][k]
            + coef[88] * A[t%2][i-2][j+2][k+1]
            + coef[89] * A[t%2][i-2][j+2][k+2]
            + coef[90] * A[t%2][i-2][j+2][k+3]
            + coef[91] * A[t%2][i-2][j+3][k-3]
            + coef[92] * A[t%2][i-2][j+3][k-2]
            + coef[93] * A[t%2][i-2][j+3][k-1]
            + coef[94] * A[t%2][i-2][j+3][k]
            + coef[95] * A[t%2][i-2][j+3][k+1]
            + coef[96] * A[t%2][i-2][j+3][k+2]
            + coef[97] * A[t%2][i-2][j+3][k+3]
            + coef[98] * A[t%2][i-1][j][k]
            + coef[99] * A[t%2][i-1][j-3][k-3]
            + coef[100] * A[t%2][i-1][j-3][k-2]
            + coef[101] * A[t%2][i-1][j-3][k-1]
            + coef[102] * A[t%2][i-1][j-3][k]
            + coef[103] * A[t%2][i-1][j-3][k+1]
            + coef[104] * A[t%2][i-1][j-3][k+2]
            + coef[105] * A[t%2][i-1][j-3][k+3]
            + coef[106] * A[t%2][i-1][j-2][k-3]
            + coef[107] * A[t%2][i-1][j-2][k-2]
            + coef[108] * A[t%2][i-1][j-2][k-1]
            + coef[109] * A[t%2][i-1][j-2][k]
            + coef[110] * A[t%2][i-1][j-2][k+1]
            + coef[111] * A[t%2][i-1][j-2][k+2]
            + coef[112] * A[t%2][i-1][j-2][k+3]
            + coef[113] * A[t%2][i-1][j-1][k-3]
            + coef[114] * A[t%2][i-1][j-1][k-2]
            + coef[115] * A[t%2][i-1][j-1][k-1]
            + coef[116] * A[t%2][i-1][j-1][k]
            + coef[117] * A[t%2][i-1][j-1][k+1]
            + coef[118] * A[t%2][i-1][j-1][k+2]
            + coef[119] * A[t%2][i-1][j-1][k+3]
            + coef[120] * A[t%2][i-1][j][k-3]
            + coef[121] * A[t%2][i-1][j][k-2]
            + coef[122] * A[t%2][i-1][j][k-1]
            + coef[123] * A[t%2][i-1][j][k+1]
            + coef[124] * A[t%2][i-1][j][k+2]
            + coef[125] * A[t%2][i-1][j][k+3]
            + coef[126] * A[t%2][i-1][j+1][k-3]
            + coef[127] * A[t%2][i-1][j+1][k-2]
            + coef[128] * A[t%2][i-1][j+1][k-1]
            + coef[129] * A[t%2][i-1][j+1][k]
            + coef[130] * A[t%2][i-1][j+1][k+1]
            + coef[131] * A[t%2][i-1][j+1][k+2]
            + coef[132] * A[t%2][i-1][j+1][k+3]
            + coef[133] * A[t%2][i-1][j+2][k-3]
            + coef[134] * A[t%2][i-1][j+2][k-2]
            + coef[135] * A[t%2][i-1][j+2][k-1]
            + coef[136] * A[t%2][i-1][j+2][k]
            + coef[137] * A[t%2][i-1][j+2][k+1]
            + coef[138] * A[t%2][i-1][j+2][k+2]
            + coef[139] * A[t%2][i-1][j+2][k+3]
            + coef[140] * A[t%2][i-1][j+3][k-3]
            + coef[141] * A[t%2][i-1][j+3][k-2]
            + coef[142] * A[t%2][i-1][j+3][k-1]
            + coef[143] * A[t%2][i-1][j+3][k]
            + coef[144] * A[t%2][i-1][j+3][k+1]
            + coef[145] * A[t%2][i-1][j+3][k+2]
            + coef[146] * A[t%2][i-1][j+3][k+3]
            + coef[147] * A[t%2][i][j][k]
            + coef[148] * A[t%2][i][j-3][k-3]
            + coef[149] * A[t%2][i][j-3][k-2]
            + coef[150] * A[t%2][i][j-3][k-1]
            + coef[151] * A[t%2][i][j-3][k]
            + coef[152] * A[t%2][i][j-3][k+1]
            + coef[153] * A[t%2][i][j-3][k+2]
            + coef[154] * A[t%2][i][j-3][k+3]
            + coef[155] * A[t%2][i][j-2][k-3]
            + coef[156] * A[t%2][i][j-2][k-2]
            + coef[157] * A[t%2][i][j-2][k-1]
            + coef[158] * A[t%2][i][j-2][k]
            + coef[159] * A[t%2][i][j-2][k+1]
            + coef[160] * A[t%2][i][j-2][k+2]
            + coef[161] * A[t%2][i][j-2][k+3]
            + coef[162] * A[t%2][i][j-1][k-3]
            + coef[163] * A[t%2][i][j-1][k-2]
            + coef[164] * A[t%2][i][j-1][k-1]
            + coef[165] * A[t%2][i][j-1][k]
            + coef[166] * A[t%2][i][j-1][k+1]
            + coef[167] * A[t%2][i][j-1][k+2]
            + coef[168] * A[t%2][i][j-1][k+3]
            + coef[169] * A[t%2][i][j][k-3]
            + coef[170] * A[t%2][i][j][k-2]
            + coef[171] * A[t%2][i][j][k-1]
            + coef[172] * A[t%2][i][j][k+1]
            + coef[173] * A[t%2][i][j][k+2]
            + coef[174] * A[t%2][i][j][k+3]
            + coef[175] * A[t%2][i][j+1][k-3]
            + coef[176] * A[t%2][i][j+1][k-2]
            + coef[177] * A[t%2][i][j+1][k-1]
            + coef[178] * A[t%2][i][j+1][k]
            + coef[179] * A[t%2][i][j+1][k+1]
            + coef[180] * A[t%2][i][j+1][k+2]
            + coef[181] * A[t%2][i][j+1][k+3]
            + coef[182] * A[t%2][i][j+2][k-3]
            + coef[183] * A[t%2][i][j+2][k-2]
            + coef[184] * A[t%2][i][j+2][k-1]
            + coef[185] * A[t%2][i][j+2][k]
            + coef[186] * A[t%2][i][j+2][k+1]
            + coef[187] * A[t%2][i][j+2][k+2]
            + coef[188] * A[t%2][i][j+2][k+3]
            + coef[189] * A[t%2][i][j+3][k-3]
            + coef[190] * A[t%2][i][j+3][k-2]
            + coef[191] * A[t%2][i][j+3][k-1]
            + coef[192] * A[t%2][i][j+3][k]
            + coef[193] * A[t%2][i][j+3][k+1]
            + coef[194] * A[t%2][i][j+3][k+2]
            + coef[195] * A[t%2][i][j+3][k+3]
            + coef[196] * A[t%2][i+1][j][k]
            + coef[197] * A[t%2][i+1][j-3][k-3]
            + coef[198] * A[t%2][i+1][j-3][k-2]
            + coef[199] * A[t%2][i+1][j-3][k-1]
            + coef[200] * A[t%2][i+1][j-3][k]
            + coef[201] * A[t%2][i+1][j-3][k+1]
            + coef[202] * A[t%2][i+1][j-3][k+2]
            + coef[203] * A[t%2][i+1][j-3][k+3]
            + coef[204] * A[t%2][i+1][j-2][k-3]
            + coef[205] * A[t%2][i+1][j-2][k-2]
            + coef[206] * A[t%2][i+1][j-2][k-1]
            + coef[207] * A[t%2][i+1][j-2][k]
            + coef[208] * A[t%2][i+1][j-2][k+1]
            + coef[209] * A[t%2][i+1][j-2][k+2]
            + coef[210] * A[t%2][i+1][j-2][k+3]
            + coef[211] * A[t%2][i+1][j-1][k-3]
            + coef[212] * A[t%2][i+1][j-1][k-2]
            + coef[213] * A[t%2][i+1][j-1][k-1]
            + coef[214] * A[t%2][i+1][j-1][k]
            + coef[215] * A[t%2][i+1][j-1][k+1]
            + coef[216] * A[t%2][i+1][j-1][k+2]
            + coef[217] * A[t%2][i+1][j-1][k+3]
            + coef[218] * A[t%2][i+1][j][k-3]
            + coef[219] * A[t%2][i+1][j][k-2]
            + coef[220] * A[t%2][i+1][j][k-1]
            + coef[221] * A[t%2][i+1][j][k+1]
            + coef[222] * A[t%2][i+1][j][k+2]
            + coef[223] * A[t%2][i+1][j][k+3]
            + coef[224] * A[t%2][i+1][j+1][k-3]
            + coef[225] * A[t%2][i+1][j+1][k-2]
            + coef[226] * A[t%2][i+1][j+1][k-1]
            + coef[227] * A[t%2][i+1][j+1][k]
            + coef[228] * A[t%2][i+1][j+1][k+1]
            + coef[229] * A[t%2][i+1][j+1][k+2]
            + coef[230] * A[t%2][i+1][j+1][k+3]
            + coef[231] * A[t%2][i+1][j+2][k-3]
            + coef[232] * A[t%2][i+1][j+2][k-2]
            + coef[233] * A[t%2][i+1][j+2][k-1]
            + coef[234] * A[t%2][i+1][j+2][k]
            + coef[235] * A[t%2][i+1][j+2][k+1]
            + coef[236] * A[t%2][i+1][j+2][k+2]
            + coef[237] * A[t%2][i+1][j+2][k+3]
            + coef[238] * A[t%2][i+1][j+3][k-3]
            + coef[239] * A[t%2][i+1][j+3][k-2]
            + coef[240] * A[t%2][i+1][j+3][k-1]
            + coef[241] * A[t%2][i+1][j+3][k]
            + coef[242] * A[t%2][i+1][j+3][k+1]
            + coef[243] * A[t%2][i+1][j+3][k+2]
            + coef[244] * A[t%2][i+1][j+3][k+3]
            + coef[245] * A[t%2][i+2][j][k]
            + coef[246] * A[t%2][i+2][j-3][k-3]
            + coef[247] * A[t%2][i+2][j-3][k-2]
            + coef[248] * A[t%2][i+2][j-3][k-1]
            + coef[249] * A[t%2][i+2][j-3][k]
            + coef[250] * A[t%2][i+2][j-3][k+1]
            + coef[251] * A[t%2][i+2][j-3][k+2]
            + coef[252] * A[t%2][i+2][j-3][k+3]
            + coef[253] * A[t%2][i+2][j-2][k-3]
            + coef[254] * A[t%2][i+2][j-2][k-2]
            + coef[255] * A[t%2][i+2][j-2][k-1]
            + coef[256] * A[t%2][i+2][j-2][k]
            + coef[257] * A[t%2][i+2][j-2][k+1]
            + coef[258] * A[t%2][i+2][j-2][k+2]
            + coef[259] * A[t%2][i+2][j-2][k+3]
            + coef[260] * A[t%2][i+2][j-1][k-3]
            + coef[261] * A[t%2][i+2][j-1][k-2]
            + coef[262] * A[t%2][i+2][j-1][k-1]
            + coef[263] * A[t%2][i+2][j-1][k]
            + coef[264] * A[t%2][i+2][j-1][k+1]
            + coef[265] * A[t%2][i+2][j-1][k+2]
            + coef[266] * A[t%2][i+2][j-1][k+3]
            + coef[267] * A[t%2][i+2][j][k-3]
            + coef[268] * A[t%2][i+2][j][k-2]
            + coef[269] * A[t%2][i+2][j][k-1]
            + coef[270] * A[t%2][i+2][j][k+1]
            + coef[271] * A[t%2][i+2][j][k+2]
            + coef[272] * A[t%2][i+2][j][k+3]
            + coef[273] * A[t%2][i+2][j+1][k-3]
            + coef[274] * A[t%2][i+2][j+1][k-2]
            + coef[275] * A[t%2][i+2][j+1][k-1]
            + coef[276] * A[t%2][i+2][j+1][k]
            + coef[277] * A[t%2][i+2][j+1][k+1]
            + coef[278] * A[t%2][i+2][j+1][k+2]
            + coef[279] * A[t%2][i+2][j+1][k+3]
            + coef[280] * A[t%2][i+2][j+2][k-3]
            + coef[281] * A[t%2][i+2][j+2][k-2]
            + coef[282] * A[t%2][i+2][j+2][k-1]
            + coef[283] * A[t%2][i+2][j+2][k]
            + coef[284] * A[t%2][i+2][j+2][k+1]
            + coef[285] * A[t%2][i+2][j+2][k+2]
            + coef[286] * A[t%2][i+2][j+2][k+3]
            + coef[287] * A[t%2][i+2][j+3][k-3]
            + coef[288] * A[t%2][i+2][j+3][k-2]
            + coef[289] * A[t%2][i+2][j+3][k-1]
            + coef[290] * A[t%2][i+2][j+3][k]
            + coef[291] * A[t%2][i+2][j+3][k+1]
            + coef[292] * A[t%2][i+2][j+3][k+2]
            + coef[293] * A[t%2][i+2][j+3][k+3]
            + coef[294] * A[t%2][i+3][j][k]
            + coef[295] * A[t%2][i+3][j-3][k-3]
            + coef[296] * A[t%2][i+3][j-3][k-2]
            + coef[297] * A[t%2][i+3][j-3][k-1]
            + coef[298] * A[t%2][i+3][j-3][k]
            + coef[299] * A[t%2][i+3][j-3][k+1]
            + coef[300] * A[t%2][i+3][j-3][k+2]
            + coef[301] * A[t%2][i+3][j-3][k+3]
            + coef[302] * A[t%2][i+3][j-2][k-3]
            + coef[303] * A[t%2][i+3][j-2][k-2]
            + coef[304] * A[t%2][i+3][j-2][k-1]
            + coef[305] * A[t%2][i+3][j-2][k]
            + coef[306] * A[t%2][i+3][j-2][k+1]
            + coef[307] * A[t%2][i+3][j-2][k+2]
            + coef[308] * A[t%2][i+3][j-2][k+3]
            + coef[309] * A[t%2][i+3][j-1][k-3]
            + coef[310] * A[t%2][i+3][j-1][k-2]
            + coef[311] * A[t%2][i+3][j-1][k-1]
            + coef[312] * A[t%2][i+3][j-1][k]
            + coef[313] * A[t%2][i+3][j-1][k+1]
            + coef[314] * A[t%2][i+3][j-1][k+2]
            + coef[315] * A[t%2][i+3][j-1][k+3]
            + coef[316] * A[t%2][i+3][j][k-3]
            + coef[317] * A[t%2][i+3][j][k-2]
            + coef[318] * A[t%2][i+3][j][k-1]
            + coef[319] * A[t%2][i+3][j][k+1]
            + coef[320] * A[t%2][i+3][j][k+2]
            + coef[321] * A[t%2][i+3][j][k+3]
            + coef[322] * A[t%2][i+3][j+1][k-3]
            + coef[323] * A[t%2][i+3][j+1][k-2]
            + coef[324] * A[t%2][i+3][j+1][k-1]
            + coef[325] * A[t%2][i+3][j+1][k]
            + coef[326] * A[t%2][i+3][j+1][k+1]
            + coef[327] * A[t%2][i+3][j+1][k+2]
            + coef[328] * A[t%2][i+3][j+1][k+3]
            + coef[329] * A[t%2][i+3][j+2][k-3]
            + coef[330] * A[t%2][i+3][j+2][k-2]
            + coef[331] * A[t%2][i+3][j+2][k-1]
            + coef[332] * A[t%2][i+3][j+2][k]
            + coef[333] * A[t%2][i+3][j+2][k+1]
            + coef[334] * A[t%2][i+3][j+2][k+2]
            + coef[335] * A[t%2][i+3][j+2][k+3]
            + coef[336] * A[t%2][i+3][j+3][k-3]
            + coef[337] * A[t%2][i+3][j+3][k-2]
            + coef[338] * A[t%2][i+3][j+3][k-1]
            + coef[339] * A[t%2][i+3][j+3][k]
            + coef[340] * A[t%2][i+3][j+3][k+1]
            + coef[341] * A[t%2][i+3][j+3][k+2]
            + coef[342] * A[t%2][i+3][j+3][k+3];
  }
}

void oracle_box3d4r_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-4][j][k]
            + coef[1] * A[t%2][i-4][j-4][k-4]
            + coef[2] * A[t%2][i-4][j-4][k-3]
            + coef[3] * A[t%2][i-4][j-4][k-2]
            + coef[4] * A[t%2][i-4][j-4][k-1]
            + coef[5] * A[t%2][i-4][j-4][k]
            + coef[6] * A[t%2][i-4][j-4][k+1]
            + coef[7] * A[t%2][i-4][j-4][k+2]
            + coef[8] * A[t%2][i-4][j-4][k+3]
            + coef[9] * A[t%2][i-4][j-4][k+4]
            + coef[10] * A[t%2][i-4][j-3][k-4]
            + coef[11] * A[t%2][i-4][j-3][k-3]
            + coef[12] * A[t%2][i-4][j-3][k-2]
            + coef[13] * A[t%2][i-4][j-3][k-1]
            + coef[14] * A[t%2][i-4][j-3][k]
            + coef[15] * A[t%2][i-4][j-3][k+1]
            + coef[16] * A[t%2][i-4][j-3][k+2]
            + coef[17] * A[t%2][i-4][j-3][k+3]
            + coef[18] * A[t%2][i-4][j-3][k+4]
            + coef[19] * A[t%2][i-4][j-2][k-4]
            + coef[20] * A[t%2][i-4][j-2][k-3]
            + coef[21] * A[t%2][i-4][j-2][k-2]
            + coef[22] * A[t%2][i-4][j-2][k-1]
            + coef[23] * A[t%2][i-4][j-2][k]
            + coef[24] * A[t%2][i-4][j-2][k+1]
            + coef[25] * A[t%2][i-4][j-2][k+2]
            + coef[26] * A[t%2][i-4][j-2][k+3]
            + coef[27] * A[t%2][i-4][j-2][k+4]
            + coef[28] * A[t%2][i-4][j-1][k-4]
            + coef[29] * A[t%2][i-4][j-1][k-3]
            + coef[30] * A[t%2][i-4][j-1][k-2]
            + coef[31] * A[t%2][i-4][j-1][k-1]
            + coef[32] * A[t%2][i-4][j-1][k]
            + coef[33] * A[t%2][i-4][j-1][k+1]
            + coef[34] * A[t%2][i-4][j-1][k+2]
            + coef[35] * A[t%2][i-4][j-1][k+3]
            + coef[36] * A[t%2][i-4][j-1][k+4]
            + coef[37] * A[t%2][i-4][j][k-4]
            + coef[38] * A[t%2][i-4][j][k-3]
            + coef[39] * A[t%2][i-4][j][k-2]
            + coef[40] * A[t%2][i-4][j][k-1]
            + coef[41] * A[t%2][i-4][j][k+1]
            + coef[42] * A[t%2][i-4][j][k+2]
            + coef[43] * A[t%2][i-4][j][k+3]
            + coef[44] * A[t%2][i-4][j][k+4]
            + coef[45] * A[t%2][i-4][j+1][k-4]
            + coef[46] * A[t%2][i-4][j+1][k-3]
            + coef[47] * A[t%2][i-4][j+1][k-2]
            + coef[48] * A[t%2][i-4][j+1][k-1]
            + coef[49] * A[t%2][i-4][j+1][k]
            + coef[50] * A[t%2][i-4][j+1][k+1]
            + coef[51] * A[t%2][i-4][j+1][k+2]
            + coef[52] * A[t%2][i-4][j+1][k+3]
            + coef[53] * A[t%2][i-4][j+1][k+4]
            + coef[54] * A[t%2][i-4][j+2][k-4]
            + coef[55] * A[t%2][i-4][j+2][k-3]
            + coef[56] * A[t%2][i-4][j+2][k-2]
            + coef[57] * A[t%2][i-4][j+2][k-1]
            + coef[58] * A[t%2][i-4][j+2][k]
            + coef[59] * A[t%2][i-4][j+2][k+1]
            + coef[60] * A[t%2][i-4][j+2][k+2]
            + coef[61] * A[t%2][i-4][j+2][k+3]
            + coef[62] * A[t%2][i-4][j+2][k+4]
            + coef[63] * A[t%2][i-4][j+3][k-4]
            + coef[64] * A[t%2][i-4][j+3][k-3]
            + coef[65] * A[t%2][i-4][j+3][k-2]
            + coef[66] * A[t%2][i-4][j+3][k-1]
            + coef[67] * A[t%2][i-4][j+3][k]
            + coef[68] * A[t%2][i-4][j+3][k+1]
            + coef[69] * A[t%2][i-4][j+3][k+2]
            + coef[70] * A[t%2][i-4][j+3][k+3]
            + coef[71] * A[t%2][i-4][j+3][k+4]
            + coef[72] * A[t%2][i-4][j+4][k-4]
            + coef[73] * A[t%2][i-4][j+4][k-3]
            + coef[74] * A[t%2][i-4][j+4][k-2]
            + coef[75] * A[t%2][i-4][j+4][k-1]
            + coef[76] * A[t%2][i-4][j+4][k]
            + coef[77] * A[t%2][i-4][j+4][k+1]
            + coef[78] * A[t%2][i-4][j+4][k+2]
            + coef[79] * A[t%2][i-4][j+4][k+3]
            + coef[80] * A[t%2][i-4][j+4][k+4]
            + coef[81] * A[t%2][i-3][j][k]
            + coef[82] * A[t%2][i-3][j-4][k-4]
            + coef[83] * A[t%2][i-3][j-4][k-3]
            + coef[84] * A[t%2][i-3][j-4][k-2]
            + coef[85] * A[t%2][i-3][j-4][k-1]
            + coef[86] * A[t%2][i-3][j-4][k]
            + coef[87] * A[t%2][i-3][j-4][k+1]
            + coef[88] * A[t%2][i-3][j-4][k+2]
            + coef[89] * A[t%2][i-3][j-4][k+3]
            + coef[90] * A[t%2][i-3][j-4][k+4]
            + coef[91] * A[t%2][i-3][j-3][k-4]
            + coef[92] * A[t%2][i-3][j-3][k-3]
            + coef[93] * A[t%2][i-3][j-3][k-2]
            + coef[94] * A[t%2][i-3][j-3][k-1]
            + coef[95] * A[t%2][i-3][j-3][k]
            + coef[96] * A[t%2][i-3][j-3][k+1]
            + coef[97] * A[t%2][i-3][j-3][k+2]
            + coef[98] * A[t%2][i-3][j-3][k+3]
            + coef[99] * A[t%2][i-3][j-3][k+4]
            + coef[100] * A[t%2][i-3][j-2][k-4]
            + coef[101] * A[t%2][i-3][j-2][k-3]
            + coef[102] * A[t%2][i-3][j-2][k-2]
            + coef[103] * A[t%2][i-3][j-2][k-1]
            + coef[104] * A[t%2][i-3][j-2][k]
            + coef[105] * A[t%2][i-3][j-2][k+1]
            + coef[106] * A[t%2][i-3][j-2][k+2]
            + coef[107] * A[t%2][i-3][j-2][k+3]
            + coef[108] * A[t%2][i-3][j-2][k+4]
            + coef[109] * A[t%2][i-3][j-1][k-4]
            + coef[110] * A[t%2][i-3][j-1][k-3]
            + coef[111] * A[t%2][i-3][j-1][k-2]
            + coef[112] * A[t%2][i-3][j-1][k-1]
            + coef[113] * A[t%2][i-3][j-1][k]
            + coef[114] * A[t%2][i-3][j-1][k+1]
            + coef[115] * A[t%2][i-3][j-1][k+2]
            + coef[116] * A[t%2][i-3][j-1][k+3]
            + coef[117] * A[t%2][i-3][j-1][k+4]
            + coef[118] * A[t%2][i-3][j][k-4]
            + coef[119] * A[t%2][i-3][j][k-3]
            + coef[120] * A[t%2][i-3][j][k-2]
            + coef[121] * A[t%2][i-3][j][k-1]
            + coef[122] * A[t%2][i-3][j][k+1]
            + coef[123] * A[t%2][i-3][j][k+2]
            + coef[124] * A[t%2][i-3][j][k+3]
            + coef[125] * A[t%2][i-3][j][k+4]
            + coef[126] * A[t%2][i-3][j+1][k-4]
            + coef[127] * A[t%2][i-3][j+1][k-3]
            + coef[128] * A[t%2][i-3][j+1][k-2]
            + coef[129] * A[t%2][i-3][j+1][k-1]
            + coef[130] * A[t%2][i-3][j+1][k]
            + coef[131] * A[t%2][i-3][j+1][k+1]
            + coef[132] * A[t%2][i-3][j+1][k+2]
            + coef[133] * A[t%2][i-3][j+1][k+3]
            + coef[134] * A[t%2][i-3][j+1][k+4]
            + coef[135] * A[t%2][i-3][j+2][k-4]
            + coef[136] * A[t%2][i-3][j+2][k-3]
            + coef[137] * A[t%2][i-3][j+2][k-2]
            + coef[138] * A[t%2][i-3][j+2][k-1]
            + coef[139] * A[t%2][i-3][j+2][k]
            + coef[140] * A[t%2][i-3][j+2][k+1]
            + coef[141] * A[t%2][i-3][j+2][k+2]
            + coef[142] * A[t%2][i-3][j+2][k+3]
            + coef[143] * A[t%2][i-3][j+2][k+4]
            + coef[144] * A[t%2][i-3][j+3][k-4]
            + coef[145] * A[t%2][i-3][j+3][k-3]
            + coef[146] * A[t%2][i-3][j+3][k-2]
            + coef[147] * A[t%2][i-3][j+3][k-1]
            + coef[148] * A[t%2][i-3][j+3][k]
            + coef[149] * A[t%2][i-3][j+3][k+1]
            + coef[150] * A[t%2][i-3][j+3][k+2]
            + coef[151] * A[t%2][i-3][j+3][k+3]
            + coef[152] * A[t%2][i-3][j+3][k+4]
            + coef[153] * A[t%2][i-3][j+4][k-4]
            + coef[154] * A[t%2][i-3][j+4][k-3]
            + coef[155] * A[t%2][i-3][j+4][k-2]
            + coef[156] * A[t%2][i-3][j+4][k-1]
            + coef[157] * A[t%2][i-3][j+4][k]
            + coef[158] * A[t%2][i-3][j+4][k+1]
            + coef[159] * A[t%2][i-3][j+4][k+2]
            + coef[160] * A[t%2][i-3][j+4][k+3]
            + coef[161] * A[t%2][i-3][j+4][k+4]
            + coef[162] * A[t%2][i-2][j][k]
            + coef[163] * A[t%2][i-2][j-4][k-4]
            + coef[164] * A[t%2][i-2][j-4][k-3]
            + coef[165] * A[t%2][i-2][j-4][k-2]
            + coef[166] * A[t%2][i-2][j-4][k-1]
            + coef[167] * A[t%2][i-2][j-4][k]
            + coef[168] * A[t%2][i-2][j-4][k+1]
            + coef[169] * A[t%2][i-2][j-4][k+2]
            + coef[170] * A[t%2][i-2][j-4][k+3]
            + coef[171] * A[t%2][i-2][j-4][k+4]
            + coef[172] * A[t%2][i-2][j-3][k-4]
            + coef[173] * A[t%2][i-2][j-3][k-3]
            + coef[174] * A[t%2][i-2][j-3][k-2]
            + coef[175] * A[t%2][i-2][j-3][k-1]
            + coef[176] * A[t%2][i-2][j-3][k]
            + coef[177] * A[t%2][i-2][j-3][k+1]
            + coef[178] * A[t%2][i-2][j-3][k+2]
            + coef[179] * A[t%2][i-2][j-3][k+3]
            + coef[180] * A[t%2][i-2][j-3][k+4]
            + coef[181] * A[t%2][i-2][j-2][k-4]
            + coef[182] * A[t%2][i-2][j-2][k-3]
            + coef[183] * A[t%2][i-2][j-2][k-2]
            + coef[184] * A[t%2][i-2][j-2][k-1]
            + coef[185] * A[t%2][i-2][j-2][k]
            + coef[186] * A[t%2][i-2][j-2][k+1]
            + coef[187] * A[t%2][i-2][j-2][k+2]
            + coef[188] * A[t%2][i-2][j-2][k+3]
            + coef[189] * A[t%2][i-2][j-2][k+4]
            + coef[190] * A[t%2][i-2][j-1][k-4]
            + coef[191] * A[t%2][i-2][j-1][k-3]
            + coef[192] * A[t%2][i-2][j-1][k-2]
            + coef[193] * A[t%2][i-2][j-1][k-1]
            + coef[194] * A[t%2][i-2][j-1][k]
            + coef[195] * A[t%2][i-2][j-1][k+1]
            + coef[196] * A[t%2][i-2][j-1][k+2]
            + coef[197] * A[t%2][i-2][j-1][k+3]
            + coef[198] * A[t%2][i-2][j-1][k+4]
            + coef[199] * A[t%2][i-2][j][k-4]
            + coef[200] * A[t%2][i-2][j][k-3]
            + coef[201] * A[t%2][i-2][j][k-2]
            + coef[202] * A[t%2][i-2][j][k-1]
            + coef[203] * A[t%2][i-2][j][k+1]
            + coef[204] * A[t%2][i-2][j][k+2]
            + coef[205] * A[t%2][i-2][j][k+3]
            + coef[206] * A[t%2][i-2][j][k+4]
            + coef[207] * A[t%2][i-2][j+1][k-4]
            + coef[208] * A[t%2][i-2][j+1][k-3]
            + coef[209] * A[t%2][i-2][j+1][k-2]
            + coef[210] * A[t%2][i-2][j+1][k-1]
            + coef[211] * A[t%2][i-2][j+1][k]
            + coef[212] * A[t%2][i-2][j+1][k+1]
            + coef[213] * A[t%2][i-2][j+1][k+2]
            + coef[214] * A[t%2][i-2][j+1][k+3]
            + coef[215] * A[t%2][i-2][j+1][k+4]
            + coef[216] * A[t%2][i-2][j+2][k-4]
            + coef[217] * A[t%2][i-2][j+2][k-3]
            + coef[218] * A[t%2][i-2][j+2][k-2]
            + coef[219] * A[t%2][i-2][j+2][k-1]
            + coef[220] * A[t%2][i-2][j+2][k]
            + coef[221] * A[t%2][i-2][j+2][k+1]
            + coef[222] * A[t%2][i-2][j+2][k+2]
            + coef[223] * A[t%2][i-2][j+2][k+3]
            + coef[224] * A[t%2][i-2][j+2][k+4]
            + coef[225] * A[t%2][i-2][j+3][k-4]
            + coef[226] * A[t%2][i-2][j+3][k-3]
            + coef[227] * A[t%2][i-2][j+3][k-2]
            + coef[228] * A[t%2][i-2][j+3][k-1]
            + coef[229] * A[t%2][i-2][j+3][k]
            + coef[230] * A[t%2][i-2][j+3][k+1]
            + coef[231] * A[t%2][i-2][j+3][k+2]
            + coef[232] * A[t%2][i-2][j+3][k+3]
            + coef[233] * A[t%2][i-2][j+3][k+4]
            + coef[234] * A[t%2][i-2][j+4][k-4]
            + coef[235] * A[t%2][i-2][j+4][k-3]
            + coef[236] * A[t%2][i-2][j+4][k-2]
            + coef[237] * A[t%2][i-2][j+4][k-1]
            + coef[238] * A[t%2][i-2][j+4][k]
            + coef[239] * A[t%2][i-2][j+4][k+1]
            + coef[240] * A[t%2][i-2][j+4][k+2]
            + coef[241] * A[t%2][i-2][j+4][k+3]
            + coef[242] * A[t%2][i-2][j+4][k+4]
            + coef[243] * A[t%2][i-1][j][k]
            + coef[244] * A[t%2][i-1][j-4][k-4]
            + coef[245] * A[t%2][i-1][j-4][k-3]
            + coef[246] * A[t%2][i-1][j-4][k-2]
            + coef[247] * A[t%2][i-1][j-4][k-1]
            + coef[248] * A[t%2][i-1][j-4][k]
            + coef[249] * A[t%2][i-1][j-4][k+1]
            + coef[250] * A[t%2][i-1][j-4][k+2]
            + coef[251] * A[t%2][i-1][j-4][k+3]
            + coef[252] * A[t%2][i-1][j-4][k+4]
            + coef[253] * A[t%2][i-1][j-3][k-4]
            + coef[254] * A[t%2][i-1][j-3][k-3]
            + coef[255] * A[t%2][i-1][j-3][k-2]
            + coef[256] * A[t%2][i-1][j-3][k-1]
            + coef[257] * A[t%2][i-1][j-3][k]
            + coef[258] * A[t%2][i-1][j-3][k+1]
            + coef[259] * A[t%2][i-1][j-3][k+2]
            + coef[260] * A[t%2][i-1][j-3][k+3]
            + coef[261] * A[t%2][i-1][j-3][k+4]
            + coef[262] * A[t%2][i-1][j-2][k-4]
            + coef[263] * A[t%2][i-1][j-2][k-3]
            + coef[264] * A[t%2][i-1][j-2][k-2]
            + coef[265] * A[t%2][i-1][j-2][k-1]
            + coef[266] * A[t%2][i-1][j-2][k]
            + coef[267] * A[t%2][i-1][j-2][k+1]
            + coef[268] * A[t%2][i-1][j-2][k+2]
            + coef[269] * A[t%2][i-1][j-2][k+3]
            + coef[270] * A[t%2][i-1][j-2][k+4]
            + coef[271] * A[t%2][i-1][j-1][k-4]
            + coef[272] * A[t%2][i-1][j-1][k-3]
            + coef[273] * A[t%2][i-1][j-1][k-2]
            + coef[274] * A[t%2][i-1][j-1][k-1]
            + coef[275] * A[t%2][i-1][j-1][k]
            + coef[276] * A[t%2][i-1][j-1][k+1]
            + coef[277] * A[t%2][i-1][j-1][k+2]
            + coef[278] * A[t%2][i-1][j-1][k+3]
            + coef[279] * A[t%2][i-1][j-1][k+4]
            + coef[280] * A[t%2][i-1][j][k-4]
            + coef[281] * A[t%2][i-1][j][k-3]
            + coef[282] * A[t%2][i-1][j][k-2]
            + coef[283] * A[t%2][i-1][j][k-1]
            + coef[284] * A[t%2][i-1][j][k+1]
            + coef[285] * A[t%2][i-1][j][k+2]
            + coef[286] * A[t%2][i-1][j][k+3]
            + coef[287] * A[t%2][i-1][j][k+4]
            + coef[288] * A[t%2][i-1][j+1][k-4]
            + coef[289] * A[t%2][i-1][j+1][k-3]
            + coef[290] * A[t%2][i-1][j+1][k-2]
            + coef[291] * A[t%2][i-1][j+1][k-1]
            + coef[292] * A[t%2][i-1][j+1][k]
            + coef[293] * A[t%2][i-1][j+1][k+1]
            + coef[294] * A[t%2][i-1][j+1][k+2]
            + coef[295] * A[t%2][i-1][j+1][k+3]
            + coef[296] * A[t%2][i-1][j+1][k+4]
            + coef[297] * A[t%2][i-1][j+2][k-4]
            + coef[298] * A[t%2][i-1][j+2][k-3]
            + coef[299] * A[t%2][i-1][j+2][k-2]
            + coef[300] * A[t%2][i-1][j+2][k-1]
            + coef[301] * A[t%2][i-1][j+2][k]
            + coef[302] * A[t%2][i-1][j+2][k+1]
            + coef[303] * A[t%2][i-1][j+2][k+2]
            + coef[304] * A[t%2][i-1][j+2][k+3]
            + coef[305] * A[t%2][i-1][j+2][k+4]
            + coef[306] * A[t%2][i-1][j+3][k-4]
            + coef[307] * A[t%2][i-1][j+3][k-3]
            + coef[308] * A[t%2][i-1][j+3][k-2]
            + coef[309] * A[t%2][i-1][j+3][k-1]
            + coef[310] * A[t%2][i-1][j+3][k]
            + coef[311] * A[t%2][i-1][j+3][k+1]
            + coef[312] * A[t%2][i-1][j+3][k+2]
            + coef[313] * A[t%2][i-1][j+3][k+3]
            + coef[314] * A[t%2][i-1][j+3][k+4]
            + coef[315] * A[t%2][i-1][j+4][k-4]
            + coef[316] * A[t%2][i-1][j+4][k-3]
            + coef[317] * A[t%2][i-1][j+4][k-2]
            + coef[318] * A[t%2][i-1][j+4][k-1]
            + coef[319] * A[t%2][i-1][j+4][k]
            + coef[320] * A[t%2][i-1][j+4][k+1]
            + coef[321] * A[t%2][i-1][j+4][k+2]
            + coef[322] * A[t%2][i-1][j+4][k+3]
            + coef[323] * A[t%2][i-1][j+4][k+4]
            + coef[324] * A[t%2][i][j][k]
            + coef[325] * A[t%2][i][j-4][k-4]
            + coef[326] * A[t%2][i][j-4][k-3]
            + coef[327] * A[t%2][i][j-4][k-2]
            + coef[328] * A[t%2][i][j-4][k-1]
            + coef[329] * A[t%2][i][j-4][k]
            + coef[330] * A[t%2][i][j-4][k+1]
            + coef[331] * A[t%2][i][j-4][k+2]
            + coef[332] * A[t%2][i][j-4][k+3]
            + coef[333] * A[t%2][i][j-4][k+4]
            + coef[334] * A[t%2][i][j-3][k-4]
            + coef[335] * A[t%2][i][j-3][k-3]
            + coef[336] * A[t%2][i][j-3][k-2]
            + coef[337] * A[t%2][i][j-3][k-1]
            + coef[338] * A[t%2][i][j-3][k]
            + coef[339] * A[t%2][i][j-3][k+1]
            + coef[340] * A[t%2][i][j-3][k+2]
            + coef[341] * A[t%2][i][j-3][k+3]
            + coef[342] * A[t%2][i][j-3][k+4]
            + coef[343] * A[t%2][i][j-2][k-4]
            + coef[344] * A[t%2][i][j-2][k-3]
            + coef[345] * A[t%2][i][j-2][k-2]
            + coef[346] * A[t%2][i][j-2][k-1]
            + coef[347] * A[t%2][i][j-2][k]
            + coef[348] * A[t%2][i][j-2][k+1]
            + coef[349] * A[t%2][i][j-2][k+2]
            + coef[350] * A[t%2][i][j-2][k+3]
            + coef[351] * A[t%2][i][j-2][k+4]
            + coef[352] * A[t%2][i][j-1][k-4]
            + coef[353] * A[t%2][i][j-1][k-3]
            + coef[354] * A[t%2][i][j-1][k-2]
            + coef[355] * A[t%2][i][j-1][k-1]
            + coef[356] * A[t%2][i][j-1][k]
            + coef[357] * A[t%2][i][j-1][k+1]
            + coef[358] * A[t%2][i][j-1][k+2]
            + coef[359] * A[t%2][i][j-1][k+3]
            + coef[360] * A[t%2][i][j-1][k+4]
            + coef[361] * A[t%2][i][j][k-4]
            + coef[362] * A[t%2][i][j][k-3]
            + coef[363] * A[t%2][i][j][k-2]
            + coef[364] * A[t%2][i][j][k-1]
            + coef[365] * A[t%2][i][j][k+1]
            + coef[366] * A[t%2][i][j][k+2]
            + coef[367] * A[t%2][i][j][k+3]
            + coef[368] * A[t%2][i][j][k+4]
            + coef[369] * A[t%2][i][j+1][k-4]
            + coef[370] * A[t%2][i][j+1][k-3]
            + coef[371] * A[t%2][i][j+1][k-2]
            + coef[372] * A[t%2][i][j+1][k-1]
            + coef[373] * A[t%2][i][j+1][k]
            + coef[374] * A[t%2][i][j+1][k+1]
            + coef[375] * A[t%2][i][j+1][k+2]
            + coef[376] * A[t%2][i][j+1][k+3]
            + coef[377] * A[t%2][i][j+1][k+4]
            + coef[378] * A[t%2][i][j+2][k-4]
            + coef[379] * A[t%2][i][j+2][k-3]
            + coef[380] * A[t%2][i][j+2][k-2]
            + coef[381] * A[t%2][i][j+2][k-1]
            + coef[382] * A[t%2][i][j+2][k]
            + coef[383] * A[t%2][i][j+2][k+1]
            + coef[384] * A[t%2][i][j+2][k+2]
            + coef[385] * A[t%2][i][j+2][k+3]
            + coef[386] * A[t%2][i][j+2][k+4]
            + coef[387] * A[t%2][i][j+3][k-4]
            + coef[388] * A[t%2][i][j+3][k-3]
            + coef[389] * A[t%2][i][j+3][k-2]
            + coef[390] * A[t%2][i][j+3][k-1]
            + coef[391] * A[t%2][i][j+3][k]
            + coef[392] * A[t%2][i][j+3][k+1]
            + coef[393] * A[t%2][i][j+3][k+2]
            + coef[394] * A[t%2][i][j+3][k+3]
            + coef[395] * A[t%2][i][j+3][k+4]
            + coef[396] * A[t%2][i][j+4][k-4]
            + coef[397] * A[t%2][i][j+4][k-3]
            + coef[398] * A[t%2][i][j+4][k-2]
            + coef[399] * A[t%2][i][j+4][k-1]
            + coef[400] * A[t%2][i][j+4][k]
            + coef[401] * A[t%2][i][j+4][k+1]
            + coef[402] * A[t%2][i][j+4][k+2]
            + coef[403] * A[t%2][i][j+4][k+3]
            + coef[404] * A[t%2][i][j+4][k+4]
            + coef[405] * A[t%2][i+1][j][k]
            + coef[406] * A[t%2][i+1][j-4][k-4]
            + coef[407] * A[t%2][i+1][j-4][k-3]
            + coef[408] * A[t%2][i+1][j-4][k-2]
            + coef[409] * A[t%2][i+1][j-4][k-1]
            + coef[410] * A[t%2][i+1][j-4][k]
            + coef[411] * A[t%2][i+1][j-4][k+1]
            + coef[412] * A[t%2][i+1][j-4][k+2]
            + coef[413] * A[t%2][i+1][j-4][k+3]
            + coef[414] * A[t%2][i+1][j-4][k+4]
            + coef[415] * A[t%2][i+1][j-3][k-4]
            + coef[416] * A[t%2][i+1][j-3][k-3]
            + coef[417] * A[t%2][i+1][j-3][k-2]
            + coef[418] * A[t%2][i+1][j-3][k-1]
            + coef[419] * A[t%2][i+1][j-3][k]
            + coef[420] * A[t%2][i+1][j-3][k+1]
            + coef[421] * A[t%2][i+1][j-3][k+2]
            + coef[422] * A[t%2][i+1][j-3][k+3]
            + coef[423] * A[t%2][i+1][j-3][k+4]
            + coef[424] * A[t%2][i+1][j-2][k-4]
            + coef[425] * A[t%2][i+1][j-2][k-3]
            + coef[426] * A[t%2][i+1][j-2][k-2]
            + coef[427] * A[t%2][i+1][j-2][k-1]
            + coef[428] * A[t%2][i+1][j-2][k]
            + coef[429] * A[t%2][i+1][j-2][k+1]
            + coef[430] * A[t%2][i+1][j-2][k+2]
            + coef[431] * A[t%2][i+1][j-2][k+3]
            + coef[432] * A[t%2][i+1][j-2][k+4]
            + coef[433] * A[t%2][i+1][j-1][k-4]
            + coef[434] * A[t%2][i+1][j-1][k-3]
            + coef[435] * A[t%2][i+1][j-1][k-2]
            + coef[436] * A[t%2][i+1][j-1][k-1]
            + coef[437] * A[t%2][i+1][j-1][k]
            + coef[438] * A[t%2][i+1][j-1][k+1]
            + coef[439] * A[t%2][i+1][j-1][k+2]
            + coef[440] * A[t%2][i+1][j-1][k+3]
            + coef[441] * A[t%2][i+1][j-1][k+4]
            + coef[442] * A[t%2][i+1][j][k-4]
            + coef[443] * A[t%2][i+1][j][k-3]
            + coef[444] * A[t%2][i+1][j][k-2]
            + coef[445] * A[t%2][i+1][j][k-1]
            + coef[446] * A[t%2][i+1][j][k+1]
            + coef[447] * A[t%2][i+1][j][k+2]
            + coef[448] * A[t%2][i+1][j][k+3]
            + coef[449] * A[t%2][i+1][j][k+4]
            + coef[450] * A[t%2][i+1][j+1][k-4]
            + coef[451] * A[t%2][i+1][j+1][k-3]
            + coef[452] * A[t%2][i+1][j+1][k-2]
            + coef[453] * A[t%2][i+1][j+1][k-1]
            + coef[454] * A[t%2][i+1][j+1][k]
            + coef[455] * A[t%2][i+1][j+1][k+1]
            + coef[456] * A[t%2][i+1][j+1][k+2]
            + coef[457] * A[t%2][i+1][j+1][k+3]
            + coef[458] * A[t%2][i+1][j+1][k+4]
            + coef[459] * A[t%2][i+1][j+2][k-4]
            + coef[460] * A[t%2][i+1][j+2][k-3]
            + coef[461] * A[t%2][i+1][j+2][k-2]
            + coef[462] * A[t%2][i+1][j+2][k-1]
            + coef[463] * A[t%2][i+1][j+2][k]
            + coef[464] * A[t%2][i+1][j+2][k+1]
            + coef[465] * A[t%2][i+1][j+2][k+2]
            + coef[466] * A[t%2][i+1][j+2][k+3]
            + coef[467] * A[t%2][i+1][j+2][k+4]
            + coef[468] * A[t%2][i+1][j+3][k-4]
            + coef[469] * A[t%2][i+1][j+3][k-3]
            + coef[470] * A[t%2][i+1][j+3][k-2]
            + coef[471] * A[t%2][i+1][j+3][k-1]
            + coef[472] * A[t%2][i+1][j+3][k]
            + coef[473] * A[t%2][i+1][j+3][k+1]
            + coef[474] * A[t%2][i+1][j+3][k+2]
            + coef[475] * A[t%2][i+1][j+3][k+3]
            + coef[476] * A[t%2][i+1][j+3][k+4]
            + coef[477] * A[t%2][i+1][j+4][k-4]
            + coef[478] * A[t%2][i+1][j+4][k-3]
            + coef[479] * A[t%2][i+1][j+4][k-2]
            + coef[480] * A[t%2][i+1][j+4][k-1]
            + coef[481] * A[t%2][i+1][j+4][k]
            + coef[482] * A[t%2][i+1][j+4][k+1]
            + coef[483] * A[t%2][i+1][j+4][k+2]
            + coef[484] * A[t%2][i+1][j+4][k+3]
            + coef[485] * A[t%2][i+1][j+4][k+4]
            + coef[486] * A[t%2][i+2][j][k]
            + coef[487] * A[t%2][i+2][j-4][k-4]
            + coef[488] * A[t%2][i+2][j-4][k-3]
            + coef[489] * A[t%2][i+2][j-4][k-2]
            + coef[490] * A[t%2][i+2][j-4][k-1]
            + coef[491] * A[t%2][i+2][j-4][k]
            + coef[492] * A[t%2][i+2][j-4][k+1]
            + coef[493] * A[t%2][i+2][j-4][k+2]
            + coef[494] * A[t%2][i+2][j-4][k+3]
            + coef[495] * A[t%2][i+2][j-4][k+4]
            + coef[496] * A[t%2][i+2][j-3][k-4]
            + coef[497] * A[t%2][i+2][j-3][k-3]
            + coef[498] * A[t%2][i+2][j-3][k-2]
            + coef[499] * A[t%2][i+2][j-3][k-1]
            + coef[500] * A[t%2][i+2][j-3][k]
            + coef[501] * A[t%2][i+2][j-3][k+1]
            + coef[502] * A[t%2][i+2][j-3][k+2]
            + coef[503] * A[t%2][i+2][j-3][k+3]
            + coef[504] * A[t%2][i+2][j-3][k+4]
            + coef[505] * A[t%2][i+2][j-2][k-4]
            + coef[506] * A[t%2][i+2][j-2][k-3]
            + coef[507] * A[t%2][i+2][j-2][k-2]
            + coef[508] * A[t%2][i+2][j-2][k-1]
            + coef[509] * A[t%2][i+2][j-2][k]
            + coef[510] * A[t%2][i+2][j-2][k+1]
            + coef[511] * A[t%2][i+2][j-2][k+2]
            + coef[512] * A[t%2][i+2][j-2][k+3]
            + coef[513] * A[t%2][i+2][j-2][k+4]
            + coef[514] * A[t%2][i+2][j-1][k-4]
            + coef[515] * A[t%2][i+2][j-1][k-3]
            + coef[516] * A[t%2][i+2][j-1][k-2]
            + coef[517] * A[t%2][i+2][j-1][k-1]
            + coef[518] * A[t%2][i+2][j-1][k]
            + coef[519] * A[t%2][i+2][j-1][k+1]
            + coef[520] * A[t%2][i+2][j-1][k+2]
            + coef[521] * A[t%2][i+2][j-1][k+3]
            + coef[522] * A[t%2][i+2][j-1][k+4]
            + coef[523] * A[t%2][i+2][j][k-4]
            + coef[524] * A[t%2][i+2][j][k-3]
            + coef[525] * A[t%2][i+2][j][k-2]
            + coef[526] * A[t%2][i+2][j][k-1]
            + coef[527] * A[t%2][i+2][j][k+1]
            + coef[528] * A[t%2][i+2][j][k+2]
            + coef[529] * A[t%2][i+2][j][k+3]
            + coef[530] * A[t%2][i+2][j][k+4]
            + coef[531] * A[t%2][i+2][j+1][k-4]
            + coef[532] * A[t%2][i+2][j+1][k-3]
            + coef[533] * A[t%2][i+2][j+1][k-2]
            + coef[534] * A[t%2][i+2][j+1][k-1]
            + coef[535] * A[t%2][i+2][j+1][k]
            + coef[536] * A[t%2][i+2][j+1][k+1]
            + coef[537] * A[t%2][i+2][j+1][k+2]
            + coef[538] * A[t%2][i+2][j+1][k+3]
            + coef[539] * A[t%2][i+2][j+1][k+4]
            + coef[540] * A[t%2][i+2][j+2][k-4]
            + coef[541] * A[t%2][i+2][j+2][k-3]
            + coef[542] * A[t%2][i+2][j+2][k-2]
            + coef[543] * A[t%2][i+2][j+2][k-1]
            + coef[544] * A[t%2][i+2][j+2][k]
            + coef[545] * A[t%2][i+2][j+2][k+1]
            + coef[546] * A[t%2][i+2][j+2][k+2]
            + coef[547] * A[t%2][i+2][j+2][k+3]
            + coef[548] * A[t%2][i+2][j+2][k+4]
            + coef[549] * A[t%2][i+2][j+3][k-4]
            + coef[550] * A[t%2][i+2][j+3][k-3]
            + coef[551] * A[t%2][i+2][j+3][k-2]
            + coef[552] * A[t%2][i+2][j+3][k-1]
            + coef[553] * A[t%2][i+2][j+3][k]
            + coef[554] * A[t%2][i+2][j+3][k+1]
            + coef[555] * A[t%2][i+2][j+3][k+2]
            + coef[556] * A[t%2][i+2][j+3][k+3]
            + coef[557] * A[t%2][i+2][j+3][k+4]
            + coef[558] * A[t%2][i+2][j+4][k-4]
            + coef[559] * A[t%2][i+2][j+4][k-3]
            + coef[560] * A[t%2][i+2][j+4][k-2]
            + coef[561] * A[t%2][i+2][j+4][k-1]
            + coef[562] * A[t%2][i+2][j+4][k]
            + coef[563] * A[t%2][i+2][j+4][k+1]
            + coef[564] * A[t%2][i+2][j+4][k+2]
            + coef[565] * A[t%2][i+2][j+4][k+3]
            + coef[566] * A[t%2][i+2][j+4][k+4]
            + coef[567] * A[t%2][i+3][j][k]
            + coef[568] * A[t%2][i+3][j-4][k-4]
            + coef[569] * A[t%2][i+3][j-4][k-3]
            + coef[570] * A[t%2][i+3][j-4][k-2]
            + coef[571] * A[t%2][i+3][j-4][k-1]
            + coef[572] * A[t%2][i+3][j-4][k]
            + coef[573] * A[t%2][i+3][j-4][k+1]
            + coef[574] * A[t%2][i+3][j-4][k+2]
            + coef[575] * A[t%2][i+3][j-4][k+3]
            + coef[576] * A[t%2][i+3][j-4][k+4]
            + coef[577] * A[t%2][i+3][j-3][k-4]
            + coef[578] * A[t%2][i+3][j-3][k-3]
            + coef[579] * A[t%2][i+3][j-3][k-2]
            + coef[580] * A[t%2][i+3][j-3][k-1]
            + coef[581] * A[t%2][i+3][j-3][k]
            + coef[582] * A[t%2][i+3][j-3][k+1]
            + coef[583] * A[t%2][i+3][j-3][k+2]
            + coef[584] * A[t%2][i+3][j-3][k+3]
            + coef[585] * A[t%2][i+3][j-3][k+4]
            + coef[586] * A[t%2][i+3][j-2][k-4]
            + coef[587] * A[t%2][i+3][j-2][k-3]
            + coef[588] * A[t%2][i+3][j-2][k-2]
            + coef[589] * A[t%2][i+3][j-2][k-1]
            + coef[590] * A[t%2][i+3][j-2][k]
            + coef[591] * A[t%2][i+3][j-2][k+1]
            + coef[592] * A[t%2][i+3][j-2][k+2]
            + coef[593] * A[t%2][i+3][j-2][k+3]
            + coef[594] * A[t%2][i+3][j-2][k+4]
            + coef[595] * A[t%2][i+3][j-1][k-4]
            + coef[596] * A[t%2][i+3][j-1][k-3]
            + coef[597] * A[t%2][i+3][j-1][k-2]
            + coef[598] * A[t%2][i+3][j-1][k-1]
            + coef[599] * A[t%2][i+3][j-1][k]
            + coef[600] * A[t%2][i+3][j-1][k+1]
            + coef[601] * A[t%2][i+3][j-1][k+2]
            + coef[602] * A[t%2][i+3][j-1][k+3]
            + coef[603] * A[t%2][i+3][j-1][k+4]
            + coef[604] * A[t%2][i+3][j][k-4]
            + coef[605] * A[t%2][i+3][j][k-3]
            + coef[606] * A[t%2][i+3][j][k-2]
            + coef[607] * A[t%2][i+3][j][k-1]
            + coef[608] * A[t%2][i+3][j][k+1]
            + coef[609] * A[t%2][i+3][j][k+2]
            + coef[610] * A[t%2][i+3][j][k+3]
            + coef[611] * A[t%2][i+3][j][k+4]
            + coef[612] * A[t%2][i+3][j+1][k-4]
            + coef[613] * A[t%2][i+3][j+1][k-3]
            + coef[614] * A[t%2][i+3][j+1][k-2]
            + coef[615] * A[t%2][i+3][j+1][k-1]
            + coef[616] * A[t%2][i+3][j+1][k]
            + coef[617] * A[t%2][i+3][j+1][k+1]
            + coef[618] * A[t%2][i+3][j+1][k+2]
            + coef[619] * A[t%2][i+3][j+1][k+3]
            + coef[620] * A[t%2][i+3][j+1][k+4]
            + coef[621] * A[t%2][i+3][j+2][k-4]
            + coef[622] * A[t%2][i+3][j+2][k-3]
            + coef[623] * A[t%2][i+3][j+2][k-2]
            + coef[624] * A[t%2][i+3][j+2][k-1]
            + coef[625] * A[t%2][i+3][j+2][k]
            + coef[626] * A[t%2][i+3][j+2][k+1]
            + coef[627] * A[t%2][i+3][j+2][k+2]
            + coef[628] * A[t%2][i+3][j+2][k+3]
            + coef[629] * A[t%2][i+3][j+2][k+4]
            + coef[630] * A[t%2][i+3][j+3][k-4]
            + coef[631] * A[t%2][i+3][j+3][k-3]
            + coef[632] * A[t%2][i+3][j+3][k-2]
            + coef[633] * A[t%2][i+3][j+3][k-1]
            + coef[634] * A[t%2][i+3][j+3][k]
            + coef[635] * A[t%2][i+3][j+3][k+1]
            + coef[636] * A[t%2][i+3][j+3][k+2]
            + coef[637] * A[t%2][i+3][j+3][k+3]
            + coef[638] * A[t%2][i+3][j+3][k+4]
            + coef[639] * A[t%2][i+3][j+4][k-4]
            + coef[640] * A[t%2][i+3][j+4][k-3]
            + coef[641] * A[t%2][i+3][j+4][k-2]
            + coef[642] * A[t%2][i+3][j+4][k-1]
            + coef[643] * A[t%2][i+3][j+4][k]
            + coef[644] * A[t%2][i+3][j+4][k+1]
            + coef[645] * A[t%2][i+3][j+4][k+2]
            + coef[646] * A[t%2][i+3][j+4][k+3]
            + coef[647] * A[t%2][i+3][j+4][k+4]
            + coef[648] * A[t%2][i+4][j][k]
            + coef[649] * A[t%2][i+4][j-4][k-4]
            + coef[650] * A[t%2][i+4][j-4][k-3]
            + coef[651] * A[t%2][i+4][j-4][k-2]
            + coef[652] * A[t%2][i+4][j-4][k-1]
            + coef[653] * A[t%2][i+4][j-4][k]
            + coef[654] * A[t%2][i+4][j-4][k+1]
            + coef[655] * A[t%2][i+4][j-4][k+2]
            + coef[656] * A[t%2][i+4][j-4][k+3]
            + coef[657] * A[t%2][i+4][j-4][k+4]
            + coef[658] * A[t%2][i+4][j-3][k-4]
            + coef[659] * A[t%2][i+4][j-3][k-3]
            + coef[660] * A[t%2][i+4][j-3][k-2]
            + coef[661] * A[t%2][i+4][j-3][k-1]
            + coef[662] * A[t%2][i+4][j-3][k]
            + coef[663] * A[t%2][i+4][j-3][k+1]
            + coef[664] * A[t%2][i+4][j-3][k+2]
            + coef[665] * A[t%2][i+4][j-3][k+3]
            + coef[666] * A[t%2][i+4][j-3][k+4]
            + coef[667] * A[t%2][i+4][j-2][k-4]
            + coef[668] * A[t%2][i+4][j-2][k-3]
            + coef[669] * A[t%2][i+4][j-2][k-2]
            + coef[670] * A[t%2][i+4][j-2][k-1]
            + coef[671] * A[t%2][i+4][j-2][k]
            + coef[672] * A[t%2][i+4][j-2][k+1]
            + coef[673] * A[t%2][i+4][j-2][k+2]
            + coef[674] * A[t%2][i+4][j-2][k+3]
            + coef[675] * A[t%2][i+4][j-2][k+4]
            + coef[676] * A[t%2][i+4][j-1][k-4]
            + coef[677] * A[t%2][i+4][j-1][k-3]
            + coef[678] * A[t%2][i+4][j-1][k-2]
            + coef[679] * A[t%2][i+4][j-1][k-1]
            + coef[680] * A[t%2][i+4][j-1][k]
            + coef[681] * A[t%2][i+4][j-1][k+1]
            + coef[682] * A[t%2][i+4][j-1][k+2]
            + coef[683] * A[t%2][i+4][j-1][k+3]
            + coef[684] * A[t%2][i+4][j-1][k+4]
            + coef[685] * A[t%2][i+4][j][k-4]
            + coef[686] * A[t%2][i+4][j][k-3]
            + coef[687] * A[t%2][i+4][j][k-2]
            + coef[688] * A[t%2][i+4][j][k-1]
            + coef[689] * A[t%2][i+4][j][k+1]
            + coef[690] * A[t%2][i+4][j][k+2]
            + coef[691] * A[t%2][i+4][j][k+3]
            + coef[692] * A[t%2][i+4][j][k+4]
            + coef[693] * A[t%2][i+4][j+1][k-4]
            + coef[694] * A[t%2][i+4][j+1][k-3]
            + coef[695] * A[t%2][i+4][j+1][k-2]
            + coef[696] * A[t%2][i+4][j+1][k-1]
            + coef[697] * A[t%2][i+4][j+1][k]
            + coef[698] * A[t%2][i+4][j+1][k+1]
            + coef[699] * A[t%2][i+4][j+1][k+2]
            + coef[700] * A[t%2][i+4][j+1][k+3]
            + coef[701] * A[t%2][i+4][j+1][k+4]
            + coef[702] * A[t%2][i+4][j+2][k-4]
            + coef[703] * A[t%2][i+4][j+2][k-3]
            + coef[704] * A[t%2][i+4][j+2][k-2]
            + coef[705] * A[t%2][i+4][j+2][k-1]
            + coef[706] * A[t%2][i+4][j+2][k]
            + coef[707] * A[t%2][i+4][j+2][k+1]
            + coef[708] * A[t%2][i+4][j+2][k+2]
            + coef[709] * A[t%2][i+4][j+2][k+3]
            + coef[710] * A[t%2][i+4][j+2][k+4]
            + coef[711] * A[t%2][i+4][j+3][k-4]
            + coef[712] * A[t%2][i+4][j+3][k-3]
            + coef[713] * A[t%2][i+4][j+3][k-2]
            + coef[714] * A[t%2][i+4][j+3][k-1]
            + coef[715] * A[t%2][i+4][j+3][k]
            + coef[716] * A[t%2][i+4][j+3][k+1]
            + coef[717] * A[t%2][i+4][j+3][k+2]
            + coef[718] * A[t%2][i+4][j+3][k+3]
            + coef[719] * A[t%2][i+4][j+3][k+4]
            + coef[720] * A[t%2][i+4][j+4][k-4]
            + coef[721] * A[t%2][i+4][j+4][k-3]
            + coef[722] * A[t%2][i+4][j+4][k-2]
            + coef[723] * A[t%2][i+4][j+4][k-1]
            + coef[724] * A[t%2][i+4][j+4][k]
            + coef[725] * A[t%2][i+4][j+4][k+1]
            + coef[726] * A[t%2][i+4][j+4][k+2]
            + coef[727] * A[t%2][i+4][j+4][k+3]
            + coef[728] * A[t%2][i+4][j+4][k+4];
  }
}

void oracle_box3d4r_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-4][j][k]
            + coef[1] * A[t%2][i-4][j-4][k-4]
            + coef[2] * A[t%2][i-4][j-4][k-3]
            + coef[3] * A[t%2][i-4][j-4][k-2]
            + coef[4] * A[t%2][i-4][j-4][k-1]
            + coef[5] * A[t%2][i-4][j-4][k]
            + coef[6] * A[t%2][i-4][j-4][k+1]
            + coef[7] * A[t%2][i-4][j-4][k+2]
            + coef[8] * A[t%2][i-4][j-4][k+3]
            + coef[9] * A[t%2][i-4][j-4][k+4]
            + coef[10] * A[t%2][i-4][j-3][k-4]
            + coef[11] * A[t%2][i-4][j-3][k-3]
            + coef[12] * A[t%2][i-4][j-3][k-2]
            + coef[13] * A[t%2][i-4][j-3][k-1]
            + coef[14] * A[t%2][i-4][j-3][k]
            + coef[15] * A[t%2][i-4][j-3][k+1]
            + coef[16] * A[t%2][i-4][j-3][k+2]
            + coef[17] * A[t%2][i-4][j-3][k+3]
            + coef[18] * A[t%2][i-4][j-3][k+4]
            + coef[19] * A[t%2][i-4][j-2][k-4]
            + coef[20] * A[t%2][i-4][j-2][k-3]
            + coef[21] * A[t%2][i-4][j-2][k-2]
            + coef[22] * A[t%2][i-4][j-2][k-1]
            + coef[23] * A[t%2][i-4][j-2][k]
            + coef[24] * A[t%2][i-4][j-2][k+1]
            + coef[25] * A[t%2][i-4][j-2][k+2]
            + coef[26] * A[t%2][i-4][j-2][k+3]
            + coef[27] * A[t%2][i-4][j-2][k+4]
            + coef[28] * A[t%2][i-4][j-1][k-4]
            + coef[29] * A[t%2][i-4][j-1][k-3]
            + coef[30] * A[t%2][i-4][j-1][k-2]
            + coef[31] * A[t%2][i-4][j-1][k-1]
            + coef[32] * A[t%2][i-4][j-1][k]
            + coef[33] * A[t%2][i-4][j-1][k+1]
            + coef[34] * A[t%2][i-4][j-1][k+2]
            + coef[35] * A[t%2][i-4][j-1][k+3]
            + coef[36] * A[t%2][i-4][j-1][k+4]
            + coef[37] * A[t%2][i-4][j][k-4]
            + coef[38] * A[t%2][i-4][j][k-3]
            + coef[39] * A[t%2][i-4][j][k-2]
            + coef[40] * A[t%2][i-4][j][k-1]
            + coef[41] * A[t%2][i-4][j][k+1]
            + coef[42] * A[t%2][i-4][j][k+2]
            + coef[43] * A[t%2][i-4][j][k+3]
            + coef[44] * A[t%2][i-4][j][k+4]
            + coef[45] * A[t%2][i-4][j+1][k-4]
            + coef[46] * A[t%2][i-4][j+1][k-3]
            + coef[47] * A[t%2][i-4][j+1][k-2]
            + coef[48] * A[t%2][i-4][j+1][k-1]
            + coef[49] * A[t%2][i-4][j+1][k]
            + coef[50] * A[t%2][i-4][j+1][k+1]
            + coef[51] * A[t%2][i-4][j+1][k+2]
            + coef[52] * A[t%2][i-4][j+1][k+3]
            + coef[53] * A[t%2][i-4][j+1][k+4]
            + coef[54] * A[t%2][i-4][j+2][k-4]
            + coef[55] * A[t%2][i-4][j+2][k-3]
            + coef[56] * A[t%2][i-4][j+2][k-2]
            + coef[57] * A[t%2][i-4][j+2][k-1]
            + coef[58] * A[t%2][i-4][j+2][k]
            + coef[59] * A[t%2][i-4][j+2][k+1]
            + coef[60] * A[t%2][i-4][j+2][k+2]
            + coef[61] * A[t%2][i-4][j+2][k+3]
            + coef[62] * A[t%2][i-4][j+2][k+4]
            + coef[63] * A[t%2][i-4][j+3][k-4]
            + coef[64] * A[t%2][i-4][j+3][k-3]
            + coef[65] * A[t%2][i-4][j+3][k-2]
            + coef[66] * A[t%2][i-4][j+3][k-1]
            + coef[67] * A[t%2][i-4][j+3][k]
            + coef[68] * A[t%2][i-4][j+3][k+1]
            + coef[69] * A[t%2][i-4][j+3][k+2]
            + coef[70] * A[t%2][i-4][j+3][k+3]
            + coef[71] * A[t%2][i-4][j+3][k+4]
            + coef[72] * A[t%2][i-4][j+4][k-4]
            + coef[73] * A[t%2][i-4][j+4][k-3]
            + coef[74] * A[t%2][i-4][j+4][k-2]
            + coef[75] * A[t%2][i-4][j+4][k-1]
            + coef[76] * A[t%2][i-4][j+4][k]
            + coef[77] * A[t%2][i-4][j+4][k+1]
            + coef[78] * A[t%2][i-4][j+4][k+2]
            + coef[79] * A[t%2][i-4][j+4][k+3]
            + coef[80] * A[t%2][i-4][j+4][k+4]
            + coef[81] * A[t%2][i-3][j][k]
            + coef[82] * A[t%2][i-3][j-4][k-4]
            + coef[83] * A[t%2][i-3][j-4][k-3]
            + coef[84] * A[t%2][i-3][j-4][k-2]
            + coef[85] * A[t%2][i-3][j-4][k-1]
            + coef[86] * A[t%2][i-3][j-4][k]
            + coef[87] * A[t%2][i-3][j-4][k+1]
            + coef[88] * A[t%2][i-3][j-4][k+2]
            + coef[89] * A[t%2][i-3][j-4][k+3]
            + coef[90] * A[t%2][i-3][j-4][k+4]
            + coef[91] * A[t%2][i-3][j-3][k-4]
            + coef[92] * A[t%2][i-3][j-3][k-3]
            + coef[93] * A[t%2][i-3][j-3][k-2]
            + coef[94] * A[t%2][i-3][j-3][k-1]
            + coef[95] * A[t%2][i-3][j-3][k]
            + coef[96] * A[t%2][i-3][j-3][k+1]
            + coef[97] * A[t%2][i-3][j-3][k+2]
            + coef[98] * A[t%2][i-3][j-3][k+3]
            + coef[99] * A[t%2][i-3][j-3][k+4]
            + coef[100] * A[t%2][i-3][j-2][k-4]
            + coef[101] * A[t%2][i-3][j-2][k-3]
            + coef[102] * A[t%2][i-3][j-2][k-2]
            + coef[103] * A[t%2][i-3][j-2][k-1]
            + coef[104] * A[t%2][i-3][j-2][k]
            + coef[105] * A[t%2][i-3][j-2][k+1]
            + coef[106] * A[t%2][i-3][j-2][k+2]
            + coef[107] * A[t%2][i-3][j-2][k+3]
            + coef[108] * A[t%2][i-3][j-2][k+4]
            + coef[109] * A[t%2][i-3][j-1][k-4]
            + coef[110] * A[t%2][i-3][j-1][k-3]
            + coef[111] * A[t%2][i-3][j-1][k-2]
            + coef[112] * A[t%2][i-3][j-1][k-1]
            + coef[113] * A[t%2][i-3][j-1][k]
            + coef[114] * A[t%2][i-3][j-1][k+1]
            + coef[115] * A[t%2][i-3][j-1][k+2]
            + coef[116] * A[t%2][i-3][j-1][k+3]
            + coef[117] * A[t%2][i-3][j-1][k+4]
            + coef[118] * A[t%2][i-3][j][k-4]
            + coef[119] * A[t%2][i-3][j][k-3]
            + coef[120] * A[t%2][i-3][j][k-2]
            + coef[121] * A[t%2][i-3][j][k-1]
            + coef[122] * A[t%2][i-3][j][k+1]
            + coef[123] * A[t%2][i-3][j][k+2]
            + coef[124] * A[t%2][i-3][j][k+3]
            + coef[125] * A[t%2][i-3][j][k+4]
            + coef[126] * A[t%2][i-3][j+1][k-4]
            + coef[127] * A[t%2][i-3][j+1][k-3]
            + coef[128] * A[t%2][i-3][j+1][k-2]
            + coef[129] * A[t%2][i-3][j+1][k-1]
            + coef[130] * A[t%2][i-3][j+1][k]
            + coef[131] * A[t%2][i-3][j+1][k+1]
            + coef[132] * A[t%2][i-3][j+1][k+2]
            + coef[133] * A[t%2][i-3][j+1][k+3]
            + coef[134] * A[t%2][i-3][j+1][k+4]
            + coef[135] * A[t%2][i-3][j+2][k-4]
            + coef[136] * A[t%2][i-3][j+2][k-3]
            + coef[137] * A[t%2][i-3][j+2][k-2]
            + coef[138] * A[t%2][i-3][j+2][k-1]
            + coef[139] * A[t%2][i-3][j+2][k]
            + coef[140] * A[t%2][i-3][j+2][k+1]
            + coef[141] * A[t%2][i-3][j+2][k+2]
            + coef[142] * A[t%2][i-3][j+2][k+3]
            + coef[143] * A[t%2][i-3][j+2][k+4]
            + coef[144] * A[t%2][i-3][j+3][k-4]
            + coef[145] * A[t%2][i-3][j+3][k-3]
            + coef[146] * A[t%2][i-3][j+3][k-2]
            + coef[147] * A[t%2][i-3][j+3][k-1]
            + coef[148] * A[t%2][i-3][j+3][k]
            + coef[149] * A[t%2][i-3][j+3][k+1]
            + coef[150] * A[t%2][i-3][j+3][k+2]
            + coef[151] * A[t%2][i-3][j+3][k+3]
            + coef[152] * A[t%2][i-3][j+3][k+4]
            + coef[153] * A[t%2][i-3][j+4][k-4]
            + coef[154] * A[t%2][i-3][j+4][k-3]
            + coef[155] * A[t%2][i-3][j+4][k-2]
            + coef[156] * A[t%2][i-3][j+4][k-1]
            + coef[157] * A[t%2][i-3][j+4][k]
            + coef[158] * A[t%2][i-3][j+4][k+1]
            + coef[159] * A[t%2][i-3][j+4][k+2]
            + coef[160] * A[t%2][i-3][j+4][k+3]
            + coef[161] * A[t%2][i-3][j+4][k+4]
            + coef[162] * A[t%2][i-2][j][k]
            + coef[163] * A[t%2][i-2][j-4][k-4]
            + coef[164] * A[t%2][i-2][j-4][k-3]
            + coef[165] * A[t%2][i-2][j-4][k-2]
            + coef[166] * A[t%2][i-2][j-4][k-1]
            + coef[167] * A[t%2][i-2][j-4][k]
            + coef[168] * A[t%2][i-2][j-4][k+1]
            + coef[169] * A[t%2][i-2][j-4][k+2]
            + coef[170] * A[t%2][i-2][j-4][k+3]
            + coef[171] * A[t%2][i-2][j-4][k+4]
            + coef[172] * A[t%2][i-2][j-3][k-4]
            + coef[173] * A[t%2][i-2][j-3][k-3]
            + coef[174] * A[t%2][i-2][j-3][k-2]
            + coef[175] * A[t%2][i-2][j-3][k-1]
            + coef[176] * A[t%2][i-2][j-3][k]
            + coef[177] * A[t%2][i-2][j-3][k+1]
            + coef[178] * A[t%2][i-2][j-3][k+2]
            + coef[179] * A[t%2][i-2][j-3][k+3]
            + coef[180] * A[t%2][i-2][j-3][k+4]
            + coef[181] * A[t%2][i-2][j-2][k-4]
            + coef[182] * A[t%2][i-2][j-2][k-3]
            + coef[183] * A[t%2][i-2][j-2][k-2]
            + coef[184] * A[t%2][i-2][j-2][k-1]
            + coef[185] * A[t%2][i-2][j-2][k]
            + coef[186] * A[t%2][i-2][j-2][k+1]
            + coef[187] * A[t%2][i-2][j-2][k+2]
            + coef[188] * A[t%2][i-2][j-2][k+3]
            + coef[189] * A[t%2][i-2][j-2][k+4]
            + coef[190] * A[t%2][i-2][j-1][k-4]
            + coef[191] * A[t%2][i-2][j-1][k-3]
            + coef[192] * A[t%2][i-2][j-1][k-2]
            + coef[193] * A[t%2][i-2][j-1][k-1]
            + coef[194] * A[t%2][i-2][j-1][k]
            + coef[195] * A[t%2][i-2][j-1][k+1]
            + coef[196] * A[t%2][i-2][j-1][k+2]
            + coef[197] * A[t%2][i-2][j-1][k+3]
            + coef[198] * A[t%2][i-2][j-1][k+4]
            + coef[199] * A[t%2][i-2][j][k-4]
            + coef[200] * A[t%2][i-2][j][k-3]
            + coef[201] * A[t%2][i-2][j][k-2]
            + coef[202] * A[t%2][i-2][j][k-1]
            + coef[203] * A[t%2][i-2][j][k+1]
            + coef[204] * A[t%2][i-2][j][k+2]
            + coef[205] * A[t%2][i-2][j][k+3]
            + coef[206] * A[t%2][i-2][j][k+4]
            + coef[207] * A[t%2][i-2][j+1][k-4]
            + coef[208] * A[t%2][i-2][j+1][k-3]
            + coef[209] * A[t%2][i-2][j+1][k-2]
            + coef[210] * A[t%2][i-2][j+1][k-1]
            + coef[211] * A[t%2][i-2][j+1][k]
            + coef[212] * A[t%2][i-2][j+1][k+1]
            + coef[213] * A[t%2][i-2][j+1][k+2]
            + coef[214] * A[t%2][i-2][j+1][k+3]
            + coef[215] * A[t%2][i-2][j+1][k+4]
            + coef[216] * A[t%2][i-2][j+2][k-4]
            + coef[217] * A[t%2][i-2][j+2][k-3]
            + coef[218] * A[t%2][i-2][j+2][k-2]
            + coef[219] * A[t%2][i-2][j+2][k-1]
            + coef[220] * A[t%2][i-2][j+2][k]
            + coef[221] * A[t%2][i-2][j+2][k+1]
            + coef[222] * A[t%2][i-2][j+2][k+2]
            + coef[223] * A[t%2][i-2][j+2][k+3]
            + coef[224] * A[t%2][i-2][j+2][k+4]
            + coef[225] * A[t%2][i-2][j+3][k-4]
            + coef[226] * A[t%2][i-2][j+3][k-3]
            + coef[227] * A[t%2][i-2][j+3][k-2]
            + coef[228] * A[t%2][i-2][j+3][k-1]
            + coef[229] * A[t%2][i-2][j+3][k]
            + coef[230] * A[t%2][i-2][j+3][k+1]
            + coef[231] * A[t%2][i-2][j+3][k+2]
            + coef[232] * A[t%2][i-2][j+3][k+3]
            + coef[233] * A[t%2][i-2][j+3][k+4]
            + coef[234] * A[t%2][i-2][j+4][k-4]
            + coef[235] * A[t%2][i-2][j+4][k-3]
            + coef[236] * A[t%2][i-2][j+4][k-2]
            + coef[237] * A[t%2][i-2][j+4][k-1]
            + coef[238] * A[t%2][i-2][j+4][k]
            + coef[239] * A[t%2][i-2][j+4][k+1]
            + coef[240] * A[t%2][i-2][j+4][k+2]
            + coef[241] * A[t%2][i-2][j+4][k+3]
            + coef[242] * A[t%2][i-2][j+4][k+4]
            + coef[243] * A[t%2][i-1][j][k]
            + coef[244] * A[t%2][i-1][j-4][k-4]
            + coef[245] * A[t%2][i-1][j-4][k-3]
            + coef[246] * A[t%2][i-1][j-4][k-2]
            + coef[247] * A[t%2][i-1][j-4][k-1]
            + coef[248] * A[t%2][i-1][j-4][k]
            + coef[249] * A[t%2][i-1][j-4][k+1]
            + coef[250] * A[t%2][i-1][j-4][k+2]
            + coef[251] * A[t%2][i-1][j-4][k+3]
            + coef[252] * A[t%2][i-1][j-4][k+4]
            + coef[253] * A[t%2][i-1][j-3][k-4]
            + coef[254] * A[t%2][i-1][j-3][k-3]
            + coef[255] * A[t%2][i-1][j-3][k-2]
            + coef[256] * A[t%2][i-1][j-3][k-1]
            + coef[257] * A[t%2][i-1][j-3][k]
            + coef[258] * A[t%2][i-1][j-3][k+1]
            + coef[259] * A[t%2][i-1][j-3][k+2]
            + coef[260] * A[t%2][i-1][j-3][k+3]
            + coef[261] * A[t%2][i-1][j-3][k+4]
            + coef[262] * A[t%2][i-1][j-2][k-4]
            + coef[263] * A[t%2][i-1][j-2][k-3]
            + coef[264] * A[t%2][i-1][j-2][k-2]
            + coef[265] * A[t%2][i-1][j-2][k-1]
            + coef[266] * A[t%2][i-1][j-2][k]
            + coef[267] * A[t%2][i-1][j-2][k+1]
            + coef[268] * A[t%2][i-1][j-2][k+2]
            + coef[269] * A[t%2][i-1][j-2][k+3]
            + coef[270] * A[t%2][i-1][j-2][k+4]
            + coef[271] * A[t%2][i-1][j-1][k-4]
            + coef[272] * A[t%2][i-1][j-1][k-3]
            + coef[273] * A[t%2][i-1][j-1][k-2]
            + coef[274] * A[t%2][i-1][j-1][k-1]
            + coef[275] * A[t%2][i-1][j-1][k]
            + coef[276] * A[t%2][i-1][j-1][k+1]
            + coef[277] * A[t%2][i-1][j-1][k+2]
            + coef[278] * A[t%2][i-1][j-1][k+3]
            + coef[279] * A[t%2][i-1][j-1][k+4]
            + coef[280] * A[t%2][i-1][j][k-4]
            + coef[281] * A[t%2][i-1][j][k-3]
            + coef[282] * A[t%2][i-1][j][k-2]
            + coef[283] * A[t%2][i-1][j][k-1]
            + coef[284] * A[t%2][i-1][j][k+1]
            + coef[285] * A[t%2][i-1][j][k+2]
            + coef[286] * A[t%2][i-1][j][k+3]
            + coef[287] * A[t%2][i-1][j][k+4]
            + coef[288] * A[t%2][i-1][j+1][k-4]
            + coef[289] * A[t%2][i-1][j+1][k-3]
            + coef[290] * A[t%2][i-1][j+1][k-2]
            + coef[291] * A[t%2][i-1][j+1][k-1]
            + coef[292] * A[t%2][i-1][j+1][k]
            + coef[293] * A[t%2][i-1][j+1][k+1]
            + coef[294] * A[t%2][i-1][j+1][k+2]
            + coef[295] * A[t%2][i-1][j+1][k+3]
            + coef[296] * A[t%2][i-1][j+1][k+4]
            + coef[297] * A[t%2][i-1][j+2][k-4]
            + coef[298] * A[t%2][i-1][j+2][k-3]
            + coef[299] * A[t%2][i-1][j+2][k-2]
            + coef[300] * A[t%2][i-1][j+2][k-1]
            + coef[301] * A[t%2][i-1][j+2][k]
            + coef[302] * A[t%2][i-1][j+2][k+1]
            + coef[303] * A[t%2][i-1][j+2][k+2]
            + coef[304] * A[t%2][i-1][j+2][k+3]
            + coef[305] * A[t%2][i-1][j+2][k+4]
            + coef[306] * A[t%2][i-1][j+3][k-4]
            + coef[307] * A[t%2][i-1][j+3][k-3]
            + coef[308] * A[t%2][i-1][j+3][k-2]
            + coef[309] * A[t%2][i-1][j+3][k-1]
            + coef[310] * A[t%2][i-1][j+3][k]
            + coef[311] * A[t%2][i-1][j+3][k+1]
            + coef[312] * A[t%2][i-1][j+3][k+2]
            + coef[313] * A[t%2][i-1][j+3][k+3]
            + coef[314] * A[t%2][i-1][j+3][k+4]
            + coef[315] * A[t%2][i-1][j+4][k-4]
            + coef[316] * A[t%2][i-1][j+4][k-3]
            + coef[317] * A[t%2][i-1][j+4][k-2]
            + coef[318] * A[t%2][i-1][j+4][k-1]
            + coef[319] * A[t%2][i-1][j+4][k]
            + coef[320] * A[t%2][i-1][j+4][k+1]
            + coef[321] * A[t%2][i-1][j+4][k+2]
            + coef[322] * A[t%2][i-1][j+4][k+3]
            + coef[323] * A[t%2][i-1][j+4][k+4]
            + coef[324] * A[t%2][i][j][k]
            + coef[325] * A[t%2][i][j-4][k-4]
            + coef[326] * A[t%2][i][j-4][k-3]
            + coef[327] * A[t%2][i][j-4][k-2]
            + coef[328] * A[t%2][i][j-4][k-1]
            + coef[329] * A[t%2][i][j-4][k]
            + coef[330] * A[t%2][i][j-4][k+1]
            + coef[331] * A[t%2][i][j-4][k+2]
            + coef[332] * A[t%2][i][j-4][k+3]
            + coef[333] * A[t%2][i][j-4][k+4]
            + coef[334] * A[t%2][i][j-3][k-4]
            + coef[335] * A[t%2][i][j-3][k-3]
            + coef[336] * A[t%2][i][j-3][k-2]
            + coef[337] * A[t%2][i][j-3][k-1]
            + coef[338] * A[t%2][i][j-3][k]
            + coef[339] * A[t%2][i][j-3][k+1]
            + coef[340] * A[t%2][i][j-3][k+2]
            + coef[341] * A[t%2][i][j-3][k+3]
            + coef[342] * A[t%2][i][j-3][k+4]
            + coef[343] * A[t%2][i][j-2][k-4]
            + coef[344] * A[t%2][i][j-2][k-3]
            + coef[345] * A[t%2][i][j-2][k-2]
            + coef[346] * A[t%2][i][j-2][k-1]
            + coef[347] * A[t%2][i][j-2][k]
            + coef[348] * A[t%2][i][j-2][k+1]
            + coef[349] * A[t%2][i][j-2][k+2]
            + coef[350] * A[t%2][i][j-2][k+3]
            + coef[351] * A[t%2][i][j-2][k+4]
            + coef[352] * A[t%2][i][j-1][k-4]
            + coef[353] * A[t%2][i][j-1][k-3]
            + coef[354] * A[t%2][i][j-1][k-2]
            + coef[355] * A[t%2][i][j-1][k-1]
            + coef[356] * A[t%2][i][j-1][k]
            + coef[357] * A[t%2][i][j-1][k+1]
            + coef[358] * A[t%2][i][j-1][k+2]
            + coef[359] * A[t%2][i][j-1][k+3]
            + coef[360] * A[t%2][i][j-1][k+4]
            + coef[361] * A[t%2][i][j][k-4]
            + coef[362] * A[t%2][i][j][k-3]
            + coef[363] * A[t%2][i][j][k-2]
            + coef[364] * A[t%2][i][j][k-1]
            + coef[365] * A[t%2][i][j][k+1]
            + coef[366] * A[t%2][i][j][k+2]
            + coef[367] * A[t%2][i][j][k+3]
            + coef[368] * A[t%2][i][j][k+4]
            + coef[369] * A[t%2][i][j+1][k-4]
            + coef[370] * A[t%2][i][j+1][k-3]
            + coef[371] * A[t%2][i][j+1][k-2]
            + coef[372] * A[t%2][i][j+1][k-1]
            + coef[373] * A[t%2][i][j+1][k]
            + coef[374] * A[t%2][i][j+1][k+1]
            + coef[375] * A[t%2][i][j+1][k+2]
            + coef[376] * A[t%2][i][j+1][k+3]
            + coef[377] * A[t%2][i][j+1][k+4]
            + coef[378] * A[t%2][i][j+2][k-4]
            + coef[379] * A[t%2][i][j+2][k-3]
            + coef[380] * A[t%2][i][j+2][k-2]
            + coef[381] * A[t%2][i][j+2][k-1]
            + coef[382] * A[t%2][i][j+2][k]
            + coef[383] * A[t%2][i][j+2][k+1]
            + coef[384] * A[t%2][i][j+2][k+2]
            + coef[385] * A[t%2][i][j+2][k+3]
            + coef[386] * A[t%2][i][j+2][k+4]
            + coef[387] * A[t%2][i][j+3][k-4]
            + coef[388] * A[t%2][i][j+3][k-3]
            + coef[389] * A[t%2][i][j+3][k-2]
            + coef[390] * A[t%2][i][j+3][k-1]
            + coef[391] * A[t%2][i][j+3][k]
            + coef[392] * A[t%2][i][j+3][k+1]
            + coef[393] * A[t%2][i][j+3][k+2]
            + coef[394] * A[t%2][i][j+3][k+3]
            + coef[395] * A[t%2][i][j+3][k+4]
            + coef[396] * A[t%2][i][j+4][k-4]
            + coef[397] * A[t%2][i][j+4][k-3]
            + coef[398] * A[t%2][i][j+4][k-2]
            + coef[399] * A[t%2][i][j+4][k-1]
            + coef[400] * A[t%2][i][j+4][k]
            + coef[401] * A[t%2][i][j+4][k+1]
            + coef[402] * A[t%2][i][j+4][k+2]
            + coef[403] * A[t%2][i][j+4][k+3]
            + coef[404] * A[t%2][i][j+4][k+4]
            + coef[405] * A[t%2][i+1][j][k]
            + coef[406] * A[t%2][i+1][j-4][k-4]
            + coef[407] * A[t%2][i+1][j-4][k-3]
            + coef[408] * A[t%2][i+1][j-4][k-2]
            + coef[409] * A[t%2][i+1][j-4][k-1]
            + coef[410] * A[t%2][i+1][j-4][k]
            + coef[411] * A[t%2][i+1][j-4][k+1]
            + coef[412] * A[t%2][i+1][j-4][k+2]
            + coef[413] * A[t%2][i+1][j-4][k+3]
            + coef[414] * A[t%2][i+1][j-4][k+4]
            + coef[415] * A[t%2][i+1][j-3][k-4]
            + coef[416] * A[t%2][i+1][j-3][k-3]
            + coef[417] * A[t%2][i+1][j-3][k-2]
            + coef[418] * A[t%2][i+1][j-3][k-1]
            + coef[419] * A[t%2][i+1][j-3][k]
            + coef[420] * A[t%2][i+1][j-3][k+1]
            + coef[421] * A[t%2][i+1][j-3][k+2]
            + coef[422] * A[t%2][i+1][j-3][k+3]
            + coef[423] * A[t%2][i+1][j-3][k+4]
            + coef[424] * A[t%2][i+1][j-2][k-4]
            + coef[425] * A[t%2][i+1][j-2][k-3]
            + coef[426] * A[t%2][i+1][j-2][k-2]
            + coef[427] * A[t%2][i+1][j-2][k-1]
            + coef[428] * A[t%2][i+1][j-2][k]
            + coef[429] * A[t%2][i+1][j-2][k+1]
            + coef[430] * A[t%2][i+1][j-2][k+2]
            + coef[431] * A[t%2][i+1][j-2][k+3]
            + coef[432] * A[t%2][i+1][j-2][k+4]
            + coef[433] * A[t%2][i+1][j-1][k-4]
            + coef[434] * A[t%2][i+1][j-1][k-3]
            + coef[435] * A[t%2][i+1][j-1][k-2]
            + coef[436] * A[t%2][i+1][j-1][k-1]
            + coef[437] * A[t%2][i+1][j-1][k]
            + coef[438] * A[t%2][i+1][j-1][k+1]
            + coef[439] * A[t%2][i+1][j-1][k+2]
            + coef[440] * A[t%2][i+1][j-1][k+3]
            + coef[441] * A[t%2][i+1][j-1][k+4]
            + coef[442] * A[t%2][i+1][j][k-4]
            + coef[443] * A[t%2][i+1][j][k-3]
            + coef[444] * A[t%2][i+1][j][k-2]
            + coef[445] * A[t%2][i+1][j][k-1]
            + coef[446] * A[t%2][i+1][j][k+1]
            + coef[447] * A[t%2][i+1][j][k+2]
            + coef[448] * A[t%2][i+1][j][k+3]
            + coef[449] * A[t%2][i+1][j][k+4]
            + coef[450] * A[t%2][i+1][j+1][k-4]
            + coef[451] * A[t%2][i+1][j+1][k-3]
            + coef[452] * A[t%2][i+1][j+1][k-2]
            + coef[453] * A[t%2][i+1][j+1][k-1]
            + coef[454] * A[t%2][i+1][j+1][k]
            + coef[455] * A[t%2][i+1][j+1][k+1]
            + coef[456] * A[t%2][i+1][j+1][k+2]
            + coef[457] * A[t%2][i+1][j+1][k+3]
            + coef[458] * A[t%2][i+1][j+1][k+4]
            + coef[459] * A[t%2][i+1][j+2][k-4]
            + coef[460] * A[t%2][i+1][j+2][k-3]
            + coef[461] * A[t%2][i+1][j+2][k-2]
            + coef[462] * A[t%2][i+1][j+2][k-1]
            + coef[463] * A[t%2][i+1][j+2][k]
            + coef[464] * A[t%2][i+1][j+2][k+1]
            + coef[465] * A[t%2][i+1][j+2][k+2]
            + coef[466] * A[t%2][i+1][j+2][k+3]
            + coef[467] * A[t%2][i+1][j+2][k+4]
            + coef[468] * A[t%2][i+1][j+3][k-4]
            + coef[469] * A[t%2][i+1][j+3][k-3]
            + coef[470] * A[t%2][i+1][j+3][k-2]
            + coef[471] * A[t%2][i+1][j+3][k-1]
            + coef[472] * A[t%2][i+1][j+3][k]
            + coef[473] * A[t%2][i+1][j+3][k+1]
            + coef[474] * A[t%2][i+1][j+3][k+2]
            + coef[475] * A[t%2][i+1][j+3][k+3]
            + coef[476] * A[t%2][i+1][j+3][k+4]
            + coef[477] * A[t%2][i+1][j+4][k-4]
            + coef[478] * A[t%2][i+1][j+4][k-3]
            + coef[479] * A[t%2][i+1][j+4][k-2]
            + coef[480] * A[t%2][i+1][j+4][k-1]
            + coef[481] * A[t%2][i+1][j+4][k]
            + coef[482] * A[t%2][i+1][j+4][k+1]
            + coef[483] * A[t%2][i+1][j+4][k+2]
            + coef[484] * A[t%2][i+1][j+4][k+3]
            + coef[485] * A[t%2][i+1][j+4][k+4]
            + coef[486] * A[t%2][i+2][j][k]
            + coef[487] * A[t%2][i+2][j-4][k-4]
            + coef[488] * A[t%2][i+2][j-4][k-3]
            + coef[489] * A[t%2][i+2][j-4][k-2]
            + coef[490] * A[t%2][i+2][j-4][k-1]
            + coef[491] * A[t%2][i+2][j-4][k]
            + coef[492] * A[t%2][i+2][j-4][k+1]
            + coef[493] * A[t%2][i+2][j-4][k+2]
            + coef[494] * A[t%2][i+2][j-4][k+3]
            + coef[495] * A[t%2][i+2][j-4][k+4]
            + coef[496] * A[t%2][i+2][j-3][k-4]
            + coef[497] * A[t%2][i+2][j-3][k-3]
            + coef[498] * A[t%2][i+2][j-3][k-2]
            + coef[499] * A[t%2][i+2][j-3][k-1]
            + coef[500] * A[t%2][i+2][j-3][k]
            + coef[501] * A[t%2][i+2][j-3][k+1]
            + coef[502] * A[t%2][i+2][j-3][k+2]
            + coef[503] * A[t%2][i+2][j-3][k+3]
            + coef[504] * A[t%2][i+2][j-3][k+4]
            + coef[505] * A[t%2][i+2][j-2][k-4]
            + coef[506] * A[t%2][i+2][j-2][k-3]
            + coef[507] * A[t%2][i+2][j-2][k-2]
            + coef[508] * A[t%2][i+2][j-2][k-1]
            + coef[509] * A[t%2][i+2][j-2][k]
            + coef[510] * A[t%2][i+2][j-2][k+1]
            + coef[511] * A[t%2][i+2][j-2][k+2]
            + coef[512] * A[t%2][i+2][j-2][k+3]
            + coef[513] * A[t%2][i+2][j-2][k+4]
            + coef[514] * A[t%2][i+2][j-1][k-4]
            + coef[515] * A[t%2][i+2][j-1][k-3]
            + coef[516] * A[t%2][i+2][j-1][k-2]
            + coef[517] * A[t%2][i+2][j-1][k-1]
            + coef[518] * A[t%2][i+2][j-1][k]
            + coef[519] * A[t%2][i+2][j-1][k+1]
            + coef[520] * A[t%2][i+2][j-1][k+2]
            + coef[521] * A[t%2][i+2][j-1][k+3]
            + coef[522] * A[t%2][i+2][j-1][k+4]
            + coef[523] * A[t%2][i+2][j][k-4]
            + coef[524] * A[t%2][i+2][j][k-3]
            + coef[525] * A[t%2][i+2][j][k-2]
            + coef[526] * A[t%2][i+2][j][k-1]
            + coef[527] * A[t%2][i+2][j][k+1]
            + coef[528] * A[t%2][i+2][j][k+2]
            + coef[529] * A[t%2][i+2][j][k+3]
            + coef[530] * A[t%2][i+2][j][k+4]
            + coef[531] * A[t%2][i+2][j+1][k-4]
            + coef[532] * A[t%2][i+2][j+1][k-3]
            + coef[533] * A[t%2][i+2][j+1][k-2]
            + coef[534] * A[t%2][i+2][j+1][k-1]
            + coef[535] * A[t%2][i+2][j+1][k]
            + coef[536] * A[t%2][i+2][j+1][k+1]
            + coef[537] * A[t%2][i+2][j+1][k+2]
            + coef[538] * A[t%2][i+2][j+1][k+3]
            + coef[539] * A[t%2][i+2][j+1][k+4]
            + coef[540] * A[t%2][i+2][j+2][k-4]
            + coef[541] * A[t%2][i+2][j+2][k-3]
            + coef[542] * A[t%2][i+2][j+2][k-2]
            + coef[543] * A[t%2][i+2][j+2][k-1]
            + coef[544] * A[t%2][i+2][j+2][k]
            + coef[545] * A[t%2][i+2][j+2][k+1]
            + coef[546] * A[t%2][i+2][j+2][k+2]
            + coef[547] * A[t%2][i+2][j+2][k+3]
            + coef[548] * A[t%2][i+2][j+2][k+4]
            + coef[549] * A[t%2][i+2][j+3][k-4]
            + coef[550] * A[t%2][i+2][j+3][k-3]
            + coef[551] * A[t%2][i+2][j+3][k-2]
            + coef[552] * A[t%2][i+2][j+3][k-1]
            + coef[553] * A[t%2][i+2][j+3][k]
            + coef[554] * A[t%2][i+2][j+3][k+1]
            + coef[555] * A[t%2][i+2][j+3][k+2]
            + coef[556] * A[t%2][i+2][j+3][k+3]
            + coef[557] * A[t%2][i+2][j+3][k+4]
            + coef[558] * A[t%2][i+2][j+4][k-4]
            + coef[559] * A[t%2][i+2][j+4][k-3]
            + coef[560] * A[t%2][i+2][j+4][k-2]
            + coef[561] * A[t%2][i+2][j+4][k-1]
            + coef[562] * A[t%2][i+2][j+4][k]
            + coef[563] * A[t%2][i+2][j+4][k+1]
            + coef[564] * A[t%2][i+2][j+4][k+2]
            + coef[565] * A[t%2][i+2][j+4][k+3]
            + coef[566] * A[t%2][i+2][j+4][k+4]
            + coef[567] * A[t%2][i+3][j][k]
            + coef[568] * A[t%2][i+3][j-4][k-4]
            + coef[569] * A[t%2][i+3][j-4][k-3]
            + coef[570] * A[t%2][i+3][j-4][k-2]
            + coef[571] * A[t%2][i+3][j-4][k-1]
            + coef[572] * A[t%2][i+3][j-4][k]
            + coef[573] * A[t%2][i+3][j-4][k+1]
            + coef[574] * A[t%2][i+3][j-4][k+2]
            + coef[575] * A[t%2][i+3][j-4][k+3]
            + coef[576] * A[t%2][i+3][j-4][k+4]
            + coef[577] * A[t%2][i+3][j-3][k-4]
            + coef[578] * A[t%2][i+3][j-3][k-3]
            + coef[579] * A[t%2][i+3][j-3][k-2]
            + coef[580] * A[t%2][i+3][j-3][k-1]
            + coef[581] * A[t%2][i+3][j-3][k]
            + coef[582] * A[t%2][i+3][j-3][k+1]
            + coef[583] * A[t%2][i+3][j-3][k+2]
            + coef[584] * A[t%2][i+3][j-3][k+3]
            + coef[585] * A[t%2][i+3][j-3][k+4]
            + coef[586] * A[t%2][i+3][j-2][k-4]
            + coef[587] * A[t%2][i+3][j-2][k-3]
            + coef[588] * A[t%2][i+3][j-2][k-2]
            + coef[589] * A[t%2][i+3][j-2][k-1]
            + coef[590] * A[t%2][i+3][j-2][k]
            + coef[591] * A[t%2][i+3][j-2][k+1]
            + coef[592] * A[t%2][i+3][j-2][k+2]
            + coef[593] * A[t%2][i+3][j-2][k+3]
            + coef[594] * A[t%2][i+3][j-2][k+4]
            + coef[595] * A[t%2][i+3][j-1][k-4]
            + coef[596] * A[t%2][i+3][j-1][k-3]
            + coef[597] * A[t%2][i+3][j-1][k-2]
            + coef[598] * A[t%2][i+3][j-1][k-1]
            + coef[599] * A[t%2][i+3][j-1][k]
            + coef[600] * A[t%2][i+3][j-1][k+1]
            + coef[601] * A[t%2][i+3][j-1][k+2]
            + coef[602] * A[t%2][i+3][j-1][k+3]
            + coef[603] * A[t%2][i+3][j-1][k+4]
            + coef[604] * A[t%2][i+3][j][k-4]
            + coef[605] * A[t%2][i+3][j][k-3]
            + coef[606] * A[t%2][i+3][j][k-2]
            + coef[607] * A[t%2][i+3][j][k-1]
            + coef[608] * A[t%2][i+3][j][k+1]
            + coef[609] * A[t%2][i+3][j][k+2]
            + coef[610] * A[t%2][i+3][j][k+3]
            + coef[611] * A[t%2][i+3][j][k+4]
            + coef[612] * A[t%2][i+3][j+1][k-4]
            + coef[613] * A[t%2][i+3][j+1][k-3]
            + coef[614] * A[t%2][i+3][j+1][k-2]
            + coef[615] * A[t%2][i+3][j+1][k-1]
            + coef[616] * A[t%2][i+3][j+1][k]
            + coef[617] * A[t%2][i+3][j+1][k+1]
            + coef[618] * A[t%2][i+3][j+1][k+2]
            + coef[619] * A[t%2][i+3][j+1][k+3]
            + coef[620] * A[t%2][i+3][j+1][k+4]
            + coef[621] * A[t%2][i+3][j+2][k-4]
            + coef[622] * A[t%2][i+3][j+2][k-3]
            + coef[623] * A[t%2][i+3][j+2][k-2]
            + coef[624] * A[t%2][i+3][j+2][k-1]
            + coef[625] * A[t%2][i+3][j+2][k]
            + coef[626] * A[t%2][i+3][j+2][k+1]
            + coef[627] * A[t%2][i+3][j+2][k+2]
            + coef[628] * A[t%2][i+3][j+2][k+3]
            + coef[629] * A[t%2][i+3][j+2][k+4]
            + coef[630] * A[t%2][i+3][j+3][k-4]
            + coef[631] * A[t%2][i+3][j+3][k-3]
            + coef[632] * A[t%2][i+3][j+3][k-2]
            + coef[633] * A[t%2][i+3][j+3][k-1]
            + coef[634] * A[t%2][i+3][j+3][k]
            + coef[635] * A[t%2][i+3][j+3][k+1]
            + coef[636] * A[t%2][i+3][j+3][k+2]
            + coef[637] * A[t%2][i+3][j+3][k+3]
            + coef[638] * A[t%2][i+3][j+3][k+4]
            + coef[639] * A[t%2][i+3][j+4][k-4]
            + coef[640] * A[t%2][i+3][j+4][k-3]
            + coef[641] * A[t%2][i+3][j+4][k-2]
            + coef[642] * A[t%2][i+3][j+4][k-1]
            + coef[643] * A[t%2][i+3][j+4][k]
            + coef[644] * A[t%2][i+3][j+4][k+1]
            + coef[645] * A[t%2][i+3][j+4][k+2]
            + coef[646] * A[t%2][i+3][j+4][k+3]
            + coef[647] * A[t%2][i+3][j+4][k+4]
            + coef[648] * A[t%2][i+4][j][k]
            + coef[649] * A[t%2][i+4][j-4][k-4]
            + coef[650] * A[t%2][i+4][j-4][k-3]
            + coef[651] * A[t%2][i+4][j-4][k-2]
            + coef[652] * A[t%2][i+4][j-4][k-1]
            + coef[653] * A[t%2][i+4][j-4][k]
            + coef[654] * A[t%2][i+4][j-4][k+1]
            + coef[655] * A[t%2][i+4][j-4][k+2]
            + coef[656] * A[t%2][i+4][j-4][k+3]
            + coef[657] * A[t%2][i+4][j-4][k+4]
            + coef[658] * A[t%2][i+4][j-3][k-4]
            + coef[659] * A[t%2][i+4][j-3][k-3]
            + coef[660] * A[t%2][i+4][j-3][k-2]
            + coef[661] * A[t%2][i+4][j-3][k-1]
            + coef[662] * A[t%2][i+4][j-3][k]
            + coef[663] * A[t%2][i+4][j-3][k+1]
            + coef[664] * A[t%2][i+4][j-3][k+2]
            + coef[665] * A[t%2][i+4][j-3][k+3]
            + coef[666] * A[t%2][i+4][j-3][k+4]
            + coef[667] * A[t%2][i+4][j-2][k-4]
            + coef[668] * A[t%2][i+4][j-2][k-3]
            + coef[669] * A[t%2][i+4][j-2][k-2]
            + coef[670] * A[t%2][i+4][j-2][k-1]
            + coef[671] * A[t%2][i+4][j-2][k]
            + coef[672] * A[t%2][i+4][j-2][k+1]
            + coef[673] * A[t%2][i+4][j-2][k+2]
            + coef[674] * A[t%2][i+4][j-2][k+3]
            + coef[675] * A[t%2][i+4][j-2][k+4]
            + coef[676] * A[t%2][i+4][j-1][k-4]
            + coef[677] * A[t%2][i+4][j-1][k-3]
            + coef[678] * A[t%2][i+4][j-1][k-2]
            + coef[679] * A[t%2][i+4][j-1][k-1]
            + coef[680] * A[t%2][i+4][j-1][k]
            + coef[681] * A[t%2][i+4][j-1][k+1]
            + coef[682] * A[t%2][i+4][j-1][k+2]
            + coef[683] * A[t%2][i+4][j-1][k+3]
            + coef[684] * A[t%2][i+4][j-1][k+4]
            + coef[685] * A[t%2][i+4][j][k-4]
            + coef[686] * A[t%2][i+4][j][k-3]
            + coef[687] * A[t%2][i+4][j][k-2]
            + coef[688] * A[t%2][i+4][j][k-1]
            + coef[689] * A[t%2][i+4][j][k+1]
            + coef[690] * A[t%2][i+4][j][k+2]
            + coef[691] * A[t%2][i+4][j][k+3]
            + coef[692] * A[t%2][i+4][j][k+4]
            + coef[693] * A[t%2][i+4][j+1][k-4]
            + coef[694] * A[t%2][i+4][j+1][k-3]
            + coef[695] * A[t%2][i+4][j+1][k-2]
            + coef[696] * A[t%2][i+4][j+1][k-1]
            + coef[697] * A[t%2][i+4][j+1][k]
            + coef[698] * A[t%2][i+4][j+1][k+1]
            + coef[699] * A[t%2][i+4][j+1][k+2]
            + coef[700] * A[t%2][i+4][j+1][k+3]
            + coef[701] * A[t%2][i+4][j+1][k+4]
            + coef[702] * A[t%2][i+4][j+2][k-4]
            + coef[703] * A[t%2][i+4][j+2][k-3]
            + coef[704] * A[t%2][i+4][j+2][k-2]
            + coef[705] * A[t%2][i+4][j+2][k-1]
            + coef[706] * A[t%2][i+4][j+2][k]
            + coef[707] * A[t%2][i+4][j+2][k+1]
            + coef[708] * A[t%2][i+4][j+2][k+2]
            + coef[709] * A[t%2][i+4][j+2][k+3]
            + coef[710] * A[t%2][i+4][j+2][k+4]
            + coef[711] * A[t%2][i+4][j+3][k-4]
            + coef[712] * A[t%2][i+4][j+3][k-3]
            + coef[713] * A[t%2][i+4][j+3][k-2]
            + coef[714] * A[t%2][i+4][j+3][k-1]
            + coef[715] * A[t%2][i+4][j+3][k]
            + coef[716] * A[t%2][i+4][j+3][k+1]
            + coef[717] * A[t%2][i+4][j+3][k+2]
            + coef[718] * A[t%2][i+4][j+3][k+3]
            + coef[719] * A[t%2][i+4][j+3][k+4]
            + coef[720] * A[t%2][i+4][j+4][k-4]
            + coef[721] * A[t%2][i+4][j+4][k-3]
            + coef[722] * A[t%2][i+4][j+4][k-2]
            + coef[723] * A[t%2][i+4][j+4][k-1]
            + coef[724] * A[t%2][i+4][j+4][k]
            + coef[725] * A[t%2][i+4][j+4][k+1]
            + coef[726] * A[t%2][i+4][j+4][k+2]
            + coef[727] * A[t%2][i+4][j+4][k+3]
            + coef[728] * A[t%2][i+4][j+4][k+4];
  }
}

void oracle_box3d4r_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 8, d1 = n[1] + 8, d2 = n[2] + 8;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 4; i < d0 - 4; i++)
      for (long j = 4; j < d1 - 4; j++)
        for (long k = 4; k < d2 - 4; k++)
          A[(t+1)%2][i][j][k] =
            coef[0] * A[t%2][i-4][j][k]
            + coef[1] * A[t%2][i-4][j-4][k-4]
            + coef[2] * A[t%2][i-4][j-4][k-3]
            + coef[3] * A[t%2][i-4][j-4][k-2]
            + coef[4] * A[t%2][i-4][j-4][k-1]
            + coef[5] * A[t%2][i-4][j-4][k]
            + coef[6] * A[t%2][i-4][j-4][k+1]
            + coef[7] * A[t%2][i-4][j-4][k+2]
            + coef[8] * A[t%2][i-4][j-4][k+3]
            + coef[9] * A[t%2][i-4][j-4][k+4]
            + coef[10] * A[t%2][i-4][j-3][k-4]
            + coef[11] * A[t%2][i-4][j-3][k-3]
            + coef[12] * A[t%2][i-4][j-3][k-2]
            + coef[13] * A[t%2][i-4][j-3][k-1]
            + coef[14] * A[t%2][i-4][j-3][k]
            + coef[15] * A[t%2][i-4][j-3][k+1]
            + coef[16] * A[t%2][i-4][j-3][k+2]
            + coef[17] * A[t%2][i-4][j-3][k+3]
            + coef[18] * A[t%2][i-4][j-3][k+4]
            + coef[19] * A[t%2][i-4][j-2][k-4]
            + coef[20] * A[t%2][i-4][j-2][k-3]
            + coef[21] * A[t%2][i-4][j-2][k-2]
            + coef[22] * A[t%2][i-4][j-2][k-1]
            + coef[23] * A[t%2][i-4][j-2][k]
            + coef[24] * A[t%2][i-4][j-2][k+1]
            + coef[25] * A[t%2][i-4][j-2][k+2]
            + coef[26] * A[t%2][i-4][j-2][k+3]
            + coef[27] * A[t%2][i-4][j-2][k+4]
            + coef[28] * A[t%2][i-4][j-1][k-4]
            + coef[29] * A[t%2][i-4][j-1][k-3]
            + coef[30] * A[t%2][i-4][j-1][k-2]
            + coef[31] * A[t%2][i-4][j-1][k-1]
            + coef[32] * A[t%2][i-4][j-1][k]
            + coef[33] * A[t%2][i-4][j-1][k+1]
            + coef[34] * A[t%2][i-4][j-1][k+2]
            + coef[35] * A[t%2][i-4][j-1][k+3]
            + coef[36] * A[t%2][i-4][j-1][k+4]
            + coef[37] * A[t%2][i-4][j][k-4]
            + coef[38] * A[t%2][i-4][j][k-3]
            + coef[39] * A[t%2][i-4][j][k-2]
            + coef[40] * A[t%2][i-4][j][k-1]
            + coef[41] * A[t%2][i-4][j][k+1]
            + coef[42] * A[t%2][i-4][j][k+2]
            + coef[43] * A[t%2][i-4][j][k+3]
            + coef[44] * A[t%2][i-4][j][k+4]
            + coef[45] * A[t%2][i-4][j+1][k-4]
            + coef[46] * A[t%2][i-4][j+1][k-3]
            + coef[47] * A[t%2][i-4][j+1][k-2]
            + coef[48] * A[t%2][i-4][j+1][k-1]
            + coef[49] * A[t%2][i-4][j+1][k]
            + coef[50] * A[t%2][i-4][j+1][k+1]
            + coef[51] * A[t%2][i-4][j+1][k+2]
            + coef[52] * A[t%2][i-4][j+1][k+3]
            + coef[53] * A[t%2][i-4][j+1][k+4]
            + coef[54] * A[t%2][i-4][j+2][k-4]
            + coef[55] * A[t%2][i-4][j+2][k-3]
            + coef[56] * A[t%2][i-4][j+2][k-2]
            + coef[57] * A[t%2][i-4][j+2][k-1]
            + coef[58] * A[t%2][i-4][j+2][k]
            + coef[59] * A[t%2][i-4][j+2][k+1]
            + coef[60] * A[t%2][i-4][j+2][k+2]
            + coef[61] * A[t%2][i-4][j+2][k+3]
            + coef[62] * A[t%2][i-4][j+2][k+4]
            + coef[63] * A[t%2][i-4][j+3][k-4]
            + coef[64] * A[t%2][i-4][j+3][k-3]
            + coef[65] * A[t%2][i-4][j+3][k-2]
            + coef[66] * A[t%2][i-4][j+3][k-1]
            + coef[67] * A[t%2][i-4][j+3][k]
            + coef[68] * A[t%2][i-4][j+3][k+1]
            + coef[69] * A[t%2][i-4][j+3][k+2]
            + coef[70] * A[t%2][i-4][j+3][k+3]
            + coef[71] * A[t%2][i-4][j+3][k+4]
            + coef[72] * A[t%2][i-4][j+4][k-4]
            + coef[73] * A[t%2][i-4][j+4][k-3]
            + coef[74] * A[t%2][i-4][j+4][k-2]
            + coef[75] * A[t%2][i-4][j+4][k-1]
            + coef[76] * A[t%2][i-4][j+4][k]
            + coef[77] * A[t%2][i-4][j+4][k+1]
            + coef[78] * A[t%2][i-4][j+4][k+2]
            + coef[79] * A[t%2][i-4][j+4][k+3]
            + coef[80] * A[t%2][i-4][j+4][k+4]
            + coef[81] * A[t%2][i-3][j][k]
            + coef[82] * A[t%2][i-3][j-4][k-4]
            + coef[83] * A[t%2][i-3][j-4][k-3]
            + coef[84] * A[t%2][i-3][j-4][k-2]
            + coef[85] * A[t%2][i-3][j-4][k-1]
            + coef[86] * A[t%2][i-3][j-4][k]
            + coef[87] * A[t%2][i-3][j-4][k+1]
            + coef[88] * A[t%2][i-3][j-4][k+2]
            + coef[89] * A[t%2][i-3][j-4][k+3]
            + coef[90] * A[t%2][i-3][j-4][k+4]
            + coef[91] * A[t%2][i-3][j-3][k-4]
            + coef[92] * A[t%2][i-3][j-3][k-3]
            + coef[93] * A[t%2][i-3][j-3][k-2]
            + coef[94] * A[t%2][i-3][j-3][k-1]
            + coef[95] * A[t%2][i-3][j-3][k]
            + coef[96] * A[t%2][i-3][j-3][k+1]
            + coef[97] * A[t%2][i-3][j-3][k+2]
            + coef[98] * A[t%2][i-3][j-3][k+3]
            + coef[99] * A[t%2][i-3][j-3][k+4]
            + coef[100] * A[t%2][i-3][j-2][k-4]
            + coef[101] * A[t%2][i-3][j-2][k-3]
            + coef[102] * A[t%2][i-3][j-2][k-2]
            + coef[103] * A[t%2][i-3][j-2][k-1]
            + coef[104] * A[t%2][i-3][j-2][k]
            + coef[105] * A[t%2][i-3][j-2][k+1]
            + coef[106] * A[t%2][i-3][j-2][k+2]
            + coef[107] * A[t%2][i-3][j-2][k+3]
            + coef[108] * A[t%2][i-3][j-2][k+4]
            + coef[109] * A[t%2][i-3][j-1][k-4]
            + coef[110] * A[t%2][i-3][j-1][k-3]
            + coef[111] * A[t%2][i-3][j-1][k-2]
            + coef[112] * A[t%2][i-3][j-1][k-1]
            + coef[113] * A[t%2][i-3][j-1][k]
            + coef[114] * A[t%2][i-3][j-1][k+1]
            + coef[115] * A[t%2][i-3][j-1][k+2]
            + coef[116] * A[t%2][i-3][j-1][k+3]
            + coef[117] * A[t%2][i-3][j-1][k+4]
            + coef[118] * A[t%2][i-3][j][k-4]
            + coef[119] * A[t%2][i-3][j][k-3]
            + coef[120] * A[t%2][i-3][j][k-2]
            + coef[121] * A[t%2][i-3][j][k-1]
            + coef[122] * A[t%2][i-3][j][k+1]
            + coef[123] * A[t%2][i-3][j][k+2]
            + coef[124] * A[t%2][i-3][j][k+3]
            + coef[125] * A[t%2][i-3][j][k+4]
            + coef[126] * A[t%2][i-3][j+1][k-4]
            + coef[127] * A[t%2][i-3][j+1][k-3]
            + coef[128] * A[t%2][i-3][j+1][k-2]
            + coef[129] * A[t%2][i-3][j+1][k-1]
            + coef[130] * A[t%2][i-3][j+1][k]
            + coef[131] * A[t%2][i-3][j+1][k+1]
            + coef[132] * A[t%2][i-3][j+1][k+2]
            + coef[133] * A[t%2][i-3][j+1][k+3]
            + coef[134] * A[t%2][i-3][j+1][k+4]
            + coef[135] * A[t%2][i-3][j+2][k-4]
            + coef[136] * A[t%2][i-3][j+2][k-3]
            + coef[137] * A[t%2][i-3][j+2][k-2]
            + coef[138] * A[t%2][i-3][j+2][k-1]
            + coef[139] * A[t%2][i-3][j+2][k]
            + coef[140] * A[t%2][i-3][j+2][k+1]
            + coef[141] * A[t%2][i-3][j+2][k+2]
            + coef[142] * A[t%2][i-3][j+2][k+3]
            + coef[143] * A[t%2][i-3][j+2][k+4]
            + coef[144] * A[t%2][i-3][j+3][k-4]
            + coef[145] * A[t%2][i-3][j+3][k-3]
            + coef[146] * A[t%2][i-3][j+3][k-2]
            + coef[147] * A[t%2][i-3][j+3][k-1]
            + coef[148] * A[t%2][i-3][j+3][k]
            + coef[149] * A[t%2][i-3][j+3][k+1]
            + coef[150] * A[t%2][i-3][j+3][k+2]
            + coef[151] * A[t%2][i-3][j+3][k+3]
            + coef[152] * A[t%2][i-3][j+3][k+4]
            + coef[153] * A[t%2][i-3][j+4][k-4]
            + coef[154] * A[t%2][i-3][j+4][k-3]
            + coef[155] * A[t%2][i-3][j+4][k-2]
            + coef[156] * A[t%2][i-3][j+4][k-1]
            + coef[157] * A[t%2][i-3][j+4][k]
            + coef[158] * A[t%2][i-3][j+4][k+1]
            + coef[159] * A[t%2][i-3][j+4][k+2]
            + coef[160] * A[t%2][i-3][j+4][k+3]
            + coef[161] * A[t%2][i-3][j+4][k+4]
            + coef[162] * A[t%2][i-2][j][k]
            + coef[163] * A[t%2][i-2][j-4][k-4]
            + coef[164] * A[t%2][i-2][j-4][k-3]
            + coef[165] * A[t%2][i-2][j-4][k-2]
            + coef[166] * A[t%2][i-2][j-4][k-1]
            + coef[167] * A[t%2][i-2][j-4][k]
            + coef[168] * A[t%2][i-2][j-4][k+1]
            + coef[169] * A[t%2][i-2][j-4][k+2]
            + coef[170] * A[t%2][i-2][j-4][k+3]
            + coef[171] * A[t%2][i-2][j-4][k+4]
            + coef[172] * A[t%2][i-2][j-3][k-4]
            + coef[173] * A[t%2][i-2][j-3][k-3]
            + coef[174] * A[t%2][i-2][j-3][k-2]
            + coef[175] * A[t%2][i-2][j-3][k-1]
            + coef[176] * A[t%2][i-2][j-3][k]
            + coef[177] * A[t%2][i-2][j-3][k+1]
            + coef[178] * A[t%2][i-2][j-3][k+2]
            + coef[179] * A[t%2][i-2][j-3][k+3]
            + coef[180] * A[t%2][i-2][j-3][k+4]
            + coef[181] * A[t%2][i-2][j-2][k-4]
            + coef[182] * A[t%2][i-2][j-2][k-3]
            + coef[183] * A[t%2][i-2][j-2][k-2]
            + coef[184] * A[t%2][i-2][j-2][k-1]
            + coef[185] * A[t%2][i-2][j-2][k]
            + coef[186] * A[t%2][i-2][j-2][k+1]
            + coef[187] * A[t%2][i-2][j-2][k+2]
            + coef[188] * A[t%2][i-2][j-2][k+3]
            + coef[189] * A[t%2][i-2][j-2][k+4]
            + coef[190] * A[t%2][i-2][j-1][k-4]
            + coef[191] * A[t%2][i-2][j-1][k-3]
            + coef[192] * A[t%2][i-2][j-1][k-2]
            + coef[193] * A[t%2][i-2][j-1][k-1]
            + coef[194] * A[t%2][i-2][j-1][k]
            + coef[195] * A[t%2][i-2][j-1][k+1]
            + coef[196] * A[t%2][i-2][j-1][k+2]
            + coef[197] * A[t%2][i-2][j-1][k+3]
            + coef[198] * A[t%2][i-2][j-1][k+4]
            + coef[199] * A[t%2][i-2][j][k-4]
            + coef[200] * A[t%2][i-2][j][k-3]
            + coef[201] * A[t%2][i-2][j][k-2]
            + coef[202] * A[t%2][i-2][j][k-1]
            + coef[203] * A[t%2][i-2][j][k+1]
            + coef[204] * A[t%2][i-2][j][k+2]
            + coef[205] * A[t%2][i-2][j][k+3]
            + coef[206] * A[t%2][i-2][j][k+4]
            + coef[207] * A[t%2][i-2][j+1][k-4]
            + coef[208] * A[t%2][i-2][j+1][k-3]
            + coef[209] * A[t%2][i-2][j+1][k-2]
            + coef[210] * A[t%2][i-2][j+1][k-1]
            + coef[211] * A[t%2][i-2][j+1][k]
            + coef[212] * A[t%2][i-2][j+1][k+1]
            + coef[213] * A[t%2][i-2][j+1][k+2]
            + coef[214] * A[t%2][i-2][j+1][k+3]
            + coef[215] * A[t%2][i-2][j+1][k+4]
            + coef[216] * A[t%2][i-2][j+2][k-4]
            + coef[217] * A[t%2][i-2][j+2][k-3]
            + coef[218] * A[t%2][i-2][j+2][k-2]
            + coef[219] * A[t%2][i-2][j+2][k-1]
            + coef[220] * A[t%2][i-2][j+2][k]
            + coef[221] * A[t%2][i-2][j+2][k+1]
            + coef[222] * A[t%2][i-2][j+2][k+2]
            + coef[223] * A[t%2][i-2][j+2][k+3]
            + coef[224] * A[t%2][i-2][j+2][k+4]
            + coef[225] * A[t%2][i-2][j+3][k-4]
            + coef[226] * A[t%2][i-2][j+3][k-3]
            + coef[227] * A[t%2][i-2][j+3][k-2]
            + coef[228] * A[t%2][i-2][j+3][k-1]
            + coef[229] * A[t%2][i-2][j+3][k]
            + coef[230] * A[t%2][i-2][j+3][k+1]
            + coef[231] * A[t%2][i-2][j+3][k+2]
            + coef[232] * A[t%2][i-2][j+3][k+3]
            + coef[233] * A[t%2][i-2][j+3][k+4]
            + coef[234] * A[t%2][i-2][j+4][k-4]
            + coef[235] * A[t%2][i-2][j+4][k-3]
            + coef[236] * A[t%2][i-2][j+4][k-2]
            + coef[237] * A[t%2][i-2][j+4][k-1]
            + coef[238] * A[t%2][i-2][j+4][k]
            + coef[239] * A[t%2][i-2][j+4][k+1]
            + coef[240] * A[t%2][i-2][j+4][k+2]
            + coef[241] * A[t%2][i-2][j+4][k+3]
            + coef[242] * A[t%2][i-2][j+4][k+4]
            + coef[243] * A[t%2][i-1][j][k]
            + coef[244] * A[t%2][i-1][j-4][k-4]
            + coef[245] * A[t%2][i-1][j-4][k-3]
            + coef[246] * A[t%2][i-1][j-4][k-2]
            + coef[247] * A[t%2][i-1][j-4][k-1]
            + coef[248] * A[t%2][i-1][j-4][k]
            + coef[249] * A[t%2][i-1][j-4][k+1]
            + coef[250] * A[t%2][i-1][j-4][k+2]
            + coef[251] * A[t%2][i-1][j-4][k+3]
            + coef[252] * A[t%2][i-1][j-4][k+4]
            + coef[253] * A[t%2][i-1][j-3][k-4]
            + coef[254] * A[t%2][i-1][j-3][k-3]
            + coef[255] * A[t%2][i-1][j-3][k-2]
            + coef[256] * A[t%2][i-1][j-3][k-1]
            + coef[257] * A[t%2][i-1][j-3][k]
            + coef[258] * A[t%2][i-1][j-3][k+1]
            + coef[259] * A[t%2][i-1][j-3][k+2]
            + coef[260] * A[t%2][i-1][j-3][k+3]
            + coef[261] * A[t%2][i-1][j-3][k+4]
            + coef[262] * A[t%2][i-1][j-2][k-4]
            + coef[263] * A[t%2][i-1][j-2][k-3]
            + coef[264] * A[t%2][i-1][j-2][k-2]
            + coef[265] * A[t%2][i-1][j-2][k-1]
            + coef[266] * A[t%2][i-1][j-2][k]
            + coef[267] * A[t%2][i-1][j-2][k+1]
            + coef[268] * A[t%2][i-1][j-2][k+2]
            + coef[269] * A[t%2][i-1][j-2][k+3]
            + coef[270] * A[t%2][i-1][j-2][k+4]
            + coef[271] * A[t%2][i-1][j-1][k-4]
            + coef[272] * A[t%2][i-1][j-1][k-3]
            + coef[273] * A[t%2][i-1][j-1][k-2]
            + coef[274] * A[t%2][i-1][j-1][k-1]
            + coef[275] * A[t%2][i-1][j-1][k]
            + coef[276] * A[t%2][i-1][j-1][k+1]
            + coef[277] * A[t%2][i-1][j-1][k+2]
            + coef[278] * A[t%2][i-1][j-1][k+3]
            + coef[279] * A[t%2][i-1][j-1][k+4]
            + coef[280] * A[t%2][i-1][j][k-4]
            + coef[281] * A[t%2][i-1][j][k-3]
            + coef[282] * A[t%2][i-1][j][k-2]
            + coef[283] * A[t%2][i-1][j][k-1]
            + coef[284] * A[t%2][i-1][j][k+1]
            + coef[285] * A[t%2][i-1][j][k+2]
            + coef[286] * A[t%2][i-1][j][k+3]
            + coef[287] * A[t%2][i-1][j][k+4]
            + coef[288] * A[t%2][i-1][j+1][k-4]
            + coef[289] * A[t%2][i-1][j+1][k-3]
            + coef[290] * A[t%2][i-1][j+1][k-2]
            + coef[291] * A[t%2][i-1][j+1][k-1]
            + coef[292] * A[t%2][i-1][j+1][k]
            + coef[293] * A[t%2][i-1][j+1][k+1]
            + coef[294] * A[t%2][i-1][j+1][k+2]
            + coef[295] * A[t%2][i-1][j+1][k+3]
            + coef[296] * A[t%2][i-1][j+1][k+4]
            + coef[297] * A[t%2][i-1][j+2][k-4]
            + coef[298] * A[t%2][i-1][j+2][k-3]
            + coef[299] * A[t%2][i-1][j+2][k-2]
            + coef[300] * A[t%2][i-1][j+2][k-1]
            + coef[301] * A[t%2][i-1][j+2][k]
            + coef[302] * A[t%2][i-1][j+2][k+1]
            + coef[303] * A[t%2][i-1][j+2][k+2]
            + coef[304] * A[t%2][i-1][j+2][k+3]
            + coef[305] * A[t%2][i-1][j+2][k+4]
            + coef[306] * A[t%2][i-1][j+3][k-4]
            + coef[307] * A[t%2][i-1][j+3][k-3]
            + coef[308] * A[t%2][i-1][j+3][k-2]
            + coef[309] * A[t%2][i-1][j+3][k-1]
            + coef[310] * A[t%2][i-1][j+3][k]
            + coef[311] * A[t%2][i-1][j+3][k+1]
            + coef[312] * A[t%2][i-1][j+3][k+2]
            + coef[313] * A[t%2][i-1][j+3][k+3]
            + coef[314] * A[t%2][i-1][j+3][k+4]
            + coef[315] * A[t%2][i-1][j+4][k-4]
            + coef[316] * A[t%2][i-1][j+4][k-3]
            + coef[317] * A[t%2][i-1][j+4][k-2]
            + coef[318] * A[t%2][i-1][j+4][k-1]
            + coef[319] * A[t%2][i-1][j+4][k]
            + coef[320] * A[t%2][i-1][j+4][k+1]
            + coef[321] * A[t%2][i-1][j+4][k+2]
            + coef[322] * A[t%2][i-1][j+4][k+3]
            + coef[323] * A[t%2][i-1][j+4][k+4]
            + coef[324] * A[t%2][i][j][k]
            + coef[325] * A[t%2][i][j-4][k-4]
            + coef[326] * A[t%2][i][j-4][k-3]
            + coef[327] * A[t%2][i][j-4][k-2]
            + coef[328] * A[t%2][i][j-4][k-1]
            + coef[329] * A[t%2][i][j-4][k]
            + coef[330] * A[t%2][i][j-4][k+1]
            + coef[331] * A[t%2][i][j-4][k+2]
            + coef[332] * A[t%2][i][j-4][k+3]
            + coef[333] * A[t%2][i][j-4][k+4]
            + coef[334] * A[t%2][i][j-3][k-4]
            + coef[335] * A[t%2][i][j-3][k-3]
            + coef[336] * A[t%2][i][j-3][k-2]
            + coef[337] * A[t%2][i][j-3][k-1]
            + coef[338] * A[t%2][i][j-3][k]
            + coef[339] * A[t%2][i][j-3][k+1]
            + coef[340] * A[t%2][i][j-3][k+2]
            + coef[341] * A[t%2][i][j-3][k+3]
            + coef[342] * A[t%2][i][j-3][k+4]
            + coef[343] * A[t%2][i][j-2][k-4]
            + coef[344] * A[t%2][i][j-2][k-3]
            + coef[345] * A[t%2][i][j-2][k-2]
            + coef[346] * A[t%2][i][j-2][k-1]
            + coef[347] * A[t%2][i][j-2][k]
            + coef[348] * A[t%2][i][j-2][k+1]
            + coef[349] * A[t%2][i][j-2][k+2]
            + coef[350] * A[t%2][i][j-2][k+3]
            + coef[351] * A[t%2][i][j-2][k+4]
            + coef[352] * A[t%2][i][j-1][k-4]
            + coef[353] * A[t%2][i][j-1][k-3]
            + coef[354] * A[t%2][i][j-1][k-2]
            + coef[355] * A[t%2][i][j-1][k-1]
            + coef[356] * A[t%2][i][j-1][k]
            + coef[357] * A[t%2][i][j-1][k+1]
            + coef[358] * A[t%2][i][j-1][k+2]
            + coef[359] * A[t%2][i][j-1][k+3]
            + coef[360] * A[t%2][i][j-1][k+4]
            + coef[361] * A[t%2][i][j][k-4]
            + coef[362] * A[t%2][i][j][k-3]
            + coef[363] * A[t%2][i][j][k-2]
            + coef[364] * A[t%2][i][j][k-1]
            + coef[365] * A[t%2][i][j][k+1]
            + coef[366] * A[t%2][i][j][k+2]
            + coef[367] * A[t%2][i][j][k+3]
            + coef[368] * A[t%2][i][j][k+4]
            + coef[369] * A[t%2][i][j+1][k-4]
            + coef[370] * A[t%2][i][j+1][k-3]
            + coef[371] * A[t%2][i][j+1][k-2]
            + coef[372] * A[t%2][i][j+1][k-1]
            + coef[373] * A[t%2][i][j+1][k]
            + coef[374] * A[t%2][i][j+1][k+1]
            + coef[375] * A[t%2][i][j+1][k+2]
            + coef[376] * A[t%2][i][j+1][k+3]
            + coef[377] * A[t%2][i][j+1][k+4]
            + coef[378] * A[t%2][i][j+2][k-4]
            + coef[379] * A[t%2][i][j+2][k-3]
            + coef[380] * A[t%2][i][j+2][k-2]
            + coef[381] * A[t%2][i][j+2][k-1]
            + coef[382] * A[t%2][i][j+2][k]
            + coef[383] * A[t%2][i][j+2][k+1]
            + coef[384] * A[t%2][i][j+2][k+2]
            + coef[385] * A[t%2][i][j+2][k+3]
            + coef[386] * A[t%2][i][j+2][k+4]
            + coef[387] * A[t%2][i][j+3][k-4]
            + coef[388] * A[t%2][i][j+3][k-3]
            + coef[389] * A[t%2][i][j+3][k-2]
            + coef[390] * A[t%2][i][j+3][k-1]
            + coef[391] * A[t%2][i][j+3][k]
            + coef[392] * A[t%2][i][j+3][k+1]
            + coef[393] * A[t%2][i][j+3][k+2]
            + coef[394] * A[t%2][i][j+3][k+3]
            + coef[395] * A[t%2][i][j+3][k+4]
            + coef[396] * A[t%2][i][j+4][k-4]
            + coef[397] * A[t%2][i][j+4][k-3]
            + coef[398] * A[t%2][i][j+4][k-2]
            + coef[399] * A[t%2][i][j+4][k-1]
            + coef[400] * A[t%2][i][j+4][k]
            + coef[401] * A[t%2][i][j+4][k+1]
            + coef[402] * A[t%2][i][j+4][k+2]
            + coef[403] * A[t%2][i][j+4][k+3]
            + coef[404] * A[t%2][i][j+4][k+4]
            + coef[405] * A[t%2][i+1][j][k]
            + coef[406] * A[t%2][i+1][j-4][k-4]
            + coef[407] * A[t%2][i+1][j-4][k-3]
            + coef[408] * A[t%2][i+1][j-4][k-2]
            + coef[409] * A[t%2][i+1][j-4][k-1]
            + coef[410] * A[t%2][i+1][j-4][k]
            + coef[411] * A[t%2][i+1][j-4][k+1]
            + coef[412] * A[t%2][i+1][j-4][k+2]
            + coef[413] * A[t%2][i+1][j-4][k+3]
            + coef[414] * A[t%2][i+1][j-4][k+4]
            + coef[415] * A[t%2][i+1][j-3][k-4]
            + coef[416] * A[t%2][i+1][j-3][k-3]
            + coef[417] * A[t%2][i+1][j-3][k-2]
            + coef[418] * A[t%2][i+1][j-3][k-1]
            + coef[419] * A[t%2][i+1][j-3][k]
            + coef[420] * A[t%2][i+1][j-3][k+1]
            + coef[421] * A[t%2][i+1][j-3][k+2]
            + coef[422] * A[t%2][i+1][j-3][k+3]
            + coef[423] * A[t%2][i+1][j-3][k+4]
            + coef[424] * A[t%2][i+1][j-2][k-4]
            + coef[425] * A[t%2][i+1][j-2][k-3]
            + coef[426] * A[t%2][i+1][j-2][k-2]
            + coef[427] * A[t%2][i+1][j-2][k-1]
            + coef[428] * A[t%2][i+1][j-2][k]
            + coef[429] * A[t%2][i+1][j-2][k+1]
            + coef[430] * A[t%2][i+1][j-2][k+2]
            + coef[431] * A[t%2][i+1][j-2][k+3]
            + coef[432] * A[t%2][i+1][j-2][k+4]
            + coef[433] * A[t%2][i+1][j-1][k-4]
            + coef[434] * A[t%2][i+1][j-1][k-3]
            + coef[435] * A[t%2][i+1][j-1][k-2]
            + coef[436] * A[t%2][i+1][j-1][k-1]
            + coef[437] * A[t%2][i+1][j-1][k]
            + coef[438] * A[t%2][i+1][j-1][k+1]
            + coef[439] * A[t%2][i+1][j-1][k+2]
            + coef[440] * A[t%2][i+1][j-1][k+3]
            + coef[441] * A[t%2][i+1][j-1][k+4]
            + coef[442] * A[t%2][i+1][j][k-4]
            + coef[443] * A[t%2][i+1][j][k-3]
            + coef[444] * A[t%2][i+1][j][k-2]
            + coef[445] * A[t%2][i+1][j][k-1]
            + coef[446] * A[t%2][i+1][j][k+1]
            + coef[447] * A[t%2][i+1][j][k+2]
            + coef[448] * A[t%2][i+1][j][k+3]
            + coef[449] * A[t%2][i+1][j][k+4]
            + coef[450] * A[t%2][i+1][j+1][k-4]
            + coef[451] * A[t%2][i+1][j+1][k-3]
            + coef[452] * A[t%2][i+1][j+1][k-2]
            + coef[453] * A[t%2][i+1][j+1][k-1]
            + coef[454] * A[t%2][i+1][j+1][k]
            + coef[455] * A[t%2][i+1][j+1][k+1]
            + coef[456] * A[t%2][i+1][j+1][k+2]
            + coef[457] * A[t%2][i+1][j+1][k+3]
            + coef[458] * A[t%2][i+1][j+1][k+4]
            + coef[459] * A[t%2][i+1][j+2][k-4]
            + coef[460] * A[t%2][i+1][j+2][k-3]
            + coef[461] * A[t%2][i+1][j+2][k-2]
            + coef[462] * A[t%2][i+1][j+2][k-1]
            + coef[463] * A[t%2][i+1][j+2][k]
            + coef[464] * A[t%2][i+1][j+2][k+1]
            + coef[465] * A[t%2][i+1][j+2][k+2]
            + coef[466] * A[t%2][i+1][j+2][k+3]
            + coef[467] * A[t%2][i+1][j+2][k+4]
            + coef[468] * A[t%2][i+1][j+3][k-4]
            + coef[469] * A[t%2][i+1][j+3][k-3]
            + coef[470] * A[t%2][i+1][j+3][k-2]
            + coef[471] * A[t%2][i+1][j+3][k-1]
            + coef[472] * A[t%2][i+1][j+3][k]
            + coef[473] * A[t%2][i+1][j+3][k+1]
            + coef[474] * A[t%2][i+1][j+3][k+2]
            + coef[475] * A[t%2][i+1][j+3][k+3]
            + coef[476] * A[t%2][i+1][j+3][k+4]
            + coef[477] * A[t%2][i+1][j+4][k-4]
            + coef[478] * A[t%2][i+1][j+4][k-3]
            + coef[479] * A[t%2][i+1][j+4][k-2]
            + coef[480] * A[t%2][i+1][j+4][k-1]
            + coef[481] * A[t%2][i+1][j+4][k]
            + coef[482] * A[t%2][i+1][j+4][k+1]
            + coef[483] * A[t%2][i+1][j+4][k+2]
            + coef[484] * A[t%2][i+1][j+4][k+3]
            + coef[485] * A[t%2][i+1][j+4][k+4]
            + coef[486] * A[t%2][i+2][j][k]
            + coef[487] * A[t%2][i+2][j-4][k-4]
            + coef[488] * A[t%2][i+2][j-4][k-3]
            + coef[489] * A[t%2][i+2][j-4][k-2]
            + coef[490] * A[t%2][i+2][j-4][k-1]
            + coef[491] * A[t%2][i+2][j-4][k]
            + coef[492] * A[t%2][i+2][j-4][k+1]
            + coef[493] * A[t%2][i+2][j-4][k+2]
            + coef[494] * A[t%2][i+2][j-4][k+3]
            + coef[495] * A[t%2][i+2][j-4][k+4]
            + coef[496] * A[t%2][i+2][j-3][k-4]
            + coef[497] * A[t%2][i+2][j-3][k-3]
            + coef[498] * A[t%2][i+2][j-3][k-2]
            + coef[499] * A[t%2][i+2][j-3][k-1]
            + coef[500] * A[t%2][i+2][j-3][k]
            + coef[501] * A[t%2][i+2][j-3][k+1]
            + coef[502] * A[t%2][i+2][j-3][k+2]
            + coef[503] * A[t%2][i+2][j-3][k+3]
            + coef[504] * A[t%2][i+2][j-3][k+4]
            + coef[505] * A[t%2][i+2][j-2][k-4]
            + coef[506] * A[t%2][i+2][j-2][k-3]
            + coef[507] * A[t%2][i+2][j-2][k-2]
            + coef[508] * A[t%2][i+2][j-2][k-1]
            + coef[509] * A[t%2][i+2][j-2][k]
            + coef[510] * A[t%2][i+2][j-2][k+1]
            + coef[511] * A[t%2][i+2][j-2][k+2]
            + coef[512] * A[t%2][i+2][j-2][k+3]
            + coef[513] * A[t%2][i+2][j-2][k+4]
            + coef[514] * A[t%2][i+2][j-1][k-4]
            + coef[515] * A[t%2][i+2][j-1][k-3]
            + coef[516] * A[t%2][i+2][j-1][k-2]
            + coef[517] * A[t%2][i+2][j-1][k-1]
            + coef[518] * A[t%2][i+2][j-1][k]
            + coef[519] * A[t%2][i+2][j-1][k+1]
            + coef[520] * A[t%2][i+2][j-1][k+2]
            + coef[521] * A[t%2][i+2][j-1][k+3]
            + coef[522] * A[t%2][i+2][j-1][k+4]
            + coef[523] * A[t%2][i+2][j][k-4]
            + coef[524] * A[t%2][i+2][j][k-3]
            + coef[525] * A[t%2][i+2][j][k-2]
            + coef[526] * A[t%2][i+2][j][k-1]
            + coef[527] * A[t%2][i+2][j][k+1]
            + coef[528] * A[t%2][i+2][j][k+2]
            + coef[529] * A[t%2][i+2][j][k+3]
            + coef[530] * A[t%2][i+2][j][k+4]
            + coef[531] * A[t%2][i+2][j+1][k-4]
            + coef[532] * A[t%2][i+2][j+1][k-3]
            + coef[533] * A[t%2][i+2][j+1][k-2]
            + coef[534] * A[t%2][i+2][j+1][k-1]
            + coef[535] * A[t%2][i+2][j+1][k]
            + coef[536] * A[t%2][i+2][j+1][k+1]
            + coef[537] * A[t%2][i+2][j+1][k+2]
            + coef[538] * A[t%2][i+2][j+1][k+3]
            + coef[539] * A[t%2][i+2][j+1][k+4]
            + coef[540] * A[t%2][i+2][j+2][k-4]
            + coef[541] * A[t%2][i+2][j+2][k-3]
            + coef[542] * A[t%2][i+2][j+2][k-2]
            + coef[543] * A[t%2][i+2][j+2][k-1]
            + coef[544] * A[t%2][i+2][j+2][k]
            + coef[545] * A[t%2][i+2][j+2][k+1]
            + coef[546] * A[t%2][i+2][j+2][k+2]
            + coef[547] * A[t%2][i+2][j+2][k+3]
            + coef[548] * A[t%2][i+2][j+2][k+4]
            + coef[549] * A[t%2][i+2][j+3][k-4]
            + coef[550] * A[t%2][i+2][j+3][k-3]
            + coef[551] * A[t%2][i+2][j+3][k-2]
            + coef[552] * A[t%2][i+2][j+3][k-1]
            + coef[553] * A[t%2][i+2][j+3][k]
            + coef[554] * A[t%2][i+2][j+3][k+1]
            + coef[555] * A[t%2][i+2][j+3][k+2]
            + coef[556] * A[t%2][i+2][j+3][k+3]
            + coef[557] * A[t%2][i+2][j+3][k+4]
            + coef[558] * A[t%2][i+2][j+4][k-4]
            + coef[559] * A[t%2][i+2][j+4][k-3]
            + coef[560] * A[t%2][i+2][j+4][k-2]
            + coef[561] * A[t%2][i+2][j+4][k-1]
            + coef[562] * A[t%2][i+2][j+4][k]
            + coef[563] * A[t%2][i+2][j+4][k+1]
            + coef[564] * A[t%2][i+2][j+4][k+2]
            + coef[565] * A[t%2][i+2][j+4][k+3]
            + coef[566] * A[t%2][i+2][j+4][k+4]
            + coef[567] * A[t%2][i+3][j][k]
            + coef[568] * A[t%2][i+3][j-4][k-4]
            + coef[569] * A[t%2][i+3][j-4][k-3]
            + coef[570] * A[t%2][i+3][j-4][k-2]
            + coef[571] * A[t%2][i+3][j-4][k-1]
            + coef[572] * A[t%2][i+3][j-4][k]
            + coef[573] * A[t%2][i+3][j-4][k+1]
            + coef[574] * A[t%2][i+3][j-4][k+2]
            + coef[575] * A[t%2][i+3][j-4][k+3]
            + coef[576] * A[t%2][i+3][j-4][k+4]
            + coef[577] * A[t%2][i+3][j-3][k-4]
            + coef[578] * A[t%2][i+3][j-3][k-3]
            + coef[579] * A[t%2][i+3][j-3][k-2]
            + coef[580] * A[t%2][i+3][j-3][k-1]
            + coef[581] * A[t%2][i+3][j-3][k]
            + coef[582] * A[t%2][i+3][j-3][k+1]
            + coef[583] * A[t%2][i+3][j-3][k+2]
            + coef[584] * A[t%2][i+3][j-3][k+3]
            + coef[585] * A[t%2][i+3][j-3][k+4]
            + coef[586] * A[t%2][i+3][j-2][k-4]
            + coef[587] * A[t%2][i+3][j-2][k-3]
            + coef[588] * A[t%2][i+3][j-2][k-2]
            + coef[589] * A[t%2][i+3][j-2][k-1]
            + coef[590] * A[t%2][i+3][j-2][k]
            + coef[591] * A[t%2][i+3][j-2][k+1]
            + coef[592] * A[t%2][i+3][j-2][k+2]
            + coef[593] * A[t%2][i+3][j-2][k+3]
            + coef[594] * A[t%2][i+3][j-2][k+4]
            + coef[595] * A[t%2][i+3][j-1][k-4]
            + coef[596] * A[t%2][i+3][j-1][k-3]
            + coef[597] * A[t%2][i+3][j-1][k-2]
            + coef[598] * A[t%2][i+3][j-1][k-1]
            + coef[599] * A[t%2][i+3][j-1][k]
            + coef[600] * A[t%2][i+3][j-1][k+1]
            + coef[601] * A[t%2][i+3][j-1][k+2]
            + coef[602] * A[t%2][i+3][j-1][k+3]
            + coef[603] * A[t%2][i+3][j-1][k+4]
            + coef[604] * A[t%2][i+3][j][k-4]
            + coef[605] * A[t%2][i+3][j][k-3]
            + coef[606] * A[t%2][i+3][j][k-2]
            + coef[607] * A[t%2][i+3][j][k-1]
            + coef[608] * A[t%2][i+3][j][k+1]
            + coef[609] * A[t%2][i+3][j][k+2]
            + coef[610] * A[t%2][i+3][j][k+3]
            + coef[611] * A[t%2][i+3][j][k+4]
            + coef[612] * A[t%2][i+3][j+1][k-4]
            + coef[613] * A[t%2][i+3][j+1][k-3]
            + coef[614] * A[t%2][i+3][j+1][k-2]
            + coef[615] * A[t%2][i+3][j+1][k-1]
            + coef[616] * A[t%2][i+3][j+1][k]
            + coef[617] * A[t%2][i+3][j+1][k+1]
            + coef[618] * A[t%2][i+3][j+1][k+2]
            + coef[619] * A[t%2][i+3][j+1][k+3]
            + coef[620] * A[t%2][i+3][j+1][k+4]
            + coef[621] * A[t%2][i+3][j+2][k-4]
            + coef[622] * A[t%2][i+3][j+2][k-3]
            + coef[623] * A[t%2][i+3][j+2][k-2]
            + coef[624] * A[t%2][i+3][j+2][k-1]
            + coef[625] * A[t%2][i+3][j+2][k]
            + coef[626] * A[t%2][i+3][j+2][k+1]
            + coef[627] * A[t%2][i+3][j+2][k+2]
            + coef[628] * A[t%2][i+3][j+2][k+3]
            + coef[629] * A[t%2][i+3][j+2][k+4]
            + coef[630] * A[t%2][i+3][j+3][k-4]
            + coef[631] * A[t%2][i+3][j+3][k-3]
            + coef[632] * A[t%2][i+3][j+3][k-2]
            + coef[633] * A[t%2][i+3][j+3][k-1]
            + coef[634] * A[t%2][i+3][j+3][k]
            + coef[635] * A[t%2][i+3][j+3][k+1]
            + coef[636] * A[t%2][i+3][j+3][k+2]
            + coef[637] * A[t%2][i+3][j+3][k+3]
            + coef[638] * A[t%2][i+3][j+3][k+4]
            + coef[639] * A[t%2][i+3][j+4][k-4]
            + coef[640] * A[t%2][i+3][j+4][k-3]
            + coef[641] * A[t%2][i+3][j+4][k-2]
            + coef[642] * A[t%2][i+3][j+4][k-1]
            + coef[643] * A[t%2][i+3][j+4][k]
            + coef[644] * A[t%2][i+3][j+4][k+1]
            + coef[645] * A[t%2][i+3][j+4][k+2]
            + coef[646] * A[t%2][i+3][j+4][k+3]
            + coef[647] * A[t%2][i+3][j+4][k+4]
            + coef[648] * A[t%2][i+4][j][k]
            + coef[649] * A[t%2][i+4][j-4][k-4]
            + coef[650] * A[t%2][i+4][j-4][k-3]
            + coef[651] * A[t%2][i+4][j-4][k-2]
            + coef[652] * A[t%2][i+4][j-4][k-1]
            + coef[653] * A[t%2][i+4][j-4][k]
            + coef[654] * A[t%2][i+4][j-4][k+1]
            + coef[655] * A[t%2][i+4][j-4][k+2]
            + coef[656] * A[t%2][i+4][j-4][k+3]
            + coef[657] * A[t%2][i+4][j-4][k+4]
            + coef[658] * A[t%2][i+4][j-3][k-4]
            + coef[659] * A[t%2][i+4][j-3][k-3]
            + coef[660] * A[t%2][i+4][j-3][k-2]
            + coef[661] * A[t%2][i+4][j-3][k-1]
            + coef[662] * A[t%2][i+4][j-3][k]
            + coef[663] * A[t%2][i+4][j-3][k+1]
            + coef[664] * A[t%2][i+4][j-3][k+2]
            + coef[665] * A[t%2][i+4][j-3][k+3]
            + coef[666] * A[t%2][i+4][j-3][k+4]
            + coef[667] * A[t%2][i+4][j-2][k-4]
            + coef[668] * A[t%2][i+4][j-2][k-3]
            + coef[669] * A[t%2][i+4][j-2][k-2]
            + coef[670] * A[t%2][i+4][j-2][k-1]
            + coef[671] * A[t%2][i+4][j-2][k]
            + coef[672] * A[t%2][i+4][j-2][k+1]
            + coef[673] * A[t%2][i+4][j-2][k+2]
            + coef[674] * A[t%2][i+4][j-2][k+3]
            + coef[675] * A[t%2][i+4][j-2][k+4]
            + coef[676] * A[t%2][i+4][j-1][k-4]
            + coef[677] * A[t%2][i+4][j-1][k-3]
            + coef[678] * A[t%2][i+4][j-1][k-2]
            + coef[679] * A[t%2][i+4][j-1][k-1]
            + coef[680] * A[t%2][i+4][j-1][k]
            + coef[681] * A[t%2][i+4][j-1][k+1]
            + coef[682] * A[t%2][i+4][j-1][k+2]
            + coef[683] * A[t%2][i+4][j-1][k+3]
            + coef[684] * A[t%2][i+4][j-1][k+4]
            + coef[685] * A[t%2][i+4][j][k-4]
            + coef[686] * A[t%2][i+4][j][k-3]
            + coef[687] * A[t%2][i+4][j][k-2]
            + coef[688] * A[t%2][i+4][j][k-1]
            + coef[689] * A[t%2][i+4][j][k+1]
            + coef[690] * A[t%2][i+4][j][k+2]
            + coef[691] * A[t%2][i+4][j][k+3]
            + coef[692] * A[t%2][i+4][j][k+4]
            + coef[693] * A[t%2][i+4][j+1][k-4]
            + coef[694] * A[t%2][i+4][j+1][k-3]
            + coef[695] * A[t%2][i+4][j+1][k-2]
            + coef[696] * A[t%2][i+4][j+1][k-1]
            + coef[697] * A[t%2][i+4][j+1][k]
            + coef[698] * A[t%2][i+4][j+1][k+1]
            + coef[699] * A[t%2][i+4][j+1][k+2]
            + coef[700] * A[t%2][i+4][j+1][k+3]
            + coef[701] * A[t%2][i+4][j+1][k+4]
            + coef[702] * A[t%2][i+4][j+2][k-4]
            + coef[703] * A[t%2][i+4][j+2][k-3]
            + coef[704] * A[t%2][i+4][j+2][k-2]
            + coef[705] * A[t%2][i+4][j+2][k-1]
            + coef[706] * A[t%2][i+4][j+2][k]
            + coef[707] * A[t%2][i+4][j+2][k+1]
            + coef[708] * A[t%2][i+4][j+2][k+2]
            + coef[709] * A[t%2][i+4][j+2][k+3]
            + coef[710] * A[t%2][i+4][j+2][k+4]
            + coef[711] * A[t%2][i+4][j+3][k-4]
            + coef[712] * A[t%2][i+4][j+3][k-3]
            + coef[713] * A[t%2][i+4][j+3][k-2]
            + coef[714] * A[t%2][i+4][j+3][k-1]
            + coef[715] * A[t%2][i+4][j+3][k]
            + coef[716] * A[t%2][i+4][j+3][k+1]
            + coef[717] * A[t%2][i+4][j+3][k+2]
            + coef[718] * A[t%2][i+4][j+3][k+3]
            + coef[719] * A[t%2][i+4][j+3][k+4]
            + coef[720] * A[t%2][i+4][j+4][k-4]
            + coef[721] * A[t%2][i+4][j+4][k-3]
            + coef[722] * A[t%2][i+4][j+4][k-2]
            + coef[723] * A[t%2][i+4][j+4][k-1]
            + coef[724] * A[t%2][i+4][j+4][k]
            + coef[725] * A[t%2][i+4][j+4][k+1]
            + coef[726] * A[t%2][i+4][j+4][k+2]
            + coef[727] * A[t%2][i+4][j+4][k+3]
            + coef[728] * A[t%2][i+4][j+4][k+4];
  }
}

void oracle_j3d27pt_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            (coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1]) / divisor;
  }
}

void oracle_j3d27pt_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            (coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1]) / divisor;
  }
}

void oracle_j3d27pt_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 2, d1 = n[1] + 2, d2 = n[2] + 2;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 1; i < d0 - 1; i++)
      for (long j = 1; j < d1 - 1; j++)
        for (long k = 1; k < d2 - 1; k++)
          A[(t+1)%2][i][j][k] =
            (coef[0] * A[t%2][i-1][j][k]
            + coef[1] * A[t%2][i-1][j-1][k-1]
            + coef[2] * A[t%2][i-1][j-1][k]
            + coef[3] * A[t%2][i-1][j-1][k+1]
            + coef[4] * A[t%2][i-1][j][k-1]
            + coef[5] * A[t%2][i-1][j][k+1]
            + coef[6] * A[t%2][i-1][j+1][k-1]
            + coef[7] * A[t%2][i-1][j+1][k]
            + coef[8] * A[t%2][i-1][j+1][k+1]
            + coef[9] * A[t%2][i][j][k]
            + coef[10] * A[t%2][i][j-1][k-1]
            + coef[11] * A[t%2][i][j-1][k]
            + coef[12] * A[t%2][i][j-1][k+1]
            + coef[13] * A[t%2][i][j][k-1]
            + coef[14] * A[t%2][i][j][k+1]
            + coef[15] * A[t%2][i][j+1][k-1]
            + coef[16] * A[t%2][i][j+1][k]
            + coef[17] * A[t%2][i][j+1][k+1]
            + coef[18] * A[t%2][i+1][j][k]
            + coef[19] * A[t%2][i+1][j-1][k-1]
            + coef[20] * A[t%2][i+1][j-1][k]
            + coef[21] * A[t%2][i+1][j-1][k+1]
            + coef[22] * A[t%2][i+1][j][k-1]
            + coef[23] * A[t%2][i+1][j][k+1]
            + coef[24] * A[t%2][i+1][j+1][k-1]
            + coef[25] * A[t%2][i+1][j+1][k]
            + coef[26] * A[t%2][i+1][j+1][k+1]) / divisor;
  }
}

void oracle_3d125pt_f(float *A1, const int *n, int timestep,
    const float *coef, float divisor, float eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  float (*A)[d0][d1][d2] = (float (*)[d0][d1][d2])A1;
  const double c0 = coef ? (double)coef[0] : (double)0.75;
  const double c1 = coef ? (double)coef[16] : (double)0.76;
  const double c2 = coef ? (double)coef[20] : (double)1.132;
  const double c3 = coef ? (double)coef[50] : (double)0.217;
  const double c4 = coef ? (double)coef[70] : (double)2.13;
  const double c5 = coef ? (double)coef[95] : (double)0.331;
  const double c6 = coef ? (double)coef[121] : (double)0.332;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] = (float)(c0 * (float)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2] + A[t%2][i-1][j-1][k-1] + A[t%2][i-1][j-1][k+1] + A[t%2][i-1][j+1][k-1] + A[t%2][i-1][j+1][k+1] + A[t%2][i][j-1][k] + A[t%2][i][j][k-1] + A[t%2][i][j][k+1] + A[t%2][i][j+1][k] + A[t%2][i+1][j-1][k-1] + A[t%2][i+1][j-1][k+1] + A[t%2][i+1][j+1][k-1] + A[t%2][i+1][j+1][k+1])
            + c1 * (float)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2])
            + c2 * (float)(A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1] + A[t%2][i-1][j-2][k-2] + A[t%2][i-1][j-2][k+2] + A[t%2][i-1][j+2][k-2] + A[t%2][i-1][j+2][k+2] + A[t%2][i][j-2][k] + A[t%2][i][j][k-2] + A[t%2][i][j][k+2] + A[t%2][i][j+2][k] + A[t%2][i+1][j-2][k-2] + A[t%2][i+1][j-2][k+2] + A[t%2][i+1][j+2][k-2] + A[t%2][i+1][j+2][k+2] + A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1])
            + c3 * (float)(A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k] + A[t%2][i-1][j-1][k] + A[t%2][i-1][j][k-1] + A[t%2][i-1][j][k+1] + A[t%2][i-1][j+1][k] + A[t%2][i][j-2][k-2] + A[t%2][i][j-2][k+2] + A[t%2][i][j+2][k-2] + A[t%2][i][j+2][k+2] + A[t%2][i+1][j-1][k] + A[t%2][i+1][j][k-1] + A[t%2][i+1][j][k+1] + A[t%2][i+1][j+1][k] + A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k])
            + c4 * (float)(A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k] + A[t%2][i-1][j-2][k] + A[t%2][i-1][j][k-2] + A[t%2][i-1][j][k+2] + A[t%2][i-1][j+2][k] + A[t%2][i][j-2][k-1] + A[t%2][i][j-2][k+1] + A[t%2][i][j-1][k-2] + A[t%2][i][j-1][k+2] + A[t%2][i][j][k] + A[t%2][i][j+1][k-2] + A[t%2][i][j+1][k+2] + A[t%2][i][j+2][k-1] + A[t%2][i][j+2][k+1] + A[t%2][i+1][j-2][k] + A[t%2][i+1][j][k-2] + A[t%2][i+1][j][k+2] + A[t%2][i+1][j+2][k] + A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k])
            + c5 * (float)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1] + A[t%2][i-1][j-2][k-1] + A[t%2][i-1][j-2][k+1] + A[t%2][i-1][j-1][k-2] + A[t%2][i-1][j-1][k+2] + A[t%2][i-1][j][k] + A[t%2][i-1][j+1][k-2] + A[t%2][i-1][j+1][k+2] + A[t%2][i-1][j+2][k-1] + A[t%2][i-1][j+2][k+1] + A[t%2][i][j-1][k-1] + A[t%2][i][j-1][k+1] + A[t%2][i][j+1][k-1] + A[t%2][i][j+1][k+1] + A[t%2][i+1][j-2][k-1] + A[t%2][i+1][j-2][k+1] + A[t%2][i+1][j-1][k-2] + A[t%2][i+1][j-1][k+2] + A[t%2][i+1][j][k] + A[t%2][i+1][j+1][k-2] + A[t%2][i+1][j+1][k+2] + A[t%2][i+1][j+2][k-1] + A[t%2][i+1][j+2][k+1])
            + c6 * (float)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1]));
  }
}

void oracle_3d125pt_d(double *A1, const int *n, int timestep,
    const double *coef, double divisor, double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  double (*A)[d0][d1][d2] = (double (*)[d0][d1][d2])A1;
  const double c0 = coef ? (double)coef[0] : (double)0.75;
  const double c1 = coef ? (double)coef[16] : (double)0.76;
  const double c2 = coef ? (double)coef[20] : (double)1.132;
  const double c3 = coef ? (double)coef[50] : (double)0.217;
  const double c4 = coef ? (double)coef[70] : (double)2.13;
  const double c5 = coef ? (double)coef[95] : (double)0.331;
  const double c6 = coef ? (double)coef[121] : (double)0.332;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] = (double)(c0 * (double)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2] + A[t%2][i-1][j-1][k-1] + A[t%2][i-1][j-1][k+1] + A[t%2][i-1][j+1][k-1] + A[t%2][i-1][j+1][k+1] + A[t%2][i][j-1][k] + A[t%2][i][j][k-1] + A[t%2][i][j][k+1] + A[t%2][i][j+1][k] + A[t%2][i+1][j-1][k-1] + A[t%2][i+1][j-1][k+1] + A[t%2][i+1][j+1][k-1] + A[t%2][i+1][j+1][k+1])
            + c1 * (double)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2])
            + c2 * (double)(A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1] + A[t%2][i-1][j-2][k-2] + A[t%2][i-1][j-2][k+2] + A[t%2][i-1][j+2][k-2] + A[t%2][i-1][j+2][k+2] + A[t%2][i][j-2][k] + A[t%2][i][j][k-2] + A[t%2][i][j][k+2] + A[t%2][i][j+2][k] + A[t%2][i+1][j-2][k-2] + A[t%2][i+1][j-2][k+2] + A[t%2][i+1][j+2][k-2] + A[t%2][i+1][j+2][k+2] + A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1])
            + c3 * (double)(A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k] + A[t%2][i-1][j-1][k] + A[t%2][i-1][j][k-1] + A[t%2][i-1][j][k+1] + A[t%2][i-1][j+1][k] + A[t%2][i][j-2][k-2] + A[t%2][i][j-2][k+2] + A[t%2][i][j+2][k-2] + A[t%2][i][j+2][k+2] + A[t%2][i+1][j-1][k] + A[t%2][i+1][j][k-1] + A[t%2][i+1][j][k+1] + A[t%2][i+1][j+1][k] + A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k])
            + c4 * (double)(A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k] + A[t%2][i-1][j-2][k] + A[t%2][i-1][j][k-2] + A[t%2][i-1][j][k+2] + A[t%2][i-1][j+2][k] + A[t%2][i][j-2][k-1] + A[t%2][i][j-2][k+1] + A[t%2][i][j-1][k-2] + A[t%2][i][j-1][k+2] + A[t%2][i][j][k] + A[t%2][i][j+1][k-2] + A[t%2][i][j+1][k+2] + A[t%2][i][j+2][k-1] + A[t%2][i][j+2][k+1] + A[t%2][i+1][j-2][k] + A[t%2][i+1][j][k-2] + A[t%2][i+1][j][k+2] + A[t%2][i+1][j+2][k] + A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k])
            + c5 * (double)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1] + A[t%2][i-1][j-2][k-1] + A[t%2][i-1][j-2][k+1] + A[t%2][i-1][j-1][k-2] + A[t%2][i-1][j-1][k+2] + A[t%2][i-1][j][k] + A[t%2][i-1][j+1][k-2] + A[t%2][i-1][j+1][k+2] + A[t%2][i-1][j+2][k-1] + A[t%2][i-1][j+2][k+1] + A[t%2][i][j-1][k-1] + A[t%2][i][j-1][k+1] + A[t%2][i][j+1][k-1] + A[t%2][i][j+1][k+1] + A[t%2][i+1][j-2][k-1] + A[t%2][i+1][j-2][k+1] + A[t%2][i+1][j-1][k-2] + A[t%2][i+1][j-1][k+2] + A[t%2][i+1][j][k] + A[t%2][i+1][j+1][k-2] + A[t%2][i+1][j+1][k+2] + A[t%2][i+1][j+2][k-1] + A[t%2][i+1][j+2][k+1])
            + c6 * (double)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1]));
  }
}

void oracle_3d125pt_q(long double *A1, const int *n, int timestep,
    const long double *coef, long double divisor, long double eps)
{
  (void)eps; (void)divisor;
  const long d0 = n[0] + 4, d1 = n[1] + 4, d2 = n[2] + 4;
  long double (*A)[d0][d1][d2] = (long double (*)[d0][d1][d2])A1;
  const long double c0 = coef ? (long double)coef[0] : (long double)0.75;
  const long double c1 = coef ? (long double)coef[16] : (long double)0.76;
  const long double c2 = coef ? (long double)coef[20] : (long double)1.132;
  const long double c3 = coef ? (long double)coef[50] : (long double)0.217;
  const long double c4 = coef ? (long double)coef[70] : (long double)2.13;
  const long double c5 = coef ? (long double)coef[95] : (long double)0.331;
  const long double c6 = coef ? (long double)coef[121] : (long double)0.332;
  for (int t = 0; t < timestep; t++) {
#pragma omp parallel for schedule(static)
    for (long i = 2; i < d0 - 2; i++)
      for (long j = 2; j < d1 - 2; j++)
        for (long k = 2; k < d2 - 2; k++)
          A[(t+1)%2][i][j][k] = (long double)(c0 * (long double)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2] + A[t%2][i-1][j-1][k-1] + A[t%2][i-1][j-1][k+1] + A[t%2][i-1][j+1][k-1] + A[t%2][i-1][j+1][k+1] + A[t%2][i][j-1][k] + A[t%2][i][j][k-1] + A[t%2][i][j][k+1] + A[t%2][i][j+1][k] + A[t%2][i+1][j-1][k-1] + A[t%2][i+1][j-1][k+1] + A[t%2][i+1][j+1][k-1] + A[t%2][i+1][j+1][k+1])
            + c1 * (long double)(A[t%2][i-2][j-2][k-2] + A[t%2][i-2][j-2][k+2] + A[t%2][i-2][j+2][k-2] + A[t%2][i-2][j+2][k+2])
            + c2 * (long double)(A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1] + A[t%2][i-1][j-2][k-2] + A[t%2][i-1][j-2][k+2] + A[t%2][i-1][j+2][k-2] + A[t%2][i-1][j+2][k+2] + A[t%2][i][j-2][k] + A[t%2][i][j][k-2] + A[t%2][i][j][k+2] + A[t%2][i][j+2][k] + A[t%2][i+1][j-2][k-2] + A[t%2][i+1][j-2][k+2] + A[t%2][i+1][j+2][k-2] + A[t%2][i+1][j+2][k+2] + A[t%2][i-2][j-2][k-1] + A[t%2][i-2][j-2][k+1] + A[t%2][i-2][j-1][k-2] + A[t%2][i-2][j-1][k+2] + A[t%2][i-2][j][k] + A[t%2][i-2][j+1][k-2] + A[t%2][i-2][j+1][k+2] + A[t%2][i-2][j+2][k-1] + A[t%2][i-2][j+2][k+1])
            + c3 * (long double)(A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k] + A[t%2][i-1][j-1][k] + A[t%2][i-1][j][k-1] + A[t%2][i-1][j][k+1] + A[t%2][i-1][j+1][k] + A[t%2][i][j-2][k-2] + A[t%2][i][j-2][k+2] + A[t%2][i][j+2][k-2] + A[t%2][i][j+2][k+2] + A[t%2][i+1][j-1][k] + A[t%2][i+1][j][k-1] + A[t%2][i+1][j][k+1] + A[t%2][i+1][j+1][k] + A[t%2][i-2][j-2][k] + A[t%2][i-2][j][k-2] + A[t%2][i-2][j][k+2] + A[t%2][i-2][j+2][k])
            + c4 * (long double)(A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k] + A[t%2][i-1][j-2][k] + A[t%2][i-1][j][k-2] + A[t%2][i-1][j][k+2] + A[t%2][i-1][j+2][k] + A[t%2][i][j-2][k-1] + A[t%2][i][j-2][k+1] + A[t%2][i][j-1][k-2] + A[t%2][i][j-1][k+2] + A[t%2][i][j][k] + A[t%2][i][j+1][k-2] + A[t%2][i][j+1][k+2] + A[t%2][i][j+2][k-1] + A[t%2][i][j+2][k+1] + A[t%2][i+1][j-2][k] + A[t%2][i+1][j][k-2] + A[t%2][i+1][j][k+2] + A[t%2][i+1][j+2][k] + A[t%2][i-2][j-1][k] + A[t%2][i-2][j][k-1] + A[t%2][i-2][j][k+1] + A[t%2][i-2][j+1][k])
            + c5 * (long double)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1] + A[t%2][i-1][j-2][k-1] + A[t%2][i-1][j-2][k+1] + A[t%2][i-1][j-1][k-2] + A[t%2][i-1][j-1][k+2] + A[t%2][i-1][j][k] + A[t%2][i-1][j+1][k-2] + A[t%2][i-1][j+1][k+2] + A[t%2][i-1][j+2][k-1] + A[t%2][i-1][j+2][k+1] + A[t%2][i][j-1][k-1] + A[t%2][i][j-1][k+1] + A[t%2][i][j+1][k-1] + A[t%2][i][j+1][k+1] + A[t%2][i+1][j-2][k-1] + A[t%2][i+1][j-2][k+1] + A[t%2][i+1][j-1][k-2] + A[t%2][i+1][j-1][k+2] + A[t%2][i+1][j][k] + A[t%2][i+1][j+1][k-2] + A[t%2][i+1][j+1][k+2] + A[t%2][i+1][j+2][k-1] + A[t%2][i+1][j+2][k+1])
            + c6 * (long double)(A[t%2][i-2][j-1][k-1] + A[t%2][i-2][j-1][k+1] + A[t%2][i-2][j+1][k-1] + A[t%2][i-2][j+1][k+1]));
  }
}

typedef void (*oracle_fn_f)(float *, const int *, int, const float *, float, float);
const oracle_fn_f oracle_table_f[] = {
  oracle_star2d1r_f,
  oracle_star2d2r_f,
  oracle_star2d3r_f,
  oracle_star2d4r_f,
  oracle_box2d1r_f,
  oracle_box2d2r_f,
  oracle_box2d3r_f,
  oracle_box2d4r_f,
  oracle_j2d5pt_f,
  oracle_j2d9pt_f,
  oracle_j2d9pt_gol_f,
  oracle_gradient2d_f,
  oracle_star3d1r_f,
  oracle_star3d2r_f,
  oracle_star3d3r_f,
  oracle_star3d4r_f,
  oracle_box3d1r_f,
  oracle_box3d2r_f,
  oracle_box3d3r_f,
  oracle_box3d4r_f,
  oracle_j3d27pt_f,
  oracle_3d125pt_f,
};

typedef void (*oracle_fn_d)(double *, const int *, int, const double *, double, double);
const oracle_fn_d oracle_table_d[] = {
  oracle_star2d1r_d,
  oracle_star2d2r_d,
  oracle_star2d3r_d,
  oracle_star2d4r_d,
  oracle_box2d1r_d,
  oracle_box2d2r_d,
  oracle_box2d3r_d,
  oracle_box2d4r_d,
  oracle_j2d5pt_d,
  oracle_j2d9pt_d,
  oracle_j2d9pt_gol_d,
  oracle_gradient2d_d,
  oracle_star3d1r_d,
  oracle_star3d2r_d,
  oracle_star3d3r_d,
  oracle_star3d4r_d,
  oracle_box3d1r_d,
  oracle_box3d2r_d,
  oracle_box3d3r_d,
  oracle_box3d4r_d,
  oracle_j3d27pt_d,
  oracle_3d125pt_d,
};

typedef void (*oracle_fn_q)(long double *, const int *, int, const long double *, long double, long double);
const oracle_fn_q oracle_table_q[] = {
  oracle_star2d1r_q,
  oracle_star2d2r_q,
  oracle_star2d3r_q,
  oracle_star2d4r_q,
  oracle_box2d1r_q,
  oracle_box2d2r_q,
  oracle_box2d3r_q,
  oracle_box2d4r_q,
  oracle_j2d5pt_q,
  oracle_j2d9pt_q,
  oracle_j2d9pt_gol_q,
  oracle_gradient2d_q,
  oracle_star3d1r_q,
  oracle_star3d2r_q,
  oracle_star3d3r_q,
  oracle_star3d4r_q,
  oracle_box3d1r_q,
  oracle_box3d2r_q,
  oracle_box3d3r_q,
  oracle_box3d4r_q,
  oracle_j3d27pt_q,
  oracle_3d125pt_q,
};
