/* CPU oracle for the dense Cholesky (LLT) path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only the test suite, the smoke
 * check and the CPU-baseline / reference legs of the benchmark load it.  The GPU product never
 * links, loads or calls it.
 *
 * Contents
 *   - Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
 *     numbers: as easy as 1, 2, 3", SC'11) and Box-Muller normals: the seeded input source
 *     shared with the GPU workload generator.
 *   - Generators for the synthetic workloads (G G^T/n + I; Householder-spectrum matrices;
 *     uneven batches; RBF kernel matrices).
 *   - A plain-C restatement of Eigen's LLT: llt_inplace<Scalar,Lower>::{unblocked,blocked}
 *     (Eigen/src/Cholesky/LLT.h:312-368), the Upper variant (:377-399), the LAPACK wrappers
 *     (lapack/cholesky.cpp:14-72) and the two-sweep solve (LLT.h:483-498), for double and float.
 *   - A double-double normwise backward error.
 *   - Batched variable-size factor+solve (OpenMP over systems).
 *
 * Parity pin: tests/golden holds factors and solutions produced by Eigen itself (compiled from
 * the reference headers by oracle/build_ref.sh) and the test suite checks this restatement
 * against them.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------------------------
 * Philox-4x32-10 (published algorithm; constants from the SC'11 paper / Random123).
 * ------------------------------------------------------------------------------------------ */
static inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
  /* 10 rounds with the key bumped between rounds: the last bump is unused. */
  out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
}

/* Two 32-bit words -> a 53-bit uniform in [0, 1). */
static inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* Element `idx` of the N(0,1) stream `seed`.  Elements 2p and 2p+1 are the cosine and sine
 * halves of one Box-Muller pair drawn from counter (p_lo, p_hi, 0, 0), key (seed_lo, seed_hi). */
double oracle_normal(uint64_t seed, uint64_t idx) {
  const uint64_t p = idx >> 1;
  const uint32_t ctr[4] = {(uint32_t)p, (uint32_t)(p >> 32), 0u, 0u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  oracle_philox4x32_10(ctr, key, r);
  const double u1 = 1.0 - u53(r[0], r[1]); /* (0, 1] */
  const double u2 = u53(r[2], r[3]);
  const double rad = sqrt(-2.0 * log(u1));
  return (idx & 1) ? rad * sin(2.0 * M_PI * u2) : rad * cos(2.0 * M_PI * u2);
}

/* Element `idx` of the U[0,1) stream `seed` (counter lane 2 set to 1, so it never collides
 * with the normal stream of the same seed). */
double oracle_uniform(uint64_t seed, uint64_t idx) {
  const uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), 1u, 0u};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  oracle_philox4x32_10(ctr, key, r);
  return u53(r[0], r[1]);
}

void oracle_fill_normal(uint64_t seed, uint64_t offset, int64_t count, double* out) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t i = 0; i < count; ++i) out[i] = oracle_normal(seed, offset + (uint64_t)i);
}

void oracle_fill_uniform(uint64_t seed, uint64_t offset, int64_t count, double* out) {
  for (int64_t i = 0; i < count; ++i) out[i] = oracle_uniform(seed, offset + (uint64_t)i);
}

/* ------------------------------------------------------------------------------------------
 * Workload generators (column-major, full symmetric matrices).
 * ------------------------------------------------------------------------------------------ */

/* A = G G^T / n + shift * I, G n x n with G(i,j) = normal(seed, offset + i + j*n). */
void oracle_gen_gram(int64_t n, uint64_t seed, uint64_t offset, double shift, double* a, int64_t lda) {
  double* g = (double*)malloc((size_t)(n * n) * sizeof(double));
  oracle_fill_normal(seed, offset, n * n, g);
  /* rows of G are strided; form G^T once so that both operands of each dot are contiguous */
  double* gt = (double*)malloc((size_t)(n * n) * sizeof(double));
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) gt[j + i * n] = g[i + j * n];
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8)
#endif
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = j; i < n; ++i) {
      const double* ri = gt + i * n;
      const double* rj = gt + j * n;
      double s = 0;
      for (int64_t p = 0; p < n; ++p) s += ri[p] * rj[p];
      s /= (double)n;
      if (i == j) s += shift;
      a[i + j * lda] = s;
      a[j + i * lda] = s;
    }
  free(g);
  free(gt);
}

/* Spectrum of the Householder construction: lambda_j = kappa^(-1 + j/(n-1)) (log-spaced over
 * [1/kappa, 1]), then permuted by sorting the keys uniform(perm_seed, j). */
static int cmp_key(const void* x, const void* y) {
  const double a = ((const double*)x)[0], b = ((const double*)y)[0];
  return a < b ? -1 : a > b ? 1 : 0;
}

void oracle_spectrum(int64_t n, double kappa, uint64_t perm_seed, double* lam) {
  double* kv = (double*)malloc((size_t)(2 * n) * sizeof(double));
  for (int64_t j = 0; j < n; ++j) {
    kv[2 * j] = oracle_uniform(perm_seed, (uint64_t)j);
    kv[2 * j + 1] = n > 1 ? pow(kappa, -1.0 + (double)j / (double)(n - 1)) : 1.0;
  }
  qsort(kv, (size_t)n, 2 * sizeof(double), cmp_key);
  for (int64_t j = 0; j < n; ++j) lam[j] = kv[2 * j + 1];
  free(kv);
}

/* A = Q diag(lam) Q^T with Q = H_1 ... H_r, H_i = I - 2 v_i v_i^T / |v_i|^2 and
 * v_i(j) = normal(v_seed0 + i, j) for i = 1..r.  H_r is applied first (A <- H A H), H_1 last.
 * H A H = A - v w^T - w v^T with beta = 2/|v|^2, p = beta A v, w = p - (beta/2)(v^T p) v. */
void oracle_gen_householder(int64_t n, int nrefl, uint64_t v_seed0, const double* lam,
                            double* a, int64_t lda) {
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) a[i + j * lda] = 0.0;
    a[j + j * lda] = lam[j];
  }
  double* v = (double*)malloc((size_t)n * sizeof(double));
  double* p = (double*)malloc((size_t)n * sizeof(double));
  for (int r = nrefl; r >= 1; --r) {
    oracle_fill_normal(v_seed0 + (uint64_t)r, 0, n, v);
    double vv = 0;
    for (int64_t i = 0; i < n; ++i) vv += v[i] * v[i];
    const double beta = 2.0 / vv;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t i = 0; i < n; ++i) {
      double s = 0;
      for (int64_t j = 0; j < n; ++j) s += a[j + i * lda] * v[j]; /* A symmetric: row i = col i */
      p[i] = beta * s;
    }
    double vp = 0;
    for (int64_t i = 0; i < n; ++i) vp += v[i] * p[i];
    const double kk = 0.5 * beta * vp;
    for (int64_t i = 0; i < n; ++i) p[i] -= kk * v[i]; /* p := w */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i) a[i + j * lda] -= v[i] * p[j] + p[i] * v[j];
  }
  free(v);
  free(p);
}

/* Sizes of the uneven batch: n_i = lo + floor(uniform(seed, i) * (hi - lo + 1)). */
void oracle_batch_sizes(int64_t count, uint64_t seed, int64_t lo, int64_t hi, int64_t* sizes) {
  for (int64_t i = 0; i < count; ++i) {
    int64_t v = lo + (int64_t)(oracle_uniform(seed, (uint64_t)i) * (double)(hi - lo + 1));
    if (v > hi) v = hi;
    sizes[i] = v;
  }
}

/* RBF kernel matrix over m points x_j in [0,1]^3 with x_j(d) = uniform(seed, offset + 3j + d):
 * A(i,j) = sigma2 * exp(-|x_i - x_j|^2 / (2 ell^2)) + noise * [i == j]. */
void oracle_gen_rbf(int64_t m, uint64_t seed, uint64_t offset, double ell, double sigma2, double noise,
                    double* a, int64_t lda) {
  double* x = (double*)malloc((size_t)(3 * m) * sizeof(double));
  oracle_fill_uniform(seed, offset, 3 * m, x);
  const double inv = 1.0 / (2.0 * ell * ell);
  for (int64_t j = 0; j < m; ++j)
    for (int64_t i = 0; i < m; ++i) {
      const double d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1], d2 = x[3 * i + 2] - x[3 * j + 2];
      double v = sigma2 * exp(-(d0 * d0 + d1 * d1 + d2 * d2) * inv);
      if (i == j) v += noise;
      a[i + j * lda] = v;
    }
  free(x);
}

/* ------------------------------------------------------------------------------------------
 * LLT restatement for double and float.
 * ------------------------------------------------------------------------------------------ */
#define T double
#define P(x) oracle_d##x
#include "llt_oracle_body.h"
#undef T
#undef P

#define T float
#define P(x) oracle_s##x
#include "llt_oracle_body.h"
#undef T
#undef P

/* ------------------------------------------------------------------------------------------
 * Batched variable-size factor + solve: system s is the lower column-major n_s x n_s block at
 * a + aoff[s] (leading dimension n_s) and its right-hand side at b + boff[s].  Each system runs
 * the blocked LLT followed by the two-sweep solve; systems are spread over OpenMP threads
 * (the fair multicore baseline for many independent small systems).  info[s] is the LAPACK
 * info of system s (0 ok, k+1 = failing column k).
 * ------------------------------------------------------------------------------------------ */
void oracle_dbatched_posv(int64_t count, const int64_t* ns, const int64_t* aoff, const int64_t* boff,
                          double* a, double* b, int64_t* info) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t s = 0; s < count; ++s) {
    const int64_t n = ns[s];
    double* as = a + aoff[s];
    const int64_t ret = n > 0 ? oracle_dllt_blocked(n, as, 1, n) : -1;
    info[s] = ret >= 0 ? ret + 1 : 0;
    if (ret < 0 && n > 0) oracle_dpotrs('L', n, 1, as, n, b + boff[s], n);
  }
}

void oracle_sbatched_posv(int64_t count, const int64_t* ns, const int64_t* aoff, const int64_t* boff,
                          float* a, float* b, int64_t* info) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t s = 0; s < count; ++s) {
    const int64_t n = ns[s];
    float* as = a + aoff[s];
    const int64_t ret = n > 0 ? oracle_sllt_blocked(n, as, 1, n) : -1;
    info[s] = ret >= 0 ? ret + 1 : 0;
    if (ret < 0 && n > 0) oracle_spotrs('L', n, 1, as, n, b + boff[s], n);
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}
