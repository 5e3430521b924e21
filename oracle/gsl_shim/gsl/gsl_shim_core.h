/*
 * Minimal GSL-compatible shim, written for this project so that the
 * reference JURASSIC sources (which include <gsl/...>) compile in a
 * container without GSL.  TEST INFRASTRUCTURE ONLY: this header is used to
 * build the reference-as-oracle library under oracle/_ref and nothing in the
 * product links it.
 *
 * Only the symbols the reference forward model, Jacobian and retrieval use
 * are provided: vector/matrix containers, naive BLAS (ddot, dgemv, dgemm),
 * an unblocked Cholesky factorisation/solve/inverse, min/max statistics,
 * log1p/expm1 and a tiny uniform RNG.  Summation orders are the textbook
 * ones, so retrieval results agree with a GSL/CBLAS build to rounding level.
 */
#ifndef JGB_GSL_SHIM_CORE_H
#define JGB_GSL_SHIM_CORE_H

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  size_t size;
  size_t stride;
  double *data;
  void *block;
  int owner;
} gsl_vector;

typedef struct {
  size_t size1;
  size_t size2;
  size_t tda;
  double *data;
  void *block;
  int owner;
} gsl_matrix;

typedef enum { CblasNoTrans = 111, CblasTrans = 112 } CBLAS_TRANSPOSE_t;

/* ---------------- containers ---------------- */

static inline gsl_vector *gsl_vector_alloc(size_t n) {
  gsl_vector *v = (gsl_vector *) malloc(sizeof(gsl_vector));
  v->size = n;
  v->stride = 1;
  v->data = (double *) calloc(n ? n : 1, sizeof(double));
  v->block = NULL;
  v->owner = 1;
  return v;
}

static inline void gsl_vector_free(gsl_vector *v) {
  if (!v)
    return;
  free(v->data);
  free(v);
}

static inline double gsl_vector_get(const gsl_vector *v, size_t i) {
  return v->data[i * v->stride];
}

static inline void gsl_vector_set(gsl_vector *v, size_t i, double x) {
  v->data[i * v->stride] = x;
}

static inline int gsl_vector_memcpy(gsl_vector *dst, const gsl_vector *src) {
  for (size_t i = 0; i < src->size; i++)
    dst->data[i * dst->stride] = src->data[i * src->stride];
  return 0;
}

static inline int gsl_vector_add(gsl_vector *a, const gsl_vector *b) {
  for (size_t i = 0; i < a->size; i++)
    a->data[i * a->stride] += b->data[i * b->stride];
  return 0;
}

static inline int gsl_vector_sub(gsl_vector *a, const gsl_vector *b) {
  for (size_t i = 0; i < a->size; i++)
    a->data[i * a->stride] -= b->data[i * b->stride];
  return 0;
}

static inline gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2) {
  gsl_matrix *m = (gsl_matrix *) malloc(sizeof(gsl_matrix));
  m->size1 = n1;
  m->size2 = n2;
  m->tda = n2;
  m->data = (double *) calloc((n1 * n2) ? n1 * n2 : 1, sizeof(double));
  m->block = NULL;
  m->owner = 1;
  return m;
}

static inline void gsl_matrix_free(gsl_matrix *m) {
  if (!m)
    return;
  free(m->data);
  free(m);
}

static inline double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j) {
  return m->data[i * m->tda + j];
}

static inline void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j,
                                  double x) {
  m->data[i * m->tda + j] = x;
}

static inline void gsl_matrix_set_zero(gsl_matrix *m) {
  for (size_t i = 0; i < m->size1; i++)
    for (size_t j = 0; j < m->size2; j++)
      m->data[i * m->tda + j] = 0.0;
}

static inline int gsl_matrix_memcpy(gsl_matrix *dst, const gsl_matrix *src) {
  for (size_t i = 0; i < src->size1; i++)
    for (size_t j = 0; j < src->size2; j++)
      dst->data[i * dst->tda + j] = src->data[i * src->tda + j];
  return 0;
}

static inline int gsl_matrix_add(gsl_matrix *a, const gsl_matrix *b) {
  for (size_t i = 0; i < a->size1; i++)
    for (size_t j = 0; j < a->size2; j++)
      a->data[i * a->tda + j] += b->data[i * b->tda + j];
  return 0;
}

static inline int gsl_matrix_scale(gsl_matrix *a, double s) {
  for (size_t i = 0; i < a->size1; i++)
    for (size_t j = 0; j < a->size2; j++)
      a->data[i * a->tda + j] *= s;
  return 0;
}

/* ---------------- BLAS (textbook loop order) ---------------- */

static inline int gsl_blas_ddot(const gsl_vector *x, const gsl_vector *y,
                                double *r) {
  double s = 0.0;
  for (size_t i = 0; i < x->size; i++)
    s += x->data[i * x->stride] * y->data[i * y->stride];
  *r = s;
  return 0;
}

/* y = alpha op(A) x + beta y */
static inline int gsl_blas_dgemv(CBLAS_TRANSPOSE_t ta, double alpha,
                                 const gsl_matrix *a, const gsl_vector *x,
                                 double beta, gsl_vector *y) {
  if (ta == CblasNoTrans) {
    for (size_t i = 0; i < a->size1; i++) {
      double s = 0.0;
      for (size_t j = 0; j < a->size2; j++)
        s += a->data[i * a->tda + j] * x->data[j * x->stride];
      y->data[i * y->stride] = alpha * s + beta * y->data[i * y->stride];
    }
  } else {
    for (size_t j = 0; j < a->size2; j++) {
      double s = 0.0;
      for (size_t i = 0; i < a->size1; i++)
        s += a->data[i * a->tda + j] * x->data[i * x->stride];
      y->data[j * y->stride] = alpha * s + beta * y->data[j * y->stride];
    }
  }
  return 0;
}

/* C = alpha op(A) op(B) + beta C */
static inline int gsl_blas_dgemm(CBLAS_TRANSPOSE_t ta, CBLAS_TRANSPOSE_t tb,
                                 double alpha, const gsl_matrix *a,
                                 const gsl_matrix *b, double beta,
                                 gsl_matrix *c) {
  const size_t m = c->size1, n = c->size2;
  const size_t k = (ta == CblasNoTrans) ? a->size2 : a->size1;
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < n; j++) {
      double s = 0.0;
      for (size_t l = 0; l < k; l++) {
        const double av = (ta == CblasNoTrans) ? a->data[i * a->tda + l]
                                               : a->data[l * a->tda + i];
        const double bv = (tb == CblasNoTrans) ? b->data[l * b->tda + j]
                                               : b->data[j * b->tda + l];
        s += av * bv;
      }
      c->data[i * c->tda + j] = alpha * s + beta * c->data[i * c->tda + j];
    }
  return 0;
}

/* ---------------- Cholesky ---------------- */

/* Lower factor L in the lower triangle, L^T mirrored into the upper one
   (the storage convention GSL documents for gsl_linalg_cholesky_decomp). */
static inline int gsl_linalg_cholesky_decomp(gsl_matrix *a) {
  const size_t n = a->size1;
  for (size_t j = 0; j < n; j++) {
    double d = a->data[j * a->tda + j];
    for (size_t k = 0; k < j; k++)
      d -= a->data[j * a->tda + k] * a->data[j * a->tda + k];
    if (d <= 0.0) {
      fprintf(stderr, "gsl shim: matrix not positive definite\n");
      exit(EXIT_FAILURE);
    }
    const double ljj = sqrt(d);
    a->data[j * a->tda + j] = ljj;
    for (size_t i = j + 1; i < n; i++) {
      double s = a->data[i * a->tda + j];
      for (size_t k = 0; k < j; k++)
        s -= a->data[i * a->tda + k] * a->data[j * a->tda + k];
      a->data[i * a->tda + j] = s / ljj;
    }
  }
  for (size_t i = 0; i < n; i++)
    for (size_t j = i + 1; j < n; j++)
      a->data[i * a->tda + j] = a->data[j * a->tda + i];
  return 0;
}

static inline int gsl_linalg_cholesky_solve(const gsl_matrix *l,
                                            const gsl_vector *b,
                                            gsl_vector *x) {
  const size_t n = l->size1;
  for (size_t i = 0; i < n; i++)
    x->data[i * x->stride] = b->data[i * b->stride];
  for (size_t i = 0; i < n; i++) {
    double s = x->data[i * x->stride];
    for (size_t k = 0; k < i; k++)
      s -= l->data[i * l->tda + k] * x->data[k * x->stride];
    x->data[i * x->stride] = s / l->data[i * l->tda + i];
  }
  for (size_t ii = n; ii-- > 0;) {
    double s = x->data[ii * x->stride];
    for (size_t k = ii + 1; k < n; k++)
      s -= l->data[k * l->tda + ii] * x->data[k * x->stride];
    x->data[ii * x->stride] = s / l->data[ii * l->tda + ii];
  }
  return 0;
}

/* Inverse from the factor: solve L L^T X = I column by column. */
static inline int gsl_linalg_cholesky_invert(gsl_matrix *l) {
  const size_t n = l->size1;
  gsl_matrix *inv = gsl_matrix_alloc(n, n);
  gsl_vector *e = gsl_vector_alloc(n), *col = gsl_vector_alloc(n);
  for (size_t j = 0; j < n; j++) {
    for (size_t i = 0; i < n; i++)
      e->data[i] = (i == j) ? 1.0 : 0.0;
    gsl_linalg_cholesky_solve(l, e, col);
    for (size_t i = 0; i < n; i++)
      inv->data[i * n + j] = col->data[i];
  }
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < n; j++)
      l->data[i * l->tda + j] = 0.5 * (inv->data[i * n + j] + inv->data[j * n + i]);
  gsl_matrix_free(inv);
  gsl_vector_free(e);
  gsl_vector_free(col);
  return 0;
}

/* ---------------- statistics ---------------- */

static inline void gsl_stats_minmax(double *mn, double *mx, const double *d,
                                    size_t stride, size_t n) {
  double lo = d[0], hi = d[0];
  for (size_t i = 0; i < n; i++) {
    const double x = d[i * stride];
    if (x < lo)
      lo = x;
    if (x > hi)
      hi = x;
    if (isnan(x)) {
      lo = hi = x;
      break;
    }
  }
  *mn = lo;
  *mx = hi;
}

static inline size_t gsl_stats_min_index(const double *d, size_t stride,
                                         size_t n) {
  double lo = d[0];
  size_t idx = 0;
  for (size_t i = 0; i < n; i++) {
    const double x = d[i * stride];
    if (x < lo) {
      lo = x;
      idx = i;
    }
    if (isnan(x))
      return i;
  }
  return idx;
}

/* ---------------- math ---------------- */

static inline double gsl_log1p(double x) { return log1p(x); }
static inline double gsl_expm1(double x) { return expm1(x); }

/* ---------------- random numbers (used by a timing task only) ---------- */

typedef struct {
  uint64_t s;
} gsl_rng;
typedef int gsl_rng_type;
static const gsl_rng_type gsl_rng_default_type = 0;
#define gsl_rng_default (&gsl_rng_default_type)

static inline void gsl_rng_env_setup(void) {}

static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) {
  (void) t;
  gsl_rng *r = (gsl_rng *) malloc(sizeof(gsl_rng));
  r->s = 0x9E3779B97F4A7C15ull;
  return r;
}

static inline double gsl_rng_uniform(gsl_rng *r) {
  r->s ^= r->s << 13;
  r->s ^= r->s >> 7;
  r->s ^= r->s << 17;
  return (double) (r->s >> 11) * (1.0 / 9007199254740992.0);
}

#endif
