/* A C program written against the reference's API only (vnec_gb300.h restates
 * OpenSparseBLAS.h's types and entry points), following the reference harness's
 * flow (src/operation/test/test_spmv_vnec.cpp:140-275): build a CSR SpB_Matrix
 * in place, pick the format with IRD_VNEC (VNEC-L for n >= 3e6 rows), build the
 * handle, run SpMV_VNEC_* on host vectors, compare with a serial loop
 * (test_spmv_vnec.hpp:57-79), free the handle.  Also runs SpB_mxv with a NULL
 * handle, the known-answer pattern A_ij = i, x_j = j (exact in any order) and
 * pipelined host calls.  Prints one line per check; exits non-zero on failure.
 *
 *   c_harness <n_rows> <nnz_per_row> <seed>
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vnec_gb300.h"

static uint64_t rng_state;
static uint64_t rng_next(void) { /* splitmix64 */
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double rng_unit(void) { return (double)(rng_next() >> 11) * (1.0 / 9007199254740992.0); }

static int cmp_index(const void *a, const void *b) {
  const SpB_Index x = *(const SpB_Index *)a, y = *(const SpB_Index *)b;
  return x < y ? -1 : x > y;
}

/* Rows of exactly k distinct sorted columns (k <= n), values U(-1, 1). */
static SpB_Matrix_CSC_or_CSR *make_matrix(SpB_Index n, int k) {
  SpB_Matrix_CSC_or_CSR *A = calloc(1, sizeof(*A));
  A->matrix_base.element_type = SpB_FP64;
  A->matrix_base.format_type = SpB_CSR;
  A->matrix_base.row = n;
  A->matrix_base.col = n;
  A->matrix_base.element_size = sizeof(double);
  A->nnz = n * (SpB_Index)k;
  A->capacity = A->nnz;
  A->ptr_len = n + 1;
  A->ptr = malloc(sizeof(SpB_Index) * (n + 1));
  A->indices = malloc(sizeof(SpB_Index) * (A->nnz ? A->nnz : 1));
  A->val = malloc(sizeof(double) * (A->nnz ? A->nnz : 1));
  double *v = A->val;
  for (SpB_Index r = 0; r <= n; ++r) A->ptr[r] = r * (SpB_Index)k;
  for (SpB_Index r = 0; r < n; ++r) {
    SpB_Index *c = A->indices + r * (SpB_Index)k;
    for (int j = 0; j < k; ++j) {
      int fresh;
      do { /* distinct columns */
        c[j] = rng_next() % n;
        fresh = 1;
        for (int i = 0; i < j; ++i) fresh &= c[i] != c[j];
      } while (!fresh);
    }
    qsort(c, (size_t)k, sizeof(SpB_Index), cmp_index);
    for (int j = 0; j < k; ++j) v[r * (SpB_Index)k + (SpB_Index)j] = 2.0 * rng_unit() - 1.0;
  }
  return A;
}

static void free_matrix(SpB_Matrix_CSC_or_CSR *A) {
  free(A->ptr);
  free(A->indices);
  free(A->val);
  free(A);
}

static SpB_Vector_Dense *make_vector(SpB_Index n) {
  SpB_Vector_Dense *v = calloc(1, sizeof(*v));
  v->vector_base.element_type = SpB_FP64;
  v->vector_base.format_type = SpB_DENSE;
  v->vector_base.n = n;
  v->vector_base.element_size = sizeof(double);
  v->values = calloc(n ? n : 1, sizeof(double));
  return v;
}

/* The serial loop of the reference's test, with the row's sum of |a x| for
 * the row-wise criterion. */
static void serial(const SpB_Matrix_CSC_or_CSR *A, const double *x, double *y, double *cond) {
  const double *v = A->val;
  for (SpB_Index r = 0; r + 1 < A->ptr_len; ++r) {
    double s = 0.0, c = 0.0;
    for (SpB_Index q = A->ptr[r]; q < A->ptr[r + 1]; ++q) {
      s += v[q] * x[A->indices[q]];
      c += fabs(v[q] * x[A->indices[q]]);
    }
    y[r] = s;
    cond[r] = c;
  }
}

static int check(const char *what, const double *y, const double *ref, const double *cond, SpB_Index n,
                 double tol) {
  double worst = 0.0;
  for (SpB_Index i = 0; i < n; ++i) {
    const double e = fabs(y[i] - ref[i]) / (cond[i] > 0 ? cond[i] : 1.0);
    if (!(e <= worst)) worst = e; /* NaN propagates */
  }
  const int ok = worst <= tol;
  printf("%s %s: max row-wise error %.3e (bound %.0e)\n", ok ? "ok  " : "FAIL", what, worst, tol);
  return ok;
}

int main(int argc, char **argv) {
  const SpB_Index n = argc > 1 ? (SpB_Index)strtoull(argv[1], NULL, 10) : 100000;
  const int k = argc > 2 ? atoi(argv[2]) : 16;
  rng_state = argc > 3 ? strtoull(argv[3], NULL, 10) : 1;
  int ok = 1;

  SpB_Matrix_CSC_or_CSR *A = make_matrix(n, k);
  SpB_Matrix M = (SpB_Matrix)A;
  SpB_Vector_Dense *x = make_vector(n), *y = make_vector(n);
  double *xv = x->values, *ref = malloc(sizeof(double) * n), *cond = malloc(sizeof(double) * n);
  for (SpB_Index i = 0; i < n; ++i) xv[i] = 2.0 * rng_unit() - 1.0;
  serial(A, xv, ref, cond);

  /* The harness's dispatch. */
  if (n >= 3000000) {
    VNEC_L *h = Build_VNEC_L(M);
    ok &= h != NULL;
    if (h) {
      SpMV_VNEC_L_FP64((SpB_Vector)y, M, (SpB_Vector)x, h);
      ok &= check("IRD dispatch -> VNEC-L", y->values, ref, cond, n, 1e-12);
      VNEC_L_free_ext(h);
    }
  } else if (IRD_VNEC(M, SpB_FP64) == SpB_VNEC_D) {
    VNEC_D_FP64 *h = Build_VNEC_D_FP64(M);
    ok &= h != NULL;
    if (h) {
      SpMV_VNEC_D_FP64((SpB_Vector)y, M, (SpB_Vector)x, h);
      ok &= check("IRD dispatch -> VNEC-D", y->values, ref, cond, n, 1e-12);
      VNEC_D_free_fp64(h);
    }
  } else {
    VNEC_S_FP64 *h = Build_VNEC_S_FP64(M);
    ok &= h != NULL;
    if (h) {
      SpMV_VNEC_S_FP64((SpB_Vector)y, M, (SpB_Vector)x, h);
      ok &= check("IRD dispatch -> VNEC-S", y->values, ref, cond, n, 1e-12);
      VNEC_S_free_fp64(h);
    }
  }

  /* SpB_mxv with a NULL handle: automatic selection, plan cached against A. */
  memset(y->values, 0, sizeof(double) * n);
  ok &= SpB_mxv((SpB_Vector)y, M, (SpB_Vector)x, NULL) == SpB_SUCCESS;
  ok &= check("SpB_mxv (NULL handle)", y->values, ref, cond, n, 1e-12);

  /* Pipelined host calls on an explicit plan: four right-hand sides. */
  {
    SpB_VNEC_options_ext o;
    memset(&o, 0, sizeof(o));
    o.kernel = SpB_VNEC_KERNEL_S;
    void *plan = SpB_VNEC_plan_matrix_ext(&o, M);
    ok &= plan != NULL;
    if (plan) {
      double *xs = malloc(sizeof(double) * n * 4), *ys = malloc(sizeof(double) * n * 4);
      for (SpB_Index i = 0; i < n * 4; ++i) xs[i] = 2.0 * rng_unit() - 1.0;
      for (int r = 0; r < 4; ++r) ok &= SpB_mxv_host_async_ext(plan, xs + n * r, ys + n * r) == SpB_SUCCESS;
      ok &= SpB_VNEC_host_wait_ext(plan) == SpB_SUCCESS;
      for (int r = 0; r < 4; ++r) {
        serial(A, xs + n * r, ref, cond);
        ok &= check("SpB_mxv_host_async_ext", ys + n * r, ref, cond, n, 1e-12);
      }
      free(xs);
      free(ys);
      SpB_VNEC_plan_free_ext(plan);
    }
  }

  /* Known-answer pattern of the reference's test (test_spmv_vnec.cpp:169,185):
   * A_ij = i, x_j = j gives exact integers, equal bit for bit in any order. */
  {
    double *v = A->val;
    for (SpB_Index r = 0; r < n; ++r)
      for (SpB_Index q = A->ptr[r]; q < A->ptr[r + 1]; ++q) v[q] = (double)r;
    for (SpB_Index i = 0; i < n; ++i) xv[i] = (double)i;
    SpB_VNEC_forget_ext(M); /* A changed in place */
    serial(A, xv, ref, cond);
    ok &= SpB_mxv((SpB_Vector)y, M, (SpB_Vector)x, NULL) == SpB_SUCCESS;
    const double *yv = y->values;
    SpB_Index bad = 0;
    for (SpB_Index i = 0; i < n; ++i) bad += yv[i] != ref[i];
    printf("%s known-answer A_ij = i, x_j = j: %lu rows differ\n", bad ? "FAIL" : "ok  ", (unsigned long)bad);
    ok &= bad == 0;
  }

  if (!ok) printf("last error: %s\n", SpB_VNEC_last_error_ext());
  SpB_VNEC_forget_ext(M);
  free(ref);
  free(cond);
  free(x->values);
  free(x);
  free(y->values);
  free(y);
  free_matrix(A);
  return ok ? 0 : 1;
}
