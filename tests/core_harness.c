/* The reference harness's flow (src/operation/test/test_spmv_vnec.cpp:140-275)
 * on objects made by the reference's OWN core library: this file is linked
 * with the reference's core sources (src/core/src, compiled from the reference's
 * sources) and with libvnec_gb300.so in place of the reference's operation
 * module.  It includes the reference's OpenSparseBLAS.h, so every type and
 * constructor is the reference's, and calls, in order:
 *
 *   SpB_init; SpB_Global_Option_set_ext(SpB_MATRIX_FORMAT, CSR);
 *   SpB_Matrix_new + SpB_Matrix_build_FP64 (COO -> CSR by the reference's
 *     build, src/core/src/SpB_Matrix_CSC_or_CSR.c:188-256) with A_ij = i;
 *   SpB_Vector_new + SpB_Vector_setElement_FP64 with x_j = j;
 *   a serial CSR loop (test_spmv_vnec.hpp:57-79) for the expected y;
 *   n_rows < 3,000,000: IRD_VNEC, then Build/SpMV_VNEC_D_FP64 or _S_FP64 and
 *     VNEC_D_free_fp64 / VNEC_S_free_fp64; otherwise Build_VNEC_L +
 *     SpMV_VNEC_L_FP64 and the harness's field-by-field release of the handle
 *     (:246-251) — all served by libvnec_gb300.so on the GPU;
 *   the harness's per-row check |y_i - y*_i| <= 1e-8 y*_i (:261-269), and
 *     here also bit equality (A_ij = i, x_j = j gives integer sums, exact in
 *     any order while below 2^53);
 *   SpB_Matrix_free / SpB_Vector_free.
 *
 * The graph is a seeded random graph with `deg` distinct out-neighbours per
 * vertex (the harness reads a .sg/.mtx file instead).
 *
 *   core_harness <n_rows> <deg> <seed>
 * Prints one "ok"/"FAIL" line per check; exits non-zero on failure.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "OpenSparseBLAS.h"
#include "SpB_Vector_Dense.h"
#include "SpB_Matrix_CSC_or_CSR.h"
#define VNEC_HAVE_OPENSPARSEBLAS_H
#include "vnec_gb300.h"

static uint64_t rng_state;
static uint64_t rng_next(void) { /* splitmix64 */
  uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static int failures = 0;
static void report(int ok, const char *what) {
  printf("%s  %s\n", ok ? "ok  " : "FAIL", what);
  failures += !ok;
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s <n_rows> <deg> <seed>\n", argv[0]);
    return 2;
  }
  const SpB_Index n = (SpB_Index)strtoull(argv[1], NULL, 10);
  const int deg = atoi(argv[2]);
  rng_state = strtoull(argv[3], NULL, 10);
  const SpB_Index nvals = n * (SpB_Index)deg;

  /* COO tuples, rows in order, `deg` distinct columns per row (unsorted: the
   * reference's build sorts them). */
  SpB_Index *I = malloc(sizeof(SpB_Index) * nvals);
  SpB_Index *J = malloc(sizeof(SpB_Index) * nvals);
  double *X = malloc(sizeof(double) * nvals);
  for (SpB_Index r = 0; r < n; ++r) {
    SpB_Index *c = J + r * (SpB_Index)deg;
    for (int k = 0; k < deg; ++k) {
      int fresh;
      do {
        c[k] = rng_next() % n;
        fresh = 1;
        for (int q = 0; q < k; ++q) fresh &= c[q] != c[k];
      } while (!fresh);
      I[r * (SpB_Index)deg + (SpB_Index)k] = r;
      X[r * (SpB_Index)deg + (SpB_Index)k] = (double)r; /* test_spmv_vnec.cpp:169 */
    }
  }

  SpB_init();
  SpB_Object_Format_ext format;
  format.matrix_format = SpB_CSR;
  SpB_Global_Option_set_ext(SpB_MATRIX_FORMAT, format);
  SpB_Matrix G = NULL;
  report(SpB_Matrix_new(&G, SpB_FP64, n, n) == SpB_SUCCESS, "SpB_Matrix_new (reference core)");
  report(SpB_Matrix_build_FP64(G, I, J, X, nvals, SpB_BINARYOP_NULL) == SpB_SUCCESS,
         "SpB_Matrix_build_FP64 (reference core, COO -> CSR)");
  free(I);
  free(J);
  free(X);
  SpB_Vector x, y_serial, y_opt;
  report(SpB_Vector_new(&x, SpB_FP64, n) == SpB_SUCCESS, "SpB_Vector_new x");
  for (SpB_Index j = 0; j < n; ++j) SpB_Vector_setElement_FP64(x, (double)j, j); /* :185 */
  SpB_Vector_new(&y_serial, SpB_FP64, n);
  SpB_Vector_new(&y_opt, SpB_FP64, n);

  /* Serial CSR product, as SpB_mxv_FP64_serial (test_spmv_vnec.hpp:57-79). */
  {
    const SpB_Matrix_CSC_or_CSR *a = (const SpB_Matrix_CSC_or_CSR *)G;
    const double *xv = ((SpB_Vector_Dense *)x)->values;
    double *yv = ((SpB_Vector_Dense *)y_serial)->values;
    for (SpB_Index i = 0; i < n; ++i) {
      double t = 0.0;
      for (SpB_Index p = a->ptr[i]; p < a->ptr[i + 1]; ++p) t += ((const double *)a->val)[p] * xv[a->indices[p]];
      yv[i] = t;
    }
  }

  const char *which;
  if (n < 3000000) {
    SpB_VNEC_type t = IRD_VNEC(G, SpB_FP64);
    if (t == SpB_VNEC_D) {
      which = "IRD_VNEC -> D: Build_VNEC_D_FP64 + SpMV_VNEC_D_FP64";
      VNEC_D_FP64 *h = Build_VNEC_D_FP64(G);
      report(h != NULL, "Build_VNEC_D_FP64");
      for (int rep = 0; rep < 2 && h; ++rep) SpMV_VNEC_D_FP64(y_opt, G, x, h);
      VNEC_D_free_fp64(h);
    } else {
      which = "IRD_VNEC -> S: Build_VNEC_S_FP64 + SpMV_VNEC_S_FP64";
      VNEC_S_FP64 *h = Build_VNEC_S_FP64(G);
      report(h != NULL, "Build_VNEC_S_FP64");
      for (int rep = 0; rep < 2 && h; ++rep) SpMV_VNEC_S_FP64(y_opt, G, x, h);
      VNEC_S_free_fp64(h);
    }
  } else {
    which = "L: Build_VNEC_L + SpMV_VNEC_L_FP64";
    VNEC_L *h = Build_VNEC_L(G);
    report(h != NULL, "Build_VNEC_L");
    for (int rep = 0; rep < 2 && h; ++rep) SpMV_VNEC_L_FP64(y_opt, G, x, h);
    if (h) { /* the harness's own release of an L handle (test_spmv_vnec.cpp:246-251) */
      free(h->diagonal_start);
      free(h->diagonal_end);
      free(h->nz_indices);
      free(h->thread_coord_start);
      free(h->thread_coord_end);
      free(h);
    }
  }
  report(SpB_VNEC_last_error_ext()[0] == '\0', SpB_VNEC_last_error_ext()[0] ? SpB_VNEC_last_error_ext() : "no error");

  int within = 1, exact = 1;
  for (SpB_Index i = 0; i < n; ++i) {
    double want, got;
    SpB_Vector_extractElement_FP64(&want, y_serial, i);
    SpB_Vector_extractElement_FP64(&got, y_opt, i);
    within &= fabs(want - got) <= want * 1e-8; /* test_spmv_vnec.cpp:261-269 */
    exact &= want == got;
  }
  report(within, which);
  report(exact, "bit-exact known answer (A_ij = i, x_j = j)");

  SpB_Matrix_free(&G);
  SpB_Vector_free(&x);
  SpB_Vector_free(&y_opt);
  SpB_Vector_free(&y_serial);
  return failures ? 1 : 0;
}
