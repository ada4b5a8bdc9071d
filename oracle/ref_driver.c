/*
 * Driver compiled together with the reference's own sources into
 * oracle/_ref/libvnec_ref.so (oracle/Makefile, target `ref`).
 * TEST INFRASTRUCTURE ONLY: it lets Python tests and the fixture generator
 * (tests/golden/make_golden.py) run the reference's VNEC SpMV functions on a
 * CSR matrix given as plain arrays.
 *
 * The matrix and vectors are built with the reference's own constructors
 * (SpB_Matrix_CSC_or_CSR_new, src/core/src/SpB_Matrix_CSC_or_CSR.c:40-77;
 * SpB_Vector_Dense_new, src/core/src/SpB_Vector_Dense.c:9-37) and the CSR
 * arrays are filled directly in the reference layout (64-bit SpB_Index
 * offsets and columns).  The dispatch mirrors the reference test harness
 * (src/operation/test/test_spmv_vnec.cpp:140-275): IRD_VNEC picks D or S when
 * n_rows < 3,000,000, otherwise L.  Handles are released field by field as
 * the harness does (src/operation/test/test_spmv_vnec.hpp:81-176).
 */
#include <stdint.h>
#include <stdio.h>
#include <unistd.h>

#include "SpB_mxv.h"

enum { REF_AUTO = 0, REF_D = 1, REF_S = 2, REF_L = 3, REF_SERIAL = 4 };

int ref_num_threads(void) { return NUM_THREADS; }
int ref_nlanes_f64(void) { return nLanes_f64; }
int ref_nlanes_f32(void) { return nLanes_f32; }
double ref_ird_thr_f64(void) { return IRD_thr_fp64; }
double ref_ird_thr_f32(void) { return IRD_thr_fp32; }

static SpB_Matrix make_matrix(SpB_Type type, int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr,
                              const int32_t *col, const void *val) {
  SpB_Matrix G = NULL;
  if (SpB_Matrix_CSC_or_CSR_new(&G, type, (SpB_Index)n_rows, (SpB_Index)n_cols, SpB_CSR) != SpB_SUCCESS) return NULL;
  SpB_Matrix_CSC_or_CSR *m = (SpB_Matrix_CSC_or_CSR *)G;
  size_t es = type == SpB_FP64 ? sizeof(double) : sizeof(float);
  free(m->ptr);
  m->ptr = (SpB_Index *)malloc(sizeof(SpB_Index) * (size_t)(n_rows + 1));
  m->indices = (SpB_Index *)malloc(sizeof(SpB_Index) * (size_t)(nnz > 0 ? nnz : 1));
  m->val = malloc(es * (size_t)(nnz > 0 ? nnz : 1));
  for (int64_t i = 0; i <= n_rows; ++i) m->ptr[i] = (SpB_Index)row_ptr[i];
  for (int64_t p = 0; p < nnz; ++p) m->indices[p] = (SpB_Index)col[p];
  memcpy(m->val, val, es * (size_t)nnz);
  m->nnz = (SpB_Index)nnz;
  m->capacity = (SpB_Index)nnz;
  m->ptr_len = (SpB_Index)(n_rows + 1);
  return G;
}

static SpB_Vector make_vector(SpB_Type type, int64_t n, const void *src) {
  SpB_Vector v = NULL;
  if (SpB_Vector_Dense_new(&v, type, (SpB_Index)n) != SpB_SUCCESS) return NULL;
  if (src) memcpy(((SpB_Vector_Dense *)v)->values, src, (type == SpB_FP64 ? 8 : 4) * (size_t)n);
  return v;
}

static void free_matrix(SpB_Matrix G) {
  SpB_Matrix_CSC_or_CSR *m = (SpB_Matrix_CSC_or_CSR *)G;
  free(m->ptr);
  free(m->indices);
  free(m->val);
  free(m);
}

static void free_vector(SpB_Vector v) {
  free(((SpB_Vector_Dense *)v)->values);
  free(v);
}

/* Runs IRD_VNEC with its printf captured; returns the choice and parses the
 * printed IRD ratio into *ird. */
static SpB_VNEC_type run_ird(SpB_Matrix G, SpB_Type type, float *ird) {
  fflush(stdout);
  FILE *tmp = tmpfile();
  int saved = dup(fileno(stdout));
  dup2(fileno(tmp), fileno(stdout));
  SpB_VNEC_type t = IRD_VNEC(G, type);
  fflush(stdout);
  dup2(saved, fileno(stdout));
  close(saved);
  rewind(tmp);
  float v = -1.0f;
  if (fscanf(tmp, " IRD_mat = %f", &v) != 1) v = -1.0f;
  fclose(tmp);
  if (ird) *ird = v;
  return t;
}

static void free_d64(VNEC_D_FP64 *h) {
  free(h->thread_coord_start); free(h->thread_coord_end); free(h->ecr_indices); free(h->NEC_NUM);
  for (int i = 0; i < NUM_THREADS; i++) { free(h->use_x_indices[i]); free(h->ecr_xx_val[i]); }
  free(h->use_x_indices); free(h->ecr_xx_val); free(h->col_start); free(h->v_row_ptr); free(h->val_align);
  free(h);
}
static void free_d32(VNEC_D_FP32 *h) {
  free(h->thread_coord_start); free(h->thread_coord_end); free(h->ecr_indices); free(h->NEC_NUM);
  for (int i = 0; i < NUM_THREADS; i++) { free(h->use_x_indices[i]); free(h->ecr_xx_val[i]); }
  free(h->use_x_indices); free(h->ecr_xx_val); free(h->col_start); free(h->v_row_ptr); free(h->val_align);
  free(h);
}
static void free_s64(VNEC_S_FP64 *h) {
  free(h->NEC_NUM); free(h->spvv8_len);
  for (int i = 0; i < NUM_THREADS; i++) { free(h->use_x_indices[i]); free(h->ecr_xx_val[i]); free(h->tasks[i]); }
  free(h->use_x_indices); free(h->ecr_xx_val); free(h->tasks);
  free(h->reorder_mat.nnz); free(h->reorder_mat.col); free(h->reorder_mat.row_begin); free(h->reorder_mat.row_end);
  free(h->reorder_mat.task_start); free(h->reorder_mat.task_end);
  free(h);
}
static void free_s32(VNEC_S_FP32 *h) {
  free(h->NEC_NUM); free(h->spvv16_len);
  for (int i = 0; i < NUM_THREADS; i++) { free(h->use_x_indices[i]); free(h->ecr_xx_val[i]); free(h->tasks[i]); }
  free(h->use_x_indices); free(h->ecr_xx_val); free(h->tasks);
  free(h->reorder_mat.nnz); free(h->reorder_mat.col); free(h->reorder_mat.row_begin); free(h->reorder_mat.row_end);
  free(h->reorder_mat.task_start); free(h->reorder_mat.task_end);
  free(h);
}
static void free_l(VNEC_L *h) {
  free(h->diagonal_start); free(h->diagonal_end); free(h->nz_indices);
  free(h->thread_coord_start); free(h->thread_coord_end);
  free(h);
}

/* y = A x with the reference's FP64 path.  variant: REF_AUTO (harness
 * dispatch), REF_D, REF_S, REF_L or REF_SERIAL (SpB_mxv_FP64_serial restated
 * from test_spmv_vnec.hpp:57-79, which is test code and not in the library).
 * Returns the variant actually run; *ird gets the IRD ratio when IRD_VNEC ran. */
int ref_spmv_f64(int variant, int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr,
                 const int32_t *col, const double *val, const double *x, double *y, float *ird) {
  SpB_Matrix G = make_matrix(SpB_FP64, n_rows, n_cols, nnz, row_ptr, col, val);
  SpB_Vector xv = make_vector(SpB_FP64, n_cols, x);
  SpB_Vector yv = make_vector(SpB_FP64, n_rows, NULL);
  if (ird) *ird = -1.0f;
  if (variant == REF_AUTO) {
    if (n_rows < 3000000)
      variant = run_ird(G, SpB_FP64, ird) == SpB_VNEC_D ? REF_D : REF_S;
    else
      variant = REF_L;
  }
  if (variant == REF_D) {
    VNEC_D_FP64 *h = Build_VNEC_D_FP64(G);
    SpMV_VNEC_D_FP64(yv, G, xv, h);
    free_d64(h);
  } else if (variant == REF_S) {
    VNEC_S_FP64 *h = Build_VNEC_S_FP64(G);
    SpMV_VNEC_S_FP64(yv, G, xv, h);
    free_s64(h);
  } else if (variant == REF_L) {
    VNEC_L *h = Build_VNEC_L(G);
    SpMV_VNEC_L_FP64(yv, G, xv, h);
    free_l(h);
  } else {
    SpB_Matrix_CSC_or_CSR *a = (SpB_Matrix_CSC_or_CSR *)G;
    double *yy = (double *)((SpB_Vector_Dense *)yv)->values;
    const double *xx = (const double *)((SpB_Vector_Dense *)xv)->values;
    for (SpB_Index i = 0; i < (SpB_Index)n_rows; i++) {
      double t1 = 0.0f;
      for (SpB_Index j = a->ptr[i]; j < a->ptr[i + 1]; j++) t1 += ((double *)a->val)[j] * xx[a->indices[j]];
      yy[i] = t1;
    }
  }
  memcpy(y, ((SpB_Vector_Dense *)yv)->values, sizeof(double) * (size_t)n_rows);
  free_vector(xv);
  free_vector(yv);
  free_matrix(G);
  return variant;
}

/* FP32 twin of ref_spmv_f64. */
int ref_spmv_f32(int variant, int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr,
                 const int32_t *col, const float *val, const float *x, float *y, float *ird) {
  SpB_Matrix G = make_matrix(SpB_FP32, n_rows, n_cols, nnz, row_ptr, col, val);
  SpB_Vector xv = make_vector(SpB_FP32, n_cols, x);
  SpB_Vector yv = make_vector(SpB_FP32, n_rows, NULL);
  if (ird) *ird = -1.0f;
  if (variant == REF_AUTO) {
    if (n_rows < 3000000)
      variant = run_ird(G, SpB_FP32, ird) == SpB_VNEC_D ? REF_D : REF_S;
    else
      variant = REF_L;
  }
  if (variant == REF_D) {
    VNEC_D_FP32 *h = Build_VNEC_D_FP32(G);
    SpMV_VNEC_D_FP32(yv, G, xv, h);
    free_d32(h);
  } else if (variant == REF_S) {
    VNEC_S_FP32 *h = Build_VNEC_S_FP32(G);
    SpMV_VNEC_S_FP32(yv, G, xv, h);
    free_s32(h);
  } else if (variant == REF_L) {
    VNEC_L *h = Build_VNEC_L(G);
    SpMV_VNEC_L_FP32(yv, G, xv, h);
    free_l(h);
  } else {
    SpB_Matrix_CSC_or_CSR *a = (SpB_Matrix_CSC_or_CSR *)G;
    float *yy = (float *)((SpB_Vector_Dense *)yv)->values;
    const float *xx = (const float *)((SpB_Vector_Dense *)xv)->values;
    for (SpB_Index i = 0; i < (SpB_Index)n_rows; i++) {
      float t1 = 0.0f;
      for (SpB_Index j = a->ptr[i]; j < a->ptr[i + 1]; j++) t1 += ((float *)a->val)[j] * xx[a->indices[j]];
      yy[i] = t1;
    }
  }
  memcpy(y, ((SpB_Vector_Dense *)yv)->values, sizeof(float) * (size_t)n_rows);
  free_vector(xv);
  free_vector(yv);
  free_matrix(G);
  return variant;
}

/* IRD_VNEC alone: returns the SpB_VNEC_type, *ird receives the printed ratio. */
int ref_ird(int fp64, int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr, const int32_t *col,
            const void *val, float *ird) {
  SpB_Type type = fp64 ? SpB_FP64 : SpB_FP32;
  SpB_Matrix G = make_matrix(type, n_rows, n_cols, nnz, row_ptr, col, val);
  SpB_VNEC_type t = run_ird(G, type, ird);
  free_matrix(G);
  return (int)t;
}

/* Times the reference harness's FP64 path (test_spmv_vnec.cpp:197-256): for
 * n_rows < 3,000,000 IRD_VNEC picks D or S (variant REF_AUTO; REF_D / REF_S
 * force one), otherwise VNEC-L; the handle is built once, then `warm` untimed
 * and `reps` timed back-to-back SpMV calls.  Returns seconds per call;
 * *used receives the variant run. */
double ref_time_f64(int variant, int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr,
                    const int32_t *col, const double *val, const double *x, int warm, int reps, int *used) {
  SpB_Matrix G = make_matrix(SpB_FP64, n_rows, n_cols, nnz, row_ptr, col, val);
  SpB_Vector xv = make_vector(SpB_FP64, n_cols, x);
  SpB_Vector yv = make_vector(SpB_FP64, n_rows, NULL);
  if (variant == REF_AUTO) {
    if (n_rows < 3000000)
      variant = run_ird(G, SpB_FP64, NULL) == SpB_VNEC_D ? REF_D : REF_S;
    else
      variant = REF_L;
  }
  if (used) *used = variant;
  double secs = -1.0;
  if (variant == REF_D) {
    VNEC_D_FP64 *h = Build_VNEC_D_FP64(G);
    for (int i = 0; i < warm; ++i) SpMV_VNEC_D_FP64(yv, G, xv, h);
    double t0 = omp_get_wtime();
    for (int i = 0; i < reps; ++i) SpMV_VNEC_D_FP64(yv, G, xv, h);
    secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
    free_d64(h);
  } else if (variant == REF_S) {
    VNEC_S_FP64 *h = Build_VNEC_S_FP64(G);
    for (int i = 0; i < warm; ++i) SpMV_VNEC_S_FP64(yv, G, xv, h);
    double t0 = omp_get_wtime();
    for (int i = 0; i < reps; ++i) SpMV_VNEC_S_FP64(yv, G, xv, h);
    secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
    free_s64(h);
  } else if (variant == REF_L) {
    VNEC_L *h = Build_VNEC_L(G);
    for (int i = 0; i < warm; ++i) SpMV_VNEC_L_FP64(yv, G, xv, h);
    double t0 = omp_get_wtime();
    for (int i = 0; i < reps; ++i) SpMV_VNEC_L_FP64(yv, G, xv, h);
    secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
    free_l(h);
  }
  free_vector(xv);
  free_vector(yv);
  free_matrix(G);
  return secs;
}

/* Times `reps` back-to-back SpMV_VNEC_L_FP64 calls after one warm-up, as the
 * harness does (test_spmv_vnec.cpp:235-256).  Returns seconds per call. */
double ref_time_L_f64(int64_t n_rows, int64_t n_cols, int64_t nnz, const int64_t *row_ptr, const int32_t *col,
                      const double *val, const double *x, int warm, int reps) {
  SpB_Matrix G = make_matrix(SpB_FP64, n_rows, n_cols, nnz, row_ptr, col, val);
  SpB_Vector xv = make_vector(SpB_FP64, n_cols, x);
  SpB_Vector yv = make_vector(SpB_FP64, n_rows, NULL);
  VNEC_L *h = Build_VNEC_L(G);
  for (int i = 0; i < warm; ++i) SpMV_VNEC_L_FP64(yv, G, xv, h);
  double t0 = omp_get_wtime();
  for (int i = 0; i < reps; ++i) SpMV_VNEC_L_FP64(yv, G, xv, h);
  double secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
  free_l(h);
  free_vector(xv);
  free_vector(yv);
  free_matrix(G);
  return secs;
}
