/*
 * CPU oracle for the VNEC mxv (SpMV) path — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the algorithms of the reference library's
 * VNEC SpMV path so that tests and the CPU-baseline leg of the benchmark can
 * check (and time) the GPU implementation against them.  Nothing in the
 * product library links or calls this code.
 *
 * Every function names the reference lines it follows (paths relative to the
 * reference project root).  The restatement is parameterised by the two
 * compile-time constants of the reference (src/operation/include/SpB_mxv.h:17-32):
 *   nparts  = NUM_THREADS  (36 on the x86 build, 48 on the ARM build)
 *   nlanes  = nLanes_f64 / nLanes_f32 (8/16 on x86 AVX-512, 2/4 on ARM NEON)
 * so the same code reproduces either build.  Floating-point operation order
 * follows the reference: `acc += a * b` in the reference is compiled with
 * floating-point contraction (GNU C default) and is restated as fma(); SIMD
 * lane accumulators are restated lane by lane, and the horizontal reductions
 * use the pairwise tree of the respective intrinsic (restated in
 * reduce_lanes_*).
 *
 * Pinning: tests/test_oracle.py checks both parameterisations bit for bit
 * against outputs of the reference itself, compiled from its own sources by
 * oracle/Makefile into oracle/_ref/: the X86_SIMD build on an AVX-512 x86 host
 * (fixtures in tests/golden/) and the ARM_NEON build on the aarch64 GPU host
 * (fixtures in tests/golden/arm/).  The two builds' compilers evaluate the
 * multiply-adds differently; orc_loop_mode and orc_lane_fused hold each
 * build's pinned choice (set per call by oracle/oracle.py).
 *
 * Deliberate differences from the reference (none changes arithmetic):
 *   - 64-bit merge coordinates (the reference's `int` coordinates overflow past
 *     2^31 merge items);
 *   - the L/D carry fix-up runs serially in partition order (the reference's
 *     parallel `+=` races when a row spans more than two partitions);
 *   - a carry into row n_rows (empty trailing partitions) is skipped (the
 *     reference adds 0.0 one element past y);
 *   - the D kernel's read past the compressed x window
 *     (spmv_vnec_D_for_mxv.c:448-449) sees 0.0, as with the zero-filled
 *     padded allocation used for the reference build.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

/* Scalar multiply-accumulate loops.  The reference's scalar loops
 * `acc += val[p] * x[idx[p]]` are compiled by GCC with contraction enabled and
 * with the products vectorised: for a loop of n iterations the first
 * g*floor(n/g) products are computed as rounded products (vector multiplies)
 * and added in order, and the remaining n mod g iterations are fused
 * multiply-adds.  The group width g differs per loop (1 = every product
 * rounded, 0 = every iteration fused).  Each loop below carries the mode that
 * reproduces the reference build bit for bit (tests/test_oracle.py), held in
 * orc_loop_mode[] so a test can re-derive it.  This file is compiled with
 * -ffp-contract=off so that `a + b * c` here stays unfused. */
enum {
  LOOP_SERIAL_F64, LOOP_SERIAL_F32, LOOP_L_ROW_F64, LOOP_L_TAIL_F32, LOOP_D_CARRY_F64, LOOP_D_CARRY_F32,
  LOOP_S_TAIL_F64, LOOP_S_TAIL_F32, LOOP_L_CARRY_F64, LOOP_L_CARRY_F32, LOOP_COUNT
};
int orc_loop_mode[LOOP_COUNT] = {4, 0, 4, 0, 0, 4, 0, 4, 4, 0};

/* Lane multiply-accumulate of the D kernels and of the FP32 L kernel's lane
 * loop.  The x86 build uses _mm512_fmadd_* (fused, 1).  The ARM build uses
 * vmlaq_f64 / vmlaq_f32 (spmv_vnec_D_for_mxv.c:469, spmv_vnec_L_for_mxv.c:63),
 * which the ARM build computes as a rounded product followed by a rounded
 * add (0).  The S kernels use vfmaq / _mm512_fmadd on both builds (fused). */
int orc_lane_fused = 1;
static inline double lane_mac_f64(double a, double b, double c) {
  if (orc_lane_fused) return fma(a, b, c);
  double p = a * b;
  return c + p;
}
static inline float lane_mac_f32(float a, float b, float c) {
  if (orc_lane_fused) return fmaf(a, b, c);
  float p = a * b;
  return c + p;
}

static inline double mac_run_f64(int loop, double acc, const double *v, const int32_t *idx, const double *xv, i64 n) {
  int g = orc_loop_mode[loop];
  i64 vec = g > 0 ? (n / g) * g : 0;
  i64 i = 0;
  for (; i < vec; ++i) {
    double p = v[i] * xv[idx[i]];
    acc = acc + p;
  }
  for (; i < n; ++i) acc = fma(v[i], xv[idx[i]], acc);
  return acc;
}

static inline float mac_run_f32(int loop, float acc, const float *v, const int32_t *idx, const float *xv, i64 n) {
  int g = orc_loop_mode[loop];
  i64 vec = g > 0 ? (n / g) * g : 0;
  i64 i = 0;
  for (; i < vec; ++i) {
    float p = v[i] * xv[idx[i]];
    acc = acc + p;
  }
  for (; i < n; ++i) acc = fmaf(v[i], xv[idx[i]], acc);
  return acc;
}

/* ------------------------------------------------------------------------ */
/* Merge-path partitioning                                                   */
/* ------------------------------------------------------------------------ */

/* MergePathDivide, src/operation/src/spmv_vnec_common.c:3-33.  Binary search on
 * diagonal `diag` of the merge of A = row_end (= row_ptr + 1, length a_len) and
 * B = 0..b_len-1.  Moves right while A[pivot] <= B[diag - pivot - 1]. */
void orc_merge_path_divide(i64 diag, const i64 *row_end, i64 a_len, i64 b_len, i64 *x, i64 *y) {
  i64 x_min = diag - b_len > 0 ? diag - b_len : 0;
  i64 x_max = diag < a_len ? diag : a_len;
  while (x_min < x_max) {
    i64 pivot = (x_min + x_max) >> 1;
    if (row_end[pivot] <= diag - pivot - 1)
      x_min = pivot + 1;
    else
      x_max = pivot;
  }
  *x = x_min < a_len ? x_min : a_len;
  *y = diag - x_min;
}

/* Per-partition merge coordinates as in Build_VNEC_L,
 * src/operation/src/spmv_vnec_L_for_mxv.c:10-33 (identical in the D builder
 * spmv_vnec_D_for_mxv.c:252-269 and IRD_VNEC ird_calc.c:7-25). */
void orc_partition(int nparts, i64 n_rows, i64 nnz, const i64 *row_ptr, i64 *sx, i64 *sy, i64 *ex, i64 *ey) {
  i64 items = nnz + n_rows;
  i64 per = (items + nparts - 1) / nparts;
  for (int t = 0; t < nparts; ++t) {
    i64 d0 = per * t < items ? per * t : items;
    i64 d1 = d0 + per < items ? d0 + per : items;
    orc_merge_path_divide(d0, row_ptr + 1, n_rows, nnz, sx + t, sy + t);
    orc_merge_path_divide(d1, row_ptr + 1, n_rows, nnz, ex + t, ey + t);
  }
}

/* Row-rounded partitions of Build_VNEC_S, spmv_vnec_S_for_mxv.c:356-371: the
 * merge row coordinate + 1 (except the first start / last end), nnz bounds
 * taken from row_ptr. */
void orc_partition_rows(int nparts, i64 n_rows, i64 nnz, const i64 *row_ptr, i64 *sx, i64 *sy, i64 *ex, i64 *ey) {
  orc_partition(nparts, n_rows, nnz, row_ptr, sx, sy, ex, ey);
  for (int t = 0; t < nparts; ++t) {
    sx[t] += 1;
    ex[t] += 1;
    if (t == 0) sx[t] -= 1;
    if (t == nparts - 1) ex[t] -= 1;
    /* The reference indexes past ptr here when a partition starts at the end
     * of the merge path (tiny matrices); the restatement clamps instead. */
    if (sx[t] > n_rows) sx[t] = n_rows;
    if (ex[t] > n_rows) ex[t] = n_rows;
    sy[t] = row_ptr[sx[t]];
    ey[t] = row_ptr[ex[t]];
  }
}

/* ------------------------------------------------------------------------ */
/* Horizontal lane reductions                                                */
/* ------------------------------------------------------------------------ */

/* Pairwise halving tree: lanes [0,n/2) + [n/2,n), repeated.  This is the order
 * of the AVX-512 reduce-add intrinsics (512 -> 256 -> 128 -> 64 bit halves)
 * and of the NEON across-vector adds for 2 and 4 lanes. */
static double reduce_lanes_f64(const double *v, int n) {
  double t[16];
  for (int i = 0; i < n; ++i) t[i] = v[i];
  for (int w = n / 2; w >= 1; w /= 2)
    for (int i = 0; i < w; ++i) t[i] = t[i] + t[i + w];
  return t[0];
}
static float reduce_lanes_f32(const float *v, int n) {
  float t[32];
  for (int i = 0; i < n; ++i) t[i] = v[i];
  if (n == 4) {
    /* NEON vaddvq_f32: (v0 + v1) + (v2 + v3) (pairwise adjacent). */
    return (t[0] + t[1]) + (t[2] + t[3]);
  }
  for (int w = n / 2; w >= 1; w /= 2)
    for (int i = 0; i < w; ++i) t[i] = t[i] + t[i + w];
  return t[0];
}

/* ------------------------------------------------------------------------ */
/* Serial CSR oracles                                                        */
/* ------------------------------------------------------------------------ */

/* SpB_mxv_FP64_serial, src/operation/test/test_spmv_vnec.hpp:57-79: y_i = sum of
 * val*x in CSR order (t1 += t2*t3, contracted). */
void orc_spmv_serial_f64(i64 n_rows, const i64 *row_ptr, const int32_t *col, const double *val, const double *x,
                         double *y) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n_rows; ++i) {
    double t1 = 0.0;
    t1 = mac_run_f64(LOOP_SERIAL_F64, t1, val + row_ptr[i], col + row_ptr[i], x, row_ptr[i + 1] - row_ptr[i]);
    y[i] = t1;
  }
}

/* SpB_mxv_FP32_serial, src/operation/test/test_spmv_vnec.hpp:34-56. */
void orc_spmv_serial_f32(i64 n_rows, const i64 *row_ptr, const int32_t *col, const float *val, const float *x,
                         float *y) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n_rows; ++i) {
    float t1 = 0.0f;
    t1 = mac_run_f32(LOOP_SERIAL_F32, t1, val + row_ptr[i], col + row_ptr[i], x, row_ptr[i + 1] - row_ptr[i]);
    y[i] = t1;
  }
}

/* Compensated (Neumaier) FP64 SpMV — the accuracy oracle, not a reference
 * restatement.  Also returns the conditioning denominator cond_i = sum |a_ij x_j|
 * used by the row-wise error criterion |y_i - yhat_i| <= tol * cond_i. */
void orc_spmv_neumaier_f64(i64 n_rows, const i64 *row_ptr, const int32_t *col, const double *val, const double *x,
                           double *y, double *cond) {
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < n_rows; ++i) {
    double s = 0.0, c = 0.0, a = 0.0;
    for (i64 p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      double prod = val[p] * x[col[p]];
      double perr = fma(val[p], x[col[p]], -prod); /* exact product error */
      double t = s + prod;
      if (fabs(s) >= fabs(prod))
        c += (s - t) + prod;
      else
        c += (prod - t) + s;
      s = t;
      c += perr;
      a += fabs(prod);
    }
    y[i] = s + c;
    if (cond) cond[i] = a;
  }
}

/* Multi-right-hand-side form of orc_spmv_neumaier_f64 for the batched path
 * (which has no reference counterpart: the reference's SpB_mxv takes one
 * vector).  X is row-major n_cols x k, Y and cond row-major n_rows x k;
 * column j of Y is the compensated FP64 product of the matrix with column j
 * of X, and cond its sum_p |a_p x_p|. */
void orc_spmm_neumaier_f64(i64 n_rows, const i64 *row_ptr, const int32_t *col, const double *val, int k,
                           const double *X, double *Y, double *cond) {
#pragma omp parallel for schedule(dynamic, 64)
  for (i64 i = 0; i < n_rows; ++i) {
    for (int j = 0; j < k; ++j) {
      double s = 0.0, c = 0.0, a = 0.0;
      for (i64 p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
        const double xv = X[(i64)col[p] * k + j];
        double prod = val[p] * xv;
        double perr = fma(val[p], xv, -prod);
        double t = s + prod;
        if (fabs(s) >= fabs(prod))
          c += (s - t) + prod;
        else
          c += (prod - t) + s;
        s = t;
        c += perr;
        a += fabs(prod);
      }
      Y[i * k + j] = s + c;
      if (cond) cond[i * k + j] = a;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* VNEC-L: merge-path CSR                                                    */
/* ------------------------------------------------------------------------ */

/* SpMV_VNEC_L_FP64, src/operation/src/spmv_vnec_L_for_mxv.c:124-165. */
void orc_spmv_L_f64(int nparts, i64 n_rows, i64 nnz, const i64 *row_ptr, const int32_t *col, const double *val,
                    const double *x, double *y) {
  i64 *sx = malloc(sizeof(i64) * nparts), *sy = malloc(sizeof(i64) * nparts);
  i64 *ex = malloc(sizeof(i64) * nparts), *ey = malloc(sizeof(i64) * nparts);
  i64 *crow = malloc(sizeof(i64) * nparts);
  double *cval = malloc(sizeof(double) * nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, sx, sy, ex, ey);
  const i64 *row_end = row_ptr + 1;
#pragma omp parallel for schedule(static) num_threads(nparts)
  for (int t = 0; t < nparts; ++t) {
    i64 cx = sx[t], cy = sy[t];
    for (; cx < ex[t]; ++cx) {
      double rt = 0.0;
      rt = mac_run_f64(LOOP_L_ROW_F64, rt, val + cy, col + cy, x, row_end[cx] - cy);
      cy = row_end[cx] > cy ? row_end[cx] : cy;
      y[cx] = rt;
    }
    double rt = 0.0;
    rt = mac_run_f64(LOOP_L_CARRY_F64, rt, val + cy, col + cy, x, ey[t] - cy);
    crow[t] = ex[t];
    cval[t] = rt;
  }
  for (int t = 0; t < nparts - 1; ++t)
    if (crow[t] < n_rows) y[crow[t]] += cval[t];
  free(sx); free(sy); free(ex); free(ey); free(crow); free(cval);
}

/* SpMV_VNEC_L_FP32, src/operation/src/spmv_vnec_L_for_mxv.c:36-122: complete rows
 * use nlanes-wide lane accumulators while more than nlanes nonzeros remain
 * (strict `<` against row_end - nlanes), then a horizontal reduction, then a
 * scalar tail. */
void orc_spmv_L_f32(int nparts, int nlanes, i64 n_rows, i64 nnz, const i64 *row_ptr, const int32_t *col,
                    const float *val, const float *x, float *y) {
  i64 *sx = malloc(sizeof(i64) * nparts), *sy = malloc(sizeof(i64) * nparts);
  i64 *ex = malloc(sizeof(i64) * nparts), *ey = malloc(sizeof(i64) * nparts);
  i64 *crow = malloc(sizeof(i64) * nparts);
  float *cval = malloc(sizeof(float) * nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, sx, sy, ex, ey);
  const i64 *row_end = row_ptr + 1;
#pragma omp parallel for schedule(static) num_threads(nparts)
  for (int t = 0; t < nparts; ++t) {
    i64 cx = sx[t], cy = sy[t];
    for (; cx < ex[t]; ++cx) {
      float lanes[32];
      for (int l = 0; l < nlanes; ++l) lanes[l] = 0.0f;
      i64 loop_end = row_end[cx] - nlanes;
      for (; cy < loop_end; cy += nlanes)
        for (int l = 0; l < nlanes; ++l) lanes[l] = lane_mac_f32(x[col[cy + l]], val[cy + l], lanes[l]);
      float rt = reduce_lanes_f32(lanes, nlanes);
      rt = mac_run_f32(LOOP_L_TAIL_F32, rt, val + cy, col + cy, x, row_end[cx] - cy);
      cy = row_end[cx] > cy ? row_end[cx] : cy;
      y[cx] = rt;
    }
    float rt = 0.0f;
    rt = mac_run_f32(LOOP_L_CARRY_F32, rt, val + cy, col + cy, x, ey[t] - cy);
    crow[t] = ex[t];
    cval[t] = rt;
  }
  for (int t = 0; t < nparts - 1; ++t)
    if (crow[t] < n_rows) y[crow[t]] += cval[t];
  free(sx); free(sy); free(ex); free(ey); free(crow); free(cval);
}

/* ------------------------------------------------------------------------ */
/* ECR: efficient column compression per partition                           */
/* ------------------------------------------------------------------------ */

typedef struct {
  int nparts;
  i64 *sx, *sy, *ex, *ey; /* partition coordinates */
  int32_t *ecr;           /* compressed column per nonzero (nnz) */
  i64 *nec;               /* distinct columns per partition */
  int32_t **use_cols;     /* sorted distinct columns per partition */
} orc_ecr_t;

/* The ECR pass of Build_VNEC_D_FP64, spmv_vnec_D_for_mxv.c:280-338 (same in
 * Build_VNEC_S_FP64 :388-441 and IRD_VNEC ird_calc.c:29-65): within each
 * partition's nonzero range, columns are renumbered by rank among the distinct
 * columns the partition uses (IDX_MAP[c] = c - #unused columns <= c). */
static void ecr_build(orc_ecr_t *e, i64 n_cols, i64 nnz, const int32_t *col) {
  e->ecr = calloc((size_t)nnz + 16, sizeof(int32_t));
  e->nec = calloc((size_t)e->nparts, sizeof(i64));
  e->use_cols = calloc((size_t)e->nparts, sizeof(int32_t *));
#pragma omp parallel for schedule(static)
  for (int t = 0; t < e->nparts; ++t) {
    int32_t *rank = malloc(sizeof(int32_t) * (size_t)(n_cols > 0 ? n_cols : 1));
    char *used = calloc((size_t)(n_cols > 0 ? n_cols : 1), 1);
    for (i64 p = e->sy[t]; p < e->ey[t]; ++p) used[col[p]] = 1;
    i64 k = 0;
    for (i64 c = 0; c < n_cols; ++c) k += used[c];
    e->use_cols[t] = malloc(sizeof(int32_t) * (size_t)(k > 0 ? k : 1));
    k = 0;
    for (i64 c = 0; c < n_cols; ++c)
      if (used[c]) { rank[c] = (int32_t)k; e->use_cols[t][k++] = (int32_t)c; }
    e->nec[t] = k;
    for (i64 p = e->sy[t]; p < e->ey[t]; ++p) e->ecr[p] = rank[col[p]];
    free(rank);
    free(used);
  }
}

static void ecr_free(orc_ecr_t *e) {
  for (int t = 0; t < e->nparts; ++t) free(e->use_cols[t]);
  free(e->use_cols); free(e->nec); free(e->ecr);
  free(e->sx); free(e->sy); free(e->ex); free(e->ey);
}

static void ecr_alloc_parts(orc_ecr_t *e, int nparts) {
  e->nparts = nparts;
  e->sx = malloc(sizeof(i64) * nparts); e->sy = malloc(sizeof(i64) * nparts);
  e->ex = malloc(sizeof(i64) * nparts); e->ey = malloc(sizeof(i64) * nparts);
}

/* ------------------------------------------------------------------------ */
/* VNEC-D: dense blocks of nlanes consecutive compressed columns              */
/* ------------------------------------------------------------------------ */

/* Block grouping of Build_VNEC_D_FP64, spmv_vnec_D_for_mxv.c:355-392 (and the
 * dry run in IRD_VNEC, ird_calc.c:68-101).  For each complete row of each
 * partition (from max(row start, partition start)), the first nonzero opens a
 * block at its compressed column; a later nonzero whose distance to the open
 * block's start is < nlanes goes to slot `dist`, otherwise it opens a new block.
 * Outputs col_start[block], v_row_ptr[row+1] = cumulative block count and (when
 * val/val_align are given) the zero-padded block values.  Returns the number of
 * blocks. */
static i64 d_group(const orc_ecr_t *e, int nlanes, i64 n_rows, const i64 *row_ptr, const double *val_d,
                   const float *val_f, i64 *v_row_ptr, int32_t *col_start, double *va_d, float *va_f) {
  i64 g = 0;
  v_row_ptr[0] = 0;
  for (int t = 0; t < e->nparts; ++t) {
    for (i64 i = e->sx[t]; i < e->ex[t]; ++i) {
      i64 p0 = row_ptr[i] > e->sy[t] ? row_ptr[i] : e->sy[t];
      i64 len = row_ptr[i + 1] - p0;
      if (len > 0) {
        int32_t cs = e->ecr[p0];
        if (col_start) col_start[g] = cs;
        if (va_d) va_d[g * nlanes] = val_d[p0];
        if (va_f) va_f[g * nlanes] = val_f[p0];
        for (i64 j = 1; j < len; ++j) {
          i64 dist = (i64)e->ecr[p0 + j] - cs;
          if (dist < nlanes) {
            if (va_d) va_d[g * nlanes + dist] = val_d[p0 + j];
            if (va_f) va_f[g * nlanes + dist] = val_f[p0 + j];
          } else {
            ++g;
            cs = e->ecr[p0 + j];
            if (col_start) col_start[g] = cs;
            if (va_d) va_d[g * nlanes] = val_d[p0 + j];
            if (va_f) va_f[g * nlanes] = val_f[p0 + j];
          }
        }
        ++g;
      }
      v_row_ptr[i + 1] = g;
    }
  }
  return g;
}

/* IRD_VNEC, src/operation/src/ird_calc.c:2-122: IRD = nnz / (blocks * nlanes) in
 * single precision; returns 0 (SpB_VNEC_D) if IRD >= threshold else 1
 * (SpB_VNEC_S).  `ird_out` receives the ratio. */
int orc_ird(int nparts, int nlanes, float threshold, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
            const int32_t *col, float *ird_out) {
  orc_ecr_t e;
  ecr_alloc_parts(&e, nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, e.sx, e.sy, e.ex, e.ey);
  ecr_build(&e, n_cols, nnz, col);
  i64 *vrp = calloc((size_t)n_rows + 1, sizeof(i64));
  i64 blocks = d_group(&e, nlanes, n_rows, row_ptr, NULL, NULL, vrp, NULL, NULL, NULL);
  (void)blocks;
  int denom = (int)(vrp[n_rows] * nlanes);
  float ird = (float)nnz / (float)denom;
  if (ird_out) *ird_out = ird;
  free(vrp);
  ecr_free(&e);
  return ird >= threshold ? 0 : 1;
}

/* Build_VNEC_D_FP64 (spmv_vnec_D_for_mxv.c:242-398) followed by SpMV_VNEC_D_FP64
 * (:400-485): per partition, gather the compressed x window; per complete row,
 * nlanes lane accumulators over its blocks (fma), then the horizontal
 * reduction overwrites y[i]; the tail carry restarts at row_end[ex-1] (=
 * row_ptr[ex]) as the reference does (:471); then y[carry_row] += carry.
 * `reps` repeats the SpMV part only (for timing); the build runs once. */
void orc_spmv_D_f64(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                    const int32_t *col, const double *val, const double *x, double *y, int reps) {
  orc_ecr_t e;
  ecr_alloc_parts(&e, nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, e.sx, e.sy, e.ex, e.ey);
  ecr_build(&e, n_cols, nnz, col);
  i64 *vrp = calloc((size_t)n_rows + 1, sizeof(i64));
  int32_t *cs = calloc((size_t)nnz + 1, sizeof(int32_t));
  double *va = calloc((size_t)(nnz + 1) * nlanes, sizeof(double));
  d_group(&e, nlanes, n_rows, row_ptr, val, NULL, vrp, cs, va, NULL);
  double **win = malloc(sizeof(double *) * nparts);
  for (int t = 0; t < nparts; ++t) win[t] = calloc((size_t)e.nec[t] + 2 * nlanes, sizeof(double));
  i64 *crow = malloc(sizeof(i64) * nparts);
  double *cval = malloc(sizeof(double) * nparts);
  for (int rep = 0; rep < reps; ++rep) {
#pragma omp parallel for schedule(static) num_threads(nparts)
    for (int t = 0; t < nparts; ++t) {
      double *w = win[t];
      for (i64 j = 0; j < e.nec[t]; ++j) w[j] = x[e.use_cols[t][j]];
      for (i64 i = e.sx[t]; i < e.ex[t]; ++i) {
        double lanes[16];
        for (int l = 0; l < nlanes; ++l) lanes[l] = 0.0;
        for (i64 b = vrp[i]; b < vrp[i + 1]; ++b)
          for (int l = 0; l < nlanes; ++l) lanes[l] = lane_mac_f64(va[b * nlanes + l], w[cs[b] + l], lanes[l]);
        y[i] = reduce_lanes_f64(lanes, nlanes);
      }
      double rt = 0.0;
      i64 p0 = row_ptr[e.ex[t]];
      rt = mac_run_f64(LOOP_D_CARRY_F64, rt, val + p0, e.ecr + p0, w, e.ey[t] - p0);
      crow[t] = e.ex[t];
      cval[t] = rt;
    }
    for (int t = 0; t < nparts - 1; ++t)
      if (crow[t] < n_rows) y[crow[t]] += cval[t];
  }
  for (int t = 0; t < nparts; ++t) free(win[t]);
  free(win); free(crow); free(cval); free(vrp); free(cs); free(va);
  ecr_free(&e);
}

/* FP32 twin: Build_VNEC_D_FP32 / SpMV_VNEC_D_FP32, spmv_vnec_D_for_mxv.c:2-241. */
void orc_spmv_D_f32(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                    const int32_t *col, const float *val, const float *x, float *y, int reps) {
  orc_ecr_t e;
  ecr_alloc_parts(&e, nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, e.sx, e.sy, e.ex, e.ey);
  ecr_build(&e, n_cols, nnz, col);
  i64 *vrp = calloc((size_t)n_rows + 1, sizeof(i64));
  int32_t *cs = calloc((size_t)nnz + 1, sizeof(int32_t));
  float *va = calloc((size_t)(nnz + 1) * nlanes, sizeof(float));
  d_group(&e, nlanes, n_rows, row_ptr, NULL, val, vrp, cs, NULL, va);
  float **win = malloc(sizeof(float *) * nparts);
  for (int t = 0; t < nparts; ++t) win[t] = calloc((size_t)e.nec[t] + 2 * nlanes, sizeof(float));
  i64 *crow = malloc(sizeof(i64) * nparts);
  float *cval = malloc(sizeof(float) * nparts);
  for (int rep = 0; rep < reps; ++rep) {
#pragma omp parallel for schedule(static) num_threads(nparts)
    for (int t = 0; t < nparts; ++t) {
      float *w = win[t];
      for (i64 j = 0; j < e.nec[t]; ++j) w[j] = x[e.use_cols[t][j]];
      for (i64 i = e.sx[t]; i < e.ex[t]; ++i) {
        float lanes[32];
        for (int l = 0; l < nlanes; ++l) lanes[l] = 0.0f;
        for (i64 b = vrp[i]; b < vrp[i + 1]; ++b)
          for (int l = 0; l < nlanes; ++l) lanes[l] = lane_mac_f32(va[b * nlanes + l], w[cs[b] + l], lanes[l]);
        y[i] = reduce_lanes_f32(lanes, nlanes);
      }
      float rt = 0.0f;
      i64 p0 = row_ptr[e.ex[t]];
      rt = mac_run_f32(LOOP_D_CARRY_F32, rt, val + p0, e.ecr + p0, w, e.ey[t] - p0);
      crow[t] = e.ex[t];
      cval[t] = rt;
    }
    for (int t = 0; t < nparts - 1; ++t)
      if (crow[t] < n_rows) y[crow[t]] += cval[t];
  }
  for (int t = 0; t < nparts; ++t) free(win[t]);
  free(win); free(crow); free(cval); free(vrp); free(cs); free(va);
  ecr_free(&e);
}

/* ------------------------------------------------------------------------ */
/* VNEC-S: equal-length row groups (cross-row) + single rows (in-row)        */
/* ------------------------------------------------------------------------ */

typedef struct {
  orc_ecr_t e;
  i64 *task_rows;   /* original row of each reordered row (n_rows) */
  i64 *task_start;  /* per partition, first reordered row */
  i64 *task_end;
  i64 *group_len;   /* per partition, rows in cross-row groups */
  i64 *row_begin;   /* reordered storage offsets */
  i64 *row_end;
  int32_t *rcol;    /* reordered compressed columns (interleaved in groups) */
  double *rval_d;
  float *rval_f;
} orc_s_t;

/* Build_VNEC_S_FP64, spmv_vnec_S_for_mxv.c:336-588 (FP32 twin :3-334): row-rounded
 * partitions, ECR, per-partition bucketing of rows by length (ascending
 * lengths; a length <= 32 contributes its first nlanes*floor(count/nlanes) rows,
 * in row order, to the cross-row list, the rest go to the in-row list), reorder
 * into contiguous storage, then interleave each group of nlanes equal-length
 * rows so that element l of group row r sits at base + l*nlanes + r. */
static void s_build(orc_s_t *s, int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                    const int32_t *col, const double *val_d, const float *val_f) {
  orc_ecr_t *e = &s->e;
  ecr_alloc_parts(e, nparts);
  orc_partition_rows(nparts, n_rows, nnz, row_ptr, e->sx, e->sy, e->ex, e->ey);
  ecr_build(e, n_cols, nnz, col);
  s->task_rows = malloc(sizeof(i64) * (size_t)(n_rows + 1));
  s->task_start = malloc(sizeof(i64) * nparts);
  s->task_end = malloc(sizeof(i64) * nparts);
  s->group_len = malloc(sizeof(i64) * nparts);
  i64 start = 0;
  for (int t = 0; t < nparts; ++t) {
    i64 nr = e->ex[t] - e->sx[t];
    s->task_start[t] = start;
    s->task_end[t] = start + nr;
    i64 maxlen = 0;
    for (i64 r = e->sx[t]; r < e->ex[t]; ++r)
      if (row_ptr[r + 1] - row_ptr[r] > maxlen) maxlen = row_ptr[r + 1] - row_ptr[r];
    i64 *count = calloc((size_t)maxlen + 1, sizeof(i64));
    for (i64 r = e->sx[t]; r < e->ex[t]; ++r) count[row_ptr[r + 1] - row_ptr[r]]++;
    /* For each length, the first `bulk` rows (row order) go to the group list. */
    i64 *bulk = calloc((size_t)maxlen + 1, sizeof(i64));
    i64 ngroup = 0;
    for (i64 len = 0; len <= maxlen; ++len) {
      i64 left = len > 32 ? count[len] : count[len] % nlanes;
      bulk[len] = count[len] - left;
      ngroup += bulk[len];
    }
    s->group_len[t] = ngroup;
    /* Offsets: group rows ordered by length, then remaining rows by length. */
    i64 *gpos = calloc((size_t)maxlen + 1, sizeof(i64)), *rpos = calloc((size_t)maxlen + 1, sizeof(i64));
    i64 *seen = calloc((size_t)maxlen + 1, sizeof(i64));
    i64 og = 0, orr = ngroup;
    for (i64 len = 0; len <= maxlen; ++len) { gpos[len] = og; og += bulk[len]; }
    for (i64 len = 0; len <= maxlen; ++len) { rpos[len] = orr; orr += count[len] - bulk[len]; }
    for (i64 r = e->sx[t]; r < e->ex[t]; ++r) {
      i64 len = row_ptr[r + 1] - row_ptr[r];
      i64 slot = seen[len] < bulk[len] ? gpos[len]++ : rpos[len]++;
      seen[len]++;
      s->task_rows[start + slot] = r;
    }
    free(count); free(bulk); free(gpos); free(rpos); free(seen);
    start += nr;
  }
  s->row_begin = malloc(sizeof(i64) * (size_t)(n_rows + 1));
  s->row_end = malloc(sizeof(i64) * (size_t)(n_rows + 1));
  s->rcol = malloc(sizeof(int32_t) * (size_t)(nnz + 1));
  s->rval_d = val_d ? malloc(sizeof(double) * (size_t)(nnz + 1)) : NULL;
  s->rval_f = val_f ? malloc(sizeof(float) * (size_t)(nnz + 1)) : NULL;
  i64 np = 0;
  for (i64 q = 0; q < start; ++q) {
    i64 r = s->task_rows[q];
    s->row_begin[q] = np;
    s->row_end[q] = np + row_ptr[r + 1] - row_ptr[r];
    for (i64 p = row_ptr[r]; p < row_ptr[r + 1]; ++p) {
      if (s->rval_d) s->rval_d[np] = val_d[p];
      if (s->rval_f) s->rval_f[np] = val_f[p];
      s->rcol[np++] = e->ecr[p];
    }
  }
  /* Interleave groups (spmv_vnec_S_for_mxv.c:558-585). */
  for (int t = 0; t < nparts; ++t) {
    for (i64 c = 0; c < s->group_len[t]; c += nlanes) {
      i64 q = s->task_start[t] + c;
      i64 len = s->row_end[q] - s->row_begin[q], base = s->row_begin[q];
      if (len == 0) continue;
      int32_t *tc = malloc(sizeof(int32_t) * (size_t)(len * nlanes));
      double *td = s->rval_d ? malloc(sizeof(double) * (size_t)(len * nlanes)) : NULL;
      float *tf = s->rval_f ? malloc(sizeof(float) * (size_t)(len * nlanes)) : NULL;
      memcpy(tc, s->rcol + base, sizeof(int32_t) * (size_t)(len * nlanes));
      if (td) memcpy(td, s->rval_d + base, sizeof(double) * (size_t)(len * nlanes));
      if (tf) memcpy(tf, s->rval_f + base, sizeof(float) * (size_t)(len * nlanes));
      for (i64 l = 0; l < len; ++l)
        for (int r = 0; r < nlanes; ++r) {
          s->rcol[base + l * nlanes + r] = tc[r * len + l];
          if (td) s->rval_d[base + l * nlanes + r] = td[r * len + l];
          if (tf) s->rval_f[base + l * nlanes + r] = tf[r * len + l];
        }
      free(tc); free(td); free(tf);
    }
  }
}

static void s_free(orc_s_t *s) {
  free(s->task_rows); free(s->task_start); free(s->task_end); free(s->group_len);
  free(s->row_begin); free(s->row_end); free(s->rcol); free(s->rval_d); free(s->rval_f);
  ecr_free(&s->e);
}

/* SpMV_VNEC_S_FP64, spmv_vnec_S_for_mxv.c:589-660 with the micro-kernels of
 * src/operation/include/SpB_mxv.h: cross-row groups (AVX512_spvv_cross_row_fp64
 * :154-190 / NEON :303-324) accumulate each lane = row sequentially with fma;
 * in-row rows (AVX512_spvv_in_row_fp64 :127-152 / NEON :277-301) use nlanes lane
 * accumulators while i < rowlen - (nlanes - 1), sum = 0 + reduction, then a
 * scalar fma tail.  No carry: partitions hold whole rows. */
/* `warm` untimed then `reps` timed calls after one build (the reference times
 * only SpMV_VNEC_S_FP64, test_spmv_vnec.cpp:205-214); seconds per timed call. */
static double s_run_f64(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                        const int32_t *col, const double *val, const double *x, double *y, int warm, int reps) {
  orc_s_t s;
  s_build(&s, nparts, nlanes, n_rows, n_cols, nnz, row_ptr, col, val, NULL);
  double **win = malloc(sizeof(double *) * nparts);
  for (int t = 0; t < nparts; ++t) win[t] = calloc((size_t)s.e.nec[t] + 1, sizeof(double));
  double t0 = 0.0;
  for (int rep = 0; rep < warm + reps; ++rep) {
#ifdef _OPENMP
    if (rep == warm) t0 = omp_get_wtime();
#endif
#pragma omp parallel for schedule(static) num_threads(nparts)
    for (int t = 0; t < nparts; ++t) {
      double *w = win[t];
      for (i64 j = 0; j < s.e.nec[t]; ++j) w[j] = x[s.e.use_cols[t][j]];
      i64 q = s.task_start[t], c = 0;
      for (; c < s.group_len[t]; q += nlanes, c += nlanes) {
        i64 len = s.row_end[q] - s.row_begin[q], base = s.row_begin[q];
        double acc[16];
        for (int r = 0; r < nlanes; ++r) acc[r] = 0.0;
        for (i64 l = 0; l < len; ++l)
          for (int r = 0; r < nlanes; ++r)
            acc[r] = fma(s.rval_d[base + l * nlanes + r], w[s.rcol[base + l * nlanes + r]], acc[r]);
        for (int r = 0; r < nlanes; ++r) y[s.task_rows[q + r]] = acc[r];
      }
      for (; q < s.task_end[t]; ++q) {
        i64 b = s.row_begin[q], len = s.row_end[q] - b;
        double lanes[16];
        for (int l = 0; l < nlanes; ++l) lanes[l] = 0.0;
        i64 i = 0;
        for (; i < len - (nlanes - 1); i += nlanes)
          for (int l = 0; l < nlanes; ++l) lanes[l] = fma(s.rval_d[b + i + l], w[s.rcol[b + i + l]], lanes[l]);
        double sum = 0.0;
        sum += reduce_lanes_f64(lanes, nlanes);
        sum = mac_run_f64(LOOP_S_TAIL_F64, sum, s.rval_d + b + i, s.rcol + b + i, w, len - i);
        y[s.task_rows[q]] = sum;
      }
    }
  }
  double secs = 0.0;
#ifdef _OPENMP
  secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
#endif
  for (int t = 0; t < nparts; ++t) free(win[t]);
  free(win);
  s_free(&s);
  return secs;
}

void orc_spmv_S_f64(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                    const int32_t *col, const double *val, const double *x, double *y, int reps) {
  s_run_f64(nparts, nlanes, n_rows, n_cols, nnz, row_ptr, col, val, x, y, 0, reps);
}

/* Timed S-variant loop for the CPU baseline; seconds per call. */
double orc_time_S_f64(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                      const int32_t *col, const double *val, const double *x, double *y, int warm, int reps) {
  return s_run_f64(nparts, nlanes, n_rows, n_cols, nnz, row_ptr, col, val, x, y, warm, reps);
}

/* SpMV_VNEC_S_FP32, spmv_vnec_S_for_mxv.c:255-334 with the FP32 micro-kernels
 * (SpB_mxv.h:40-125 AVX-512, :194-275 NEON). */
void orc_spmv_S_f32(int nparts, int nlanes, i64 n_rows, i64 n_cols, i64 nnz, const i64 *row_ptr,
                    const int32_t *col, const float *val, const float *x, float *y, int reps) {
  orc_s_t s;
  s_build(&s, nparts, nlanes, n_rows, n_cols, nnz, row_ptr, col, NULL, val);
  float **win = malloc(sizeof(float *) * nparts);
  for (int t = 0; t < nparts; ++t) win[t] = calloc((size_t)s.e.nec[t] + 1, sizeof(float));
  for (int rep = 0; rep < reps; ++rep) {
#pragma omp parallel for schedule(static) num_threads(nparts)
    for (int t = 0; t < nparts; ++t) {
      float *w = win[t];
      for (i64 j = 0; j < s.e.nec[t]; ++j) w[j] = x[s.e.use_cols[t][j]];
      i64 q = s.task_start[t], c = 0;
      for (; c < s.group_len[t]; q += nlanes, c += nlanes) {
        i64 len = s.row_end[q] - s.row_begin[q], base = s.row_begin[q];
        float acc[32];
        for (int r = 0; r < nlanes; ++r) acc[r] = 0.0f;
        for (i64 l = 0; l < len; ++l)
          for (int r = 0; r < nlanes; ++r)
            acc[r] = fmaf(s.rval_f[base + l * nlanes + r], w[s.rcol[base + l * nlanes + r]], acc[r]);
        for (int r = 0; r < nlanes; ++r) y[s.task_rows[q + r]] = acc[r];
      }
      for (; q < s.task_end[t]; ++q) {
        i64 b = s.row_begin[q], len = s.row_end[q] - b;
        float lanes[32];
        for (int l = 0; l < nlanes; ++l) lanes[l] = 0.0f;
        i64 i = 0;
        for (; i < len - (nlanes - 1); i += nlanes)
          for (int l = 0; l < nlanes; ++l) lanes[l] = fmaf(s.rval_f[b + i + l], w[s.rcol[b + i + l]], lanes[l]);
        float sum = 0.0f;
        sum += reduce_lanes_f32(lanes, nlanes);
        sum = mac_run_f32(LOOP_S_TAIL_F32, sum, s.rval_f + b + i, s.rcol + b + i, w, len - i);
        y[s.task_rows[q]] = sum;
      }
    }
  }
  for (int t = 0; t < nparts; ++t) free(win[t]);
  free(win);
  s_free(&s);
}

/* Timed L-variant loop for the CPU baseline: `reps` SpMV calls after the
 * partition is built once (the reference builds VNEC_L once and times only
 * SpMV_VNEC_L_FP64, test_spmv_vnec.cpp:235-256).  Returns seconds per call. */
double orc_time_L_f64(int nparts, i64 n_rows, i64 nnz, const i64 *row_ptr, const int32_t *col, const double *val,
                      const double *x, double *y, int warm, int reps) {
  i64 *sx = malloc(sizeof(i64) * nparts), *sy = malloc(sizeof(i64) * nparts);
  i64 *ex = malloc(sizeof(i64) * nparts), *ey = malloc(sizeof(i64) * nparts);
  i64 *crow = malloc(sizeof(i64) * nparts);
  double *cval = malloc(sizeof(double) * nparts);
  orc_partition(nparts, n_rows, nnz, row_ptr, sx, sy, ex, ey);
  const i64 *row_end = row_ptr + 1;
  double t0 = 0.0;
  for (int rep = 0; rep < warm + reps; ++rep) {
#ifdef _OPENMP
    if (rep == warm) t0 = omp_get_wtime();
#endif
#pragma omp parallel for schedule(static) num_threads(nparts)
    for (int t = 0; t < nparts; ++t) {
      i64 cx = sx[t], cy = sy[t];
      for (; cx < ex[t]; ++cx) {
        double rt = 0.0;
        rt = mac_run_f64(LOOP_L_ROW_F64, rt, val + cy, col + cy, x, row_end[cx] - cy);
      cy = row_end[cx] > cy ? row_end[cx] : cy;
        y[cx] = rt;
      }
      double rt = 0.0;
      rt = mac_run_f64(LOOP_L_CARRY_F64, rt, val + cy, col + cy, x, ey[t] - cy);
      crow[t] = ex[t];
      cval[t] = rt;
    }
    for (int t = 0; t < nparts - 1; ++t)
      if (crow[t] < n_rows) y[crow[t]] += cval[t];
  }
  double secs = 0.0;
#ifdef _OPENMP
  secs = (omp_get_wtime() - t0) / (reps > 0 ? reps : 1);
#endif
  free(sx); free(sy); free(ex); free(ey); free(crow); free(cval);
  return secs;
}

int orc_num_procs(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}
