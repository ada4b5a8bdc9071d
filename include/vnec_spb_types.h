/*
 * Layout-compatible declarations of the OpenSparseBLAS types that the VNEC
 * mxv path touches, for callers that do not include the reference's own
 * OpenSparseBLAS.h.  Every enum value, field order and field type matches the
 * reference so that a matrix or vector built by the reference's core library
 * can be handed to this library unchanged:
 *
 *   SpB_Info                     include/OpenSparseBLAS.h:32-37
 *   SpB_Type                     include/OpenSparseBLAS.h:42-57
 *   SpB_Index                    include/OpenSparseBLAS.h:252  (64-bit unsigned)
 *   SpB_Vector_Format_Value_ext  include/OpenSparseBLAS.h:2542-2547
 *   SpB_Matrix_Format_Value_ext  include/OpenSparseBLAS.h:2553-2558
 *   struct SpB_Matrix_opaque     src/core/include/SpB_Matrix.h:10-17
 *   struct SpB_Vector_opaque     src/core/include/SpB_Vector.h:10-16
 *   SpB_Matrix_CSC_or_CSR        src/core/include/SpB_Matrix_CSC_or_CSR.h:12-21
 *   SpB_Vector_Dense             src/core/include/SpB_Vector_Dense.h:15-19
 *   SpB_VNEC_type, coord, VNEC_* include/OpenSparseBLAS.h:1954-2073
 *
 * A caller that already includes OpenSparseBLAS.h defines
 * VNEC_HAVE_OPENSPARSEBLAS_H before including vnec_gb300.h and skips this file.
 */
#ifndef VNEC_SPB_TYPES_H
#define VNEC_SPB_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { SpB_SUCCESS = 0, SpB_FAILURE = 1, SpB_NO_VALUE = -1 } SpB_Info;

typedef enum {
  SpB_NULL_TYPE,
  SpB_BOOL,
  SpB_INT8,
  SpB_INT16,
  SpB_INT32,
  SpB_INT64,
  SpB_UINT8,
  SpB_UINT16,
  SpB_UINT32,
  SpB_UINT64,
  SpB_FP32,
  SpB_FP64,
  SpB_Type_N
} SpB_Type;

typedef unsigned long int SpB_Index;

typedef enum { SpB_DENSE = 0, SpB_SPARSE = 1, SpB_VECTOR_NO_FORMAT = -1 } SpB_Vector_Format_Value_ext;
typedef enum { SpB_CSC = 0, SpB_CSR = 1, SpB_MATRIX_NO_FORMAT = -1 } SpB_Matrix_Format_Value_ext;

struct SpB_Matrix_opaque {
  SpB_Type element_type;
  SpB_Matrix_Format_Value_ext format_type;
  SpB_Index row;
  SpB_Index col;
  size_t element_size;
};
typedef struct SpB_Matrix_opaque *SpB_Matrix;

struct SpB_Vector_opaque {
  SpB_Type element_type;
  SpB_Vector_Format_Value_ext format_type;
  SpB_Index n;
  size_t element_size;
};
typedef struct SpB_Vector_opaque *SpB_Vector;

typedef struct {
  struct SpB_Matrix_opaque matrix_base;
  void *val;          /* nnz values, element_type */
  SpB_Index *indices; /* CSR: column of each value */
  SpB_Index *ptr;     /* CSR: row offsets, ptr_len = rows + 1 */
  SpB_Index ptr_len;
  SpB_Index nnz;
  SpB_Index capacity;
} SpB_Matrix_CSC_or_CSR;

typedef struct {
  struct SpB_Vector_opaque vector_base;
  void *values; /* n elements, element_type, host memory */
} SpB_Vector_Dense;

typedef enum { SpB_VNEC_D = 0, SpB_VNEC_S = 1 } SpB_VNEC_type;

typedef struct coord {
  int x;
  int y;
} coord;

typedef struct VNEC_D_FP32 {
  coord *thread_coord_start;
  coord *thread_coord_end;
  int *ecr_indices;
  int *NEC_NUM;
  int **use_x_indices;
  float **ecr_xx_val;
  int *v_row_ptr;
  int *col_start;
  float *val_align;
} VNEC_D_FP32;

struct csr_f32 {
  float *nnz;
  int *col, *row_begin, *row_end;
  int *task_start;
  int *task_end;
};

typedef struct VNEC_S_FP32 {
  int *NEC_NUM;
  int **use_x_indices;
  float **ecr_xx_val;
  int *spvv16_len;
  int **tasks;
  struct csr_f32 reorder_mat;
} VNEC_S_FP32;

typedef struct VNEC_L {
  int num_merge_items;
  int items_per_thread;
  int *diagonal_start;
  int *diagonal_end;
  coord *thread_coord_start;
  coord *thread_coord_end;
  int *nz_indices;
} VNEC_L;

typedef struct VNEC_D_FP64 {
  coord *thread_coord_start;
  coord *thread_coord_end;
  int *ecr_indices;
  int *NEC_NUM;
  int **use_x_indices;
  double **ecr_xx_val;
  int *v_row_ptr;
  int *col_start;
  double *val_align;
} VNEC_D_FP64;

struct csr_f64 {
  double *nnz;
  int *col, *row_begin, *row_end;
  int *task_start;
  int *task_end;
};

typedef struct VNEC_S_FP64 {
  int *NEC_NUM;
  int **use_x_indices;
  double **ecr_xx_val;
  int *spvv8_len;
  int **tasks;
  struct csr_f64 reorder_mat;
} VNEC_S_FP64;

#ifdef __cplusplus
}
#endif

#endif /* VNEC_SPB_TYPES_H */
