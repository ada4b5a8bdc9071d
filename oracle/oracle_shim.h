/*
 * Force-included (-include) into every reference source file when the
 * reference is compiled as a test oracle (oracle/Makefile, target `ref`).
 * TEST INFRASTRUCTURE ONLY.
 *
 * It replaces the allocation calls of the reference with versions that
 * over-allocate by 4 KiB and zero-fill, which neutralises the reference's
 * known out-of-bounds accesses without touching any arithmetic line:
 *   - Build_VNEC_S_* writes one element past a bucket array
 *     (src/operation/src/spmv_vnec_S_for_mxv.c:460-467, FP32 :137-144);
 *   - Build_VNEC_D_* copies val[0 .. nnz + nLanes) (spmv_vnec_D_for_mxv.c:341-344);
 *   - SpMV_VNEC_D_* reads up to nLanes-1 elements past the compressed x window
 *     (spmv_vnec_D_for_mxv.c:448-449, FP32 :205-206); zero fill makes those
 *     lanes contribute 0 * 0.
 * Memory obtained here is released with the reference's own free/_mm_free.
 */
#ifndef VNEC_ORACLE_SHIM_H
#define VNEC_ORACLE_SHIM_H

#include <stdlib.h>
#include <string.h>
#if defined(__x86_64__)
#include <immintrin.h> /* declares _mm_malloc before it is redirected below */
#endif

#define ORC_PAD_BYTES 4096

static inline void *orc_pad_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n + ORC_PAD_BYTES) != 0) return NULL;
  memset(p, 0, n + ORC_PAD_BYTES);
  return p;
}

static inline void *orc_pad_aligned_alloc(size_t align, size_t n) {
  void *p = NULL;
  if (align < sizeof(void *)) align = sizeof(void *);
  if (posix_memalign(&p, align, n + ORC_PAD_BYTES) != 0) return NULL;
  memset(p, 0, n + ORC_PAD_BYTES);
  return p;
}

static inline int orc_pad_posix_memalign(void **pp, size_t align, size_t n) {
  int rc = posix_memalign(pp, align, n + ORC_PAD_BYTES);
  if (rc == 0) memset(*pp, 0, n + ORC_PAD_BYTES);
  return rc;
}

static inline void *orc_pad_mm_malloc(size_t n, size_t align) { return orc_pad_aligned_alloc(align, n); }

#define malloc(n) orc_pad_malloc(n)
#define aligned_alloc(a, n) orc_pad_aligned_alloc((a), (n))
#define posix_memalign(pp, a, n) orc_pad_posix_memalign((pp), (a), (n))
#define _mm_malloc(n, a) orc_pad_mm_malloc((n), (a))

#endif /* VNEC_ORACLE_SHIM_H */
