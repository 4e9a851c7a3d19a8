/*
 * or_internal.h -- TEST INFRASTRUCTURE ONLY: the oracle's assembled H-matrix,
 * shared by oracle.c (assembly, checker products) and cpu_mul.c (the timed
 * CPU product).
 */
#ifndef HMGPU_OR_INTERNAL_H
#define HMGPU_OR_INTERNAL_H
#include <stdint.h>

typedef struct {
  int64_t rs, re, cs, ce; /* 1-based inclusive, permuted index space */
  int64_t r;              /* rank (approx blocks)                    */
  double *D;              /* dense: m x n row-major                   */
  double *U;              /* approx: m x r row-major                  */
  double *V;              /* approx: r x n row-major                  */
} or_block;

struct or_hmatrix {
  int64_t m, n;
  int64_t *tmap, *smap;
  int64_t tlen, slen;
  or_block *dense;
  int64_t nd;
  or_block *approx;
  int64_t na;
  int64_t ncand;       /* admissible leaves that were processed      */
  int64_t *aca_rank;   /* per candidate: rank before recompression   */
  int64_t *final_rank; /* per candidate: rank kept, -1 if went dense */
};

#endif
