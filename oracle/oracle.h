/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU, FP64, plain-C restatement of the H-matrix path of HMatrixGPU.jl:
 * cluster tree (src/tree.jl), block tree + merge + traversal (src/block.jl),
 * ACA+ and SVD recompression (src/aca.jl), block assembly and flattening
 * (src/hmatrix.jl) and both matrix-vector products (src/mult.jl).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load this code, and only as the checker or as the timed CPU baseline.  The
 * product library never links or calls it.
 *
 * Parity status: Julia is not available to run the reference, so the oracle
 * is pinned by the reference's own known-answer tests (test/test_aca.jl,
 * test/test_hmatrix.jl, test/test_hmatrix_vector.jl, test/test_tree.jl,
 * test/test_block.jl), whose assertions are restated in tests/.  Bit-level
 * agreement with Julia's BLAS/LAPACK calls (gemv, qr, svd) and with Julia's
 * SIMD `sum` is not claimed; everything else follows the reference's
 * operation order.
 *
 * Conventions: all indices that cross this API are 1-based and inclusive
 * exactly as in the reference, except node/end indices of the cluster tree,
 * which keep the reference's exclusive `end_idx` (src/tree.jl:6-14).
 * Coordinates are 3xN column-major (Julia's `coordinates[:, i]`).
 */
#ifndef HMGPU_ORACLE_H
#define HMGPU_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- cluster tree: src/tree.jl:45-137 ---------------------------------- */
typedef struct or_tree or_tree;
int or_cluster_tree(const double *coords, int64_t npts, int64_t max_points_per_leaf,
                    int64_t dims, or_tree **out);
int64_t or_tree_num_nodes(const or_tree *t);
int64_t or_tree_index_len(const or_tree *t);
/* Arrays sized num_nodes (index_map: index_len). Nodes are numbered in creation
 * order (pre-order, left before right); left/right are node numbers or -1. */
void or_tree_export(const or_tree *t, int64_t *index_map, int64_t *start, int64_t *end,
                    int8_t *is_leaf, int64_t *left, int64_t *right, double *center,
                    double *radius);
void or_tree_free(or_tree *t);

/* ---- block tree: src/block.jl:31-155 ----------------------------------- */
typedef struct or_blocks or_blocks;
/* Builds the block tree, merges dense subtrees when merge != 0 and collects
 * the leaves by the reference's pre-order traversal. */
int or_block_tree(const or_tree *X, const or_tree *Y, double eta, int merge, or_blocks **out);
int64_t or_blocks_num_dense(const or_blocks *b);
int64_t or_blocks_num_approx(const or_blocks *b);
int64_t or_blocks_num_nodes(const or_blocks *b);
/* (target node, source node) pairs in traversal order. */
void or_blocks_export(const or_blocks *b, int64_t *dense_pairs, int64_t *approx_pairs);
/* Every block-tree node: target node, source node, admissible flag, dense flag,
 * left child, right child (-1 if none). */
void or_blocks_export_nodes(const or_blocks *b, int64_t *target, int64_t *source,
                            int8_t *admissible, int8_t *dense, int64_t *left, int64_t *right);
void or_blocks_free(or_blocks *b);

/* ---- matrix entry sources ---------------------------------------------- */
enum {
  OR_KERNEL_EXPLICIT = 0,  /* entries read from a column-major matrix          */
  OR_KERNEL_LAPLACE3D = 1, /* 1/(4 pi r), 0 at r == 0                          */
  OR_KERNEL_YUKAWA = 2,    /* exp(-r)/r, 0 at r == 0                           */
  OR_KERNEL_LOG2D = 3,     /* test/test_hmatrix.jl:170-173                     */
  OR_KERNEL_VECTOR_R = 4,  /* test/test_hmatrix_vector.jl:334-340 (3N columns) */
  OR_KERNEL_DIPOLAR = 5    /* examples/hmatrix_vector.jl:12-54 (3N x 3N)       */
};
typedef struct {
  int32_t type;
  int64_t nrows, ncols;  /* size(K)                                 */
  const double *X;       /* target coordinates, 3 x nX column-major */
  const double *Y;       /* source coordinates, 3 x nY column-major */
  const double *A;       /* explicit matrix, column-major, lda      */
  int64_t lda;
} or_kernel;
/* K[i, j] with 1-based original (unpermuted) indices. */
double or_kernel_entry(const or_kernel *K, int64_t i, int64_t j);
/* Dense product y = K * x over the whole matrix (reference test check). */
void or_kernel_matvec(const or_kernel *K, const double *x, double *y);
/* sparsify_hmatrix(K, X, Y; eta), src/hmatrix.jl:234-274: the entries of every
 * dense leaf of the merged block tree, leaves in traversal order, each block row
 * by row, as 1-based (I, J, V) triplets (the arrays the reference hands to
 * sparse()). Returns the number of entries; fills I, J, V when non-NULL. */
int64_t or_sparsify(const or_kernel *K, const or_tree *X, const or_tree *Y, double eta, int64_t *I,
                    int64_t *J, double *V);

/* ---- ACA+ and recompression: src/aca.jl:9-143 ---------------------------- */
/* ACA+ on the sub-block K[rows, cols] (1-based original indices). U is m x cap
 * column-major, V is cap x n column-major (leading dimension cap). Returns the
 * rank through *rank; cap must be >= min(m, n, max_iter). */
int or_aca_plus(const or_kernel *K, const int64_t *rows, int64_t m, const int64_t *cols,
                int64_t n, double eps, int64_t max_iter, int64_t cap, double *U, double *V,
                int64_t *rank);
/* SVD_recompress on U (m x k, col-major, ld m) and V (k x n, col-major, ld k).
 * Writes U_out (m x r, ld m) and V_out (r x n, ld r); r <= k. */
int or_svd_recompress(int64_t m, int64_t n, int64_t k, const double *U, const double *V,
                      double eps, double *U_out, double *V_out, int64_t *r);
/* Householder QR and one-sided Jacobi SVD, exposed for cross-checks. The QR's
 * sums run in the order of a team of nt lanes (32 or 256; see oracle.c). */
int or_qr(int64_t m, int64_t k, double *A, double *tau, double *R, int nt);
int or_jacobi_svd(int64_t k, double *A, double *Vj, double *sigma, int64_t *order);

/* ---- assembly + flatten: src/hmatrix.jl:72-217 ------------------------- */
typedef struct or_hmatrix or_hmatrix;
/* sample_stride > 1 assembles only every sample_stride-th dense and admissible
 * block (used to time a bounded sample of a large matrix). */
int or_hmatrix_build(const or_kernel *K, const or_tree *X, const or_tree *Y, double eta,
                     double eps, int svd_recompress, int64_t sample_stride, int nthreads,
                     or_hmatrix **out);
/* Sizes of the flattened HMatrix{T} fields (src/hmatrix.jl:46-57, 96-147). */
void or_hmatrix_sizes(const or_hmatrix *h, int64_t *m, int64_t *n, int64_t *nD, int64_t *nA,
                      int64_t *R, int64_t *dense_len, int64_t *U_len, int64_t *V_len);
/* Flattened fields; index tables are column-major 5 x nD, 5 x nA, 3 x R. */
void or_hmatrix_export(const or_hmatrix *h, int64_t *tmap, int64_t *smap, int64_t *dense_idx,
                       int64_t *U_idx, int64_t *V_idx, double *dense_data, double *U_data,
                       double *V_data);
/* Per-block ACA rank before recompression, in approx-list order (-1 if the
 * block went dense), and whether each admissible block was kept low-rank. */
void or_hmatrix_aca_ranks(const or_hmatrix *h, int64_t *aca_rank, int64_t *final_rank);
int64_t or_hmatrix_num_approx_candidates(const or_hmatrix *h);
void or_hmatrix_free(or_hmatrix *h);

/* ---- products: src/mult.jl -------------------------------------------------- */
/* CPU mul! (src/mult.jl:6-32). nthreads > 1 splits the block loop into
 * contiguous ranges with private accumulators summed in a fixed order. */
int or_mul_cpu(const or_hmatrix *h, const double *x, double *y, int nthreads);
/* Same, on the block subsets that a sampled matrix holds; returns seconds of
 * wall time for `reps` repetitions. */
double or_mul_cpu_timed(const or_hmatrix *h, const double *x, double *y, int nthreads,
                        int reps);
/* Flattened mul! semantics (src/mult.jl:41-146), sequential order; fills Vx. */
int or_mul_flat(const or_hmatrix *h, const double *x, double *y, double *Vx);

/* ---- the timed CPU baseline (cpu_mul.c) --------------------------------- */
/* mul!(result, ::HMatrixCPU, x) (src/mult.jl:6-32) with BLAS-like dot products
 * (vector accumulators, fused multiply-adds): one permutation of x, one gemv
 * per dense block, two per low-rank block and one scatter per product. A plan
 * fixes the thread count, the split of the block list and the buffers. */
typedef struct or_cpu_mul or_cpu_mul;
or_cpu_mul *or_cpu_mul_plan(const or_hmatrix *h, int nthreads);
/* Runs `reps` whole products y = H x; returns their wall time in seconds. */
double or_cpu_mul_run(or_cpu_mul *p, const double *x, double *y, int reps);
void or_cpu_mul_free(or_cpu_mul *p);
/* Stored FP64 entries of all blocks (8 bytes each are read per product). */
int64_t or_hmatrix_stored_entries(const or_hmatrix *h);

#ifdef __cplusplus
}
#endif
#endif
