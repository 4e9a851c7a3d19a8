/*
 * hmgpu.h -- C ABI of libhmgpu, a CUDA (sm_103a) implementation of the
 * H-matrix path of HMatrixGPU.jl: cluster tree, block tree, ACA+ with SVD
 * recompression, H-matrix assembly and the product mul!(y, H, x) / H * x.
 *
 * Every function returns HMGPU_OK (0) or a negative status; the message of
 * the last failure on the calling thread is available from hmgpu_last_error().
 * Plain pointers and sizes only.  Index arguments follow the reference's
 * conventions: 1-based, ranges inclusive, tables column-major as Julia stores
 * them.  Device-side objects are bound to the CUDA device that was current
 * when they were created.  A handle may be used by one stream at a time.
 *
 * Reference interfaces replaced (paths inside the HMatrixGPU.jl project):
 *   ClusterTree(coords; max_points_per_leaf, dims)   src/tree.jl:45
 *   info(::ClusterTree)                              src/tree.jl:153
 *   BlockTree(X, Y; eta) + merge + traverse          src/block.jl:31, :98, :127
 *   ACA_plus(n_rows, n_cols, rows, cols, eps)        src/aca.jl:36
 *   SVD_recompress(U, V, eps)                        src/aca.jl:123
 *   HMatrix(K, X, Y; eta, eps, ...)                  src/hmatrix.jl:72
 *   HMatrix{T} flattened fields                      src/hmatrix.jl:46-57
 *   info(::HMatrixCPU)                               src/hmatrix.jl:289
 *   mul!(y, ::HMatrix{T}, x), *(::HMatrix{T}, x)     src/mult.jl:159, :203
 */
#ifndef HMGPU_H
#define HMGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HMGPU_ABI_VERSION 2

/* status codes */
#define HMGPU_OK 0
#define HMGPU_ERR_INVALID (-1)   /* an argument or an imported table is invalid     */
#define HMGPU_ERR_CUDA (-2)      /* a CUDA runtime call failed                      */
#define HMGPU_ERR_NOMEM (-3)     /* host or device allocation failed                */
#define HMGPU_ERR_TREE (-4)      /* a cluster cannot be split (coincident points)   */
#define HMGPU_ERR_TIMEOUT (-5)   /* a bounded device-side wait expired              */
#define HMGPU_ERR_UNSUPPORTED (-6)

/* storage / arithmetic modes of an H-matrix */
#define HMGPU_F64 0   /* all factors FP64, FP64 arithmetic; x, y are double        */
#define HMGPU_F32 1   /* all factors FP32, FP32 arithmetic; x, y are float         */
#define HMGPU_MIXED 2 /* FP32 factors with compensated FP32 accumulation for
                         few right-hand sides; for more, a copy of every block
                         as FP16 pairs hi + lo (hi = fp16(s a), lo = fp16(s a -
                         hi), 22 significant bits) under power-of-two scales s
                         per panel row, per rank row and per right-hand side,
                         multiplied on the tensor cores with FP32 accumulation,
                         one pass per 64 right-hand sides (the threshold is
                         hmgpu_hmatrix_autotune's); x, y are float             */

/* matrix entry generators for on-device assembly */
#define HMGPU_KERNEL_EXPLICIT 0  /* entries of a given column-major matrix        */
#define HMGPU_KERNEL_LAPLACE3D 1 /* 1/(4 pi r), 0 at r = 0                         */
#define HMGPU_KERNEL_YUKAWA 2    /* exp(-r)/r, 0 at r = 0                          */
#define HMGPU_KERNEL_LOG2D 3     /* -log(r)/(2 pi), 1 at r < 1e-12                 */
#define HMGPU_KERNEL_VECTOR_R 4  /* R_c/r^2 over 3 columns per source point        */
#define HMGPU_KERNEL_DIPOLAR 5   /* 3x3 demagnetising tensor per point pair        */
#define HMGPU_KERNEL_USER 6      /* f(x_i, y_j) of the caller's own, compiled at run
                                    time (hmgpu_user_kernel_compile)               */

/* Returns the message of the last failed call on this thread ("" if none). */
const char *hmgpu_last_error(void);
int hmgpu_abi_version(void);

/* ---------------------------------------------------------------------- */
/* Cluster tree: replaces ClusterTree(coords; max_points_per_leaf, dims)     */
/* (src/tree.jl:45-137) and info(::ClusterTree) (src/tree.jl:153-187).      */
/* Host or GPU build, both bit-exact with the reference's bisection.        */
/* ---------------------------------------------------------------------- */
typedef struct hmgpu_tree hmgpu_tree;

/* coords: 3 x npts column-major (Julia's coordinates[:, i]). */
int hmgpu_tree_build(const double *coords, int64_t npts, int64_t max_points_per_leaf,
                     int64_t dims, hmgpu_tree **out);
/* The same tree built on the current GPU, bit-identical to hmgpu_tree_build
 * (same permutation, ranges, centers and radii; same errors). Replaces the
 * same reference call; coords may be host or device memory; npts < 2^30.
 * Level by level, one CTA per node; the centroid sums keep the reference's
 * sequential order. */
int hmgpu_tree_build_device(const double *coords, int64_t npts, int64_t max_points_per_leaf,
                            int64_t dims, hmgpu_tree **out);
/* nnodes, index-map length (dims*npts), and info(): depth, max/min points. */
int hmgpu_tree_info(const hmgpu_tree *t, int64_t *nnodes, int64_t *index_len, int64_t *depth,
                    int64_t *max_points, int64_t *min_points);
/* index_map (1-based), per node: start (1-based), end (exclusive, as
 * ClusterNode.end_idx), leaf flag, children (node numbers, -1 if none; nodes
 * are numbered in pre-order), center (3 per node), radius. Any pointer may be
 * NULL. */
int hmgpu_tree_export(const hmgpu_tree *t, int64_t *index_map, int64_t *start, int64_t *end,
                      int8_t *is_leaf, int64_t *left, int64_t *right, double *center,
                      double *radius);
int hmgpu_tree_free(hmgpu_tree *t);

/* ---------------------------------------------------------------------- */
/* Block tree: replaces BlockTree(X, Y; eta) (src/block.jl:31-90),          */
/* merge_dense_matrices! (:98-112) and traverse (:127-155).                 */
/* ---------------------------------------------------------------------- */
typedef struct hmgpu_blocks hmgpu_blocks;

int hmgpu_blocks_build(const hmgpu_tree *X, const hmgpu_tree *Y, double eta, int merge,
                       hmgpu_blocks **out);
/* The same block tree built on the current GPU, bit-identical to
 * hmgpu_blocks_build: node numbers, flags, children and both traverse lists.
 * Breadth first, then a bottom-up sweep (merge, subtree counts) and a top-down
 * sweep that reproduces the host's pre-order numbering. */
int hmgpu_blocks_build_device(const hmgpu_tree *X, const hmgpu_tree *Y, double eta, int merge,
                              hmgpu_blocks **out);
int hmgpu_blocks_counts(const hmgpu_blocks *b, int64_t *ndense, int64_t *napprox,
                        int64_t *nnodes);
/* (target node, source node) pairs of traverse()'s direct_list / approx_list. */
int hmgpu_blocks_export(const hmgpu_blocks *b, int64_t *dense_pairs, int64_t *approx_pairs);
/* Every block-tree node: target/source node, admissible and dense flags,
 * children (-1 if none). */
int hmgpu_blocks_export_nodes(const hmgpu_blocks *b, int64_t *target, int64_t *source,
                              int8_t *admissible, int8_t *dense, int64_t *left,
                              int64_t *right);
int hmgpu_blocks_free(hmgpu_blocks *b);

/* ---------------------------------------------------------------------- */
/* H-matrix                                                                  */
/* ---------------------------------------------------------------------- */
typedef struct hmgpu_hmatrix hmgpu_hmatrix;

typedef struct hmgpu_rank_model hmgpu_rank_model;
typedef struct hmgpu_user_kernel hmgpu_user_kernel;

typedef struct {
  int32_t precision;   /* HMGPU_F64, HMGPU_F32 or HMGPU_MIXED                     */
  int32_t compensated; /* FP32 modes: 1 = compensated (Dot2) accumulation        */
  int32_t keep_factors;/* 1 = keep the FP64 block factors for export             */
  int32_t lean;        /* HMGPU_MIXED: 1 = keep only the tensor-core copy (FP16
                          pairs): the FP32 layout is freed once the copy is
                          packed, halving the matrix's memory; every product,
                          1 and 2 right-hand sides too, runs on the tensor
                          cores. A lean H-matrix cannot be saved, sharded,
                          batched or used by hmgpu_matvec_noalloc; autotuning
                          leaves it as it is.                                */
  /* Optional learned rank predictor (see below): when set, hmgpu_hmatrix_build
   * sizes each admissible block's ACA workspace from the predicted rank and
   * batches blocks of similar predicted rank together; blocks that need more
   * terms are rerun with room for min(m, n). NULL = fixed workspace. */
  const hmgpu_rank_model *rank_model;
} hmgpu_options;

typedef struct {
  int32_t kind;    /* HMGPU_KERNEL_*                                              */
  int32_t reserved;
  const double *X; /* target points, 3 x nX column-major (host)                   */
  int64_t nX;
  const double *Y; /* source points, 3 x nY column-major (host)                   */
  int64_t nY;
  const double *A; /* HMGPU_KERNEL_EXPLICIT: column-major matrix, host or device  */
  int64_t lda;
  const hmgpu_user_kernel *user; /* HMGPU_KERNEL_USER: the compiled entry function */
  const double *params;          /* HMGPU_KERNEL_USER: its parameters, host or device */
  int64_t nparams;               /* HMGPU_KERNEL_USER: 0 to 64 parameters          */
} hmgpu_kernel;

/* A matrix K[i, j] = f(x_i, y_j) of the caller's own, for hmgpu_hmatrix_build
 * and hmgpu_sparsify: the reference builds an HMatrix from any K it can index
 * (HMatrix(K, X, Y), src/hmatrix.jl:183,195-196 read K[i, j]). `source` is CUDA
 * C++ that defines
 *   __device__ double hmgpu_entry(const double *x, const double *y, const double *p, int a, int b)
 * (x the target point and y the source point, 3 coordinates each; p the
 * kernel's parameters, hmgpu_kernel.params; a and b the components of a vector
 * or tensor kernel: with trees of dims d_x and d_y, row i is component i mod
 * d_x of target point i / d_x and column j component j mod d_y of source
 * point j / d_y; 0 for a scalar kernel). It is compiled with NVRTC for
 * sm_103a into the library's own ACA+, dense-block and sparsify kernels,
 * without FMA contraction, like the built-in kernels; the module is loaded on
 * each device at its first use. On failure the compiler's log is copied to
 * `log` (log_len bytes, NUL-terminated; NULL for none) and HMGPU_ERR_INVALID
 * returned; HMGPU_ERR_UNSUPPORTED when the NVRTC library cannot be loaded. */
int hmgpu_user_kernel_compile(const char *source, hmgpu_user_kernel **out, char *log, int64_t log_len);
int hmgpu_user_kernel_free(hmgpu_user_kernel *uk);

/* Imports a reference-layout flattened HMatrix{Float64} (src/hmatrix.jl:46-57,
 * built at :95-147): m x n operator, target/source index maps (1-based), dense
 * index table 5 x nD (row_start,row_end,col_start,col_end,offset0), dense data
 * (row-major blocks), U table 5 x nA (row_start,row_end,vx_start,vx_end,
 * offset0), U data (row-major m x r), V table 3 x R (col_start,col_end,
 * offset0), V data (row-major r x n).  Host or device pointers.  The tables
 * are validated, the data is converted to the requested precision and
 * re-laid out on the device; the caller keeps ownership of its arrays. */
int hmgpu_hmatrix_import_flat(const hmgpu_options *opt, int64_t m, int64_t n,
                              const int64_t *target_map, const int64_t *source_map,
                              const int64_t *dense_idx, int64_t nD, const double *dense_data,
                              int64_t dense_len, const int64_t *U_idx, int64_t nA,
                              const double *U_data, int64_t U_len, const int64_t *V_idx,
                              int64_t R, const double *V_data, int64_t V_len,
                              hmgpu_hmatrix **out);

/* HMatrix(K, X, Y; eta, eps, svd_recompress) (src/hmatrix.jl:72-217) with the
 * entries generated on the device: dense blocks filled from K, admissible
 * blocks compressed by batched ACA+ at eps/10 and recompressed by batched
 * QR+SVD at eps (FP64), blocks that do not compress stored dense. */
int hmgpu_hmatrix_build(const hmgpu_options *opt, const hmgpu_kernel *K, const hmgpu_tree *X,
                        const hmgpu_tree *Y, double eta, double eps, int svd_recompress,
                        hmgpu_hmatrix **out);

/* mul!(y, H, x) (src/mult.jl:159-189) for nrhs right-hand sides: x is n x nrhs
 * and y is m x nrhs, column-major with leading dimensions ldx >= n and
 * ldy >= m, device pointers of the mode's element type (double for HMGPU_F64,
 * float otherwise).  y is overwritten in the original (unpermuted) order.
 * Stream-ordered on `stream` (a cudaStream_t; NULL = the legacy default
 * stream); returns without synchronising. */
int hmgpu_matvec(hmgpu_hmatrix *H, const void *x, void *y, int64_t nrhs, int64_t ldx,
                 int64_t ldy, void *stream);
/* H * x (src/mult.jl:203-209) on host buffers: copies x to the device, runs
 * hmgpu_matvec and copies y back, synchronously. */
int hmgpu_matvec_host(hmgpu_hmatrix *H, const void *x, void *y, int64_t nrhs, int64_t ldx,
                      int64_t ldy);

/* No counterpart in the reference. The single-right-hand-side product of
 * hmgpu_matvec (y = H x, device pointers, stream-ordered) for callers that
 * cannot allocate device memory while they run it -- code being captured into
 * a CUDA graph where plain allocation is not allowed, loops that fix their
 * memory up front, hosts whose allocator belongs to another framework. Its
 * scratch -- the ticket counter of the near/U pass and XT (the permuted x,
 * then t = V x) -- lives in one statically sized device array of
 * HMGPU_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until
 * the process exits; the call allocates nothing. The status word of the
 * bounded waits stays in H's own allocation. An H-matrix needing more scratch is rejected with HMGPU_ERR_INVALID.
 * The first call on a device looks up the array's address (make that first
 * call before any stream capture). All calls share the array: calls that
 * overlap on the GPU (other streams, other threads, other H-matrices) race. */
#define HMGPU_NOALLOC_SCRATCH_BYTES (32u << 20)
int hmgpu_matvec_noalloc(hmgpu_hmatrix *H, const void *x, void *y, void *stream);

typedef struct {
  int64_t m, n;                  /* size(K)                                        */
  int64_t n_dense, n_approx;     /* full_leaves, admissible_leaves                  */
  int64_t min_rank, max_rank;
  int64_t min_dense_size, max_dense_size;
  int64_t total_rank;            /* R = length(Vx_buffer)                           */
  int64_t dense_entries;         /* sum over dense blocks of m*n                    */
  int64_t far_entries;           /* sum over low-rank blocks of r*(m+n)             */
  double compression_ratio;      /* m*n / (dense_entries + far_entries)             */
  int64_t matrix_bytes;          /* bytes of factor data one product streams        */
  int64_t device_bytes;          /* bytes held on the device                        */
  int64_t n_tiles;               /* row tiles of the near/U pass                    */
  int32_t precision;
  int32_t hi_only_blocks;        /* 0: mixed precision keeps hi and lo for every block */
  double build_seconds;          /* wall time of the last import/build              */
  int64_t aca_batches;           /* device ACA batches of the build                 */
  int64_t aca_reruns;            /* blocks rerun after outgrowing their workspace   */
  int64_t aca_workspace_bytes;   /* workspace bytes summed over the batches         */
  int64_t aca_continued;         /* blocks that outgrew a learned workspace cap and
                                    went on from their state in the same batch      */
} hmgpu_info;
/* info(::HMatrixCPU) (src/hmatrix.jl:289-330) plus storage figures. */
int hmgpu_hmatrix_info(const hmgpu_hmatrix *H, hmgpu_info *info);

/* Wall time of the phases of the last build (no counterpart in the reference;
 * the reference's only timing hook is an @time around assembly), in seconds:
 *   [0] block tree, [1] device copies of geometry and maps and the ACA job
 *   list, [2] ACA + recompression, [3] block lists and the gather of the
 *   factors, [4] product plan (host) and its upload, [5] packing of the
 *   factors and generation of the dense blocks, [6] tensor-core copy (mixed
 *   precision). Imports fill [4..6] only. Writes min(n, HMGPU_BUILD_PHASES). */
#define HMGPU_BUILD_PHASES 7
int hmgpu_hmatrix_build_profile(const hmgpu_hmatrix *H, double *seconds, int32_t n);

/* Device status of the products run so far (no counterpart in the reference):
 * synchronises the device; *status = 0 if every bounded wait inside the
 * kernels completed, else the code of the first one that expired (then
 * returns HMGPU_ERR_TIMEOUT and clears the code). */
int hmgpu_hmatrix_status(hmgpu_hmatrix *H, int *status);
/* Self-test of the bounded device-side wait that the tensor-core product uses
 * (no counterpart in the reference): one thread waits, with the same code
 * path, on a barrier that nothing completes, limited to limit_ns (1 ms to
 * 2 s). The wait must give up and record its code; *code receives the device
 * status (90 when the wait expired as it should) and *waited_ms the device
 * time spent waiting. The context stays usable afterwards. */
int hmgpu_selftest_bounded_wait(int64_t limit_ns, int32_t *code, double *waited_ms);

/* Phase timing (no counterpart in the reference): while on, every product
 * records CUDA events on its stream between its kernels.  phase_times
 * synchronises, returns the summed device time in milliseconds of the phases
 * [x permutation, V pass, near/U pass] and the kernel launches and products
 * recorded since profiling was switched on, and clears them. */
int hmgpu_hmatrix_set_profiling(hmgpu_hmatrix *H, int on);
int hmgpu_hmatrix_phase_times(hmgpu_hmatrix *H, double *ms3, int64_t *launches,
                              int64_t *products);

/* Block lists of the H-matrix in the reference's order: dense blocks (tree
 * dense leaves, then admissible leaves that did not compress) as 4 x nD
 * (row_start,row_end,col_start,col_end), low-rank blocks as 5 x nA
 * (row_start,row_end,col_start,col_end,rank). */
int hmgpu_hmatrix_blocks(const hmgpu_hmatrix *H, int64_t *dense_idx, int64_t *approx_idx);
/* Index maps (1-based) of the H-matrix. */
int hmgpu_hmatrix_index_maps(const hmgpu_hmatrix *H, int64_t *target_map, int64_t *source_map);
/* FP64 factors of low-rank block b (0-based, in approx_idx order) into host
 * arrays U (m x r row-major) and V (r x n row-major); requires keep_factors. */
int hmgpu_hmatrix_block_factors(const hmgpu_hmatrix *H, int64_t b, double *U, double *V);
/* ACA ranks before recompression per admissible leaf of the block tree, in
 * traversal order (builds only; -1 where not computed). */
int hmgpu_hmatrix_aca_ranks(const hmgpu_hmatrix *H, int64_t *aca_rank, int64_t *final_rank);
int hmgpu_hmatrix_free(hmgpu_hmatrix *H);

/* ---------------------------------------------------------------------- */
/* Single-block compression: ACA_plus (src/aca.jl:36-106) and                */
/* SVD_recompress (src/aca.jl:123-143) on an explicit m x n block           */
/* (column-major, host or device), run by the batched device kernels.       */
/* ---------------------------------------------------------------------- */
/* U: m x cap column-major, V: cap x n column-major (ld cap), host arrays;
 * cap >= min(m, n, max_iter); max_iter <= 0 means n_rows. */
int hmgpu_aca_plus(const double *A, int64_t lda, int64_t m, int64_t n, double eps,
                   int64_t max_iter, int64_t cap, double *U, double *V, int64_t *rank);
/* U: m x k (ld m), V: k x n (ld k) host arrays in; U_out m x r (ld m), V_out
 * r x n (ld r) host arrays out (room for k columns/rows). */
int hmgpu_svd_recompress(int64_t m, int64_t n, int64_t k, const double *U, const double *V,
                         double eps, double *U_out, double *V_out, int64_t *r);

/* ---------------------------------------------------------------------- */
/* Learned ACA-rank predictor (no counterpart in the reference): an          */
/* 8 -> 64 -> 64 -> 1 ReLU MLP in FP32 mapping block features to the rank    */
/* plain ACA+ reaches, trained and evaluated by the library's own kernels.   */
/* Used only to size and batch ACA work; results never depend on it.         */
/* sparsify_hmatrix(K, X, Y; eta) (src/hmatrix.jl:234-274): the entries of every
 * dense leaf of BlockTree(X, Y; eta) after merge_dense_matrices!, leaves in
 * traversal order and each block row by row, as 1-based triplets (I, J, V) in
 * original index order, exactly the arrays the reference gives sparse(). The
 * values come from the device entry generator. With I, J and V all NULL only
 * *nnz is set; otherwise all three must hold *nnz entries (I and J in host
 * memory, V in host or device memory). */
int hmgpu_sparsify(const hmgpu_kernel *K, const hmgpu_tree *X, const hmgpu_tree *Y, double eta,
                   int64_t *I, int64_t *J, double *V, int64_t *nnz);

/* ---- row shards for products over several GPUs --------------------------- */
/* Row ownership follows the reference's product, which writes every row of the
 * permuted output exactly once (DU_mult_vec_kernel!, src/mult.jl:80-146; the
 * store at :144), so the rows split over GPUs with no reduction.
 * hmgpu_hmatrix_shard gives shard `rank` of `world`: a handle on the current
 * device (H's) holding a contiguous range of H's row tiles, balanced by stored
 * entries, and the V rows of every source group those tiles read. Its rows are
 * the permuted rows [row_begin, row_end) of hmgpu_shard_rows (0-based; the
 * shards of one H cover 0..m once, in rank order). H may be freed afterwards.
 * hmgpu_matvec_shard computes those rows of y = H x for one right-hand side:
 * x_perm holds all n entries of x in the permuted source order (x_perm[j] =
 * x[source_map[j] - 1]; the caller gathers it from the ranks first), y_rows
 * receives row_end - row_begin values, y_rows[i] = (H x)[target_map[row_begin
 * + i] - 1]. Device pointers of the mode's element type; stream-ordered. Each
 * owned row is bitwise the row hmgpu_matvec computes on H. A shard serves only
 * this entry point (the other product, batch, autotune and save calls refuse
 * it). */
int hmgpu_hmatrix_shard(const hmgpu_hmatrix *H, int32_t rank, int32_t world, hmgpu_hmatrix **out);
int hmgpu_shard_rows(const hmgpu_hmatrix *S, int64_t *row_begin, int64_t *row_end);
int hmgpu_matvec_shard(hmgpu_hmatrix *S, const void *x_perm, void *y_rows, void *stream);

/* ---- batches, CUDA graphs, autotuning (no counterpart in the reference) -- */
/* One H-matrix made of `count` members: the block-diagonal operator
 * diag(H_1, ..., H_count), of size (sum m_k) x (sum n_k). Its products take
 * x = [x_1; x_2; ...] (member k's entries at offset sum_{j<k} n_j) and write
 * y = [y_1; y_2; ...], and run all members in the same kernel launches. The
 * members must live on the current device and share precision and
 * compensation; their device data is copied, so they stay usable and may be
 * freed. Products of the batch equal the members' own products bit for bit. */
int hmgpu_hmatrix_batch(hmgpu_hmatrix *const *members, int32_t count, hmgpu_hmatrix **out);

/* hmgpu_matvec(H, x, y, nrhs, ldx, ldy) captured once into a CUDA graph and
 * replayed by hmgpu_graph_launch on any stream (x and y are fixed device
 * pointers; their contents may change between launches). Creation runs the
 * product once, uncaptured, to allocate its scratch. H must outlive the
 * graph, and replays of graphs of the same H must not overlap. */
typedef struct hmgpu_graph hmgpu_graph;
int hmgpu_graph_create(hmgpu_hmatrix *H, const void *x, void *y, int64_t nrhs, int64_t ldx,
                       int64_t ldy, hmgpu_graph **out);
int hmgpu_graph_launch(hmgpu_graph *G, void *stream);
int hmgpu_graph_free(hmgpu_graph *G);

/* Times the product's free parameters on H's own data (about a second of
 * products) and keeps the fastest: rows per near/U unit (8, 16, 32 or 64;
 * units above 16 rows only for tiles whose vector entries fit one 16 KB
 * shared-memory chunk, which a unit then gathers once), bytes per
 * V unit (32, 64 or 128 KiB), the V schedule (see hmgpu_hmatrix_tuning) and
 * the number of right-hand sides from which one multi-RHS pass replaces
 * repeated single-RHS products. None of them changes
 * any result. With `cache_path` (a text file; NULL for none) the choice is
 * looked up first and stored after, keyed by the H-matrix's structure and the
 * device. result (optional, 4 values): unit rows, V unit KiB, multi-RHS
 * threshold (1 << 30: never), 1 if it came from the cache. */
int hmgpu_hmatrix_autotune(hmgpu_hmatrix *H, const char *cache_path, int32_t *result);
/* The product parameters in force (no counterpart in the reference): rows per
 * near/U unit, V unit KiB, multi-RHS threshold, V schedule (0: each warp owns
 * a byte-balanced range of V units, 1: warps take V units from a ticket
 * counter; the autotuner times both). Writes min(n, 4) values. */
int hmgpu_hmatrix_tuning(const hmgpu_hmatrix *H, int32_t *values, int32_t n);
/* Sets those four parameters directly (for instance from an earlier autotune
 * on the same structure); n must be 4. Results do not depend on them. */
int hmgpu_hmatrix_set_tuning(hmgpu_hmatrix *H, const int32_t *values, int32_t n);

/* An assembled H-matrix on disk (no counterpart in the reference; the
 * reference's flattened HMatrix has no file form): the device layout, index
 * maps and block set as they are, with a checksum, so that a load needs no
 * assembly. load validates every table against the data sizes before anything
 * reaches the device and places the matrix on the current device. */
int hmgpu_hmatrix_save(const hmgpu_hmatrix *H, const char *path);
int hmgpu_hmatrix_load(const char *path, hmgpu_hmatrix **out);

/* ---------------------------------------------------------------------- */
#define HMGPU_RANK_MODEL_PARAMS 4801
#define HMGPU_RANK_FEATURES 8
int hmgpu_rank_model_create(uint64_t seed, hmgpu_rank_model **out);
/* Adam on the mean squared error over n samples (X: n x 8 row-major, Y: ACA
 * ranks), mini-batches of `batch`; features are standardised with the
 * training set's mean and deviation. final_loss: 0.5 * mean squared error. */
int hmgpu_rank_model_train(hmgpu_rank_model *M, const float *X, const float *Y, int64_t n,
                           int64_t epochs, int64_t batch, float lr, uint64_t seed,
                           float *final_loss);
int hmgpu_rank_model_predict(hmgpu_rank_model *M, const float *X, int64_t n, float *out);
/* Gradient of 0.5 * mean((f(x) - y)^2) with respect to the parameters. */
int hmgpu_rank_model_gradients(hmgpu_rank_model *M, const float *X, const float *Y, int64_t n,
                               float *grad, float *loss);
/* Read and/or write the parameters (W1 64x8, b1, W2 64x64, b2, W3 1x64, b3,
 * row-major, concatenated) and the feature scaling (8 means, 8 deviations). */
int hmgpu_rank_model_params(hmgpu_rank_model *M, float *get, const float *set, float *norm_get,
                            const float *norm_set);
int hmgpu_rank_model_free(hmgpu_rank_model *M);
/* Features of the admissible leaves of BlockTree(X, Y; eta) in traversal order
 * (the order of hmgpu_hmatrix_aca_ranks): log m, log n, log diameters of the
 * target and source clusters, log centre distance, distance / (rX + rY),
 * log10 eps, log min(m, n). out: count x 8 (may be NULL to count). */
int hmgpu_block_features(const hmgpu_tree *X, const hmgpu_tree *Y, double eta, double eps,
                         float *out, int64_t *count);

#ifdef __cplusplus
}
#endif
#endif
