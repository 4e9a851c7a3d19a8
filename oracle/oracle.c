/*
 * oracle.c -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * FP64 CPU restatement of HMatrixGPU.jl's H-matrix path.  Every function cites
 * the reference file:line it follows.  Compiled with -O2 -ffp-contract=off so
 * that no multiply-add is fused: Julia does not contract either.
 */
#define _GNU_SOURCE
#include "oracle.h"
#include "or_internal.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------ */
/* small helpers                                                              */
/* ------------------------------------------------------------------------ */

/* Julia's isless-based "greater than" for Float64 as used by
 * sortperm(...; rev=true): NaN sorts above every number. */
static int jl_gt(double a, double b) {
  if (isnan(a)) return !isnan(b);
  if (isnan(b)) return 0;
  return a > b;
}

/* LinearAlgebra.generic_norm2 for a length-3 vector (Julia 1.10): unscaled
 * sequential sum of squares unless length*maxabs^2 overflows or maxabs^2
 * underflows, in which case the scaled loop is used. */
static double jl_norm3(double a, double b, double c) {
  if (isnan(a) || isnan(b) || isnan(c)) return NAN;
  double m = fabs(a);
  if (fabs(b) > m) m = fabs(b);
  if (fabs(c) > m) m = fabs(c);
  if (m == 0.0 || isinf(m)) return m;
  if (isfinite(3.0 * m * m) && m * m != 0.0) {
    double s = a * a;
    s += b * b;
    s += c * c;
    return sqrt(s);
  }
  double ta = fabs(a) / m, tb = fabs(b) / m, tc = fabs(c) / m;
  double s = ta * ta;
  s += tb * tb;
  s += tc * tc;
  return m * sqrt(s);
}

static int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }

/* Summation order of the sums inside ACA+ and the recompression.
 *
 * Julia reaches these sums through LAPACK (qr, svd: src/aca.jl:125-129) and
 * through `sum` (src/aca.jl:95-96), whose orders are blocked or SIMD-split and
 * are not pinned by any reference test. The oracle fixes one order instead,
 * the one a team of lanes gives when it sums a strided vector: a team of
 * `nt` lanes (32, or 256 for blocks with m + n >= 4096), lane t adding the
 * terms t, t + nt, t + 2 nt, ... in that order from 0.0; each group of 32
 * lanes folded by a butterfly (partners at distance 16, 8, 4, 2, 1); the
 * groups' sums then added in group order. Every term and every product
 * inside a term is the reference's. */
#define OR_TEAM_MIN_MN 4096
static int team_size(int64_t m, int64_t n) { return m + n >= OR_TEAM_MIN_MN ? 256 : 32; }

/* Folds the lane sums p[0..nt) in the order above. */
static double team_fold(const double *p, int nt) {
  double s = 0.0;
  for (int g = 0; g < nt / 32; g++) {
    double v[32], nv[32];
    memcpy(v, p + 32 * g, sizeof v);
    for (int o = 16; o > 0; o >>= 1) {
      for (int l = 0; l < 32; l++) nv[l] = v[l] + v[l ^ o];
      memcpy(v, nv, sizeof v);
    }
    s = g == 0 ? v[0] : s + v[0];
  }
  return s;
}

/* sum_{i0 <= i < len} a[i*sa] * b[i*sb], term i on lane (i - i0) mod nt. */
static double team_dot(const double *a, int64_t sa, const double *b, int64_t sb, int64_t i0,
                       int64_t len, int nt) {
  double p[256];
  for (int t = 0; t < nt; t++) p[t] = 0.0;
  for (int64_t base = i0; base < len; base += nt) {
    const int64_t cnt = len - base < nt ? len - base : nt;
    for (int64_t t = 0; t < cnt; t++) p[t] += a[(base + t) * sa] * b[(base + t) * sb];
  }
  return team_fold(p, nt);
}

/* ------------------------------------------------------------------------ */
/* cluster tree: src/tree.jl:45-137                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t start, end; /* 1-based start, exclusive end (src/tree.jl:6-14) */
  int8_t is_leaf;
  int64_t left, right;
  double center[3];
  double radius;
} or_node;

struct or_tree {
  int64_t npts, dims;
  int64_t *index_map; /* length dims*npts, 1-based */
  or_node *nodes;
  int64_t nnodes, cap;
};

static int64_t tree_push(or_tree *t) {
  if (t->nnodes == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 64;
    t->nodes = (or_node *)realloc(t->nodes, (size_t)t->cap * sizeof(or_node));
  }
  memset(&t->nodes[t->nnodes], 0, sizeof(or_node));
  return t->nnodes++;
}

/* build_tree_node, src/tree.jl:70-116. `idx` is the 1-based index map being
 * permuted in place; `scratch` has room for npts entries. */
static int build_tree_node(or_tree *t, const double *coords, int64_t leaf, int64_t *idx,
                           int64_t *scratch, int64_t start, int64_t end, int64_t *out) {
  int64_t me = tree_push(t);
  int64_t cnt = end - start;
  int64_t *view = idx + (start - 1);
  double mn[3], mx[3], sum[3] = {0.0, 0.0, 0.0};
  for (int a = 0; a < 3; a++) mn[a] = mx[a] = coords[3 * (view[0] - 1) + a];
  /* minimum/maximum(points; dims=2) (:78-79) and sum(points; dims=2) (:85):
   * sequential over columns. */
  for (int64_t p = 0; p < cnt; p++) {
    const double *q = coords + 3 * (view[p] - 1);
    for (int a = 0; a < 3; a++) {
      if (q[a] < mn[a] || isnan(q[a])) mn[a] = isnan(mn[a]) ? mn[a] : q[a];
      if (q[a] > mx[a] || isnan(q[a])) mx[a] = isnan(mx[a]) ? mx[a] : q[a];
      sum[a] += q[a];
    }
  }
  double box[3];
  for (int a = 0; a < 3; a++) box[a] = mx[a] - mn[a];
  int axis = 0; /* argmax(box_lengths): first maximum (:81) */
  for (int a = 1; a < 3; a++)
    if (jl_gt(box[a], box[axis])) axis = a;
  double center[3];
  for (int a = 0; a < 3; a++) center[a] = sum[a] / (double)cnt;
  double r1 = jl_norm3(center[0] - mx[0], center[1] - mx[1], center[2] - mx[2]);
  double r2 = jl_norm3(center[0] - mn[0], center[1] - mn[1], center[2] - mn[2]);
  double radius = (isnan(r1) || isnan(r2)) ? NAN : (r2 > r1 ? r2 : r1); /* :86-87 */

  or_node *nd = &t->nodes[me];
  nd->start = start;
  nd->end = end;
  memcpy(nd->center, center, sizeof center);
  nd->radius = radius;
  nd->left = nd->right = -1;
  if (cnt <= leaf) { /* :90-93 */
    nd->is_leaf = 1;
    *out = me;
    return 0;
  }
  /* stable split on x_axis < c_axis (:96-105) */
  int64_t nl = 0, nr = 0;
  for (int64_t p = 0; p < cnt; p++)
    if (coords[3 * (view[p] - 1) + axis] < center[axis]) scratch[nl++] = view[p];
  for (int64_t p = 0; p < cnt; p++)
    if (!(coords[3 * (view[p] - 1) + axis] < center[axis])) scratch[nl + nr++] = view[p];
  if (nl == 0 || nr == 0) return -2; /* the reference recurses without end here */
  memcpy(view, scratch, (size_t)cnt * sizeof(int64_t));
  int64_t split = start + nl, l, r;
  int rc = build_tree_node(t, coords, leaf, idx, scratch, start, split, &l);
  if (rc) return rc;
  rc = build_tree_node(t, coords, leaf, idx, scratch, split, end, &r);
  if (rc) return rc;
  t->nodes[me].left = l;
  t->nodes[me].right = r;
  *out = me;
  return 0;
}

int or_cluster_tree(const double *coords, int64_t npts, int64_t leaf, int64_t dims,
                    or_tree **out) {
  if (dims <= 0) return -1; /* src/tree.jl:46-48 */
  if (npts <= 0 || leaf <= 0) return -1;
  or_tree *t = (or_tree *)calloc(1, sizeof(or_tree));
  t->npts = npts;
  t->dims = dims;
  int64_t *idx = (int64_t *)malloc((size_t)npts * sizeof(int64_t));
  int64_t *scratch = (int64_t *)malloc((size_t)npts * sizeof(int64_t));
  for (int64_t i = 0; i < npts; i++) idx[i] = i + 1;
  int64_t root;
  int rc = build_tree_node(t, coords, leaf, idx, scratch, 1, npts + 1, &root);
  free(scratch);
  if (rc) {
    free(idx);
    or_tree_free(t);
    return rc;
  }
  if (dims > 1) {
    /* expanded index map (:59-61) and update_tree_indices! (:123-137) */
    int64_t *e = (int64_t *)malloc((size_t)(npts * dims) * sizeof(int64_t));
    for (int64_t p = 0; p < npts; p++)
      for (int64_t i = 1; i <= dims; i++) e[p * dims + (i - 1)] = dims * idx[p] - (dims - i);
    free(idx);
    idx = e;
    for (int64_t k = 0; k < t->nnodes; k++) {
      or_node *nd = &t->nodes[k];
      int64_t s = nd->start;
      nd->start = dims * (s - 1) + 1;
      nd->end = dims * (nd->end - s) + nd->start;
    }
  }
  t->index_map = idx;
  *out = t;
  return 0;
}

int64_t or_tree_num_nodes(const or_tree *t) { return t->nnodes; }
int64_t or_tree_index_len(const or_tree *t) { return t->npts * t->dims; }

void or_tree_export(const or_tree *t, int64_t *index_map, int64_t *start, int64_t *end,
                    int8_t *is_leaf, int64_t *left, int64_t *right, double *center,
                    double *radius) {
  if (index_map) memcpy(index_map, t->index_map, (size_t)(t->npts * t->dims) * sizeof(int64_t));
  for (int64_t k = 0; k < t->nnodes; k++) {
    const or_node *nd = &t->nodes[k];
    if (start) start[k] = nd->start;
    if (end) end[k] = nd->end;
    if (is_leaf) is_leaf[k] = nd->is_leaf;
    if (left) left[k] = nd->left;
    if (right) right[k] = nd->right;
    if (center) memcpy(center + 3 * k, nd->center, 3 * sizeof(double));
    if (radius) radius[k] = nd->radius;
  }
}

void or_tree_free(or_tree *t) {
  if (!t) return;
  free(t->index_map);
  free(t->nodes);
  free(t);
}

/* ------------------------------------------------------------------------ */
/* block tree: src/block.jl:31-155                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t x, y; /* target node, source node */
  int8_t adm, dense;
  int64_t left, right;
} or_bnode;

struct or_blocks {
  or_bnode *nodes;
  int64_t nnodes, cap;
  int64_t *dense, *approx; /* pairs */
  int64_t nd, na, capd, capa;
};

static int64_t bpush(or_blocks *b, int64_t x, int64_t y) {
  if (b->nnodes == b->cap) {
    b->cap = b->cap ? 2 * b->cap : 256;
    b->nodes = (or_bnode *)realloc(b->nodes, (size_t)b->cap * sizeof(or_bnode));
  }
  or_bnode *n = &b->nodes[b->nnodes];
  n->x = x;
  n->y = y;
  n->adm = n->dense = 0;
  n->left = n->right = -1;
  return b->nnodes++;
}

/* build_block_tree!, src/block.jl:58-90 */
static void build_block(or_blocks *b, const or_tree *X, const or_tree *Y, int64_t k, double eta) {
  const or_node *x = &X->nodes[b->nodes[k].x];
  const or_node *y = &Y->nodes[b->nodes[k].y];
  double dist = jl_norm3(x->center[0] - y->center[0], x->center[1] - y->center[1],
                         x->center[2] - y->center[2]);
  if (dist > eta * (x->radius + y->radius)) {
    b->nodes[k].adm = 1;
    return;
  } else if (x->is_leaf && y->is_leaf) {
    b->nodes[k].dense = 1;
    return;
  }
  int split_y = (!y->is_leaf && y->radius > x->radius) || x->is_leaf;
  int64_t xi = b->nodes[k].x, yi = b->nodes[k].y, l, r;
  if (split_y) {
    l = bpush(b, xi, y->left);
    r = bpush(b, xi, y->right);
  } else {
    l = bpush(b, x->left, yi);
    r = bpush(b, x->right, yi);
  }
  b->nodes[k].left = l;
  b->nodes[k].right = r;
  build_block(b, X, Y, l, eta);
  build_block(b, X, Y, r, eta);
}

/* merge_dense_matrices!, src/block.jl:98-112 */
static void merge_dense(or_blocks *b, int64_t k) {
  or_bnode *n = &b->nodes[k];
  if (n->left >= 0 && n->right >= 0) {
    merge_dense(b, n->left);
    merge_dense(b, n->right);
    n = &b->nodes[k];
    n->dense = b->nodes[n->left].dense && b->nodes[n->right].dense;
  }
}

static void push_pair(int64_t **arr, int64_t *len, int64_t *cap, int64_t x, int64_t y) {
  if (*len == *cap) {
    *cap = *cap ? 2 * *cap : 256;
    *arr = (int64_t *)realloc(*arr, (size_t)(2 * *cap) * sizeof(int64_t));
  }
  (*arr)[2 * *len] = x;
  (*arr)[2 * *len + 1] = y;
  (*len)++;
}

/* traverse, src/block.jl:127-155: pre-order, left before right. */
static void traverse(or_blocks *b, int64_t k) {
  const or_bnode *n = &b->nodes[k];
  if (n->adm)
    push_pair(&b->approx, &b->na, &b->capa, n->x, n->y);
  else if (n->dense)
    push_pair(&b->dense, &b->nd, &b->capd, n->x, n->y);
  if (!n->dense && !n->adm) {
    if (n->left >= 0) traverse(b, n->left);
    if (n->right >= 0) traverse(b, n->right);
  }
}

int or_block_tree(const or_tree *X, const or_tree *Y, double eta, int merge, or_blocks **out) {
  or_blocks *b = (or_blocks *)calloc(1, sizeof(or_blocks));
  bpush(b, 0, 0);
  build_block(b, X, Y, 0, eta);
  if (merge) merge_dense(b, 0);
  traverse(b, 0);
  *out = b;
  return 0;
}

int64_t or_sparsify(const or_kernel *K, const or_tree *X, const or_tree *Y, double eta, int64_t *I,
                    int64_t *J, double *V) {
  or_blocks *b = NULL;
  or_block_tree(X, Y, eta, 1, &b); /* BlockTree + merge_dense_matrices! (:236-237), traverse (:239) */
  int64_t cnt = 0;
  for (int64_t p = 0; p < b->nd; p++) { /* :250-264 */
    const or_node *a = &X->nodes[b->dense[2 * p]], *c = &Y->nodes[b->dense[2 * p + 1]];
    for (int64_t i = a->start; i < a->end; i++) {
      const int64_t row = X->index_map[i - 1];
      for (int64_t j = c->start; j < c->end; j++, cnt++) {
        if (!I) continue;
        const int64_t col = Y->index_map[j - 1];
        I[cnt] = row;
        J[cnt] = col;
        V[cnt] = or_kernel_entry(K, row, col);
      }
    }
  }
  or_blocks_free(b);
  return cnt;
}

int64_t or_blocks_num_dense(const or_blocks *b) { return b->nd; }
int64_t or_blocks_num_approx(const or_blocks *b) { return b->na; }
int64_t or_blocks_num_nodes(const or_blocks *b) { return b->nnodes; }
void or_blocks_export(const or_blocks *b, int64_t *dense_pairs, int64_t *approx_pairs) {
  if (dense_pairs && b->nd) memcpy(dense_pairs, b->dense, (size_t)(2 * b->nd) * sizeof(int64_t));
  if (approx_pairs && b->na)
    memcpy(approx_pairs, b->approx, (size_t)(2 * b->na) * sizeof(int64_t));
}
void or_blocks_export_nodes(const or_blocks *b, int64_t *target, int64_t *source,
                            int8_t *admissible, int8_t *dense, int64_t *left, int64_t *right) {
  for (int64_t k = 0; k < b->nnodes; k++) {
    target[k] = b->nodes[k].x;
    source[k] = b->nodes[k].y;
    admissible[k] = b->nodes[k].adm;
    dense[k] = b->nodes[k].dense;
    left[k] = b->nodes[k].left;
    right[k] = b->nodes[k].right;
  }
}
void or_blocks_free(or_blocks *b) {
  if (!b) return;
  free(b->nodes);
  free(b->dense);
  free(b->approx);
  free(b);
}

/* ------------------------------------------------------------------------ */
/* matrix entries                                                             */
/* ------------------------------------------------------------------------ */

static const double OR_INV4PI = 0.07957747154594767; /* 1/(4 pi) rounded to FP64 */

static double dip_xx(double x, double y, double z) { /* examples/hmatrix_vector.jl:12-19 */
  double R = x * x + y * y + z * z;
  if (R == 0) return 0.0;
  return -(2 * x * x - y * y - z * z) / (R * R * sqrt(R)) / (4 * M_PI);
}
static double dip_xy(double x, double y, double z) { /* :21-28 */
  double R = x * x + y * y + z * z;
  if (R == 0) return 0.0;
  return -3 * x * y / (R * R * sqrt(R)) / (4 * M_PI);
}

double or_kernel_entry(const or_kernel *K, int64_t i, int64_t j) {
  switch (K->type) {
  case OR_KERNEL_EXPLICIT:
    return K->A[(i - 1) + (j - 1) * K->lda];
  case OR_KERNEL_LAPLACE3D:
  case OR_KERNEL_YUKAWA: {
    const double *p = K->X + 3 * (i - 1), *q = K->Y + 3 * (j - 1);
    double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (r == 0.0) return 0.0;
    return K->type == OR_KERNEL_LAPLACE3D ? OR_INV4PI / r : exp(-r) / r;
  }
  case OR_KERNEL_LOG2D: { /* test/test_hmatrix.jl:170-173 */
    const double *p = K->X + 3 * (i - 1), *q = K->Y + 3 * (j - 1);
    double d = jl_norm3(p[0] - q[0], p[1] - q[1], p[2] - q[2]);
    return d < 1e-12 ? 1.0 : (-0.5 / M_PI) * log(d);
  }
  case OR_KERNEL_VECTOR_R: { /* test/test_hmatrix_vector.jl:334-340 */
    int64_t J = (j - 1) / 3, c = (j - 1) % 3;
    const double *p = K->X + 3 * (i - 1), *q = K->Y + 3 * J;
    double R[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
    double r = jl_norm3(R[0], R[1], R[2]);
    return r < 1e-12 ? 1.0 : R[c] / (r * r);
  }
  case OR_KERNEL_DIPOLAR: { /* examples/hmatrix_vector.jl:46-80 */
    int64_t pi_ = (i - 1) / 3, a = (i - 1) % 3, pj = (j - 1) / 3, b = (j - 1) % 3;
    const double *p = K->X + 3 * pi_, *q = K->Y + 3 * pj;
    double x = p[0] - q[0], y = p[1] - q[1], z = p[2] - q[2];
    int ab = a < b ? a * 3 + b : b * 3 + a;
    switch (ab) {
    case 0: return dip_xx(x, y, z);
    case 1: return dip_xy(x, y, z);
    case 2: return dip_xy(x, z, y);
    case 4: return dip_xx(y, x, z);
    case 5: return dip_xy(y, z, x);
    default: return dip_xx(z, y, x);
    }
  }
  }
  return NAN;
}

void or_kernel_matvec(const or_kernel *K, const double *x, double *y) {
  for (int64_t i = 1; i <= K->nrows; i++) {
    double s = 0.0;
    for (int64_t j = 1; j <= K->ncols; j++) s += or_kernel_entry(K, i, j) * x[j - 1];
    y[i - 1] = s;
  }
}

/* ------------------------------------------------------------------------ */
/* ACA+: src/aca.jl:9-106                                                     */
/* ------------------------------------------------------------------------ */

/* argmax_not_in_list (src/aca.jl:9-17) over |a|: the maximum under
 * sortperm(rev=true), ties broken by the lowest index; -1 if all are used. */
static int64_t argmax_not_in(const double *a, int64_t n, const char *used) {
  int64_t best = -1;
  for (int64_t i = 0; i < n; i++) {
    if (used[i]) continue;
    if (best < 0 || jl_gt(fabs(a[i]), fabs(a[best]))) best = i;
  }
  return best;
}

/* ACA+ core. U (m x k, column-major, ld m) and V (k x n, row-major) are
 * allocated here and doubled as terms are added, so a block of rank k holds
 * O(k (m + n)) memory whatever its size. */
static int aca_core(const or_kernel *K, const int64_t *rows, int64_t m, const int64_t *cols,
                    int64_t n, double eps, int64_t max_iter, double **Up, double **Vp,
                    int64_t *rank) {
  if (max_iter <= 0) max_iter = m; /* default max_iter = n_rows (:36) */
  max_iter = imin(imin(m, n), max_iter);
  const int nt = team_size(m, n);
  int64_t cap = imin(max_iter, 16);
  if (cap < 1) cap = 1;
  double *U = (double *)malloc((size_t)(m * cap) * sizeof(double));
  double *V = (double *)malloc((size_t)(cap * n) * sizeof(double));
  double *rrow = (double *)calloc((size_t)n, sizeof(double));
  double *rcol = (double *)calloc((size_t)m, sizeof(double));
  char *used_r = (char *)calloc((size_t)m, 1), *used_c = (char *)calloc((size_t)n, 1);
  if (!U || !V || !rrow || !rcol || !used_r || !used_c) return -2;
  int64_t k = 0;
  for (int64_t it = 1; it <= max_iter; it++) {
    int64_t rp, cp;
    if (it == 1) {
      rp = cp = 0; /* :69-70 */
    } else {     /* :72-73, from the previous residuals */
      cp = argmax_not_in(rrow, n, used_c);
      rp = argmax_not_in(rcol, m, used_r);
    }
    double cval = fabs(rrow[cp]), rval = fabs(rcol[rp]);
    /* calc_residual_rows / calc_residual_cols (:43-58): K entries minus the
     * accumulated terms, one term at a time in order. */
#define RES_ROW(I)                                                            \
  do {                                                                        \
    for (int64_t j = 0; j < n; j++) rrow[j] = or_kernel_entry(K, rows[I], cols[j]); \
    for (int64_t q = 0; q < k; q++) {                                         \
      double s = U[(I) + q * m];                                              \
      const double *vq = V + q * n;                                           \
      for (int64_t j = 0; j < n; j++) rrow[j] -= s * vq[j];                   \
    }                                                                         \
  } while (0)
#define RES_COL(J)                                                            \
  do {                                                                        \
    for (int64_t i = 0; i < m; i++) rcol[i] = or_kernel_entry(K, rows[i], cols[J]); \
    for (int64_t q = 0; q < k; q++) {                                         \
      double s = V[q * n + (J)];                                              \
      const double *uq = U + q * m;                                           \
      for (int64_t i = 0; i < m; i++) rcol[i] -= uq[i] * s;                   \
    }                                                                         \
  } while (0)
    if (rval > cval) { /* :79-82 */
      RES_ROW(rp);
      cp = argmax_not_in(rrow, n, used_c);
      RES_COL(cp);
    } else { /* :83-87 */
      RES_COL(cp);
      rp = argmax_not_in(rcol, m, used_r);
      RES_ROW(rp);
    }
#undef RES_ROW
#undef RES_COL
    used_r[rp] = 1;
    used_c[cp] = 1;
    if (k == cap) { /* room for more terms */
      cap = imin(2 * cap, max_iter);
      U = (double *)realloc(U, (size_t)(m * cap) * sizeof(double));
      V = (double *)realloc(V, (size_t)(cap * n) * sizeof(double));
      if (!U || !V) return -2;
    }
    double piv = rrow[cp];
    double *vk = V + k * n, *uk = U + k * m;
    for (int64_t j = 0; j < n; j++) vk[j] = rrow[j] / piv; /* :92 */
    for (int64_t i = 0; i < m; i++) uk[i] = rcol[i];       /* :93 */
    /* sum(v.^2), sum(u.^2) in the team order (top of this file) */
    double sv = team_dot(vk, 1, vk, 1, 0, n, nt);
    double su = team_dot(uk, 1, uk, 1, 0, m, nt);
    k++;
    if (sqrt(su * sv) < eps) break; /* :95-99 */
  }
  free(rrow);
  free(rcol);
  free(used_r);
  free(used_c);
  *Up = U;
  *Vp = V;
  *rank = k;
  return 0;
}

int or_aca_plus(const or_kernel *K, const int64_t *rows, int64_t m, const int64_t *cols,
                int64_t n, double eps, int64_t max_iter, int64_t cap, double *U, double *V,
                int64_t *rank) {
  int64_t mi = max_iter <= 0 ? m : max_iter;
  if (cap < imin(imin(m, n), mi)) return -1;
  double *Uc, *Vr;
  int64_t k;
  int rc = aca_core(K, rows, m, cols, n, eps, max_iter, &Uc, &Vr, &k);
  if (rc) return rc;
  memcpy(U, Uc, (size_t)(m * k) * sizeof(double));
  for (int64_t q = 0; q < k; q++)
    for (int64_t j = 0; j < n; j++) V[q + j * cap] = Vr[q * n + j];
  free(Uc);
  free(Vr);
  *rank = k;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Householder QR and one-sided Jacobi SVD (published methods; FP64)          */
/* ------------------------------------------------------------------------ */

/* Unblocked Householder QR of A (m x k, col-major, m >= k), LAPACK dgeqr2
 * conventions: reflectors below the diagonal, tau[j], R (k x k, col-major).
 * The column norms and the reflections' dot products are sums in the team
 * order of `nt` lanes (top of this file). */
static void reflect(const double *x, int64_t len, double tau, double *y, int nt) {
  /* y := (I - tau v v') y with v = [1; x[1..len)] */
  double w = (team_dot(x, 1, y, 1, 1, len, nt) + y[0]) * tau;
  y[0] -= w;
  for (int64_t i = 1; i < len; i++) y[i] -= w * x[i];
}

int or_qr(int64_t m, int64_t k, double *A, double *tau, double *R, int nt) {
  if (nt != 32 && nt != 256) return -1;
  for (int64_t j = 0; j < k; j++) {
    double *x = A + j + j * m;
    int64_t len = m - j;
    double xn = sqrt(team_dot(x, 1, x, 1, 1, len, nt));
    double alpha = x[0];
    if (xn == 0.0) {
      tau[j] = 0.0;
    } else {
      double beta = -copysign(sqrt(alpha * alpha + xn * xn), alpha);
      tau[j] = (beta - alpha) / beta;
      double sc = 1.0 / (alpha - beta);
      for (int64_t i = 1; i < len; i++) x[i] *= sc;
      x[0] = beta;
    }
    /* apply H_j = I - tau v v^T to the trailing columns */
    for (int64_t c = j + 1; c < k; c++) reflect(x, len, tau[j], A + j + c * m, nt);
  }
  if (R) {
    for (int64_t c = 0; c < k; c++)
      for (int64_t r = 0; r < k; r++) R[r + c * k] = r <= c ? A[r + c * m] : 0.0;
  }
  return 0;
}

/* B (m x p, col-major) := Q_thin * [C; 0] where C is k x p and Q's reflectors
 * are in QR (m x k) and tau. */
static void qr_apply_thin(int64_t m, int64_t k, const double *QR, const double *tau,
                          const double *C, int64_t p, double *B, int nt) {
  for (int64_t c = 0; c < p; c++) {
    double *y = B + c * m;
    for (int64_t i = 0; i < m; i++) y[i] = i < k ? C[i + c * k] : 0.0;
    for (int64_t j = k - 1; j >= 0; j--) reflect(QR + j + j * m, m - j, tau[j], y + j, nt);
  }
}

/* One-sided (Hestenes) Jacobi SVD of A (k x k, col-major), in place: on exit
 * the columns of A are W*Sigma, Vj (k x k) holds Z, sigma the column norms and
 * order[] the column indices sorted by decreasing sigma (stable). */
int or_jacobi_svd(int64_t k, double *A, double *Vj, double *sigma, int64_t *order) {
  for (int64_t i = 0; i < k * k; i++) Vj[i] = 0.0;
  for (int64_t i = 0; i < k; i++) Vj[i + i * k] = 1.0;
  for (int sweep = 0; sweep < 80; sweep++) {
    int rotated = 0;
    for (int64_t p = 0; p < k - 1; p++) {
      for (int64_t q = p + 1; q < k; q++) {
        double *ap = A + p * k, *aq = A + q * k;
        double alpha = 0.0, beta = 0.0, gamma = 0.0;
        for (int64_t i = 0; i < k; i++) {
          alpha += ap[i] * ap[i];
          beta += aq[i] * aq[i];
          gamma += ap[i] * aq[i];
        }
        if (gamma == 0.0 || fabs(gamma) <= 1e-15 * sqrt(alpha * beta)) continue;
        rotated = 1;
        double zeta = (beta - alpha) / (2.0 * gamma);
        double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        for (int64_t i = 0; i < k; i++) {
          double u = ap[i], v = aq[i];
          ap[i] = c * u - s * v;
          aq[i] = s * u + c * v;
        }
        double *vp = Vj + p * k, *vq = Vj + q * k;
        for (int64_t i = 0; i < k; i++) {
          double u = vp[i], v = vq[i];
          vp[i] = c * u - s * v;
          vq[i] = s * u + c * v;
        }
      }
    }
    if (!rotated) break;
  }
  for (int64_t j = 0; j < k; j++) {
    double s = 0.0;
    for (int64_t i = 0; i < k; i++) s += A[i + j * k] * A[i + j * k];
    sigma[j] = sqrt(s);
    order[j] = j;
  }
  /* stable insertion sort by decreasing sigma */
  for (int64_t i = 1; i < k; i++) {
    int64_t v = order[i], j = i - 1;
    while (j >= 0 && sigma[order[j]] < sigma[v]) {
      order[j + 1] = order[j];
      j--;
    }
    order[j + 1] = v;
  }
  return 0;
}

/* SVD_recompress, src/aca.jl:123-143. */
int or_svd_recompress(int64_t m, int64_t n, int64_t k, const double *U, const double *V,
                      double eps, double *U_out, double *V_out, int64_t *r_out) {
  if (k == 0) {
    *r_out = 0;
    return 0;
  }
  if (m < k || n < k) return -1;
  double *QU = (double *)malloc((size_t)(m * k) * sizeof(double));
  double *QV = (double *)malloc((size_t)(n * k) * sizeof(double));
  double *tu = (double *)malloc((size_t)k * sizeof(double));
  double *tv = (double *)malloc((size_t)k * sizeof(double));
  double *RU = (double *)malloc((size_t)(k * k) * sizeof(double));
  double *RV = (double *)malloc((size_t)(k * k) * sizeof(double));
  double *M = (double *)malloc((size_t)(k * k) * sizeof(double));
  double *Z = (double *)malloc((size_t)(k * k) * sizeof(double));
  double *sig = (double *)malloc((size_t)k * sizeof(double));
  int64_t *ord = (int64_t *)malloc((size_t)k * sizeof(int64_t));
  memcpy(QU, U, (size_t)(m * k) * sizeof(double));
  for (int64_t j = 0; j < n; j++) /* V' (n x k) */
    for (int64_t q = 0; q < k; q++) QV[j + q * n] = V[q + j * k];
  const int nt = team_size(m, n);
  or_qr(m, k, QU, tu, RU, nt); /* :125 */
  or_qr(n, k, QV, tv, RV, nt); /* :126 */
  for (int64_t c = 0; c < k; c++) /* RU * RV' (:129) */
    for (int64_t r = 0; r < k; r++) {
      double s = 0.0;
      for (int64_t q = 0; q < k; q++) s += RU[r + q * k] * RV[c + q * k];
      M[r + c * k] = s;
    }
  or_jacobi_svd(k, M, Z, sig, ord);
  /* tail norms sqrt(sum_{j>=i} sigma_j^2) accumulated from the smallest (:132) */
  int64_t r = k;
  double *tail = (double *)malloc((size_t)k * sizeof(double));
  double acc = 0.0;
  for (int64_t i = k - 1; i >= 0; i--) {
    acc += sig[ord[i]] * sig[ord[i]];
    tail[i] = sqrt(acc);
  }
  for (int64_t i = 0; i < k; i++)
    if (tail[i] < eps) { /* :135-136 */
      r = i;
      break;
    }
  free(tail);
  /* U_SVD = QU * (W_r .* sigma_r') -- the rotated columns already equal
   * W*Sigma; V_SVD = Z_r' * QV' (:139-140). */
  double *C = (double *)malloc((size_t)(k * (r ? r : 1)) * sizeof(double));
  for (int64_t c = 0; c < r; c++)
    for (int64_t i = 0; i < k; i++) C[i + c * k] = M[i + ord[c] * k];
  qr_apply_thin(m, k, QU, tu, C, r, U_out, nt);
  for (int64_t c = 0; c < r; c++)
    for (int64_t i = 0; i < k; i++) C[i + c * k] = Z[i + ord[c] * k];
  double *B = (double *)malloc((size_t)(n * (r ? r : 1)) * sizeof(double));
  qr_apply_thin(n, k, QV, tv, C, r, B, nt);
  for (int64_t c = 0; c < r; c++)
    for (int64_t j = 0; j < n; j++) V_out[c + j * r] = B[j + c * n];
  free(B);
  free(C);
  free(QU);
  free(QV);
  free(tu);
  free(tv);
  free(RU);
  free(RV);
  free(M);
  free(Z);
  free(sig);
  free(ord);
  *r_out = r;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* assembly: src/hmatrix.jl:72-217                                            */
/* ------------------------------------------------------------------------ */


typedef struct {
  const or_kernel *K;
  const int64_t *tmap, *smap;
  const or_tree *X, *Y;
  const int64_t *pairs;
  int64_t npairs;
  double eps;
  int svd;
  int64_t next;
  pthread_mutex_t mu;
  /* outputs per pair */
  int64_t *aca_rank, *rank;
  double **U, **V;
} build_ctx;

static void fill_dense(const or_kernel *K, const int64_t *tid, int64_t m, const int64_t *sid,
                       int64_t n, double *D) {
  for (int64_t i = 0; i < m; i++)
    for (int64_t j = 0; j < n; j++) D[i * n + j] = or_kernel_entry(K, tid[i], sid[j]);
}

/* One admissible block: ACA at eps/10, recompress at eps (:189-199). */
static void approx_one(build_ctx *c, int64_t p) {
  const or_node *a = &c->X->nodes[c->pairs[2 * p]], *b = &c->Y->nodes[c->pairs[2 * p + 1]];
  int64_t m = a->end - a->start, n = b->end - b->start;
  const int64_t *tid = c->tmap + (a->start - 1), *sid = c->smap + (b->start - 1);
  double *U, *Vr;
  int64_t k;
  aca_core(c->K, tid, m, sid, n, c->eps / 10.0, m, &U, &Vr, &k);
  c->aca_rank[p] = k;
  double *Uo = U, *Vo;
  int64_t r = k;
  /* V as k x n column-major (leading dimension k) */
  double *Vc = (double *)malloc((size_t)((k ? k : 1) * n) * sizeof(double));
  for (int64_t j = 0; j < n; j++)
    for (int64_t q = 0; q < k; q++) Vc[q + j * k] = Vr[q * n + j];
  free(Vr);
  if (c->svd) {
    double *U2 = (double *)malloc((size_t)(m * (k ? k : 1)) * sizeof(double));
    double *V2 = (double *)malloc((size_t)((k ? k : 1) * n) * sizeof(double));
    or_svd_recompress(m, n, k, U, Vc, c->eps, U2, V2, &r);
    free(U);
    free(Vc);
    Uo = U2;
    Vo = V2;
  } else {
    Vo = Vc;
  }
  c->rank[p] = r;
  c->U[p] = Uo; /* m x r col-major, ld m */
  c->V[p] = Vo; /* r x n col-major, ld r */
}

/* Runs fn(ctx, i) for i in [0, n) on nthreads threads (items handed out in
 * order from a shared counter). */
typedef struct {
  void (*fn)(void *, int64_t);
  void *ctx;
  int64_t n, next;
  pthread_mutex_t mu;
} par_ctx;

static void *par_worker(void *arg) {
  par_ctx *c = (par_ctx *)arg;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int64_t i = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (i >= c->n) break;
    c->fn(c->ctx, i);
  }
  return NULL;
}

static void par_for(int nthreads, int64_t n, void (*fn)(void *, int64_t), void *ctx) {
  par_ctx c;
  c.fn = fn;
  c.ctx = ctx;
  c.n = n;
  c.next = 0;
  pthread_mutex_init(&c.mu, NULL);
  if (nthreads <= 1) {
    par_worker(&c);
  } else {
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, par_worker, &c);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
  }
  pthread_mutex_destroy(&c.mu);
}

typedef struct {
  const or_kernel *K;
  const or_hmatrix *h;
} fill_ctx;

static void fill_one(void *arg, int64_t b) {
  fill_ctx *c = (fill_ctx *)arg;
  or_block *B = &c->h->dense[b];
  int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1;
  fill_dense(c->K, c->h->tmap + (B->rs - 1), m, c->h->smap + (B->cs - 1), n, B->D);
}

static void *build_worker(void *arg) {
  build_ctx *c = (build_ctx *)arg;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int64_t p = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (p >= c->npairs) break;
    approx_one(c, p);
  }
  return NULL;
}

int or_hmatrix_build(const or_kernel *K, const or_tree *X, const or_tree *Y, double eta,
                     double eps, int svd_recompress, int64_t stride, int nthreads,
                     or_hmatrix **out) {
  if (stride < 1) stride = 1;
  if (nthreads < 1) nthreads = 1;
  or_blocks *bt;
  or_block_tree(X, Y, eta, 1, &bt); /* :74-78 */
  or_hmatrix *h = (or_hmatrix *)calloc(1, sizeof(or_hmatrix));
  h->m = K->nrows;
  h->n = K->ncols;
  h->tlen = or_tree_index_len(X);
  h->slen = or_tree_index_len(Y);
  h->tmap = (int64_t *)malloc((size_t)h->tlen * sizeof(int64_t));
  h->smap = (int64_t *)malloc((size_t)h->slen * sizeof(int64_t));
  memcpy(h->tmap, X->index_map, (size_t)h->tlen * sizeof(int64_t));
  memcpy(h->smap, Y->index_map, (size_t)h->slen * sizeof(int64_t));

  /* sampled subsets of both lists */
  int64_t nds = (bt->nd + stride - 1) / stride, nas = (bt->na + stride - 1) / stride;
  int64_t *apairs = (int64_t *)malloc((size_t)(2 * (nas ? nas : 1)) * sizeof(int64_t));
  for (int64_t q = 0; q < nas; q++) {
    apairs[2 * q] = bt->approx[2 * q * stride];
    apairs[2 * q + 1] = bt->approx[2 * q * stride + 1];
  }
  /* dense blocks (:180-186) */
  h->dense = (or_block *)calloc((size_t)(nds + nas + 1), sizeof(or_block));
  for (int64_t q = 0; q < nds; q++) {
    const or_node *a = &X->nodes[bt->dense[2 * q * stride]];
    const or_node *b = &Y->nodes[bt->dense[2 * q * stride + 1]];
    or_block *B = &h->dense[h->nd++];
    B->rs = a->start;
    B->re = a->end - 1;
    B->cs = b->start;
    B->ce = b->end - 1;
    int64_t m = a->end - a->start, n = b->end - b->start;
    B->D = (double *)malloc((size_t)(m * n) * sizeof(double));
  }
  fill_ctx fc = {K, h};
  par_for(nthreads, h->nd, fill_one, &fc);
  /* admissible blocks (:189-214), computed in parallel, stored in order */
  build_ctx c;
  memset(&c, 0, sizeof c);
  c.K = K;
  c.tmap = h->tmap;
  c.smap = h->smap;
  c.X = X;
  c.Y = Y;
  c.pairs = apairs;
  c.npairs = nas;
  c.eps = eps;
  c.svd = svd_recompress;
  pthread_mutex_init(&c.mu, NULL);
  c.aca_rank = (int64_t *)calloc((size_t)(nas + 1), sizeof(int64_t));
  c.rank = (int64_t *)calloc((size_t)(nas + 1), sizeof(int64_t));
  c.U = (double **)calloc((size_t)(nas + 1), sizeof(double *));
  c.V = (double **)calloc((size_t)(nas + 1), sizeof(double *));
  if (nthreads == 1) {
    build_worker(&c);
  } else {
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, build_worker, &c);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
  }
  pthread_mutex_destroy(&c.mu);
  h->approx = (or_block *)calloc((size_t)(nas + 1), sizeof(or_block));
  h->ncand = nas;
  h->aca_rank = c.aca_rank;
  h->final_rank = c.rank;
  for (int64_t q = 0; q < nas; q++) {
    const or_node *a = &X->nodes[apairs[2 * q]], *b = &Y->nodes[apairs[2 * q + 1]];
    int64_t m = a->end - a->start, n = b->end - b->start, r = c.rank[q];
    if (m * r + r * n < m * n) { /* :202-207, stored row-major */
      or_block *B = &h->approx[h->na++];
      B->rs = a->start;
      B->re = a->end - 1;
      B->cs = b->start;
      B->ce = b->end - 1;
      B->r = r;
      B->U = (double *)malloc((size_t)(m * r + 1) * sizeof(double));
      B->V = (double *)malloc((size_t)(r * n + 1) * sizeof(double));
      for (int64_t i = 0; i < m; i++)
        for (int64_t q2 = 0; q2 < r; q2++) B->U[i * r + q2] = c.U[q][i + q2 * m];
      for (int64_t q2 = 0; q2 < r; q2++)
        for (int64_t j = 0; j < n; j++) B->V[q2 * n + j] = c.V[q][q2 + j * r];
    } else { /* :208-213: appended to the dense list */
      or_block *B = &h->dense[h->nd++];
      B->rs = a->start;
      B->re = a->end - 1;
      B->cs = b->start;
      B->ce = b->end - 1;
      B->D = (double *)malloc((size_t)(m * n) * sizeof(double));
      fill_dense(K, h->tmap + (a->start - 1), m, h->smap + (b->start - 1), n, B->D);
      c.rank[q] = -1;
    }
    free(c.U[q]);
    free(c.V[q]);
  }
  free(c.U);
  free(c.V);
  free(apairs);
  or_blocks_free(bt);
  *out = h;
  return 0;
}

void or_hmatrix_sizes(const or_hmatrix *h, int64_t *m, int64_t *n, int64_t *nD, int64_t *nA,
                      int64_t *R, int64_t *dense_len, int64_t *U_len, int64_t *V_len) {
  int64_t r = 0, dl = 0, ul = 0, vl = 0;
  for (int64_t b = 0; b < h->nd; b++) {
    const or_block *B = &h->dense[b];
    dl += (B->re - B->rs + 1) * (B->ce - B->cs + 1);
  }
  for (int64_t b = 0; b < h->na; b++) {
    const or_block *B = &h->approx[b];
    r += B->r;
    ul += (B->re - B->rs + 1) * B->r;
    vl += (B->ce - B->cs + 1) * B->r;
  }
  *m = h->m;
  *n = h->n;
  *nD = h->nd;
  *nA = h->na;
  *R = r;
  *dense_len = dl;
  *U_len = ul;
  *V_len = vl;
}

/* flatten, src/hmatrix.jl:95-147 */
void or_hmatrix_export(const or_hmatrix *h, int64_t *tmap, int64_t *smap, int64_t *dense_idx,
                       int64_t *U_idx, int64_t *V_idx, double *dense_data, double *U_data,
                       double *V_data) {
  if (tmap) memcpy(tmap, h->tmap, (size_t)h->tlen * sizeof(int64_t));
  if (smap) memcpy(smap, h->smap, (size_t)h->slen * sizeof(int64_t));
  int64_t off = 0;
  for (int64_t b = 0; b < h->nd; b++) {
    const or_block *B = &h->dense[b];
    int64_t len = (B->re - B->rs + 1) * (B->ce - B->cs + 1);
    if (dense_idx) {
      int64_t *d = dense_idx + 5 * b;
      d[0] = B->rs;
      d[1] = B->re;
      d[2] = B->cs;
      d[3] = B->ce;
      d[4] = off;
    }
    if (dense_data) memcpy(dense_data + off, B->D, (size_t)len * sizeof(double));
    off += len;
  }
  int64_t uoff = 0, voff = 0, row = 0;
  for (int64_t b = 0; b < h->na; b++) {
    const or_block *B = &h->approx[b];
    int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1, r = B->r;
    if (U_idx) {
      int64_t *u = U_idx + 5 * b;
      u[0] = B->rs;
      u[1] = B->re;
      u[2] = row + 1; /* :127-128 */
      u[3] = row + r;
      u[4] = uoff;
    }
    if (U_data) memcpy(U_data + uoff, B->U, (size_t)(m * r) * sizeof(double));
    if (V_data) memcpy(V_data + voff, B->V, (size_t)(r * n) * sizeof(double));
    for (int64_t q = 0; q < r; q++) { /* :115-125 */
      if (V_idx) {
        int64_t *v = V_idx + 3 * (row + q);
        v[0] = B->cs;
        v[1] = B->ce;
        v[2] = voff + q * n;
      }
    }
    uoff += m * r;
    voff += r * n;
    row += r;
  }
}

void or_hmatrix_aca_ranks(const or_hmatrix *h, int64_t *aca_rank, int64_t *final_rank) {
  if (aca_rank) memcpy(aca_rank, h->aca_rank, (size_t)h->ncand * sizeof(int64_t));
  if (final_rank) memcpy(final_rank, h->final_rank, (size_t)h->ncand * sizeof(int64_t));
}
int64_t or_hmatrix_num_approx_candidates(const or_hmatrix *h) { return h->ncand; }

void or_hmatrix_free(or_hmatrix *h) {
  if (!h) return;
  for (int64_t b = 0; b < h->nd; b++) free(h->dense[b].D);
  for (int64_t b = 0; b < h->na; b++) {
    free(h->approx[b].U);
    free(h->approx[b].V);
  }
  free(h->dense);
  free(h->approx);
  free(h->tmap);
  free(h->smap);
  free(h->aca_rank);
  free(h->final_rank);
  free(h);
}

/* ------------------------------------------------------------------------ */
/* products: src/mult.jl                                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  const or_hmatrix *h;
  const double *xo;
  double *acc; /* private accumulator, length tlen */
  int64_t b0, b1; /* range in the combined [dense | approx] block list */
  double *tmp;
} mul_ctx;

/* One block's contribution: result[rs:re] .+= D*x or U*(V*x) (src/mult.jl:13-27).
 * Each gemv row is a sequential dot product. */
static void mul_block(const or_hmatrix *h, int64_t b, const double *xo, double *acc,
                      double *tmp) {
  if (b < h->nd) {
    const or_block *B = &h->dense[b];
    int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1;
    const double *x = xo + (B->cs - 1);
    for (int64_t i = 0; i < m; i++) {
      const double *d = B->D + i * n;
      double s = 0.0;
      for (int64_t j = 0; j < n; j++) s += d[j] * x[j];
      acc[B->rs - 1 + i] += s;
    }
  } else {
    const or_block *B = &h->approx[b - h->nd];
    int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1, r = B->r;
    const double *x = xo + (B->cs - 1);
    for (int64_t q = 0; q < r; q++) {
      const double *v = B->V + q * n;
      double s = 0.0;
      for (int64_t j = 0; j < n; j++) s += v[j] * x[j];
      tmp[q] = s;
    }
    for (int64_t i = 0; i < m; i++) {
      const double *u = B->U + i * r;
      double s = 0.0;
      for (int64_t q = 0; q < r; q++) s += u[q] * tmp[q];
      acc[B->rs - 1 + i] += s;
    }
  }
}

static void *mul_worker(void *arg) {
  mul_ctx *c = (mul_ctx *)arg;
  for (int64_t b = c->b0; b < c->b1; b++) mul_block(c->h, b, c->xo, c->acc, c->tmp);
  return NULL;
}

static int64_t max_rank(const or_hmatrix *h) {
  int64_t r = 1;
  for (int64_t b = 0; b < h->na; b++)
    if (h->approx[b].r > r) r = h->approx[b].r;
  return r;
}

static int64_t block_work(const or_hmatrix *h, int64_t b) {
  if (b < h->nd) {
    const or_block *B = &h->dense[b];
    return (B->re - B->rs + 1) * (B->ce - B->cs + 1);
  }
  const or_block *B = &h->approx[b - h->nd];
  return B->r * ((B->re - B->rs + 1) + (B->ce - B->cs + 1)) + 1;
}

int or_mul_cpu(const or_hmatrix *h, const double *x, double *y, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  int64_t tl = h->tlen;
  double *xo = (double *)malloc((size_t)h->slen * sizeof(double));
  for (int64_t j = 0; j < h->slen; j++) xo[j] = x[h->smap[j] - 1]; /* :10 */
  int64_t nb = h->nd + h->na, mr = max_rank(h);
  double *res = (double *)calloc((size_t)tl, sizeof(double)); /* :7 */
  if (nthreads == 1) {
    double *tmp = (double *)malloc((size_t)mr * sizeof(double));
    for (int64_t b = 0; b < nb; b++) mul_block(h, b, xo, res, tmp);
    free(tmp);
  } else {
    int64_t total = 0;
    for (int64_t b = 0; b < nb; b++) total += block_work(h, b);
    mul_ctx *cs = (mul_ctx *)calloc((size_t)nthreads, sizeof(mul_ctx));
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    int64_t b = 0, acc = 0;
    for (int t = 0; t < nthreads; t++) {
      cs[t].h = h;
      cs[t].xo = xo;
      cs[t].acc = (double *)calloc((size_t)tl, sizeof(double));
      cs[t].tmp = (double *)malloc((size_t)mr * sizeof(double));
      cs[t].b0 = b;
      int64_t goal = (total * (t + 1)) / nthreads;
      while (b < nb && (acc < goal || t == nthreads - 1)) acc += block_work(h, b++);
      cs[t].b1 = b;
    }
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, mul_worker, &cs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    for (int t = 0; t < nthreads; t++) {
      for (int64_t i = 0; i < tl; i++) res[i] += cs[t].acc[i];
      free(cs[t].acc);
      free(cs[t].tmp);
    }
    free(cs);
    free(th);
  }
  for (int64_t i = 0; i < tl; i++) y[h->tmap[i] - 1] = res[i]; /* :30 */
  free(res);
  free(xo);
  return 0;
}

double or_mul_cpu_timed(const or_hmatrix *h, const double *x, double *y, int nthreads,
                        int reps) {
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  for (int r = 0; r < reps; r++) or_mul_cpu(h, x, y, nthreads);
  clock_gettime(CLOCK_MONOTONIC, &b);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}

/* Flattened product (src/mult.jl:41-146), restated as sequential loops. */
int or_mul_flat(const or_hmatrix *h, const double *x, double *y, double *Vx) {
  int64_t nD, nA, R, dl, ul, vl, m, n;
  or_hmatrix_sizes(h, &m, &n, &nD, &nA, &R, &dl, &ul, &vl);
  int64_t *di = (int64_t *)malloc((size_t)(5 * nD + 1) * sizeof(int64_t));
  int64_t *ui = (int64_t *)malloc((size_t)(5 * nA + 1) * sizeof(int64_t));
  int64_t *vi = (int64_t *)malloc((size_t)(3 * R + 1) * sizeof(int64_t));
  double *dd = (double *)malloc((size_t)(dl + 1) * sizeof(double));
  double *ud = (double *)malloc((size_t)(ul + 1) * sizeof(double));
  double *vd = (double *)malloc((size_t)(vl + 1) * sizeof(double));
  or_hmatrix_export(h, NULL, NULL, di, ui, vi, dd, ud, vd);
  const int64_t *sm = h->smap, *tm = h->tmap;
  for (int64_t k = 0; k < R; k++) { /* V_mult_vec_kernel! (:41-78) */
    int64_t cs = vi[3 * k], ce = vi[3 * k + 1], off = vi[3 * k + 2];
    double s = 0.0;
    for (int64_t j = cs; j <= ce; j++) s += vd[off + (j - cs)] * x[sm[j - 1] - 1];
    Vx[k] = s;
  }
  for (int64_t I = 1; I <= h->tlen; I++) { /* DU_mult_vec_kernel! (:80-146) */
    double s = 0.0;
    for (int64_t b = 0; b < nD; b++) {
      int64_t rs = di[5 * b], re = di[5 * b + 1], cs = di[5 * b + 2], ce = di[5 * b + 3],
              off = di[5 * b + 4];
      if (I < rs || I > re) continue;
      const double *d = dd + off + (I - rs) * (ce - cs + 1);
      for (int64_t j = cs; j <= ce; j++) s += d[j - cs] * x[sm[j - 1] - 1];
    }
    for (int64_t b = 0; b < nA; b++) {
      int64_t rs = ui[5 * b], re = ui[5 * b + 1], vs = ui[5 * b + 2], ve = ui[5 * b + 3],
              off = ui[5 * b + 4];
      if (I < rs || I > re) continue;
      const double *u = ud + off + (I - rs) * (ve - vs + 1);
      for (int64_t j = vs; j <= ve; j++) s += u[j - vs] * Vx[j - 1];
    }
    y[tm[I - 1] - 1] = s;
  }
  free(di);
  free(ui);
  free(vi);
  free(dd);
  free(ud);
  free(vd);
  return 0;
}
