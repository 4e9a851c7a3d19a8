// Host-side cluster tree and block tree of libhmgpu.
//
// The arithmetic is the reference's, operation for operation, so that the
// permutation and the block partition come out bit-identical:
//   * ClusterTree / build_tree_node        src/tree.jl:45-116
//   * dims expansion, update_tree_indices!  src/tree.jl:59-64, :123-137
//   * build_block_tree!                     src/block.jl:58-90
//   * merge_dense_matrices!                 src/block.jl:98-112
//   * traverse                              src/block.jl:127-155
// This file must be compiled without floating-point contraction
// (-ffp-contract=off): Julia never fuses a multiply and an add.
#include <cmath>
#include <cstring>
#include <mutex>

#include "hm_internal.h"

namespace hm {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

// Julia's Base.isless ordering as used by argmax/sortperm: NaN above all numbers.
static inline bool isless_gt(double a, double b) {
  if (std::isnan(a)) return !std::isnan(b);
  if (std::isnan(b)) return false;
  return a > b;
}

// LinearAlgebra.generic_norm2 of a 3-vector (the path `norm` takes for
// arrays shorter than 32): plain sum of squares left to right, or the
// maxabs-scaled sum when squaring would overflow or underflow.
static double norm3(double a, double b, double c) {
  if (std::isnan(a) || std::isnan(b) || std::isnan(c)) return NAN;
  double mx = std::fabs(a);
  if (std::fabs(b) > mx) mx = std::fabs(b);
  if (std::fabs(c) > mx) mx = std::fabs(c);
  if (mx == 0.0 || std::isinf(mx)) return mx;
  if (std::isfinite(3.0 * mx * mx) && mx * mx != 0.0) {
    double s = a * a;
    s = s + b * b;
    s = s + c * c;
    return std::sqrt(s);
  }
  double qa = std::fabs(a) / mx, qb = std::fabs(b) / mx, qc = std::fabs(c) / mx;
  double s = qa * qa;
  s = s + qb * qb;
  s = s + qc * qc;
  return mx * std::sqrt(s);
}

// ---------------------------------------------------------------------------
// cluster tree
// ---------------------------------------------------------------------------
int build_tree(const double *coords, int64_t npts, int64_t leaf, int64_t dims, Tree &t) {
  if (dims <= 0) return fail(HMGPU_ERR_INVALID, "Parameter `dims` must be a positive integer.");
  if (npts <= 0) return fail(HMGPU_ERR_INVALID, "cluster tree needs at least one point");
  if (leaf <= 0) return fail(HMGPU_ERR_INVALID, "max_points_per_leaf must be positive");
  if (!coords) return fail(HMGPU_ERR_INVALID, "coords is NULL");
  t.npts = npts;
  t.dims = dims;
  t.nodes.clear();
  std::vector<int64_t> perm(npts), tmp(npts);
  for (int64_t i = 0; i < npts; i++) perm[i] = i + 1;

  // Explicit pre-order work stack: (node slot, start, end); a node's children
  // are created when it is processed, left popped first.
  struct Work {
    int64_t slot, start, end;
  };
  std::vector<Work> stack;
  t.nodes.push_back(Node{});
  stack.push_back({0, 1, npts + 1});
  while (!stack.empty()) {
    Work w = stack.back();
    stack.pop_back();
    const int64_t cnt = w.end - w.start;
    int64_t *view = perm.data() + (w.start - 1);
    double lo[3], hi[3], sum[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < 3; a++) lo[a] = hi[a] = coords[3 * (view[0] - 1) + a];
    for (int64_t p = 0; p < cnt; p++) {  // minimum/maximum/sum over dims=2, column order
      const double *q = coords + 3 * (view[p] - 1);
      for (int a = 0; a < 3; a++) {
        double v = q[a];
        if (std::isnan(v) || std::isnan(lo[a])) lo[a] = NAN;
        else if (v < lo[a]) lo[a] = v;
        if (std::isnan(v) || std::isnan(hi[a])) hi[a] = NAN;
        else if (v > hi[a]) hi[a] = v;
        sum[a] = sum[a] + v;
      }
    }
    int axis = 0;
    double len[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    for (int a = 1; a < 3; a++)
      if (isless_gt(len[a], len[axis])) axis = a;
    Node nd;
    for (int a = 0; a < 3; a++) nd.center[a] = sum[a] / static_cast<double>(cnt);
    double r1 = norm3(nd.center[0] - hi[0], nd.center[1] - hi[1], nd.center[2] - hi[2]);
    double r2 = norm3(nd.center[0] - lo[0], nd.center[1] - lo[1], nd.center[2] - lo[2]);
    nd.radius = (std::isnan(r1) || std::isnan(r2)) ? NAN : (r2 > r1 ? r2 : r1);
    nd.start = w.start;
    nd.end = w.end;
    nd.left = nd.right = -1;
    nd.leaf = cnt <= leaf;
    if (!nd.leaf) {
      const double c = nd.center[axis];
      int64_t nl = 0;
      for (int64_t p = 0; p < cnt; p++)
        if (coords[3 * (view[p] - 1) + axis] < c) tmp[nl++] = view[p];
      int64_t k = nl;
      for (int64_t p = 0; p < cnt; p++)
        if (!(coords[3 * (view[p] - 1) + axis] < c)) tmp[k++] = view[p];
      if (nl == 0 || nl == cnt)
        return fail(HMGPU_ERR_TREE,
                    "cluster of " + std::to_string(cnt) +
                        " points cannot be bisected (coincident points exceed the leaf size)");
      std::memcpy(view, tmp.data(), sizeof(int64_t) * cnt);
      nd.left = static_cast<int64_t>(t.nodes.size());
      nd.right = nd.left + 1;
      t.nodes.push_back(Node{});
      t.nodes.push_back(Node{});
      // Numbering: children get consecutive slots when the parent is processed.
      // Renumbered into pre-order below.
      stack.push_back({nd.right, w.start + nl, w.end});
      stack.push_back({nd.left, w.start, w.start + nl});
    }
    t.nodes[w.slot] = nd;
  }
  finish_tree(t, perm, dims);
  return HMGPU_OK;
}

// Nodes (children created in consecutive slots when their parent is processed,
// root in slot 0) renumbered into pre-order, and the dims expansion of the
// ranges and the index map (src/tree.jl:59-64, :123-137). perm: the final
// point order, 1-based.
void finish_tree(Tree &t, std::vector<int64_t> &perm, int64_t dims) {
  const int64_t npts = static_cast<int64_t>(perm.size());
  // Renumber into pre-order (parent, left subtree, right subtree).
  {
    std::vector<int64_t> newid(t.nodes.size(), -1), order;
    order.reserve(t.nodes.size());
    std::vector<int64_t> st = {0};
    while (!st.empty()) {
      int64_t k = st.back();
      st.pop_back();
      newid[k] = static_cast<int64_t>(order.size());
      order.push_back(k);
      if (t.nodes[k].right >= 0) st.push_back(t.nodes[k].right);
      if (t.nodes[k].left >= 0) st.push_back(t.nodes[k].left);
    }
    std::vector<Node> nn(order.size());
    for (size_t i = 0; i < order.size(); i++) {
      Node n = t.nodes[order[i]];
      if (n.left >= 0) n.left = newid[n.left];
      if (n.right >= 0) n.right = newid[n.right];
      nn[i] = n;
    }
    t.nodes.swap(nn);
  }
  if (dims > 1) {
    t.index_map.resize(npts * dims);
    for (int64_t p = 0; p < npts; p++)
      for (int64_t i = 1; i <= dims; i++) t.index_map[p * dims + (i - 1)] = dims * perm[p] - (dims - i);
    for (Node &n : t.nodes) {
      int64_t s = n.start;
      n.start = dims * (s - 1) + 1;
      n.end = dims * (n.end - s) + n.start;
    }
  } else {
    t.index_map.swap(perm);
  }
}

// ---------------------------------------------------------------------------
// block tree
// ---------------------------------------------------------------------------
void build_blocks(const Tree &X, const Tree &Y, double eta, bool merge, Blocks &b) {
  b.nodes.clear();
  b.dense.clear();
  b.approx.clear();
  b.nodes.push_back(BNode{0, 0, -1, -1, false, false});
  std::vector<int32_t> stack = {0};
  while (!stack.empty()) {  // pre-order; children created when the parent is visited
    int32_t k = stack.back();
    stack.pop_back();
    const Node &x = X.nodes[b.nodes[k].x];
    const Node &y = Y.nodes[b.nodes[k].y];
    double dist = norm3(x.center[0] - y.center[0], x.center[1] - y.center[1],
                        x.center[2] - y.center[2]);
    if (dist > eta * (x.radius + y.radius)) {
      b.nodes[k].adm = true;
      continue;
    }
    if (x.leaf && y.leaf) {
      b.nodes[k].dense = true;
      continue;
    }
    bool split_y = (!y.leaf && y.radius > x.radius) || x.leaf;
    int32_t xi = b.nodes[k].x, yi = b.nodes[k].y;
    int32_t l = static_cast<int32_t>(b.nodes.size());
    if (split_y) {
      b.nodes.push_back(BNode{xi, static_cast<int32_t>(y.left), -1, -1, false, false});
      b.nodes.push_back(BNode{xi, static_cast<int32_t>(y.right), -1, -1, false, false});
    } else {
      b.nodes.push_back(BNode{static_cast<int32_t>(x.left), yi, -1, -1, false, false});
      b.nodes.push_back(BNode{static_cast<int32_t>(x.right), yi, -1, -1, false, false});
    }
    b.nodes[k].left = l;
    b.nodes[k].right = l + 1;
    stack.push_back(l + 1);
    stack.push_back(l);
  }
  if (merge) {
    // Children are always created after their parent, so a reverse sweep is a
    // valid post-order for the merge.
    for (int64_t k = static_cast<int64_t>(b.nodes.size()) - 1; k >= 0; k--) {
      BNode &n = b.nodes[k];
      if (n.left >= 0 && n.right >= 0) n.dense = b.nodes[n.left].dense && b.nodes[n.right].dense;
    }
  }
  std::vector<int32_t> st = {0};
  while (!st.empty()) {
    int32_t k = st.back();
    st.pop_back();
    const BNode &n = b.nodes[k];
    if (n.adm) {
      b.approx.push_back(n.x);
      b.approx.push_back(n.y);
    } else if (n.dense) {
      b.dense.push_back(n.x);
      b.dense.push_back(n.y);
    }
    if (!n.dense && !n.adm) {
      if (n.right >= 0) st.push_back(n.right);
      if (n.left >= 0) st.push_back(n.left);
    }
  }
}

}  // namespace hm

// ---------------------------------------------------------------------------
// C ABI: trees and blocks
// ---------------------------------------------------------------------------
extern "C" {

const char *hmgpu_last_error(void) { return hm::g_err.c_str(); }
int hmgpu_abi_version(void) { return HMGPU_ABI_VERSION; }

int hmgpu_tree_build(const double *coords, int64_t npts, int64_t leaf, int64_t dims,
                     hmgpu_tree **out) {
  if (!out) return hm::fail(HMGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  auto *h = new (std::nothrow) hmgpu_tree;
  if (!h) return hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  int rc;
  try {
    rc = hm::build_tree(coords, npts, leaf, dims, h->t);
  } catch (const std::bad_alloc &) {
    rc = hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  }
  if (rc != HMGPU_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return HMGPU_OK;
}

int hmgpu_tree_info(const hmgpu_tree *h, int64_t *nnodes, int64_t *index_len, int64_t *depth,
                    int64_t *max_points, int64_t *min_points) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "tree is NULL");
  const hm::Tree &t = h->t;
  // info(::ClusterTree) (src/tree.jl:153-187): depth counted from 1 at the root
  int64_t dmax = 0, pmax = 0, pmin = INT64_MAX;
  std::vector<std::pair<int64_t, int64_t>> st = {{0, 1}};
  while (!st.empty()) {
    auto [k, d] = st.back();
    st.pop_back();
    const hm::Node &n = t.nodes[k];
    if (d > dmax) dmax = d;
    if (n.leaf) {
      int64_t c = n.end - n.start;
      if (c > pmax) pmax = c;
      if (c < pmin) pmin = c;
    }
    if (n.left >= 0) st.push_back({n.left, d + 1});
    if (n.right >= 0) st.push_back({n.right, d + 1});
  }
  if (nnodes) *nnodes = static_cast<int64_t>(t.nodes.size());
  if (index_len) *index_len = static_cast<int64_t>(t.index_map.size());
  if (depth) *depth = dmax;
  if (max_points) *max_points = pmax;
  if (min_points) *min_points = pmin == INT64_MAX ? 0 : pmin;
  return HMGPU_OK;
}

int hmgpu_tree_export(const hmgpu_tree *h, int64_t *index_map, int64_t *start, int64_t *end,
                      int8_t *is_leaf, int64_t *left, int64_t *right, double *center,
                      double *radius) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "tree is NULL");
  const hm::Tree &t = h->t;
  if (index_map) std::memcpy(index_map, t.index_map.data(), sizeof(int64_t) * t.index_map.size());
  for (size_t k = 0; k < t.nodes.size(); k++) {
    const hm::Node &n = t.nodes[k];
    if (start) start[k] = n.start;
    if (end) end[k] = n.end;
    if (is_leaf) is_leaf[k] = n.leaf ? 1 : 0;
    if (left) left[k] = n.left;
    if (right) right[k] = n.right;
    if (center) std::memcpy(center + 3 * k, n.center, sizeof n.center);
    if (radius) radius[k] = n.radius;
  }
  return HMGPU_OK;
}

int hmgpu_tree_free(hmgpu_tree *h) {
  delete h;
  return HMGPU_OK;
}

int hmgpu_blocks_build(const hmgpu_tree *X, const hmgpu_tree *Y, double eta, int merge,
                       hmgpu_blocks **out) {
  if (!X || !Y || !out) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  auto *h = new (std::nothrow) hmgpu_blocks;
  if (!h) return hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  try {
    hm::build_blocks(X->t, Y->t, eta, merge != 0, h->b);
  } catch (const std::bad_alloc &) {
    delete h;
    return hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  }
  *out = h;
  return HMGPU_OK;
}

int hmgpu_blocks_counts(const hmgpu_blocks *h, int64_t *nd, int64_t *na, int64_t *nn) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "blocks is NULL");
  if (nd) *nd = static_cast<int64_t>(h->b.dense.size() / 2);
  if (na) *na = static_cast<int64_t>(h->b.approx.size() / 2);
  if (nn) *nn = static_cast<int64_t>(h->b.nodes.size());
  return HMGPU_OK;
}

int hmgpu_blocks_export(const hmgpu_blocks *h, int64_t *dense_pairs, int64_t *approx_pairs) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "blocks is NULL");
  if (dense_pairs)
    for (size_t i = 0; i < h->b.dense.size(); i++) dense_pairs[i] = h->b.dense[i];
  if (approx_pairs)
    for (size_t i = 0; i < h->b.approx.size(); i++) approx_pairs[i] = h->b.approx[i];
  return HMGPU_OK;
}

int hmgpu_blocks_export_nodes(const hmgpu_blocks *h, int64_t *target, int64_t *source,
                              int8_t *adm, int8_t *dense, int64_t *left, int64_t *right) {
  if (!h) return hm::fail(HMGPU_ERR_INVALID, "blocks is NULL");
  for (size_t k = 0; k < h->b.nodes.size(); k++) {
    const hm::BNode &n = h->b.nodes[k];
    if (target) target[k] = n.x;
    if (source) source[k] = n.y;
    if (adm) adm[k] = n.adm;
    if (dense) dense[k] = n.dense;
    if (left) left[k] = n.left;
    if (right) right[k] = n.right;
  }
  return HMGPU_OK;
}

int hmgpu_blocks_free(hmgpu_blocks *h) {
  delete h;
  return HMGPU_OK;
}

}  // extern "C"
