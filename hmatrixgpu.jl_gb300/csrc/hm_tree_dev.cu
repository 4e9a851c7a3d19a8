// Cluster tree and block tree built on the GPU, bit-identical to the host
// builds (hm_tree.cpp).
//
// The reference builds the tree recursively on the host (src/tree.jl:70-116,
// build_tree_node): bounding box and centroid of the node's points in their
// current order, split along the longest box edge at the centroid with a stable
// partition (`sortperm` of the predicate `x[axis] < center[axis]`, left part
// first), leaf iff the node holds at most max_points_per_leaf points.
//
// Here the tree grows level by level, one CTA per node of the level:
//   pass 1  bounding box (any order: only min/max, as ordered integer keys)
//           and the centroid sums; a sum is one floating-point chain in the
//           points' current order, exactly as `sum(x; dims=2)` over the node's
//           columns in src/tree.jl:83, evaluated by one warp per axis 32
//           values at a time (seq_sum32: an exact integer form of the chain
//           while it stays in one binade, the plain chain otherwise) while the
//           other warps stage the next chunk of coordinates in shared memory;
//   pass 2  count of the points left of the centroid;
//   pass 3  stable scatter of the point indices and their coordinates into the
//           other buffer (left part in order, then the right part in order).
// The coordinates travel with the indices (structure of arrays, ping-pong
// buffers), so every pass reads contiguous memory. Leaves copy their index
// range into the final permutation. Nodes get slots in the order their parents
// finish; the shared host step renumbers them into pre-order, so the slot order
// does not matter.
//
// All floating-point arithmetic goes through the _rn intrinsics (no
// contraction); the norm is LinearAlgebra.generic_norm2 of a 3-vector as in the
// host build. Comparisons of coordinates run on their bits as integers.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <memory>
#include <vector>

#include "hm_api.h"
#include "hm_internal.h"

namespace hm {
namespace {

constexpr int kTreeThreads = 512;
constexpr int kWarps = kTreeThreads / 32;
constexpr int kChunk = 512;   // coordinates per axis staged per step of pass 1
constexpr int kItems = 4;     // points per thread per step of pass 3

struct DNode {
  int32_t start, cnt;   // 0-based first point and number of points
  int32_t left, right;  // child slots, -1 for none
  double center[3];
  double radius;
  int32_t leaf, pad;
};

struct Level {
  const double *cx, *cy, *cz;  // coordinates of the current order
  const int32_t *cperm;        // current order (0-based point indices)
  double *nx, *ny, *nz;        // next order, written by splitting nodes
  int32_t *nperm;
  int32_t *final_perm;         // order of the finished tree
  DNode *nodes;
  int32_t first, next_base, cap;
  int32_t leaf;
  int32_t *ctl;  // [0] next-level slots taken, [1] error code, [2] size of the failed node
};

// Base.isless ordering used by argmax: NaN above all numbers.
__device__ __forceinline__ bool isless_gt(double a, double b) {
  if (isnan(a)) return !isnan(b);
  if (isnan(b)) return false;
  return a > b;
}

// Bits of a double as an int64 that orders like the number (NaN excluded; -0
// sorts just below +0, which no result here depends on).
__device__ __forceinline__ long long ord_key(double v) {
  const long long b = __double_as_longlong(v);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}
__device__ __forceinline__ double from_key(long long k) {
  return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffll));
}
__device__ __forceinline__ bool is_nan_bits(long long b) {
  return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}
// a < b for non-NaN doubles as integers (+0 and -0 equal)
__device__ __forceinline__ long long less_key(double v) {
  long long b = __double_as_longlong(v);
  if (b == static_cast<long long>(0x8000000000000000ull)) b = 0;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

// The sequential sum s + v_0 + v_1 + ... + v_{cnt-1} (each addition rounded to
// nearest even, left to right) of the values lane j holds, returned in every
// lane; bit for bit the chain of __dadd_rn. Fast path: with s = S 2^e (S the
// 53-bit significand), each step rounds S + v_j / 2^e to an integer as long as
// the sum stays inside [2^52, 2^53): then the rounded increments r_j (integer
// parts of v_j / 2^e, rounded to nearest) are independent of the order and
// the partial sums are S plus a prefix sum of the r_j, computed by a warp
// scan. The fast path is taken when every partial sum stays strictly inside
// that range with a margin and no v_j / 2^e has a fractional part of exactly
// one half (where the rounding would depend on the parity of the partial
// sum); otherwise, and for zero, subnormal, infinite or NaN operands, the
// values are added one by one.
__device__ double seq_sum32(double s, double v, int cnt) {
  const int lane = threadIdx.x & 31;
  const long long sb = __double_as_longlong(s);
  const int E = static_cast<int>((sb >> 52) & 0x7ff);
  if (E != 0 && E != 0x7ff) {
    const bool neg = sb < 0;
    long long vb = __double_as_longlong(v);
    if (neg) vb ^= static_cast<long long>(0x8000000000000000ull);  // the mirror image: RNE is symmetric
    const int vexp = static_cast<int>((vb >> 52) & 0x7ff);
    bool ok = vexp != 0x7ff, tie = false;
    long long m = vb & 0x000fffffffffffffll;
    int ve = vexp;
    if (vexp != 0)
      m |= 0x0010000000000000ll;
    else
      ve = 1;  // subnormal: m 2^(1 - 1075)
    const int d = ve - E;  // v / 2^e = m 2^d
    long long r = 0;
    if (m != 0) {
      if (d >= 0) {
        if (d > 0)
          ok = false;  // |v| >= 2^53 ulp: the sum leaves the binade (and no sum can overflow)
        else
          r = m;
      } else if (-d < 62) {
        const int sh = -d;
        const long long q = m >> sh, rem = m & ((1ll << sh) - 1), half = 1ll << (sh - 1);
        r = q + (rem > half ? 1 : 0);
        tie = rem == half;
      }  // else |v| < 2^-9 ulp: rounds to nothing, never a tie
    }
    if (vb < 0) r = -r;
    if (lane >= cnt) {
      r = 0;
      ok = true;
      tie = false;
    }
    long long pre = r;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const long long S = (sb & 0x000fffffffffffffll) | 0x0010000000000000ll;
    const long long P = S + pre;
    const bool inside = P >= 0x0010000000000001ll && P <= 0x001ffffffffffffell;
    if (__all_sync(0xffffffffu, ok && !tie && inside)) {
      const long long Pend = __shfl_sync(0xffffffffu, P, 31);
      long long nb = (static_cast<long long>(E) << 52) | (Pend - 0x0010000000000000ll);
      if (neg) nb |= static_cast<long long>(0x8000000000000000ull);
      return __longlong_as_double(nb);
    }
  }
  double acc = s;
  for (int i = 0; i < cnt; i++) acc = __dadd_rn(acc, __shfl_sync(0xffffffffu, v, i));
  return acc;
}

// LinearAlgebra.generic_norm2 of a 3-vector, as the host build computes it.
__device__ double norm3_dev(double a, double b, double c) {
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  if (isnan(a) || isnan(b) || isnan(c)) return qnan;
  double mx = fabs(a);
  if (fabs(b) > mx) mx = fabs(b);
  if (fabs(c) > mx) mx = fabs(c);
  if (mx == 0.0 || isinf(mx)) return mx;
  const double m2 = __dmul_rn(mx, mx);
  if (isfinite(__dmul_rn(__dmul_rn(3.0, mx), mx)) && m2 != 0.0) {
    double s = __dmul_rn(a, a);
    s = __dadd_rn(s, __dmul_rn(b, b));
    s = __dadd_rn(s, __dmul_rn(c, c));
    return __dsqrt_rn(s);
  }
  const double qa = __ddiv_rn(fabs(a), mx), qb = __ddiv_rn(fabs(b), mx), qc = __ddiv_rn(fabs(c), mx);
  double s = __dmul_rn(qa, qa);
  s = __dadd_rn(s, __dmul_rn(qb, qb));
  s = __dadd_rn(s, __dmul_rn(qc, qc));
  return __dmul_rn(mx, __dsqrt_rn(s));
}

__global__ void tree_init_kernel(const double *__restrict__ coords, int32_t npts, double *x, double *y,
                                 double *z, int32_t *perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = coords[3 * i];
    y[i] = coords[3 * i + 1];
    z[i] = coords[3 * i + 2];
    perm[i] = static_cast<int32_t>(i);
  }
}

// Exclusive block scan of one int per thread; returns the prefix and sets *total.
__device__ int block_exclusive_scan(int v, int *warp_tot, int *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    int t = lane < kWarps ? warp_tot[lane] : 0;
    int s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    if (lane < kWarps) warp_tot[lane] = s - t;  // exclusive warp offsets
    if (lane == kWarps - 1) warp_tot[kWarps] = s;
  }
  __syncthreads();
  const int r = warp_tot[w] + inc - v;
  *total = warp_tot[kWarps];
  __syncthreads();  // warp_tot is reused by the next call
  return r;
}

__global__ void __launch_bounds__(kTreeThreads) tree_level_kernel(Level L) {
  __shared__ double stage[2][3][kChunk];
  __shared__ long long red_lo[kWarps][3], red_hi[kWarps][3];
  __shared__ int red_nan[kWarps];
  __shared__ double sums[3];
  __shared__ double s_center;
  __shared__ int s_axis, s_split;
  __shared__ int warp_tot[kWarps + 1];

  const int slot = L.first + blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int32_t start = L.nodes[slot].start, cnt = L.nodes[slot].cnt;
  const double *src[3] = {L.cx + start, L.cy + start, L.cz + start};

  // ---- pass 1: bounding box and the three sequential sums -----------------
  // warps 0..2 sum axis 0..2 (seq_sum32, 32 values per step); the other
  // warps stage the next chunk and keep the box as ordered integer keys
  constexpr int kSum = 3;
  long long lo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, hi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  int nan_seen = 0;
  double acc = 0.0;  // warp a < 3: the sum of axis a
  const int nch = (cnt + kChunk - 1) / kChunk;
  for (int k = 0; k <= nch; k++) {
    if (warp >= kSum) {
      if (k < nch) {
        const int base = k * kChunk, len = min(kChunk, cnt - base);
        double(*buf)[kChunk] = stage[k & 1];
        for (int i = tid - 32 * kSum; i < len; i += kTreeThreads - 32 * kSum) {
#pragma unroll
          for (int a = 0; a < 3; a++) {
            const double v = src[a][base + i];
            buf[a][i] = v;
            const long long b = __double_as_longlong(v);
            if (is_nan_bits(b)) {
              nan_seen |= 1 << a;
            } else {
              const long long kk = ord_key(v);
              lo[a] = kk < lo[a] ? kk : lo[a];
              hi[a] = kk > hi[a] ? kk : hi[a];
            }
          }
        }
      }
    } else if (k > 0) {
      const int base = (k - 1) * kChunk, len = min(kChunk, cnt - base);
      const double *row = stage[(k - 1) & 1][warp];
      for (int i0 = 0; i0 < len; i0 += 32) {
        const int n = min(32, len - i0);
        acc = seq_sum32(acc, lane < n ? row[i0 + lane] : 0.0, n);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 3; a++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ol = __shfl_xor_sync(0xffffffffu, lo[a], o), oh = __shfl_xor_sync(0xffffffffu, hi[a], o);
      lo[a] = ol < lo[a] ? ol : lo[a];
      hi[a] = oh > hi[a] ? oh : hi[a];
    }
  }
  nan_seen = __reduce_or_sync(0xffffffffu, nan_seen);
  if (lane == 0) {
    for (int a = 0; a < 3; a++) {
      red_lo[warp][a] = lo[a];
      red_hi[warp][a] = hi[a];
    }
    red_nan[warp] = nan_seen;
  }
  if (warp < kSum && lane == 0) sums[warp] = acc;
  __syncthreads();
  if (tid == 0) {
    double blo[3], bhi[3], len[3];
    DNode nd;
    int nans = 0;
    for (int w = 0; w < kWarps; w++) nans |= red_nan[w];
    for (int a = 0; a < 3; a++) {
      long long kl = LLONG_MAX, kh = LLONG_MIN;
      for (int w = 0; w < kWarps; w++) {
        kl = red_lo[w][a] < kl ? red_lo[w][a] : kl;
        kh = red_hi[w][a] > kh ? red_hi[w][a] : kh;
      }
      const double qnan = __longlong_as_double(0x7ff8000000000000ll);
      blo[a] = (nans >> a) & 1 ? qnan : from_key(kl);  // minimum/maximum propagate NaN
      bhi[a] = (nans >> a) & 1 ? qnan : from_key(kh);
      len[a] = __dsub_rn(bhi[a], blo[a]);
      nd.center[a] = __ddiv_rn(sums[a], static_cast<double>(cnt));
    }
    int axis = 0;
    for (int a = 1; a < 3; a++)
      if (isless_gt(len[a], len[axis])) axis = a;
    const double r1 = norm3_dev(__dsub_rn(nd.center[0], bhi[0]), __dsub_rn(nd.center[1], bhi[1]),
                                __dsub_rn(nd.center[2], bhi[2]));
    const double r2 = norm3_dev(__dsub_rn(nd.center[0], blo[0]), __dsub_rn(nd.center[1], blo[1]),
                                __dsub_rn(nd.center[2], blo[2]));
    nd.radius = (isnan(r1) || isnan(r2)) ? __longlong_as_double(0x7ff8000000000000ll) : (r2 > r1 ? r2 : r1);
    nd.start = start;
    nd.cnt = cnt;
    nd.left = nd.right = -1;
    nd.leaf = cnt <= L.leaf;
    nd.pad = 0;
    L.nodes[slot] = nd;
    s_center = nd.center[axis];
    s_axis = axis;
    s_split = !nd.leaf;
  }
  __syncthreads();

  if (!s_split) {  // a leaf: its order is final
    for (int i = tid; i < cnt; i += kTreeThreads) L.final_perm[start + i] = L.cperm[start + i];
    return;
  }
  // v < c as integers: never true for a NaN on either side
  const bool c_nan = isnan(s_center);
  const long long ck = less_key(s_center);
  const double *key = s_axis == 0 ? src[0] : (s_axis == 1 ? src[1] : src[2]);
  auto left_of = [&](double v) {
    return !c_nan && !is_nan_bits(__double_as_longlong(v)) && less_key(v) < ck;
  };

  // ---- pass 2: size of the left part ---------------------------------------
  int nleft = 0;
  for (int i = tid; i < cnt; i += kTreeThreads) nleft += left_of(key[i]) ? 1 : 0;
  int nl = 0;
  block_exclusive_scan(nleft, warp_tot, &nl);
  if (nl == 0 || nl == cnt) {  // a coincident cluster: the host reports it
    if (tid == 0) {
      atomicCAS(L.ctl + 1, 0, HMGPU_ERR_TREE);
      atomicMax(L.ctl + 2, cnt);
    }
    return;
  }

  // ---- pass 3: stable scatter ------------------------------------------------
  double *dst[3] = {L.nx + start, L.ny + start, L.nz + start};
  const int32_t *pin = L.cperm + start;
  int32_t *pout = L.nperm + start;
  int left_before = 0;  // left points in earlier steps
  for (int base = 0; base < cnt; base += kTreeThreads * kItems) {
    const int i0 = base + tid * kItems;
    bool f[kItems];
    int nf = 0;
#pragma unroll
    for (int j = 0; j < kItems; j++) {
      f[j] = i0 + j < cnt && left_of(key[i0 + j]);
      nf += f[j] ? 1 : 0;
    }
    int step_total = 0;
    int lb = left_before + block_exclusive_scan(nf, warp_tot, &step_total);
#pragma unroll
    for (int j = 0; j < kItems; j++) {
      const int i = i0 + j;
      if (i >= cnt) break;
      const int d = f[j] ? lb : nl + (i - lb);
      lb += f[j] ? 1 : 0;
      pout[d] = pin[i];
#pragma unroll
      for (int a = 0; a < 3; a++) dst[a][d] = src[a][i];
    }
    left_before += step_total;
  }
  if (tid == 0) {
    const int s = atomicAdd(L.ctl, 2);
    const int l = L.next_base + s;
    if (l + 1 >= L.cap) {
      atomicCAS(L.ctl + 1, 0, 1);  // out of node slots
      return;
    }
    DNode ch{};
    ch.left = ch.right = -1;
    ch.start = start;
    ch.cnt = nl;
    L.nodes[l] = ch;
    ch.start = start + nl;
    ch.cnt = cnt - nl;
    L.nodes[l + 1] = ch;
    L.nodes[slot].left = l;
    L.nodes[slot].right = l + 1;
  }
}

// ---------------------------------------------------------------------------
// block tree (src/block.jl:58-155) level by level
// ---------------------------------------------------------------------------
// The host build numbers block-tree nodes in creation order of a pre-order walk:
// the children of the j-th internal node (counted in pre-order) get the numbers
// 1 + 2j and 2 + 2j. Here the tree grows breadth first; a bottom-up sweep then
// counts the internal nodes of every subtree (and applies the dense merge and
// the traverse counts), and a top-down sweep gives every node its pre-order
// internal rank, its number and its place in the traverse lists.

struct CNodes {  // a cluster tree, pre-order, structure of arrays
  const double *center;  // 3 per node
  const double *radius;
  const int32_t *left, *right;
  const int8_t *leaf;
};

struct BLevel {  // one breadth-first level of the block tree
  int32_t *x, *y;     // target and source cluster nodes
  int32_t *child;     // first child in the next level, -1 for none
  int8_t *kind;       // 0 split, 1 admissible, 2 dense leaf
  int8_t *dn;         // dense after the merge
  int8_t *reached;    // visited by traverse (no emitting ancestor)
  int32_t *nint;      // internal nodes in the subtree
  int32_t *na, *nd;   // traverse emissions in the subtree (approx, dense)
  int32_t *rank;      // pre-order rank among internal nodes (internal nodes only)
  int32_t *id;        // number in the host numbering
  int32_t *offa, *offd;
};

__global__ void bt_level_kernel(int32_t n, BLevel cur, BLevel nxt, CNodes X, CNodes Y, double eta,
                                int32_t *counter) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t xi = cur.x[i], yi = cur.y[i];
    const double *cx = X.center + 3 * static_cast<int64_t>(xi), *cy = Y.center + 3 * static_cast<int64_t>(yi);
    const double rx = X.radius[xi], ry = Y.radius[yi];
    const double dist = norm3_dev(__dsub_rn(cx[0], cy[0]), __dsub_rn(cx[1], cy[1]), __dsub_rn(cx[2], cy[2]));
    int8_t kind;
    int32_t child = -1;
    if (dist > __dmul_rn(eta, __dadd_rn(rx, ry))) {
      kind = 1;
    } else if (X.leaf[xi] && Y.leaf[yi]) {
      kind = 2;
    } else {
      kind = 0;
      const bool split_y = (!Y.leaf[yi] && ry > rx) || X.leaf[xi];
      child = atomicAdd(counter, 2);
      if (split_y) {
        nxt.x[child] = xi;
        nxt.y[child] = Y.left[yi];
        nxt.x[child + 1] = xi;
        nxt.y[child + 1] = Y.right[yi];
      } else {
        nxt.x[child] = X.left[xi];
        nxt.y[child] = yi;
        nxt.x[child + 1] = X.right[xi];
        nxt.y[child + 1] = yi;
      }
    }
    cur.kind[i] = kind;
    cur.child[i] = child;
  }
}

// Bottom-up: merge_dense_matrices! (src/block.jl:98-112) and the subtree counts.
__global__ void bt_up_kernel(int32_t n, BLevel cur, BLevel nxt, int merge) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int8_t kind = cur.kind[i];
    int8_t dn = kind == 2;
    int32_t nint = 0, na = kind == 1, nd = dn;
    if (kind == 0) {
      const int32_t l = cur.child[i];
      dn = merge && nxt.dn[l] && nxt.dn[l + 1];
      nint = 1 + nxt.nint[l] + nxt.nint[l + 1];
      na = dn ? 0 : nxt.na[l] + nxt.na[l + 1];
      nd = dn ? 1 : nxt.nd[l] + nxt.nd[l + 1];
    }
    cur.dn[i] = dn;
    cur.nint[i] = nint;
    cur.na[i] = na;
    cur.nd[i] = nd;
  }
}

// Top-down: numbers, node records in the host numbering, traverse lists
// (src/block.jl:127-155: admissible and dense nodes in pre-order, no descent
// below them).
__global__ void bt_down_kernel(int32_t n, BLevel cur, BLevel nxt, int32_t *ox, int32_t *oy, int32_t *ol,
                               int32_t *orr, int8_t *oadm, int8_t *odense, int32_t *approx,
                               int32_t *dense) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int8_t kind = cur.kind[i], dn = cur.dn[i], reached = cur.reached[i];
    const int32_t id = cur.id[i], x = cur.x[i], y = cur.y[i];
    ox[id] = x;
    oy[id] = y;
    oadm[id] = kind == 1;
    odense[id] = dn;
    ol[id] = orr[id] = -1;
    if (reached && kind == 1) {
      approx[2 * cur.offa[i]] = x;
      approx[2 * cur.offa[i] + 1] = y;
    }
    if (reached && dn) {
      dense[2 * cur.offd[i]] = x;
      dense[2 * cur.offd[i] + 1] = y;
    }
    if (kind == 0) {
      const int32_t l = cur.child[i], j = cur.rank[i];
      ol[id] = 1 + 2 * j;
      orr[id] = 2 + 2 * j;
      nxt.id[l] = 1 + 2 * j;
      nxt.id[l + 1] = 2 + 2 * j;
      nxt.rank[l] = j + 1;
      nxt.rank[l + 1] = j + 1 + nxt.nint[l];
      const int8_t go = reached && !dn;
      nxt.reached[l] = nxt.reached[l + 1] = go;
      nxt.offa[l] = cur.offa[i];
      nxt.offa[l + 1] = cur.offa[i] + nxt.na[l];
      nxt.offd[l] = cur.offd[i];
      nxt.offd[l + 1] = cur.offd[i] + nxt.nd[l];
    }
  }
}

struct Buf {
  void *p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
  template <typename V>
  V *as() const {
    return static_cast<V *>(p);
  }
};

}  // namespace

int build_tree_device(const double *coords, int64_t npts, int64_t leaf, int64_t dims, Tree &t) {
  if (dims <= 0) return fail(HMGPU_ERR_INVALID, "Parameter `dims` must be a positive integer.");
  if (npts <= 0) return fail(HMGPU_ERR_INVALID, "cluster tree needs at least one point");
  if (leaf <= 0) return fail(HMGPU_ERR_INVALID, "max_points_per_leaf must be positive");
  if (!coords) return fail(HMGPU_ERR_INVALID, "coords is NULL");
  if (npts >= (int64_t{1} << 30))
    return fail(HMGPU_ERR_INVALID, "the device tree build takes fewer than 2^30 points");
  const int32_t n = static_cast<int32_t>(npts);
  const int32_t cap = 2 * n - 1 + 2;  // a binary tree over n points has at most 2n - 1 nodes
  Buf dcoords, dxyz, dperm, dfinal, dnodes, dctl;
  cudaError_t e = cudaSuccess;
  if ((e = dcoords.alloc(sizeof(double) * 3 * npts)) != cudaSuccess ||
      (e = dxyz.alloc(sizeof(double) * 6 * npts)) != cudaSuccess ||
      (e = dperm.alloc(sizeof(int32_t) * 2 * npts)) != cudaSuccess ||
      (e = dfinal.alloc(sizeof(int32_t) * npts)) != cudaSuccess ||
      (e = dnodes.alloc(sizeof(DNode) * static_cast<size_t>(cap))) != cudaSuccess ||
      (e = dctl.alloc(sizeof(int32_t) * 4)) != cudaSuccess) {
    cudaGetLastError();
    return fail(HMGPU_ERR_NOMEM, "device memory for the tree build");
  }
  e = cudaMemcpy(dcoords.p, coords, sizeof(double) * 3 * npts, cudaMemcpyDefault);
  if (e != cudaSuccess) return cuda_fail(e, "copying coordinates");
  double *xyz = dxyz.as<double>();
  int32_t *perm = dperm.as<int32_t>();
  tree_init_kernel<<<std::min<int64_t>((npts + 255) / 256, 4096), 256>>>(dcoords.as<double>(), n, xyz,
                                                                          xyz + npts, xyz + 2 * npts, perm);
  DNode root{};
  root.start = 0;
  root.cnt = n;
  root.left = root.right = -1;
  cudaMemcpy(dnodes.p, &root, sizeof root, cudaMemcpyHostToDevice);
  cudaMemset(dctl.p, 0, sizeof(int32_t) * 4);

  int32_t first = 0, count = 1, cur = 0;
  const int32_t lf = static_cast<int32_t>(std::min<int64_t>(leaf, INT32_MAX));
  while (count > 0) {
    Level L;
    const double *c = xyz + static_cast<size_t>(cur) * 3 * npts;
    double *nb = xyz + static_cast<size_t>(cur ^ 1) * 3 * npts;
    L.cx = c;
    L.cy = c + npts;
    L.cz = c + 2 * npts;
    L.cperm = perm + static_cast<size_t>(cur) * npts;
    L.nx = nb;
    L.ny = nb + npts;
    L.nz = nb + 2 * npts;
    L.nperm = perm + static_cast<size_t>(cur ^ 1) * npts;
    L.final_perm = dfinal.as<int32_t>();
    L.nodes = dnodes.as<DNode>();
    L.first = first;
    L.next_base = first + count;
    L.cap = cap;
    L.leaf = lf;
    L.ctl = dctl.as<int32_t>();
    tree_level_kernel<<<count, kTreeThreads>>>(L);
    int32_t ctl[4];
    e = cudaMemcpy(ctl, dctl.p, sizeof ctl, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "tree level kernel");
    if (ctl[1] == HMGPU_ERR_TREE)
      return fail(HMGPU_ERR_TREE, "cluster of " + std::to_string(ctl[2]) +
                                      " points cannot be bisected (coincident points exceed the leaf size)");
    if (ctl[1] != 0) return fail(HMGPU_ERR_CUDA, "tree build ran out of node slots");
    first += count;
    count = ctl[0];
    cudaMemset(dctl.p, 0, sizeof(int32_t));
    cur ^= 1;
  }
  const int32_t nnodes = first;
  std::vector<DNode> hn(nnodes);
  std::vector<int32_t> hp(npts);
  e = cudaMemcpy(hn.data(), dnodes.p, sizeof(DNode) * nnodes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hp.data(), dfinal.p, sizeof(int32_t) * npts, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the tree back");
  t.npts = npts;
  t.dims = dims;
  t.index_map.clear();
  t.nodes.resize(nnodes);
  for (int32_t k = 0; k < nnodes; k++) {
    const DNode &d = hn[k];
    Node &q = t.nodes[k];
    q.start = int64_t{d.start} + 1;
    q.end = q.start + d.cnt;
    q.left = d.left;
    q.right = d.right;
    std::memcpy(q.center, d.center, sizeof q.center);
    q.radius = d.radius;
    q.leaf = d.leaf != 0;
  }
  std::vector<int64_t> p64(npts);
  for (int64_t i = 0; i < npts; i++) p64[i] = int64_t{hp[i]} + 1;
  finish_tree(t, p64, dims);
  return HMGPU_OK;
}


// ---------------------------------------------------------------------------
// block tree, host orchestration
// ---------------------------------------------------------------------------
namespace {

struct LevelStore {
  Buf mem;
  BLevel v{};
  int32_t n = 0;
  cudaError_t alloc(int32_t count) {
    n = count;
    const size_t c = static_cast<size_t>(std::max<int32_t>(count, 1));
    const size_t bytes = c * (11 * sizeof(int32_t) + 3 * sizeof(int8_t)) + 64;
    cudaError_t e = mem.alloc(bytes);
    if (e != cudaSuccess) return e;
    char *p = mem.as<char>();
    auto i32 = [&]() {
      int32_t *q = reinterpret_cast<int32_t *>(p);
      p += c * sizeof(int32_t);
      return q;
    };
    v.x = i32();
    v.y = i32();
    v.child = i32();
    v.nint = i32();
    v.na = i32();
    v.nd = i32();
    v.rank = i32();
    v.id = i32();
    v.offa = i32();
    v.offd = i32();
    i32();  // spare, keeps the byte arrays after 4-byte data
    v.kind = reinterpret_cast<int8_t *>(p);
    v.dn = v.kind + c;
    v.reached = v.dn + c;
    return cudaSuccess;
  }
};

struct TreeDev {
  Buf mem;
  CNodes c{};
  cudaError_t upload(const Tree &t) {
    const size_t nn = t.nodes.size();
    std::vector<double> ctr(3 * nn), rad(nn);
    std::vector<int32_t> lr(2 * nn);
    std::vector<int8_t> lf(nn);
    for (size_t k = 0; k < nn; k++) {
      const Node &q = t.nodes[k];
      std::memcpy(&ctr[3 * k], q.center, sizeof q.center);
      rad[k] = q.radius;
      lr[k] = static_cast<int32_t>(q.left);
      lr[nn + k] = static_cast<int32_t>(q.right);
      lf[k] = q.leaf ? 1 : 0;
    }
    cudaError_t e = mem.alloc(nn * (4 * sizeof(double) + 2 * sizeof(int32_t) + 1));
    if (e != cudaSuccess) return e;
    char *p = mem.as<char>();
    double *dc = reinterpret_cast<double *>(p), *dr = dc + 3 * nn;
    int32_t *dl = reinterpret_cast<int32_t *>(dr + nn);
    int8_t *df = reinterpret_cast<int8_t *>(dl + 2 * nn);
    if ((e = cudaMemcpy(dc, ctr.data(), 3 * nn * sizeof(double), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dr, rad.data(), nn * sizeof(double), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dl, lr.data(), 2 * nn * sizeof(int32_t), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(df, lf.data(), nn, cudaMemcpyHostToDevice)))
      return e;
    c.center = dc;
    c.radius = dr;
    c.left = dl;
    c.right = dl + nn;
    c.leaf = df;
    return cudaSuccess;
  }
};

int grid_for(int32_t n) { return static_cast<int>(std::min<int64_t>((int64_t{n} + 255) / 256, 152 * 16)); }

}  // namespace

int build_blocks_device(const Tree &X, const Tree &Y, double eta, bool merge, Blocks &b) {
  if (X.nodes.empty() || Y.nodes.empty()) return fail(HMGPU_ERR_INVALID, "empty cluster tree");
  if (X.nodes.size() >= (size_t{1} << 30) || Y.nodes.size() >= (size_t{1} << 30))
    return fail(HMGPU_ERR_INVALID, "cluster tree too large for the device block build");
  TreeDev dx, dy;
  cudaError_t e;
  if ((e = dx.upload(X)) != cudaSuccess || (e = dy.upload(Y)) != cudaSuccess)
    return cuda_fail(e, "uploading cluster trees");
  Buf dctr;
  if ((e = dctr.alloc(sizeof(int32_t))) != cudaSuccess) return cuda_fail(e, "block tree counter");
  int32_t *counter = dctr.as<int32_t>();

  std::vector<std::unique_ptr<LevelStore>> lv;
  lv.emplace_back(new LevelStore);
  if ((e = lv[0]->alloc(1)) != cudaSuccess) return cuda_fail(e, "block tree level");
  {
    const int32_t zero = 0;
    const int8_t one = 1;
    cudaMemcpy(lv[0]->v.x, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.y, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.rank, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.id, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.offa, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.offd, &zero, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(lv[0]->v.reached, &one, 1, cudaMemcpyHostToDevice);
  }
  int64_t total = 1;
  for (;;) {
    LevelStore &c = *lv.back();
    const int64_t cap = 2 * int64_t{c.n};
    if (total + cap >= (int64_t{1} << 31)) return fail(HMGPU_ERR_INVALID, "block tree too large for the device build");
    std::unique_ptr<LevelStore> nx(new LevelStore);
    if ((e = nx->alloc(static_cast<int32_t>(cap))) != cudaSuccess) return cuda_fail(e, "block tree level");
    cudaMemset(counter, 0, sizeof(int32_t));
    bt_level_kernel<<<grid_for(c.n), 256>>>(c.n, c.v, nx->v, dx.c, dy.c, eta, counter);
    int32_t got = 0;
    if ((e = cudaMemcpy(&got, counter, sizeof got, cudaMemcpyDeviceToHost)) != cudaSuccess)
      return cuda_fail(e, "block tree level kernel");
    if (got == 0) break;
    nx->n = got;
    total += got;
    lv.push_back(std::move(nx));
  }
  const int nl = static_cast<int>(lv.size());
  BLevel none{};
  for (int l = nl - 1; l >= 0; l--)
    bt_up_kernel<<<grid_for(lv[l]->n), 256>>>(lv[l]->n, lv[l]->v, l + 1 < nl ? lv[l + 1]->v : none,
                                               merge ? 1 : 0);
  int32_t na = 0, nd = 0;
  cudaMemcpy(&na, lv[0]->v.na, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&nd, lv[0]->v.nd, 4, cudaMemcpyDeviceToHost);
  Buf out;
  const size_t T = static_cast<size_t>(total);
  if ((e = out.alloc(T * (4 * sizeof(int32_t) + 2) + 2 * sizeof(int32_t) * (size_t(na) + nd) + 64)) != cudaSuccess)
    return cuda_fail(e, "block tree output");
  int32_t *ox = out.as<int32_t>(), *oy = ox + T, *ol = oy + T, *orr = ol + T;
  int32_t *oa = orr + T, *od = oa + 2 * size_t(na);
  int8_t *oadm = reinterpret_cast<int8_t *>(od + 2 * size_t(nd)), *oden = oadm + T;
  for (int l = 0; l < nl; l++)
    bt_down_kernel<<<grid_for(lv[l]->n), 256>>>(lv[l]->n, lv[l]->v, l + 1 < nl ? lv[l + 1]->v : none, ox, oy,
                                                 ol, orr, oadm, oden, oa, od);
  std::vector<int32_t> hx(T), hy(T), hl(T), hr(T);
  std::vector<int8_t> hadm(T), hden(T);
  b.approx.resize(2 * size_t(na));
  b.dense.resize(2 * size_t(nd));
  if ((e = cudaMemcpy(hx.data(), ox, 4 * T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(hy.data(), oy, 4 * T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(hl.data(), ol, 4 * T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(hr.data(), orr, 4 * T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(hadm.data(), oadm, T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(hden.data(), oden, T, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(b.approx.data(), oa, 8 * size_t(na), cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(b.dense.data(), od, 8 * size_t(nd), cudaMemcpyDeviceToHost)))
    return cuda_fail(e, "reading the block tree back");
  b.nodes.resize(T);
  for (size_t k = 0; k < T; k++)
    b.nodes[k] = BNode{hx[k], hy[k], hl[k], hr[k], hadm[k] != 0, hden[k] != 0};
  return HMGPU_OK;
}
}  // namespace hm

extern "C" int hmgpu_tree_build_device(const double *coords, int64_t npts, int64_t leaf, int64_t dims,
                                       hmgpu_tree **out) {
  if (!out) return hm::fail(HMGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  auto *h = new (std::nothrow) hmgpu_tree;
  if (!h) return hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  int rc;
  try {
    rc = hm::build_tree_device(coords, npts, leaf, dims, h->t);
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

extern "C" int hmgpu_blocks_build_device(const hmgpu_tree *X, const hmgpu_tree *Y, double eta, int merge,
                                         hmgpu_blocks **out) {
  if (!X || !Y || !out) return hm::fail(HMGPU_ERR_INVALID, "NULL argument");
  *out = nullptr;
  auto *h = new (std::nothrow) hmgpu_blocks;
  if (!h) return hm::fail(HMGPU_ERR_NOMEM, "host allocation failed");
  int rc;
  try {
    rc = hm::build_blocks_device(X->t, Y->t, eta, merge != 0, h->b);
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
