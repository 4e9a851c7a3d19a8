/*
 * cpu_mul.c -- TEST INFRASTRUCTURE ONLY: the timed CPU baseline.
 *
 * The reference's CPU product mul!(result, ::HMatrixCPU, x) (src/mult.jl:6-32)
 * on the oracle's assembled H-matrix, shaped as the reference runs it:
 *
 *   fill!(result, 0)                                   (:7)
 *   x_ordered = x[source_index_map]                    (:10), once per product
 *   result[rs:re] .+= D * x_ordered[cs:ce]             (:13-18), one gemv per dense block
 *   result[rs:re] .+= U * (V * x_ordered[cs:ce])       (:21-27), two gemvs per low-rank block
 *   result[target_index_map] .= result                 (:30), once per product
 *
 * Julia hands each gemv to BLAS, whose kernels keep several vector
 * accumulators in flight and fuse multiply-adds. The dot products here do the
 * same (four 2-wide accumulators through GCC's generic vector types, compiled
 * with contraction on), so the loop streams the factors at memory speed
 * rather than at the latency of one scalar add chain. Results therefore agree
 * with oracle.c's checker product (sequential sums, no FMA) to rounding only;
 * this file is never the checker.
 *
 * With nthreads > 1 the block list is cut into contiguous, byte-balanced
 * ranges; each thread accumulates into its own result vector, and the vectors
 * are summed in thread order by row slices before the scatter. Permutation,
 * zeroing, reduction and scatter are all inside every timed product.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "oracle.h"
#include "or_internal.h"

typedef double v2d __attribute__((vector_size(16)));

static inline v2d ld2(const double *p) {
  v2d v;
  memcpy(&v, p, sizeof v);
  return v;
}

/* sum_j a[j] * x[j] with eight products in flight */
static double dot(const double *a, const double *x, int64_t n) {
  v2d s0 = {0.0, 0.0}, s1 = s0, s2 = s0, s3 = s0;
  int64_t j = 0;
  for (; j + 8 <= n; j += 8) {
    s0 += ld2(a + j) * ld2(x + j);
    s1 += ld2(a + j + 2) * ld2(x + j + 2);
    s2 += ld2(a + j + 4) * ld2(x + j + 4);
    s3 += ld2(a + j + 6) * ld2(x + j + 6);
  }
  for (; j + 2 <= n; j += 2) s0 += ld2(a + j) * ld2(x + j);
  v2d s = (s0 + s1) + (s2 + s3);
  double r = s[0] + s[1];
  for (; j < n; j++) r += a[j] * x[j];
  return r;
}

struct or_cpu_mul {
  const or_hmatrix *h;
  int nthreads;
  int64_t *b0;      /* thread t runs blocks [b0[t], b0[t+1]) of [dense | approx] */
  double **acc;     /* per-thread result vectors (tlen)                           */
  double **tmp;     /* per-thread V*x buffers (max rank)                          */
  double *xo;       /* x_ordered (slen)                                           */
  pthread_barrier_t bar;
  const double *x;  /* current product's input and output                        */
  double *y;
};

typedef struct {
  or_cpu_mul *p;
  int t;
} worker_arg;

static void run_block(const or_hmatrix *h, int64_t b, const double *xo, double *acc, double *tmp) {
  if (b < h->nd) { /* :13-18 */
    const or_block *B = &h->dense[b];
    const int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1;
    const double *x = xo + (B->cs - 1);
    double *out = acc + (B->rs - 1);
    for (int64_t i = 0; i < m; i++) out[i] += dot(B->D + i * n, x, n);
  } else { /* :21-27 */
    const or_block *B = &h->approx[b - h->nd];
    const int64_t m = B->re - B->rs + 1, n = B->ce - B->cs + 1, r = B->r;
    const double *x = xo + (B->cs - 1);
    for (int64_t q = 0; q < r; q++) tmp[q] = dot(B->V + q * n, x, n);
    double *out = acc + (B->rs - 1);
    for (int64_t i = 0; i < m; i++) out[i] += dot(B->U + i * r, tmp, r);
  }
}

static void *worker(void *arg) {
  worker_arg *w = (worker_arg *)arg;
  or_cpu_mul *p = w->p;
  const or_hmatrix *h = p->h;
  const int t = w->t, nt = p->nthreads;
  /* x_ordered = x[source_index_map], this thread's slice (:10) */
  const int64_t s0 = h->slen * t / nt, s1 = h->slen * (t + 1) / nt;
  for (int64_t j = s0; j < s1; j++) p->xo[j] = p->x[h->smap[j] - 1];
  memset(p->acc[t], 0, (size_t)h->tlen * sizeof(double)); /* fill!(result, 0) (:7) */
  if (nt > 1) pthread_barrier_wait(&p->bar);
  for (int64_t b = p->b0[t]; b < p->b0[t + 1]; b++) run_block(h, b, p->xo, p->acc[t], p->tmp[t]);
  if (nt > 1) pthread_barrier_wait(&p->bar);
  /* sum of the per-thread results in thread order, then the scatter (:30) */
  const int64_t r0 = h->tlen * t / nt, r1 = h->tlen * (t + 1) / nt;
  for (int64_t i = r0; i < r1; i++) {
    double s = p->acc[0][i];
    for (int u = 1; u < nt; u++) s += p->acc[u][i];
    p->y[h->tmap[i] - 1] = s;
  }
  return NULL;
}

static int64_t block_bytes(const or_hmatrix *h, int64_t b) {
  if (b < h->nd) {
    const or_block *B = &h->dense[b];
    return (B->re - B->rs + 1) * (B->ce - B->cs + 1) + 1;
  }
  const or_block *B = &h->approx[b - h->nd];
  return B->r * ((B->re - B->rs + 1) + (B->ce - B->cs + 1)) + 1;
}

or_cpu_mul *or_cpu_mul_plan(const or_hmatrix *h, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  or_cpu_mul *p = (or_cpu_mul *)calloc(1, sizeof(or_cpu_mul));
  p->h = h;
  p->nthreads = nthreads;
  p->b0 = (int64_t *)calloc((size_t)nthreads + 1, sizeof(int64_t));
  p->acc = (double **)calloc((size_t)nthreads, sizeof(double *));
  p->tmp = (double **)calloc((size_t)nthreads, sizeof(double *));
  p->xo = (double *)malloc((size_t)(h->slen + 1) * sizeof(double));
  int64_t mr = 1;
  for (int64_t b = 0; b < h->na; b++)
    if (h->approx[b].r > mr) mr = h->approx[b].r;
  const int64_t nb = h->nd + h->na;
  int64_t total = 0;
  for (int64_t b = 0; b < nb; b++) total += block_bytes(h, b);
  int64_t b = 0, acc = 0;
  for (int t = 0; t < nthreads; t++) {
    p->acc[t] = (double *)malloc((size_t)(h->tlen + 1) * sizeof(double));
    p->tmp[t] = (double *)malloc((size_t)mr * sizeof(double));
    p->b0[t] = b;
    const int64_t goal = total * (t + 1) / nthreads;
    while (b < nb && (acc < goal || t == nthreads - 1)) acc += block_bytes(h, b++);
  }
  p->b0[nthreads] = nb;
  if (nthreads > 1) pthread_barrier_init(&p->bar, NULL, (unsigned)nthreads);
  return p;
}

double or_cpu_mul_run(or_cpu_mul *p, const double *x, double *y, int reps) {
  struct timespec a, b;
  const int nt = p->nthreads;
  worker_arg *args = (worker_arg *)malloc((size_t)nt * sizeof(worker_arg));
  pthread_t *th = (pthread_t *)malloc((size_t)nt * sizeof(pthread_t));
  clock_gettime(CLOCK_MONOTONIC, &a);
  for (int r = 0; r < reps; r++) {
    p->x = x;
    p->y = y;
    for (int t = 0; t < nt; t++) {
      args[t].p = p;
      args[t].t = t;
    }
    if (nt == 1) {
      worker(&args[0]);
    } else {
      for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, worker, &args[t]);
      for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
    }
  }
  clock_gettime(CLOCK_MONOTONIC, &b);
  free(args);
  free(th);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}

void or_cpu_mul_free(or_cpu_mul *p) {
  if (!p) return;
  for (int t = 0; t < p->nthreads; t++) {
    free(p->acc[t]);
    free(p->tmp[t]);
  }
  if (p->nthreads > 1) pthread_barrier_destroy(&p->bar);
  free(p->acc);
  free(p->tmp);
  free(p->b0);
  free(p->xo);
  free(p);
}

/* Bytes of factor data one product reads: 8 per stored FP64 entry. */
int64_t or_hmatrix_stored_entries(const or_hmatrix *h) {
  int64_t e = 0;
  for (int64_t b = 0; b < h->nd + h->na; b++) e += block_bytes(h, b) - 1;
  return e;
}
