/*
 * ORACLE — test infrastructure only.  This file is the CPU checker for the
 * GPU ε-self-join; nothing in the product library links, loads or calls it.
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark use it.
 *
 * It restates the reference's CPU brute-force join, `brute_force` in
 * src/utils.cu:285-317 of bwd29/self-join-MiSTIC:
 *
 *   for every ordered pair (i, j):
 *       distance = 0
 *       for k in 0..dim-1:                      natural column order
 *           if distance > epsilon*epsilon: break   (early exit)
 *           distance += (A[i*dim+k] - A[j*dim+k]) * (A[i*dim+k] - A[j*dim+k])
 *       if distance <= epsilon*epsilon: count++
 *
 * in FP64, with the subtraction, the product and the addition each rounded
 * (no fused multiply-add: this file is compiled with -ffp-contract=off so
 * x86-64 and aarch64 produce the same bits).  The early exit cannot change
 * the outcome because adding a non-negative term never decreases a
 * round-to-nearest sum, so it is kept only as a speed-up.
 *
 * The reference counts ordered pairs including i == j in an `unsigned int`
 * (utils.cu:287); here the count is 64-bit and the pair set is emitted as
 * canonical unordered pairs (i < j, ascending by i then j), from which the
 * reference's number is 2*U + n.  FP32 inputs are widened to FP64 first, the
 * same predicate the GPU applies to them.
 *
 * Parity pin: tests/golden holds counts produced by the reference's own
 * brute_force compiled from its unmodified source (oracle/build_ref.sh) on
 * seeded inputs; the test suite checks this file against them.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_F64 0
#define ORACLE_F32 1

static inline double coord(const void* pts, int dtype, uint64_t idx) {
  return dtype == ORACLE_F32 ? (double)((const float*)pts)[idx]
                             : ((const double*)pts)[idx];
}

/* The predicate of utils.cu:296-309: sequential FP64 sum of rounded squares
 * of rounded differences, compared with the rounded product epsilon*epsilon. */
static inline double sqdist_seq(const void* pts, int dtype, uint64_t i,
                                uint64_t j, uint32_t d, double eps2, int early) {
  double s = 0.0;
  for (uint32_t k = 0; k < d; ++k) {
    if (early && s > eps2) break;
    double t = coord(pts, dtype, i * d + k) - coord(pts, dtype, j * d + k);
    double sq = t * t;
    s = s + sq;
  }
  return s;
}

/* Exact FP64 squared distance of the predicate (no early exit). */
double oracle_sqdist(const void* pts, int dtype, uint64_t i, uint64_t j,
                     uint32_t d) {
  return sqdist_seq(pts, dtype, i, j, d, 0.0, 0);
}

typedef struct {
  uint32_t* buf;
  uint64_t len, cap;
} pairbuf;

static void pb_push(pairbuf* b, uint32_t i, uint32_t j) {
  if (b->len == b->cap) {
    uint64_t nc = b->cap ? b->cap * 2 : 1024;
    uint32_t* nb = (uint32_t*)realloc(b->buf, nc * 2 * sizeof(uint32_t));
    if (!nb) abort();
    b->buf = nb;
    b->cap = nc;
  }
  b->buf[2 * b->len] = i;
  b->buf[2 * b->len + 1] = j;
  b->len++;
}

/*
 * Brute-force ε-self-join over n points of dimension d.
 *   pts       row-major n x d, FP64 (dtype 0) or FP32 (dtype 1)
 *   eps       distance threshold; the comparison is s <= eps*eps
 *   out_pairs optional: receives a malloc'd array of 2*U uint32 (i, j),
 *             i < j, ascending; free with oracle_free
 *   out_ambig optional: number of pairs with |s - eps*eps| <= 4 ulp(eps*eps)
 * Returns U, the number of unordered pairs i < j within ε.
 */
uint64_t oracle_brute_pairs(const void* pts, int dtype, uint64_t n, uint32_t d,
                            double eps, uint32_t** out_pairs,
                            uint64_t* out_ambig, int threads) {
  const double eps2 = eps * eps;
  const double ulp4 = 4.0 * (nextafter(eps2, INFINITY) - eps2);
  const uint64_t blk = 64;
  const uint64_t nblk = (n + blk - 1) / blk;
  pairbuf* bufs = (pairbuf*)calloc(nblk ? nblk : 1, sizeof(pairbuf));
  uint64_t total = 0, ambig = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total, ambig)
#endif
  for (uint64_t b = 0; b < nblk; ++b) {
    uint64_t i0 = b * blk, i1 = i0 + blk < n ? i0 + blk : n;
    for (uint64_t i = i0; i < i1; ++i) {
      for (uint64_t j = i + 1; j < n; ++j) {
        double s = sqdist_seq(pts, dtype, i, j, d, eps2, !out_ambig);
        if (out_ambig && fabs(s - eps2) <= ulp4) ambig++;
        if (s <= eps2) {
          total++;
          if (out_pairs) pb_push(&bufs[b], (uint32_t)i, (uint32_t)j);
        }
      }
    }
  }
  if (out_pairs) {
    uint32_t* all = (uint32_t*)malloc((total ? total : 1) * 2 * sizeof(uint32_t));
    uint64_t pos = 0;
    for (uint64_t b = 0; b < nblk; ++b) {
      if (bufs[b].len)
        memcpy(all + 2 * pos, bufs[b].buf, bufs[b].len * 2 * sizeof(uint32_t));
      pos += bufs[b].len;
    }
    *out_pairs = all;
  }
  for (uint64_t b = 0; b < nblk; ++b) free(bufs[b].buf);
  free(bufs);
  if (out_ambig) *out_ambig = ambig;
  return total;
}

/*
 * Neighbours of selected query rows against all n rows, same predicate.
 * For each query q (ascending list), appends every j != q with s <= eps2 as
 * a pair (min(q,j), max(q,j)).  Used to check full-size GPU runs on a sample
 * of rows.  Returns the number of pairs written (allocated in *out_pairs).
 */
uint64_t oracle_query_pairs(const void* pts, int dtype, uint64_t n, uint32_t d,
                            double eps, const uint32_t* queries, uint64_t nq,
                            uint32_t** out_pairs, int threads) {
  const double eps2 = eps * eps;
  pairbuf* bufs = (pairbuf*)calloc(nq ? nq : 1, sizeof(pairbuf));
  uint64_t total = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
#endif
  for (uint64_t t = 0; t < nq; ++t) {
    uint64_t q = queries[t];
    for (uint64_t j = 0; j < n; ++j) {
      if (j == q) continue;
      double s = sqdist_seq(pts, dtype, q, j, d, eps2, 1);
      if (s <= eps2) {
        total++;
        pb_push(&bufs[t], (uint32_t)(q < j ? q : j), (uint32_t)(q < j ? j : q));
      }
    }
  }
  uint32_t* all = (uint32_t*)malloc((total ? total : 1) * 2 * sizeof(uint32_t));
  uint64_t pos = 0;
  for (uint64_t t = 0; t < nq; ++t) {
    if (bufs[t].len)
      memcpy(all + 2 * pos, bufs[t].buf, bufs[t].len * 2 * sizeof(uint32_t));
    pos += bufs[t].len;
    free(bufs[t].buf);
  }
  free(bufs);
  *out_pairs = all;
  return total;
}

/* Ordered count including self, exactly as the reference's brute_force
 * reports it (2*U + n), for timing the reference algorithm as written: it
 * visits all n*n ordered pairs. */
uint64_t oracle_brute_count_ordered(const void* pts, int dtype, uint64_t n,
                                    uint32_t d, double eps, int threads) {
  const double eps2 = eps * eps;
  uint64_t total = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
#endif
  for (uint64_t i = 0; i < n; ++i) {
    for (uint64_t j = 0; j < n; ++j) {
      double s = sqdist_seq(pts, dtype, i, j, d, eps2, 1);
      if (s <= eps2) total++;
    }
  }
  return total;
}

/* Ordered count over a row range [i0, i1) against all n rows: a bounded
 * sample of the reference algorithm for CPU timing. */
uint64_t oracle_brute_count_rows(const void* pts, int dtype, uint64_t n,
                                 uint32_t d, double eps, uint64_t i0,
                                 uint64_t i1, int threads) {
  const double eps2 = eps * eps;
  uint64_t total = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
#endif
  for (uint64_t i = i0; i < i1; ++i) {
    for (uint64_t j = 0; j < n; ++j) {
      double s = sqdist_seq(pts, dtype, i, j, d, eps2, 1);
      if (s <= eps2) total++;
    }
  }
  return total;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_free(void* p) { free(p); }
