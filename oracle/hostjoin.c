/*
 * CPU BASELINE — measurement infrastructure only.  Nothing in the product
 * library links, loads or calls this file; the benchmark times it as the
 * project's own indexed host join beside the reference's brute force.
 *
 * An OpenMP grid join on the host cores with the same index as the GPU
 * library: FP64 distances of every point to k reference points (given by the
 * caller), fields of width w = eps (1 + delta) with
 * delta = max(2^-20, 8 (d + 4) 2^-53 (1 + Dmax / eps)), packed into one
 * 63-bit key (field 0 most significant; uninformative fields dropped),
 * points sorted by key, non-empty bins as runs, and for each home bin the
 * bins >= it whose every field is within one of its own (depth-first walk
 * with binary searches over the sorted bin keys).  Each candidate pair is
 * decided with the reference's FP64 predicate, brute_force in
 * src/utils.cu:296-309: a sequential sum in column order, every operation
 * rounded (this file is compiled with -ffp-contract=off), compared with the
 * rounded eps * eps.  The ±1 relation is the completeness argument of
 * src/nodes.cu:416-435: the triangle inequality bounds |D_j(p) - D_j(q)| by
 * the distance, and delta covers the FP64 rounding of the distances.
 *
 * hostjoin_count() joins every home bin whose index is a multiple of
 * `home_stride` (1: all) and returns the unordered pairs (i < j) it found;
 * it also reports the candidate pairs of those home bins and of all bins,
 * the seconds of the index build plus the enumeration of every bin's
 * neighbours, and the seconds of the distance work of the sampled bins, so a
 * caller can scale a sampled run to the whole join.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define HJ_MAX_K 16

static double hj_now(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

typedef struct {
  uint64_t key;
  uint32_t idx;
} hj_item;

/* LSD radix sort of (key, idx) on the low `bits` bits, 8 bits a pass; stable. */
static void hj_sort(hj_item* a, hj_item* tmp, uint64_t n, int bits) {
  for (int sh = 0; sh < bits; sh += 8) {
    uint64_t cnt[257];
    memset(cnt, 0, sizeof cnt);
    for (uint64_t i = 0; i < n; ++i) cnt[((a[i].key >> sh) & 255u) + 1]++;
    for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
    for (uint64_t i = 0; i < n; ++i) tmp[cnt[(a[i].key >> sh) & 255u]++] = a[i];
    memcpy(a, tmp, n * sizeof(hj_item));
  }
}

static uint64_t hj_lower(const uint64_t* a, uint64_t lo, uint64_t hi, uint64_t v) {
  while (lo < hi) {
    uint64_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

typedef struct {
  int k;
  int shift[HJ_MAX_K];
  uint64_t mask[HJ_MAX_K];
  uint64_t maxkey[HJ_MAX_K];
} hj_layout;

/* Visits the bins >= h whose fields are all within one of bin h's, in
 * ascending order: fn(b, ctx) for each. */
static void hj_neighbours(const uint64_t* bkey, uint64_t m, uint64_t h, const hj_layout* L,
                          void (*fn)(uint64_t, void*), void* ctx) {
  if (L->k == 0) {
    fn(h, ctx);
    return;
  }
  int64_t kf[HJ_MAX_K];
  for (int j = 0; j < L->k; ++j) kf[j] = (int64_t)((bkey[h] >> L->shift[j]) & L->mask[j]);
  uint64_t lo[HJ_MAX_K + 1], hi[HJ_MAX_K + 1], base[HJ_MAX_K + 1];
  int di[HJ_MAX_K + 1];
  lo[0] = 0;
  hi[0] = m;
  base[0] = 0;
  di[0] = 0;
  int j = 0;
  while (j >= 0) {
    if (di[j] == 3) {
      --j;
      if (j >= 0) ++di[j];
      continue;
    }
    const int64_t cv = kf[j] + di[j] - 1;
    if (cv < 0 || (uint64_t)cv > L->maxkey[j]) {
      ++di[j];
      continue;
    }
    const uint64_t lower = base[j] | ((uint64_t)cv << L->shift[j]);
    const uint64_t upper = lower + (1ull << L->shift[j]);
    const uint64_t a = hj_lower(bkey, lo[j], hi[j], lower);
    const uint64_t b = hj_lower(bkey, a, hi[j], upper);
    if (a == b || b <= h) {
      ++di[j];
      continue;
    }
    if (j == L->k - 1) {
      fn(a, ctx);
      ++di[j];
      continue;
    }
    base[j + 1] = lower;
    lo[j + 1] = a;
    hi[j + 1] = b;
    di[j + 1] = 0;
    ++j;
  }
}

typedef struct {
  const double* xs; /* sorted rows */
  const uint64_t* bstart;
  uint32_t d;
  double eps2;
  uint64_t h;
  uint64_t pairs, cands;
  int join;
} hj_ctx;

static void hj_visit(uint64_t b, void* vp) {
  hj_ctx* c = (hj_ctx*)vp;
  const uint64_t h0 = c->bstart[c->h], h1 = c->bstart[c->h + 1];
  const uint64_t b0 = c->bstart[b], b1 = c->bstart[b + 1];
  const uint32_t d = c->d;
  if (b == c->h) {
    const uint64_t s = h1 - h0;
    c->cands += s * (s - 1) / 2;
  } else {
    c->cands += (h1 - h0) * (b1 - b0);
  }
  if (!c->join) return;
  for (uint64_t p = h0; p < h1; ++p) {
    const double* xp = c->xs + p * d;
    for (uint64_t q = (b == c->h ? p + 1 : b0); q < b1; ++q) {
      const double* xq = c->xs + q * d;
      double s = 0.0;
      for (uint32_t k = 0; k < d; ++k) {
        if (s > c->eps2) break; /* cannot change the outcome: the sum never decreases */
        const double t = xp[k] - xq[k];
        const double sq = t * t;
        s = s + sq;
      }
      if (s <= c->eps2) c->pairs++;
    }
  }
}

uint64_t hostjoin_count(const double* x, uint64_t n, uint32_t d, const double* rps, int k, double eps,
                        uint64_t home_stride, int threads, uint64_t* cand_sampled, uint64_t* cand_all,
                        double* sec_index, double* sec_join, uint64_t* n_bins) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  if (home_stride == 0) home_stride = 1;
  const double t0 = hj_now();
  const double eps2 = eps * eps;
  if (k > HJ_MAX_K) k = HJ_MAX_K;
  double* D = (double*)malloc(sizeof(double) * (n ? n : 1) * (k ? k : 1));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i)
    for (int j = 0; j < k; ++j) {
      double s = 0.0;
      for (uint32_t c = 0; c < d; ++c) {
        const double t = x[(uint64_t)i * d + c] - rps[(uint64_t)j * d + c];
        s = s + t * t;
      }
      D[(uint64_t)i * k + j] = sqrt(s);
    }
  /* key layout */
  hj_layout L;
  memset(&L, 0, sizeof L);
  int col[HJ_MAX_K];
  double dmin[HJ_MAX_K], w[HJ_MAX_K];
  int bits_acc = 0, fb[HJ_MAX_K];
  for (int j = 0; j < k; ++j) {
    double lo = INFINITY, hi = -INFINITY;
    for (uint64_t i = 0; i < n; ++i) {
      const double v = D[i * k + j];
      if (v < lo) lo = v;
      if (v > hi) hi = v;
    }
    if (!isfinite(lo) || !isfinite(hi) || !(hi >= lo)) continue;
    const double u64 = ldexp(1.0, -53);
    const double ratio = eps > 0 ? hi / eps : 0.0;
    double delta = 8.0 * (d + 4) * u64 * (1.0 + ratio);
    if (delta < ldexp(1.0, -20)) delta = ldexp(1.0, -20);
    double wj = eps * (1.0 + delta);
    const double span = hi - lo;
    if (!(wj > 0) || span / wj > ldexp(1.0, 30)) wj = fmax(wj, span / ldexp(1.0, 30));
    if (!(wj > 0)) wj = 1.0;
    const double mk = fmin(floor(span / wj), ldexp(1.0, 30));
    if (mk < 1.0) continue;
    int b = 0;
    for (uint64_t v = (uint64_t)mk; v; v >>= 1) ++b;
    if (bits_acc + b > 63) break;
    col[L.k] = j;
    dmin[L.k] = lo;
    w[L.k] = wj;
    L.maxkey[L.k] = (uint64_t)mk;
    fb[L.k] = b;
    bits_acc += b;
    L.k++;
  }
  int sh = bits_acc;
  for (int f = 0; f < L.k; ++f) {
    sh -= fb[f];
    L.shift[f] = sh;
    L.mask[f] = (1ull << fb[f]) - 1ull;
  }
  hj_item* it = (hj_item*)malloc(sizeof(hj_item) * (n ? n : 1));
  hj_item* tmp = (hj_item*)malloc(sizeof(hj_item) * (n ? n : 1));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t key = 0;
    for (int f = 0; f < L.k; ++f) {
      double q = floor((D[(uint64_t)i * k + col[f]] - dmin[f]) / w[f]);
      if (q < 0) q = 0;
      if (q > (double)L.maxkey[f]) q = (double)L.maxkey[f];
      key |= (uint64_t)q << L.shift[f];
    }
    it[i].key = key;
    it[i].idx = (uint32_t)i;
  }
  free(D);
  hj_sort(it, tmp, n, bits_acc);
  free(tmp);
  /* bins and sorted rows */
  uint64_t* bstart = (uint64_t*)malloc(sizeof(uint64_t) * (n + 1));
  uint64_t* bkey = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i)
    if (i == 0 || it[i].key != it[i - 1].key) {
      bstart[m] = i;
      bkey[m] = it[i].key;
      ++m;
    }
  bstart[m] = n;
  double* xs = (double*)malloc(sizeof(double) * (n ? n : 1) * d);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) memcpy(xs + (uint64_t)i * d, x + (uint64_t)it[i].idx * d, d * sizeof(double));
  free(it);
  uint64_t pairs = 0, cs = 0, ca = 0;
  /* candidate pairs of every home bin (enumeration only) */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : ca)
  for (int64_t h = 0; h < (int64_t)m; ++h) {
    hj_ctx c = {xs, bstart, d, eps2, (uint64_t)h, 0, 0, 0};
    hj_neighbours(bkey, m, (uint64_t)h, &L, hj_visit, &c);
    ca += c.cands;
  }
  const double t2 = hj_now();
  /* the join of the sampled home bins */
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : pairs, cs)
  for (int64_t h = 0; h < (int64_t)m; h += (int64_t)home_stride) {
    hj_ctx c = {xs, bstart, d, eps2, (uint64_t)h, 0, 0, 1};
    hj_neighbours(bkey, m, (uint64_t)h, &L, hj_visit, &c);
    pairs += c.pairs;
    cs += c.cands;
  }
  const double t3 = hj_now();
  free(xs);
  free(bstart);
  free(bkey);
  if (cand_sampled) *cand_sampled = cs;
  if (cand_all) *cand_all = ca;
  if (sec_index) *sec_index = t2 - t0; /* index build and neighbour enumeration of all bins */
  if (sec_join) *sec_join = t3 - t2;  /* distance work of the sampled home bins */
  if (n_bins) *n_bins = m;
  return pairs;
}
