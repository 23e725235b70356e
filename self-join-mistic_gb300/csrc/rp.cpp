// Reference-point selection (host).
//
// Reference counterpart: createRPArray, src/utils.cu:66-281, which draws 2k
// uniform points in [0,1)^d with glibc rand(), keeps the k/2 whose distances
// over a 1% sample have the largest spread, and adds "box corner" points;
// buildNodeNet then scores 32 such candidates per layer
// (src/nodes.cu:168-222).  The goal is the same here — reference points whose
// distance fields spread the data over many ε-wide bins — reached directly:
// the k points sit far outside the data along its k leading principal axes
// (sample covariance, orthogonal iteration), so each distance field behaves
// like a projection on one principal axis and successive fields are nearly
// uncorrelated.  MISTIC_RP_BOX reproduces the plain "uniform in the bounding
// box" choice with a seeded generator; MISTIC_RP_USER takes the caller's.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace mistic {

namespace {

// SplitMix64: small deterministic generator for seeded choices.
struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
};

// Modified Gram-Schmidt on the k columns of V (d x k, column-major).
void orthonormalise(std::vector<double>& V, uint32_t d, uint32_t k, SplitMix& rng) {
  for (uint32_t c = 0; c < k; ++c) {
    double* v = &V[(size_t)c * d];
    for (int pass = 0; pass < 2; ++pass) {
      for (uint32_t p = 0; p < c; ++p) {
        const double* u = &V[(size_t)p * d];
        double dot = 0;
        for (uint32_t i = 0; i < d; ++i) dot += u[i] * v[i];
        for (uint32_t i = 0; i < d; ++i) v[i] -= dot * u[i];
      }
    }
    double nrm = 0;
    for (uint32_t i = 0; i < d; ++i) nrm += v[i] * v[i];
    nrm = sqrt(nrm);
    if (nrm < 1e-300) {  // degenerate direction: replace with a random one
      for (uint32_t i = 0; i < d; ++i) v[i] = rng.normal();
      --c;  // redo this column
      continue;
    }
    for (uint32_t i = 0; i < d; ++i) v[i] /= nrm;
  }
}

}  // namespace

void select_reference_points(const mistic_opts& o, uint32_t d, uint32_t k, const std::vector<double>& mean,
                             const std::vector<double>& mn, const std::vector<double>& mx,
                             const std::vector<double>& cov, std::vector<double>& rps) {
  rps.assign((size_t)k * d, 0.0);
  if (k == 0) return;
  if (o.rp_mode == MISTIC_RP_USER) {
    if (!o.rp_user) throw Error(MISTIC_ERR_INVALID_ARG, "rp_mode USER needs opts.rp_user");
    for (size_t i = 0; i < (size_t)k * d; ++i) {
      if (!std::isfinite(o.rp_user[i])) throw Error(MISTIC_ERR_INVALID_ARG, "rp_user has a non-finite value");
      rps[i] = o.rp_user[i];
    }
    return;
  }
  SplitMix rng(o.seed ^ 0x6d69737469637270ull);
  if (o.rp_mode == MISTIC_RP_BOX || cov.empty()) {
    for (uint32_t j = 0; j < k; ++j)
      for (uint32_t i = 0; i < d; ++i) rps[(size_t)j * d + i] = mn[i] + (mx[i] - mn[i]) * rng.uniform();
    return;
  }
  // PCA: orthogonal iteration for the top-kk eigenvectors of cov.
  const uint32_t kk = std::min(k, d);
  std::vector<double> V((size_t)kk * d), W((size_t)kk * d);
  for (auto& v : V) v = rng.normal();
  orthonormalise(V, d, kk, rng);
  const int iters = d <= 64 ? 200 : 60;
  for (int it = 0; it < iters; ++it) {
    for (uint32_t c = 0; c < kk; ++c) {
      const double* v = &V[(size_t)c * d];
      double* wv = &W[(size_t)c * d];
      for (uint32_t a = 0; a < d; ++a) {
        const double* row = &cov[(size_t)a * d];
        double s = 0;
        for (uint32_t b = 0; b < d; ++b) s += row[b] * v[b];
        wv[a] = s;
      }
    }
    std::swap(V, W);
    orthonormalise(V, d, kk, rng);
  }
  // Order the converged directions by Rayleigh quotient (largest first).
  std::vector<std::pair<double, uint32_t>> rq(kk);
  for (uint32_t c = 0; c < kk; ++c) {
    const double* v = &V[(size_t)c * d];
    double s = 0;
    for (uint32_t a = 0; a < d; ++a) {
      double r = 0;
      for (uint32_t b = 0; b < d; ++b) r += cov[(size_t)a * d + b] * v[b];
      s += v[a] * r;
    }
    rq[c] = {-s, c};
  }
  std::sort(rq.begin(), rq.end());
  double diam = 0;
  for (uint32_t i = 0; i < d; ++i) diam += (mx[i] - mn[i]) * (mx[i] - mn[i]);
  diam = sqrt(diam);
  if (!(diam > 0)) diam = 1.0;
  const double far = 64.0 * diam;
  for (uint32_t j = 0; j < k; ++j) {
    double* r = &rps[(size_t)j * d];
    if (j < kk) {
      const double* v = &V[(size_t)rq[j].second * d];
      for (uint32_t i = 0; i < d; ++i) r[i] = mean[i] - far * v[i];
    } else {  // more reference points than dimensions: seeded box points
      for (uint32_t i = 0; i < d; ++i) r[i] = mn[i] + (mx[i] - mn[i]) * rng.uniform();
    }
  }
}

// Scored reference points (MISTIC_RP_SCORED): the reference's per-layer
// selection, buildNodeNet's candidate scoring (src/nodes.cu:168-222) over
// createRPArray's candidate sets (src/utils.cu:66-136), restated: layer by
// layer, every candidate point bins a sample of the data into eps-wide
// distance fields, and the candidate that leaves the fewest sample pairs
// within one field of each other on every layer chosen so far (the
// neighbour relation of the join) is kept.  Candidates: far points along the
// sample's leading principal axes on both sides, sample points, and seeded
// box points.
void select_reference_points_scored(const mistic_opts& o, uint32_t d, uint32_t k, double eps,
                                    const std::vector<double>& mean, const std::vector<double>& mn,
                                    const std::vector<double>& mx, const std::vector<double>& cov,
                                    const std::vector<double>& sample, uint32_t S, std::vector<double>& rps) {
  rps.assign((size_t)k * d, 0.0);
  if (k == 0) return;
  // candidate pool
  const uint32_t na = std::min<uint32_t>(2 * k, d);
  std::vector<double> pca;
  {
    mistic_opts o2 = o;
    o2.rp_mode = MISTIC_RP_PCA;
    select_reference_points(o2, d, na, mean, mn, mx, cov, pca);  // far points on one side of each axis
  }
  std::vector<double> cand;
  for (uint32_t a = 0; a < na; ++a) {
    const double* p = &pca[(size_t)a * d];
    for (int side = 0; side < 2; ++side)
      for (uint32_t i = 0; i < d; ++i) cand.push_back(side == 0 ? p[i] : 2.0 * mean[i] - p[i]);
  }
  SplitMix rng(o.seed ^ 0x73636f7265647270ull);
  for (int c = 0; c < 8 && S > 0; ++c) {
    const uint32_t r = (uint32_t)(rng.next() % S);
    for (uint32_t i = 0; i < d; ++i) cand.push_back(sample[(size_t)r * d + i]);
  }
  for (int c = 0; c < 8; ++c)
    for (uint32_t i = 0; i < d; ++i) cand.push_back(mn[i] + (mx[i] - mn[i]) * rng.uniform());
  const uint32_t C = (uint32_t)(cand.size() / d);
  // scoring sample: up to 1024 of the sample rows, evenly spaced
  const uint32_t T = std::min<uint32_t>(S, 1024);
  std::vector<uint32_t> rows(T);
  for (uint32_t t = 0; t < T; ++t) rows[t] = (uint32_t)((uint64_t)t * S / std::max(1u, T));
  const double w = eps > 0 ? eps : 1.0;
  std::vector<int64_t> fld((size_t)C * T);
  for (uint32_t c = 0; c < C; ++c)
    for (uint32_t t = 0; t < T; ++t) {
      const double* x = &sample[(size_t)rows[t] * d];
      const double* r = &cand[(size_t)c * d];
      double s2 = 0;
      for (uint32_t i = 0; i < d; ++i) s2 += (x[i] - r[i]) * (x[i] - r[i]);
      fld[(size_t)c * T + t] = (int64_t)std::floor(std::sqrt(s2) / w);
    }
  // surviving sample pairs (a < b), as a flat bitmap
  const size_t NP = (size_t)T * (T - (T > 0)) / 2;
  std::vector<uint8_t> alive(NP, 1);
  std::vector<uint8_t> used(C, 0);
  for (uint32_t j = 0; j < k; ++j) {
    uint32_t best = UINT32_MAX;
    size_t best_n = SIZE_MAX;
    for (uint32_t c = 0; c < C; ++c) {
      if (used[c]) continue;
      const int64_t* f = &fld[(size_t)c * T];
      size_t cnt = 0, pi = 0;
      for (uint32_t a = 0; a < T; ++a)
        for (uint32_t b = a + 1; b < T; ++b, ++pi)
          if (alive[pi] && std::llabs(f[a] - f[b]) <= 1) ++cnt;
      if (cnt < best_n) {
        best_n = cnt;
        best = c;
      }
    }
    if (best == UINT32_MAX) break;
    used[best] = 1;
    const int64_t* f = &fld[(size_t)best * T];
    size_t pi = 0;
    for (uint32_t a = 0; a < T; ++a)
      for (uint32_t b = a + 1; b < T; ++b, ++pi)
        if (alive[pi] && std::llabs(f[a] - f[b]) > 1) alive[pi] = 0;
    for (uint32_t i = 0; i < d; ++i) rps[(size_t)j * d + i] = cand[(size_t)best * d + i];
  }
}

}  // namespace mistic
