// mistic: command-line front end with the reference's argument order,
//
//   mistic <file.bin> <dim> <numRP> <epsilon> [options]
//
// (bwd29/self-join-MiSTIC src/main.cu:25-31: file, dimensionality, number of
// reference points, ε).  The input is the reference's format: raw
// little-endian FP64 row-major, n = bytes / 8 / dim (src/main.cu:42-50).
// stdout carries the reference's report lines, including
// "Total results Set Size: N" with N = ordered pairs including self pairs
// (src/launcher.cu:3513), so scripts that parse the reference keep working;
// stderr carries one JSON line with the full result.
//
// Options (none exist in the reference):
//   --f32              input file holds FP32 rows
//   --mode auto|fp64|fp32|bf16|tf32
//   --rp pca|box|scored  reference-point placement
//   --seed S
//   --pairs out.bin    write the i<j pair list as uint32 (i, j) rows, sorted
//   --device N
//
//   mistic --to-bin <in.txt> <out.bin>
// converts a comma/white-space separated text file into the raw FP64 input
// format (the reference's toBin tool, toCSV.cpp:52-85) and prints the
// number of values, as that tool does.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/mistic.h"

static int usage(const char* p) {
  fprintf(stderr,
          "usage: %s <file.bin> <dim> <numRP> <epsilon> [--f32] [--mode auto|fp64|fp32|bf16|tf32] "
          "[--rp pca|box|scored] [--seed S] [--pairs out.bin] [--device N]\n"
          "       %s --to-bin <in.txt> <out.bin>\n",
          p, p);
  return 2;
}

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "--to-bin") {
    uint64_t cnt = 0;
    const mistic_status s = mistic_convert_text(argv[2], argv[3], &cnt);
    if (s != MISTIC_OK) {
      fprintf(stderr, "%s\n", mistic_strerror(s));
      return 1;
    }
    printf("size of data: %llu\n", (unsigned long long)cnt);
    return 0;
  }
  if (argc < 5) return usage(argv[0]);
  const char* file = argv[1];
  const unsigned dim = (unsigned)strtoul(argv[2], nullptr, 10);
  const unsigned numRP = (unsigned)strtoul(argv[3], nullptr, 10);
  double eps = 0;
  if (sscanf(argv[4], "%lf", &eps) != 1) return usage(argv[0]);
  mistic_opts o;
  mistic_opts_init(&o);
  mistic_dtype dt = MISTIC_F64;
  const char* pairs_out = nullptr;
  int device = 0;
  for (int i = 5; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : nullptr; };
    if (a == "--f32") {
      dt = MISTIC_F32;
    } else if (a == "--mode") {
      const char* v = next();
      if (!v) return usage(argv[0]);
      std::string m = v;
      o.mode = m == "fp64"   ? MISTIC_MODE_FP64
               : m == "fp32" ? MISTIC_MODE_FP32
               : m == "bf16" ? MISTIC_MODE_BF16
               : m == "tf32" ? MISTIC_MODE_TF32
                             : MISTIC_MODE_AUTO;
    } else if (a == "--rp") {
      const char* v = next();
      if (!v) return usage(argv[0]);
      o.rp_mode = std::string(v) == "box" ? MISTIC_RP_BOX : (std::string(v) == "scored" ? MISTIC_RP_SCORED : MISTIC_RP_PCA);
    } else if (a == "--seed") {
      const char* v = next();
      if (!v) return usage(argv[0]);
      o.seed = strtoull(v, nullptr, 10);
    } else if (a == "--pairs") {
      pairs_out = next();
      if (!pairs_out) return usage(argv[0]);
      o.pairs = MISTIC_PAIRS_HOST;
      o.sort_pairs = 1;
    } else if (a == "--device") {
      const char* v = next();
      if (!v) return usage(argv[0]);
      device = atoi(v);
    } else {
      return usage(argv[0]);
    }
  }
  const auto t0 = std::chrono::steady_clock::now();
  void* pts = nullptr;
  uint64_t n = 0;
  mistic_status s = mistic_read_points(file, dim, dt, &pts, &n);
  if (s != MISTIC_OK) {
    fprintf(stderr, "error: cannot read %s: %s\n", file, mistic_strerror(s));
    return 1;
  }
  const auto t1 = std::chrono::steady_clock::now();
  printf("\nTime to read in file: %f\n", std::chrono::duration<double>(t1 - t0).count());
  printf("\nNumber points: %llu ", (unsigned long long)n);
  printf("\nNumber Dimensions: %u ", dim);
  printf("\nNumber Reference Points: %u ", numRP);
  printf("\nDistance Threshold: %f \n*********************************\n\n", eps);
  mistic_handle h = nullptr;
  s = mistic_create(&h, device, nullptr);
  if (s != MISTIC_OK) {
    fprintf(stderr, "error: %s\n", mistic_strerror(s));
    mistic_free_host(pts);
    return 1;
  }
  mistic_result r;
  s = mistic_selfjoin(h, pts, n, dim, dt, numRP, eps, &o, &r);
  if (s != MISTIC_OK) {
    fprintf(stderr, "error: %s: %s\n", mistic_strerror(s), mistic_last_error(h));
    mistic_destroy(h);
    mistic_free_host(pts);
    return 1;
  }
  const auto t2 = std::chrono::steady_clock::now();
  printf("Total results Set Size: %llu \n", (unsigned long long)r.pairs_ordered_incl_self);
  printf("Kernel Time: %f\n", r.ms_join / 1e3);
  printf("Total Time: %f\n", std::chrono::duration<double>(t2 - t1).count());
  fprintf(stderr,
          "{\"n\": %llu, \"d\": %u, \"k_used\": %u, \"eps\": %.17g, \"pairs_ij\": %llu, "
          "\"pairs_ordered_incl_self\": %llu, \"candidates\": %llu, \"band_pairs\": %llu, "
          "\"ulp_ambiguous\": %llu, \"bins\": %llu, \"bin_pairs\": %llu, \"mode\": %d, "
          "\"ms\": {\"h2d\": %.3f, \"prep\": %.3f, \"keys\": %.3f, \"sort\": %.3f, \"bins\": %.3f, "
          "\"enum\": %.3f, \"join\": %.3f, \"d2h\": %.3f, \"total\": %.3f, \"wall\": %.3f}}\n",
          (unsigned long long)r.n, r.d, r.k_used, eps, (unsigned long long)r.pairs_ij,
          (unsigned long long)r.pairs_ordered_incl_self, (unsigned long long)r.candidates,
          (unsigned long long)r.band_pairs, (unsigned long long)r.ulp_ambiguous, (unsigned long long)r.n_bins,
          (unsigned long long)r.n_bin_pairs, (int)r.mode_used, r.ms_h2d, r.ms_prep, r.ms_keys, r.ms_sort,
          r.ms_bins, r.ms_enum, r.ms_join, r.ms_d2h, r.ms_total, r.ms_wall);
  int rc = 0;
  if (pairs_out) {
    FILE* f = fopen(pairs_out, "wb");
    if (!f || fwrite(r.pairs, 8, r.pairs_len, f) != r.pairs_len) {
      fprintf(stderr, "error: cannot write %s\n", pairs_out);
      rc = 1;
    }
    if (f) fclose(f);
  }
  mistic_result_free(&r);
  mistic_destroy(h);
  mistic_free_host(pts);
  return rc;
}
