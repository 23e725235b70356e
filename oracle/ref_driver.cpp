// Driver for the reference's own CPU brute force (src/utils.cu:285-317 of
// bwd29/self-join-MiSTIC), compiled from the unmodified reference source by
// oracle/build_ref.sh.  It reads a raw FP64 row-major point file the way the
// reference's main does (src/main.cu:42-50), calls brute_force, and prints
// one JSON line.  Test infrastructure only: used to pin the oracle.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>
#include <omp.h>

unsigned int brute_force(unsigned int num_points, unsigned int dim, double epsilon, double* A);

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s <file.bin> <dim> <epsilon>\n", argv[0]);
    return 2;
  }
  unsigned dim = (unsigned)atoi(argv[2]);
  double eps = 0;
  sscanf(argv[3], "%lf", &eps);
  std::ifstream f(argv[1], std::ios::in | std::ios::binary);
  f.seekg(0, std::ios::end);
  size_t size = (size_t)f.tellg();
  f.seekg(0, std::ios::beg);
  std::vector<char> buf(size);
  f.read(buf.data(), size);
  unsigned n = (unsigned)(size / sizeof(double) / dim);
  double t0 = omp_get_wtime();
  unsigned cnt = brute_force(n, dim, eps, reinterpret_cast<double*>(buf.data()));
  double t1 = omp_get_wtime();
  fprintf(stdout, "{\"n\": %u, \"d\": %u, \"ordered_incl_self\": %u, \"seconds\": %.3f, \"threads\": %d}\n",
          n, dim, cnt, t1 - t0, omp_get_max_threads());
  return 0;
}
