// Text -> binary point-file converter.
//
// Reference counterpart: toCSV.cpp:52-85 (the `toBin` tool).  That program
// reads the input with `fscanf("%lf, ")` in a loop: skip white space, read
// a double, optionally consume one ',' (and the white space after it), and
// stop at the first token that does not parse as a number (a header line, a
// ';', a comma preceded by white space ...).  Every value read is written as
// raw little-endian FP64, which is the input format of the reference's main
// (src/main.cu:42-50) and of mistic_read_points.
//
// Here the file is read at once and parsed by several host threads.  The
// split points are white-space characters: there the sequential parser is
// always in its "skip white space" state, so every chunk can be parsed on
// its own; the output is the chunks' values in order, up to and including
// the values of the first chunk that stopped early.
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mistic.h"

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Parses [b, e) (NUL-terminated at e); returns true if it stopped at a
// token that is not a number before reaching e.
bool parse_chunk(const char* b, const char* e, std::vector<double>& out) {
  const char* p = b;
  for (;;) {
    while (p < e && is_space(*p)) ++p;
    if (p >= e) return false;
    char* q = nullptr;
    const double v = strtod(p, &q);
    if (q == p || q > e) return true;
    out.push_back(v);
    p = q;
    if (p < e && *p == ',') ++p;
  }
}

}  // namespace

extern "C" mistic_status mistic_convert_text(const char* text_path, const char* bin_path, uint64_t* out_count) {
  if (out_count) *out_count = 0;
  if (!text_path || !bin_path) return MISTIC_ERR_INVALID_ARG;
  std::ifstream f(text_path, std::ios::in | std::ios::binary);
  if (!f) return MISTIC_ERR_IO;
  f.seekg(0, std::ios::end);
  const std::streamoff size = f.tellg();
  if (size < 0) return MISTIC_ERR_IO;
  f.seekg(0, std::ios::beg);
  std::string buf;
  try {
    buf.resize((size_t)size + 1);
  } catch (...) {
    return MISTIC_ERR_OUT_OF_MEMORY;
  }
  if (size && !f.read(&buf[0], size)) return MISTIC_ERR_IO;
  buf[(size_t)size] = '\0';
  const char* data = buf.data();
  const size_t n = (size_t)size;

  // chunk boundaries at white space, about 8 MB apart
  const unsigned threads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  const size_t want = std::max<size_t>(1, std::min<size_t>(threads * 4, n / (8u << 20) + 1));
  std::vector<size_t> cut{0};
  for (size_t i = 1; i < want; ++i) {
    size_t c = std::max(cut.back(), n * i / want);
    while (c < n && !is_space(data[c])) ++c;
    if (c < n && c > cut.back()) cut.push_back(c);
  }
  cut.push_back(n);
  const size_t nch = cut.size() - 1;
  std::vector<std::vector<double>> vals(nch);
  std::vector<char> stopped(nch, 0);
  std::vector<std::thread> pool;
  std::vector<std::string> owned(nch);
  auto work = [&](size_t t0) {
    for (size_t c = t0; c < nch; c += threads) {
      // a NUL-terminated copy of the chunk keeps strtod inside it
      owned[c].assign(data + cut[c], data + cut[c + 1]);
      const char* b = owned[c].c_str();
      stopped[c] = parse_chunk(b, b + owned[c].size(), vals[c]) ? 1 : 0;
      std::string().swap(owned[c]);
    }
  };
  for (unsigned t = 0; t < std::min<size_t>(threads, nch); ++t) pool.emplace_back(work, t);
  for (auto& t : pool) t.join();

  FILE* o = fopen(bin_path, "wb");
  if (!o) return MISTIC_ERR_IO;
  uint64_t total = 0;
  for (size_t c = 0; c < nch; ++c) {
    if (!vals[c].empty() && fwrite(vals[c].data(), sizeof(double), vals[c].size(), o) != vals[c].size()) {
      fclose(o);
      return MISTIC_ERR_IO;
    }
    total += vals[c].size();
    if (stopped[c]) break;
  }
  if (fclose(o) != 0) return MISTIC_ERR_IO;
  if (out_count) *out_count = total;
  return MISTIC_OK;
}
