// The reference's file formats (src/io/parser.cu:68-217), exposed through the C ABI.
//
// Histogram rows are `<value> <frequency>` and cell types `<ratio> <mean> <stddev>`, read
// with `std::istream >> double >> uint64_t` exactly as the reference does, so parsing stops
// at the first token that does not convert. The output is written with an
// std::ostream at precision(10) in the default float format, tab separated, one row per
// value with a nonzero total, followed by std::endl (parser.cu:187-217).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <new>
#include <fstream>
#include <iostream>
#include <vector>

#include "../../include/procell.h"
#include "pc_guard.h"

extern "C" {

int pc_load_histogram(const char* path, pc_bin** out, uint64_t* n) {
  PC_GUARD_BEGIN
  if (!path || !out || !n) return PC_ERR_INVALID;
  *out = nullptr;
  *n = 0;
  std::ifstream in(path);
  if (!in.is_open()) return PC_ERR_IO;
  std::vector<pc_bin> rows;
  double value = 0.0;
  uint64_t frequency = 0;
  while (in >> value >> frequency) rows.push_back(pc_bin{value, frequency});
  *out = (pc_bin*)std::malloc((rows.size() ? rows.size() : 1) * sizeof(pc_bin));
  if (!*out) return PC_ERR_NOMEM;
  for (size_t i = 0; i < rows.size(); ++i) (*out)[i] = rows[i];
  *n = rows.size();
  return PC_OK;
  PC_GUARD_END_NOCTX
}

int pc_load_cell_types(const char* path, pc_cell_type** out, uint32_t* n) {
  PC_GUARD_BEGIN
  if (!path || !out || !n) return PC_ERR_INVALID;
  *out = nullptr;
  *n = 0;
  std::ifstream in(path);
  if (!in.is_open()) return PC_ERR_IO;
  std::vector<pc_cell_type> rows;
  double ratio = 0.0, mean = 0.0, sd = 0.0;
  while (in >> ratio >> mean >> sd) rows.push_back(pc_cell_type{ratio, mean, sd});
  // assert_proportion_sum (parser.cu:46-66): the ratios must sum to 1 within 1e-8.
  double sum = 0.0;
  for (const auto& r : rows) sum += r.ratio;
  *out = (pc_cell_type*)std::malloc((rows.size() ? rows.size() : 1) * sizeof(pc_cell_type));
  if (!*out) return PC_ERR_NOMEM;
  for (size_t i = 0; i < rows.size(); ++i) (*out)[i] = rows[i];
  *n = (uint32_t)rows.size();
  if (std::abs(1.0 - sum) > 1e-8) {
    std::free(*out);
    *out = nullptr;
    *n = 0;
    return PC_ERR_INVALID;
  }
  return PC_OK;
  PC_GUARD_END_NOCTX
}

static void write_rows(std::ostream& stream, const pc_histogram* h, int track_ratio) {
  stream.precision(10);
  for (uint64_t i = 0; i < h->n_values; ++i) {
    if (h->totals[i] == 0) continue;
    stream << h->values[i] << "\t" << h->totals[i];
    if (track_ratio)
      for (uint32_t k = 0; k < h->n_types; ++k) stream << "\t" << h->per_type[i * h->n_types + k];
    stream << std::endl;
  }
}

int pc_write_histogram(const char* path, const pc_histogram* h, int track_ratio) {
  PC_GUARD_BEGIN
  if (!h) return PC_ERR_INVALID;
  if (!path || (path[0] == '-' && path[1] == '\0')) {
    write_rows(std::cout, h, track_ratio);
    std::cout.flush();
    return std::cout.good() ? PC_OK : PC_ERR_IO;
  }
  std::ofstream stream(path);
  if (!stream.is_open()) return PC_ERR_IO;
  write_rows(stream, h, track_ratio);
  stream.close();
  return stream.fail() ? PC_ERR_IO : PC_OK;
  PC_GUARD_END_NOCTX
}

void pc_free(void* p) { std::free(p); }

// Logarithmic bin edges as the reference's utils::log_space (src/utils/util.cu:90-111):
// exponents ceil(log_base(start)) .. ceil(log_base(end)) in n equally spaced steps (its
// linear_space, util.cu:76-88), each edge base^exponent, the last one exactly base^end.
int pc_log_space(double start, double end, uint64_t n, double base, double* edges) {
  PC_GUARD_BEGIN
  if (!edges || n < 2 || !(start > 0.0) || !(end > 0.0) || !(base > 0.0) || base == 1.0 ||
      !std::isfinite(start) || !std::isfinite(end) || !std::isfinite(base))
    return PC_ERR_INVALID;
  const double e0 = std::ceil(std::log(start) / std::log(base));
  const double e1 = std::ceil(std::log(end) / std::log(base));
  const double delta = (e1 - e0) / (double)(n - 1);
  for (uint64_t i = 0; i + 1 < n; ++i) edges[i] = std::pow(base, e0 + delta * (double)i);
  edges[n - 1] = std::pow(base, e1);
  return PC_OK;
  PC_GUARD_END_NOCTX
}

// The reference's utils::rebin (util.cu:113-138): counts of an ascending histogram summed
// into the bins of log_space(lower, upper, n_bins, 10), a value landing in the first bin
// whose edge is >= the value. The reference walks past its array for values above the
// last edge; here that is an error.
int pc_rebin(const double* values, const uint64_t* counts, uint64_t n_values, double lower, double upper,
             uint64_t n_bins, double* edges_out, uint64_t* counts_out) {
  PC_GUARD_BEGIN
  if ((n_values && (!values || !counts)) || !edges_out || !counts_out) return PC_ERR_INVALID;
  const int rc = pc_log_space(lower, upper, n_bins, 10.0, edges_out);
  if (rc != PC_OK) return rc;
  for (uint64_t i = 0; i < n_bins; ++i) counts_out[i] = 0;
  uint64_t pos = 0;
  for (uint64_t i = 0; i < n_values; ++i) {
    if (i > 0 && values[i] < values[i - 1]) return PC_ERR_INVALID;  // not ascending
    while (pos < n_bins && values[i] > edges_out[pos]) ++pos;
    if (pos == n_bins) return PC_ERR_INVALID;  // above the last edge
    counts_out[pos] += counts[i];
  }
  return PC_OK;
  PC_GUARD_END_NOCTX
}

}  // extern "C"
