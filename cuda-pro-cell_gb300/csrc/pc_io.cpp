// The reference's file formats (src/io/parser.cu:68-217), exposed through the C ABI.
//
// Histogram rows are `<value> <frequency>` and cell types `<ratio> <mean> <stddev>`, read
// with `std::istream >> double >> uint64_t` exactly as the reference does, so parsing stops
// at the first token that does not convert. The output is written with an
// std::ostream at precision(10) in the default float format, tab separated, one row per
// value with a nonzero total, followed by std::endl (parser.cu:187-217).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "../../include/procell.h"

extern "C" {

int pc_load_histogram(const char* path, pc_bin** out, uint64_t* n) {
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
}

int pc_load_cell_types(const char* path, pc_cell_type** out, uint32_t* n) {
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
}

void pc_free(void* p) { std::free(p); }

}  // extern "C"
