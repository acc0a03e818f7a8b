// The engine's root chunk and key layout (pc::key_layout) and output value set
// (pc::host_value_set), host functions exported by libprocell.so, for
// tests/test_key_layout.py.
#include <stdint.h>

#include "procell.h"

namespace pc {
struct KeyLayout {
  uint64_t chunk;
  uint32_t g_store_max;
  bool narrow;
};
KeyLayout key_layout(uint64_t roots, uint32_t gmax, bool batched, uint64_t max_root_chunk);
}

extern "C" void layout(uint64_t roots, uint32_t gmax, int batched, uint64_t max_root_chunk, uint64_t* chunk,
                       uint32_t* g_store_max, int* narrow) {
  const pc::KeyLayout k = pc::key_layout(roots, gmax, batched != 0, max_root_chunk);
  *chunk = k.chunk;
  *g_store_max = k.g_store_max;
  *narrow = k.narrow ? 1 : 0;
}

namespace pc {
int host_value_set(const ::pc_bin* bins, uint64_t n_bins, double phi, double* values, uint64_t capacity,
                   uint64_t* n_values);
}

extern "C" int value_set(const pc_bin* bins, uint64_t n_bins, double phi, double* values, uint64_t capacity,
                         uint64_t* n_values) {
  return pc::host_value_set(bins, n_bins, phi, values, capacity, n_values);
}
