// The engine's normal sampler (csrc/pc_rng.h, which the kernels compile for the device)
// compiled for the host, for tests/test_host_sampler.py: the first-attempt pair-block draw,
// the ziggurat with its wedge and tail steps and the node's private stream, exactly as
// k_debug_normals evaluates them, over the engine's own tables (pc::host_zig_tables).
#include <stdint.h>

#include "pc_rng.h"

namespace pc {
ZigTables host_zig_tables();
}

extern "C" int host_normals(uint64_t seed, uint32_t root, uint64_t first_parent, uint64_t count, float* z) {
  static const pc::ZigTables Z = pc::host_zig_tables();
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (uint64_t i = 0; i < count; ++i) {
    const uint64_t parent = first_parent + i / 2;
    const uint32_t c = (uint32_t)(i & 1u);
    const pc::u32x4 P = pc::philox(pc::u32x4{(uint32_t)parent, (uint32_t)(parent >> 32), root, pc::kPurposePair}, k0, k1);
    pc::ChildStream cs = pc::child_stream(2ull * parent + c, root, k0, k1);
    uint32_t budget = 1u << 16;
    z[i] = pc::zig_normal(c ? P.y : P.x, pc::pair_layer(P, c), true, pc::pair_wedge_bits(P, c), cs, Z, budget);
    if (budget == 0u) return 1;
  }
  return 0;
}
