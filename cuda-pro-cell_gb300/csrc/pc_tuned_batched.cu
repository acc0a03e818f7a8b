// The batched form's sweeps on the narrow key layout, in every tuned configuration
// (threads per block x cells per lane x leaf-count privatisation; see pc_sweeps.cuh).
#include "pc_sweeps.cuh"

namespace pc {

const SweepKernels& tuned_batched(int config) { return tuned_kernels<true, true>(config); }

}  // namespace pc
