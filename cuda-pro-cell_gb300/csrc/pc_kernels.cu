// sm_103a kernels of the proliferation path: the wide key layout (trees deeper than 32
// generations) in the default configuration, the diagnostics, and the dispatch over all
// compiled configurations. The narrow layout's tuned configurations are instantiated in
// pc_tuned_plain.cu and pc_tuned_batched.cu, which compile in parallel with this file.
#include "pc_sweeps.cuh"

namespace pc {

namespace {

// ------------------------------------------------------------------ diagnostics -----
__global__ void k_debug_philox(const uint32_t* ctr, uint64_t n, uint32_t k0, uint32_t k1,
                               uint32_t* out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const u32x4 r = philox(u32x4{ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]}, k0, k1);
  out[4 * i] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
}

__global__ void k_debug_normals(const ZigTables* zig, uint32_t k0, uint32_t k1, uint32_t root,
                                uint64_t first_parent, uint64_t count, float* z) {
  __shared__ ZigTables Z;
  for (uint32_t i = threadIdx.x; i < sizeof(ZigTables) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(&Z)[i] = reinterpret_cast<const uint32_t*>(zig)[i];
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint64_t parent = first_parent + i / 2;
  const uint32_t c = (uint32_t)(i & 1u);
  const u32x4 P = philox(u32x4{(uint32_t)parent, (uint32_t)(parent >> 32), root, kPurposePair}, k0, k1);
  ChildStream cs = child_stream(2ull * parent + c, root, k0, k1);
  uint32_t budget = kRoundBudget;
  z[i] = zig_normal(c ? P.y : P.x, pair_layer(P, c), true, pair_wedge_bits(P, c), cs, Z, budget);
}

// Grid barriers of the persistent driver, for the failure-detection tests. mode 0: one
// barrier. mode 1: the host presets the arrival counter far above the grid size, so no
// block is ever the last to arrive (a flag that nothing sets) and every block's wait runs
// into the timeout, sets error bit 2 and returns. mode 2: two barriers; block 1 skips the
// second, which can then never complete; block 0 waits there with timeout_ns and every
// other block with long_ns, so they can only leave early by seeing block 0's error bit.
__global__ void k_barrier_probe(uint32_t* bar, unsigned long long timeout_ns, unsigned long long long_ns,
                                uint32_t* error, uint32_t* passed, int mode) {
  if (mode != 2) {
    if (grid_barrier(bar, timeout_ns, error) && threadIdx.x == 0) atomicAdd(passed, 1u);
    return;
  }
  if (!grid_barrier(bar, timeout_ns, error)) return;
  if (blockIdx.x == 1) return;
  if (grid_barrier(bar, blockIdx.x == 0 ? timeout_ns : long_ns, error) && threadIdx.x == 0) atomicAdd(passed, 1u);
}

// Throughput probes for the roofline denominators (FP64 and FP32 fused multiply-add, INT32
// multiply-add). Each thread runs 8 independent dependent chains, so with a few blocks per
// SM the pipe, not the latency, bounds the launch. The chains converge to a fixed point
// (no overflow, no subnormals); the sum is written only if it is impossible, which keeps
// the loop from being optimised away.
template <int Kind>
__global__ void __launch_bounds__(256) k_peak(uint32_t iters, double* sink) {
  constexpr int kChains = 8;
  double acc = 0.0;
  if constexpr (Kind == 0) {
    double a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = 1.0 + 1e-7 * i + 1e-9 * threadIdx.x;
    const double b = 0.9999999, c = 1e-7;
    for (uint32_t it = 0; it < iters; ++it)
#pragma unroll
      for (int i = 0; i < kChains; ++i) a[i] = fma(a[i], b, c);
#pragma unroll
    for (int i = 0; i < kChains; ++i) acc += a[i];
  } else if constexpr (Kind == 1) {
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = 1.0f + 1e-3f * i + 1e-6f * threadIdx.x;
    const float b = 0.999f, c = 1e-3f;
    for (uint32_t it = 0; it < iters; ++it)
#pragma unroll
      for (int i = 0; i < kChains; ++i) a[i] = __fmaf_rn(a[i], b, c);
#pragma unroll
    for (int i = 0; i < kChains; ++i) acc += a[i];
  } else {
    uint32_t a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) a[i] = threadIdx.x + 977u * i;
    // inline PTX, so that the compiler cannot fold the chain of multiply-adds
    for (uint32_t it = 0; it < iters; ++it)
#pragma unroll
      for (int i = 0; i < kChains; ++i)
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(0x9E3779B9u), "r"((uint32_t)i));
    uint32_t x = 0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) x ^= a[i];
    if (x == iters + 0x5EEDu) sink[threadIdx.x] = (double)x;  // not provably false: keeps the chain
  }
  if (acc == -1.0) sink[threadIdx.x] = acc;
}

// One instance's leaf counts merged into its output value histogram: thread (g, b) reads the
// nt counts of bin b at generation g (row g of the plan's [generation][class] table, classes
// from class_begin, b-major), adds them to per_type[v][file type] and their sum to totals[v],
// v = vidx[b][g] the index of the bin's value halved g times in the value set. A nonzero count
// with no value (v < 0, which the leaf rule never produces) sets bit 0 of *error.
__global__ void __launch_bounds__(256) k_merge_counts(const unsigned long long* __restrict__ h, uint64_t nclass,
                                                      uint64_t class_begin, uint32_t hist_gens, uint32_t nb,
                                                      uint32_t nt, const int32_t* __restrict__ vidx,
                                                      uint32_t vidx_stride, const uint32_t* __restrict__ s2f,
                                                      unsigned long long* __restrict__ totals,
                                                      unsigned long long* __restrict__ per_type, uint32_t* error) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)hist_gens * nb) return;
  const uint32_t g = (uint32_t)(i / nb), b = (uint32_t)(i % nb);
  const unsigned long long* row = h + (uint64_t)g * nclass + class_begin + (uint64_t)b * nt;
  const int32_t v = vidx[(uint64_t)b * vidx_stride + g];
  unsigned long long sum = 0ull;
  for (uint32_t k = 0; k < nt; ++k) {
    const unsigned long long c = row[k];
    if (c == 0ull) continue;
    if (v < 0) {
      atomicOr(error, 1u);
      continue;
    }
    atomicAdd(per_type + (uint64_t)v * nt + s2f[k], c);
    sum += c;
  }
  if (sum != 0ull) atomicAdd(totals + v, sum);
}

}  // namespace

int launch_merge_counts(const unsigned long long* hist, uint64_t nclass, uint64_t class_begin, uint32_t hist_gens,
                        uint32_t nb, uint32_t nt, const int32_t* vidx, uint32_t vidx_stride, const uint32_t* s2f,
                        unsigned long long* totals, unsigned long long* per_type, uint32_t* error, void* stream) {
  const uint64_t n = (uint64_t)hist_gens * nb;
  if (n == 0 || nt == 0) return 0;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_merge_counts<<<blocks, 256, 0, (cudaStream_t)stream>>>(hist, nclass, class_begin, hist_gens, nb, nt, vidx,
                                                             vidx_stride, s2f, totals, per_type, error);
  return (int)cudaGetLastError();
}

int launch_peak_probe(int kind, uint32_t iters, int blocks, double* sink, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (kind == 0)
    k_peak<0><<<blocks, 256, 0, st>>>(iters, sink);
  else if (kind == 1)
    k_peak<1><<<blocks, 256, 0, st>>>(iters, sink);
  else
    k_peak<2><<<blocks, 256, 0, st>>>(iters, sink);
  return (int)cudaGetLastError();
}

int launch_barrier_probe(uint32_t* bar, unsigned long long timeout_ns, unsigned long long long_ns, uint32_t* error,
                         uint32_t* passed, int mode, int blocks, void* stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(128u);
  cfg.stream = (cudaStream_t)stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return (int)cudaLaunchKernelEx(&cfg, k_barrier_probe, bar, timeout_ns, long_ns, error, passed, mode);
}

// Narrow-layout tables (pc_tuned_plain.cu, pc_tuned_batched.cu).
const SweepKernels& tuned_plain(int config);
const SweepKernels& tuned_batched(int config);

const SweepKernels& sweep_kernels(bool narrow, bool batched, int config) {
  if (config < 0 || config >= kNumSweepConfigs) config = kDefaultSweepConfig;
  if (narrow) return batched ? tuned_batched(config) : tuned_plain(config);
  static const SweepKernels wide_plain = make_kernels<false, false, DefaultCfg>();
  static const SweepKernels wide_batched = make_kernels<false, true, DefaultCfg>();
  return batched ? wide_batched : wide_plain;
}

int launch_root_sweep(const RunArgs& a, uint64_t root_lo, uint64_t root_hi, const LevelOut& out,
                      int blocks, bool narrow, void* stream) {
  return sweep_kernels(narrow, a.btypes != nullptr, kDefaultSweepConfig).roots(a, root_lo, root_hi, out, blocks, stream);
}

int launch_divide_sweep(const RunArgs& a, const LevelIn& in, uint32_t gen, const LevelOut& out,
                        int blocks, bool narrow, void* stream) {
  return sweep_kernels(narrow, a.btypes != nullptr, kDefaultSweepConfig).divide(a, in, gen, out, blocks, stream);
}

int launch_debug_philox(const uint32_t* ctr, uint64_t n, uint32_t k0, uint32_t k1, uint32_t* out,
                        void* stream) {
  if (n == 0) return 0;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_debug_philox<<<blocks, 256, 0, (cudaStream_t)stream>>>(ctr, n, k0, k1, out);
  return (int)cudaGetLastError();
}

int launch_debug_normals(const ZigTables* zig, uint32_t k0, uint32_t k1, uint32_t root,
                         uint64_t first_parent, uint64_t count, float* z, void* stream) {
  if (count == 0) return 0;
  const unsigned blocks = (unsigned)((count + 255) / 256);
  k_debug_normals<<<blocks, 256, 0, (cudaStream_t)stream>>>(zig, k0, k1, root, first_parent, count, z);
  return (int)cudaGetLastError();
}

// Resident blocks per SM of the default configuration's sweeps (the smaller over the
// narrow/wide and plain/batched instantiations).
int occupancy_blocks_per_sm(int* root_blocks, int* divide_blocks) {
  int r = 1 << 30, d = 1 << 30;
  for (int narrow = 0; narrow < 2; ++narrow)
    for (int batched = 0; batched < 2; ++batched) {
      int rr = 0, dd = 0, pp = 0;
      const int e = sweep_kernels(narrow != 0, batched != 0, kDefaultSweepConfig).occupancy(&rr, &dd, &pp);
      if (e != 0) return e;
      r = std::min(r, rr);
      d = std::min(d, dd);
    }
  *root_blocks = r;
  *divide_blocks = d;
  return 0;
}

}  // namespace pc
