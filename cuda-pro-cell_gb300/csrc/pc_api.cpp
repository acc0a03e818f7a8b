// Host side of libprocell: the C ABI of include/procell.h.
//
// pc_plan_create restates the host part of the reference's pipeline once per input:
// the output value set and bin layout of io::load_fluorescences (src/io/parser.cu:68-154),
// the type table of io::load_cell_types (parser.cu:156-185), and the per-bin "phi cap"
// that the division test `fluorescence / 2 > threshold` (proliferation.cu:323) implies.
// pc_plan_run replaces simulation::proliferate's host loop (proliferation.cu:26-215):
// instead of allocating every tree level at full size and recursing on the device, it
// runs one root sweep per chunk of initial cells and then one division sweep per
// generation slice, depth-first over a stack of level buffers whose size is fixed by a
// memory budget, so the peak footprint is bounded and independent of the tree shape.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <new>
#include <cstring>
#include <atomic>
#include <chrono>
#include <map>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/procell.h"
#include "pc_guard.h"
#include "pc_engine.h"

using namespace pc;

struct LevelBuf {
  ulonglong2* cells = nullptr;
  unsigned long long* count = nullptr;
  unsigned long long* prefix = nullptr;
  uint32_t* ticket = nullptr;
  bool busy = false;
};

struct pc_context {
  // a device buffer kept for reuse
  struct Spare {
    void* p = nullptr;
    size_t bytes = 0;
  };
  static constexpr int kSpares = 2;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  int sms = 0, root_bps = 0, div_bps = 0;
  double opt_budget = 0.0;
  uint64_t opt_max_slice = 0, opt_max_root_chunk = 0;
  int opt_grid_blocks = 0;
  int opt_config = kDefaultSweepConfig;  // sweep configuration (narrow key layout)
  int opt_driver = 0;                    // 0: one launch per sweep, 1: persistent launch
  int opt_graph = 0;                     // persistent driver: replay a captured CUDA graph
  int opt_smooth_predraw = 1;            // smoothed plans keep their lineages' draws in HBM
  int opt_device_merge = 1;              // single-instance results merged on the device
  uint32_t opt_batch_parts = 4;          // pc_simulate_batch: sub-batches at most
  // resident blocks per SM of each configuration's kernels: [narrow][batched][config]
  int occ[2][2][kNumSweepConfigs][3] = {};
  uint32_t* persist_ctl = nullptr;       // [2] barrier + [8] run totals (u64 [4])
  // the two large per-plan device buffers (root records, count table) of destroyed plans,
  // kept for the next plans of this context: two of each kind, the largest (the consecutive
  // sub-batches of pc_simulate_batch alternate between two live plans)
  Spare spare_rec[kSpares], spare_hist[kSpares];
  Spare spare_tables[kSpares];  // ... and of their small tables (one allocation per plan)
  std::vector<pc_plan*> live;  // plans created on this context and not yet destroyed
  // pinned host copy of the last count table read back (plan id and run number it holds)
  unsigned long long* stage = nullptr;
  size_t stage_elems = 0;
  uint64_t stage_plan = 0, stage_run = 0;
  // a second pinned count table: pc_simulate_batch reads one sub-batch's table back while
  // host threads merge the previous one's
  unsigned long long* stage2 = nullptr;
  size_t stage2_elems = 0;
  // the device merge of a plan's result: device scratch (value map, type order, merged
  // counts) and the pinned copy of the merged counts, both grown on demand
  void* merge_dev = nullptr;
  size_t merge_dev_bytes = 0;
  unsigned long long* merge_host = nullptr;
  size_t merge_host_bytes = 0;
  ZigTables zig_host;
  ZigTables* zig_dev = nullptr;
  std::vector<LevelBuf> pool;
  uint64_t pool_cells = 0;   // capacity of each pool buffer (cells)
  uint32_t pool_segs = 0;    // segments each buffer's count/prefix arrays hold
  unsigned long long* stats_dev = nullptr;  // [4]
  uint32_t* error_dev = nullptr;
  unsigned long long* pinned = nullptr;     // host staging for small reads
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // pc_simulate_batch: count tables copied back on a second stream while the next part runs
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_done[2] = {nullptr, nullptr};
  uint64_t free_at_start = 0;
  // host-side fault injection (option fail_nth_call): CUDA calls the library made for this
  // context, the call number that fails next (0: none) and the failures injected so far
  uint64_t cuda_calls = 0, fail_at = 0, faults_injected = 0;
};

// One simulation input: a histogram, a type set, t_max, phi and a seed, prepared once.
struct InstanceHost {
  std::vector<double> bin_value;  // nonzero bins, file order
  std::vector<uint64_t> bin_freq;
  std::vector<uint32_t> cap;      // phi cap per bin: generations a lineage may divide
  std::vector<double> values;     // output value set, ascending
  std::vector<TypeDev> types;     // sorted by ratio, descending
  std::vector<uint32_t> sorted_to_file;
  uint32_t fallback = 0, gmax = 0;
  double t_max = 0.0, phi = 0.0;
  uint64_t seed = 0, roots = 0;
  // placement in the plan
  uint64_t root_begin = 0, class_begin = 0;
  uint32_t bin_begin = 0, type_begin = 0, hist_gens = 1;
  uint32_t vidx_stride = 1;   // gmax + 1
  std::vector<int32_t> vidx;  // [nbins][vidx_stride] -> output value index or -1
};

struct pc_plan {
  std::vector<InstanceHost> inst;  // one for pc_plan_create, many for pc_batch_create
  bool batched = false;
  std::vector<uint64_t> bin_start;  // [nbins + 1] over all instances' bins
  std::vector<uint32_t> bin_info;
  uint32_t nbins = 0, gmax = 0, hist_gens = 1, g_store_max = 0;
  uint64_t nclass = 0;
  uint64_t roots_total = 0, root_begin = 0, root_end = 0, chunk = 1;
  TypeDev* types_dev = nullptr;         // plain form
  BatchType* btypes_dev = nullptr;      // batched form
  InstanceDev* inst_dev = nullptr;
  uint32_t* bin_inst_dev = nullptr;
  uint32_t* bin_class_dev = nullptr;
  uint32_t* bin_info_dev = nullptr;
  uint64_t* bin_start_dev = nullptr;
  void* tables_dev = nullptr;           // the tables above, one allocation
  size_t tables_bytes = 0;
  unsigned long long* root_rec_dev = nullptr;
  unsigned long long* hist_dev = nullptr;
  size_t hist_elems = 0;
  uint64_t id = 0, run_id = 0;                // identity of the counts in the pinned stage
  pc_context* owner = nullptr;                // receives the large buffers on destroy
  size_t rec_bytes = 0, hist_bytes = 0;
  cudaGraphExec_t graph = nullptr;           // persistent driver: the captured run
  PersistArgs graph_args;                    // ... and the arguments it was captured with
  int graph_config = -1, graph_grid = 0;
  pc_stats stats;
  uint64_t upload_bytes = 0;
  bool ran = false;
};

struct pc_batch : pc_plan {};

namespace {

thread_local std::string g_create_error;

int fail(pc_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define PC_CUDA(ctx, call)                                                                    \
  do {                                                                                        \
    cudaError_t e__ = (call);                                                                 \
    if (e__ != cudaSuccess)                                                                   \
      return fail((ctx), e__ == cudaErrorMemoryAllocation ? PC_ERR_NOMEM : PC_ERR_CUDA,       \
                  std::string(#call) + ": " + cudaGetErrorString(e__));                       \
  } while (0)

// ---- Host-side fault injection -----------------------------------------------------------
// Every allocation, copy, memset, synchronisation, event record and kernel or graph launch
// this file makes goes through the wrappers below. Inside an entry point that names its
// context (FaultScope), each counts as one call of that context; when the option
// fail_nth_call = n is set, call n from then on does not reach CUDA and returns an error
// instead (cudaErrorMemoryAllocation for allocations, cudaErrorLaunchOutOfResources for
// launches, cudaErrorInvalidValue otherwise), once. Live device allocations are counted
// process-wide, so tests can check that a failed call leaks nothing.
thread_local pc_context* t_fault_ctx = nullptr;
std::atomic<long long> g_live_device_allocs{0};

struct FaultScope {
  pc_context* prev;
  explicit FaultScope(pc_context* c) : prev(t_fault_ctx) { t_fault_ctx = c; }
  ~FaultScope() { t_fault_ctx = prev; }
};

cudaError_t injected(cudaError_t code) {
  pc_context* c = t_fault_ctx;
  if (!c) return cudaSuccess;
  ++c->cuda_calls;
  if (c->fail_at != 0 && c->cuda_calls == c->fail_at) {
    c->fail_at = 0;
    ++c->faults_injected;
    return code;
  }
  return cudaSuccess;
}

template <class T>
cudaError_t pc_cuda_malloc(T** p, size_t bytes) {
  if (cudaError_t f = injected(cudaErrorMemoryAllocation)) return f;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) ++g_live_device_allocs;
  return e;
}
cudaError_t pc_cuda_free(void* p) {
  if (p) --g_live_device_allocs;
  return cudaFree(p);
}
template <class T>
cudaError_t pc_cuda_malloc_host(T** p, size_t bytes) {
  if (cudaError_t f = injected(cudaErrorMemoryAllocation)) return f;
  return cudaMallocHost(p, bytes);
}
cudaError_t pc_cuda_copy(void* dst, const void* src, size_t n, cudaMemcpyKind k, cudaStream_t s) {
  if (cudaError_t f = injected(cudaErrorInvalidValue)) return f;
  return cudaMemcpyAsync(dst, src, n, k, s);
}
cudaError_t pc_cuda_copy_sync(void* dst, const void* src, size_t n, cudaMemcpyKind k) {
  if (cudaError_t f = injected(cudaErrorInvalidValue)) return f;
  return cudaMemcpy(dst, src, n, k);
}
cudaError_t pc_cuda_memset(void* p, int v, size_t n, cudaStream_t s) {
  if (cudaError_t f = injected(cudaErrorInvalidValue)) return f;
  return cudaMemsetAsync(p, v, n, s);
}
cudaError_t pc_cuda_sync(cudaStream_t s) {
  if (cudaError_t f = injected(cudaErrorInvalidValue)) return f;
  return cudaStreamSynchronize(s);
}
cudaError_t pc_cuda_event_record(cudaEvent_t e, cudaStream_t s) {
  if (cudaError_t f = injected(cudaErrorInvalidValue)) return f;
  return cudaEventRecord(e, s);
}
cudaError_t pc_cuda_graph_launch(cudaGraphExec_t g, cudaStream_t s) {
  if (cudaError_t f = injected(cudaErrorLaunchOutOfResources)) return f;
  return cudaGraphLaunch(g, s);
}
// A kernel launch through one of the launch functions (they return a cudaError_t as int);
// an injected failure skips the launch.
#define PC_LAUNCH(expr) \
  (injected(cudaErrorLaunchOutOfResources) != cudaSuccess ? cudaErrorLaunchOutOfResources : (cudaError_t)(expr))

// Ziggurat tables for f(x) = exp(-x^2/2), kZigLayers layers (Marsaglia & Tsang 2000): the layer
// edges follow x_{i+1} = sqrt(-2 ln(v/x_i + f(x_i))) from x_1 = r; the base strip's
// effective width is v/f(r).
ZigTables build_zig_tables() {
  const double r = kZigR, v = kZigV, scale = 2147483648.0;
  double x[kZigLayers + 1];
  x[1] = r;
  for (int i = 1; i + 1 < kZigLayers; ++i) {
    const double fx = std::exp(-0.5 * x[i] * x[i]);
    x[i + 1] = std::sqrt(-2.0 * std::log(v / x[i] + fx));
  }
  x[kZigLayers] = 0.0;
  const double base = v / std::exp(-0.5 * r * r);
  ZigTables t;
  t.k[0] = (uint32_t)std::floor(r / base * scale);
  t.w[0] = (float)(base / scale);
  t.f[0] = 0.0f;
  for (int i = 1; i < kZigLayers; ++i) {
    t.k[i] = (uint32_t)std::floor(x[i + 1] / x[i] * scale);
    t.w[i] = (float)(x[i] / scale);
    t.f[i] = (float)std::exp(-0.5 * x[i] * x[i]);
  }
  t.f[kZigLayers] = 1.0f;
  return t;
}

// Smallest (sigma > 0) or largest (sigma < 0) FP32 z with fma(sigma, z, mu) > 0: the
// truncation tau > 0 of determine_cell_timer (cell.cu:114-118) as an FP32 test on z.
void truncation_bounds(double mu, double sigma, float& zlo, float& zhi) {
  const float inf = INFINITY;
  zlo = -inf;
  zhi = inf;
  if (sigma == 0.0) return;
  auto ok = [&](float z) { return std::fma(sigma, (double)z, mu) > 0.0; };
  float z = (float)(-mu / sigma);
  if (std::isnan(z)) z = 0.0f;
  if (sigma > 0.0) {
    for (int i = 0; i < 4096 && std::isfinite(z) && ok(z); ++i) z = std::nextafter(z, -inf);
    for (int i = 0; i < 4096 && !ok(z); ++i) z = std::nextafter(z, inf);
    zlo = z;
  } else {
    for (int i = 0; i < 4096 && std::isfinite(z) && ok(z); ++i) z = std::nextafter(z, inf);
    for (int i = 0; i < 4096 && !ok(z); ++i) z = std::nextafter(z, -inf);
    zhi = z;
  }
}


void free_pool(pc_context* ctx) {
  for (auto& b : ctx->pool) {
    pc_cuda_free(b.cells);
    pc_cuda_free(b.count);
    pc_cuda_free(b.prefix);
    pc_cuda_free(b.ticket);
  }
  ctx->pool.clear();
  ctx->pool_cells = 0;
  ctx->pool_segs = 0;
}

int acquire(pc_context* ctx, int* idx) {
  for (size_t i = 0; i < ctx->pool.size(); ++i) {
    if (!ctx->pool[i].busy) {
      ctx->pool[i].busy = true;
      *idx = (int)i;
      return PC_OK;
    }
  }
  LevelBuf b;
  PC_CUDA(ctx, pc_cuda_malloc(&b.cells, ctx->pool_cells * sizeof(ulonglong2)));
  cudaError_t e = pc_cuda_malloc(&b.count, ctx->pool_segs * sizeof(unsigned long long));
  if (e == cudaSuccess) e = pc_cuda_malloc(&b.prefix, (ctx->pool_segs + 1) * sizeof(unsigned long long));
  if (e == cudaSuccess) e = pc_cuda_malloc(&b.ticket, sizeof(uint32_t));
  if (e == cudaSuccess) e = pc_cuda_memset(b.ticket, 0, sizeof(uint32_t), ctx->stream);
  if (e != cudaSuccess) {
    pc_cuda_free(b.cells);
    pc_cuda_free(b.count);
    pc_cuda_free(b.prefix);
    pc_cuda_free(b.ticket);
    return fail(ctx, PC_ERR_NOMEM, std::string("level buffer allocation: ") + cudaGetErrorString(e));
  }
  b.busy = true;
  ctx->pool.push_back(b);
  *idx = (int)ctx->pool.size() - 1;
  return PC_OK;
}

int max_blocks(const pc_context* ctx, int per_sm) {
  int b = ctx->sms * std::max(1, per_sm);
  if (ctx->opt_grid_blocks > 0) b = std::min(b, ctx->opt_grid_blocks);
  return std::max(1, b);
}

int grid_for(const pc_context* ctx, uint64_t n, int per_sm, int threads) {
  const uint64_t want = (n + (uint64_t)threads * 4 - 1) / ((uint64_t)threads * 4);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)max_blocks(ctx, per_sm)));
}

// A device buffer of at least `need` bytes: the context's spare one when it is large enough,
// else a new allocation.
// The smallest spare of at least `need` bytes, else a new allocation of `need` bytes.
using Spare = pc_context::Spare;
constexpr int kSpares = pc_context::kSpares;

cudaError_t take_spare(Spare* spare, size_t need, void** out, size_t* out_bytes) {
  int best = -1;
  for (int i = 0; i < kSpares; ++i)
    if (spare[i].p && spare[i].bytes >= need && (best < 0 || spare[i].bytes < spare[best].bytes)) best = i;
  if (best >= 0) {
    *out = spare[best].p;
    *out_bytes = spare[best].bytes;
    spare[best] = Spare();
    return cudaSuccess;
  }
  *out_bytes = need;
  return pc_cuda_malloc(out, need);
}

// Keep the kSpares largest of `buf` and the spares, free the rest.
void give_spare(Spare* spare, void* buf, size_t bytes) {
  if (!buf) return;
  int slot = 0;  // an empty slot, else the smallest spare
  for (int i = 0; i < kSpares; ++i) {
    if (!spare[i].p) {
      slot = i;
      break;
    }
    if (spare[i].bytes < spare[slot].bytes) slot = i;
  }
  if (spare[slot].p && spare[slot].bytes >= bytes) {
    pc_cuda_free(buf);
    return;
  }
  pc_cuda_free(spare[slot].p);
  spare[slot].p = buf;
  spare[slot].bytes = bytes;
}

// f(i) for i in [0, n) on up to `threads` host threads (0 = all cores), the calling thread
// among them. A thread that cannot be started leaves its share to the others.
template <class F>
void parallel_for(uint32_t n, F&& f, unsigned threads = 0) {
  unsigned nt = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(std::min<unsigned>(nt, 64u), n);
  if (nt <= 1) {
    for (uint32_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<uint32_t> next{0};
  auto work = [&]() {
    for (uint32_t i; (i = next.fetch_add(1)) < n;) f(i);
  };
  std::vector<std::thread> pool;
  pool.reserve(nt - 1);
  for (unsigned t = 0; t + 1 < nt; ++t) {
    try {
      pool.emplace_back(work);
    } catch (...) {
      break;
    }
  }
  work();
  for (auto& th : pool) th.join();
}

uint32_t bits_for(uint64_t n) {  // bits needed for values in [0, n)
  uint32_t b = 0;
  while (b < 64 && (n - 1) >> b) ++b;
  return n <= 1 ? 0 : b;
}

}  // namespace

namespace pc {
// Host helpers shared with the allocation-free entry point (pc_noalloc.cu).
ZigTables host_zig_tables() { return build_zig_tables(); }

KeyLayout key_layout(uint64_t roots, uint32_t gmax, bool batched, uint64_t max_root_chunk) {
  // key = root_local * 2^g + path must fit 64 bits for every generation a key can have,
  // gmax path bits; the narrow layout (root_local << 32 | heap node 2^g + path) holds
  // generations up to 31 and needs root_local < 2^32
  uint64_t chunk = std::max<uint64_t>(1, roots);
  const uint32_t want_bits = gmax >= 45 ? 20u : 64u - gmax;
  if (want_bits < 64) chunk = std::min<uint64_t>(chunk, 1ull << want_bits);
  if (gmax <= kNarrowMaxGen) chunk = std::min<uint64_t>(chunk, 1ull << 32);
  if (batched) chunk = std::min<uint64_t>(chunk, 1ull << 28);  // 2 GiB of root records
  if (max_root_chunk) chunk = std::min<uint64_t>(chunk, std::max<uint64_t>(1, max_root_chunk));
  KeyLayout k;
  k.chunk = chunk;
  k.g_store_max = std::min<uint32_t>(62u, 63u - bits_for(chunk));  // its daughters' keys fit as well
  k.narrow = gmax <= kNarrowMaxGen;
  return k;
}
void host_truncation_bounds(double mu, double sigma, float& zlo, float& zhi) {
  truncation_bounds(mu, sigma, zlo, zhi);
}
}  // namespace pc

extern "C" {

const char* pc_version(void) { return "procell-gb300 0.1 (sm_103a)"; }

const char* pc_last_error(const pc_context* ctx) {
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

int pc_create(pc_context** out, int device) {
  PC_GUARD_BEGIN
  if (!out) return PC_ERR_INVALID;
  *out = nullptr;
  pc_context* ctx = new (std::nothrow) pc_context();
  if (!ctx) return PC_ERR_NOMEM;
  auto bail = [&](cudaError_t e, const char* what) {
    g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    delete ctx;
    return PC_ERR_CUDA;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bail(e, "cudaSetDevice");
  ctx->device = device;
  e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return bail(e, "cudaDeviceGetAttribute");
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(e, "cudaStreamCreate");
  ctx->stream = ctx->own_stream;
  const int oe = occupancy_blocks_per_sm(&ctx->root_bps, &ctx->div_bps);
  if (oe != 0) return bail((cudaError_t)oe, "occupancy query (is the sm_103a binary loadable?)");
  ctx->zig_host = build_zig_tables();
  if ((e = pc_cuda_malloc(&ctx->zig_dev, sizeof(ZigTables))) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = pc_cuda_copy_sync(ctx->zig_dev, &ctx->zig_host, sizeof(ZigTables), cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(e, "cudaMemcpy");
  if ((e = pc_cuda_malloc(&ctx->stats_dev, 4 * sizeof(unsigned long long))) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = pc_cuda_malloc(&ctx->error_dev, sizeof(uint32_t))) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = pc_cuda_malloc(&ctx->persist_ctl, 48)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = pc_cuda_malloc_host(&ctx->pinned, 64 * sizeof(unsigned long long))) != cudaSuccess)
    return bail(e, "cudaMallocHost");
  for (auto& ev : ctx->ev)
    if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e, "cudaEventCreate");
  size_t fr = 0, tot = 0;
  if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) return bail(e, "cudaMemGetInfo");
  ctx->free_at_start = fr;
  *out = ctx;
  return PC_OK;
  PC_GUARD_END(nullptr)
}

void pc_destroy(pc_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) pc_cuda_sync(ctx->stream);
  if (ctx->copy_stream) pc_cuda_sync(ctx->copy_stream);
  free_pool(ctx);
  for (pc_plan* p : ctx->live) p->owner = nullptr;  // plans outliving their context free their own buffers
  for (int i = 0; i < kSpares; ++i) {
    pc_cuda_free(ctx->spare_rec[i].p);
    pc_cuda_free(ctx->spare_hist[i].p);
    pc_cuda_free(ctx->spare_tables[i].p);
  }
  pc_cuda_free(ctx->merge_dev);
  cudaFreeHost(ctx->merge_host);
  pc_cuda_free(ctx->zig_dev);
  pc_cuda_free(ctx->stats_dev);
  pc_cuda_free(ctx->error_dev);
  pc_cuda_free(ctx->persist_ctl);
  cudaFreeHost(ctx->pinned);
  cudaFreeHost(ctx->stage);
  cudaFreeHost(ctx->stage2);
  for (auto& ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : ctx->copy_done)
    if (ev) cudaEventDestroy(ev);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

int pc_set_stream(pc_context* ctx, void* stream) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx) return PC_ERR_INVALID;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_set_option(pc_context* ctx, const char* name, double value) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !name) return PC_ERR_INVALID;
  if (!(value >= 0.0) || !std::isfinite(value)) return fail(ctx, PC_ERR_INVALID, "option value must be >= 0");
  const std::string n(name);
  if (n == "memory_budget_bytes") {
    ctx->opt_budget = value;
  } else if (n == "max_slice_cells") {
    ctx->opt_max_slice = (uint64_t)value;
  } else if (n == "max_root_chunk") {
    ctx->opt_max_root_chunk = (uint64_t)value;
  } else if (n == "grid_blocks") {
    ctx->opt_grid_blocks = (int)value;
  } else if (n == "sweep_config") {
    if (value >= kNumSweepConfigs) return fail(ctx, PC_ERR_INVALID, "sweep_config must be 0..7");
    ctx->opt_config = (int)value;
  } else if (n == "driver") {
    if (value > 1) return fail(ctx, PC_ERR_INVALID, "driver must be 0 (per sweep) or 1 (persistent)");
    ctx->opt_driver = (int)value;
  } else if (n == "graph") {
    ctx->opt_graph = value != 0.0 ? 1 : 0;
  } else if (n == "smooth_predraw") {
    ctx->opt_smooth_predraw = value != 0.0 ? 1 : 0;
  } else if (n == "device_merge") {
    ctx->opt_device_merge = value != 0.0 ? 1 : 0;
  } else if (n == "batch_parts") {
    if (value < 1 || value > 64) return fail(ctx, PC_ERR_INVALID, "batch_parts must be 1..64");
    ctx->opt_batch_parts = (uint32_t)value;
  } else if (n == "fail_nth_call") {
    // counted from the calls made so far: the n-th call after this one fails (0: none)
    ctx->fail_at = value >= 1.0 ? ctx->cuda_calls + (uint64_t)value : 0;
  } else {
    return fail(ctx, PC_ERR_INVALID, "unknown option " + n);
  }
  if (n == "memory_budget_bytes" || n == "grid_blocks") free_pool(ctx);
  return PC_OK;
  PC_GUARD_END(ctx)
}

}  // extern "C"

namespace {

// Host part of the reference's pipeline for one input: the output value set and bin
// layout of io::load_fluorescences (src/io/parser.cu:68-154), the type table of
// io::load_cell_types (parser.cu:156-185), and the per-bin phi cap implied by the
// division test `fluorescence / 2 > threshold` (proliferation.cu:323).
// The type tables of an instance (I.t_max set): ratio-sum check, stable sort by ratio
// descending, cumulative ratios in that order (parser.cu:46-66,184; cell.cu:81-104),
// truncation bounds and the fallback type. Replaces I's type fields.
int prepare_types(const pc_cell_type* types, uint32_t n_types, InstanceHost& I, std::string& msg) {
  if (n_types && !types) return msg = "null argument", PC_ERR_INVALID;
  if (n_types == 0)
    return msg = "ERROR: proportion distribution of cell types does not sum to 1, aborting.", PC_ERR_INVALID;
  if (n_types > (uint32_t)kMaxTypes) return msg = "at most 64 cell types are supported", PC_ERR_UNSUPPORTED;
  I.types.clear();
  I.sorted_to_file.clear();
  double sum = 0.0;
  for (uint32_t i = 0; i < n_types; ++i) {
    if (!std::isfinite(types[i].ratio) || !std::isfinite(types[i].mean) || !std::isfinite(types[i].sd))
      return msg = "cell type parameters must be finite", PC_ERR_INVALID;
    if (types[i].mean > 0.0 && !(std::fabs(types[i].sd) < kMaxSigma))
      return msg = "cell type standard deviations must be below 2^127", PC_ERR_UNSUPPORTED;
    sum += types[i].ratio;
  }
  if (std::fabs(1.0 - sum) > 1.0 / std::pow(10.0, 8.0))
    return msg = "ERROR: proportion distribution of cell types does not sum to 1, aborting.", PC_ERR_INVALID;
  std::vector<uint32_t> order(n_types);
  for (uint32_t i = 0; i < n_types; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return types[a].ratio > types[b].ratio; });
  double acc = 0.0;
  for (uint32_t s = 0; s < n_types; ++s) {
    const pc_cell_type& src = types[order[s]];
    TypeDev t;
    std::memset(&t, 0, sizeof(t));
    acc += src.ratio;
    t.cum = acc;
    t.mu = src.mean;
    t.sigma = std::ldexp(src.sd, kSigmaShift);
    t.t_max = I.t_max;
    t.mode = src.mean < 0.0 ? kModeQuiescent : (src.mean == 0.0 ? kModeZeroMean : kModeNormal);
    truncation_bounds(src.mean, src.sd, t.zlo, t.zhi);
    if (t.mode == kModeZeroMean) {
      // tau = 0 for every cell of the type: with sigma = mu = 0, fma(0, z, 0) = +0 for any
      // z, so the kernels need no special case (and accept every z)
      t.sigma = 0.0;
      t.zlo = -INFINITY;
      t.zhi = INFINITY;
    }
    I.types.push_back(t);
    I.sorted_to_file.push_back(order[s]);
  }
  I.fallback = 0;
  for (uint32_t s = 0; s < n_types; ++s)
    if (types[order[s]].ratio > 0.0) I.fallback = s;
  return PC_OK;
}

// Output value set of a prepared instance (parser.cu:98-151): every nonzero bin's halving
// chain v, v/2, ... while >= phi, sorted and deduplicated, together with the
// (bin, generation) -> value index map of the result merge. Reads the instance's bins and
// phi, writes only values, vidx and vidx_stride (the run reads none of the three).
void build_value_set(InstanceHost& I) {
  const double threshold = I.phi;
  const size_t nb = I.bin_value.size();
  std::vector<uint32_t> chain_len(nb);  // chain length per nonzero bin
  uint64_t chain_total = 0;
  uint32_t longest = 0;
  for (size_t b = 0; b < nb; ++b) {
    uint32_t g = 0;
    for (double cur = I.bin_value[b]; cur >= threshold; cur = cur / 2) ++g;
    chain_len[b] = g;
    chain_total += g;
    longest = std::max(longest, g);
  }
  // Every generation a leaf can have (<= gmax) has a row; chains are never longer.
  I.vidx_stride = std::max(I.gmax, longest) + 1;
  I.vidx.assign(nb * (size_t)I.vidx_stride, -1);
  I.values.clear();

  // The chain of a normal value keeps its mantissa and lowers its exponent by one per
  // halving (phi >= 2^-1000 keeps every chain value normal), so the value set is enumerated
  // exponent by exponent, each exponent's values in mantissa order. Used when that grid is
  // dense; otherwise all chain values are sorted.
  bool normal = threshold >= 0x1p-1000;
  struct Chain {
    uint64_t mant;
    int32_t e_hi, len;
    uint32_t bin;
  };
  std::vector<Chain> ch;
  int32_t e_min = INT32_MAX, e_max = INT32_MIN;
  for (size_t b = 0; b < nb && normal; ++b) {
    if (!chain_len[b]) continue;
    uint64_t bits;
    std::memcpy(&bits, &I.bin_value[b], sizeof(bits));
    const int32_t e = (int32_t)((bits >> 52) & 0x7FF);
    if (e == 0) {
      normal = false;
      break;
    }
    ch.push_back(Chain{bits & ((1ull << 52) - 1), e, (int32_t)chain_len[b], (uint32_t)b});
    e_max = std::max(e_max, e);
    e_min = std::min(e_min, e - (int32_t)chain_len[b] + 1);
  }
  if (normal && !ch.empty() && (uint64_t)(e_max - e_min + 1) * ch.size() <= 8 * chain_total + 1024) {
    std::stable_sort(ch.begin(), ch.end(), [](const Chain& x, const Chain& y) { return x.mant < y.mant; });
    for (int32_t E = e_min; E <= e_max; ++E) {
      bool have = false;
      uint64_t prev = 0;
      for (const Chain& c : ch) {
        if (E > c.e_hi || E <= c.e_hi - c.len) continue;
        if (!have || c.mant != prev) {
          const uint64_t bits = ((uint64_t)E << 52) | c.mant;
          double v;
          std::memcpy(&v, &bits, sizeof(v));
          I.values.push_back(v);
          prev = c.mant;
          have = true;
        }
        I.vidx[(size_t)c.bin * I.vidx_stride + (uint32_t)(c.e_hi - E)] = (int32_t)(I.values.size() - 1);
      }
    }
  } else if (nb) {
    struct Link {
      double v;
      uint32_t bin, gen;
    };
    std::vector<Link> chain;
    chain.reserve(chain_total);
    for (size_t b = 0; b < nb; ++b) {
      uint32_t g = 0;
      for (double cur = I.bin_value[b]; g < chain_len[b]; cur = cur / 2) chain.push_back(Link{cur, (uint32_t)b, g++});
    }
    std::sort(chain.begin(), chain.end(), [](const Link& x, const Link& y) { return x.v < y.v; });
    for (size_t i = 0; i < chain.size(); ++i) {
      if (i == 0 || chain[i].v != chain[i - 1].v) I.values.push_back(chain[i].v);
      I.vidx[(size_t)chain[i].bin * I.vidx_stride + chain[i].gen] = (int32_t)(I.values.size() - 1);
    }
  }
}

// An instance's bins, phi caps and types from the caller's arrays; with_values also builds
// its output value set (build_value_set), which only the result merge reads.
int prepare_instance(const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types, uint32_t n_types,
                     double t_max, double phi, uint64_t seed, InstanceHost& I, std::string& msg,
                     bool with_values = true) {
  if ((n_bins && !bins) || (n_types && !types)) return msg = "null argument", PC_ERR_INVALID;
  if (!(t_max >= 0.0) || std::isinf(t_max)) return msg = "t_max must be finite and >= 0", PC_ERR_INVALID;
  if (!(phi >= 0.0) || std::isinf(phi)) return msg = "phi must be finite and > 0 (0 = automatic)", PC_ERR_INVALID;
  if (n_types == 0)
    return msg = "ERROR: proportion distribution of cell types does not sum to 1, aborting.", PC_ERR_INVALID;
  if (n_types > (uint32_t)kMaxTypes) return msg = "at most 64 cell types are supported", PC_ERR_UNSUPPORTED;

  // Threshold (parser.cu:80-96: with no threshold given, the smallest value with a
  // nonzero frequency; the `threshold == 0.0 ||` test is the reference's).
  double threshold = phi;
  if (threshold == 0.0) {
    for (uint64_t i = 0; i < n_bins; ++i)
      if (bins[i].frequency > 0 && (threshold == 0.0 || bins[i].value < threshold)) threshold = bins[i].value;
  }
  if (!(threshold > 0.0) || std::isinf(threshold)) return msg = "phi must be finite and > 0", PC_ERR_INVALID;
  I.phi = threshold;
  I.t_max = (t_max == 0.0) ? 0.0 : t_max;  // normalise -0
  I.seed = seed;

  // Bins with a nonzero frequency, in file order.
  uint64_t total = 0;
  for (uint64_t i = 0; i < n_bins; ++i) {
    if (bins[i].frequency == 0) continue;
    const double v = bins[i].value;
    if (!std::isfinite(v)) return msg = "histogram values must be finite", PC_ERR_INVALID;
    if (bins[i].frequency > 0xFFFFFFFFull - total) return msg = "more than 2^32-1 initial cells", PC_ERR_UNSUPPORTED;
    if (I.bin_value.size() + 1 >= (1u << 24)) return msg = "at most 2^24 nonzero bins", PC_ERR_UNSUPPORTED;
    total += bins[i].frequency;
    I.bin_value.push_back(v);
    I.bin_freq.push_back(bins[i].frequency);
  }
  I.roots = total;

  // Phi cap per bin: a cell of generation g divides only while its fluorescence, the bin
  // value halved g times, still satisfies `f / 2 > phi` (proliferation.cu:323).
  const size_t nb = I.bin_value.size();
  I.cap.resize(nb);
  I.gmax = 0;
  for (size_t b = 0; b < nb; ++b) {
    uint32_t c = 0;
    for (double f = I.bin_value[b]; f / 2 > threshold && c < 4096; f = f / 2) ++c;
    I.cap[b] = c;
    I.gmax = std::max(I.gmax, c);
  }
  const int rc = prepare_types(types, n_types, I, msg);
  if (rc == PC_OK && with_values) build_value_set(I);
  return rc;
}

// The batched form's per-type and per-instance device tables (instances already placed).
void batch_type_tables(const pc_plan* p, std::vector<BatchType>& btypes, std::vector<InstanceDev>& idev) {
  btypes.clear();
  idev.clear();
  for (uint32_t i = 0; i < (uint32_t)p->inst.size(); ++i) {
    const InstanceHost& I = p->inst[i];
    const uint32_t nt = (uint32_t)I.types.size();
    for (uint32_t k = 0; k < nt; ++k) {
      BatchType bt;
      std::memset(&bt, 0, sizeof(bt));
      bt.t = I.types[k];
      bt.k0 = (uint32_t)I.seed;
      bt.k1 = (uint32_t)(I.seed >> 32);
      bt.root_begin = I.root_begin;
      bt.instance = i;
      btypes.push_back(bt);
    }
    InstanceDev d;
    std::memset(&d, 0, sizeof(d));
    d.type_begin = I.type_begin;
    d.ntypes = nt;
    d.fallback = I.fallback;
    d.k0 = (uint32_t)I.seed;
    d.k1 = (uint32_t)(I.seed >> 32);
    d.root_begin = I.root_begin;
    d.t_max = I.t_max;
    idev.push_back(d);
  }
}

// Lays the plan's instances out one after another (initial cells, bins, types, histogram
// classes), fixes the root chunk and key layout, and uploads the tables.
std::atomic<uint64_t> g_plan_ids{1};

// Host-side tables of a plan, kept from its host part until its device part uploads them.
struct PlanTables {
  std::vector<uint32_t> bin_inst, bin_class;
  std::vector<BatchType> btypes;
  std::vector<InstanceDev> idev;
};

// The layout and host tables of a plan whose instances are prepared. Touches no context
// state and makes no CUDA call, so it can run on any thread.
int finalize_host(pc_plan* p, uint64_t max_root_chunk, PlanTables& t, std::string& msg) {
  uint64_t roots = 0, classes = 0;
  uint32_t bins = 0, ntypes_all = 0, gmax = 0;
  for (auto& I : p->inst) {
    I.root_begin = roots;
    I.bin_begin = bins;
    I.type_begin = ntypes_all;
    I.class_begin = classes;
    roots += I.roots;
    bins += (uint32_t)I.bin_value.size();
    ntypes_all += (uint32_t)I.types.size();
    classes += (uint64_t)I.bin_value.size() * I.types.size();
    gmax = std::max(gmax, I.gmax);
    if (bins >= (1u << 24)) return msg = "at most 2^24 nonzero bins in one run", PC_ERR_UNSUPPORTED;
  }
  if (p->batched && ntypes_all > 0xFFFFu) return msg = "at most 65535 cell types in one batch", PC_ERR_UNSUPPORTED;
  if (classes > 0xFFFFFFFFull) return msg = "more than 2^32-1 (bin, type) classes in one run", PC_ERR_UNSUPPORTED;
  p->nbins = bins;
  p->gmax = gmax;
  p->nclass = classes;
  p->roots_total = roots;
  p->root_begin = 0;
  p->root_end = roots;

  // Root chunk and key layout (key_layout): every key, a stored cell's or a parked
  // daughter's one generation below the deepest stored one, fits 64 bits.
  const KeyLayout kl = key_layout(roots, gmax, p->batched, max_root_chunk);
  p->chunk = kl.chunk;
  p->g_store_max = kl.g_store_max;
  p->hist_gens = std::min(gmax, p->g_store_max + 1) + 1;

  // Per-bin tables (first initial cell, cap and flags; in a batch also the instance and first
  // class). Each instance fills its own slice, on host threads when there are many.
  auto& bin_inst = t.bin_inst;
  auto& bin_class = t.bin_class;
  p->bin_start.assign((size_t)bins + 1, 0);
  p->bin_info.assign(bins, 0);
  if (p->batched) {
    bin_inst.assign(bins, 0);
    bin_class.assign(bins, 0);
  }
  auto fill = [&](uint32_t i) {
    InstanceHost& I = p->inst[i];
    const uint32_t nt = (uint32_t)I.types.size();
    uint64_t start = I.root_begin;
    for (size_t b = 0; b < I.bin_value.size(); ++b) {
      const size_t at = I.bin_begin + b;
      start += I.bin_freq[b];
      p->bin_start[at + 1] = start;
      uint32_t c = I.cap[b];
      uint32_t clamped = 0;
      if (c > p->g_store_max + 1) {
        c = p->g_store_max + 1;
        clamped = 0x200u;
      }
      p->bin_info[at] = c | (I.bin_value[b] >= I.phi ? 0x100u : 0u) | clamped;
      if (p->batched) {
        bin_inst[at] = i;
        bin_class[at] = (uint32_t)(I.class_begin + b * nt);
      }
    }
    I.hist_gens = std::min(I.gmax, p->g_store_max + 1) + 1;
  };
  const uint32_t ninst = (uint32_t)p->inst.size();
  if (ninst >= 64 && bins >= (1u << 16)) {
    parallel_for(ninst, fill);
  } else {
    for (uint32_t i = 0; i < ninst; ++i) fill(i);
  }
  if (p->batched) batch_type_tables(p, t.btypes, t.idev);
  return PC_OK;
}

// The allocations and uploads of a plan whose host part is done (on the context's thread).
int finalize_device(pc_context* ctx, pc_plan* p, const PlanTables& t) {
  const auto& bin_inst = t.bin_inst;
  const auto& bin_class = t.bin_class;
  const auto& btypes = t.btypes;
  const auto& idev = t.idev;
  const uint64_t chunk = p->chunk;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t nb = p->nbins;
  p->hist_elems = (size_t)p->hist_gens * std::max<uint64_t>(1, p->nclass);
  p->upload_bytes = nb * sizeof(uint32_t) + (nb + 1) * sizeof(uint64_t);
  // The plan's small tables share one device allocation (a spare of the context when one is
  // large enough), each at a 16-byte boundary: no allocator call per table on creation or
  // destruction.
  size_t tables = 0;
  auto place = [&tables](size_t bytes) {
    const size_t at = tables;
    tables += (std::max<size_t>(1, bytes) + 15) & ~size_t(15);
    return at;
  };
  const size_t nt = p->batched ? 0 : p->inst[0].types.size();
  const size_t o_info = place(nb * sizeof(uint32_t)), o_start = place((nb + 1) * sizeof(uint64_t));
  const size_t o_types = place(nt * sizeof(TypeDev)), o_btypes = place(btypes.size() * sizeof(BatchType));
  const size_t o_inst = place(idev.size() * sizeof(InstanceDev));
  const size_t o_binst = place(p->batched ? nb * sizeof(uint32_t) : 0), o_bclass = place(p->batched ? nb * sizeof(uint32_t) : 0);
  p->owner = ctx;
  ctx->live.push_back(p);
  cudaError_t e = take_spare(ctx->spare_tables, tables, &p->tables_dev, &p->tables_bytes);
  if (e == cudaSuccess) {
    char* base = static_cast<char*>(p->tables_dev);
    p->bin_info_dev = reinterpret_cast<uint32_t*>(base + o_info);
    p->bin_start_dev = reinterpret_cast<uint64_t*>(base + o_start);
    if (!p->batched) {
      p->types_dev = reinterpret_cast<TypeDev*>(base + o_types);
    } else {
      p->btypes_dev = reinterpret_cast<BatchType*>(base + o_btypes);
      p->inst_dev = reinterpret_cast<InstanceDev*>(base + o_inst);
      p->bin_inst_dev = reinterpret_cast<uint32_t*>(base + o_binst);
      p->bin_class_dev = reinterpret_cast<uint32_t*>(base + o_bclass);
    }
  }
  if (e == cudaSuccess)
    e = take_spare(ctx->spare_rec, std::max<uint64_t>(1, chunk) * sizeof(unsigned long long),
                   reinterpret_cast<void**>(&p->root_rec_dev), &p->rec_bytes);
  if (e == cudaSuccess)
    e = take_spare(ctx->spare_hist, p->hist_elems * sizeof(unsigned long long),
                   reinterpret_cast<void**>(&p->hist_dev), &p->hist_bytes);
  if (e == cudaSuccess && nb)
    e = pc_cuda_copy(p->bin_info_dev, p->bin_info.data(), nb * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = pc_cuda_copy(p->bin_start_dev, p->bin_start.data(), (nb + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
  if (!p->batched) {
    if (e == cudaSuccess)
      e = pc_cuda_copy(p->types_dev, p->inst[0].types.data(), nt * sizeof(TypeDev), cudaMemcpyHostToDevice, st);
    p->upload_bytes += nt * sizeof(TypeDev);
  } else {
    if (e == cudaSuccess)
      e = pc_cuda_copy(p->btypes_dev, btypes.data(), btypes.size() * sizeof(BatchType), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = pc_cuda_copy(p->inst_dev, idev.data(), idev.size() * sizeof(InstanceDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nb)
      e = pc_cuda_copy(p->bin_inst_dev, bin_inst.data(), nb * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nb)
      e = pc_cuda_copy(p->bin_class_dev, bin_class.data(), nb * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    p->upload_bytes += btypes.size() * sizeof(BatchType) + idev.size() * sizeof(InstanceDev) + 2 * nb * sizeof(uint32_t);
  }
  if (e == cudaSuccess) e = pc_cuda_sync(st);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PC_ERR_NOMEM : PC_ERR_CUDA,
                std::string("plan upload: ") + cudaGetErrorString(e));
  return PC_OK;
}

int finalize_plan(pc_context* ctx, pc_plan* p) {
  PlanTables t;
  std::string msg;
  const int rc = finalize_host(p, ctx->opt_max_root_chunk, t, msg);
  if (rc != PC_OK) return fail(ctx, rc, msg);
  return finalize_device(ctx, p, t);
}

// The host part of a batch: its instances prepared on host threads, then its layout and
// tables. Touches no context state and makes no CUDA call (runs on any thread); messages
// number the instances from `first`.
int prepare_batch(const pc_instance* instances, uint32_t n, uint32_t first, uint64_t max_root_chunk,
                  pc_batch** out, PlanTables& t, std::string& msg) {
  *out = nullptr;
  if (n == 0) return msg = "a batch needs at least one instance", PC_ERR_INVALID;
  pc_batch* b = new (std::nothrow) pc_batch();
  if (!b) return msg = "host allocation", PC_ERR_NOMEM;
  std::memset(&b->stats, 0, sizeof(b->stats));
  b->id = g_plan_ids.fetch_add(1);
  b->batched = true;
  b->inst.resize(n);
  std::vector<int> codes(n, PC_OK);
  std::vector<std::string> msgs(n);
  parallel_for(n, [&](uint32_t i) {
    const pc_instance& x = instances[i];
    codes[i] = prepare_instance(x.bins, x.n_bins, x.types, x.n_types, x.t_max, x.phi, x.seed, b->inst[i], msgs[i]);
  });
  int rc = PC_OK;
  for (uint32_t i = 0; i < n && rc == PC_OK; ++i)
    if (codes[i] != PC_OK) {
      rc = codes[i];
      msg = "instance " + std::to_string(first + i) + ": " + msgs[i];
    }
  if (rc == PC_OK) rc = finalize_host(b, max_root_chunk, t, msg);
  if (rc != PC_OK) {
    delete b;
    return rc;
  }
  *out = b;
  return PC_OK;
}

// Raw counts of one instance in its own [hist_gens][bins][types] layout, types in file
// order, from the plan's [generation][class] table.
void instance_counts(const pc_plan* p, const InstanceHost& I, const unsigned long long* h, uint64_t* out) {
  const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
  for (uint32_t g = 0; g < I.hist_gens; ++g)
    for (uint32_t b = 0; b < nb; ++b)
      for (uint32_t k = 0; k < nt; ++k)
        out[((uint64_t)g * nb + b) * nt + I.sorted_to_file[k]] = h[g * p->nclass + I.class_begin + (uint64_t)b * nt + k];
}

// The merged histogram of one instance (value set ascending, totals, per-type columns).
// Touches nothing shared, so instances can be merged on several threads.
int instance_result(const pc_plan* p, const InstanceHost& I, const unsigned long long* h, pc_histogram* out,
                    const char** msg) {
  const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
  const uint64_t nv = I.values.size();
  out->n_values = nv;
  out->n_types = nt;
  out->values = (double*)std::malloc(std::max<uint64_t>(1, nv) * sizeof(double));
  out->totals = (uint64_t*)std::calloc(std::max<uint64_t>(1, nv), sizeof(uint64_t));
  out->per_type = (uint64_t*)std::calloc(std::max<uint64_t>(1, nv * nt), sizeof(uint64_t));
  if (!out->values || !out->totals || !out->per_type) {
    pc_histogram_free(out);
    *msg = "host allocation";
    return PC_ERR_NOMEM;
  }
  if (nv) std::memcpy(out->values, I.values.data(), nv * sizeof(double));
  uint64_t leaves = 0;
  for (uint32_t g = 0; g < I.hist_gens; ++g)
    for (uint32_t b = 0; b < nb; ++b) {
      const int64_t vi = I.vidx[(uint64_t)b * I.vidx_stride + g];
      for (uint32_t k = 0; k < nt; ++k) {
        const uint64_t c = h[g * p->nclass + I.class_begin + (uint64_t)b * nt + k];
        if (!c) continue;
        if (vi < 0) {
          pc_histogram_free(out);
          *msg = "internal: leaf counted outside the output value set";
          return PC_ERR_CUDA;
        }
        out->totals[vi] += c;
        out->per_type[(uint64_t)vi * nt + I.sorted_to_file[k]] += c;
        leaves += c;
      }
    }
  out->stats.leaves = leaves;
  return PC_OK;
}


// Device scratch of the result merge above this size is not kept: such plans merge on host
// threads instead.
constexpr size_t kMaxMergeScratch = size_t(256) << 20;

size_t round16(size_t n) { return (n + 15) & ~size_t(15); }

// The merged histogram of a single-instance plan, merged on the device from the count table
// the run left there: the value map and type order go up (nbins x generations int32), the
// merged counts (values x (1 + types) u64) come back, instead of the whole [generation][class]
// table and a host loop over it. Returns PC_ERR_UNSUPPORTED when the scratch would exceed
// kMaxMergeScratch.
int device_result(pc_context* ctx, pc_plan* p, pc_histogram* out) {
  const InstanceHost& I = p->inst[0];
  const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
  const uint64_t nv = I.values.size();
  const size_t vidx_bytes = round16((size_t)nb * I.vidx_stride * sizeof(int32_t));
  const size_t s2f_bytes = round16((size_t)nt * sizeof(uint32_t));
  const size_t counts = (size_t)nv * (1u + nt) + 2u;  // totals, per_type, error word
  const size_t need = vidx_bytes + s2f_bytes + counts * sizeof(unsigned long long);
  if (need > kMaxMergeScratch) return PC_ERR_UNSUPPORTED;
  cudaStream_t st = ctx->stream;
  if (ctx->merge_dev_bytes < need) {
    pc_cuda_free(ctx->merge_dev);
    ctx->merge_dev = nullptr;
    ctx->merge_dev_bytes = 0;
    PC_CUDA(ctx, pc_cuda_malloc(&ctx->merge_dev, need));
    ctx->merge_dev_bytes = need;
  }
  if (ctx->merge_host_bytes < counts * sizeof(unsigned long long)) {
    cudaFreeHost(ctx->merge_host);
    ctx->merge_host = nullptr;
    ctx->merge_host_bytes = 0;
    PC_CUDA(ctx, pc_cuda_malloc_host(&ctx->merge_host, counts * sizeof(unsigned long long)));
    ctx->merge_host_bytes = counts * sizeof(unsigned long long);
  }
  char* base = static_cast<char*>(ctx->merge_dev);
  int32_t* vidx = reinterpret_cast<int32_t*>(base);
  uint32_t* s2f = reinterpret_cast<uint32_t*>(base + vidx_bytes);
  unsigned long long* merged = reinterpret_cast<unsigned long long*>(base + vidx_bytes + s2f_bytes);
  unsigned long long* totals = merged;
  unsigned long long* per_type = merged + nv;
  uint32_t* error = reinterpret_cast<uint32_t*>(merged + nv * (1u + nt));
  if (nb)
    PC_CUDA(ctx, pc_cuda_copy(vidx, I.vidx.data(), (size_t)nb * I.vidx_stride * sizeof(int32_t),
                              cudaMemcpyHostToDevice, st));
  PC_CUDA(ctx, pc_cuda_copy(s2f, I.sorted_to_file.data(), (size_t)nt * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  PC_CUDA(ctx, pc_cuda_memset(merged, 0, counts * sizeof(unsigned long long), st));
  PC_CUDA(ctx, PC_LAUNCH(launch_merge_counts(p->hist_dev, p->nclass, I.class_begin, I.hist_gens, nb, nt, vidx,
                                             I.vidx_stride, s2f, totals, per_type, error, st)));
  PC_CUDA(ctx, pc_cuda_copy(ctx->merge_host, merged, counts * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  PC_CUDA(ctx, pc_cuda_sync(st));
  const unsigned long long* hm = ctx->merge_host;
  if (static_cast<uint32_t>(hm[nv * (1u + nt)]) & 1u)
    return fail(ctx, PC_ERR_CUDA, "internal: leaf counted outside the output value set");
  out->n_values = nv;
  out->n_types = nt;
  out->values = (double*)std::malloc(std::max<uint64_t>(1, nv) * sizeof(double));
  out->totals = (uint64_t*)std::malloc(std::max<uint64_t>(1, nv) * sizeof(uint64_t));
  out->per_type = (uint64_t*)std::malloc(std::max<uint64_t>(1, nv * nt) * sizeof(uint64_t));
  if (!out->values || !out->totals || !out->per_type) {
    pc_histogram_free(out);
    return fail(ctx, PC_ERR_NOMEM, "host allocation");
  }
  if (nv) {
    std::memcpy(out->values, I.values.data(), nv * sizeof(double));
    std::memcpy(out->totals, hm, nv * sizeof(uint64_t));
    std::memcpy(out->per_type, hm + nv, nv * nt * sizeof(uint64_t));
  }
  uint64_t leaves = 0;
  for (uint64_t v = 0; v < nv; ++v) leaves += hm[v];
  out->stats.leaves = leaves;
  out->stats.h2d_bytes = (uint64_t)nb * I.vidx_stride * sizeof(int32_t) + (uint64_t)nt * sizeof(uint32_t);
  out->stats.d2h_bytes = counts * sizeof(unsigned long long);
  return PC_OK;
}

// The plan's count table after its last run, in the context's pinned stage (read back
// once per run; the stage grows to the largest table and is reused).
int stage_table(pc_context* ctx, pc_plan* p, const unsigned long long** out) {
  if (ctx->stage_plan != p->id || ctx->stage_run != p->run_id || !ctx->stage) {
    if (ctx->stage_elems < p->hist_elems) {
      cudaFreeHost(ctx->stage);
      ctx->stage = nullptr;
      ctx->stage_elems = 0;
      PC_CUDA(ctx, pc_cuda_malloc_host(&ctx->stage, p->hist_elems * sizeof(unsigned long long)));
      ctx->stage_elems = p->hist_elems;
    }
    ctx->stage_plan = 0;
    PC_CUDA(ctx, pc_cuda_copy(ctx->stage, p->hist_dev, p->hist_elems * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    PC_CUDA(ctx, pc_cuda_sync(ctx->stream));
    ctx->stage_plan = p->id;
    ctx->stage_run = p->run_id;
  }
  *out = ctx->stage;
  return PC_OK;
}

// The count table of a run into pinned stage `which` (0: the stage stage_table caches, whose
// cache this clears; 1: the second stage), without caching.
int copy_table(pc_context* ctx, pc_plan* p, int which, const unsigned long long** out,
               cudaEvent_t* async_done = nullptr) {
  unsigned long long** buf = which ? &ctx->stage2 : &ctx->stage;
  size_t* cap = which ? &ctx->stage2_elems : &ctx->stage_elems;
  if (!which) ctx->stage_plan = 0;
  if (*cap < p->hist_elems) {
    cudaFreeHost(*buf);
    *buf = nullptr;
    *cap = 0;
    PC_CUDA(ctx, pc_cuda_malloc_host(buf, p->hist_elems * sizeof(unsigned long long)));
    *cap = p->hist_elems;
  }
  *out = *buf;
  const size_t bytes = p->hist_elems * sizeof(unsigned long long);
  if (!async_done) {
    PC_CUDA(ctx, pc_cuda_copy(*buf, p->hist_dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    PC_CUDA(ctx, pc_cuda_sync(ctx->stream));
    return PC_OK;
  }
  // the run that wrote the table has completed (pc_plan_run returns after it): the copy goes
  // on the second stream and `*async_done` completes with it, while the caller's stream runs on
  if (!ctx->copy_stream) PC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  cudaEvent_t& ev = ctx->copy_done[which];
  if (!ev) PC_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  PC_CUDA(ctx, pc_cuda_copy(*buf, p->hist_dev, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream));
  PC_CUDA(ctx, pc_cuda_event_record(ev, ctx->copy_stream));
  *async_done = ev;
  return PC_OK;
}

// Frees a plan's host tables once its results are merged (for a sub-batch of thousands of
// instances, tens of thousands of vectors: milliseconds that pc_simulate_batch spends on a
// merge thread rather than on the thread that feeds the device). Touches no device state.
void release_host_tables(pc_plan* p) {
  std::vector<InstanceHost>().swap(p->inst);
  std::vector<uint64_t>().swap(p->bin_start);
  std::vector<uint32_t>().swap(p->bin_info);
}

// A single-instance plan; without its output value set when with_values is false (the
// caller then builds it with build_value_set before the result merge).
int plan_create(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types, uint32_t n_types,
                double t_max, double phi, uint64_t seed, bool with_values, pc_plan** out) {
  if (!ctx || !out) return fail(ctx, PC_ERR_INVALID, "null argument");
  *out = nullptr;
  pc_plan* p = new (std::nothrow) pc_plan();
  if (!p) return fail(ctx, PC_ERR_NOMEM, "host allocation");
  std::memset(&p->stats, 0, sizeof(p->stats));
  p->id = g_plan_ids.fetch_add(1);
  p->inst.resize(1);
  std::string msg;
  int rc = prepare_instance(bins, n_bins, types, n_types, t_max, phi, seed, p->inst[0], msg, with_values);
  if (rc != PC_OK) {
    delete p;
    return fail(ctx, rc, msg);
  }
  rc = finalize_plan(ctx, p);
  if (rc != PC_OK) {
    pc_plan_destroy(p);
    return rc;
  }
  *out = p;
  return PC_OK;
}

}  // namespace

namespace pc {

int host_value_set(const pc_bin* bins, uint64_t n_bins, double phi, double* values, uint64_t capacity,
                   uint64_t* n_values) {
  InstanceHost I;
  std::string msg;
  const pc_cell_type one{1.0, 1.0, 0.0};
  const int rc = prepare_instance(bins, n_bins, &one, 1, 0.0, phi, 0, I, msg);
  if (rc != PC_OK) return rc;
  *n_values = I.values.size();
  if (I.values.size() > capacity) return PC_ERR_INVALID;
  std::copy(I.values.begin(), I.values.end(), values);
  return PC_OK;
}

}  // namespace pc

extern "C" {

int pc_get_option(pc_context* ctx, const char* name, double* value) {
  if (!ctx || !name || !value) return PC_ERR_INVALID;
  const std::string n(name);
  if (n == "cuda_calls") {
    *value = (double)ctx->cuda_calls;
  } else if (n == "faults_injected") {
    *value = (double)ctx->faults_injected;
  } else if (n == "device_allocations") {
    *value = (double)g_live_device_allocs.load();
  } else if (n == "level_buffers") {
    *value = (double)ctx->pool.size();
  } else {
    return fail(ctx, PC_ERR_INVALID, "unknown option " + n);
  }
  return PC_OK;
}

int pc_plan_create(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                   uint32_t n_types, double t_max, double phi, uint64_t seed, pc_plan** out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  return plan_create(ctx, bins, n_bins, types, n_types, t_max, phi, seed, true, out);
  PC_GUARD_END(ctx)
}

int pc_plan_set_roots(pc_context* ctx, pc_plan* p, uint64_t root_begin, uint64_t root_end) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p) return PC_ERR_INVALID;
  if (root_begin > root_end || root_end > p->roots_total)
    return fail(ctx, PC_ERR_INVALID, "root range outside [0, number of initial cells]");
  p->root_begin = root_begin;
  p->root_end = root_end;
  return PC_OK;
  PC_GUARD_END(ctx)
}

void pc_plan_destroy(pc_plan* p) {
  if (!p) return;
  if (p->graph) cudaGraphExecDestroy(p->graph);
  if (p->owner) {
    pc_context* ctx = p->owner;
    ctx->live.erase(std::remove(ctx->live.begin(), ctx->live.end(), p), ctx->live.end());
    give_spare(ctx->spare_tables, p->tables_dev, p->tables_bytes);
    give_spare(ctx->spare_rec, p->root_rec_dev, p->rec_bytes);
    give_spare(ctx->spare_hist, p->hist_dev, p->hist_bytes);
  } else {
    pc_cuda_free(p->tables_dev);
    pc_cuda_free(p->root_rec_dev);
    pc_cuda_free(p->hist_dev);
  }
  delete p;
}

}  // extern "C"

namespace {

RunArgs make_args(const pc_context* ctx, const pc_plan* p) {
  RunArgs a;
  std::memset(&a, 0, sizeof(a));
  const InstanceHost& I0 = p->inst[0];
  if (!p->batched) {
    a.k0 = (uint32_t)I0.seed;
    a.k1 = (uint32_t)(I0.seed >> 32);
    philox_key_schedule(a.k0, a.k1, a.ks);
    a.t_max = I0.t_max;
    a.ntypes = (uint32_t)I0.types.size();
    a.fallback = I0.fallback;
    a.types = p->types_dev;
  } else {
    a.btypes = p->btypes_dev;
    a.inst = p->inst_dev;
    a.bin_inst = p->bin_inst_dev;
    a.bin_class = p->bin_class_dev;
  }
  a.nbins = p->nbins;
  a.nclass = (uint32_t)p->nclass;
  a.hist_gens = p->hist_gens;
  a.g_store_max = p->g_store_max;
  a.zig = ctx->zig_dev;
  a.bin_info = p->bin_info_dev;
  a.bin_start = p->bin_start_dev;
  a.root_rec = p->root_rec_dev;
  a.rec_cap = p->rec_bytes / sizeof(unsigned long long);
  a.hist = p->hist_dev;
  a.stats = ctx->stats_dev;
  a.error = ctx->error_dev;
  return a;
}

// Resident blocks per SM of a configuration's root, division and persistent kernels.
int kernel_occupancy(pc_context* ctx, bool narrow, bool batched, int config, const SweepKernels& K, int occ[3]) {
  int* c = ctx->occ[narrow ? 1 : 0][batched ? 1 : 0][config];
  if (c[0] == 0) {
    const int e = K.occupancy(&c[0], &c[1], &c[2]);
    if (e != 0) {
      c[0] = 0;
      return fail(ctx, PC_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString((cudaError_t)e));
    }
    for (int i = 0; i < 3; ++i) c[i] = std::max(1, c[i]);
  }
  for (int i = 0; i < 3; ++i) occ[i] = c[i];
  return PC_OK;
}

// Level buffers of `cells` cells each (at least `want`, reused when large enough and not
// above `cap`), with count/prefix arrays for `segs` segments.
int ensure_pool_geometry(pc_context* ctx, uint64_t want, uint64_t cap, uint32_t segs) {
  if (ctx->pool_cells < want || ctx->pool_cells > std::max(cap, want) || ctx->pool_segs < segs) {
    PC_CUDA(ctx, pc_cuda_sync(ctx->stream));
    free_pool(ctx);
    ctx->pool_cells = want;
    ctx->pool_segs = segs;
  }
  return PC_OK;
}

double budget_bytes(const pc_context* ctx) {
  return ctx->opt_budget > 0 ? ctx->opt_budget : 0.5 * (double)ctx->free_at_start;
}

// The host driver: one root sweep per chunk, then division sweeps depth-first over a stack
// of level buffers, the host reading each output level's size.
int run_per_sweep(pc_context* ctx, pc_plan* p, const SweepKernels& K, const int occ[3], RunArgs& a) {
  cudaStream_t st = ctx->stream;
  const uint64_t nroots = p->root_end - p->root_begin;
  const uint32_t warps = (uint32_t)K.threads / 32u;
  // Level-buffer geometry from the memory budget: the depth-first stack never holds more
  // than one buffer per generation plus one, so (levels + 2) buffers always fit.
  const int rmax = max_blocks(ctx, occ[0]), dmax = max_blocks(ctx, occ[1]);
  const uint32_t segs = (uint32_t)std::max(rmax, dmax) * warps;
  const uint32_t levels = std::min<uint32_t>(p->gmax, 40u) + 2u;
  // Any size <= budget / levels is safe; a buffer near 64 cells per root usually holds a
  // whole generation, so most generations run as a single sweep.
  const uint64_t cap = (uint64_t)(budget_bytes(ctx) / levels / sizeof(ulonglong2));
  uint64_t want = std::min<uint64_t>(cap, std::max<uint64_t>(1ull << 24, 64ull * nroots));
  want = std::max<uint64_t>(want, 4ull * segs + 1024);
  int rc = ensure_pool_geometry(ctx, want, cap, segs);
  if (rc != PC_OK) return rc;
  const uint64_t cells = ctx->pool_cells;
  uint64_t max_slice = (cells - 2ull * segs) / 2;
  if (ctx->opt_max_slice) max_slice = std::min<uint64_t>(max_slice, std::max<uint64_t>(1, ctx->opt_max_slice));
  const uint64_t chunk = std::min<uint64_t>(p->chunk, cells - segs);

  struct Entry {
    int buf;
    uint32_t gen, nseg;
    uint64_t stride, pos, n;
  };
  std::vector<Entry> stack;
  float ms = 0.f;
  double dev_ms = 0.0, div_ms = 0.0;
  uint64_t divisions = 0;
  uint32_t sweeps = 0, max_gen = 0, chunks = 0;

  for (uint64_t c0 = p->root_begin; c0 < p->root_end; c0 += chunk) {
    const uint64_t n = std::min<uint64_t>(chunk, p->root_end - c0);
    a.root_base = c0;
    ++chunks;
    int b0 = -1;
    rc = acquire(ctx, &b0);
    if (rc != PC_OK) return rc;
    LevelBuf& L = ctx->pool[b0];
    const int blocks = grid_for(ctx, n, occ[0], K.threads);
    const uint32_t nseg = (uint32_t)blocks * warps;
    LevelOut o{L.cells, L.count, L.prefix, L.ticket, (n + nseg - 1) / nseg};
    PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[0], st));
    PC_CUDA(ctx, PC_LAUNCH(K.roots(a, 0, n, o, blocks, st)));
    PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[1], st));
    PC_CUDA(ctx, pc_cuda_copy(ctx->pinned, L.prefix + nseg, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    PC_CUDA(ctx, pc_cuda_sync(st));
    PC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    dev_ms += ms;
    const uint64_t n0 = ctx->pinned[0];
    if (n0 == 0) {
      L.busy = false;
      continue;
    }
    stack.push_back(Entry{b0, 0u, nseg, o.stride, 0, n0});
    while (!stack.empty()) {
      Entry& top = stack.back();
      const uint64_t len = std::min<uint64_t>(top.n - top.pos, max_slice);
      int bo = -1;
      rc = acquire(ctx, &bo);
      if (rc != PC_OK) return rc;
      const LevelBuf& In = ctx->pool[top.buf];
      const LevelBuf& Out = ctx->pool[bo];
      const int blocks_d = grid_for(ctx, len, occ[1], K.threads);
      const uint32_t oseg = (uint32_t)blocks_d * warps;
      LevelIn li{In.cells, In.prefix, top.nseg, top.stride, top.pos, top.pos + len};
      LevelOut lo{Out.cells, Out.count, Out.prefix, Out.ticket, 2 * ((len + oseg - 1) / oseg)};
      const uint32_t gen = top.gen;
      PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[2], st));
      PC_CUDA(ctx, PC_LAUNCH(K.divide(a, li, gen, lo, blocks_d, st)));
      PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[3], st));
      PC_CUDA(ctx, pc_cuda_copy(ctx->pinned, Out.prefix + oseg, sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, st));
      divisions += len;
      ++sweeps;
      max_gen = std::max(max_gen, gen + 1);
      top.pos += len;
      if (top.pos == top.n) {
        ctx->pool[top.buf].busy = false;  // stream order protects the in-flight read
        stack.pop_back();
      }
      PC_CUDA(ctx, pc_cuda_sync(st));
      PC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
      dev_ms += ms;
      div_ms += ms;
      const uint64_t n_out = ctx->pinned[0];
      if (n_out > 0 && gen + 1 <= p->g_store_max) {
        stack.push_back(Entry{bo, gen + 1, oseg, lo.stride, 0, n_out});
      } else {
        ctx->pool[bo].busy = false;
      }
    }
  }
  PC_CUDA(ctx, pc_cuda_copy(ctx->pinned, ctx->stats_dev, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  PC_CUDA(ctx, pc_cuda_copy(ctx->pinned + 8, ctx->error_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  PC_CUDA(ctx, pc_cuda_sync(st));
  p->stats.divisions = divisions;
  p->stats.sweeps = sweeps;
  p->stats.root_sweeps = chunks;
  p->stats.kernel_launches = sweeps + chunks;
  p->stats.max_generation = max_gen;
  p->stats.device_ms = dev_ms;
  p->stats.divide_ms = div_ms;
  p->stats.d2h_bytes = (uint64_t)(sweeps + chunks) * 8u + 40u;
  return PC_OK;
}

// The operations of one persistent run, in stream order (also what a graph captures):
// clear the counts and control words, the cooperative launch, the totals back to pinned.
int enqueue_persistent(pc_context* ctx, pc_plan* p, const SweepKernels& K, const PersistArgs& pa, int grid,
                       cudaStream_t s) {
  PC_CUDA(ctx, pc_cuda_memset(p->hist_dev, 0, p->hist_elems * sizeof(unsigned long long), s));
  PC_CUDA(ctx, pc_cuda_memset(ctx->stats_dev, 0, 4 * sizeof(unsigned long long), s));
  PC_CUDA(ctx, pc_cuda_memset(ctx->error_dev, 0, sizeof(uint32_t), s));
  PC_CUDA(ctx, pc_cuda_memset(ctx->persist_ctl, 0, 48, s));
  PC_CUDA(ctx, PC_LAUNCH(K.persist(pa, grid, s)));
  PC_CUDA(ctx, pc_cuda_copy(ctx->pinned, ctx->stats_dev, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  PC_CUDA(ctx, pc_cuda_copy(ctx->pinned + 8, ctx->error_dev, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  PC_CUDA(ctx, pc_cuda_copy(ctx->pinned + 16, ctx->persist_ctl + 4, 4 * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, s));
  return PC_OK;
}

// The persistent driver: the whole run as one cooperative launch (optionally replayed from
// a captured CUDA graph). Returns PC_ERR_UNSUPPORTED when the plan needs more level
// buffers than the kernel's schedule holds (the caller then uses the host driver).
int run_persistent(pc_context* ctx, pc_plan* p, const SweepKernels& K, const int occ[3], const RunArgs& a) {
  cudaStream_t st = ctx->stream;
  const uint32_t nbuf = std::min<uint32_t>(p->gmax, p->g_store_max + 1u) + 2u;
  if (nbuf > (uint32_t)kMaxPool) return PC_ERR_UNSUPPORTED;
  const uint64_t nroots = p->root_end - p->root_begin;
  const uint32_t warps = (uint32_t)K.threads / 32u;
  int grid = ctx->sms * occ[2];
  if (ctx->opt_grid_blocks > 0) grid = std::min(grid, ctx->opt_grid_blocks);
  const uint32_t segs = (uint32_t)grid * warps;
  const uint64_t cap = (uint64_t)(budget_bytes(ctx) / nbuf / sizeof(ulonglong2));
  uint64_t want = std::min<uint64_t>(cap, std::max<uint64_t>(1ull << 24, 64ull * nroots));
  want = std::max<uint64_t>(want, 4ull * segs + 1024);
  int rc = ensure_pool_geometry(ctx, want, cap, segs);
  if (rc != PC_OK) return rc;
  const uint64_t cells = ctx->pool_cells;
  std::vector<int> held;
  for (uint32_t i = 0; i < nbuf; ++i) {
    int b = -1;
    rc = acquire(ctx, &b);
    if (rc != PC_OK) {
      for (int h : held) ctx->pool[h].busy = false;
      return rc;
    }
    held.push_back(b);
  }
  PersistArgs pa;
  std::memset(&pa, 0, sizeof(pa));
  pa.a = a;
  for (uint32_t i = 0; i < nbuf; ++i) {
    const LevelBuf& L = ctx->pool[held[i]];
    pa.cells[i] = L.cells;
    pa.count[i] = L.count;
    pa.prefix[i] = L.prefix;
    pa.ticket[i] = L.ticket;
  }
  for (int h : held) ctx->pool[h].busy = false;  // stream order protects the run
  pa.nbuf = nbuf;
  pa.g_limit = p->g_store_max;
  pa.root_lo = p->root_begin;
  pa.root_hi = p->root_end;
  pa.chunk = std::min<uint64_t>(p->chunk, cells - segs);
  pa.max_slice = (cells - 2ull * segs) / 2;
  if (ctx->opt_max_slice) pa.max_slice = std::min<uint64_t>(pa.max_slice, std::max<uint64_t>(1, ctx->opt_max_slice));
  pa.barrier = ctx->persist_ctl;
  pa.out = reinterpret_cast<unsigned long long*>(ctx->persist_ctl + 4);
  pa.timeout_ns = 20000000000ull;

  float ms = 0.f;
  PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[0], st));
  bool use_graph = ctx->opt_graph != 0;
  if (use_graph) {
    const bool same = p->graph && p->graph_config == ctx->opt_config && p->graph_grid == grid &&
                      std::memcmp(&p->graph_args, &pa, sizeof(pa)) == 0;
    if (!same) {
      if (p->graph) cudaGraphExecDestroy(p->graph);
      p->graph = nullptr;
      cudaStream_t cap_st = ctx->own_stream;
      PC_CUDA(ctx, pc_cuda_sync(st));
      PC_CUDA(ctx, cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
      rc = enqueue_persistent(ctx, p, K, pa, grid, cap_st);
      cudaGraph_t g = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(cap_st, &g);
      cudaError_t ei = cudaErrorUnknown;
      if (rc == PC_OK && ee == cudaSuccess) ei = cudaGraphInstantiate(&p->graph, g, 0);
      if (g) cudaGraphDestroy(g);
      if (rc != PC_OK || ee != cudaSuccess || ei != cudaSuccess) {
        // capture or instantiation not possible here: run the same operations directly
        (void)cudaGetLastError();
        p->graph = nullptr;
        use_graph = false;
      } else {
        p->graph_args = pa;
        p->graph_config = ctx->opt_config;
        p->graph_grid = grid;
      }
    }
  }
  if (use_graph) {
    PC_CUDA(ctx, pc_cuda_graph_launch(p->graph, st));
  } else {
    rc = enqueue_persistent(ctx, p, K, pa, grid, st);
    if (rc != PC_OK) return rc;
  }
  PC_CUDA(ctx, pc_cuda_event_record(ctx->ev[1], st));
  PC_CUDA(ctx, pc_cuda_sync(st));
  PC_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
  p->stats.divisions = ctx->pinned[16];
  p->stats.sweeps = (uint32_t)ctx->pinned[17];
  p->stats.max_generation = (uint32_t)ctx->pinned[18];
  p->stats.root_sweeps = (uint32_t)ctx->pinned[19];
  p->stats.kernel_launches = 1;
  p->stats.device_ms = ms;
  p->stats.divide_ms = ms;  // root and division sweeps share the launch
  p->stats.d2h_bytes = 72u;
  return PC_OK;
}

// Bins from which simulate_one builds the output value set on a helper thread.
constexpr size_t kValueSetThreadBins = 256;

// pc_simulate and pc_simulate_shard: one plan created, run and merged. The output value set,
// which only the merge reads, is built on a helper thread while the calling thread runs the
// plan (the run reads none of the instance's value-set fields); small inputs build it first.
int simulate_one(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types, uint32_t n_types,
                 double t_max, double phi, uint64_t seed, const uint64_t* roots, pc_histogram* out) {
  if (!out) return fail(ctx, PC_ERR_INVALID, "null argument");
  std::memset(out, 0, sizeof(*out));
  pc_plan* p = nullptr;
  int rc = plan_create(ctx, bins, n_bins, types, n_types, t_max, phi, seed, false, &p);
  if (rc != PC_OK) return rc;
  if (roots) rc = pc_plan_set_roots(ctx, p, roots[0], roots[1]);
  if (rc != PC_OK) {
    pc_plan_destroy(p);
    return rc;
  }
  InstanceHost& I = p->inst[0];
  std::atomic<bool> built{false};
  std::thread helper;
  if (I.bin_value.size() >= kValueSetThreadBins) {
    try {
      helper = std::thread([&I, &built] {
        try {
          build_value_set(I);
          built = true;
        } catch (...) {
        }
      });
    } catch (...) {  // no thread: build it here
    }
  }
  if (!helper.joinable()) {
    try {
      build_value_set(I);
      built = true;
    } catch (...) {
    }
  }
  rc = pc_plan_run(ctx, p);
  if (helper.joinable()) helper.join();
  if (rc == PC_OK && !built) rc = fail(ctx, PC_ERR_NOMEM, "host allocation");
  if (rc == PC_OK) rc = pc_plan_result(ctx, p, out);
  pc_plan_destroy(p);
  return rc;
}

}  // namespace

extern "C" {

int pc_plan_run(pc_context* ctx, pc_plan* p) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p) return PC_ERR_INVALID;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  // a run that failed part way may have left level buffers marked in use; every run is
  // complete (or failed) when its call returns, and work in flight is ordered on the stream
  for (auto& lb : ctx->pool) lb.busy = false;
  std::memset(&p->stats, 0, sizeof(p->stats));
  const uint64_t nroots = p->root_end - p->root_begin;
  p->stats.roots = nroots;
  p->ran = true;
  ++p->run_id;
  const bool narrow = p->gmax <= kNarrowMaxGen;
  const int config = narrow ? ctx->opt_config : kDefaultSweepConfig;
  const SweepKernels& K = sweep_kernels(narrow, p->batched, config);
  int occ[3];
  int rc = kernel_occupancy(ctx, narrow, p->batched, config, K, occ);
  if (rc != PC_OK) return rc;
  RunArgs a = make_args(ctx, p);
  rc = PC_ERR_UNSUPPORTED;
  if (ctx->opt_driver == 1 && nroots > 0 && p->nbins > 0) rc = run_persistent(ctx, p, K, occ, a);
  if (rc == PC_ERR_UNSUPPORTED) {
    PC_CUDA(ctx, pc_cuda_memset(p->hist_dev, 0, p->hist_elems * sizeof(unsigned long long), st));
    PC_CUDA(ctx, pc_cuda_memset(ctx->stats_dev, 0, 4 * sizeof(unsigned long long), st));
    PC_CUDA(ctx, pc_cuda_memset(ctx->error_dev, 0, sizeof(uint32_t), st));
    if (nroots == 0 || p->nbins == 0) {
      PC_CUDA(ctx, pc_cuda_sync(st));
      return PC_OK;
    }
    rc = run_per_sweep(ctx, p, K, occ, a);
  }
  if (rc != PC_OK) return rc;
  p->stats.vanished = ctx->pinned[0];
  p->stats.uncounted = ctx->pinned[1];
  p->stats.h2d_bytes = p->upload_bytes;
  const uint32_t err = (uint32_t)(ctx->pinned[8] & 0xFFFFFFFFu);
  if (err & 16u) return fail(ctx, PC_ERR_INTERNAL, "internal: a device bounds check failed (checked build)");
  if (err & 4u) return fail(ctx, PC_ERR_CUDA, "persistent driver: a grid barrier timed out");
  if (err & 8u) return fail(ctx, PC_ERR_CUDA, "internal: the persistent schedule ran out of level buffers");
  if (err & 2u) return fail(ctx, PC_ERR_CUDA, "internal: the normal sampler exceeded its rejection budget");
  if (err & 1u)
    return fail(ctx, PC_ERR_DEPTH, "a lineage exceeded the deepest generation the key layout holds");
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_plan_stats(pc_context* ctx, const pc_plan* p, pc_stats* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p || !out) return PC_ERR_INVALID;
  if (!p->ran) return fail(ctx, PC_ERR_INVALID, "plan has not run");
  *out = p->stats;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_plan_raw_counts(pc_context* ctx, pc_plan* p, uint64_t* host_out, uint64_t capacity,
                       uint64_t* n_elems, uint32_t dims[3]) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p || p->inst.empty()) return PC_ERR_INVALID;
  const InstanceHost& I = p->inst[0];
  const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
  const uint64_t n = (uint64_t)I.hist_gens * nb * nt;
  if (n_elems) *n_elems = n;
  if (dims) {
    dims[0] = I.hist_gens;
    dims[1] = nb;
    dims[2] = nt;
  }
  if (!host_out) return PC_OK;
  if (capacity < n) return fail(ctx, PC_ERR_INVALID, "raw count buffer too small");
  if (!p->ran) return fail(ctx, PC_ERR_INVALID, "plan has not run");
  const unsigned long long* h = nullptr;
  const int rc = stage_table(ctx, p, &h);
  if (rc != PC_OK) return rc;
  instance_counts(p, I, h, host_out);
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_plan_result(pc_context* ctx, pc_plan* p, pc_histogram* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p || !out || p->inst.empty()) return PC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  if (!p->ran) return fail(ctx, PC_ERR_INVALID, "plan has not run");
  int rc = ctx->opt_device_merge ? device_result(ctx, p, out) : PC_ERR_UNSUPPORTED;
  uint64_t h2d = 0, d2h = 0;
  if (rc == PC_OK) {
    h2d = out->stats.h2d_bytes;
    d2h = out->stats.d2h_bytes;
  } else if (rc == PC_ERR_UNSUPPORTED) {
    // merge scratch too large for the device (or the device merge switched off): read the
    // count table back, merge on the host
    const unsigned long long* h = nullptr;
    rc = stage_table(ctx, p, &h);
    if (rc != PC_OK) return rc;
    const char* msg = "";
    rc = instance_result(p, p->inst[0], h, out, &msg);
    if (rc != PC_OK) return fail(ctx, rc, msg);
    d2h = p->hist_elems * sizeof(unsigned long long);
  } else {
    return rc;
  }
  const uint64_t leaves = out->stats.leaves;
  out->stats = p->stats;
  out->stats.leaves = leaves;
  out->stats.h2d_bytes += h2d;
  out->stats.d2h_bytes += d2h;
  return PC_OK;
  PC_GUARD_END(ctx)
}

void pc_histogram_free(pc_histogram* h) {
  if (!h) return;
  std::free(h->values);
  std::free(h->totals);
  std::free(h->per_type);
  h->values = nullptr;
  h->totals = nullptr;
  h->per_type = nullptr;
  h->n_values = 0;
}

int pc_simulate(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                uint32_t n_types, double t_max, double phi, uint64_t seed, pc_histogram* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  return simulate_one(ctx, bins, n_bins, types, n_types, t_max, phi, seed, nullptr, out);
  PC_GUARD_END(ctx)
}

int pc_simulate_shard(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                      uint32_t n_types, double t_max, double phi, uint64_t seed, uint64_t root_begin,
                      uint64_t root_end, pc_histogram* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  const uint64_t roots[2] = {root_begin, root_end};
  return simulate_one(ctx, bins, n_bins, types, n_types, t_max, phi, seed, roots, out);
  PC_GUARD_END(ctx)
}

int pc_histogram_accumulate(pc_histogram* dst, const pc_histogram* src) {
  PC_GUARD_BEGIN
  if (!dst || !src) return PC_ERR_INVALID;
  if (dst->n_values != src->n_values || dst->n_types != src->n_types) return PC_ERR_INVALID;
  const uint64_t nv = dst->n_values;
  if (nv && (!dst->values || !src->values || !dst->totals || !src->totals || !dst->per_type || !src->per_type))
    return PC_ERR_INVALID;
  for (uint64_t v = 0; v < nv; ++v)
    if (std::memcmp(&dst->values[v], &src->values[v], sizeof(double)) != 0) return PC_ERR_INVALID;
  for (uint64_t v = 0; v < nv; ++v) dst->totals[v] += src->totals[v];
  for (uint64_t i = 0; i < nv * dst->n_types; ++i) dst->per_type[i] += src->per_type[i];
  pc_stats& a = dst->stats;
  const pc_stats& b = src->stats;
  a.roots += b.roots;
  a.divisions += b.divisions;
  a.leaves += b.leaves;
  a.uncounted += b.uncounted;
  a.vanished += b.vanished;
  a.max_generation = std::max(a.max_generation, b.max_generation);
  a.sweeps += b.sweeps;
  a.root_sweeps += b.root_sweeps;
  a.kernel_launches += b.kernel_launches;
  a.device_ms += b.device_ms;
  a.divide_ms += b.divide_ms;
  a.h2d_bytes += b.h2d_bytes;
  a.d2h_bytes += b.d2h_bytes;
  return PC_OK;
  PC_GUARD_END(nullptr)
}

int pc_batch_create(pc_context* ctx, const pc_instance* instances, uint32_t n_instances, pc_batch** out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !out) return fail(ctx, PC_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_instances && !instances) return fail(ctx, PC_ERR_INVALID, "null argument");
  PlanTables t;
  std::string msg;
  pc_batch* b = nullptr;
  int rc = prepare_batch(instances, n_instances, 0, ctx->opt_max_root_chunk, &b, t, msg);
  if (rc != PC_OK) return fail(ctx, rc, msg);
  rc = finalize_device(ctx, b, t);
  if (rc != PC_OK) {
    pc_batch_destroy(b);
    return rc;
  }
  *out = b;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_batch_run(pc_context* ctx, pc_batch* b) { return pc_plan_run(ctx, b); }

int pc_batch_stats(pc_context* ctx, const pc_batch* b, pc_stats* out) { return pc_plan_stats(ctx, b, out); }

uint32_t pc_batch_size(const pc_batch* b) { return b ? (uint32_t)b->inst.size() : 0u; }

static int batch_table(pc_context* ctx, pc_batch* b, uint32_t instance, const unsigned long long** h) {
  if (instance >= b->inst.size()) return fail(ctx, PC_ERR_INVALID, "instance index out of range");
  if (!b->ran) return fail(ctx, PC_ERR_INVALID, "batch has not run");
  return stage_table(ctx, b, h);
}

int pc_batch_raw_counts(pc_context* ctx, pc_batch* b, uint32_t instance, uint64_t* host_out, uint64_t capacity,
                        uint64_t* n_elems, uint32_t dims[3]) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !b) return PC_ERR_INVALID;
  if (instance >= b->inst.size()) return fail(ctx, PC_ERR_INVALID, "instance index out of range");
  const InstanceHost& I = b->inst[instance];
  const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
  const uint64_t n = (uint64_t)I.hist_gens * nb * nt;
  if (n_elems) *n_elems = n;
  if (dims) {
    dims[0] = I.hist_gens;
    dims[1] = nb;
    dims[2] = nt;
  }
  if (!host_out) return PC_OK;
  if (capacity < n) return fail(ctx, PC_ERR_INVALID, "raw count buffer too small");
  const unsigned long long* h = nullptr;
  const int rc = batch_table(ctx, b, instance, &h);
  if (rc != PC_OK) return rc;
  instance_counts(b, I, h, host_out);
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_batch_result(pc_context* ctx, pc_batch* b, uint32_t instance, pc_histogram* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !b || !out) return PC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  const unsigned long long* h = nullptr;
  int rc = batch_table(ctx, b, instance, &h);
  if (rc != PC_OK) return rc;
  const InstanceHost& I = b->inst[instance];
  const char* msg = "";
  rc = instance_result(b, I, h, out, &msg);
  if (rc != PC_OK) return fail(ctx, rc, msg);
  out->stats.roots = I.roots;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_batch_set_types(pc_context* ctx, pc_batch* b, const pc_cell_type* types) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !b || !types) return fail(ctx, PC_ERR_INVALID, "null argument");
  if (!b->batched) return fail(ctx, PC_ERR_INVALID, "not a batch");
  // validate every instance's new types before changing anything
  const uint32_t n = (uint32_t)b->inst.size();
  std::vector<InstanceHost> next(n);
  uint64_t off = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t nt = (uint32_t)b->inst[i].types.size();
    next[i].t_max = b->inst[i].t_max;
    std::string msg;
    const int rc = prepare_types(types + off, nt, next[i], msg);
    if (rc != PC_OK) return fail(ctx, rc, "instance " + std::to_string(i) + ": " + msg);
    off += nt;
  }
  for (uint32_t i = 0; i < n; ++i) {
    InstanceHost& I = b->inst[i];
    I.types.swap(next[i].types);
    I.sorted_to_file.swap(next[i].sorted_to_file);
    I.fallback = next[i].fallback;
  }
  std::vector<BatchType> btypes;
  std::vector<InstanceDev> idev;
  batch_type_tables(b, btypes, idev);
  b->ran = false;  // counts of the previous run belong to the previous types
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  PC_CUDA(ctx, pc_cuda_copy(b->btypes_dev, btypes.data(), btypes.size() * sizeof(BatchType),
                               cudaMemcpyHostToDevice, ctx->stream));
  PC_CUDA(ctx, pc_cuda_copy(b->inst_dev, idev.data(), idev.size() * sizeof(InstanceDev), cudaMemcpyHostToDevice,
                               ctx->stream));
  PC_CUDA(ctx, pc_cuda_sync(ctx->stream));  // the host tables are temporaries
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_batch_totals(pc_context* ctx, pc_batch* b, uint64_t* out, uint64_t capacity, uint64_t* offsets) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !b) return PC_ERR_INVALID;
  const uint32_t n = (uint32_t)b->inst.size();
  std::vector<uint64_t> off(n + 1, 0);
  for (uint32_t i = 0; i < n; ++i) off[i + 1] = off[i] + b->inst[i].values.size();
  if (offsets) std::memcpy(offsets, off.data(), (n + 1) * sizeof(uint64_t));
  if (!out) return PC_OK;
  if (capacity < off[n]) return fail(ctx, PC_ERR_INVALID, "totals buffer too small");
  if (!b->ran) return fail(ctx, PC_ERR_INVALID, "batch has not run");
  const unsigned long long* h = nullptr;
  const int rc = stage_table(ctx, b, &h);
  if (rc != PC_OK) return rc;
  std::vector<int> bad(n, 0);
  parallel_for(n, [&](uint32_t i) {
    const InstanceHost& I = b->inst[i];
    const uint32_t nb = (uint32_t)I.bin_value.size(), nt = (uint32_t)I.types.size();
    uint64_t* t = out + off[i];
    std::fill(t, t + I.values.size(), 0ull);
    for (uint32_t g = 0; g < I.hist_gens; ++g)
      for (uint32_t bb = 0; bb < nb; ++bb) {
        const int64_t vi = I.vidx[(uint64_t)bb * I.vidx_stride + g];
        const unsigned long long* row = h + g * b->nclass + I.class_begin + (uint64_t)bb * nt;
        for (uint32_t k = 0; k < nt; ++k) {
          if (!row[k]) continue;
          if (vi < 0) {
            bad[i] = 1;
            continue;
          }
          t[vi] += row[k];
        }
      }
  });
  for (uint32_t i = 0; i < n; ++i)
    if (bad[i]) return fail(ctx, PC_ERR_CUDA, "internal: leaf counted outside the output value set");
  return PC_OK;
  PC_GUARD_END(ctx)
}

void pc_batch_destroy(pc_batch* b) { pc_plan_destroy(b); }

int pc_simulate_batch(pc_context* ctx, const pc_instance* instances, uint32_t n_instances, pc_histogram* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !out) return fail(ctx, PC_ERR_INVALID, "null argument");
  if (n_instances && !instances) return fail(ctx, PC_ERR_INVALID, "null argument");
  for (uint32_t i = 0; i < n_instances; ++i) std::memset(out + i, 0, sizeof(pc_histogram));
  // Large batches run as min(batch_parts, n / 256) consecutive sub-batches. While the device runs one part, a host thread prepares the next (its
  // instances, layout and tables: everything but the uploads) and host threads merge the
  // previous part's histograms (for 4096 instances about 0.5 GB of host output). Every
  // instance's counts depend on that instance alone, so the split changes no result.
  const uint32_t parts = std::min<uint32_t>(ctx->opt_batch_parts, std::max<uint32_t>(1u, n_instances / 256u));
  const uint64_t max_root_chunk = ctx->opt_max_root_chunk;
  // the first and the last part, whose preparation and merge overlap nothing, are a quarter
  // of the size of the others (weights 1, 4, ..., 4, 1)
  auto first_of = [&](uint32_t part) {
    if (parts == 1) return part == 0 ? 0u : n_instances;
    const uint64_t total = 4ull * parts - 6ull;
    const uint64_t w = part == 0 ? 0ull : (part == parts ? total : 4ull * part - 3ull);
    return (uint32_t)((uint64_t)n_instances * w / total);
  };
  std::vector<int> codes(n_instances, PC_OK);
  std::vector<const char*> msgs(n_instances, "");
  auto merge = [&codes, &msgs, out](pc_batch* b, const unsigned long long* h, uint32_t first) {
    parallel_for((uint32_t)b->inst.size(), [&](uint32_t i) {
      codes[first + i] = instance_result(b, b->inst[i], h, out + first + i, &msgs[first + i]);
      out[first + i].stats.roots = b->inst[i].roots;
    });
  };
  // A part's host preparation; a batch it still owns is destroyed with it.
  struct Prepared {
    pc_batch* b = nullptr;
    PlanTables t;
    int rc = PC_OK;
    std::string msg;
    ~Prepared() { pc_batch_destroy(b); }
  };
  auto prepare_part = [&](uint32_t part, Prepared& pr) {
    try {
      pr.rc = prepare_batch(instances + first_of(part), first_of(part + 1) - first_of(part), first_of(part),
                            max_root_chunk, &pr.b, pr.t, pr.msg);
    } catch (...) {
      pr.rc = PC_ERR_NOMEM;
      pr.msg = "host allocation";
    }
  };
  Prepared prep[2];
  // the thread preparing the next part, and the part being merged on its own thread (its
  // batch destroyed when the merge is done); both joined on every path
  struct Joined {
    std::thread th;
    ~Joined() {
      if (th.joinable()) th.join();
    }
  } preparer;
  struct Merging {
    std::thread th;
    pc_batch* b = nullptr;
    void finish() {
      if (th.joinable()) th.join();
      pc_batch_destroy(b);
      b = nullptr;
    }
    ~Merging() { finish(); }
  } merging;
  prepare_part(0, prep[0]);
  int rc = PC_OK;
  for (uint32_t part = 0; part < parts && rc == PC_OK; ++part) {
    Prepared& cur = prep[part & 1u];
    Prepared& nxt = prep[(part + 1u) & 1u];
    if (cur.rc != PC_OK) {
      rc = fail(ctx, cur.rc, cur.msg);
      break;
    }
    pc_batch* b = cur.b;
    cur.b = nullptr;
    rc = finalize_device(ctx, b, cur.t);
    if (rc == PC_OK && part + 1 < parts) {
      pc_batch_destroy(nxt.b);
      nxt.b = nullptr;
      nxt.t = PlanTables();
      nxt.rc = PC_OK;
      nxt.msg.clear();
      try {
        preparer.th = std::thread([&prepare_part, &nxt, part]() { prepare_part(part + 1u, nxt); });
      } catch (...) {
        prepare_part(part + 1u, nxt);  // no thread to overlap with: prepare here
      }
    }
    if (rc == PC_OK) rc = pc_batch_run(ctx, b);
    const unsigned long long* h = nullptr;
    // every part but the last has its count table copied back while the next part runs;
    // its merge waits for that copy
    const bool last = part + 1 == parts;
    cudaEvent_t copied = nullptr;
    if (rc == PC_OK) rc = copy_table(ctx, b, (int)(part & 1u), &h, last ? nullptr : &copied);
    merging.finish();  // the previous part's merge read the other stage
    if (preparer.th.joinable()) preparer.th.join();
    if (rc != PC_OK) {
      pc_batch_destroy(b);
      break;
    }
    merging.b = b;
    const uint32_t first = first_of(part);
    // a part's merge once its count table is on the host (false: the copy failed)
    auto merge_copied = [merge, &codes, &msgs](pc_batch* pb, const unsigned long long* ph, uint32_t pfirst,
                                               cudaEvent_t ev) {
      if (ev && cudaEventSynchronize(ev) != cudaSuccess) {
        for (uint32_t i = 0; i < (uint32_t)pb->inst.size(); ++i) {
          codes[pfirst + i] = PC_ERR_CUDA;
          msgs[pfirst + i] = "count table copy failed";
        }
        return false;
      }
      merge(pb, ph, pfirst);
      return true;
    };
    if (last) {
      merge(b, h, first);  // nothing left to overlap with
    } else {
      try {
        merging.th = std::thread([merge_copied, &codes, &msgs, b, h, first, copied]() {
          try {
            if (merge_copied(b, h, first, copied)) release_host_tables(b);
          } catch (...) {
            for (uint32_t i = 0; i < (uint32_t)b->inst.size(); ++i) {
              codes[first + i] = PC_ERR_NOMEM;
              msgs[first + i] = "host allocation";
            }
          }
        });
      } catch (...) {
        merge_copied(b, h, first, copied);  // no thread to overlap with: merge here
      }
    }
  }
  merging.finish();
  if (preparer.th.joinable()) preparer.th.join();
  for (uint32_t i = 0; rc == PC_OK && i < n_instances; ++i)
    if (codes[i] != PC_OK) rc = fail(ctx, codes[i], msgs[i]);
  if (rc != PC_OK)
    for (uint32_t i = 0; i < n_instances; ++i) pc_histogram_free(out + i);
  return rc;
  PC_GUARD_END(ctx)
}

int pc_autotune(pc_context* ctx, pc_plan* p, uint32_t repeats, pc_tuning* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !p || !out) return PC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  repeats = std::max<uint32_t>(1, repeats);
  const bool narrow = p->gmax <= kNarrowMaxGen;
  const int saved[3] = {ctx->opt_config, ctx->opt_driver, ctx->opt_graph};
  double best = 1e300, dflt = 0.0, best_persist = 1e300;
  int best_cfg = kDefaultSweepConfig, best_drv = 0, n = 0, persist_cfg = kDefaultSweepConfig;
  for (int drv = 0; drv < 2; ++drv)
    for (int cfg = 0; cfg < kNumSweepConfigs; ++cfg) {
      if (!narrow && cfg != kDefaultSweepConfig) continue;
      ctx->opt_config = cfg;
      ctx->opt_driver = drv;
      ctx->opt_graph = drv;
      int rc = pc_plan_run(ctx, p);  // warm-up (and graph capture)
      double t_best = 1e300;
      for (uint32_t r = 0; rc == PC_OK && r < repeats; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        rc = pc_plan_run(ctx, p);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        t_best = std::min(t_best, ms);
      }
      if (rc != PC_OK) {
        ctx->opt_config = saved[0];
        ctx->opt_driver = saved[1];
        ctx->opt_graph = saved[2];
        return rc;
      }
      ++n;
      if (drv == 0 && cfg == kDefaultSweepConfig) dflt = t_best;
      if (drv == 1 && t_best < best_persist) {
        best_persist = t_best;
        persist_cfg = cfg;
      }
      if (t_best < best) {
        best = t_best;
        best_cfg = cfg;
        best_drv = drv;
      }
    }
  // within 1% (the spread of single timings) the persistent driver wins: one graph-replayed
  // launch per run and no host round trip per sweep
  if (best_drv == 0 && best_persist <= 1.01 * best) {
    best = best_persist;
    best_cfg = persist_cfg;
    best_drv = 1;
  }
  ctx->opt_config = best_cfg;
  ctx->opt_driver = best_drv;
  ctx->opt_graph = best_drv;
  const SweepKernels& K = sweep_kernels(narrow, p->batched, best_cfg);
  out->config = best_cfg;
  out->driver = best_drv;
  out->threads = K.threads;
  out->cells_per_lane = K.cells;
  out->global_hist = K.global_hist;
  out->candidates = n;
  out->ms = best;
  out->ms_default = dflt;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_batch_autotune(pc_context* ctx, pc_batch* b, uint32_t repeats, pc_tuning* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  return pc_autotune(ctx, b, repeats, out);
  PC_GUARD_END(ctx)
}

int pc_debug_barrier(pc_context* ctx, int starve, double timeout_ms, uint32_t* error_bits, uint32_t* passed) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !error_bits || !passed || !(timeout_ms > 0.0) || timeout_ms > 10000.0)
    return fail(ctx, PC_ERR_INVALID, "timeout must be in (0, 10000] ms");
  if (starve < 0 || starve > 2) return fail(ctx, PC_ERR_INVALID, "starve must be 0, 1 or 2");
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  uint32_t* d = nullptr;  // [0..1] barrier (arrivals, generation), [2] error bits, [3] blocks through
  PC_CUDA(ctx, pc_cuda_malloc(&d, 4 * sizeof(uint32_t)));
  const uint32_t init[4] = {starve == 1 ? 0x40000000u : 0u, 0u, 0u, 0u};
  uint32_t host[4] = {0u, 0u, 0u, 0u};
  const int blocks = std::max(starve == 2 ? 3 : 1, std::min(ctx->sms, 8));
  const unsigned long long t_ns = (unsigned long long)(timeout_ms * 1e6);
  const unsigned long long long_ns = std::min<unsigned long long>(100ull * t_ns, 10000000000ull);  // at most 10 s
  cudaError_t e = pc_cuda_copy(d, init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = (cudaError_t)launch_barrier_probe(d, t_ns, long_ns, d + 2, d + 3, starve, blocks, st);
  if (e == cudaSuccess) e = pc_cuda_copy(host, d, sizeof(host), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = pc_cuda_sync(st);
  pc_cuda_free(d);
  if (e != cudaSuccess) return fail(ctx, PC_ERR_CUDA, std::string("barrier probe: ") + cudaGetErrorString(e));
  *error_bits = host[2];
  *passed = host[3];
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_debug_peak(pc_context* ctx, int kind, double* lane_ops_per_s) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !lane_ops_per_s || kind < 0 || kind > 2) return fail(ctx, PC_ERR_INVALID, "kind must be 0, 1 or 2");
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const int blocks = 4 * std::max(1, ctx->sms);
  double* sink = nullptr;
  PC_CUDA(ctx, pc_cuda_malloc(&sink, 256 * sizeof(double)));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  // a short launch sizes the timed one to about 30 ms
  uint32_t iters = 256;
  float ms = 0.0f;
  for (int round = 0; e == cudaSuccess && round < 4; ++round) {
    e = (cudaError_t)launch_peak_probe(kind, iters, blocks, sink, st);  // warm-up at this size
    if (e == cudaSuccess) e = pc_cuda_event_record(e0, st);
    if (e == cudaSuccess) e = (cudaError_t)launch_peak_probe(kind, iters, blocks, sink, st);
    if (e == cudaSuccess) e = pc_cuda_event_record(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess || ms >= 20.0f) break;
    const double scale = 30.0 / std::max(0.05, (double)ms);
    iters = (uint32_t)std::min(1e8, std::max(2.0 * iters, iters * scale));
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  pc_cuda_free(sink);
  if (e != cudaSuccess) return fail(ctx, PC_ERR_CUDA, std::string("peak probe: ") + cudaGetErrorString(e));
  *lane_ops_per_s = (double)blocks * 256.0 * 8.0 * iters / (ms * 1e-3);
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_debug_philox(pc_context* ctx, const uint32_t* ctr, uint64_t n, const uint32_t key[2], uint32_t* out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || (n && (!ctr || !out)) || !key) return PC_ERR_INVALID;
  if (n == 0) return PC_OK;
  uint32_t *dc = nullptr, *dout = nullptr;
  PC_CUDA(ctx, pc_cuda_malloc(&dc, n * 16));
  cudaError_t e = pc_cuda_malloc(&dout, n * 16);
  if (e == cudaSuccess) e = pc_cuda_copy(dc, ctr, n * 16, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = (cudaError_t)launch_debug_philox(dc, n, key[0], key[1], dout, ctx->stream);
  if (e == cudaSuccess) e = pc_cuda_copy(out, dout, n * 16, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = pc_cuda_sync(ctx->stream);
  pc_cuda_free(dc);
  pc_cuda_free(dout);
  if (e != cudaSuccess) return fail(ctx, PC_ERR_CUDA, std::string("debug philox: ") + cudaGetErrorString(e));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_debug_normals(pc_context* ctx, uint64_t seed, uint32_t root, uint64_t first_parent, uint64_t count, float* z) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || (count && !z)) return PC_ERR_INVALID;
  if (count == 0) return PC_OK;
  float* dz = nullptr;
  PC_CUDA(ctx, pc_cuda_malloc(&dz, count * sizeof(float)));
  cudaError_t e = (cudaError_t)launch_debug_normals(ctx->zig_dev, (uint32_t)seed, (uint32_t)(seed >> 32), root,
                                                    first_parent, count, dz, ctx->stream);
  if (e == cudaSuccess) e = pc_cuda_copy(z, dz, count * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = pc_cuda_sync(ctx->stream);
  pc_cuda_free(dz);
  if (e != cudaSuccess) return fail(ctx, PC_ERR_CUDA, std::string("debug normals: ") + cudaGetErrorString(e));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_debug_tables(pc_context* ctx, uint32_t* k, uint32_t* w_bits, uint32_t* f_bits) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx) return PC_ERR_INVALID;
  ZigTables t;
  PC_CUDA(ctx, pc_cuda_copy_sync(&t, ctx->zig_dev, sizeof(t), cudaMemcpyDeviceToHost));
  if (k) std::memcpy(k, t.k, sizeof(t.k));
  if (w_bits) std::memcpy(w_bits, t.w, sizeof(t.w));
  if (f_bits) std::memcpy(f_bits, t.f, sizeof(t.f));
  return PC_OK;
  PC_GUARD_END(ctx)
}

}  // extern "C"

// ---- Smoothed (differentiable) form ------------------------------------------------------
struct pc_smooth {
  InstanceHost I;  // bins, phi caps, output value set and (bin, generation) -> value map
  uint32_t ntypes = 0, paths = 1, rows = 1;
  double h = 0.5;
  uint64_t* bin_start_dev = nullptr;
  uint32_t* bin_cap_dev = nullptr;  // [2 nbins]: phi caps, then the bins' launch order
  int32_t* vidx_dev = nullptr;
  uint32_t* inv_off_dev = nullptr;
  uint32_t* inv_idx_dev = nullptr;
  double* e_raw_dev = nullptr;   // [cand_cap][ntypes][nbins][rows]
  double* part_dev = nullptr;    // [cand_cap][nbins][ntypes * 3]
  uint32_t cand_cap = 0;
  double* jac_raw_dev = nullptr;  // [jac_cap][nbins][rows][ntypes * 3], allocated on first use
  uint32_t jac_cap = 0;
  uint32_t* order_dev = nullptr;  // [ntypes][order_cap]: candidates by mean, per type
  uint32_t order_cap = 0;
  float* lin_z_dev = nullptr;      // [lineages][zrow]: every lineage's normals (null: drawn per pass)
  LineageU* lin_u_dev = nullptr;   // [lineages]: every lineage's initial age
  uint32_t zrow = 0;
};

namespace {

SmoothArgs smooth_args(const pc_context* ctx, const pc_smooth* s) {
  SmoothArgs A;
  std::memset(&A, 0, sizeof(A));
  A.k0 = (uint32_t)s->I.seed;
  A.k1 = (uint32_t)(s->I.seed >> 32);
  A.nbins = (uint32_t)s->I.bin_value.size();
  A.rows = s->rows;
  A.ntypes = s->ntypes;
  A.paths = s->paths;
  A.ncells = (uint32_t)s->I.roots;
  A.t_max = s->I.t_max;
  A.inv_h = 1.0 / s->h;
  A.bin_start = s->bin_start_dev;
  A.bin_cap = s->bin_cap_dev;
  A.bin_order = s->bin_cap_dev + s->I.bin_value.size();
  A.zig = ctx->zig_dev;
  A.error = ctx->error_dev;
  A.order = s->order_dev;
  A.lin_z = s->lin_z_dev;
  A.lin_u = s->lin_u_dev;
  A.zrow = s->zrow;
  return A;
}

int order_scratch(pc_context* ctx, pc_smooth* s, uint32_t ncand) {
  if (ncand <= s->order_cap) return PC_OK;
  pc_cuda_free(s->order_dev);
  s->order_dev = nullptr;
  s->order_cap = 0;
  PC_CUDA(ctx, pc_cuda_malloc(&s->order_dev, (size_t)ncand * s->ntypes * sizeof(uint32_t)));
  s->order_cap = ncand;
  return PC_OK;
}

int smooth_scratch(pc_context* ctx, pc_smooth* s, uint32_t ncand) {
  const int rc = order_scratch(ctx, s, ncand);
  if (rc != PC_OK) return rc;
  if (ncand <= s->cand_cap) return PC_OK;
  pc_cuda_free(s->e_raw_dev);
  pc_cuda_free(s->part_dev);
  s->e_raw_dev = nullptr;
  s->part_dev = nullptr;
  s->cand_cap = 0;
  const size_t nb = std::max<size_t>(1, s->I.bin_value.size());
  PC_CUDA(ctx, pc_cuda_malloc(&s->e_raw_dev, (size_t)ncand * s->ntypes * nb * s->rows * sizeof(double)));
  PC_CUDA(ctx, pc_cuda_malloc(&s->part_dev, (size_t)ncand * nb * s->ntypes * 3 * sizeof(double)));
  s->cand_cap = ncand;
  return PC_OK;
}

int jacobian_scratch(pc_context* ctx, pc_smooth* s, uint32_t ncand) {
  const int rc = order_scratch(ctx, s, ncand);
  if (rc != PC_OK) return rc;
  if (ncand <= s->jac_cap) return PC_OK;
  pc_cuda_free(s->jac_raw_dev);
  s->jac_raw_dev = nullptr;
  s->jac_cap = 0;
  const size_t nb = std::max<size_t>(1, s->I.bin_value.size());
  PC_CUDA(ctx, pc_cuda_malloc(&s->jac_raw_dev, (size_t)ncand * nb * s->rows * s->ntypes * 3 * sizeof(double)));
  s->jac_cap = ncand;
  return PC_OK;
}

}  // namespace

extern "C" {

int pc_smooth_create(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, uint32_t n_types, double t_max,
                     double phi, double h, uint32_t paths_per_cell, uint64_t seed, pc_smooth** out) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !out) return fail(ctx, PC_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_types == 0 || n_types > (uint32_t)kSmoothMaxTypes)
    return fail(ctx, PC_ERR_UNSUPPORTED, "the smoothed form supports 1 to 8 cell types");
  if (!(h > 0.0) || std::isinf(h)) return fail(ctx, PC_ERR_INVALID, "h must be finite and > 0");
  if (paths_per_cell == 0) return fail(ctx, PC_ERR_INVALID, "paths_per_cell must be >= 1");
  pc_smooth* s = new (std::nothrow) pc_smooth();
  if (!s) return fail(ctx, PC_ERR_NOMEM, "host allocation");
  std::string msg;
  const pc_cell_type one{1.0, 1.0, 0.0};  // the value set and caps do not depend on the types
  int rc = prepare_instance(bins, n_bins, &one, 1, t_max, phi, seed, s->I, msg);
  if (rc == PC_OK && s->I.gmax + 1 > (uint32_t)kSmoothMaxRows) {
    rc = PC_ERR_UNSUPPORTED;
    msg = "the smoothed form supports at most 63 generations per bin";
  }
  if (rc == PC_OK && (uint64_t)s->I.roots * paths_per_cell > 0xFFFFFFFFull) {
    rc = PC_ERR_UNSUPPORTED;
    msg = "initial cells x paths_per_cell must stay below 2^32";
  }
  if (rc != PC_OK) {
    delete s;
    return fail(ctx, rc, msg);
  }
  s->ntypes = n_types;
  s->paths = paths_per_cell;
  s->h = h;
  s->rows = s->I.gmax + 1;
  InstanceHost& I = s->I;
  const size_t nb = I.bin_value.size();
  std::vector<uint64_t> start(nb + 1, 0);
  for (size_t b = 0; b < nb; ++b) start[b + 1] = start[b] + I.bin_freq[b];
  std::vector<int32_t> vidx(nb * s->rows, -1);
  std::vector<uint32_t> cnt(I.values.size() + 1, 0);
  for (size_t b = 0; b < nb; ++b)
    for (uint32_t g = 0; g <= I.cap[b] && g < I.vidx_stride; ++g) {
      const int32_t v = I.vidx[b * I.vidx_stride + g];
      vidx[b * s->rows + g] = v;
      if (v >= 0) ++cnt[v + 1];
    }
  for (size_t v = 0; v < I.values.size(); ++v) cnt[v + 1] += cnt[v];
  std::vector<uint32_t> inv(cnt.back()), fill(cnt.begin(), cnt.end() - 1);
  for (size_t b = 0; b < nb; ++b)
    for (uint32_t g = 0; g < s->rows; ++g) {
      const int32_t v = vidx[b * s->rows + g];
      if (v >= 0) inv[fill[v]++] = (uint32_t)(b * s->rows + g);
    }
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = pc_cuda_malloc(&s->bin_start_dev, (nb + 1) * sizeof(uint64_t));
  // caps, then the bins in the order their blocks are launched: most expensive first
  // (initial cells x generations), so that the last blocks of a launch are short ones
  std::vector<uint32_t> cap_order(I.cap.begin(), I.cap.end());
  {
    std::vector<uint32_t> order(nb);
    for (size_t b = 0; b < nb; ++b) order[b] = (uint32_t)b;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
      return I.bin_freq[x] * (I.cap[x] + 1ull) > I.bin_freq[y] * (I.cap[y] + 1ull);
    });
    cap_order.insert(cap_order.end(), order.begin(), order.end());
  }
  if (e == cudaSuccess) e = pc_cuda_malloc(&s->bin_cap_dev, std::max<size_t>(1, 2 * nb) * sizeof(uint32_t));
  if (e == cudaSuccess) e = pc_cuda_malloc(&s->vidx_dev, std::max<size_t>(1, vidx.size()) * sizeof(int32_t));
  if (e == cudaSuccess) e = pc_cuda_malloc(&s->inv_off_dev, cnt.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = pc_cuda_malloc(&s->inv_idx_dev, std::max<size_t>(1, inv.size()) * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = pc_cuda_copy(s->bin_start_dev, start.data(), (nb + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nb)
    e = pc_cuda_copy(s->bin_cap_dev, cap_order.data(), 2 * nb * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !vidx.empty())
    e = pc_cuda_copy(s->vidx_dev, vidx.data(), vidx.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = pc_cuda_copy(s->inv_off_dev, cnt.data(), cnt.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !inv.empty())
    e = pc_cuda_copy(s->inv_idx_dev, inv.data(), inv.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  // Every lineage's draws (normals and initial age depend on the seed and the bins, not on
  // the parameters), made once here when they fit in 1 GB: every pass then reads them back
  // instead of drawing them again in each of its (bin, candidate group, type) blocks.
  const uint64_t nlin = s->I.roots * s->paths;
  const uint32_t zrow = (s->rows + 3u) & ~3u;
  const uint64_t lin_bytes = nlin * zrow * sizeof(float) + nlin * sizeof(LineageU);
  if (e == cudaSuccess && ctx->opt_smooth_predraw && nlin > 0 && lin_bytes <= (uint64_t(1) << 30)) {
    s->zrow = zrow;
    e = pc_cuda_malloc(&s->lin_z_dev, nlin * zrow * sizeof(float));
    if (e == cudaSuccess) e = pc_cuda_malloc(&s->lin_u_dev, nlin * sizeof(LineageU));
    if (e == cudaSuccess) e = PC_LAUNCH(launch_smooth_draws(smooth_args(ctx, s), s->lin_z_dev, s->lin_u_dev, st));
  }
  if (e == cudaSuccess) e = pc_cuda_sync(st);
  if (e != cudaSuccess) {
    pc_smooth_destroy(s);
    return fail(ctx, e == cudaErrorMemoryAllocation ? PC_ERR_NOMEM : PC_ERR_CUDA,
                std::string("smoothed plan upload: ") + cudaGetErrorString(e));
  }
  *out = s;
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_smooth_info(const pc_smooth* s, uint64_t* n_values, uint32_t* n_types, uint64_t* n_cells) {
  PC_GUARD_BEGIN
  if (!s) return PC_ERR_INVALID;
  if (n_values) *n_values = s->I.values.size();
  if (n_types) *n_types = s->ntypes;
  if (n_cells) *n_cells = s->I.roots;
  return PC_OK;
  PC_GUARD_END(nullptr)
}

int pc_smooth_values(const pc_smooth* s, double* values) {
  PC_GUARD_BEGIN
  if (!s || (!values && !s->I.values.empty())) return PC_ERR_INVALID;
  if (!s->I.values.empty()) std::memcpy(values, s->I.values.data(), s->I.values.size() * sizeof(double));
  return PC_OK;
  PC_GUARD_END(nullptr)
}

int pc_smooth_forward(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                      double* expected) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !s || (n_candidates && (!params || !expected))) return fail(ctx, PC_ERR_INVALID, "null argument");
  if (n_candidates == 0) return PC_OK;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = smooth_scratch(ctx, s, n_candidates);
  if (rc != PC_OK) return rc;
  const SmoothArgs A = smooth_args(ctx, s);
  const uint32_t nv = (uint32_t)s->I.values.size();
  PC_CUDA(ctx, PC_LAUNCH(launch_smooth_forward(A, params, n_candidates, s->e_raw_dev, ctx->stream)));
  PC_CUDA(ctx, PC_LAUNCH(launch_smooth_merge(s->e_raw_dev, n_candidates, A.ntypes, A.nbins * A.rows,
                                                s->inv_off_dev, s->inv_idx_dev, nv, expected, ctx->stream)));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_smooth_backward(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                       const double* grad_expected, double* grad_params) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !s || (n_candidates && (!params || !grad_expected || !grad_params)))
    return fail(ctx, PC_ERR_INVALID, "null argument");
  if (n_candidates == 0) return PC_OK;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = smooth_scratch(ctx, s, n_candidates);
  if (rc != PC_OK) return rc;
  const SmoothArgs A = smooth_args(ctx, s);
  PC_CUDA(ctx, PC_LAUNCH(launch_smooth_backward(A, params, n_candidates, grad_expected,
                                                   (uint32_t)s->I.values.size(), s->vidx_dev, s->part_dev,
                                                   grad_params, ctx->stream)));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_smooth_jacobian(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                       double* expected, double* jacobian) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !s || (n_candidates && (!params || !expected || !jacobian)))
    return fail(ctx, PC_ERR_INVALID, "null argument");
  if (n_candidates == 0) return PC_OK;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = jacobian_scratch(ctx, s, n_candidates);
  if (rc != PC_OK) return rc;
  const SmoothArgs A = smooth_args(ctx, s);
  PC_CUDA(ctx, PC_LAUNCH(launch_smooth_jacobian(A, params, n_candidates, s->inv_off_dev, s->inv_idx_dev,
                                                   (uint32_t)s->I.values.size(), s->jac_raw_dev, expected,
                                                   jacobian, ctx->stream)));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_smooth_gauss_newton(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                           const double* target, double* loss, double* jtj, double* jtr) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx || !s || (n_candidates && (!params || !target || !loss || !jtj || !jtr)))
    return fail(ctx, PC_ERR_INVALID, "null argument");
  if (n_candidates == 0) return PC_OK;
  PC_CUDA(ctx, cudaSetDevice(ctx->device));
  int rc = jacobian_scratch(ctx, s, n_candidates);
  if (rc != PC_OK) return rc;
  const SmoothArgs A = smooth_args(ctx, s);
  PC_CUDA(ctx, PC_LAUNCH(launch_smooth_gauss_newton(A, params, n_candidates, s->inv_off_dev, s->inv_idx_dev,
                                                       (uint32_t)s->I.values.size(), target, s->jac_raw_dev, loss,
                                                       jtj, jtr, ctx->stream)));
  return PC_OK;
  PC_GUARD_END(ctx)
}

int pc_smooth_sync(pc_context* ctx) {
  PC_GUARD_BEGIN
  FaultScope fault_scope__(ctx);
  if (!ctx) return PC_ERR_INVALID;
  PC_CUDA(ctx, pc_cuda_sync(ctx->stream));
  uint32_t err = 0;
  PC_CUDA(ctx, pc_cuda_copy_sync(&err, ctx->error_dev, sizeof(err), cudaMemcpyDeviceToHost));
  if (err & 2u) return fail(ctx, PC_ERR_CUDA, "internal: the normal sampler exceeded its rejection budget");
  return PC_OK;
  PC_GUARD_END(ctx)
}

void pc_smooth_destroy(pc_smooth* s) {
  if (!s) return;
  pc_cuda_free(s->bin_start_dev);
  pc_cuda_free(s->bin_cap_dev);
  pc_cuda_free(s->vidx_dev);
  pc_cuda_free(s->inv_off_dev);
  pc_cuda_free(s->inv_idx_dev);
  pc_cuda_free(s->e_raw_dev);
  pc_cuda_free(s->part_dev);
  pc_cuda_free(s->jac_raw_dev);
  pc_cuda_free(s->order_dev);
  pc_cuda_free(s->lin_z_dev);
  pc_cuda_free(s->lin_u_dev);
  delete s;
}

}  // extern "C"

