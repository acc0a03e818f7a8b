// pc_simulate_noalloc: the whole plain simulation without allocating anything.
//
// Some callers cannot allocate device memory: code that runs inside a host application
// which owns every byte of the GPU through its own pool (the pool would not see a
// cudaMalloc and a cudaMalloc can fail or fragment it), code that must not trigger the
// implicit device synchronisation cudaMalloc/cudaFree imply, and code with a fixed memory
// budget certified in advance. For them this entry point keeps every intermediate (the
// uploaded inputs, the per-bin tables, the root records, the level buffers and the
// (generation, bin, type) counts) in one file-scope device array of PC_NOALLOC_SCRATCH_BYTES,
// which every GPU that loads the library reserves until the process exits. It calls no
// cudaMalloc, cudaFree or other allocating routine, and no host heap allocation either:
// host-side tables live on the stack and per-bin tables are built by a device kernel.
//
// The array is shared by all calls and keeps the last call's contents; each call clears
// what must start at zero (counts, statistics, error flags, level-buffer tickets). Calls
// that overlap on the GPU (two streams, two host threads) race on the array: callers
// serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/procell.h"
#include "pc_engine.h"

namespace pc {
namespace {

static __device__ __align__(256) unsigned char g_scratch[PC_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
constexpr int kMaxBufs = 42;  // level buffers: at most min(gmax, 40) + 2

struct DeviceSetup {
  unsigned char* scratch;  // device address of g_scratch on this device
  int sms, root_bps, div_bps;
};
std::mutex g_mutex;
DeviceSetup g_dev[kMaxDevices];
bool g_ready[kMaxDevices];

int fail(char* err, size_t len, int code, const char* msg) {
  if (err && len) {
    std::strncpy(err, msg, len - 1);
    err[len - 1] = '\0';
  }
  return code;
}

int fail_cuda(char* err, size_t len, const char* what, cudaError_t e) {
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return fail(err, len, e == cudaErrorMemoryAllocation ? PC_ERR_NOMEM : PC_ERR_CUDA, buf);
}

uint64_t align256(uint64_t x) { return (x + 255u) & ~uint64_t(255u); }

// Per-bin tables from the caller's rows, on the device (one block): the nonzero rows in
// file order become bins with their phi cap, countability and first root, exactly as
// pc_plan_create derives them on the host.
__global__ void k_noalloc_bins(const pc_bin* rows, uint64_t nrows, double phi, uint32_t g_store_max,
                               uint32_t* bin_info, unsigned long long* bin_start) {
  __shared__ unsigned long long s_n[1024], s_f[1024];
  const uint32_t t = threadIdx.x;
  const uint64_t per = (nrows + blockDim.x - 1) / blockDim.x;
  const uint64_t b = min(nrows, (uint64_t)t * per), e = min(nrows, b + per);
  unsigned long long cnt = 0, fr = 0;
  for (uint64_t i = b; i < e; ++i)
    if (rows[i].frequency) {
      ++cnt;
      fr += rows[i].frequency;
    }
  s_n[t] = cnt;
  s_f[t] = fr;
  __syncthreads();
  if (t == 0) {
    unsigned long long rn = 0, rf = 0;
    for (uint32_t i = 0; i < blockDim.x; ++i) {
      const unsigned long long a = s_n[i], c = s_f[i];
      s_n[i] = rn;
      s_f[i] = rf;
      rn += a;
      rf += c;
    }
    bin_start[rn] = rf;
  }
  __syncthreads();
  unsigned long long bi = s_n[t], start = s_f[t];
  for (uint64_t i = b; i < e; ++i) {
    if (!rows[i].frequency) continue;
    const double v = rows[i].value;
    uint32_t c = 0;
    for (double f = v; f / 2 > phi && c < 4096u; f = f / 2) ++c;
    uint32_t clamped = 0;
    if (c > g_store_max + 1u) {
      c = g_store_max + 1u;
      clamped = 0x200u;
    }
    bin_info[bi] = c | (v >= phi ? 0x100u : 0u) | clamped;
    bin_start[bi] = start;
    start += rows[i].frequency;
    ++bi;
  }
}

struct Buf {
  ulonglong2* cells;
  unsigned long long* count;
  unsigned long long* prefix;
  uint32_t* ticket;
  bool busy;
};

}  // namespace
}  // namespace pc

using namespace pc;

extern "C" int pc_simulate_noalloc(const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                                   uint32_t n_types, double t_max, double phi, uint64_t seed, void* stream,
                                   uint64_t* raw_counts, uint64_t capacity, uint32_t dims[3],
                                   pc_stats* stats, char* err, size_t err_len) {
  if ((n_bins && !bins) || (n_types && !types) || !dims) return fail(err, err_len, PC_ERR_INVALID, "null argument");
  dims[0] = dims[1] = dims[2] = 0;
  if (!(t_max >= 0.0) || std::isinf(t_max)) return fail(err, err_len, PC_ERR_INVALID, "t_max must be finite and >= 0");
  if (!(phi >= 0.0) || std::isinf(phi))
    return fail(err, err_len, PC_ERR_INVALID, "phi must be finite and > 0 (0 = automatic)");
  if (n_types == 0)
    return fail(err, err_len, PC_ERR_INVALID,
                "ERROR: proportion distribution of cell types does not sum to 1, aborting.");
  if (n_types > (uint32_t)kMaxTypes) return fail(err, err_len, PC_ERR_UNSUPPORTED, "at most 64 cell types are supported");
  cudaStream_t st = (cudaStream_t)stream;

  // --- host plan, in fixed-size storage (the same rules as pc_plan_create) -----------
  double threshold = phi;
  if (threshold == 0.0)
    for (uint64_t i = 0; i < n_bins; ++i)
      if (bins[i].frequency > 0 && (threshold == 0.0 || bins[i].value < threshold)) threshold = bins[i].value;
  if (!(threshold > 0.0) || std::isinf(threshold)) return fail(err, err_len, PC_ERR_INVALID, "phi must be finite and > 0");
  const double tmax = (t_max == 0.0) ? 0.0 : t_max;
  uint64_t nb = 0, total = 0;
  uint32_t gmax = 0;
  for (uint64_t i = 0; i < n_bins; ++i) {
    if (bins[i].frequency == 0) continue;
    if (!std::isfinite(bins[i].value)) return fail(err, err_len, PC_ERR_INVALID, "histogram values must be finite");
    if (bins[i].frequency > 0xFFFFFFFFull - total)
      return fail(err, err_len, PC_ERR_UNSUPPORTED, "more than 2^32-1 initial cells");
    total += bins[i].frequency;
    ++nb;
    uint32_t c = 0;
    for (double f = bins[i].value; f / 2 > threshold && c < 4096; f = f / 2) ++c;
    gmax = std::max(gmax, c);
  }
  if (nb >= (1u << 24)) return fail(err, err_len, PC_ERR_UNSUPPORTED, "at most 2^24 nonzero bins");

  double sum = 0.0;
  for (uint32_t i = 0; i < n_types; ++i) {
    if (!std::isfinite(types[i].ratio) || !std::isfinite(types[i].mean) || !std::isfinite(types[i].sd))
      return fail(err, err_len, PC_ERR_INVALID, "cell type parameters must be finite");
    if (types[i].mean > 0.0 && !(std::fabs(types[i].sd) < kMaxSigma))
      return fail(err, err_len, PC_ERR_UNSUPPORTED, "cell type standard deviations must be below 2^127");
    sum += types[i].ratio;
  }
  if (std::fabs(1.0 - sum) > 1.0 / std::pow(10.0, 8.0))
    return fail(err, err_len, PC_ERR_INVALID,
                "ERROR: proportion distribution of cell types does not sum to 1, aborting.");
  uint32_t order[kMaxTypes];
  for (uint32_t i = 0; i < n_types; ++i) order[i] = i;
  for (uint32_t i = 1; i < n_types; ++i) {  // stable insertion sort, ratio descending
    const uint32_t o = order[i];
    uint32_t j = i;
    while (j > 0 && types[order[j - 1]].ratio < types[o].ratio) {
      order[j] = order[j - 1];
      --j;
    }
    order[j] = o;
  }
  TypeDev tdev[kMaxTypes];
  double acc = 0.0;
  uint32_t fallback = 0;
  for (uint32_t s = 0; s < n_types; ++s) {
    const pc_cell_type& src = types[order[s]];
    TypeDev& t = tdev[s];
    std::memset(&t, 0, sizeof(t));
    acc += src.ratio;
    t.cum = acc;
    t.mu = src.mean;
    t.sigma = std::ldexp(src.sd, kSigmaShift);
    t.t_max = tmax;
    t.mode = src.mean < 0.0 ? kModeQuiescent : (src.mean == 0.0 ? kModeZeroMean : kModeNormal);
    host_truncation_bounds(src.mean, src.sd, t.zlo, t.zhi);
    if (t.mode == kModeZeroMean) {
      t.sigma = 0.0;
      t.zlo = -INFINITY;
      t.zhi = INFINITY;
    }
    if (src.ratio > 0.0) fallback = s;
  }

  // key layout (as pc_plan_create): the generation limit follows the full root count
  const KeyLayout kl = key_layout(total, gmax, false, 0);
  const uint32_t g_store_max = kl.g_store_max;
  const uint32_t hist_gens = std::min(gmax, g_store_max + 1) + 1;
  const uint64_t hist_elems = (uint64_t)hist_gens * nb * n_types;
  dims[0] = hist_gens;
  dims[1] = (uint32_t)nb;
  dims[2] = n_types;
  if (!raw_counts || capacity < hist_elems) {
    char b[160];
    std::snprintf(b, sizeof(b), "raw count buffer holds %llu of the %llu counts needed (dims are set)",
                  (unsigned long long)capacity, (unsigned long long)hist_elems);
    return fail(err, err_len, PC_ERR_INVALID, b);
  }

  // --- per-device set-up: the device address of the scratch array --------------------
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda(err, err_len, "cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return fail(err, err_len, PC_ERR_UNSUPPORTED, "device ordinal >= 64");
  DeviceSetup ds;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_ready[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess) return fail_cuda(err, err_len, "cudaGetSymbolAddress", e);
      DeviceSetup d;
      d.scratch = (unsigned char*)p;
      e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return fail_cuda(err, err_len, "cudaDeviceGetAttribute", e);
      const int oe = occupancy_blocks_per_sm(&d.root_bps, &d.div_bps);
      if (oe != 0) return fail_cuda(err, err_len, "occupancy query", (cudaError_t)oe);
      g_dev[dev] = d;
      g_ready[dev] = true;
    }
    ds = g_dev[dev];
  }

  // --- scratch layout ------------------------------------------------------------------
  const uint32_t max_blocks = (uint32_t)std::max(1, ds.sms);  // one block per SM per launch
  const uint32_t segs = max_blocks * kWarpsPerBlock;
  uint64_t off = 0;
  const uint64_t rows_off = off;
  off = align256(off + 16ull * n_bins);
  const uint64_t info_off = off;
  off = align256(off + 4ull * nb);
  const uint64_t start_off = off;
  off = align256(off + 8ull * (nb + 1));
  const uint64_t types_off = off;
  off = align256(off + sizeof(TypeDev) * n_types);
  const uint64_t zig_off = off;
  off = align256(off + sizeof(ZigTables));
  const uint64_t stats_off = off;
  off = align256(off + 64);
  const uint64_t hist_off = off;
  off = align256(off + 8ull * hist_elems);
  const uint64_t fixed = off;
  const uint32_t levels = std::min<uint32_t>(gmax, 40u) + 2u;
  const uint64_t per_buf_extra = align256(8ull * segs) + align256(8ull * (segs + 1)) + 256;
  uint64_t cells = 0;
  if (fixed + 4096 < (uint64_t)PC_NOALLOC_SCRATCH_BYTES) {
    const uint64_t room = (uint64_t)PC_NOALLOC_SCRATCH_BYTES - fixed - 4096;  // alignment slack
    if (room > levels * (per_buf_extra + 256)) cells = (room - levels * (per_buf_extra + 256)) / (8 + 16ull * levels);
  }
  if (cells < 4ull * segs + 1024) {
    char b[200];
    std::snprintf(b, sizeof(b),
                  "input needs more than the %u-byte allocation-free scratch (%llu bytes of inputs, tables and "
                  "counts before the level buffers)",
                  (unsigned)PC_NOALLOC_SCRATCH_BYTES, (unsigned long long)fixed);
    return fail(err, err_len, PC_ERR_NOMEM, b);
  }
  const uint64_t chunk = std::min<uint64_t>(std::max<uint64_t>(1, total), std::min<uint64_t>(kl.chunk, cells - segs));
  const uint64_t rec_off = align256(fixed);
  uint64_t boff = align256(rec_off + 8ull * chunk);
  Buf bufs[kMaxBufs];
  unsigned char* const S = ds.scratch;
  for (uint32_t i = 0; i < levels; ++i) {
    bufs[i].cells = (ulonglong2*)(S + boff);
    boff = align256(boff + 16ull * cells);
    bufs[i].count = (unsigned long long*)(S + boff);
    boff += align256(8ull * segs);
    bufs[i].prefix = (unsigned long long*)(S + boff);
    boff += align256(8ull * (segs + 1));
    bufs[i].ticket = (uint32_t*)(S + boff);
    boff += 256;
    bufs[i].busy = false;
  }
  if (boff > (uint64_t)PC_NOALLOC_SCRATCH_BYTES) return fail(err, err_len, PC_ERR_NOMEM, "internal: scratch layout overflow");
  const uint64_t max_slice = (cells - 2ull * segs) / 2;

  // --- uploads and clearing (no allocation: copies into the scratch array) ------------
  const ZigTables zig = host_zig_tables();
  unsigned long long* stats_dev = (unsigned long long*)(S + stats_off);
  uint32_t* error_dev = (uint32_t*)(S + stats_off + 32);
  if (n_bins) e = cudaMemcpyAsync(S + rows_off, bins, 16ull * n_bins, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + types_off, tdev, sizeof(TypeDev) * n_types, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S + zig_off, &zig, sizeof(ZigTables), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S + stats_off, 0, 64, st);
  if (e == cudaSuccess && hist_elems) e = cudaMemsetAsync(S + hist_off, 0, 8ull * hist_elems, st);
  for (uint32_t i = 0; e == cudaSuccess && i < levels; ++i) e = cudaMemsetAsync(bufs[i].ticket, 0, 4, st);
  if (e == cudaSuccess && nb) {
    k_noalloc_bins<<<1, 1024, 0, st>>>((const pc_bin*)(S + rows_off), n_bins, threshold, g_store_max,
                                       (uint32_t*)(S + info_off), (unsigned long long*)(S + start_off));
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail_cuda(err, err_len, "upload", e);

  RunArgs a;
  std::memset(&a, 0, sizeof(a));
  a.k0 = (uint32_t)seed;
  a.k1 = (uint32_t)(seed >> 32);
  philox_key_schedule(a.k0, a.k1, a.ks);
  a.t_max = tmax;
  a.ntypes = n_types;
  a.nbins = (uint32_t)nb;
  a.nclass = (uint32_t)(nb * n_types);
  a.fallback = fallback;
  a.hist_gens = hist_gens;
  a.g_store_max = g_store_max;
  a.types = (const TypeDev*)(S + types_off);
  a.zig = (const ZigTables*)(S + zig_off);
  a.bin_info = (const uint32_t*)(S + info_off);
  a.bin_start = (const uint64_t*)(S + start_off);
  a.root_rec = (unsigned long long*)(S + rec_off);
  a.rec_cap = chunk;
  a.hist = (unsigned long long*)(S + hist_off);
  a.stats = stats_dev;
  a.error = error_dev;
  const bool narrow = kl.narrow;

  // --- root chunks, then generation slices depth-first (as pc_plan_run) ---------------
  struct Entry {
    int buf;
    uint32_t gen, nseg;
    uint64_t stride, pos, n;
  };
  Entry stack[kMaxBufs];
  int depth = 0;
  auto acquire = [&]() -> int {
    for (uint32_t i = 0; i < levels; ++i)
      if (!bufs[i].busy) {
        bufs[i].busy = true;
        return (int)i;
      }
    return -1;
  };
  auto grid = [&](uint64_t n) -> int {
    const uint64_t want = (n + (uint64_t)kBlock * 4 - 1) / ((uint64_t)kBlock * 4);
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, max_blocks));
  };
  uint64_t total_h = 0, divisions = 0;
  uint32_t sweeps = 0, max_gen = 0;
  for (uint64_t c0 = 0; c0 < total; c0 += chunk) {
    const uint64_t n = std::min<uint64_t>(chunk, total - c0);
    a.root_base = c0;
    const int b0 = acquire();
    if (b0 < 0) return fail(err, err_len, PC_ERR_NOMEM, "internal: no free level buffer");
    const int blocks = grid(n);
    const uint32_t nseg = (uint32_t)blocks * kWarpsPerBlock;
    const LevelOut o{bufs[b0].cells, bufs[b0].count, bufs[b0].prefix, bufs[b0].ticket, (n + nseg - 1) / nseg};
    e = (cudaError_t)launch_root_sweep(a, 0, n, o, blocks, narrow, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total_h, bufs[b0].prefix + nseg, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(err, err_len, "root sweep", e);
    if (total_h == 0) {
      bufs[b0].busy = false;
      continue;
    }
    stack[depth++] = Entry{b0, 0u, nseg, o.stride, 0, total_h};
    while (depth > 0) {
      Entry& top = stack[depth - 1];
      const uint64_t len = std::min<uint64_t>(top.n - top.pos, max_slice);
      const int bo = acquire();
      if (bo < 0) return fail(err, err_len, PC_ERR_NOMEM, "lineages deeper than the scratch's level buffers");
      const int blocks_d = grid(len);
      const uint32_t oseg = (uint32_t)blocks_d * kWarpsPerBlock;
      const LevelIn li{bufs[top.buf].cells, bufs[top.buf].prefix, top.nseg, top.stride, top.pos, top.pos + len};
      const LevelOut lo{bufs[bo].cells, bufs[bo].count, bufs[bo].prefix, bufs[bo].ticket,
                        2 * ((len + oseg - 1) / oseg)};
      const uint32_t gen = top.gen;
      e = (cudaError_t)launch_divide_sweep(a, li, gen, lo, blocks_d, narrow, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&total_h, bufs[bo].prefix + oseg, 8, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return fail_cuda(err, err_len, "division sweep", e);
      divisions += len;
      ++sweeps;
      max_gen = std::max(max_gen, gen + 1);
      top.pos += len;
      if (top.pos == top.n) {
        bufs[top.buf].busy = false;
        --depth;
      }
      if (total_h > 0 && gen + 1 <= g_store_max) {
        if (depth >= kMaxBufs) return fail(err, err_len, PC_ERR_NOMEM, "internal: level stack overflow");
        stack[depth++] = Entry{bo, gen + 1, oseg, lo.stride, 0, total_h};
      } else {
        bufs[bo].busy = false;
      }
    }
  }

  // --- results: counts to the caller's buffer, types into file order -------------------
  unsigned long long st_h[5] = {0, 0, 0, 0, 0};
  if (hist_elems) e = cudaMemcpyAsync(raw_counts, S + hist_off, 8ull * hist_elems, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st_h, stats_dev, 40, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_cuda(err, err_len, "result copy", e);
  uint64_t leaves = 0;
  uint64_t row[kMaxTypes];
  for (uint64_t gb = 0; gb < (uint64_t)hist_gens * nb; ++gb) {
    uint64_t* r = raw_counts + gb * n_types;
    for (uint32_t k = 0; k < n_types; ++k) {
      row[order[k]] = r[k];
      leaves += r[k];
    }
    std::memcpy(r, row, 8ull * n_types);
  }
  const uint32_t flags = (uint32_t)(st_h[4] & 0xFFFFFFFFu);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->roots = total;
    stats->divisions = divisions;
    stats->leaves = leaves;
    stats->uncounted = st_h[1];
    stats->vanished = st_h[0];
    stats->max_generation = max_gen;
    stats->sweeps = sweeps;
    stats->root_sweeps = (uint32_t)((total + chunk - 1) / chunk);
    stats->kernel_launches = sweeps + stats->root_sweeps + 1u;  // + the bin setup kernel
    stats->h2d_bytes = 16ull * n_bins + sizeof(TypeDev) * n_types + sizeof(ZigTables);
    stats->d2h_bytes = 8ull * hist_elems + 40 + 8ull * (sweeps + (total + chunk - 1) / chunk);
  }
  if (flags & 16u) return fail(err, err_len, PC_ERR_INTERNAL, "internal: a device bounds check failed (checked build)");
  if (flags & 2u) return fail(err, err_len, PC_ERR_CUDA, "internal: the normal sampler exceeded its rejection budget");
  if (flags & 1u)
    return fail(err, err_len, PC_ERR_DEPTH, "a lineage exceeded the deepest generation the key layout holds");
  return PC_OK;
}
