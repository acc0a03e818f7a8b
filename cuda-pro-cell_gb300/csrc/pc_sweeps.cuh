// Device code of the proliferation sweeps, shared by the translation units that
// instantiate it (pc_kernels.cu: the wide key layout and the diagnostics; pc_tuned_*.cu:
// the narrow layout in every tuned configuration).
//
// The reference runs one thread per cell and recurses one tree level per CUDA Dynamic
// Parallelism child grid (device::proliferate, src/simulation/proliferation.cu:289-402),
// reading 40-byte cells from full-size level buffers that are mostly empty. Here each
// generation is one data-parallel sweep over a dense, sorted buffer of the cells that
// will divide:
//
//   root sweep     one lane per initial cell: type, first division time and initial age
//                  (create_cell with type -1, src/simulation/cell.cu:25-79), then either
//                  a gen-0 leaf, a vanished root, or a dividing cell written to level 0.
//   division sweep one lane per dividing cell of generation g: one Philox block gives both
//                  daughters' first-attempt normals, the daughters' due times are
//                  computed, leaves (due > t_max, proliferation.cu:404-410) are counted
//                  straight into the (generation, bin, type) histogram and never stored,
//                  and daughters that will divide again are written to level g+1.
//
// Memory traffic per division is one 16-byte read plus one 16-byte write per daughter
// that divides again; leaves and vanished cells cost no HBM bytes. Each warp owns a
// contiguous slice of the input and its own output segment, so compaction needs only
// warp ballots, and the output stays sorted by (root, path) with no atomics.
//
// Two drivers run the sweeps: one launch per sweep (k_roots, k_divide; the host reads
// each level's size) or one persistent cooperative launch for a whole run (k_persist),
// whose blocks walk the same schedule on the device with grid barriers between sweeps.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "pc_engine.h"

namespace pc {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

// A compiled configuration of the sweeps: threads per block, input cells each lane
// carries per step of the division sweep, and leaf-count privatisation (false: a window
// of classes in shared memory per block; true: warp-aggregated atomics to the global
// table). Every configuration is compiled for 64 registers per thread (1024 resident
// threads per SM).
template <int kThreads_, int kCells_, bool kGlobalHist_>
struct Cfg {
  static constexpr int kThreads = kThreads_;
  static constexpr int kWarps = kThreads_ / 32;
  static constexpr int kCells = kCells_;
  static constexpr bool kGlobalHist = kGlobalHist_;
  static constexpr int kMinBlocks = 1024 / kThreads_;
};
using DefaultCfg = Cfg<256, 1, false>;

// Loads of data that the same launch may have written (level buffers and their prefixes,
// root records): the persistent driver reads them coherently (L2 for the streamed cells,
// ordinary loads for the root records, both ordered by its grid barrier); the one-launch-
// per-sweep driver uses the read-only path.
template <bool Coherent, class T>
__device__ __forceinline__ T ld_level(const T* p) {
  if constexpr (Coherent)
    return __ldcg(p);
  else
    return __ldg(p);
}
template <bool Coherent>
__device__ __forceinline__ unsigned long long ld_rec(const unsigned long long* p) {
  if constexpr (Coherent)
    return *p;
  else
    return __ldg(p);
}

// Bounds checks of the checked build (compiled with PC_CHECKED, the stand-in for a memory
// sanitizer): a failed check sets error bit 4 (value 16) and the caller skips the access or
// uses a safe value; nothing traps. In the normal build every check is true at compile time.
__device__ __forceinline__ bool in_bounds(bool ok, uint32_t* error) {
#ifdef PC_CHECKED
  if (!ok) atomicOr(error, 16u);
  return ok;
#else
  (void)ok;
  (void)error;
  return true;
#endif
}

struct Smem {
  ZigTables zig;
  TypeDev types[kMaxTypes];  // plain form only
  __device__ __forceinline__ const ZigTables& zig_or(const RunArgs&) const { return zig; }
};

__device__ __forceinline__ void stage(Smem& s, const RunArgs& a) {
  const uint32_t* zs = reinterpret_cast<const uint32_t*>(a.zig);
  uint32_t* zd = reinterpret_cast<uint32_t*>(&s.zig);
  for (uint32_t i = threadIdx.x; i < sizeof(ZigTables) / 4; i += blockDim.x) zd[i] = __ldg(zs + i);
  if (a.btypes) return;  // batched form: types come from the batch table
  const uint32_t* ts = reinterpret_cast<const uint32_t*>(a.types);
  uint32_t* td = reinterpret_cast<uint32_t*>(s.types);
  const uint32_t nt = a.ntypes * (uint32_t)(sizeof(TypeDev) / 4);
  for (uint32_t i = threadIdx.x; i < nt; i += blockDim.x) td[i] = __ldg(ts + i);
}

// Rejection path of one daughter's normal: the generic ziggurat plus the truncation
// tau > 0 (src/simulation/cell.cu:114-118), drawing from the node's private stream.
// A round budget far beyond anything a correct table produces (the acceptance rate of a
// round is above 1/2) turns a would-be endless loop into error bit 1.
constexpr uint32_t kRoundBudget = 1u << 16;

__device__ __noinline__ float slow_z(uint32_t j, uint32_t layer, uint32_t wedge, uint64_t node,
                                     uint32_t root, uint32_t k0, uint32_t k1, float zlo, float zhi,
                                     const ZigTables& Z, uint32_t* error) {
  ChildStream cs = child_stream(node, root, k0, k1);
  uint32_t budget = kRoundBudget;
  bool have_wedge = true;
  while (budget > 0u) {
    const float z = zig_normal(j, layer, have_wedge, wedge, cs, Z, budget);
    if (budget == 0u) break;
    if (z >= zlo && z <= zhi) return z;
    have_wedge = false;
    j = cs.next();
    layer = cs.next() & kZigLayerMask;
    --budget;
  }
  atomicOr(error, 2u);
  return 0.0f;
}

// First-attempt fast path (about 99.6% of draws): one strip test, one FP32 multiply.
__device__ __forceinline__ float draw_z(uint32_t j, uint32_t layer, uint32_t wedge, uint64_t node,
                                        uint32_t root, uint32_t k0, uint32_t k1, float zlo, float zhi,
                                        const ZigTables& Z, uint32_t* error) {
  const uint32_t mag = j & 0x7FFFFFFFu;
  if (mag < Z.k[layer]) {
    const float x = __fmul_rn((float)mag, Z.w[layer]);
    const float z = (j >> 31) ? -x : x;
    if (z >= zlo && z <= zhi) return z;
  }
  return slow_z(j, layer, wedge, node, root, k0, k1, zlo, zhi, Z, error);
}

enum Fate : int { kNone = 0, kLeaf = 1, kEmit = 2, kVanish = 3 };

// GB300 runs FP64 arithmetic and every FP64<->FP32 conversion on a pipe of 2 lanes per
// clock per SM, so the conversion and the comparison below are done on the bits instead.
//
// z x 2^-kSigmaShift as a double, exactly, for every finite float (zero and subnormals
// included): the float's sign, exponent and mantissa move into the double's fields
// unchanged (an arithmetic shift by 3 carries the sign, the mask clears the three bits it
// copied into the exponent's top), where the double's bias, 896 larger, reads them. The
// sweeps pair it with the type's sd stored as sd x 2^kSigmaShift, so fma(sigma, widen(z),
// mu) is fma(sd, z, mean) bit for bit: two integer operations, no rebias and no zero test.
__device__ __forceinline__ double widen_scaled(float z) {
  const uint32_t f = __float_as_uint(z);
  return __hiloint2double((int)((uint32_t)((int32_t)f >> 3) & 0x8FFFFFFFu), (int)(f << 29));
}
static_assert(kSigmaShift == 1023 - 127, "the float's exponent field read with the double's bias");

// a > b for non-negative doubles (IEEE order equals integer order of the bit patterns).
__device__ __forceinline__ bool gt_nonneg(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}

// What a cell's type, and in the batched form its instance, supplies to the sweeps.
struct TypeCtx {
  double mu, sigma;     // mean, sd x 2^kSigmaShift: tau = fma(sigma, widen_scaled(z), mu)
  float zlo, zhi;       // truncation bounds on z
  double t_max;
  uint64_t root_begin;  // batch index of the instance's first initial cell
  uint32_t k0, k1;      // the instance's seed
};

// The type's parameters from shared memory (plain form) or the batch table (batched form,
// one entry per type of every instance), in three 16-byte loads at most.
template <bool Batched>
__device__ __forceinline__ TypeCtx type_ctx(const RunArgs& a, const TypeDev* smem_types, uint32_t ty) {
  TypeCtx c;
  if (Batched) {
    const uint4* q = reinterpret_cast<const uint4*>(a.btypes + ty);
    const uint4 q0 = __ldg(q), q1 = __ldg(q + 1), q3 = __ldg(q + 3);
    c.mu = __hiloint2double((int)q0.y, (int)q0.x);
    c.sigma = __hiloint2double((int)q0.w, (int)q0.z);
    c.zlo = __uint_as_float(q1.x);
    c.zhi = __uint_as_float(q1.y);
    c.t_max = __hiloint2double((int)q1.w, (int)q1.z);
    c.k0 = q3.x;
    c.k1 = q3.y;
    c.root_begin = ((uint64_t)q3.w << 32) | q3.z;
  } else {
    const TypeDev* t = smem_types + ty;
    const double2 ms = *reinterpret_cast<const double2*>(&t->mu);
    const float2 z = *reinterpret_cast<const float2*>(&t->zlo);
    c.mu = ms.x;
    c.sigma = ms.y;
    c.zlo = z.x;
    c.zhi = z.y;
    c.t_max = a.t_max;
    c.root_begin = 0;
    c.k0 = a.k0;
    c.k1 = a.k1;
  }
  return c;
}

// Root record fields (layout in pc_engine.h).
__device__ __forceinline__ uint32_t rec_type(unsigned long long r) { return (uint32_t)(r >> 32) & 0xFFFFu; }
__device__ __forceinline__ uint32_t rec_cap(unsigned long long r) { return (uint32_t)(r >> 48) & 0xFFu; }
__device__ __forceinline__ bool rec_clamped(unsigned long long r) { return ((r >> 57) & 1ull) != 0ull; }

// Fate of one daughter born at `birth` with normal z: due = birth + fma(sd, z, mean), the
// reference's t + timer; a leaf if due > t_max (proliferation.cu:404-410), else it divides
// again when its phi cap allows and vanishes when not.
__device__ __forceinline__ int fate(double birth, float z, const TypeCtx& c, bool can_divide, double& due) {
  due = birth + fma(c.sigma, widen_scaled(z), c.mu);
  if (gt_nonneg(due, c.t_max)) return kLeaf;
  return can_divide ? kEmit : kVanish;
}

// Warp-aggregated leaf counting. Lanes hold consecutive cells of a level sorted by root,
// so equal (bin, type) classes form runs of neighbouring lanes; the first lane of each
// run adds the run's leaves with one atomic.
__device__ __forceinline__ void count_leaves(unsigned long long* hist_g, uint32_t cls,
                                             uint32_t nleaf, uint32_t lane) {
  const uint32_t b0 = __ballot_sync(kFull, (nleaf & 1u) != 0u);
  const uint32_t b1 = __ballot_sync(kFull, (nleaf & 2u) != 0u);
  if ((b0 | b1) == 0u) return;
  const uint32_t key = nleaf ? cls : 0xFFFFFFFFu;
  const uint32_t prev = __shfl_up_sync(kFull, key, 1);
  const bool head = lane == 0u || key != prev;
  const uint32_t heads = __ballot_sync(kFull, head);
  if (head && nleaf != 0u) {
    const uint32_t after = heads & ~((2u << lane) - 1u);
    const uint32_t end_mask = after ? ((1u << (__ffs(after) - 1)) - 1u) : kFull;
    const uint32_t run = end_mask & ~((1u << lane) - 1u);
    atomicAdd(hist_g + cls, (unsigned long long)(__popc(run & b0) + 2 * __popc(run & b1)));
  }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// The last block to finish turns the per-warp output counts into the exclusive prefix
// the next sweep reads (the threadfence/ticket pattern; no block waits on another).
template <int kThreads>
__device__ void finish_level(const LevelOut& out, uint32_t nseg, unsigned long long* s_sum) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = (atomicAdd(out.ticket, 1u) == gridDim.x - 1u) ? 1 : 0;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const uint32_t per = (nseg + kThreads - 1) / kThreads;
  const uint32_t b = min(nseg, threadIdx.x * per), e = min(nseg, b + per);
  unsigned long long acc = 0;
  for (uint32_t i = b; i < e; ++i) acc += __ldcg(out.count + i);
  s_sum[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (int i = 0; i < kThreads; ++i) {
      const unsigned long long t = s_sum[i];
      s_sum[i] = run;
      run += t;
    }
    out.prefix[nseg] = run;
    *out.ticket = 0u;
  }
  __syncthreads();
  unsigned long long run = s_sum[threadIdx.x];
  for (uint32_t i = b; i < e; ++i) {
    out.prefix[i] = run;
    run += __ldcg(out.count + i);
  }
}

template <bool Coherent>
__device__ __forceinline__ uint32_t last_le(const unsigned long long* prefix, uint32_t n,
                                            unsigned long long v) {
  // largest s in [0, n-1] with prefix[s] <= v (prefix[0] == 0)
  uint32_t lo = 0, hi = n - 1u;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1u) >> 1;
    if (ld_level<Coherent>(prefix + mid) <= v)
      lo = mid;
    else
      hi = mid - 1u;
  }
  return lo;
}

// ------------------------------------------------------------------ root sweep ------
// Initial cells [lo, hi) of the chunk starting at batch root index root_base.
template <bool Narrow, bool Batched, int kThreads>
__device__ void root_body(const RunArgs& a, const uint64_t root_base, const uint64_t lo, const uint64_t hi,
                          const LevelOut& out, const Smem& s, unsigned long long* s_scan) {
  constexpr uint32_t kWarps = kThreads / 32;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wg = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kWarps;
  const uint64_t len = hi - lo;
  const uint64_t ra = lo + len * wg / nw, rb = lo + len * (wg + 1u) / nw;
  ulonglong2* ob = out.cells + (uint64_t)wg * out.stride;
  uint64_t out_n = 0;
  unsigned long long uncounted = 0, vanished = 0;
  // bin of the warp's first root: largest b with bin_start[b] <= batch root index
  uint32_t bin = 0;
  {
    const uint64_t g0 = root_base + ra;
    uint32_t l = 0, h = a.nbins - 1u;
    while (l < h) {
      const uint32_t m = (l + h + 1u) >> 1;
      if (__ldg(a.bin_start + m) <= g0)
        l = m;
      else
        h = m - 1u;
    }
    bin = l;
  }
  uint64_t bin_hi = __ldg(a.bin_start + bin + 1u);
  for (uint64_t v0 = ra; v0 < rb; v0 += 32u) {
    const uint64_t rl = v0 + lane;
    const bool act = rl < rb;
    int f = kNone;
    double d0 = 0.0;
    uint32_t nleaf = 0, cls = 0;
    if (act) {
      const uint64_t rg = root_base + rl;
      while (rg >= bin_hi) {
        ++bin;
        bin_hi = __ldg(a.bin_start + bin + 1u);
      }
      // the instance: its types, seed, first root and t_max
      uint32_t type_begin = 0, ntypes = a.ntypes, fallback = a.fallback, k0 = a.k0, k1 = a.k1;
      uint64_t root_begin = 0;
      double t_max = a.t_max;
      if (Batched) {
        const InstanceDev& I = a.inst[__ldg(a.bin_inst + bin)];
        type_begin = I.type_begin;
        ntypes = I.ntypes;
        fallback = I.fallback;
        k0 = I.k0;
        k1 = I.k1;
        root_begin = I.root_begin;
        t_max = I.t_max;
      }
      const uint32_t root = (uint32_t)(rg - root_begin);
      const u32x4 R = Batched ? philox(u32x4{0u, 0u, root, kPurposeRoot}, k0, k1)
                              : philox_ks(u32x4{0u, 0u, root, kPurposeRoot}, a.ks);
      const double u_type = unit53_closed_open(R.x, R.y);
      const double u_age = unit53_open_closed(R.z, R.w);
      const TypeDev* types = Batched ? &a.btypes[type_begin].t : s.types;
      const size_t tstride = Batched ? sizeof(BatchType) : sizeof(TypeDev);
      auto type_at = [&](uint32_t i) -> const TypeDev& {
        return *reinterpret_cast<const TypeDev*>(reinterpret_cast<const char*>(types) + i * tstride);
      };
      uint32_t ty = fallback;
      for (uint32_t i = 0; i < ntypes; ++i) {
        if (u_type < type_at(i).cum) {
          ty = i;
          break;
        }
      }
      const uint32_t info = __ldg(a.bin_info + bin);
      cls = Batched ? __ldg(a.bin_class + bin) + ty : bin * a.ntypes + ty;
      if (in_bounds(rl < a.rec_cap && bin < a.nbins, a.error))
        a.root_rec[rl] = (unsigned long long)cls | ((unsigned long long)(type_begin + ty) << 32) |
                         ((unsigned long long)(info & 0xFFu) << 48) |
                         ((unsigned long long)((info >> 8) & 3u) << 56);
      const TypeDev& T = type_at(ty);
      bool leaf;
      if (T.mode == kModeQuiescent) {
        leaf = true;  // timer -1: out of time at once (cell.cu:69-75)
      } else {
        const u32x4 P = Batched ? philox(u32x4{0u, 0u, root, kPurposePair}, k0, k1)
                                : philox_ks(u32x4{0u, 0u, root, kPurposePair}, a.ks);
        const float z = draw_z(P.y, pair_layer(P, 1u), pair_wedge_bits(P, 1u), 1ull, root, k0, k1, T.zlo, T.zhi,
                               s.zig_or(a), a.error);
        const double tau = fma(T.sigma, widen_scaled(z), T.mu);  // 0 for zero-mean types
        d0 = tau * u_age + tau;  // t = tau * U (cell.cu:124-143), due = t + timer
        leaf = gt_nonneg(d0, t_max);
      }
      if (leaf) {
        if (info & 0x100u)
          nleaf = 1u;
        else
          ++uncounted;
      } else if ((info & 0xFFu) > 0u) {
        f = kEmit;
      } else {
        ++vanished;
      }
    }
    if (!in_bounds(cls < a.nclass, a.error)) nleaf = 0u;
    count_leaves(a.hist, cls, nleaf, lane);
    const uint32_t em = __ballot_sync(kFull, f == kEmit);
    if (f == kEmit) {
      const uint32_t pos = __popc(em & ((1u << lane) - 1u));
      const unsigned long long key = Narrow ? ((unsigned long long)rl << 32) | 1ull : rl;
      if (in_bounds(out_n + pos < out.stride, a.error))
        ob[out_n + pos] = make_ulonglong2((unsigned long long)__double_as_longlong(d0), key);
    }
    out_n += __popc(em);
  }
  vanished = warp_sum(vanished);
  uncounted = warp_sum(uncounted);
  if (lane == 0) {
    out.count[wg] = out_n;
    if (vanished) atomicAdd(a.stats + 0, vanished);
    if (uncounted) atomicAdd(a.stats + 1, uncounted);
    __threadfence();
  }
  finish_level<kThreads>(out, nw, s_scan);
}

// -------------------------------------------------------------- division sweep ------
// Each warp owns a contiguous slice of n input cells and an output segment of 2n slots.
// The main loop settles each daughter from its first-attempt normal: a leaf (counted
// into the histogram, never stored), a vanished cell, or a dividing cell whose exact FP64
// due time is written to the front of the segment. Daughters whose first attempt is not
// accepted by the ziggurat strip test (about 0.43%) are written as (birth, key) to the back
// of the segment and resolved after the main loop, 32 at a time with every lane busy;
// their first-attempt bits are re-derived from the parent's Philox block. The rejection
// path thus costs the main loop neither registers nor idle lanes. Resolved cells are
// appended to the front; each input cell contributes at most two cells to front + back.

// Leaf counts of one block in shared memory: a window of classes starting just below the
// class of the block's first cell (its input comes from a level sorted by root, so its
// classes are few and close together); classes outside the window go straight to global
// memory.
constexpr uint32_t kHistWindow = 2048;

struct DivideSmem {
  uint32_t hist[kHistWindow];
  uint32_t base;
};

__device__ __forceinline__ void add_leaves(DivideSmem& sm, unsigned long long* hist_g, uint32_t cls,
                                           uint32_t n) {
  const uint32_t i = cls - sm.base;
  if (i < kHistWindow)
    atomicAdd(&sm.hist[i], n);
  else
    atomicAdd(hist_g + cls, (unsigned long long)n);
}

template <bool Narrow>
__device__ __forceinline__ void decode(uint64_t key, uint32_t g, uint64_t& rl, uint64_t& node) {
  if (Narrow) {
    rl = key >> 32;
    node = (uint32_t)key;
  } else {
    rl = key >> g;
    node = (1ull << g) | (key & ((1ull << g) - 1ull));
  }
}

// The first-attempt classification of both daughters of one input cell.
struct CellDraw {
  double due0, due1;           // exact due times (valid where stored)
  unsigned long long kd;       // key of daughter 0 (daughter 1: kd + 1)
  double birth;
  uint32_t cls;
  bool em0, em1;               // stored (will divide)
  bool sl0, sl1;               // parked for the rejection path
  uint32_t nleaf, nvanish;
  bool overflow;               // a daughter vanished only because the key layout is full
};

template <bool Narrow, bool Batched, bool Coherent>
__device__ __forceinline__ CellDraw classify(const ulonglong2 c, bool act, uint32_t g, const RunArgs& a,
                                             const uint64_t root_base, const Smem& s) {
  CellDraw r;
  const uint32_t g1 = g + 1u;
  const double d = __longlong_as_double((long long)c.x);
  uint64_t rl, node;
  decode<Narrow>(c.y, g, rl, node);
  const bool rec_ok = act && in_bounds(rl < a.rec_cap, a.error);
  const unsigned long long rec = rec_ok ? ld_rec<Coherent>(a.root_rec + rl) : 0ull;  // consumed after Philox
  const uint32_t cap = rec_cap(rec);
  const bool can_divide = g1 < cap;
  const TypeCtx tc = type_ctx<Batched>(a, s.types, rec_type(rec));
  const uint32_t root = (uint32_t)(root_base + rl - tc.root_begin);
  const u32x4 P = Batched ? philox(u32x4{(uint32_t)node, (uint32_t)(node >> 32), root, kPurposePair}, tc.k0, tc.k1)
                          : philox_ks(u32x4{(uint32_t)node, (uint32_t)(node >> 32), root, kPurposePair}, a.ks);
  // first attempts of both daughters: strip test and truncation bounds (zero-mean types
  // carry sigma = mu = 0 and unbounded z, so any accepted z gives tau = 0)
  const ZigTables& Z = s.zig_or(a);
  const uint32_t l0 = pair_layer(P, 0u), l1 = pair_layer(P, 1u);
  float z0 = __fmul_rn((float)(P.x & 0x7FFFFFFFu), Z.w[l0]);
  float z1 = __fmul_rn((float)(P.y & 0x7FFFFFFFu), Z.w[l1]);
  z0 = __uint_as_float(__float_as_uint(z0) ^ (P.x & 0x80000000u));  // the sign bit of j
  z1 = __uint_as_float(__float_as_uint(z1) ^ (P.y & 0x80000000u));
  const float zlo = tc.zlo, zhi = tc.zhi;
  const bool ok0 = act && (P.x & 0x7FFFFFFFu) < Z.k[l0] && z0 >= zlo && z0 <= zhi;
  const bool ok1 = act && (P.y & 0x7FFFFFFFu) < Z.k[l1] && z1 >= zlo && z1 <= zhi;
  // exact FP64 due times (the reference's t + timer): they decide leaves and are what an
  // emitted daughter stores
  r.due0 = d + fma(tc.sigma, widen_scaled(z0), tc.mu);
  r.due1 = d + fma(tc.sigma, widen_scaled(z1), tc.mu);
  const bool leaf0 = ok0 && gt_nonneg(r.due0, tc.t_max);
  const bool leaf1 = ok1 && gt_nonneg(r.due1, tc.t_max);
  r.em0 = ok0 && !leaf0 && can_divide;
  r.em1 = ok1 && !leaf1 && can_divide;
  const bool van0 = ok0 && !leaf0 && !can_divide, van1 = ok1 && !leaf1 && !can_divide;
  r.sl0 = act && !ok0;
  r.sl1 = act && !ok1;
  r.nleaf = (leaf0 ? 1u : 0u) + (leaf1 ? 1u : 0u);
  r.nvanish = (van0 ? 1u : 0u) + (van1 ? 1u : 0u);
  r.overflow = !Narrow && rec_clamped(rec) && g1 == cap && (van0 || van1);
  r.cls = (uint32_t)rec;
  r.birth = d;
  // daughters' keys: narrow root << 32 | (2 node + c), wide 2 key + c
  r.kd = Narrow ? c.y + (uint32_t)c.y : 2ull * c.y;
  return r;
}

// Input cells [in.lo, in.hi) of generation g (chunk starting at batch root index
// root_base); the caller has staged `s` (the __syncthreads below publishes it).
template <bool Narrow, bool Batched, class C, bool Coherent>
__device__ void divide_body(const RunArgs& a, const uint64_t root_base, const LevelIn& in, const uint32_t g,
                            const LevelOut& out, const Smem& s, DivideSmem& sm, unsigned long long* s_scan) {
  constexpr int kCells = C::kCells;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wg = blockIdx.x * C::kWarps + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * C::kWarps;
  const uint64_t len = in.hi - in.lo;
  const uint64_t va = in.lo + len * wg / nw;
  const uint32_t n = (uint32_t)(in.lo + len * (wg + 1u) / nw - va);  // cells of this warp
  const uint32_t g1 = g + 1u;
  if constexpr (!C::kGlobalHist) {
    for (uint32_t i = threadIdx.x; i < kHistWindow; i += blockDim.x) sm.hist[i] = 0u;
    if (threadIdx.x == 0) {
      // histogram window: from just below the class of the block's first cell
      const uint64_t b0 = in.lo + len * (blockIdx.x * C::kWarps) / nw;
      uint32_t base = 0u;
      if (b0 < in.hi) {
        const uint32_t sg = last_le<Coherent>(in.prefix, in.nseg, b0);
        const ulonglong2 c0 =
            ld_level<Coherent>(in.cells + (uint64_t)sg * in.stride + (b0 - ld_level<Coherent>(in.prefix + sg)));
        uint64_t rl, node;
        decode<Narrow>(c0.y, g, rl, node);
        const uint32_t cls0 = (uint32_t)ld_rec<Coherent>(a.root_rec + rl);
        base = cls0 - min(cls0, (uint32_t)kMaxTypes - 1u);
      }
      sm.base = base;
    }
  }
  __syncthreads();

  // Segment cursor in warp-relative indices: input cells [.., hi_rel) of segment `seg`
  // start at seg_ptr + index.
  uint32_t seg = 0, hi_rel = 0;
  const ulonglong2* seg_ptr = in.cells;
  unsigned long long seg_hi_abs = 0ull;
  auto locate = [&](uint32_t i) -> const ulonglong2* {
    while (i >= hi_rel) {
      const unsigned long long lo_abs = seg_hi_abs;
      ++seg;
      seg_hi_abs = ld_level<Coherent>(in.prefix + seg + 1u);
      seg_ptr = in.cells + (uint64_t)seg * in.stride - (lo_abs - va);
      hi_rel = (uint32_t)min(seg_hi_abs - va, (unsigned long long)n);
    }
    return seg_ptr + i;
  };
  constexpr uint32_t kStep = 32u * kCells;
  ulonglong2 next[kCells];
#pragma unroll
  for (int k = 0; k < kCells; ++k) next[k] = make_ulonglong2(0ull, 0ull);
  if (n) {
    seg = last_le<Coherent>(in.prefix, in.nseg, va);
    const unsigned long long lo_abs = ld_level<Coherent>(in.prefix + seg);
    seg_hi_abs = ld_level<Coherent>(in.prefix + seg + 1u);
    seg_ptr = in.cells + (uint64_t)seg * in.stride - (lo_abs - va);
    hi_rel = (uint32_t)min(seg_hi_abs - va, (unsigned long long)n);
#pragma unroll
    for (int k = 0; k < kCells; ++k)
      if (32u * k + lane < n) next[k] = ld_level<Coherent>(locate(32u * k + lane));
  }

  ulonglong2* const ob = out.cells + (uint64_t)wg * out.stride;
  ulonglong2* const back = ob + 2u * n;  // pending daughters at back[-1], back[-2], ...
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t front = 0, pending = 0, vanished = 0, depth_error = 0;
  unsigned long long* const hist_g1 = a.hist + (uint64_t)g1 * a.nclass;
  // checked build: the segment holds 2n cells, and generation g + 1 has a histogram row
  const bool seg_ok = in_bounds(2ull * n <= out.stride, a.error);
  const bool row_ok = in_bounds(g1 < a.hist_gens, a.error);

  for (uint32_t i0 = 0; i0 < n; i0 += kStep) {
    CellDraw r[kCells];
#pragma unroll
    for (int k = 0; k < kCells; ++k) {
      const ulonglong2 c = next[k];
      const uint32_t i = i0 + 32u * k + lane;
      // prefetch the next step's cells while these are processed
      if (i + kStep < n) next[k] = ld_level<Coherent>(locate(i + kStep));
      r[k] = classify<Narrow, Batched, Coherent>(c, i < n, g, a, root_base, s);
    }
#pragma unroll
    for (int k = 0; k < kCells; ++k) {
      if (!in_bounds(r[k].cls < a.nclass && row_ok, a.error)) r[k].nleaf = 0u;
      if constexpr (C::kGlobalHist)
        count_leaves(hist_g1, r[k].cls, r[k].nleaf, lane);
      else if (r[k].nleaf)
        add_leaves(sm, hist_g1, r[k].cls, r[k].nleaf);
      vanished += r[k].nvanish;
      if (r[k].overflow) depth_error = 1u;
      const uint32_t e0 = __ballot_sync(kFull, r[k].em0), e1 = __ballot_sync(kFull, r[k].em1);
      const uint32_t at = front + __popc(e0 & lt) + __popc(e1 & lt);
      ulonglong2* dst = ob + at;
      const uint32_t mine = (r[k].em0 ? 1u : 0u) + (r[k].em1 ? 1u : 0u);
      const bool dst_ok = in_bounds(seg_ok && at + mine <= 2u * n, a.error);
      if (r[k].em0 && dst_ok) dst[0] = make_ulonglong2((unsigned long long)__double_as_longlong(r[k].due0), r[k].kd);
      if (r[k].em1 && dst_ok)
        dst[r[k].em0 ? 1 : 0] = make_ulonglong2((unsigned long long)__double_as_longlong(r[k].due1), r[k].kd + 1ull);
      front += __popc(e0) + __popc(e1);
      // daughters the strip test did not settle: park (birth, key) at the back
      const uint32_t p0 = __ballot_sync(kFull, r[k].sl0), p1 = __ballot_sync(kFull, r[k].sl1);
      if (p0 | p1) {
        const uint32_t below = pending + __popc(p0 & lt) + __popc(p1 & lt);  // records after this lane's
        ulonglong2* pd = back - 1u - below;
        const unsigned long long bb = (unsigned long long)__double_as_longlong(r[k].birth);
        const uint32_t parked = (r[k].sl0 ? 1u : 0u) + (r[k].sl1 ? 1u : 0u);
        const bool pd_ok = in_bounds(seg_ok && front + below + parked <= 2u * n, a.error);
        if (r[k].sl0 && pd_ok) pd[0] = make_ulonglong2(bb, r[k].kd);
        if (r[k].sl1 && pd_ok) *(pd - (r[k].sl0 ? 1 : 0)) = make_ulonglong2(bb, r[k].kd + 1ull);
        pending += __popc(p0) + __popc(p1);
      }
    }
  }

  // Resolve the parked daughters, 32 at a time: re-derive the first attempt from the
  // parent's pair block, draw with the rejection path, settle exactly, append to the front.
  // Passes take the records nearest the front first (the last parked): front + pending
  // <= 2n, so a pass's writes, at most one per record resolved so far, stay below every
  // record not yet read.
  __syncwarp();
  for (uint32_t hi = pending; hi > 0u;) {
    const uint32_t lo = hi > 32u ? hi - 32u : 0u;
    const bool act = lo + lane < hi;
    int f = kNone;
    double due = 0.0;
    unsigned long long key = 0ull;
    if (act && in_bounds(seg_ok && lo + lane < 2u * n, a.error)) {
      const ulonglong2 pc = back[-1 - (int64_t)(lo + lane)];
      key = pc.y;
      const double birth = __longlong_as_double((long long)pc.x);
      uint64_t rl, node;
      decode<Narrow>(key, g1, rl, node);
      const unsigned long long rec = in_bounds(rl < a.rec_cap, a.error) ? ld_rec<Coherent>(a.root_rec + rl) : 0ull;
      const uint32_t cap = rec_cap(rec);
      const TypeCtx tc = type_ctx<Batched>(a, s.types, rec_type(rec));
      const uint32_t root = (uint32_t)(root_base + rl - tc.root_begin);
      const uint64_t parent = node >> 1;
      const uint32_t ch = (uint32_t)(node & 1ull);
      const u32x4 P = philox(u32x4{(uint32_t)parent, (uint32_t)(parent >> 32), root, kPurposePair}, tc.k0, tc.k1);
      const float z = slow_z(ch ? P.y : P.x, pair_layer(P, ch), pair_wedge_bits(P, ch), node, root,
                             tc.k0, tc.k1, tc.zlo, tc.zhi, s.zig_or(a), a.error);
      f = fate(birth, z, tc, g1 < cap, due);
      if (f == kLeaf && !in_bounds((uint32_t)rec < a.nclass && row_ok, a.error)) f = kNone;
      if (f == kLeaf) {
        if constexpr (C::kGlobalHist)
          atomicAdd(hist_g1 + (uint32_t)rec, 1ull);
        else
          add_leaves(sm, hist_g1, (uint32_t)rec, 1u);
      }
      if (f == kVanish) {
        ++vanished;
        if (!Narrow && rec_clamped(rec) && g1 == cap) depth_error = 1u;
      }
    }
    __syncwarp();  // every parked record of this pass is read before the front grows
    const uint32_t em = __ballot_sync(kFull, f == kEmit);
    if (f == kEmit && in_bounds(front + __popc(em & lt) < 2u * n, a.error))
      ob[front + __popc(em & lt)] = make_ulonglong2((unsigned long long)__double_as_longlong(due), key);
    front += __popc(em);
    hi = lo;
  }

  const unsigned long long v = warp_sum((unsigned long long)vanished);
  depth_error = __reduce_or_sync(kFull, depth_error);
  if (lane == 0) {
    out.count[wg] = front;
    if (v) atomicAdd(a.stats + 0, v);
    if (depth_error) atomicOr(a.error, 1u);
    __threadfence();
  }
  if constexpr (!C::kGlobalHist) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kHistWindow; i += blockDim.x) {
      const uint32_t cnt = sm.hist[i];
      if (cnt && sm.base + i < a.nclass) atomicAdd(hist_g1 + sm.base + i, (unsigned long long)cnt);
    }
  }
  finish_level<C::kThreads>(out, nw, s_scan);
}

// ------------------------------------------------------------- kernels: one per sweep --
template <bool Narrow, bool Batched, class C>
__global__ void __launch_bounds__(C::kThreads) k_roots(const RunArgs a, const uint64_t lo, const uint64_t hi,
                                                      const LevelOut out) {
  __shared__ Smem s;
  __shared__ unsigned long long s_scan[C::kThreads];
  stage(s, a);
  __syncthreads();
  root_body<Narrow, Batched, C::kThreads>(a, a.root_base, lo, hi, out, s, s_scan);
}

template <bool Narrow, bool Batched, class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks) k_divide(const RunArgs a, const LevelIn in,
                                                                      const uint32_t g, const LevelOut out) {
  __shared__ Smem s;
  __shared__ DivideSmem sm;
  __shared__ unsigned long long s_scan[C::kThreads];
  stage(s, a);
  divide_body<Narrow, Batched, C, false>(a, a.root_base, in, g, out, s, sm, s_scan);
}

// --------------------------------------------------------- kernel: persistent driver --
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch (every block resident). Arrival is an atomic
// on bar[0]; the last block to arrive resets it and advances the generation bar[1], which
// the others wait for. A wait longer than timeout_ns (or 2^28 polls) sets error bit 2;
// every waiting block also polls that bit (every 256 polls, about 20 us), so all blocks leave
// within one poll period of the first timeout, wherever they wait. Returns false once that
// bit is set.
__device__ bool grid_barrier(uint32_t* bar, unsigned long long timeout_ns, uint32_t* error) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = bar + 1;
    const uint32_t g0 = *gen;
    int ok = 1;
    __threadfence();
    if (atomicAdd(bar, 1u) == gridDim.x - 1u) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      uint32_t polls = 0;
      while (*gen == g0) {
        __nanosleep(64);
        if ((++polls & 255u) == 0u) {
          if (*(volatile uint32_t*)error & 4u) {  // another block gave up
            ok = 0;
            break;
          }
          if (global_ns() - t0 > timeout_ns || polls >= (1u << 28)) {
            atomicOr(error, 4u);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    if (ok && (*(volatile uint32_t*)error & 4u)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The depth-first schedule, identical in every block (thread 0 updates it).
struct Schedule {
  struct Entry {
    uint32_t buf, gen, nseg, pad;
    uint64_t stride, pos, n;
  };
  Entry stack[kMaxPool];
  uint32_t depth;
  uint32_t busy_lo, busy_hi;  // buffers in use (bit per buffer)
  int kind;                   // 0 done, 1 root sweep, 2 division sweep
  uint32_t out_buf, out_nseg, gen, failed;
  uint64_t chunk_pos, root_base, n_roots, lo, hi, out_stride;
  unsigned long long divisions;
  uint32_t sweeps, max_gen, chunks;
};

__device__ __forceinline__ bool sched_acquire(Schedule& c, uint32_t nbuf, uint32_t& b) {
  for (uint32_t i = 0; i < nbuf; ++i) {
    uint32_t& w = i < 32u ? c.busy_lo : c.busy_hi;
    const uint32_t bit = 1u << (i & 31u);
    if (!(w & bit)) {
      w |= bit;
      b = i;
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ void sched_release(Schedule& c, uint32_t b) {
  (b < 32u ? c.busy_lo : c.busy_hi) &= ~(1u << (b & 31u));
}

// Picks the next sweep: the unfinished slice of the deepest level first (bounded memory),
// else the next root chunk, else done. Mirrors the host driver's loop.
__device__ void sched_next(Schedule& c, const PersistArgs& p, uint32_t nseg) {
  if (c.depth == 0u) {
    if (c.chunk_pos >= p.root_hi) {
      c.kind = 0;
      return;
    }
    uint32_t b;
    if (!sched_acquire(c, p.nbuf, b)) {
      c.failed = 1u;
      c.kind = 0;
      return;
    }
    c.kind = 1;
    c.out_buf = b;
    c.root_base = c.chunk_pos;
    c.n_roots = min(p.chunk, p.root_hi - c.chunk_pos);
    c.out_nseg = nseg;
    c.out_stride = (c.n_roots + nseg - 1u) / nseg;
    return;
  }
  const Schedule::Entry& top = c.stack[c.depth - 1u];
  uint32_t b;
  if (!sched_acquire(c, p.nbuf, b)) {
    c.failed = 1u;
    c.kind = 0;
    return;
  }
  const uint64_t len = min(top.n - top.pos, p.max_slice);
  c.kind = 2;
  c.out_buf = b;
  c.gen = top.gen;
  c.lo = top.pos;
  c.hi = top.pos + len;
  c.out_nseg = nseg;
  c.out_stride = 2u * ((len + nseg - 1u) / nseg);
}

// After the barrier that ends a sweep: read its output total and update the stack.
__device__ void sched_done(Schedule& c, const PersistArgs& p) {
  const unsigned long long total = __ldcg(p.prefix[c.out_buf] + c.out_nseg);
  if (c.kind == 1) {
    c.chunk_pos += c.n_roots;
    ++c.chunks;
    if (total == 0ull) {
      sched_release(c, c.out_buf);
    } else {
      c.stack[c.depth++] = Schedule::Entry{c.out_buf, 0u, c.out_nseg, 0u, c.out_stride, 0ull, total};
    }
    return;
  }
  Schedule::Entry& top = c.stack[c.depth - 1u];
  const uint64_t len = c.hi - c.lo;
  c.divisions += len;
  ++c.sweeps;
  c.max_gen = max(c.max_gen, c.gen + 1u);
  top.pos += len;
  if (top.pos == top.n) {
    sched_release(c, top.buf);
    --c.depth;
  }
  if (total > 0ull && c.gen + 1u <= p.g_limit && c.depth < (uint32_t)kMaxPool) {
    c.stack[c.depth++] = Schedule::Entry{c.out_buf, c.gen + 1u, c.out_nseg, 0u, c.out_stride, 0ull, total};
  } else {
    sched_release(c, c.out_buf);
  }
}

template <bool Narrow, bool Batched, class C>
__global__ void __launch_bounds__(C::kThreads, C::kMinBlocks) k_persist(const PersistArgs p) {
  __shared__ Smem s;
  __shared__ DivideSmem sm;
  __shared__ unsigned long long s_scan[C::kThreads];
  __shared__ Schedule c;
  const RunArgs& a = p.a;
  stage(s, a);
  const uint32_t nseg = gridDim.x * C::kWarps;
  if (threadIdx.x == 0) {
    c.depth = 0u;
    c.busy_lo = c.busy_hi = 0u;
    c.failed = 0u;
    c.chunk_pos = p.root_lo;
    c.divisions = 0ull;
    c.sweeps = c.max_gen = c.chunks = 0u;
    sched_next(c, p, nseg);
  }
  __syncthreads();
  while (c.kind != 0) {
    const uint32_t ob = c.out_buf;
    const LevelOut out{p.cells[ob], p.count[ob], p.prefix[ob], p.ticket[ob], c.out_stride};
    if (c.kind == 1) {
      root_body<Narrow, Batched, C::kThreads>(a, c.root_base, 0ull, c.n_roots, out, s, s_scan);
    } else {
      const Schedule::Entry& top = c.stack[c.depth - 1u];
      const LevelIn in{p.cells[top.buf], p.prefix[top.buf], top.nseg, top.stride, c.lo, c.hi};
      divide_body<Narrow, Batched, C, true>(a, c.root_base, in, c.gen, out, s, sm, s_scan);
    }
    if (!grid_barrier(p.barrier, p.timeout_ns, a.error)) return;
    if (threadIdx.x == 0) {
      sched_done(c, p);
      sched_next(c, p, nseg);
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (c.failed) atomicOr(a.error, 8u);
    p.out[0] = c.divisions;
    p.out[1] = c.sweeps;
    p.out[2] = c.max_gen;
    p.out[3] = c.chunks;
  }
}

// ------------------------------------------------------------------------ launchers --
template <bool Narrow, bool Batched, class C>
int launch_roots_t(const RunArgs& a, uint64_t lo, uint64_t hi, const LevelOut& out, int blocks, void* stream) {
  k_roots<Narrow, Batched, C><<<blocks, C::kThreads, 0, (cudaStream_t)stream>>>(a, lo, hi, out);
  return (int)cudaGetLastError();
}

template <bool Narrow, bool Batched, class C>
int launch_divide_t(const RunArgs& a, const LevelIn& in, uint32_t gen, const LevelOut& out, int blocks,
                    void* stream) {
  k_divide<Narrow, Batched, C><<<blocks, C::kThreads, 0, (cudaStream_t)stream>>>(a, in, gen, out);
  return (int)cudaGetLastError();
}

template <bool Narrow, bool Batched, class C>
int launch_persist_t(const PersistArgs& p, int blocks, void* stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3((unsigned)C::kThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = (cudaStream_t)stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return (int)cudaLaunchKernelEx(&cfg, k_persist<Narrow, Batched, C>, p);
}

template <bool Narrow, bool Batched, class C>
int occupancy_t(int* roots_per_sm, int* divide_per_sm, int* persist_per_sm) {
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(roots_per_sm, k_roots<Narrow, Batched, C>,
                                                                C::kThreads, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(divide_per_sm, k_divide<Narrow, Batched, C>, C::kThreads, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(persist_per_sm, k_persist<Narrow, Batched, C>, C::kThreads, 0);
  return (int)e;
}

template <bool Narrow, bool Batched, class C>
SweepKernels make_kernels() {
  return SweepKernels{C::kThreads,
                      C::kCells,
                      C::kGlobalHist ? 1 : 0,
                      &launch_roots_t<Narrow, Batched, C>,
                      &launch_divide_t<Narrow, Batched, C>,
                      &launch_persist_t<Narrow, Batched, C>,
                      &occupancy_t<Narrow, Batched, C>};
}

// The tuned configurations in index order: index = 4 * (threads == 256) + 2 * (cells == 2)
// + global_hist.
template <bool Narrow, bool Batched>
const SweepKernels& tuned_kernels(int config) {
  static const SweepKernels table[kNumSweepConfigs] = {
      make_kernels<Narrow, Batched, Cfg<128, 1, false>>(), make_kernels<Narrow, Batched, Cfg<128, 1, true>>(),
      make_kernels<Narrow, Batched, Cfg<128, 2, false>>(), make_kernels<Narrow, Batched, Cfg<128, 2, true>>(),
      make_kernels<Narrow, Batched, Cfg<256, 1, false>>(), make_kernels<Narrow, Batched, Cfg<256, 1, true>>(),
      make_kernels<Narrow, Batched, Cfg<256, 2, false>>(), make_kernels<Narrow, Batched, Cfg<256, 2, true>>(),
  };
  return table[config];
}

}  // namespace
}  // namespace pc
