// sm_103a kernels of the proliferation path.
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
#include <cuda_runtime.h>

#include <algorithm>

#include "pc_engine.h"

namespace pc {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
// Resident blocks per SM the division sweep is compiled for (caps registers per thread).
#ifndef PC_DIVIDE_MIN_BLOCKS
#define PC_DIVIDE_MIN_BLOCKS 4
#endif
constexpr int kDivideMinBlocks = PC_DIVIDE_MIN_BLOCKS;
// Input cells each lane carries per step of the division sweep.
#ifndef PC_CELLS_PER_LANE
#define PC_CELLS_PER_LANE 1
#endif
constexpr int kCellsPerLane = PC_CELLS_PER_LANE;

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
                                     uint32_t root, uint32_t k0, uint32_t k1, const TypeDev& T,
                                     const ZigTables& Z, uint32_t* error) {
  ChildStream cs = child_stream(node, root, k0, k1);
  uint32_t budget = kRoundBudget;
  bool have_wedge = true;
  while (budget > 0u) {
    const float z = zig_normal(j, layer, have_wedge, wedge, cs, Z, budget);
    if (budget == 0u) break;
    if (z >= T.zlo && z <= T.zhi) return z;
    have_wedge = false;
    j = cs.next();
    layer = cs.next() & 255u;
    --budget;
  }
  atomicOr(error, 2u);
  return 0.0f;
}

// First-attempt fast path (about 98.5% of draws): one strip test, one FP32 multiply.
__device__ __forceinline__ float draw_z(uint32_t j, uint32_t layer, uint32_t wedge, uint64_t node,
                                        uint32_t root, uint32_t k0, uint32_t k1, const TypeDev& T,
                                        const ZigTables& Z, uint32_t* error) {
  const uint32_t mag = j & 0x7FFFFFFFu;
  if (mag < Z.k[layer]) {
    const float x = __fmul_rn((float)mag, Z.w[layer]);
    const float z = (j >> 31) ? -x : x;
    if (z >= T.zlo && z <= T.zhi) return z;
  }
  return slow_z(j, layer, wedge, node, root, k0, k1, T, Z, error);
}

enum Fate : int { kNone = 0, kLeaf = 1, kEmit = 2, kVanish = 3 };

// GB300 runs FP64 arithmetic and every FP64<->FP32 conversion on a pipe of 2 lanes per
// clock per SM, so the conversions and comparisons below are done on the bits instead.
//
// Exact float -> double for zero or a normal float (z is never subnormal: |z| >= the
// smallest ziggurat strip width, about 1e-10): rebias the exponent, widen the mantissa.
__device__ __forceinline__ double f32_to_f64(float z) {
  const uint32_t f = __float_as_uint(z);
  const uint32_t a = f & 0x7FFFFFFFu;
  const uint32_t hi = (f & 0x80000000u) | (a ? (a >> 3) + (896u << 20) : 0u);
  return __hiloint2double((int)hi, (int)(f << 29));
}

// A non-negative double truncated to FP32 (values below 2^-126 become 0; the estimate's
// error band covers both truncations). Valid while d < 2^128, which est_ok guarantees.
__device__ __forceinline__ float f64_to_f32_rz(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  if (hi < (897u << 20)) return 0.0f;
  return __uint_as_float(((hi - (896u << 20)) << 3) | (lo >> 29));
}

// a > b for non-negative doubles (IEEE order equals integer order of the bit patterns).
__device__ __forceinline__ bool gt_nonneg(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}

// What a cell's type, and in the batched form its instance, supplies to the sweeps.
struct TypeCtx {
  const TypeDev* t;  // mu, sigma, truncation bounds (shared memory or the batch table)
  double t_max;
  float t_hi, t_lo;
  bool eok;
  uint64_t root_begin;  // batch index of the instance's first initial cell
  uint32_t k0, k1;      // the instance's seed
};

template <bool Batched>
__device__ __forceinline__ TypeCtx type_ctx(const RunArgs& a, const TypeDev* smem_types, uint32_t ty) {
  TypeCtx c;
  if (Batched) {
    const BatchType* b = a.btypes + ty;
    c.t = &b->t;
    c.t_max = __ldg(&b->t_max);
    c.t_hi = __ldg(&b->t_hi);
    c.t_lo = __ldg(&b->t_lo);
    c.eok = __ldg(&b->est_ok) != 0;
    c.root_begin = __ldg(&b->root_begin);
    c.k0 = __ldg(&b->k0);
    c.k1 = __ldg(&b->k1);
  } else {
    c.t = smem_types + ty;
    c.t_max = a.t_max;
    c.t_hi = a.t_hi;
    c.t_lo = a.t_lo;
    c.eok = a.est_ok != 0;
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

// Fate of one daughter born at `birth` with normal z. The FP32 estimate decides leaves
// and clear non-leaves without FP64 work; the band around t_max (8x the worst-case FP32
// error) and every daughter that is stored use the exact FP64 due time
// birth + fma(sigma, z, mu), the reference's t + timer.
__device__ __forceinline__ int fate(double birth, float birth_f, float z, const TypeCtx& c,
                                    bool can_divide, double& due) {
  const TypeDev& T = *c.t;
  bool exact = true;
  if (c.eok) {
    const float est = __fadd_rn(birth_f, __fadd_rn(T.mu_f, __fmul_rn(T.sigma_f, z)));
    if (est > c.t_hi) return kLeaf;
    if (est < c.t_lo) {
      if (!can_divide) return kVanish;
      exact = false;
    }
  }
  due = birth + fma(T.sigma, f32_to_f64(z), T.mu);
  if (exact && gt_nonneg(due, c.t_max)) return kLeaf;
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
  const uint32_t per = (nseg + kBlock - 1) / kBlock;
  const uint32_t b = min(nseg, threadIdx.x * per), e = min(nseg, b + per);
  unsigned long long acc = 0;
  for (uint32_t i = b; i < e; ++i) acc += __ldcg(out.count + i);
  s_sum[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (int i = 0; i < kBlock; ++i) {
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

__device__ __forceinline__ uint32_t last_le(const unsigned long long* prefix, uint32_t n,
                                            unsigned long long v) {
  // largest s in [0, n-1] with prefix[s] <= v (prefix[0] == 0)
  uint32_t lo = 0, hi = n - 1u;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1u) >> 1;
    if (__ldg(prefix + mid) <= v)
      lo = mid;
    else
      hi = mid - 1u;
  }
  return lo;
}

// ------------------------------------------------------------------ root sweep ------
template <bool Narrow, bool Batched>
__global__ void __launch_bounds__(kBlock) k_roots(const RunArgs a, const uint64_t lo,
                                                  const uint64_t hi, const LevelOut out) {
  __shared__ Smem s;
  __shared__ unsigned long long s_scan[kBlock];
  stage(s, a);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wg = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kWarpsPerBlock;
  const uint64_t len = hi - lo;
  const uint64_t ra = lo + len * wg / nw, rb = lo + len * (wg + 1u) / nw;
  ulonglong2* ob = out.cells + (uint64_t)wg * out.stride;
  uint64_t out_n = 0;
  unsigned long long uncounted = 0, vanished = 0;
  // bin of the warp's first root: largest b with bin_start[b] <= batch root index
  uint32_t bin = 0;
  {
    const uint64_t g0 = a.root_base + ra;
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
      const uint64_t rg = a.root_base + rl;
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
        const float z = draw_z(P.y, (P.z >> 8) & 255u, pair_wedge_bits(P, 1u), 1ull, root, k0, k1, T,
                               s.zig_or(a), a.error);
        const double tau = fma(T.sigma, f32_to_f64(z), T.mu);  // 0 for zero-mean types
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
    count_leaves(a.hist, cls, nleaf, lane);
    const uint32_t em = __ballot_sync(kFull, f == kEmit);
    if (f == kEmit) {
      const uint32_t pos = __popc(em & ((1u << lane) - 1u));
      const unsigned long long key = Narrow ? ((unsigned long long)rl << 32) | 1ull : rl;
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
  finish_level(out, nw, s_scan);
}

// -------------------------------------------------------------- division sweep ------
// Each warp owns a contiguous slice of n input cells and an output segment of 2n slots.
// The main loop settles each daughter from its first-attempt normal: a leaf (counted
// into the histogram, never stored), a vanished cell, or a dividing cell whose exact FP64
// due time is written to the front of the segment. Daughters whose first attempt is not
// accepted by the ziggurat strip test (about 1.5%) are written as (birth, key) to the back
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

template <bool Narrow, bool Batched>
__device__ __forceinline__ CellDraw classify(const ulonglong2 c, bool act, uint32_t g, const RunArgs& a,
                                             const Smem& s) {
  CellDraw r;
  const uint32_t g1 = g + 1u;
  const double d = __longlong_as_double((long long)c.x);
  uint64_t rl, node;
  decode<Narrow>(c.y, g, rl, node);
  const unsigned long long rec = act ? __ldg(a.root_rec + rl) : 0ull;  // consumed after Philox
  const uint32_t cap = rec_cap(rec);
  const bool can_divide = g1 < cap;
  const TypeCtx tc = type_ctx<Batched>(a, s.types, rec_type(rec));
  const TypeDev& T = *tc.t;
  const uint32_t root = (uint32_t)(a.root_base + rl - tc.root_begin);
  const u32x4 P = Batched ? philox(u32x4{(uint32_t)node, (uint32_t)(node >> 32), root, kPurposePair}, tc.k0, tc.k1)
                          : philox_ks(u32x4{(uint32_t)node, (uint32_t)(node >> 32), root, kPurposePair}, a.ks);
  // first attempts of both daughters: strip test and truncation bounds (zero-mean types
  // carry sigma = mu = 0 and unbounded z, so any accepted z gives tau = 0)
  const ZigTables& Z = s.zig_or(a);
  const uint32_t l0 = P.z & 255u, l1 = (P.z >> 8) & 255u;
  float z0 = __fmul_rn((float)(P.x & 0x7FFFFFFFu), Z.w[l0]);
  float z1 = __fmul_rn((float)(P.y & 0x7FFFFFFFu), Z.w[l1]);
  z0 = (P.x >> 31) ? -z0 : z0;
  z1 = (P.y >> 31) ? -z1 : z1;
  const float zlo = T.zlo, zhi = T.zhi;
  const bool ok0 = act && (P.x & 0x7FFFFFFFu) < Z.k[l0] && z0 >= zlo && z0 <= zhi;
  const bool ok1 = act && (P.y & 0x7FFFFFFFu) < Z.k[l1] && z1 >= zlo && z1 <= zhi;
  // FP32 estimates settle clear leaves and clear non-leaves; the exact FP64 due times
  // decide the band and are what gets stored
  const float df = f64_to_f32_rz(d);
  const float mu_f = T.mu_f, sigma_f = T.sigma_f;
  const float est0 = __fadd_rn(df, __fadd_rn(mu_f, __fmul_rn(sigma_f, z0)));
  const float est1 = __fadd_rn(df, __fadd_rn(mu_f, __fmul_rn(sigma_f, z1)));
  const bool eok = tc.eok;
  const bool sure0 = eok && est0 < tc.t_lo, sure1 = eok && est1 < tc.t_lo;
  const double mu = T.mu, sigma = T.sigma;
  r.due0 = d + fma(sigma, f32_to_f64(z0), mu);
  r.due1 = d + fma(sigma, f32_to_f64(z1), mu);
  const bool leaf0 = ok0 && ((eok && est0 > tc.t_hi) || (!sure0 && gt_nonneg(r.due0, tc.t_max)));
  const bool leaf1 = ok1 && ((eok && est1 > tc.t_hi) || (!sure1 && gt_nonneg(r.due1, tc.t_max)));
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

template <bool Narrow, bool Batched, int kCells>
__global__ void __launch_bounds__(kBlock, kDivideMinBlocks) k_divide(const RunArgs a, const LevelIn in,
                                                                     const uint32_t g, const LevelOut out) {
  __shared__ Smem s;
  __shared__ DivideSmem sm;
  __shared__ unsigned long long s_scan[kBlock];
  stage(s, a);
  for (uint32_t i = threadIdx.x; i < kHistWindow; i += blockDim.x) sm.hist[i] = 0u;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t wg = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  const uint32_t nw = gridDim.x * kWarpsPerBlock;
  const uint64_t len = in.hi - in.lo;
  const uint64_t va = in.lo + len * wg / nw;
  const uint32_t n = (uint32_t)(in.lo + len * (wg + 1u) / nw - va);  // cells of this warp
  const uint32_t g1 = g + 1u;
  if (threadIdx.x == 0) {
    // histogram window: from just below the class of the block's first cell
    const uint64_t b0 = in.lo + len * (blockIdx.x * kWarpsPerBlock) / nw;
    uint32_t base = 0u;
    if (b0 < in.hi) {
      const uint32_t sg = last_le(in.prefix, in.nseg, b0);
      const ulonglong2 c0 = __ldg(in.cells + (uint64_t)sg * in.stride + (b0 - __ldg(in.prefix + sg)));
      uint64_t rl, node;
      decode<Narrow>(c0.y, g, rl, node);
      const uint32_t cls0 = (uint32_t)__ldg(a.root_rec + rl);
      base = cls0 - min(cls0, (uint32_t)kMaxTypes - 1u);
    }
    sm.base = base;
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
      seg_hi_abs = __ldg(in.prefix + seg + 1u);
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
    seg = last_le(in.prefix, in.nseg, va);
    const unsigned long long lo_abs = __ldg(in.prefix + seg);
    seg_hi_abs = __ldg(in.prefix + seg + 1u);
    seg_ptr = in.cells + (uint64_t)seg * in.stride - (lo_abs - va);
    hi_rel = (uint32_t)min(seg_hi_abs - va, (unsigned long long)n);
#pragma unroll
    for (int k = 0; k < kCells; ++k)
      if (32u * k + lane < n) next[k] = __ldg(locate(32u * k + lane));
  }

  ulonglong2* const ob = out.cells + (uint64_t)wg * out.stride;
  ulonglong2* const back = ob + 2u * n;  // pending daughters at back[-1], back[-2], ...
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t front = 0, pending = 0, vanished = 0, depth_error = 0;
  unsigned long long* const hist_g1 = a.hist + (uint64_t)g1 * a.nclass;

  for (uint32_t i0 = 0; i0 < n; i0 += kStep) {
    CellDraw r[kCells];
#pragma unroll
    for (int k = 0; k < kCells; ++k) {
      const ulonglong2 c = next[k];
      const uint32_t i = i0 + 32u * k + lane;
      // prefetch the next step's cells while these are processed
      if (i + kStep < n) next[k] = __ldg(locate(i + kStep));
      r[k] = classify<Narrow, Batched>(c, i < n, g, a, s);
    }
#pragma unroll
    for (int k = 0; k < kCells; ++k) {
      if (r[k].nleaf) add_leaves(sm, hist_g1, r[k].cls, r[k].nleaf);
      vanished += r[k].nvanish;
      if (r[k].overflow) depth_error = 1u;
      const uint32_t e0 = __ballot_sync(kFull, r[k].em0), e1 = __ballot_sync(kFull, r[k].em1);
      ulonglong2* dst = ob + front + __popc(e0 & lt) + __popc(e1 & lt);
      if (r[k].em0) dst[0] = make_ulonglong2((unsigned long long)__double_as_longlong(r[k].due0), r[k].kd);
      if (r[k].em1)
        dst[r[k].em0 ? 1 : 0] = make_ulonglong2((unsigned long long)__double_as_longlong(r[k].due1), r[k].kd + 1ull);
      front += __popc(e0) + __popc(e1);
      // daughters the strip test did not settle: park (birth, key) at the back
      const uint32_t p0 = __ballot_sync(kFull, r[k].sl0), p1 = __ballot_sync(kFull, r[k].sl1);
      if (p0 | p1) {
        ulonglong2* pd = back - 1u - pending - __popc(p0 & lt) - __popc(p1 & lt);
        const unsigned long long bb = (unsigned long long)__double_as_longlong(r[k].birth);
        if (r[k].sl0) pd[0] = make_ulonglong2(bb, r[k].kd);
        if (r[k].sl1) *(pd - (r[k].sl0 ? 1 : 0)) = make_ulonglong2(bb, r[k].kd + 1ull);
        pending += __popc(p0) + __popc(p1);
      }
    }
  }

  // Resolve the parked daughters, 32 at a time: re-derive the first attempt from the
  // parent's pair block, draw with the rejection path, settle exactly, append to the front.
  // Rounds take the records nearest the front first (the last parked): front + pending
  // <= 2n, so a round's writes, at most one per record resolved so far, stay below every
  // record not yet read.
  __syncwarp();
  for (uint32_t hi = pending; hi > 0u;) {
    const uint32_t lo = hi > 32u ? hi - 32u : 0u;
    const bool act = lo + lane < hi;
    int f = kNone;
    double due = 0.0;
    unsigned long long key = 0ull;
    if (act) {
      const ulonglong2 pc = back[-1 - (int64_t)(lo + lane)];
      key = pc.y;
      const double birth = __longlong_as_double((long long)pc.x);
      uint64_t rl, node;
      decode<Narrow>(key, g1, rl, node);
      const unsigned long long rec = __ldg(a.root_rec + rl);
      const uint32_t cap = rec_cap(rec);
      const TypeCtx tc = type_ctx<Batched>(a, s.types, rec_type(rec));
      const uint32_t root = (uint32_t)(a.root_base + rl - tc.root_begin);
      const uint64_t parent = node >> 1;
      const uint32_t ch = (uint32_t)(node & 1ull);
      const u32x4 P = philox(u32x4{(uint32_t)parent, (uint32_t)(parent >> 32), root, kPurposePair}, tc.k0, tc.k1);
      const float z = slow_z(ch ? P.y : P.x, (P.z >> (8u * ch)) & 255u, pair_wedge_bits(P, ch), node, root,
                             tc.k0, tc.k1, *tc.t, s.zig_or(a), a.error);
      f = fate(birth, f64_to_f32_rz(birth), z, tc, g1 < cap, due);
      if (f == kLeaf) add_leaves(sm, hist_g1, (uint32_t)rec, 1u);
      if (f == kVanish) {
        ++vanished;
        if (!Narrow && rec_clamped(rec) && g1 == cap) depth_error = 1u;
      }
    }
    __syncwarp();  // every parked record of this round is read before the front grows
    const uint32_t em = __ballot_sync(kFull, f == kEmit);
    if (f == kEmit) ob[front + __popc(em & lt)] = make_ulonglong2((unsigned long long)__double_as_longlong(due), key);
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
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < kHistWindow; i += blockDim.x) {
    const uint32_t cnt = sm.hist[i];
    if (cnt && sm.base + i < a.nclass) atomicAdd(hist_g1 + sm.base + i, (unsigned long long)cnt);
  }
  finish_level(out, nw, s_scan);
}

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
  z[i] = zig_normal(c ? P.y : P.x, (P.z >> (8u * c)) & 255u, true, pair_wedge_bits(P, c), cs, Z, budget);
}

}  // namespace

int launch_root_sweep(const RunArgs& a, uint64_t root_lo, uint64_t root_hi, const LevelOut& out,
                      int blocks, bool narrow, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (a.btypes) {
    if (narrow)
      k_roots<true, true><<<blocks, kBlock, 0, st>>>(a, root_lo, root_hi, out);
    else
      k_roots<false, true><<<blocks, kBlock, 0, st>>>(a, root_lo, root_hi, out);
  } else {
    if (narrow)
      k_roots<true, false><<<blocks, kBlock, 0, st>>>(a, root_lo, root_hi, out);
    else
      k_roots<false, false><<<blocks, kBlock, 0, st>>>(a, root_lo, root_hi, out);
  }
  return (int)cudaGetLastError();
}

int launch_divide_sweep(const RunArgs& a, const LevelIn& in, uint32_t gen, const LevelOut& out,
                        int blocks, bool narrow, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (a.btypes) {
    if (narrow)
      k_divide<true, true, kCellsPerLane><<<blocks, kBlock, 0, st>>>(a, in, gen, out);
    else
      k_divide<false, true, kCellsPerLane><<<blocks, kBlock, 0, st>>>(a, in, gen, out);
  } else {
    if (narrow)
      k_divide<true, false, kCellsPerLane><<<blocks, kBlock, 0, st>>>(a, in, gen, out);
    else
      k_divide<false, false, kCellsPerLane><<<blocks, kBlock, 0, st>>>(a, in, gen, out);
  }
  return (int)cudaGetLastError();
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

int occupancy_blocks_per_sm(int* root_blocks, int* divide_blocks) {
  int r[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0};
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[0], k_roots<true, false>, kBlock, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[1], k_roots<false, false>, kBlock, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[2], k_roots<true, true>, kBlock, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r[3], k_roots<false, true>, kBlock, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d[0], k_divide<true, false, kCellsPerLane>, kBlock, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d[1], k_divide<false, false, kCellsPerLane>, kBlock, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d[2], k_divide<true, true, kCellsPerLane>, kBlock, 0);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d[3], k_divide<false, true, kCellsPerLane>, kBlock, 0);
  *root_blocks = *std::min_element(r, r + 4);
  *divide_blocks = *std::min_element(d, d + 4);
  return (int)e;
}

}  // namespace pc
