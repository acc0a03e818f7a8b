// Test infrastructure only: the CPU oracle for the proliferation path (see oracle.h).
//
// Written independently of the product sources. Each function names the reference
// code it restates; the random stream it consumes is the engine's documented stream
// (Philox4x32-10 counters + FP32 ziggurat), re-implemented here from its definition.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_error;

// ---------------------------------------------------------------- Philox4x32-10 ----
// Salmon et al., SC'11: per round (L0,R0,L1,R1) -> (hi(M1*L1)^R0^k0, lo(M1*L1),
// hi(M0*L0)^R1^k1, lo(M0*L0)) with (L0,R0,L1,R1) = (x,y,z,w); keys bumped by the Weyl
// constants between rounds.
void philox_block(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t x = in[0], y = in[1], z = in[2], w = in[3];
  for (int round = 0; round < 10; ++round) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * z;
    const uint32_t nx = (uint32_t)(p1 >> 32) ^ y ^ k0;
    const uint32_t ny = (uint32_t)p1;
    const uint32_t nz = (uint32_t)(p0 >> 32) ^ w ^ k1;
    const uint32_t nw = (uint32_t)p0;
    x = nx;
    y = ny;
    z = nz;
    w = nw;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = x;
  out[1] = y;
  out[2] = z;
  out[3] = w;
}

const uint32_t kRoot = 0x30000000u, kPair = 0x10000000u, kChild = 0x20000000u;

float bits_to_float(uint32_t b) {
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}
uint32_t float_to_bits(float f) {
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
}

// ------------------------------------------------- FP32 exp/log of the slow path ---
// exp: n = floor(x*log2(e) + 1/2), r = x - n*ln2 (two-part ln2), Horner form of the
// degree-7 Taylor polynomial, times 2^n built from the exponent bits.
float o_expf(float x) {
  float n = std::floor(x * 1.44269502162933349609375f + 0.5f);
  float r = (x - n * 0.693145751953125f) - n * 1.4286068203094172e-06f;
  const float c[8] = {1.984126984126984e-4f, 1.388888888888889e-3f, 8.333333333333333e-3f,
                      4.166666666666667e-2f, 1.666666666666667e-1f, 0.5f, 1.0f, 1.0f};
  float p = c[0];
  for (int i = 1; i < 8; ++i) p = p * r + c[i];
  int e = (int)n + 127;
  if (e <= 0) return 0.0f;
  return p * bits_to_float((uint32_t)e << 23);
}

// log: u = m*2^e, m moved into [sqrt(1/2), sqrt(2)); log(m) = 2 atanh(s) with
// s = (m-1)/(m+1) summed to s^9; result e*ln2_hi + (e*ln2_lo + log(m)).
float o_logf(float u) {
  const uint32_t b = float_to_bits(u);
  int e = (int)((b >> 23) & 0xFF) - 127;
  float m = bits_to_float((b & 0x7FFFFFu) | 0x3F800000u);
  if (m > 1.41421353816986083984375f) {
    m = m * 0.5f;
    e = e + 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  const float c[5] = {0.2222222222222222f, 0.2857142857142857f, 0.4f, 0.6666666666666666f,
                      2.0f};
  float p = c[0];
  for (int i = 1; i < 5; ++i) p = p * s2 + c[i];
  const float lm = p * s;
  const float fe = (float)e;
  return fe * 0.693145751953125f + (fe * 1.4286068203094172e-06f + lm);
}

// ------------------------------------------------------------ ziggurat tables ------
// Marsaglia & Tsang (2000) construction with 1024 layers for the normal density
// f(x) = exp(-x^2/2): x_1 = r, x_{i+1} = sqrt(-2 ln(v/x_i + f(x_i))), base width v/f(r),
// with r = 4.0388498461095045227 and v = 1.2263246463530880729e-3 (the closure of the
// 1024-layer construction, solved numerically by bisection; the same solver reproduces the
// published 256-layer pair r = 3.6541528853610088, v = 4.9286732339746553e-3).
const int kLayers = 1024;
const uint32_t kLayerMask = kLayers - 1;
const double kR = 4.0388498461095045227, kV = 1.2263246463530880729e-3;

struct Tables {
  uint32_t k[kLayers];
  float w[kLayers];
  float f[kLayers + 1];
};

Tables make_tables() {
  const double r = kR, v = kV, two31 = 2147483648.0;
  double x[kLayers + 1];
  x[1] = r;
  for (int i = 1; i < kLayers - 1; ++i) x[i + 1] = std::sqrt(-2.0 * std::log(v / x[i] + std::exp(-0.5 * x[i] * x[i])));
  x[kLayers] = 0.0;
  const double base = v / std::exp(-0.5 * r * r);
  Tables t;
  t.k[0] = (uint32_t)std::floor(r / base * two31);
  t.w[0] = (float)(base / two31);
  t.f[0] = 0.0f;
  for (int i = 1; i < kLayers; ++i) {
    t.k[i] = (uint32_t)std::floor(x[i + 1] / x[i] * two31);
    t.w[i] = (float)(x[i] / two31);
    t.f[i] = (float)std::exp(-0.5 * x[i] * x[i]);
  }
  t.f[kLayers] = 1.0f;
  return t;
}

const Tables& tables() {
  static const Tables t = make_tables();
  return t;
}

// The private stream of one node: blocks {node_lo, node_hi, root, CHILD | i}, words x..w.
struct NodeStream {
  uint32_t ctr[4];
  uint32_t k0, k1;
  uint32_t words[4];
  int used = 4;
  uint32_t block = 0;
  NodeStream(uint64_t node, uint32_t root, uint32_t key0, uint32_t key1) {
    ctr[0] = (uint32_t)node;
    ctr[1] = (uint32_t)(node >> 32);
    ctr[2] = root;
    k0 = key0;
    k1 = key1;
  }
  uint32_t next() {
    if (used == 4) {
      ctr[3] = kChild | block;
      ++block;
      philox_block(ctr, k0, k1, words);
      used = 0;
    }
    return words[used++];
  }
};

float u24_open_closed(uint32_t w) { return (float)((w >> 8) + 1u) * 5.9604644775390625e-8f; }
float u24_closed_open(uint32_t w) { return (float)(w >> 8) * 5.9604644775390625e-8f; }

// One ziggurat normal: fast strip test, else the tail (layer 0) or the wedge test, and a
// full restart from the node stream when the wedge rejects. The first attempt's wedge
// uniform comes from the pair block when `have_wedge` is set.
float ziggurat(uint32_t j, uint32_t layer, bool have_wedge, uint32_t wedge_bits, NodeStream& ns) {
  const Tables& t = tables();
  const float rf = (float)kR;  // the tail starts at r
  bool first = have_wedge;
  while (true) {
    const uint32_t mag = j & 0x7FFFFFFFu;
    const float sign = (j & 0x80000000u) ? -1.0f : 1.0f;
    if (mag < t.k[layer]) return sign * ((float)mag * t.w[layer]);
    if (layer == 0) {
      while (true) {
        const float a = -o_logf(u24_open_closed(ns.next())) / rf;
        const float b = -o_logf(u24_open_closed(ns.next()));
        if (b + b > a * a) return sign * (rf + a);
      }
    }
    const float x = (float)mag * t.w[layer];
    const float u = u24_closed_open(first ? wedge_bits : ns.next());
    if (t.f[layer] + u * (t.f[layer + 1] - t.f[layer]) < o_expf(-0.5f * (x * x)))
      return sign * x;
    first = false;
    j = ns.next();
    layer = ns.next() & kLayerMask;
  }
}

// Pair block of node `parent`: child c's magnitude word, layer (bits 10c..10c+9 of word 2)
// and 22 wedge bits in the top of a word (child 0: low 22 bits of word 3; child 1: top 10
// bits of word 3 above the top 12 bits of word 2).
struct PairDraw {
  uint32_t j, layer, wedge;
};

PairDraw pair_draw(uint64_t parent, uint32_t c, uint32_t root, uint32_t k0, uint32_t k1) {
  const uint32_t pc[4] = {(uint32_t)parent, (uint32_t)(parent >> 32), root, kPair};
  uint32_t pw[4];
  philox_block(pc, k0, k1, pw);
  PairDraw d;
  d.j = pw[c];
  d.layer = (pw[2] >> (10 * c)) & kLayerMask;
  d.wedge = c == 0 ? (pw[3] << 10) : (((pw[3] >> 22) << 22) | ((pw[2] >> 20) << 10));
  return d;
}

// The division time of child c of node `parent` (restates determine_cell_timer,
// src/simulation/cell.cu:106-122: tau ~ N(mean, sd) truncated to tau > 0 by rejection).
double draw_tau(uint64_t parent, uint32_t c, uint32_t root, uint32_t k0, uint32_t k1,
                double mean, double sd) {
  const PairDraw p = pair_draw(parent, c, root, k0, k1);
  uint32_t j = p.j, layer = p.layer;
  bool have_wedge = true;
  NodeStream ns(2 * parent + c, root, k0, k1);
  while (true) {
    const float z = ziggurat(j, layer, have_wedge, p.wedge, ns);
    const double tau = std::fma(sd, (double)z, mean);
    if (tau > 0.0) return tau;
    have_wedge = false;
    j = ns.next();
    layer = ns.next() & kLayerMask;
  }
}

// ---------------------------------------------------------------- the model --------
enum Mode { kNormal = 0, kQuiescent = 1, kZeroMean = 2 };

struct Type {
  double ratio, mean, sd;
  uint32_t file_index;
  int mode;
};

struct Cell {  // the reference's `cell` (src/simulation/data_types.h:12-19)
  uint32_t type;
  double fluorescence, timer, t;
};

struct Model {
  std::vector<double> bin_value;
  std::vector<uint64_t> bin_start;  // nbins + 1 root offsets
  std::vector<Type> types;          // sorted by ratio, descending (parser.cu:184)
  std::vector<double> cum;
  uint32_t fallback = 0;
  std::vector<double> values;  // the output value set, ascending
  double t_max = 0, phi = 0;
  uint32_t k0 = 0, k1 = 0;
};

struct Acc {
  std::vector<uint64_t> counts;  // [value][sorted type]
  uint64_t divisions = 0, leaves = 0, uncounted = 0, vanished = 0, max_gen = 0;
  bool depth_error = false;
};

// Leaf count (restates proliferation.cu:351-381: binary search for an exactly equal value;
// a value missing from the set is not counted).
void count_leaf(const Model& m, Acc& a, const Cell& c) {
  int64_t lo = 0, hi = (int64_t)m.values.size() - 1;
  while (lo <= hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (m.values[mid] == c.fluorescence) {
      a.counts[mid * m.types.size() + c.type] += 1;
      a.leaves += 1;
      return;
    }
    if (m.values[mid] > c.fluorescence)
      hi = mid - 1;
    else
      lo = mid + 1;
  }
  a.uncounted += 1;
}

// out_of_time (proliferation.cu:404-410) and one step of device::proliferate
// (proliferation.cu:315-381) applied depth-first.
void visit(const Model& m, Acc& a, const Cell& cell, uint64_t node, uint32_t root, uint32_t gen) {
  if (gen > a.max_gen) a.max_gen = gen;
  const bool out_of_time = (cell.timer < 0.0) || (cell.t + cell.timer > m.t_max);
  if (out_of_time) {
    count_leaf(m, a, cell);
    return;
  }
  if (!(cell.fluorescence / 2 > m.phi)) {
    a.vanished += 1;
    return;
  }
  if (gen >= 62) {
    a.depth_error = true;
    return;
  }
  a.divisions += 1;
  const Type& ty = m.types[cell.type];
  for (uint32_t c = 0; c < 2; ++c) {
    Cell child;
    child.type = cell.type;
    child.fluorescence = cell.fluorescence / 2;
    child.t = cell.t + cell.timer;
    child.timer = (ty.mode == kZeroMean) ? 0.0 : draw_tau(node, c, root, m.k0, m.k1, ty.mean, ty.sd);
    visit(m, a, child, 2 * node + c, root, gen + 1);
  }
}

// Root creation (restates create_cells_population and create_cell with type -1,
// cells_population.cu:97-117 and cell.cu:25-143).
void simulate_root(const Model& m, Acc& a, uint64_t r, uint32_t bin) {
  const uint32_t root = (uint32_t)r;
  const uint32_t rc[4] = {0u, 0u, root, kRoot};
  uint32_t rw[4];
  philox_block(rc, m.k0, m.k1, rw);
  const double u_type = (double)(((uint64_t)rw[0] << 21) | (rw[1] >> 11)) * 1.1102230246251565e-16;
  const double u_age = (double)((((uint64_t)rw[2] << 21) | (rw[3] >> 11)) + 1) * 1.1102230246251565e-16;
  uint32_t type = m.fallback;
  for (uint32_t i = 0; i < m.types.size(); ++i) {
    if (u_type < m.cum[i]) {
      type = i;
      break;
    }
  }
  const Type& ty = m.types[type];
  Cell c;
  c.type = type;
  c.fluorescence = m.bin_value[bin];
  if (ty.mode == kQuiescent) {
    c.timer = -1.0;
    c.t = 0.0;
  } else if (ty.mode == kZeroMean) {
    c.timer = 0.0;
    c.t = 0.0;
  } else {
    const double tau = draw_tau(0, 1, root, m.k0, m.k1, ty.mean, ty.sd);
    c.timer = tau;
    c.t = tau * u_age;
  }
  visit(m, a, c, 1, root, 0);
}

bool build_model(Model& m, const double* values, const uint64_t* freqs, uint64_t nrows,
                 const double* ratio, const double* mean, const double* sd, uint32_t ntypes,
                 double t_max, double phi, int phi_given, uint64_t seed) {
  if (!(t_max >= 0.0) || std::isinf(t_max)) {
    g_error = "t_max must be finite and >= 0";
    return false;
  }
  if (ntypes == 0) {
    g_error = "ERROR: proportion distribution of cell types does not sum to 1, aborting.";
    return false;
  }
  // Automatic threshold (parser.cu:80-96).
  double threshold = phi_given ? phi : 0.0;
  if (!phi_given) {
    for (uint64_t i = 0; i < nrows; ++i)
      if (freqs[i] > 0 && (threshold == 0.0 || values[i] < threshold)) threshold = values[i];
  }
  if (!(threshold > 0.0) || std::isinf(threshold)) {
    g_error = "phi must be finite and > 0";
    return false;
  }
  m.phi = threshold;
  m.t_max = (t_max == 0.0) ? 0.0 : t_max;
  std::map<double, uint64_t> set;
  uint64_t start = 0;
  m.bin_start.push_back(0);
  for (uint64_t i = 0; i < nrows; ++i) {
    if (freqs[i] == 0) continue;
    if (!std::isfinite(values[i])) {
      g_error = "histogram values must be finite";
      return false;
    }
    m.bin_value.push_back(values[i]);
    start += freqs[i];
    m.bin_start.push_back(start);
    for (double cur = values[i]; cur >= threshold; cur = cur / 2) set.insert(std::make_pair(cur, 0));
  }
  for (auto& kv : set) m.values.push_back(kv.first);
  // Types (parser.cu:156-185): ratio sum check, then a stable sort by ratio descending.
  double sum = 0.0;
  for (uint32_t i = 0; i < ntypes; ++i) {
    if (!std::isfinite(ratio[i]) || !std::isfinite(mean[i]) || !std::isfinite(sd[i])) {
      g_error = "cell type parameters must be finite";
      return false;
    }
    sum += ratio[i];
  }
  if (std::fabs(1.0 - sum) > 1.0 / std::pow(10.0, 8.0)) {
    g_error = "ERROR: proportion distribution of cell types does not sum to 1, aborting.";
    return false;
  }
  for (uint32_t i = 0; i < ntypes; ++i) {
    Type t;
    t.ratio = ratio[i];
    t.mean = mean[i];
    t.sd = sd[i];
    t.file_index = i;
    t.mode = mean[i] < 0.0 ? kQuiescent : (mean[i] == 0.0 ? kZeroMean : kNormal);
    m.types.push_back(t);
  }
  std::stable_sort(m.types.begin(), m.types.end(),
                   [](const Type& a, const Type& b) { return a.ratio > b.ratio; });
  double acc = 0.0;
  for (auto& t : m.types) {
    acc += t.ratio;
    m.cum.push_back(acc);
  }
  m.fallback = 0;
  for (uint32_t i = 0; i < m.types.size(); ++i)
    if (m.types[i].ratio > 0.0) m.fallback = i;
  m.k0 = (uint32_t)seed;
  m.k1 = (uint32_t)(seed >> 32);
  return true;
}

}  // namespace

struct oracle_result {
  std::vector<double> values;
  std::vector<uint64_t> totals, per_type;
  uint32_t ntypes = 0;
  uint64_t stats[6] = {0, 0, 0, 0, 0, 0};
};

extern "C" {

const char* oracle_last_error(void) { return g_error.c_str(); }

oracle_result* oracle_simulate(const double* values, const uint64_t* freqs, uint64_t nrows,
                               const double* ratio, const double* mean, const double* sd,
                               uint32_t ntypes, double t_max, double phi, int phi_given,
                               uint64_t seed, uint64_t root_begin, uint64_t root_end,
                               int nthreads) {
  Model m;
  if (!build_model(m, values, freqs, nrows, ratio, mean, sd, ntypes, t_max, phi, phi_given, seed))
    return nullptr;
  const uint64_t total_roots = m.bin_start.back();
  if (total_roots > 0xFFFFFFFFull) {
    g_error = "more than 2^32-1 initial cells";
    return nullptr;
  }
  const uint64_t r0 = std::min(root_begin, total_roots);
  const uint64_t r1 = std::min(root_end, total_roots);
  const uint64_t n = r1 > r0 ? r1 - r0 : 0;
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  if ((uint64_t)nt > n) nt = (int)std::max<uint64_t>(1, n);
  std::vector<Acc> accs(nt);
  // Interleaved root blocks balance the work of uneven bins across threads.
  const uint64_t kBlock = 64;
  auto work = [&](int tid) {
    Acc& a = accs[tid];
    a.counts.assign(m.values.size() * m.types.size(), 0);
    for (uint64_t b0 = r0 + (uint64_t)tid * kBlock; b0 < r1; b0 += (uint64_t)nt * kBlock) {
      const uint64_t b1 = std::min(r1, b0 + kBlock);
      uint32_t bin = (uint32_t)(std::upper_bound(m.bin_start.begin(), m.bin_start.end(), b0) -
                                m.bin_start.begin() - 1);
      for (uint64_t r = b0; r < b1; ++r) {
        while (r >= m.bin_start[bin + 1]) ++bin;
        simulate_root(m, a, r, bin);
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& t : th) t.join();

  oracle_result* res = new oracle_result();
  const uint32_t T = (uint32_t)m.types.size();
  res->ntypes = T;
  res->values = m.values;
  res->totals.assign(m.values.size(), 0);
  res->per_type.assign(m.values.size() * T, 0);
  bool depth_error = false;
  for (auto& a : accs) {
    for (uint64_t v = 0; v < m.values.size(); ++v)
      for (uint32_t k = 0; k < T; ++k) {
        const uint64_t c = a.counts[v * T + k];
        res->totals[v] += c;
        res->per_type[v * T + m.types[k].file_index] += c;
      }
    res->stats[1] += a.divisions;
    res->stats[2] += a.leaves;
    res->stats[3] += a.uncounted;
    res->stats[4] += a.vanished;
    res->stats[5] = std::max(res->stats[5], a.max_gen);
    depth_error |= a.depth_error;
  }
  res->stats[0] = n;
  if (depth_error) {
    delete res;
    g_error = "a lineage exceeded 62 generations";
    return nullptr;
  }
  return res;
}

uint64_t oracle_result_nvalues(const oracle_result* r) { return r->values.size(); }
uint32_t oracle_result_ntypes(const oracle_result* r) { return r->ntypes; }

void oracle_result_copy(const oracle_result* r, double* values, uint64_t* totals,
                        uint64_t* per_type, uint64_t* stats) {
  if (values) std::copy(r->values.begin(), r->values.end(), values);
  if (totals) std::copy(r->totals.begin(), r->totals.end(), totals);
  if (per_type) std::copy(r->per_type.begin(), r->per_type.end(), per_type);
  if (stats) std::copy(r->stats, r->stats + 6, stats);
}

void oracle_result_free(oracle_result* r) { delete r; }

void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox_block(ctr, key[0], key[1], out);
}

void oracle_tables(uint32_t* k, uint32_t* w_bits, uint32_t* f_bits) {
  const Tables& t = tables();
  for (int i = 0; i < kLayers; ++i) {
    k[i] = t.k[i];
    w_bits[i] = float_to_bits(t.w[i]);
  }
  for (int i = 0; i <= kLayers; ++i) f_bits[i] = float_to_bits(t.f[i]);
}

void oracle_normals(uint64_t seed, uint32_t root, uint64_t first_parent, uint64_t count, float* z) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (uint64_t i = 0; i < count; ++i) {
    const uint64_t parent = first_parent + i / 2;
    const uint32_t c = (uint32_t)(i & 1);
    const PairDraw p = pair_draw(parent, c, root, k0, k1);
    NodeStream ns(2 * parent + c, root, k0, k1);
    z[i] = ziggurat(p.j, p.layer, true, p.wedge, ns);
  }
}

double oracle_tau(uint64_t seed, uint32_t root, uint64_t parent, uint32_t child, double mean, double sd) {
  return draw_tau(parent, child, root, (uint32_t)seed, (uint32_t)(seed >> 32), mean, sd);
}

float oracle_expf(float x) { return o_expf(x); }
float oracle_logf(float u) { return o_logf(u); }

}  // extern "C"

// ---------------------------------------------------------------- smoothed form ----
// The smoothed, differentiable form restated in FP64, step for step as oracle/smooth_ref.py
// states it (same lineages and draws, same stopping rule), multi-threaded for the
// benchmark's CPU baseline. The reference has no smoothed form; its plain-form pieces are
// those of the oracle above (initial age, division rule, phi cap).
namespace {

const uint32_t kPath = 0x40000000u;

void log_sig(double x, double& ls, double& l1m) {
  const double L = std::log1p(std::exp(-std::fabs(x)));
  ls = -(std::max(-x, 0.0) + L);
  l1m = -(std::max(x, 0.0) + L);
}

struct SmoothBin {
  double v;
  uint64_t f, r0;
  uint32_t cap;
  std::vector<int64_t> vi;  // generation -> output value index or -1
};

}  // namespace

extern "C" int oracle_smooth(const double* values, const uint64_t* freqs, uint64_t nrows, double t_max,
                             double phi, int phi_given, double h, uint32_t paths, uint64_t seed,
                             const double* params, uint32_t ncand, uint32_t ntypes,
                             const double* grad_expected, double* expected, double* grad,
                             uint64_t nvalues_cap, uint64_t* nvalues, int nthreads) {
  std::vector<SmoothBin> bins;
  double thr = phi_given ? phi : 0.0;
  for (uint64_t i = 0; i < nrows; ++i)
    if (freqs[i] > 0 && !phi_given && (thr == 0.0 || values[i] < thr)) thr = values[i];
  std::vector<double> vals;
  uint64_t ncells = 0;
  for (uint64_t i = 0; i < nrows; ++i) {
    if (freqs[i] == 0) continue;
    SmoothBin b;
    b.v = values[i];
    b.f = freqs[i];
    b.r0 = ncells;
    ncells += freqs[i];
    b.cap = 0;
    for (double x = b.v; x / 2 > thr && b.cap < 4096; x = x / 2) ++b.cap;
    for (double x = b.v; x >= thr; x = x / 2) vals.push_back(x);
    bins.push_back(b);
  }
  std::sort(vals.begin(), vals.end());
  vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
  *nvalues = vals.size();
  if (nvalues_cap < vals.size() || ncells * paths > 0xFFFFFFFFull) return -1;
  const uint64_t V = vals.size();
  for (SmoothBin& b : bins) {
    double x = b.v;
    for (uint32_t g = 0; g <= b.cap; ++g, x = x / 2) {
      int64_t idx = -1;
      if (g > 0 || b.v >= thr) {
        auto it = std::lower_bound(vals.begin(), vals.end(), x);
        if (it != vals.end() && *it == x) idx = it - vals.begin();
      }
      b.vi.push_back(idx);
    }
  }
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const uint32_t K = ntypes, C = ncand;
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::max(1u, std::thread::hardware_concurrency());
  nt = (unsigned)std::min<uint64_t>(nt, std::max<uint64_t>(1, ncells));
  std::vector<std::vector<double>> E(nt, std::vector<double>((size_t)C * V, 0.0));
  std::vector<std::vector<double>> G(nt, std::vector<double>((size_t)C * K * 3, 0.0));
  const double ln2 = std::log(2.0);
  auto work = [&](unsigned t) {
    double* e = E[t].data();
    double* gr = G[t].data();
    std::vector<uint64_t> nodes;
    std::vector<double> zs;
    size_t bi = 0;
    const uint64_t lo = ncells * t / nt, hi = ncells * (t + 1) / nt;
    for (uint64_t r = lo; r < hi; ++r) {
      while (r >= bins[bi].r0 + bins[bi].f) ++bi;
      const SmoothBin& b = bins[bi];
      const double stop = -40.0 - ln2 * (b.cap + 1);
      for (uint32_t m = 0; m < paths; ++m) {
        const uint32_t vr = (uint32_t)(r + (uint64_t)m * ncells);
        const uint32_t rc[4] = {0u, 0u, vr, kRoot}, pc[4] = {0u, 0u, vr, kPath};
        uint32_t rw[4], pw[4];
        philox_block(rc, k0, k1, rw);
        philox_block(pc, k0, k1, pw);
        const double U = (double)((((uint64_t)rw[2] << 21) | (rw[3] >> 11)) + 1) * 1.1102230246251565e-16;
        const uint64_t bits = (uint64_t)pw[0] | ((uint64_t)pw[1] << 32);
        nodes.assign(b.cap + 1, 0);
        zs.assign(b.cap + 1, 0.0);
        uint64_t node = 1;
        for (uint32_t j = 0; j <= b.cap; ++j) {
          nodes[j] = node;
          node = 2 * node + ((bits >> j) & 1ull);
        }
        for (uint32_t j = 0; j <= b.cap; ++j) {
          const uint64_t parent = nodes[j] >> 1;
          const uint32_t c = (uint32_t)(nodes[j] & 1ull);
          const PairDraw p = pair_draw(parent, c, vr, k0, k1);
          NodeStream ns(2 * parent + c, vr, k0, k1);
          zs[j] = (double)ziggurat(p.j, p.layer, true, p.wedge, ns);
        }
        for (uint32_t c = 0; c < C; ++c)
          for (uint32_t k = 0; k < K; ++k) {
            const double* P = params + ((size_t)c * K + k) * 3;
            const double ratio = P[0], mu = P[1];
            double sd = P[2];
            double* gk = gr + ((size_t)c * K + k) * 3;
            if (mu < 0) {
              if (b.vi[0] >= 0) {
                e[(size_t)c * V + b.vi[0]] += ratio / paths;
                if (grad_expected) gk[0] += grad_expected[(size_t)c * V + b.vi[0]] / paths;
              }
              continue;
            }
            if (mu == 0) sd = 0.0;
            double S = 0.0, logp = 0.0, dS0 = 0.0, dS1 = 0.0, D0 = 0.0, D1 = 0.0;
            for (uint32_t j = 1; j <= b.cap + 1; ++j) {
              const double z = mu != 0 ? zs[j - 1] : 0.0;
              const double tau = sd * z + mu;
              if (j == 1) {
                S = tau * U + tau;
                dS0 = 1.0 + U;
                dS1 = z * (1.0 + U);
              } else {
                S += tau;
                dS0 += 1.0;
                dS1 += z;
              }
              if (mu == 0) dS0 = dS1 = 0.0;
              double ls, l1m;
              log_sig((t_max - S) / h, ls, l1m);
              const double w = std::exp(logp + l1m);
              const uint32_t g = j - 1;
              if (b.vi[g] >= 0) {
                const double two_g = std::ldexp(1.0, (int)g);
                e[(size_t)c * V + b.vi[g]] += ratio * two_g * w / paths;
                if (grad_expected) {
                  const double a = grad_expected[(size_t)c * V + b.vi[g]] * two_g * w / paths;
                  gk[0] += a;
                  const double s = std::exp(ls);
                  gk[1] += ratio * a * (D0 + s / h * dS0);
                  gk[2] += ratio * a * (D1 + s / h * dS1);
                }
              }
              const double oms = std::exp(l1m);
              D0 = D0 - oms / h * dS0;
              D1 = D1 - oms / h * dS1;
              logp += ls;
              if (logp < stop) break;
            }
          }
      }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  for (size_t i = 0; i < (size_t)C * V; ++i) {
    double s = 0.0;
    for (unsigned t = 0; t < nt; ++t) s += E[t][i];
    expected[i] = s;
  }
  if (grad)
    for (size_t i = 0; i < (size_t)C * K * 3; ++i) {
      double s = 0.0;
      for (unsigned t = 0; t < nt; ++t) s += G[t][i];
      grad[i] = s;
    }
  return 0;
}
