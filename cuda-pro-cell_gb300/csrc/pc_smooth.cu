// Smoothed, differentiable form of the proliferation path: expected histogram counts as a
// smooth function of the cell-type parameters (ratio, mean, sd), and their adjoint.
//
// Model. Along one lineage of an initial cell (type k), the due times are S_1 = tau_1 * U +
// tau_1 (the initial age, src/simulation/cells_population.cu:124-143) and S_j = S_{j-1} +
// tau_j, tau_j = mean_k + sd_k * z_j, z_j the node's standard normal from the plain form's
// Philox counters (without the truncation tau > 0). The hard rule "a cell divides iff it is
// due by t_max" (proliferation.cu:404-410) becomes s_j = sigmoid((T - S_j) / h): the weight
// of the lineage reaching generation g and stopping there (a leaf) is
//     w_g = s_1 s_2 ... s_g (1 - s_{g+1}),
// and a cell of generation g has 2^g lineages of equal law, so the expected number of
// generation-g leaves of one initial cell is E_g = sum_k ratio_k 2^g E[w_g], 0 <= g <= cap_b,
// estimated by `paths` lineages sampled per initial cell (uniform random left/right
// choices; at g = cap_b only "not due" survives, due cells vanish as in the plain form).
// Each sampled lineage is an independent replica of its initial cell: replica m of cell r
// takes every draw (initial age, normals, path) from the plain form's counters of cell
// r + m * ncells, so the estimate converges to the expectation over all randomness, and
// replica 0 shares its draws with the plain form run on the same seed.
// Types enter analytically through ratio_k, so d/d ratio is exact. Weights are running
// products of sigmoids (FP32), never negative, and a lineage stops once no later generation
// can add more than e^-40 cells, well before such a product could leave the normal range.
//
// Adjoint. dw_g/dtheta = w_g (D_g + s_{g+1} / h dS_{g+1}/dtheta) with the running tangent
// D_g = -sum_{i <= g} (1 - s_i) / h dS_i/dtheta, dS_j/dmean = U + j and dS_j/dsd = z_1 (1 + U)
// + z_2 + ... + z_j. The backward kernel walks the same lineages again with the upstream
// gradients A_g = dL/dE_g, regenerating every z from its counter (nothing of the forward pass
// is stored).
//
// Work layout: one block per (bin, group of 32 candidates, type); lane l of every warp is
// candidate 32 * group + l, and the block's 4 warps take the bin's lineages 32 at a time:
// first each lane stages one lineage's normals into shared memory, then every lane walks all
// 32 lineages for its own candidate, reading the shared draws. The draws depend on the seed
// and the bins only: a smoothed plan makes them once (k_smooth_draws: one Philox block and
// ziggurat draw per generation) and keeps them in device memory, so a pass only reads them
// back (plans too large for that draw them in every block, once per 32 candidates and type).
// Remaining time R = T - S is carried on the FP32 pipe as a float on a fixed grid plus
// a float remainder (RemGrid: exact grid sums, 11 FP32 operations per step; GB300's FP64
// pipe has 2 lanes per clock per SM), or in FP64 where that form's error bound would exceed
// 2^-22 h (RemFp64). Per-thread partial sums
// (compensated FP32) live in shared memory and are reduced over the warps in a fixed order,
// and the types are added in a fixed order by the merge, so results are deterministic.
#include <cuda_runtime.h>

#include "pc_engine.h"

namespace pc {

namespace {

constexpr int kThreads = 128;
constexpr uint32_t kBudget = 1u << 16;
// Resident blocks per SM the lineage-walk kernels are compiled for (registers per thread =
// 65536 / (128 x this)); compile-time tuning, results do not depend on it. Measured on the
// calibration input with the draws made in every pass: 5 blocks (96 registers) forward
// 1.91 ms, adjoint 2.62 ms; 6 (80 registers) 1.75 / 2.45 ms; 8 (64 registers) 3.04 / 2.45 ms:
// 6 for those kernels. With the plan's draws kept in device memory they need fewer registers:
// 6 blocks forward 1.170, adjoint 1.321, Jacobian 1.380 ms; 7 (72 registers, no spills) 1.115
// / 1.267 / 1.301 ms; 8 (64 registers) 1.066 / 1.213 ms, the Jacobian held at 7 by its shared
// memory (4 floats per generation row and thread).
constexpr int kBlocksDrawn = 6;
constexpr int kBlocksKept = 8;
constexpr int kBlocksKeptJacobian = 7;

__device__ __forceinline__ double f32_to_f64_bits(float z) {
  const uint32_t f = __float_as_uint(z);
  const uint32_t a = f & 0x7FFFFFFFu;
  const uint32_t hi = (f & 0x80000000u) | (a ? (a >> 3) + (896u << 20) : 0u);
  return __hiloint2double((int)hi, (int)(f << 29));
}

__device__ __noinline__ float node_z_slow(uint32_t j, uint32_t layer, uint32_t wedge, uint64_t node, uint32_t root,
                                          uint32_t k0, uint32_t k1, const ZigTables& Z, uint32_t* error) {
  ChildStream cs = child_stream(node, root, k0, k1);
  uint32_t budget = kBudget;
  const float z = zig_normal(j, layer, true, wedge, cs, Z, budget);
  if (budget == 0u) atomicOr(error, 2u);
  return z;
}

// The standard normal of tree node `node` (heap index; the initial cell is node 1): the
// plain form's draw for that node (first attempt from the parent's pair block, the node's
// private stream after a rejection), without the truncation.
__device__ __forceinline__ float node_z(uint64_t node, uint32_t root, uint32_t k0, uint32_t k1, const ZigTables& Z,
                                        uint32_t* error) {
  const uint64_t parent = node >> 1;
  const uint32_t c = (uint32_t)(node & 1ull);
  const u32x4 P = philox(u32x4{(uint32_t)parent, (uint32_t)(parent >> 32), root, kPurposePair}, k0, k1);
  const uint32_t j = c ? P.y : P.x;
  const uint32_t layer = pair_layer(P, c);
  const uint32_t mag = j & 0x7FFFFFFFu;
  if (mag < Z.k[layer]) {
    const float x = __fmul_rn((float)mag, Z.w[layer]);
    return (j >> 31) ? -x : x;
  }
  return node_z_slow(j, layer, pair_wedge_bits(P, c), node, root, k0, k1, Z, error);
}

// Compensated (Kahan) addition into sum = p[0], compensation = p[kThreads].
__device__ __forceinline__ void kahan_add(float* p, float x) {
  const float sum = p[0], c = p[kThreads];
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(sum, y);
  p[kThreads] = __fsub_rn(__fsub_rn(t, sum), y);
  p[0] = t;
}

// sigmoid(x) and 1 - sigmoid(x) from e = exp(-|x|) and one reciprocal: 1 / (1 + e) is the
// larger of the two and e / (1 + e) the smaller (for x >= 0, sigmoid(x) is the larger), so
// both keep their relative accuracy however far x is from 0. With the fast exp and
// reciprocal intrinsics (relative errors near 2^-22) each factor of a weight is good to a few
// 1e-7, and a weight of up to ~60 factors to about 1e-5 at worst (checked against the FP64
// CPU restatement to 2e-5 and against central differences to 1e-3).
__device__ __forceinline__ void sig_pair(float x, float& s, float& one_m_s) {
  const float e = __expf(-fabsf(x));
  const float q = __fdividef(1.0f, 1.0f + e);
  const float eq = e * q;
  s = x >= 0.0f ? q : eq;
  one_m_s = x >= 0.0f ? eq : q;
}

// A per-block flag the compiler must keep as it is: passed through an empty asm, it cannot be
// re-derived inside the lineage loops from the FP64 comparison that produced it (measured:
// the forward kernel otherwise re-evaluated the grid test about 2.6 times per lineage walk,
// which kept GB300's slow FP64 pipe 69% busy).
__device__ __forceinline__ bool opaque(bool f) {
  uint32_t u = f ? 1u : 0u;
  asm volatile("" : "+r"(u));
  return u != 0u;
}

// x == 0.0 and x < 0.0 (for x not NaN) on the integer pipes.
__device__ __forceinline__ bool zero_bits(double x) {
  return ((unsigned long long)__double_as_longlong(x) << 1) == 0ull;
}
__device__ __forceinline__ bool neg_nonzero(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) != 0ull && (u << 1) != 0ull;
}

// A double rounded toward zero to float on the integer pipes (GB300 runs FP64<->FP32
// conversions on its slow FP64 pipe). |d| < 2^-126 gives 0, |d| >= 2^128 gives inf.
__device__ __forceinline__ float f64_to_f32_rz_any(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const uint32_t sign = hi & 0x80000000u, mag = hi & 0x7FFFFFFFu;
  if (mag < (897u << 20)) return __uint_as_float(sign);
  if (mag >= (1151u << 20)) return __uint_as_float(sign | 0x7F800000u);
  return __uint_as_float(sign | ((mag - (896u << 20)) << 3) | (lo >> 29));
}

// The remaining time R = T - S_j of a walk, in one of two forms with the same interface:
// first(z_1, U, 1 + U as hi/lo floats) sets R_1 = T - tau_1 (1 + U), step(z_j) subtracts
// tau_j = mean + sd z_j, x(1/h) returns R / h in FP32.
//
// RemFp64: R in FP64 (two FP64 operations per step; GB300 runs FP64 on a pipe of 2 lanes
// per clock per SM). Used only where the grid form below would not be exact enough.
struct RemFp64 {
  double mu, sigma, t_max, R;
  __device__ __forceinline__ void first(float z, double u_age, float, float) {
    const double tau = fma(sigma, f32_to_f64_bits(z), mu);
    R = t_max - fma(tau, u_age, tau);
  }
  __device__ __forceinline__ void step(float z) { R = R - fma(sigma, f32_to_f64_bits(z), mu); }
  __device__ __forceinline__ float x(float inv_h) const { return f64_to_f32_rz_any(R) * inv_h; }
};

// RemGrid: R on the FP32 pipe as Rh + Rl. Rh only ever holds multiples of the grid step
// g = 2^(m-23) below 2^(m+1) in magnitude (at most 24 significant bits), so sums and
// differences of such numbers are exact; Rl, a float below about 2 g per step in magnitude,
// takes every remainder. A product p = sd z is split exactly into p_h + p_l (one FMA), p_h
// is rounded to the grid by adding and subtracting C = 1.5 * 2^m (exact for |p_h| < 2^(m-1))
// and its fraction goes to Rl. With |R|, |tau| and |tau (1 + U)| bounded by 2^(m-1), every
// step is 11 FP32 operations; each step's rounding of Rl (|Rl| <= 1.25 g steps) adds at most
// 0.6 * 2^-23 g steps to the error of R, so it stays below 0.6 * 2^-23 * g * steps^2, which
// grid_setup keeps below 2^-19 h (a weight's relative error below 2^-18).
struct RemGrid {
  float C, mu_g, mu_f, sg_h, sg_l, t_g, t_f, Rh, Rl;
  __device__ __forceinline__ void split(float p, float& on_grid, float& rest) const {
    on_grid = __fsub_rn(__fadd_rn(p, C), C);
    rest = __fsub_rn(p, on_grid);
  }
  // tau = mean + sd z as tg (on the grid) + tf
  __device__ __forceinline__ void tau(float z, float& tg, float& tf) const {
    const float ph = __fmul_rn(sg_h, z);
    const float pl = __fmaf_rn(sg_l, z, __fmaf_rn(sg_h, z, -ph));
    float pg, pf;
    split(ph, pg, pf);
    tg = __fadd_rn(mu_g, pg);
    tf = __fadd_rn(__fadd_rn(mu_f, pf), pl);
  }
  __device__ __forceinline__ void first(float z, double, float u_hi, float u_lo) {
    float tg, tf;
    tau(z, tg, tf);
    // S_1 = (tg + tf)(u_hi + u_lo): tg u_hi exactly as qh + ql, the other terms rounded
    const float qh = __fmul_rn(tg, u_hi);
    const float ql = __fmaf_rn(tg, u_hi, -qh);
    const float rest = __fmaf_rn(tf, u_lo, __fmaf_rn(tg, u_lo, __fmaf_rn(tf, u_hi, ql)));
    float qg, qf;
    split(qh, qg, qf);
    Rh = __fsub_rn(t_g, qg);
    Rl = __fsub_rn(__fsub_rn(t_f, qf), rest);
  }
  __device__ __forceinline__ void step(float z) {
    float tg, tf;
    tau(z, tg, tf);
    Rh = __fsub_rn(Rh, tg);
    Rl = __fsub_rn(Rl, tf);
  }
  __device__ __forceinline__ float x(float inv_h) const { return __fmul_rn(__fadd_rn(Rh, Rl), inv_h); }
};

// The grid form for one candidate and bin, or false where its error bound would exceed
// 2^-19 h (very large t_max or means relative to h, or very deep bins): then the caller
// walks in FP64. |z| <= 8.25 bounds every normal the sampler returns (the ziggurat's tail
// draw is at most r - log(2^-24) / r = 8.21), so |tau| <= |mean| + 8.25 |sd| and
// |R_j| <= |T| + j max |tau|.
__device__ __forceinline__ bool grid_setup(RemGrid& r, double mu, double sigma, double t_max, uint32_t steps,
                                           double h) {
  const double B = fabs(t_max) + (double)(steps > 2u ? steps : 2u) * (fabs(mu) + 8.25 * fabs(sigma)) + 1.0;
  int e;
  frexp(B, &e);  // B < 2^e
  const int m = e + 1;
  const double g = ldexp(1.0, m - 23);
  if (!(g * (double)steps * (double)steps <= 16.0 * h) || m > 100) return false;
  const double mu_g = ldexp(rint(ldexp(mu, 23 - m)), m - 23);
  const double t_g = ldexp(rint(ldexp(t_max, 23 - m)), m - 23);
  r.C = (float)ldexp(1.5, m);
  r.mu_g = (float)mu_g;
  r.mu_f = (float)(mu - mu_g);
  r.sg_h = (float)sigma;
  r.sg_l = (float)(sigma - (double)r.sg_h);
  r.t_g = (float)t_g;
  r.t_f = (float)(t_max - t_g);
  r.Rh = r.Rl = 0.0f;
  return true;
}

// A lineage stops once no later generation can add more than e^-40 cells: every later leaf
// weight is at most s_1 ... s_j (the running product) times 2^g <= 2^(steps - 1), so the walk
// ends when that product falls below e^-40 2^-steps (above the smallest normal float for up
// to 68 steps; deeper bins walk on, at most until the product is 0).
constexpr float kNegligible = 4.24835426e-18f;  // e^-40
__device__ __forceinline__ float stop_level(uint32_t steps) { return ldexpf(kNegligible, -(int)steps); }

// A cell due at least 24 h before t_max (x = (T - S) / h > 24) divides with sigmoid(x), which
// rounds to 1 in FP32, and stays a leaf with 1 - sigmoid(x) < e^-24 = 3.8e-11: its step adds
// no leaf weight worth counting and changes neither the running product nor the tangents, so
// the walks only advance the remaining time there (the early generations of most lineages).
constexpr float kFar = 24.0f;

// Lineage i of a bin whose initial cells start at r0 (initial cell r0 + i / paths, replica
// i % paths, which draws as initial cell r + replica * ncells): its initial age, and the
// normals of the nodes it visits (heap nodes 1, 2 + b_1, ..., b_j the path bits) into
// z[j * zstride], j < steps.
__device__ __forceinline__ void draw_lineage(const SmoothArgs& A, const ZigTables& Z, uint64_t r0, uint64_t i,
                                             uint32_t steps, float* z, uint32_t zstride, double& u_age) {
  const uint32_t m = (uint32_t)(i % A.paths);
  const uint32_t root = (uint32_t)(r0 + i / A.paths) + m * A.ncells;
  const u32x4 R = philox(u32x4{0u, 0u, root, kPurposeRoot}, A.k0, A.k1);
  u_age = unit53_open_closed(R.z, R.w);
  const u32x4 B = philox(u32x4{0u, 0u, root, kPurposePath}, A.k0, A.k1);
  const uint64_t bits = (uint64_t)B.x | ((uint64_t)B.y << 32);
  uint64_t node = 1;
  for (uint32_t j = 0; j < steps; ++j) {
    z[j * zstride] = node_z(node, root, A.k0, A.k1, Z, A.error);
    node = 2ull * node + ((bits >> j) & 1ull);
  }
}

// A lineage's initial age U for the walks of all 32 candidates: U itself (FP64 form) and
// 1 + U as a pair of floats hi + lo (grid form; hi is also the FP32 dS_1/dmean).
__device__ __forceinline__ LineageU lineage_u(double u) {
  const double one = 1.0 + u;
  const float h = __double2float_rn(one);
  return LineageU{u, h, __double2float_rn(one - (double)h)};
}

// Lineage base + lane of a bin (initial cells from r0) into the warp's shared-memory draws
// zbuf[j * 32 + lane] and the block's u tables: read back from the plan's lineage tables
// (Kept), or drawn here when the plan keeps none. The kernels are instantiated for both, so
// neither path's code (the draw's FP64 set-up in particular) runs predicated in the other.
template <bool Kept>
__device__ __forceinline__ void stage_lineage(const SmoothArgs& A, const ZigTables& Z, uint64_t r0, uint64_t i,
                                              uint32_t steps, float* zlane, double* u_age, float* u_one,
                                              float* u_one_lo) {
  LineageU lu;
  if constexpr (Kept) {
    const uint64_t L = r0 * A.paths + i;
    const float4* zr = reinterpret_cast<const float4*>(A.lin_z + L * A.zrow);
    for (uint32_t j = 0; j < steps; j += 4u) {
      const float4 q = __ldg(zr + j / 4u);
      zlane[j * 32u] = q.x;
      if (j + 1u < steps) zlane[(j + 1u) * 32u] = q.y;
      if (j + 2u < steps) zlane[(j + 2u) * 32u] = q.z;
      if (j + 3u < steps) zlane[(j + 3u) * 32u] = q.w;
    }
    lu = A.lin_u[L];
  } else {
    double u;
    draw_lineage(A, Z, r0, i, steps, zlane, 32u, u);
    lu = lineage_u(u);
  }
  *u_age = lu.u;
  *u_one = lu.hi;
  *u_one_lo = lu.lo;
}

// One lineage (its normals z[j * 32], j = 0.., and initial age U; 1 + U = u1 + u1_lo) for one
// type of one candidate, whose remaining time R = T - S_j is carried by `r`. Forward:
// acc[2g * kThreads] += w_g (compensated; the caller scales row g by ratio / paths * 2^g).
// Backward (Ag2[g] = 2^g dL/dE_g): accumulates sum_g Ag2[g] w_g and its derivatives in mean
// and sd.
template <bool Backward, class Rem>
__device__ __forceinline__ void walk(const float* z, double u_age, float u1, float u1_lo, float inv_h, uint32_t steps,
                                     float stop, Rem r, bool fixed_tau, float* acc,
                                     const float* Ag2, float& f_r, float& f_mu, float& f_sig) {
  // step 1 (the first division, S_1 = tau_1 (1 + U)) is peeled off the loop. The device code
  // is compiled without automatic FMA contraction (the random stream must round as on the
  // host), so the derivative updates below name their FMAs.
  float zj = fixed_tau ? 0.0f : z[0];
  r.first(zj, u_age, u1, u1_lo);
  float dmu = u1 * inv_h, dsig = zj * dmu;    // dS_j / d(mean, sd), divided by h
  float P = 1.0f;                             // s_1 ... s_{j-1}
  float D_mu = 0.0f, D_sig = 0.0f;
  for (uint32_t j = 1;;) {
    const float x = r.x(inv_h);
    if (x <= kFar) {
      float s, one_m_s;
      sig_pair(x, s, one_m_s);
      const float w = P * one_m_s;  // leaf weight of generation j - 1
      if constexpr (!Backward) {
        // into the compensated pair at acc[2g] (sum) / acc[2g + 1] (compensation); the
        // generation's scale ratio / paths * 2^g is applied once per row at the end
        if (w != 0.0f) kahan_add(acc + 2u * (j - 1u) * kThreads, w);
      } else {
        const float a = Ag2[j - 1];
        if (a != 0.0f && w != 0.0f) {
          const float aw = a * w;
          f_r += aw;
          if (!fixed_tau) {
            f_mu = __fmaf_rn(aw, __fmaf_rn(s, dmu, D_mu), f_mu);
            f_sig = __fmaf_rn(aw, __fmaf_rn(s, dsig, D_sig), f_sig);
          }
        }
        if (!fixed_tau) {
          D_mu = __fmaf_rn(-one_m_s, dmu, D_mu);
          D_sig = __fmaf_rn(-one_m_s, dsig, D_sig);
        }
      }
      P *= s;
      if (P < stop) break;
    }
    if (++j > steps) break;
    zj = fixed_tau ? 0.0f : z[(j - 1) * 32u];
    r.step(zj);
    dmu += inv_h;
    dsig = __fmaf_rn(zj, inv_h, dsig);
  }
}

// One lineage for one type, forward mode: for every generation g it reaches, acc rows
// 3g, 3g + 1, 3g + 2 gain w_g and dw_g/d(mean, sd) (per-thread FP32 sums; the caller scales
// generation g's rows by 2^g).
template <class Rem>
__device__ __forceinline__ void walk_jacobian(const float* z, double u_age, float u1, float u1_lo, float inv_h,
                                              uint32_t steps, float stop, Rem r, bool fixed_tau, float* acc) {
  // step 1 peeled off the loop as in walk(), derivatives divided by h as there
  float zj = fixed_tau ? 0.0f : z[0];
  r.first(zj, u_age, u1, u1_lo);
  float dmu = u1 * inv_h, dsig = zj * dmu;
  float P = 1.0f, D_mu = 0.0f, D_sig = 0.0f;  // P = s_1 ... s_{j-1}
  for (uint32_t j = 1;;) {
    const float x = r.x(inv_h);
    if (x <= kFar) {  // as in walk()
      float s, one_m_s;
      sig_pair(x, s, one_m_s);
      const float w = P * one_m_s;  // leaf weight of generation j - 1
      float* p = acc + 3u * (j - 1u) * kThreads;
      if (w != 0.0f) {  // generation j - 1's scale 2^(j-1) is applied per row at the end
        p[0] += w;
        if (!fixed_tau) {
          p[kThreads] = __fmaf_rn(w, __fmaf_rn(s, dmu, D_mu), p[kThreads]);
          p[2 * kThreads] = __fmaf_rn(w, __fmaf_rn(s, dsig, D_sig), p[2 * kThreads]);
        }
      }
      if (!fixed_tau) {
        D_mu = __fmaf_rn(-one_m_s, dmu, D_mu);
        D_sig = __fmaf_rn(-one_m_s, dsig, D_sig);
      }
      P *= s;
      if (P < stop) break;
    }
    if (++j > steps) break;
    zj = fixed_tau ? 0.0f : z[(j - 1) * 32u];
    r.step(zj);
    dmu += inv_h;
    dsig = __fmaf_rn(zj, inv_h, dsig);
  }
}

// The FP64 walks (candidates and bins where the grid form's error bound does not hold), kept
// out of line so that the compiler cannot merge them into the FP32 walks as predicated code.
template <bool Backward>
__device__ __noinline__ float3 walk_fp64(const float* z, double u_age, float u1, float u1_lo, float inv_h,
                                         uint32_t steps, float stop, RemFp64 r, bool fixed_tau, float* acc,
                                         const float* Ag2) {
  float f_r = 0.0f, f_mu = 0.0f, f_sig = 0.0f;
  walk<Backward>(z, u_age, u1, u1_lo, inv_h, steps, stop, r, fixed_tau, acc, Ag2, f_r, f_mu, f_sig);
  return make_float3(f_r, f_mu, f_sig);
}

__device__ __noinline__ void walk_jacobian_fp64(const float* z, double u_age, float u1, float u1_lo, float inv_h,
                                                uint32_t steps, float stop, RemFp64 r, bool fixed_tau, float* acc) {
  walk_jacobian(z, u_age, u1, u1_lo, inv_h, steps, stop, r, fixed_tau, acc);
}

// Jacobian of the expected counts: block (bin, group of 32 candidates, type k). out[c][b][g][k]
// = (sum 2^g w_g / paths, ratio_k / paths * sum 2^g dw_g/dmean, the same for sd), i.e.
// d E_{b,g} / d(ratio_k, mean_k, sd_k); every block draws its bin's lineages itself (the
// draws are shared by the 32 candidates of a warp, not across types).
template <bool Kept>
__global__ void __launch_bounds__(kThreads, Kept ? kBlocksKeptJacobian : kBlocksDrawn) k_smooth_jacobian(const SmoothArgs A, const double* __restrict__ params,
                                                              uint32_t ncand, double* __restrict__ out) {
  // dynamic: per-thread sums [3 * rows][kThreads], then the lineage draws [kWarps][rows][32]
  extern __shared__ float facc[];
  __shared__ ZigTables Z;
  __shared__ double u_age[kThreads];
  __shared__ float u_one[kThreads], u_one_lo[kThreads];
  constexpr uint32_t kWarps = kThreads / 32;
  const uint32_t b = A.bin_order[blockIdx.x], k = blockIdx.z;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t slot = blockIdx.y * 32u + lane;
  const bool live = slot < ncand;
  const uint32_t c = live ? A.order[(uint64_t)k * ncand + slot] : 0u;
  const uint32_t KQ = A.ntypes * 3u;
  float* zbuf = facc + (size_t)3u * A.rows * kThreads + (size_t)warp * A.rows * 32u;
  for (uint32_t i = threadIdx.x; i < sizeof(ZigTables) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(&Z)[i] = __ldg(reinterpret_cast<const uint32_t*>(A.zig) + i);
  for (uint32_t i = 0; i < 3u * A.rows; ++i) facc[i * kThreads + threadIdx.x] = 0.0f;
  double ratio = 0.0, mu = 0.0, sd = 0.0;
  if (live) {
    ratio = params[(uint64_t)c * KQ + 3u * k];
    mu = params[(uint64_t)c * KQ + 3u * k + 1u];
    sd = params[(uint64_t)c * KQ + 3u * k + 2u];
  }
  const bool quiescent = neg_nonzero(mu), fixed_tau = zero_bits(mu);
  __syncthreads();
  const uint32_t steps = __ldg(A.bin_cap + b) + 1u;
  const uint64_t r0 = __ldg(A.bin_start + b), r1 = __ldg(A.bin_start + b + 1);
  float* fmy = facc + threadIdx.x;
  const float inv_h = (float)A.inv_h;
  RemGrid rg;
  const bool grid = opaque(grid_setup(rg, mu, sd, A.t_max, steps, 1.0 / A.inv_h));
  const RemFp64 rd{mu, sd, A.t_max, 0.0};
  const float stop = stop_level(steps);  // once per block: the walks' stopping threshold
  const uint64_t nlin = (r1 - r0) * A.paths;
  for (uint64_t base = (uint64_t)warp * 32u; base < nlin; base += 32u * kWarps) {
    if (base + lane < nlin)
      stage_lineage<Kept>(A, Z, r0, base + lane, steps, zbuf + lane, u_age + threadIdx.x, u_one + threadIdx.x,
                          u_one_lo + threadIdx.x);
    __syncwarp();
    const uint32_t n = (uint32_t)((nlin - base) < 32u ? (nlin - base) : 32u);
    if (live) {
      for (uint32_t ii = 0; ii < n; ++ii) {
        const uint32_t li = warp * 32u + ii;
        if (quiescent) {
          fmy[0] += 1.0f;  // quiescent type: a leaf at generation 0 (cell.cu:69-75)
        } else if (grid) {
          walk_jacobian(zbuf + ii, u_age[li], u_one[li], u_one_lo[li], inv_h, steps, stop, rg, fixed_tau, fmy);
        } else {
          walk_jacobian_fp64(zbuf + ii, u_age[li], u_one[li], u_one_lo[li], inv_h, steps, stop, rd, fixed_tau, fmy);
        }
      }
    }
    __syncwarp();
  }
  __syncthreads();
  // sums over the warps in warp order, generation g's rows scaled by 2^g; lane l of every
  // warp holds candidate 32 * group + l, so the warps split the rows
  if (!live) return;
  const double inv_paths = 1.0 / (double)A.paths;
  double* o = out + ((uint64_t)c * A.nbins + b) * A.rows * KQ + 3u * k;
  for (uint32_t q = warp; q < 3u * A.rows; q += kWarps) {
    double v = 0.0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; ++w) v += (double)facc[q * kThreads + w * 32u + lane];
    o[(q / 3u) * KQ + q % 3u] = ldexp(v * (q % 3u == 0u ? 1.0 : ratio) * inv_paths, (int)(q / 3u));
  }
}

// Forward (e_raw[c][k][b][g] = ratio_k / paths * sum 2^g w_g over the bin's lineages) and
// adjoint (part[c][b][3k + q] = d(sum_g A_g E_g)/d(ratio_k, mean_k, sd_k)) of one type: block
// (bin, group of 32 candidates, type k). Every block draws its bin's lineages itself.
template <bool Backward, bool Kept>
__global__ void __launch_bounds__(kThreads, Kept ? kBlocksKept : kBlocksDrawn) k_smooth(const SmoothArgs A, const double* __restrict__ params,
                                                     uint32_t ncand, const double* __restrict__ grad_expected,
                                                     uint32_t nvalues, const int32_t* __restrict__ vidx,
                                                     double* __restrict__ out) {
  // dynamic: compensated FP32 accumulator pairs [arows][kThreads] (forward: 2 per generation
  // row, backward: 2 per parameter), then the lineage draws z [kWarps][rows][32]
  extern __shared__ float facc[];
  __shared__ ZigTables Z;
  __shared__ float Ag2[Backward ? 32 : 1][kSmoothMaxRows];
  __shared__ double u_age[kThreads];
  __shared__ float u_one[kThreads], u_one_lo[kThreads];
  constexpr uint32_t kWarps = kThreads / 32;
  const uint32_t b = A.bin_order[blockIdx.x], k = blockIdx.z;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t slot = blockIdx.y * 32u + lane;
  const bool live = slot < ncand;
  const uint32_t c = live ? A.order[(uint64_t)k * ncand + slot] : 0u;
  const uint32_t KQ = A.ntypes * 3u;
  const uint32_t arows = Backward ? 6u : 2u * A.rows;
  float* zbuf = facc + (size_t)arows * kThreads + (size_t)warp * A.rows * 32u;
  for (uint32_t i = threadIdx.x; i < sizeof(ZigTables) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(&Z)[i] = __ldg(reinterpret_cast<const uint32_t*>(A.zig) + i);
  for (uint32_t i = 0; i < arows; ++i) facc[i * kThreads + threadIdx.x] = 0.0f;
  const uint32_t cap = __ldg(A.bin_cap + b);
  const uint32_t steps = cap + 1u;
  if constexpr (Backward) {
    for (uint32_t i = threadIdx.x; i < 32u * kSmoothMaxRows; i += blockDim.x) {
      const uint32_t l = i / kSmoothMaxRows, g = i % kSmoothMaxRows;
      const uint32_t sl = blockIdx.y * 32u + l;
      const uint32_t cc = sl < ncand ? A.order[(uint64_t)k * ncand + sl] : 0u;
      double a = 0.0;
      if (sl < ncand && g < A.rows && g <= cap) {
        const int32_t v = vidx[(uint64_t)b * A.rows + g];
        if (v >= 0) a = ldexp(grad_expected[(uint64_t)cc * nvalues + v], (int)g);
      }
      Ag2[l][g] = (float)a;
    }
  }
  const double* my_prm = params + (uint64_t)(live ? c : 0u) * KQ + 3u * k;
  const double mu = live ? my_prm[1] : 0.0, sd = live ? my_prm[2] : 0.0;
  // per-block flags from the parameters' bits (integer tests: nothing for the FP64 pipe to
  // redo inside the lineage loops)
  const bool quiescent = neg_nonzero(mu), fixed_tau = zero_bits(mu);
  // a type of ratio 0 adds nothing to the expected counts (its adjoint rows still count)
  const bool walks = Backward || (live && !zero_bits(my_prm[0]));
  __syncthreads();
  const uint64_t r0 = __ldg(A.bin_start + b), r1 = __ldg(A.bin_start + b + 1);
  float* fmy = facc + threadIdx.x;
  const float inv_h = (float)A.inv_h;
  const float* my_ag = Backward ? Ag2[lane] : nullptr;
  RemGrid rg;
  const bool grid = opaque(grid_setup(rg, mu, sd, A.t_max, steps, 1.0 / A.inv_h));
  const RemFp64 rd{mu, sd, A.t_max, 0.0};
  const float stop = stop_level(steps);  // once per block: the walks' stopping threshold
  // lineage i of the bin: initial cell r0 + i / paths, replica i % paths
  const uint64_t nlin = (r1 - r0) * A.paths;
  for (uint64_t base = (uint64_t)warp * 32u; base < nlin; base += 32u * kWarps) {
    // this lane stages lineage base + lane
    if (base + lane < nlin)
      stage_lineage<Kept>(A, Z, r0, base + lane, steps, zbuf + lane, u_age + threadIdx.x, u_one + threadIdx.x,
                          u_one_lo + threadIdx.x);
    __syncwarp();
    const uint32_t n = (uint32_t)((nlin - base) < 32u ? (nlin - base) : 32u);
    if (live) {
      float f_r = 0.0f, f_mu = 0.0f, f_sig = 0.0f;  // adjoint terms of these (up to) 32 lineages
      for (uint32_t ii = 0; ii < n; ++ii) {
        if (quiescent) {
          // quiescent type: a leaf at generation 0 (cell.cu:69-75)
          if constexpr (Backward) {
            f_r += my_ag[0];
          } else if (walks) {
            kahan_add(fmy, 1.0f);
          }
        } else if (walks) {
          const uint32_t li = warp * 32u + ii;
          if (grid)
            walk<Backward>(zbuf + ii, u_age[li], u_one[li], u_one_lo[li], inv_h, steps, stop, rg, fixed_tau, fmy,
                           my_ag, f_r, f_mu, f_sig);
          else {
            const float3 f = walk_fp64<Backward>(zbuf + ii, u_age[li], u_one[li], u_one_lo[li], inv_h, steps, stop,
                                                 rd, fixed_tau, fmy, my_ag);
            f_r += f.x;
            f_mu += f.y;
            f_sig += f.z;
          }
        }
      }
      if constexpr (Backward) {
        // per-thread compensated FP32 sums over the batches of 32 lineages (terms of either
        // sign cancel); scaled by ratio / paths once, at the end
        kahan_add(fmy, f_r);
        kahan_add(fmy + 2 * kThreads, f_mu);
        kahan_add(fmy + 4 * kThreads, f_sig);
      }
    }
    __syncwarp();
  }
  __syncthreads();
  // sums over the warps in warp order (forward row g scaled by ratio / paths * 2^g, adjoint
  // rows by 1 / paths, and those of mean and sd by the ratio); lane l of every warp holds
  // candidate 32 * group + l, so the warps split the rows
  if (!live) return;
  const double inv_paths = 1.0 / (double)A.paths, ratio = my_prm[0];
  const uint32_t nrows = Backward ? 3u : A.rows;
  double* o = Backward ? out + ((uint64_t)c * A.nbins + b) * KQ + 3u * k
                       : out + (((uint64_t)c * A.ntypes + k) * A.nbins + b) * A.rows;
  for (uint32_t q = warp; q < nrows; q += kWarps) {
    double v = 0.0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; ++w)
      v += (double)facc[2 * q * kThreads + w * 32u + lane] - (double)facc[(2 * q + 1) * kThreads + w * 32u + lane];
    if constexpr (Backward)
      v *= (q == 0u ? 1.0 : ratio) * inv_paths;
    else
      v *= ldexp(ratio * inv_paths, (int)q);
    o[q] = v;
  }
}

// Every lineage's draws (normals of its path, initial age), which depend on the seed and the
// bins but not on the parameters: block b takes bin b's lineages.
__global__ void __launch_bounds__(256) k_smooth_draws(const SmoothArgs A, float* __restrict__ lin_z,
                                                      LineageU* __restrict__ lin_u) {
  __shared__ ZigTables Z;
  for (uint32_t i = threadIdx.x; i < sizeof(ZigTables) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t*>(&Z)[i] = __ldg(reinterpret_cast<const uint32_t*>(A.zig) + i);
  __syncthreads();
  const uint32_t b = blockIdx.x;
  const uint64_t r0 = __ldg(A.bin_start + b), r1 = __ldg(A.bin_start + b + 1);
  const uint32_t steps = __ldg(A.bin_cap + b) + 1u;
  const uint64_t nlin = (r1 - r0) * A.paths;
  for (uint64_t i = threadIdx.x; i < nlin; i += blockDim.x) {
    const uint64_t L = r0 * A.paths + i;
    double u;
    draw_lineage(A, Z, r0, i, steps, lin_z + L * A.zrow, 1u, u);
    lin_u[L] = lineage_u(u);
  }
}

// A double's bits as an unsigned key in the IEEE total order (NaNs at the ends).
__device__ __forceinline__ uint64_t order_key(double x) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | (1ull << 63));
}

// order[k][rank] = candidate: the candidates sorted by type k's mean (ties by index), so the
// 32 lanes of a warp walk lineages of similar length. Rank by counting, through shared-memory
// tiles of the keys; a permutation for any input. Above kOrderMax candidates: the identity.
constexpr uint32_t kOrderMax = 8192;
__global__ void __launch_bounds__(256) k_smooth_order(const double* __restrict__ params, uint32_t ncand,
                                                      uint32_t ntypes, uint32_t* __restrict__ order) {
  __shared__ uint64_t tile[256];
  const uint32_t k = blockIdx.y;
  const uint32_t c = blockIdx.x * 256u + threadIdx.x;
  const uint32_t kq = ntypes * 3u;
  if (ncand > kOrderMax) {
    if (c < ncand) order[(uint64_t)k * ncand + c] = c;
    return;
  }
  const uint64_t key = c < ncand ? order_key(params[(uint64_t)c * kq + 3u * k + 1u]) : 0ull;
  uint32_t rank = 0;
  for (uint32_t t0 = 0; t0 < ncand; t0 += 256u) {
    const uint32_t d = t0 + threadIdx.x;
    tile[threadIdx.x] = d < ncand ? order_key(params[(uint64_t)d * kq + 3u * k + 1u]) : ~0ull;
    __syncthreads();
    const uint32_t m = ncand - t0 < 256u ? ncand - t0 : 256u;
    for (uint32_t j = 0; j < m; ++j) {
      const uint64_t kd = tile[j];
      rank += (kd < key || (kd == key && t0 + j < c)) ? 1u : 0u;
    }
    __syncthreads();
  }
  if (c < ncand) order[(uint64_t)k * ncand + rank] = c;
}

int launch_order(const SmoothArgs& A, const double* params, uint32_t ncand, cudaStream_t st) {
  const dim3 grid((ncand + 255u) / 256u, A.ntypes);
  k_smooth_order<<<grid, 256, 0, st>>>(params, ncand, A.ntypes, A.order);
  return (int)cudaGetLastError();
}

// expected[c][v] = sum over types k and the (b, g) of value v of e_raw[c][k][b][g]
// (per_type = nbins * rows).
__global__ void k_smooth_merge(const double* __restrict__ e_raw, uint32_t ncand, uint32_t ntypes, uint32_t per_type,
                               const uint32_t* __restrict__ inv_off, const uint32_t* __restrict__ inv_idx,
                               uint32_t nvalues, double* __restrict__ expected) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)ncand * nvalues) return;
  const uint32_t c = (uint32_t)(i / nvalues), v = (uint32_t)(i % nvalues);
  double s = 0.0;
  for (uint32_t k = 0; k < ntypes; ++k) {
    const double* src = e_raw + ((uint64_t)c * ntypes + k) * per_type;
    for (uint32_t q = inv_off[v]; q < inv_off[v + 1]; ++q) s += src[inv_idx[q]];
  }
  expected[i] = s;
}

// expected[c][v] = sum_k ratio_k U, jacobian[c][v][k][q] = sum of jac_raw[c][b][g][k][q]
// over the (b, g) of value v (U = the q = 0 entry, d/d ratio_k).
__global__ void k_smooth_jacobian_merge(const double* __restrict__ jac_raw, const double* __restrict__ params,
                                        uint32_t ncand, uint32_t per_cand, uint32_t kq,
                                        const uint32_t* __restrict__ inv_off, const uint32_t* __restrict__ inv_idx,
                                        uint32_t nvalues, double* __restrict__ expected, double* __restrict__ jac) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)ncand * nvalues) return;
  const uint32_t c = (uint32_t)(i / nvalues), v = (uint32_t)(i % nvalues);
  const double* src = jac_raw + (uint64_t)c * per_cand * kq;
  double e = 0.0;
  for (uint32_t q = 0; q < kq; ++q) {
    double s = 0.0;
    for (uint32_t t = inv_off[v]; t < inv_off[v + 1]; ++t) s += src[(uint64_t)inv_idx[t] * kq + q];
    jac[i * kq + q] = s;
    if (q % 3u == 0u) e += params[(uint64_t)c * kq + q] * s;
  }
  expected[i] = e;
}

// The Gauss-Newton system of the squared log-count loss, one block per candidate c: with
// r_v = log1p(E_v) - log1p(T_v) and j_v = (dE_v / dparams) / (1 + E_v),
//   loss[c] = sum_v r_v^2, jtj[c][p][q] = sum_v j_vp j_vq, jtr[c][p] = sum_v j_vp r_v.
// E and dE come from the Jacobian pass's raw rows as in k_smooth_jacobian_merge (same order
// of additions). Values go through shared memory in tiles; each thread keeps the running sums
// of up to kGnSlots outputs (upper triangle of jtj, jtr, loss) in a fixed order.
constexpr uint32_t kGnTile = 128;
constexpr int kGnSlots = 3;
static_assert(kSmoothMaxTypes * 3 * (kSmoothMaxTypes * 3 + 1) / 2 + kSmoothMaxTypes * 3 + 1 <= kGnSlots * kGnTile,
              "outputs per candidate exceed the block's slots");

__device__ __forceinline__ void gn_pair(uint32_t o, uint32_t kq, uint32_t& a, uint32_t& b) {
  const uint32_t npair = kq * (kq + 1u) / 2u;
  if (o < npair) {
    a = 0;
    while (o >= kq - a) {
      o -= kq - a;
      ++a;
    }
    b = a + o;
  } else if (o < npair + kq) {
    a = o - npair;
    b = kq;  // the residual column
  } else {
    a = kq;
    b = kq;
  }
}

__global__ void __launch_bounds__(kGnTile) k_smooth_gauss_newton(
    const double* __restrict__ jac_raw, const double* __restrict__ params, uint32_t per_cand, uint32_t kq,
    const uint32_t* __restrict__ inv_off, const uint32_t* __restrict__ inv_idx, uint32_t nvalues,
    const double* __restrict__ target, double* __restrict__ loss, double* __restrict__ jtj,
    double* __restrict__ jtr) {
  extern __shared__ double gsm[];  // [kGnTile][kq + 1]: scaled Jacobian row, then r
  const uint32_t c = blockIdx.x;
  const uint32_t w = kq + 1u;
  const uint32_t nout = kq * (kq + 1u) / 2u + kq + 1u;
  const double* src = jac_raw + (uint64_t)c * per_cand * kq;
  const double* prm = params + (uint64_t)c * kq;
  double acc[kGnSlots];
#pragma unroll
  for (int sl = 0; sl < kGnSlots; ++sl) acc[sl] = 0.0;
  for (uint32_t v0 = 0; v0 < nvalues; v0 += kGnTile) {
    const uint32_t v = v0 + threadIdx.x;
    double* row = gsm + (size_t)threadIdx.x * w;
    if (v < nvalues) {
      double e = 0.0;
      for (uint32_t q = 0; q < kq; ++q) {
        double sum = 0.0;
        for (uint32_t t = inv_off[v]; t < inv_off[v + 1]; ++t) sum += src[(uint64_t)inv_idx[t] * kq + q];
        row[q] = sum;
        if (q % 3u == 0u) e += prm[q] * sum;
      }
      const double inv = 1.0 / (1.0 + e);
      for (uint32_t q = 0; q < kq; ++q) row[q] *= inv;
      row[kq] = log1p(e) - log1p(target[v]);
    } else {
      for (uint32_t q = 0; q <= kq; ++q) row[q] = 0.0;
    }
    __syncthreads();
    const uint32_t m = nvalues - v0 < kGnTile ? nvalues - v0 : kGnTile;
#pragma unroll
    for (int sl = 0; sl < kGnSlots; ++sl) {
      const uint32_t o = threadIdx.x + (uint32_t)sl * kGnTile;
      if (o < nout) {
        uint32_t a, b;
        gn_pair(o, kq, a, b);
        double sum = acc[sl];
        for (uint32_t t = 0; t < m; ++t) sum = fma(gsm[t * w + a], gsm[t * w + b], sum);
        acc[sl] = sum;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int sl = 0; sl < kGnSlots; ++sl) {
    const uint32_t o = threadIdx.x + (uint32_t)sl * kGnTile;
    if (o >= nout) continue;
    uint32_t a, b;
    gn_pair(o, kq, a, b);
    if (b < kq) {
      jtj[((uint64_t)c * kq + a) * kq + b] = acc[sl];
      jtj[((uint64_t)c * kq + b) * kq + a] = acc[sl];
    } else if (a < kq) {
      jtr[(uint64_t)c * kq + a] = acc[sl];
    } else {
      loss[c] = acc[sl];
    }
  }
}

__global__ void k_smooth_grad_sum(const double* __restrict__ part, uint32_t ncand, uint32_t nbins, uint32_t per_bin,
                                  double* __restrict__ grad) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)ncand * per_bin) return;
  const uint32_t c = (uint32_t)(i / per_bin), q = (uint32_t)(i % per_bin);
  double s = 0.0;
  for (uint32_t b = 0; b < nbins; ++b) s += part[((uint64_t)c * nbins + b) * per_bin + q];
  grad[i] = s;
}

// accumulator pairs (2 floats per output row and thread) + the lineage draws (kThreads
// floats per generation row)
int smem_bytes(uint32_t out_rows, uint32_t rows) {
  return (int)((2u * out_rows + rows) * kThreads * sizeof(float));
}

template <bool Backward, bool Kept>
int launch_smooth_k(const SmoothArgs& A, const double* params, uint32_t ncand, const double* grad_expected,
                    uint32_t nvalues, const int32_t* vidx, double* out, cudaStream_t st) {
  const int smem = smem_bytes(Backward ? 3u : A.rows, A.rows);
  // static shared memory plus `smem` may exceed the default 48 KB: always opt in
  const cudaError_t e =
      cudaFuncSetAttribute(k_smooth<Backward, Kept>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  const int eo = launch_order(A, params, ncand, st);
  if (eo != 0) return eo;
  const dim3 grid(A.nbins, (ncand + 31u) / 32u, A.ntypes);
  k_smooth<Backward, Kept><<<grid, kThreads, smem, st>>>(A, params, ncand, grad_expected, nvalues, vidx, out);
  return (int)cudaGetLastError();
}

template <bool Backward>
int launch_smooth_t(const SmoothArgs& A, const double* params, uint32_t ncand, const double* grad_expected,
                    uint32_t nvalues, const int32_t* vidx, double* out, cudaStream_t st) {
  return A.lin_z ? launch_smooth_k<Backward, true>(A, params, ncand, grad_expected, nvalues, vidx, out, st)
                 : launch_smooth_k<Backward, false>(A, params, ncand, grad_expected, nvalues, vidx, out, st);
}

// The Jacobian kernel of a plan that keeps its lineage draws or not.
int launch_jacobian_k(const SmoothArgs& A, const double* params, uint32_t ncand, double* jac_raw, cudaStream_t st) {
  const int smem = (int)(4u * A.rows * kThreads * sizeof(float));
  auto* k = A.lin_z ? k_smooth_jacobian<true> : k_smooth_jacobian<false>;
  const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return (int)e;
  const int eo = launch_order(A, params, ncand, st);
  if (eo != 0) return eo;
  const dim3 grid(A.nbins, (ncand + 31u) / 32u, A.ntypes);
  k<<<grid, kThreads, smem, st>>>(A, params, ncand, jac_raw);
  return (int)cudaGetLastError();
}

}  // namespace

int launch_smooth_draws(const SmoothArgs& A, float* lin_z, LineageU* lin_u, void* stream) {
  if (A.nbins == 0) return 0;
  k_smooth_draws<<<A.nbins, 256, 0, (cudaStream_t)stream>>>(A, lin_z, lin_u);
  return (int)cudaGetLastError();
}

int launch_smooth_forward(const SmoothArgs& A, const double* params, uint32_t ncand, double* e_raw, void* stream) {
  if (ncand == 0 || A.nbins == 0) return 0;
  return launch_smooth_t<false>(A, params, ncand, nullptr, 0, nullptr, e_raw, (cudaStream_t)stream);
}

int launch_smooth_merge(const double* e_raw, uint32_t ncand, uint32_t ntypes, uint32_t per_type,
                        const uint32_t* inv_off, const uint32_t* inv_idx, uint32_t nvalues, double* expected,
                        void* stream) {
  const uint64_t n = (uint64_t)ncand * nvalues;
  if (n == 0) return 0;
  k_smooth_merge<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(e_raw, ncand, ntypes, per_type,
                                                                              inv_off, inv_idx, nvalues, expected);
  return (int)cudaGetLastError();
}

int launch_smooth_jacobian(const SmoothArgs& A, const double* params, uint32_t ncand, const uint32_t* inv_off,
                           const uint32_t* inv_idx, uint32_t nvalues, double* jac_raw, double* expected,
                           double* jacobian, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t kq = A.ntypes * 3u;
  const uint64_t n = (uint64_t)ncand * nvalues;
  if (n == 0) return 0;
  if (A.nbins == 0) {
    cudaError_t e = cudaMemsetAsync(expected, 0, n * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(jacobian, 0, n * kq * sizeof(double), st);
    return (int)e;
  }
  const int ej = launch_jacobian_k(A, params, ncand, jac_raw, st);
  if (ej != 0) return ej;
  k_smooth_jacobian_merge<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(jac_raw, params, ncand, A.nbins * A.rows, kq,
                                                                      inv_off, inv_idx, nvalues, expected, jacobian);
  return (int)cudaGetLastError();
}

int launch_smooth_gauss_newton(const SmoothArgs& A, const double* params, uint32_t ncand, const uint32_t* inv_off,
                               const uint32_t* inv_idx, uint32_t nvalues, const double* target, double* jac_raw,
                               double* loss, double* jtj, double* jtr, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t kq = A.ntypes * 3u;
  if (ncand == 0) return 0;
  if (A.nbins == 0 || nvalues == 0) {
    cudaError_t e = cudaMemsetAsync(loss, 0, (size_t)ncand * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(jtj, 0, (size_t)ncand * kq * kq * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(jtr, 0, (size_t)ncand * kq * sizeof(double), st);
    return (int)e;
  }
  const int ej = launch_jacobian_k(A, params, ncand, jac_raw, st);
  if (ej != 0) return ej;
  k_smooth_gauss_newton<<<ncand, kGnTile, kGnTile * (kq + 1u) * sizeof(double), st>>>(
      jac_raw, params, A.nbins * A.rows, kq, inv_off, inv_idx, nvalues, target, loss, jtj, jtr);
  return (int)cudaGetLastError();
}

int launch_smooth_backward(const SmoothArgs& A, const double* params, uint32_t ncand, const double* grad_expected,
                           uint32_t nvalues, const int32_t* vidx, double* grad_part, double* grad_params,
                           void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t per_bin = A.ntypes * 3u;
  const uint64_t n = (uint64_t)ncand * per_bin;
  if (n == 0) return 0;
  if (A.nbins == 0) return (int)cudaMemsetAsync(grad_params, 0, n * sizeof(double), st);
  int e = launch_smooth_t<true>(A, params, ncand, grad_expected, nvalues, vidx, grad_part, st);
  if (e != 0) return e;
  k_smooth_grad_sum<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(grad_part, ncand, A.nbins, per_bin, grad_params);
  return (int)cudaGetLastError();
}

}  // namespace pc
