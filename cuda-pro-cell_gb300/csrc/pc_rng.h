// Counter-based random numbers for the proliferation path, shared verbatim by the
// host planner and the sm_103a kernels so that both evaluate the same stream.
//
// The reference draws every random number from a freshly initialised curand XORWOW
// state (src/utils/util.cu:143-169) seeded with ad-hoc arithmetic on time(NULL), the
// cell id and the parent's timer (src/simulation/cells_population.cu:108,
// src/simulation/proliferation.cu:330-331). That stream is neither reproducible nor
// independent between draws. This engine replaces it with Philox4x32-10 keyed by the
// run seed and addressed by (heap index of the tree node, root index, purpose):
//
//   counter = { node_lo, node_hi, root, purpose | index },  key = { seed_lo, seed_hi }
//
// * PURPOSE_ROOT  node 0, index 0: the root's type uniform (words x,y) and its
//                 initial-age uniform U (words z,w); see cell.cu:81-104 and :124-143.
// * PURPOSE_PAIR  node n: the first-attempt normal draws of both children 2n and 2n+1.
//                 Child c takes word c (x or y) as its sign and 31-bit magnitude, bits
//                 10c..10c+9 of word z as its ziggurat layer, and a 22-bit wedge uniform:
//                 child 0 the low 22 bits of w, child 1 the top 10 bits of w above the top
//                 12 bits of z. The root is child 1 of node 0.
// * PURPOSE_CHILD node m, index i: the i-th block of the child's private stream, used
//                 only when the first attempt is rejected (ziggurat tail, wedge
//                 rejection, or the truncation tau <= 0 of cell.cu:114-118).
//
// The normal variate is a 1024-layer ziggurat (Marsaglia & Tsang, "The Ziggurat Method
// for Generating Random Variables", J. Stat. Softw. 5(8), 2000) evaluated in FP32 with
// independent layer bits (Doornik, "An Improved Ziggurat Method to Generate Normal
// Random Samples", 2005); the first attempt of a daughter needs no Philox block beyond
// the pair block unless it falls in the tail or its wedge test rejects (about 0.2% of
// draws; 99.57% pass the strip test alone, against 98.5% with 256 layers: every draw that
// fails the strip test costs a division sweep a slow path, so 1024 layers were measured
// 8% faster on the 1e7-cell workload). Its rare wedge/tail steps need exp and log; both are written
// below from textbook range reduction plus polynomial/series evaluation with only
// IEEE-754 add, multiply and divide, so host and device produce identical bits.
// Device code must be compiled with --fmad=false and host code with
// -ffp-contract=off; the helpers also use explicit round-to-nearest intrinsics.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PC_HD __host__ __device__ __forceinline__
#define PC_HDM __host__ __device__ __forceinline__
#else
#define PC_HD static inline
#define PC_HDM inline
#endif

namespace pc {

struct u32x4 {
  uint32_t x, y, z, w;
};

// Philox4x32 constants (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy
// as 1, 2, 3", SC'11, Table 2 and Section 4.2).
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

constexpr uint32_t kPurposeRoot = 0x30000000u;
constexpr uint32_t kPurposePair = 0x10000000u;
constexpr uint32_t kPurposeChild = 0x20000000u;
constexpr uint32_t kPurposePath = 0x40000000u;  // smoothed form: lineage path choices

// One 32x32 -> 64-bit product (a single wide multiply on the GPU, which issues once where
// separate low and high halves would issue twice).
PC_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
}

// Ten Philox rounds; the key is bumped by the Weyl constants between rounds.
PC_HD u32x4 philox(u32x4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = 0; i < 10; ++i) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(kPhiloxM0, c.x, hi0, lo0);
    mulhilo32(kPhiloxM1, c.z, hi1, lo1);
    const u32x4 n = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    c = n;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}

// Philox with a precomputed key schedule ks[2i], ks[2i+1] = key + i * (W0, W1): the same
// function as philox(); in a kernel whose parameters hold `ks`, every key word becomes an
// immediate constant-bank operand of the XORs.
PC_HD u32x4 philox_ks(u32x4 c, const uint32_t* ks) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int i = 0; i < 10; ++i) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(kPhiloxM0, c.x, hi0, lo0);
    mulhilo32(kPhiloxM1, c.z, hi1, lo1);
    const u32x4 n = {hi1 ^ c.y ^ ks[2 * i], lo1, hi0 ^ c.w ^ ks[2 * i + 1], lo0};
    c = n;
  }
  return c;
}

PC_HD void philox_key_schedule(uint32_t k0, uint32_t k1, uint32_t* ks) {
  for (int i = 0; i < 10; ++i) {
    ks[2 * i] = k0;
    ks[2 * i + 1] = k1;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
}

// ---- IEEE round-to-nearest FP32 helpers (no contraction on either side) -------------
PC_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
PC_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
PC_HD float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
PC_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
PC_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  union {
    float f;
    uint32_t u;
  } v;
  v.f = f;
  return v.u;
#endif
}
PC_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  union {
    float f;
    uint32_t u;
  } v;
  v.u = u;
  return v.f;
#endif
}

// Uniforms from one 32-bit word (24 significant bits, exact in FP32).
PC_HD float unit_open_closed(uint32_t w) {  // (0, 1]
  return fmul((float)((w >> 8) + 1u), 5.9604644775390625e-8f);
}
PC_HD float unit_closed_open(uint32_t w) {  // [0, 1)
  return fmul((float)(w >> 8), 5.9604644775390625e-8f);
}
// Uniforms with 53 significant bits from two words (exact in FP64).
PC_HD double unit53_closed_open(uint32_t hi, uint32_t lo) {  // [0, 1)
  const uint64_t m = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
  return (double)m * 1.1102230246251565e-16;
}
PC_HD double unit53_open_closed(uint32_t hi, uint32_t lo) {  // (0, 1]
  const uint64_t m = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
  return (double)(m + 1u) * 1.1102230246251565e-16;
}

// exp(x) for x in [-64, 0]: Cody-Waite reduction x = n*ln2 + r, |r| <= ln2/2, then the
// degree-7 Taylor polynomial of exp(r) in Horner form and an exact scaling by 2^n.
PC_HD float zig_expf(float x) {
  const float kLog2e = 1.44269502162933349609375f;
  const float kLn2Hi = 0.693145751953125f;         // 15 significant bits: n*hi is exact
  const float kLn2Lo = 1.4286068203094172e-06f;  // ln2 - hi, rounded to FP32
  float n = fadd(fmul(x, kLog2e), 0.5f);
#if defined(__CUDA_ARCH__)
  n = floorf(n);
#else
  n = __builtin_floorf(n);
#endif
  const float r = fsub(fsub(x, fmul(n, kLn2Hi)), fmul(n, kLn2Lo));
  float p = 1.984126984126984e-4f;  // 1/5040
  p = fadd(fmul(p, r), 1.388888888888889e-3f);  // 1/720
  p = fadd(fmul(p, r), 8.333333333333333e-3f);  // 1/120
  p = fadd(fmul(p, r), 4.166666666666667e-2f);  // 1/24
  p = fadd(fmul(p, r), 1.666666666666667e-1f);  // 1/6
  p = fadd(fmul(p, r), 0.5f);
  p = fadd(fmul(p, r), 1.0f);
  p = fadd(fmul(p, r), 1.0f);
  const int e = (int)n + 127;
  if (e <= 0) return 0.0f;
  return fmul(p, u2f((uint32_t)e << 23));
}

// log(u) for u in (0, 1] (a normal FP32 number): u = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// log(m) = 2*atanh(s), s = (m-1)/(m+1), |s| <= 0.1716, series to s^9.
PC_HD float zig_logf(float u) {
  uint32_t b = f2u(u);
  int e = (int)((b >> 23) & 0xFFu) - 127;
  float m = u2f((b & 0x007FFFFFu) | 0x3F800000u);  // [1, 2)
  if (m > 1.41421353816986083984375f) {
    m = fmul(m, 0.5f);
    e += 1;
  }
  const float s = fdiv(fsub(m, 1.0f), fadd(m, 1.0f));
  const float s2 = fmul(s, s);
  float p = 0.2222222222222222f;                // 2/9
  p = fadd(fmul(p, s2), 0.2857142857142857f);   // 2/7
  p = fadd(fmul(p, s2), 0.4f);                  // 2/5
  p = fadd(fmul(p, s2), 0.6666666666666666f);   // 2/3
  p = fadd(fmul(p, s2), 2.0f);
  const float lm = fmul(p, s);
  const float fe = (float)e;
  return fadd(fmul(fe, 0.693145751953125f), fadd(fmul(fe, 1.4286068203094172e-06f), lm));
}

// Ziggurat tables. Layer 0 is the base strip (the rectangle [0,r] x [0,f(r)] plus the
// tail beyond r); layer i = 1..1023 is the rectangle [0, x_i] x [f(x_i), f(x_{i+1})] with
// x_1 = r > x_2 > ... > x_1023 and x_1024 = 0. A 31-bit magnitude `mag` in layer i maps to
// x = mag * w[i]; it lies under the curve without further tests iff mag < k[i].
// r solves the construction's closure condition (the top layer has area v) and
// v = r f(r) + integral_r^inf f; both were computed by bisection in 40-digit arithmetic
// (the same computation gives the published 256-layer constants r = 3.6541528853610088,
// v = 4.9286732339746553e-3).
constexpr int kZigLayers = 1024;
constexpr uint32_t kZigLayerMask = kZigLayers - 1;
constexpr double kZigR = 4.0388498461095045227;
constexpr double kZigV = 1.2263246463530880729e-3;  // area of each layer
constexpr float kZigRf = (float)kZigR;

struct ZigTables {
  uint32_t k[kZigLayers];
  float w[kZigLayers];
  float f[kZigLayers + 1];  // f[i] = exp(-x_i^2/2) for i >= 1, f[kZigLayers] = 1, f[0] unused
};

// The first-attempt layer of child c from its pair block (10 bits, see above).
PC_HD uint32_t pair_layer(const u32x4& P, uint32_t c) { return (P.z >> (10u * c)) & kZigLayerMask; }

// The first-attempt wedge uniform of child c from its pair block (22 bits in the top of the
// word, see above).
PC_HD uint32_t pair_wedge_bits(const u32x4& P, uint32_t c) {
  return c == 0u ? (P.w << 10) : (((P.w >> 22) << 22) | ((P.z >> 20) << 10));
}

// A node's private block stream (PURPOSE_CHILD), consumed four words at a time.
struct ChildStream {
  uint32_t c0, c1, root, k0, k1, next_block;
  u32x4 buf;
  uint32_t avail;
  PC_HDM uint32_t next() {
    if (avail == 0u) {
      buf = philox(u32x4{c0, c1, root, kPurposeChild | next_block}, k0, k1);
      ++next_block;
      avail = 4u;
    }
    const uint32_t i = 4u - avail;
    --avail;
    return i == 0u ? buf.x : (i == 1u ? buf.y : (i == 2u ? buf.z : buf.w));
  }
};

PC_HD ChildStream child_stream(uint64_t node, uint32_t root, uint32_t k0, uint32_t k1) {
  ChildStream s;
  s.c0 = (uint32_t)node;
  s.c1 = (uint32_t)(node >> 32);
  s.root = root;
  s.k0 = k0;
  s.k1 = k1;
  s.next_block = 0u;
  s.buf = u32x4{0u, 0u, 0u, 0u};
  s.avail = 0u;
  return s;
}

// One standard normal variate. (j, layer) is the first attempt; when `have_wedge` is set,
// `wedge` holds the first attempt's wedge uniform in its top 24 bits. Every further word
// comes from the node's private stream in a fixed order: tail -> (u1, u2) repeated until
// accepted; restart -> (j, layer word); wedge of any other attempt -> u. `budget` bounds
// the total number of rejection rounds (each succeeds with probability > 0.9); when it
// runs out the function returns 0 with budget == 0 so that the caller can report an
// error instead of spinning.
template <class Tables>
PC_HD float zig_normal(uint32_t j, uint32_t layer, bool have_wedge, uint32_t wedge,
                       ChildStream& cs, const Tables& T, uint32_t& budget) {
  bool first = have_wedge;
  for (; budget > 0u; --budget) {
    const uint32_t mag = j & 0x7FFFFFFFu;
    const bool neg = (j >> 31) != 0u;
    if (mag < T.k[layer]) {
      const float x = fmul((float)mag, T.w[layer]);
      return neg ? -x : x;
    }
    if (layer == 0u) {
      float a = 0.0f;
      for (;; --budget) {
        if (budget == 0u) return 0.0f;
        const float u1 = unit_open_closed(cs.next());
        const float u2 = unit_open_closed(cs.next());
        a = fdiv(-zig_logf(u1), kZigRf);
        const float b = -zig_logf(u2);
        if (fadd(b, b) > fmul(a, a)) break;
      }
      const float x = fadd(kZigRf, a);
      return neg ? -x : x;
    }
    const float x = fmul((float)mag, T.w[layer]);
    const float u = unit_closed_open(first ? wedge : cs.next());
    const float y = fadd(T.f[layer], fmul(u, fsub(T.f[layer + 1], T.f[layer])));
    if (y < zig_expf(fmul(-0.5f, fmul(x, x)))) return neg ? -x : x;
    first = false;
    j = cs.next();
    layer = cs.next() & kZigLayerMask;
  }
  return 0.0f;
}

}  // namespace pc
