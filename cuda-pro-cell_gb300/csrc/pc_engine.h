// Internal interface between the host driver (pc_api.cpp) and the sm_103a kernels
// (pc_sweeps.cuh, instantiated in pc_kernels.cu and pc_tuned_*.cu). Not part of the
// public ABI.
//
// Data layout in HBM
// ------------------
// * A live cell is 16 bytes: {double due; uint64 key}. `due` is the time at which the
//   cell is due to divide (the reference's t + timer, proliferation.cu:404-410). The key
//   names the tree node: its root (chunk-local index) and its heap index
//   node = 2^g + path for a cell of generation g, path being its g left/right choices
//   from the root (the Philox node address). Two layouts:
//     narrow (gmax <= 31, so that every key, a stored cell's or a parked daughter's one
//            generation below the deepest stored one, has g <= 31):
//            key = root_local << 32 | node, so the daughters' keys are key + node + c
//            with no carry out of the node's 32 bits;
//     wide   (deeper trees):                   key = root_local * 2^g + path, with
//            root bits + g <= 64 for every g up to gmax (chunk and g_store_max sized so).
//   Fluorescence is never stored: it is the bin value halved g times.
// * A level buffer holds the cells of one generation that will divide. It is split into
//   one segment per warp of the kernel that produced it; segment s holds count[s]
//   cells at cells + s * stride, and prefix[] (nseg + 1 entries, exclusive) is written
//   by the producer's last block. Concatenated in segment order the cells are sorted by
//   key, so every level is sorted by (root, path).
// * bin_info[b] = phi cap (bits 0-7: a cell of generation g in bin b may divide iff
//   g < cap) | countable at generation 0 (bit 8: value >= phi) | cap clamped by the key
//   layout (bit 9).
// * root_rec[r] (uint64, one per initial cell of the chunk, written by the root sweep):
//   bits 0-31 histogram class, bits 32-47 type index (sorted order; in the batched form the
//   index into the concatenated type table), bits 48-55 the bin's phi cap, bit 56
//   countable at generation 0, bit 57 cap clamped. One load gives the division sweep
//   everything it needs about a cell's root.
// * hist[g * nclass + class] counts the leaves of generation g per class. Plain form:
//   class = bin * ntypes + type. Batched form: class = bin_class[bin] + the type's index
//   within its instance, bins being the concatenated nonzero bins of all instances.
#pragma once

#include <stdint.h>

#include "pc_rng.h"

struct pc_bin;  // include/procell.h

namespace pc {

constexpr int kMaxTypes = 64;
constexpr int kBlock = 256;
constexpr int kWarpsPerBlock = kBlock / 32;

enum TypeMode : int32_t { kModeNormal = 0, kModeQuiescent = 1, kModeZeroMean = 2 };

// The sweeps keep each type's sd scaled by 2^kSigmaShift and widen a float normal z to the
// double z x 2^-kSigmaShift by moving its bits (exact, no rebias: widen_scaled in
// pc_sweeps.cuh); the FMA's product is exact, so the timer is fma(sd, z, mean) bit for bit.
// |sd| < kMaxSigma keeps the scaled sd finite.
constexpr int kSigmaShift = 896;

// Deepest phi cap (gmax) the narrow key layout serves.
constexpr uint32_t kNarrowMaxGen = 31;
constexpr double kMaxSigma = 0x1p127;

// One cell type, in the descending-ratio order the reference samples in.
// The division sweep reads bytes 0-31 (mu, sigma, zlo, zhi, t_max) as two 16-byte loads.
struct alignas(16) TypeDev {
  double mu, sigma;  // 0, 8: mean, sd x 2^kSigmaShift (tau = fma(sd, z, mean))
  float zlo, zhi;    // 16: the FP32 z range for which fma(sigma, z, mu) > 0 (the truncation)
  double t_max;      // 24: its instance's t_max (read by the batched sweeps; plain: RunArgs)
  double cum;        // 32: cumulative ratio in this order
  int32_t mode;      // 40
  int32_t pad;
};

// Batched form: the parameters of one type together with its instance's (one table
// entry per type of every instance, in instance order).
// The division sweep reads bytes 0-31 (type, t_max) and 48-63 (seed, first cell) as three
// 16-byte loads.
struct alignas(16) BatchType {
  TypeDev t;            // bytes 0-47
  uint32_t k0, k1;      // 48: the instance's seed
  uint64_t root_begin;  // 56: the instance's first initial cell in the batch
  uint32_t instance;    // 64
  uint32_t pad[3];
};
static_assert(sizeof(TypeDev) == 48 && sizeof(BatchType) == 80, "layout read by the division sweep");

struct InstanceDev {
  uint32_t type_begin, ntypes, fallback, pad;
  uint32_t k0, k1;
  uint64_t root_begin;
  double t_max;
};

struct RunArgs {
  uint32_t k0, k1;           // seed
  uint32_t ks[20];           // Philox key schedule of the seed
  double t_max;
  uint32_t ntypes, nbins, fallback;
  uint32_t hist_gens;
  uint32_t g_store_max;      // deepest generation a stored key can hold
  uint64_t root_base;        // global index of chunk-local root 0
  const TypeDev* types;      // [ntypes]
  const ZigTables* zig;
  const uint32_t* bin_info;  // [nbins]
  const uint64_t* bin_start; // [nbins + 1] global root offsets
  unsigned long long* root_rec;  // [rec_cap]
  uint64_t rec_cap;              // root records the buffer holds (checked build)
  unsigned long long* hist;  // [hist_gens][nbins][ntypes]
  unsigned long long* stats; // [0] vanished, [1] uncounted, [2] max generation
  uint32_t* error;           // bit 0: depth overflow, bit 1: sampler round budget exhausted,
                             // bit 2: grid barrier timeout, bit 3: persistent schedule out of
                             // buffers, bit 4: a bounds check of the checked build failed
  uint32_t nclass;           // histogram classes per generation
  // batched form only (null otherwise)
  const BatchType* btypes;   // [all types]
  const InstanceDev* inst;   // [instances]
  const uint32_t* bin_inst;  // [nbins] instance of each bin
  const uint32_t* bin_class; // [nbins] first histogram class of each bin
};

struct LevelIn {
  const ulonglong2* cells;
  const unsigned long long* prefix;  // nseg + 1
  uint32_t nseg;
  uint64_t stride;
  uint64_t lo, hi;  // virtual range of this launch
};

struct LevelOut {
  ulonglong2* cells;
  unsigned long long* count;   // [nseg]
  unsigned long long* prefix;  // [nseg + 1]
  uint32_t* ticket;
  uint64_t stride;
};

// Persistent driver: one launch runs every sweep of a plan. Its blocks (all resident: a
// cooperative launch) walk the same depth-first schedule of root chunks and generation
// slices as the host driver, each block keeping an identical copy of the schedule in
// shared memory and deciding from the level totals it reads after a grid barrier.
constexpr int kMaxPool = 48;

struct PersistArgs {
  RunArgs a;
  ulonglong2* cells[kMaxPool];
  unsigned long long* count[kMaxPool];
  unsigned long long* prefix[kMaxPool];
  uint32_t* ticket[kMaxPool];
  uint32_t nbuf;
  uint32_t g_limit;                 // deepest generation whose cells are stored
  uint64_t root_lo, root_hi;        // initial cells of the run
  uint64_t chunk;                   // initial cells per root sweep
  uint64_t max_slice;               // input cells per division sweep
  uint32_t* barrier;                // [2] arrivals, generation (zero before the launch)
  unsigned long long* out;          // [4] divisions, sweeps, max generation, chunks
  unsigned long long timeout_ns;    // a grid barrier waiting longer sets error bit 2
};

// One compiled configuration of the sweeps (the autotuner's search space): threads per
// block, input cells per lane per step, and where leaf counts are privatised (a window of
// classes in shared memory, or warp-aggregated atomics straight to the global table).
struct SweepKernels {
  int threads, cells, global_hist;
  int (*roots)(const RunArgs& a, uint64_t lo, uint64_t hi, const LevelOut& out, int blocks, void* stream);
  int (*divide)(const RunArgs& a, const LevelIn& in, uint32_t gen, const LevelOut& out, int blocks,
                void* stream);
  int (*persist)(const PersistArgs& p, int blocks, void* stream);  // cooperative launch
  int (*occupancy)(int* roots_per_sm, int* divide_per_sm, int* persist_per_sm);
};

constexpr int kNumSweepConfigs = 8;  // {128, 256} threads x {1, 2} cells x {smem, global}
constexpr int kDefaultSweepConfig = 4;  // 256 threads, 1 cell per lane, shared-memory window
// narrow key layout: any configuration; wide layout: the default configuration only.
const SweepKernels& sweep_kernels(bool narrow, bool batched, int config);

// Launchers of the default configuration (pc_kernels.cu). All return the cudaError_t of
// the launch as int; a.btypes != nullptr selects the batched instantiations.
int launch_root_sweep(const RunArgs& a, uint64_t root_lo, uint64_t root_hi, const LevelOut& out,
                      int blocks, bool narrow, void* stream);
int launch_divide_sweep(const RunArgs& a, const LevelIn& in, uint32_t gen, const LevelOut& out,
                        int blocks, bool narrow, void* stream);
int launch_debug_philox(const uint32_t* ctr, uint64_t n, uint32_t k0, uint32_t k1, uint32_t* out,
                        void* stream);
int launch_debug_normals(const ZigTables* zig, uint32_t k0, uint32_t k1, uint32_t root,
                         uint64_t first_parent, uint64_t count, float* z, void* stream);
int occupancy_blocks_per_sm(int* root_blocks, int* divide_blocks);
// One instance's leaf counts (rows of nclass classes, hist_gens rows; its nb x nt classes from
// class_begin) merged into totals[v] and per_type[v][nt] (file type order s2f), v = vidx[b][g];
// both zeroed by the caller. A count outside the value set sets bit 0 of *error.
int launch_merge_counts(const unsigned long long* hist, uint64_t nclass, uint64_t class_begin, uint32_t hist_gens,
                        uint32_t nb, uint32_t nt, const int32_t* vidx, uint32_t vidx_stride, const uint32_t* s2f,
                        unsigned long long* totals, unsigned long long* per_type, uint32_t* error, void* stream);
// Throughput probe (roofline denominators): kind 0 FP64 FMA, 1 FP32 FMA, 2 INT32 multiply-add;
// each of the blocks x 256 threads runs iters x 8 operations.
int launch_peak_probe(int kind, uint32_t iters, int blocks, double* sink, void* stream);
// Grid barriers in a cooperative launch of `blocks` blocks (failure-detection tests; mode as
// k_barrier_probe in pc_kernels.cu).
int launch_barrier_probe(uint32_t* bar, unsigned long long timeout_ns, unsigned long long long_ns, uint32_t* error,
                         uint32_t* passed, int mode, int blocks, void* stream);

// Smoothed (differentiable) form (pc_smooth.cu). For every candidate parameter set c
// (per type k: ratio, mean, sd) and every bin b, the expected leaf count at generation g
// of the bin's initial cells, estimated along sampled lineage paths with every hard test
// "due time <= t_max" replaced by sigmoid((t_max - S)/h).
constexpr int kSmoothMaxTypes = 8;
constexpr int kSmoothMaxRows = 64;  // generations per bin (cap + 1)

// A sampled lineage's initial age: U (FP64 form) and 1 + U as a pair of floats hi + lo.
struct LineageU {
  double u;
  float hi, lo;
};

struct SmoothArgs {
  uint32_t k0, k1;            // seed
  uint32_t nbins, rows;       // rows = max cap + 1 (generation rows per bin)
  uint32_t ntypes, paths;     // lineages sampled per initial cell (independent replicas)
  uint32_t ncells;            // initial cells; replica m of cell r draws as cell r + m * ncells
  double t_max, inv_h;
  const uint64_t* bin_start;  // [nbins + 1]
  const uint32_t* bin_cap;    // [nbins]
  const uint32_t* bin_order;  // [nbins] the bins in launch order (most expensive first)
  const ZigTables* zig;
  uint32_t* error;            // bit 1: sampler round budget exhausted
  uint32_t* order;            // [ntypes][ncand] scratch: the candidates of each type by mean
  // the lineages' draws, made once per smoothed plan (null: drawn in every pass):
  // lin_z[L * zrow + j], j < the bin's cap + 1, and lin_u[L] for lineage L = first initial
  // cell of its bin x paths + its index in the bin
  const float* lin_z;
  const LineageU* lin_u;
  uint32_t zrow;              // floats per lineage in lin_z, a multiple of 4
};

// Every lineage's draws into lin_z / lin_u (params-independent: once per smoothed plan).
int launch_smooth_draws(const SmoothArgs& A, float* lin_z, LineageU* lin_u, void* stream);
// e_raw[c][k][b][g] (FP64) for params[c][k][3] = (ratio, mean, sd): type k's part.
int launch_smooth_forward(const SmoothArgs& A, const double* params, uint32_t ncand, double* e_raw,
                          void* stream);
// expected[c][v] = sum of e_raw[c][k][b][g] over the types and the (b, g) of value v (CSR
// lists inv_off/inv_idx, inv_idx = b * rows + g; per_type = nbins * rows).
int launch_smooth_merge(const double* e_raw, uint32_t ncand, uint32_t ntypes, uint32_t per_type,
                        const uint32_t* inv_off, const uint32_t* inv_idx, uint32_t nvalues, double* expected,
                        void* stream);
// grad_params[c][k][3] = d(sum_v grad_expected[c][v] * expected[c][v]) / d params[c][k][.],
// regenerating every normal from its Philox counter; vidx[b][g] maps rows to values (-1: none).
int launch_smooth_backward(const SmoothArgs& A, const double* params, uint32_t ncand, const double* grad_expected,
                           uint32_t nvalues, const int32_t* vidx, double* grad_part, double* grad_params,
                           void* stream);

// expected[c][v] as launch_smooth_merge, and jacobian[c][v][k][3] = d expected[c][v] /
// d params[c][k][.] by forward-mode tangents along the same lineages (one walk per lineage,
// type and candidate); jac_raw is scratch [c][b][g][k][3].
int launch_smooth_jacobian(const SmoothArgs& A, const double* params, uint32_t ncand, const uint32_t* inv_off,
                           const uint32_t* inv_idx, uint32_t nvalues, double* jac_raw, double* expected,
                           double* jacobian, void* stream);

// loss[c], jtj[c][P][P], jtr[c][P] (P = 3 ntypes): the Gauss-Newton system of
// sum_v (log1p(E_cv) - log1p(target_v))^2 in the parameters, from one Jacobian pass whose
// rows are reduced on the device (nothing of size [c][v][P] is written).
int launch_smooth_gauss_newton(const SmoothArgs& A, const double* params, uint32_t ncand, const uint32_t* inv_off,
                               const uint32_t* inv_idx, uint32_t nvalues, const double* target, double* jac_raw,
                               double* loss, double* jtj, double* jtr, void* stream);

// Host helpers (pc_api.cpp).
ZigTables host_zig_tables();
void host_truncation_bounds(double mu, double sigma, float& zlo, float& zhi);

// The output value set a plan builds for this histogram and phi (0: automatic), ascending,
// into values[capacity]; PC_ERR_INVALID (with *n_values set) when it does not fit.
int host_value_set(const ::pc_bin* bins, uint64_t n_bins, double phi, double* values, uint64_t capacity,
                   uint64_t* n_values);

// Root chunk and key layout of a run with `roots` initial cells and deepest phi cap gmax:
// at most `chunk` initial cells per root sweep; keys for every generation up to
// min(gmax, g_store_max + 1) (the stored cells, g <= g_store_max, and the daughters of the
// deepest of them, parked with a key when their first draw is not settled) fit in
// bits_for(chunk) + g <= 64 bits; the narrow layout when gmax <= kNarrowMaxGen.
struct KeyLayout {
  uint64_t chunk;
  uint32_t g_store_max;
  bool narrow;
};
KeyLayout key_layout(uint64_t roots, uint32_t gmax, bool batched, uint64_t max_root_chunk);

}  // namespace pc
