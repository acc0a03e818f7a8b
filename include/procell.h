/* procell: GB300-native (sm_103a) engine for ProCell's stochastic proliferation path.
 *
 * C ABI of libprocell.so. Plain pointers and sizes only; no CUDA or C++ types cross it.
 * Every entry point returns PC_OK (0) or a PC_ERR_* code; pc_last_error() then holds a
 * one-line message. A context is used by one host thread at a time.
 *
 * What the reference exposes for this path, and what replaces it here:
 *
 *  reference (ericniso/cuda-pro-cell)                         this library
 *  ---------------------------------------------------------  --------------------------
 *  Simulator::create_cell_population                            pc_plan_create + pc_plan_run
 *    -> simulation::create_cells_population                      (root sweep on the GPU;
 *       src/simulation/cells_population.cu:18-54                  roots never leave HBM)
 *  Simulator::start_simulation                                  pc_plan_run
 *    -> bool simulation::proliferate(cell_types&, uint64_t size,
 *         uint64_t tree_depth, cell* h_cells, double t_max,
 *         double threshold, fluorescences_result&, bool track_ratio)
 *       src/simulation/proliferation.h:12-19,
 *       src/simulation/proliferation.cu:26-215
 *  the filled fluorescences_result (value, frequency, ratio[])  pc_plan_result -> pc_histogram
 *    src/simulation/data_types.h:32-37, parser.cu:126-151
 *  io::load_fluorescences / load_cell_types / save_fluorescences pc_load_histogram,
 *    src/io/parser.cu:68-217                                      pc_load_cell_types,
 *                                                                 pc_write_histogram
 *  the whole process (main, src/main.cu:18-34)                  the `procell` CLI, or
 *                                                                 pc_simulate in one call
 *
 * Differences at the boundary: the reference takes ownership of a host array of 40-byte
 * root cells that it created on the GPU and copied back (cells_population.cu:52); here
 * roots are generated in HBM from the histogram and never cross PCIe/C2C. The reference
 * reports no errors (proliferate always returns true); here every CUDA failure is
 * returned as a status. Counts are uint64 (the reference adds into the low 32 bits).
 */
#ifndef PROCELL_H
#define PROCELL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PC_OK 0
#define PC_ERR_INVALID 1     /* bad argument or input (message says which) */
#define PC_ERR_CUDA 2        /* a CUDA runtime call failed */
#define PC_ERR_NOMEM 3       /* device or host allocation failed / budget too small */
#define PC_ERR_DEPTH 4       /* a lineage went deeper than the key layout allows */
#define PC_ERR_UNSUPPORTED 5 /* e.g. more cell types than the kernels hold */
#define PC_ERR_IO 6          /* a file could not be opened or written */
#define PC_ERR_INTERNAL 7    /* an unexpected internal error (message says which) */

/* One histogram row, as in the reference's `fluorescence` (data_types.h:26-30). */
typedef struct pc_bin {
  double value;
  uint64_t frequency;
} pc_bin;

/* One cell type in file order (the reference's `cell_type` without `name`, which is the
 * 0-based line index, data_types.h:19-24). mean < 0 marks a quiescent type. */
typedef struct pc_cell_type {
  double ratio;
  double mean;
  double sd;
} pc_cell_type;

typedef struct pc_stats {
  uint64_t roots;           /* initial cells simulated */
  uint64_t divisions;       /* internal tree nodes */
  uint64_t leaves;          /* leaves counted into the histogram */
  uint64_t uncounted;       /* out-of-time roots whose value is below phi */
  uint64_t vanished;        /* due cells whose daughters would fall to phi or below */
  uint32_t max_generation;  /* deepest generation reached */
  uint32_t sweeps;          /* division sweeps (one kernel launch each, or phases of the
                               persistent launch) */
  uint32_t root_sweeps;     /* root sweeps (chunks of initial cells) */
  uint32_t kernel_launches; /* kernels launched by the run */
  double device_ms;         /* summed duration of the simulation kernels (CUDA events) */
  double divide_ms;         /* ... of the division sweeps alone */
  uint64_t h2d_bytes;       /* host-to-device bytes of the plan and the run */
  uint64_t d2h_bytes;       /* device-to-host bytes of the run and the result */
} pc_stats;

/* The output histogram: every value of the reference's output value set (each nonzero
 * bin value halved while >= phi, deduplicated, ascending; parser.cu:126-151), the total
 * count and the per-type counts (row-major [n_values][n_types], types in file order).
 * Rows with total 0 are kept; the writer skips them as the reference does. */
typedef struct pc_histogram {
  uint64_t n_values;
  uint32_t n_types;
  double* values;
  uint64_t* totals;
  uint64_t* per_type;
  pc_stats stats;
} pc_histogram;

typedef struct pc_context pc_context;
typedef struct pc_plan pc_plan;

/* Context: device, stream, memory pool. device = CUDA ordinal. */
int pc_create(pc_context** out, int device);
void pc_destroy(pc_context* ctx);
const char* pc_last_error(const pc_context* ctx); /* ctx may be NULL (creation errors) */
const char* pc_version(void);

/* Use `stream` (a cudaStream_t) for all work of this context; NULL = the context's own
 * (non-blocking) stream. The legacy default stream is selected by its handle value
 * cudaStreamLegacy ((void*)1). */
int pc_set_stream(pc_context* ctx, void* stream);

/* Tuning knobs (results never depend on them):
 *   "memory_budget_bytes" device bytes the level buffers may use (default: half of the
 *                         free memory at first use)
 *   "max_slice_cells"     cap on cells per division-sweep launch (default: from budget)
 *   "max_root_chunk"      cap on roots per root-sweep launch (default: from budget)
 *   "grid_blocks"         blocks per launch (default: resident blocks x SMs)
 *   "sweep_config"        compiled sweep configuration 0-7 (default 4; see pc_autotune)
 *   "driver"              0: one kernel launch per sweep (default); 1: one persistent
 *                         cooperative launch per run
 *   "graph"               1: the persistent driver captures its run in a CUDA graph once
 *                         per plan and replays it
 *   "device_merge"        1 (default): pc_plan_result merges the counts into the value
 *                         histogram on the device; 0: reads the count table back and
 *                         merges on the host (as it does anyway for merge scratch above
 *                         256 MB)
 *   "batch_parts"         1-64: pc_simulate_batch runs n instances as min(batch_parts,
 *                         n / 256) consecutive sub-batches, preparing the next and merging
 *                         the previous on host threads while one runs (default 4)
 *   "smooth_predraw"      1 (default): pc_smooth_create draws every sampled lineage's
 *                         normals and initial age once and keeps them in device memory
 *                         (when they fit in 1 GB); 0: every pass draws them again
 * Failure injection (no counterpart in the reference, which checks no CUDA status):
 *   "fail_nth_call"       n >= 1: the n-th CUDA call the library makes for this context
 *                         from now on (allocation, copy, memset, synchronisation, event
 *                         record, kernel or graph launch) does not reach CUDA and fails
 *                         once instead, as that call would (PC_ERR_NOMEM for allocations,
 *                         PC_ERR_CUDA otherwise); 0 disarms. For tests of the error paths:
 *                         every failure must come back as a status, leak nothing and leave
 *                         the context usable.
 */
int pc_set_option(pc_context* ctx, const char* name, double value);

/* Counters for those tests (no counterpart in the reference): "cuda_calls" (CUDA calls the
 * library made for this context so far), "faults_injected", "device_allocations" (device
 * allocations of the library live in this process, all contexts), "level_buffers" (level
 * buffers the context's pool holds). */
int pc_get_option(pc_context* ctx, const char* name, double* value);

/* phi == 0 selects the reference's automatic threshold: the smallest value with a
 * nonzero frequency (parser.cu:80-96). phi < 0 is invalid. seed keys the random stream;
 * equal inputs and seed give bit-identical histograms on any run, chunking or device. */
int pc_plan_create(pc_context* ctx, const pc_bin* bins, uint64_t n_bins,
                   const pc_cell_type* types, uint32_t n_types, double t_max, double phi,
                   uint64_t seed, pc_plan** out);
/* Restrict the plan to initial cells [root_begin, root_end) of the file order (a shard).
 * Shards of one plan are disjoint and their histograms add up to the full one. */
int pc_plan_set_roots(pc_context* ctx, pc_plan* plan, uint64_t root_begin, uint64_t root_end);
/* Run all sweeps on the device. Counts stay in HBM until pc_plan_result. */
int pc_plan_run(pc_context* ctx, pc_plan* plan);
/* Statistics of the last pc_plan_run (leaves is filled by pc_plan_result only). */
int pc_plan_stats(pc_context* ctx, const pc_plan* plan, pc_stats* out);
/* Merge equal values of the counts into `out` (free with pc_histogram_free): on the device,
 * reading back only the merged counts (values x (1 + types)); for plans whose merge scratch
 * would exceed 256 MB, by reading the count table back and merging on the host. */
int pc_plan_result(pc_context* ctx, pc_plan* plan, pc_histogram* out);
/* The raw per-(generation, bin, type) counts as uint64 [gens][bins][types], bins in file
 * order of the nonzero rows and types in file order. *n_elems gets the element count;
 * pass host_out = NULL to query the shape (gens, bins, types in dims[3]). */
int pc_plan_raw_counts(pc_context* ctx, pc_plan* plan, uint64_t* host_out, uint64_t capacity,
                       uint64_t* n_elems, uint32_t dims[3]);
void pc_plan_destroy(pc_plan* plan);

/* One call: plan, run, result, destroy. */
int pc_simulate(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                uint32_t n_types, double t_max, double phi, uint64_t seed, pc_histogram* out);
void pc_histogram_free(pc_histogram* h);

/* Sharding (one process or GPU per shard): pc_simulate on initial cells [root_begin,
 * root_end) of the file order only. Every shard's histogram has the full value set, and
 * the shards' histograms added with pc_histogram_accumulate equal the unsharded one bit for
 * bit (the random stream is keyed by initial cell, not by shard). */
int pc_simulate_shard(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                      uint32_t n_types, double t_max, double phi, uint64_t seed, uint64_t root_begin,
                      uint64_t root_end, pc_histogram* out);
/* dst += src: totals, per-type counts and statistics (summed; max_generation the larger).
 * Both must hold the same value set and type count (else PC_ERR_INVALID, dst unchanged).
 * Host only. */
int pc_histogram_accumulate(pc_histogram* dst, const pc_histogram* src);

/* ---- Batched form (no counterpart in the reference, which runs one input per process) --
 * Many independent inputs ("instances": each its own histogram, cell types, t_max, phi
 * and seed) run together: their initial cells are laid end to end and every sweep
 * processes cells of all instances at once, so the per-run fixed costs (planning,
 * launches, synchronisation, table transfers) are paid once per batch instead of once per
 * instance. Each instance's counts are bit-identical to pc_plan_run on that instance
 * alone with the same seed. Limits: at most 65535 cell types and 2^32-1 (bin, type)
 * classes over the batch. */
typedef struct pc_instance {
  const pc_bin* bins;
  uint64_t n_bins;
  const pc_cell_type* types;
  uint32_t n_types;
  uint32_t reserved; /* 0 */
  double t_max;
  double phi;        /* 0 = automatic, as pc_plan_create */
  uint64_t seed;
} pc_instance;

typedef struct pc_batch pc_batch;

/* Validates and uploads every instance (the inputs are copied; the caller's arrays may be
 * released afterwards). An invalid instance fails the call with its index in the message. */
int pc_batch_create(pc_context* ctx, const pc_instance* instances, uint32_t n_instances,
                    pc_batch** out);
int pc_batch_run(pc_context* ctx, pc_batch* batch);
/* Whole-batch statistics of the last run. */
int pc_batch_stats(pc_context* ctx, const pc_batch* batch, pc_stats* out);
uint32_t pc_batch_size(const pc_batch* batch);
/* One instance's merged histogram (stats: roots and leaves of that instance only). The
 * first call after a run copies the whole count table to the host once. */
int pc_batch_result(pc_context* ctx, pc_batch* batch, uint32_t instance, pc_histogram* out);
/* One instance's raw counts, in the layout of pc_plan_raw_counts. */
int pc_batch_raw_counts(pc_context* ctx, pc_batch* batch, uint32_t instance, uint64_t* host_out,
                        uint64_t capacity, uint64_t* n_elems, uint32_t dims[3]);
/* Replace the cell types of every instance (concatenated in instance order, each instance
 * with as many types as it was created with), keeping bins, t_max, phi and seed: the next
 * pc_batch_run simulates the new parameters (for parameter searches). All instances are
 * validated first; on error nothing changes. Results need a new run. */
int pc_batch_set_types(pc_context* ctx, pc_batch* batch, const pc_cell_type* types);
/* Merged totals of every instance after the last run, concatenated: instance i's counts per
 * value (its value set, ascending) are out[offsets[i] .. offsets[i + 1]). offsets (host,
 * n_instances + 1 entries) may be NULL; pass out = NULL to query the offsets only. */
int pc_batch_totals(pc_context* ctx, pc_batch* batch, uint64_t* out, uint64_t capacity, uint64_t* offsets);
void pc_batch_destroy(pc_batch* batch);
/* One call: create, run, results (out[n_instances], each freed with pc_histogram_free). */
int pc_simulate_batch(pc_context* ctx, const pc_instance* instances, uint32_t n_instances,
                      pc_histogram* out);

/* ---- Autotuning (no counterpart in the reference) -------------------------------------
 * The sweeps are compiled in several configurations (threads per block, input cells per
 * lane, and where leaf counts are privatised: a window of classes in shared memory per
 * block, or warp-aggregated atomics straight to the global table) and can be driven one
 * launch per sweep or by one persistent cooperative launch replayed from a CUDA graph.
 * None of this changes a single count. The context options "sweep_config" (0-7),
 * "driver" (0 per sweep, 1 persistent) and "graph" (0/1) select them; pc_autotune times
 * every combination on a prepared input and leaves the context set to the fastest, taking
 * the persistent driver when its best time is within 1% of the overall best (one graph
 * replay per run, no host round trip per sweep). */
typedef struct pc_tuning {
  int32_t config;         /* chosen "sweep_config" */
  int32_t driver;         /* chosen "driver" (graph replay is on with the persistent one) */
  int32_t threads;        /* threads per block of the chosen configuration */
  int32_t cells_per_lane;
  int32_t global_hist;    /* 1: leaf counts go straight to the global table */
  int32_t candidates;     /* combinations timed */
  double ms;              /* best wall time of one run with the choice */
  double ms_default;      /* the same for config 4, one launch per sweep */
} pc_tuning;

/* Each candidate runs once to warm up, then `repeats` times (best time kept). */
int pc_autotune(pc_context* ctx, pc_plan* plan, uint32_t repeats, pc_tuning* out);
int pc_batch_autotune(pc_context* ctx, pc_batch* batch, uint32_t repeats, pc_tuning* out);

/* ---- Smoothed, differentiable form (no counterpart in the reference) -------------------
 * Expected output-histogram counts as a smooth function of the cell-type parameters, for
 * calibrating (ratio, mean, sd) per type by gradient descent. Every hard test "due time <=
 * t_max" of the plain form becomes sigmoid((t_max - S) / h), with due times
 * S = sum(mean + sd * z) accumulated in FP64 along lineages sampled per initial cell
 * (`paths_per_cell` each), z taken from the plain form's Philox counters (untruncated).
 * The bins, t_max, phi and seed are fixed at creation; the parameters of any number of
 * candidates are passed per call. Quiescent types (mean < 0) count at generation 0.
 *
 * params:        device array [n_candidates][n_types][3] (ratio, mean, sd), FP64, types in
 *                file order (ratios are used as given: normalise them yourself)
 * expected:      device array [n_candidates][n_values] (FP64), values as pc_smooth_values
 * grad_expected: device array [n_candidates][n_values], dL/d expected
 * grad_params:   device array [n_candidates][n_types][3], dL/d params (the adjoint: the
 *                lineages are walked again, every normal regenerated from its counter)
 * jacobian:      device array [n_candidates][n_values][n_types][3], d expected[c][v] /
 *                d params[c][k][.] (forward-mode tangents in the same single pass that also
 *                writes `expected`; for Gauss-Newton / Levenberg-Marquardt searches)
 * The calls are asynchronous on the context's stream; pc_smooth_sync waits and reports. */
typedef struct pc_smooth pc_smooth;
int pc_smooth_create(pc_context* ctx, const pc_bin* bins, uint64_t n_bins, uint32_t n_types,
                     double t_max, double phi, double h, uint32_t paths_per_cell, uint64_t seed,
                     pc_smooth** out);
int pc_smooth_info(const pc_smooth* s, uint64_t* n_values, uint32_t* n_types, uint64_t* n_cells);
int pc_smooth_values(const pc_smooth* s, double* values); /* host array [n_values] */
int pc_smooth_forward(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                      double* expected);
int pc_smooth_backward(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                       const double* grad_expected, double* grad_params);
int pc_smooth_jacobian(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                       double* expected, double* jacobian);
/* The Gauss-Newton system of the squared log-count loss
 * L_c = sum_v (log(1 + E_cv) - log(1 + target_v))^2 for every candidate, from one Jacobian
 * pass reduced on the device: loss [n_candidates], jtj [n_candidates][P][P] and
 * jtr [n_candidates][P] (P = 3 n_types, parameter order of params) with J_v = (dE_v / dparams)
 * / (1 + E_v) and r_v = log(1 + E_v) - log(1 + target_v); target is a device array
 * [n_values]. For Levenberg-Marquardt searches that need neither E nor J themselves. */
int pc_smooth_gauss_newton(pc_context* ctx, pc_smooth* s, const double* params, uint32_t n_candidates,
                           const double* target, double* loss, double* jtj, double* jtr);
int pc_smooth_sync(pc_context* ctx);
void pc_smooth_destroy(pc_smooth* s);

/* ---- Histogram rebinning (the reference's utils::log_space / utils::rebin,
 * src/utils/util.cu:76-138, which its main path never calls) -------------------------------
 * pc_log_space: n >= 2 edges base^e for exponents from ceil(log_base(start)) to
 * ceil(log_base(end)) in equal steps. pc_rebin: counts of an ascending histogram summed
 * into the bins of pc_log_space(lower, upper, n_bins, 10), each value into the first bin
 * whose edge is >= the value; edges_out[n_bins], counts_out[n_bins]. Values above the last
 * edge or out of order give PC_ERR_INVALID. Host only. */
int pc_log_space(double start, double end, uint64_t n, double base, double* edges);
int pc_rebin(const double* values, const uint64_t* counts, uint64_t n_values, double lower,
             double upper, uint64_t n_bins, double* edges_out, uint64_t* counts_out);

/* File formats of the reference (parser.cu:68-217). Loaders read with the reference's
 * `in >> a >> b` semantics (stop at the first unparsable token). The loaders allocate
 * *out with malloc; release it with pc_free. pc_load_cell_types also applies the
 * reference's ratio-sum check (|1 - sum| <= 1e-8) and returns PC_ERR_INVALID with the
 * reference's message when it fails. */
int pc_load_histogram(const char* path, pc_bin** out, uint64_t* n);
int pc_load_cell_types(const char* path, pc_cell_type** out, uint32_t* n);
/* Writes rows with a nonzero total as `value\ttotal[\tper-type...]\n` with 10 significant
 * digits (the reference's std::ostream precision(10)). path NULL or "-" = stdout. */
int pc_write_histogram(const char* path, const pc_histogram* h, int track_ratio);
void pc_free(void* p);

/* Allocation-free simulation. No counterpart in the reference: it exists for callers that
 * may not allocate device memory themselves, e.g. a host application whose own pool owns
 * all GPU memory, code that must avoid the device-wide synchronisation cudaMalloc and
 * cudaFree imply, or a deployment with a memory budget certified in advance.
 *
 * It runs the same simulation as pc_simulate (bit-identical counts for the same inputs and
 * seed) with every intermediate in one static device array of PC_NOALLOC_SCRATCH_BYTES
 * (64 MiB) that each GPU loading this library reserves until the process exits; it calls
 * no cudaMalloc, cudaFree or other allocating routine, on the device or the host. Inputs
 * are host arrays in file order; the result is the raw per-(generation, bin, type) counts
 * written to the caller's `raw_counts` (capacity in elements), laid out as
 * pc_plan_raw_counts; dims receives (generations, nonzero bins, types) even when the
 * buffer is too small. Work is issued on `stream` (a cudaStream_t; NULL = the default
 * stream) of the current device and the call returns when it has finished.
 *
 * Limits: inputs whose rows, per-bin tables, counts and level buffers do not fit in the
 * array are rejected with PC_ERR_NOMEM and a message; at most 64 cell types. The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture. All calls share the array and
 * it keeps the last call's contents (each call clears what must start at zero): calls that
 * overlap on the GPU race, so serialise them. On error, a message is written to `err`
 * (err_len bytes, may be NULL). */
#define PC_NOALLOC_SCRATCH_BYTES (64u << 20)
int pc_simulate_noalloc(const pc_bin* bins, uint64_t n_bins, const pc_cell_type* types,
                        uint32_t n_types, double t_max, double phi, uint64_t seed, void* stream,
                        uint64_t* raw_counts, uint64_t capacity, uint32_t dims[3], pc_stats* stats,
                        char* err, size_t err_len);

/* Diagnostics for the parity tests: evaluate the engine's random stream on the device.
 * pc_debug_philox: out[4*i..] = Philox4x32-10(ctr[4*i..], key) for i < n.
 * pc_debug_normals: z[i] = first-attempt normal of child (i & 1) of node first_parent+i/2
 *                   under `root` (no truncation), as the division sweep computes it.
 * pc_debug_tables: the device's ziggurat tables (k[1024], w bits[1024], f bits[1025]). */
/* Grid barriers of the persistent driver in a cooperative launch of up to 8 blocks, with
 * the wait limited to timeout_ms (failure detection without a GPU fault; the context stays
 * usable). starve = 0: one barrier. starve = 1: the arrival counter is preset so that the
 * barrier can never complete: every block's wait runs out, error bit 2 (value 4) is set and
 * the kernel returns. starve = 2: two barriers, one block skips the second; one block waits
 * there with timeout_ms and the others with 100 x timeout_ms (at most 10 s), so the call
 * returns after about timeout_ms only if waiting blocks see another block's timeout.
 * *passed = blocks that got through every barrier. */
int pc_debug_barrier(pc_context* ctx, int starve, double timeout_ms, uint32_t* error_bits,
                     uint32_t* passed);
int pc_debug_philox(pc_context* ctx, const uint32_t* ctr, uint64_t n, const uint32_t key[2],
                    uint32_t* out);
/* Measured throughput of one arithmetic pipe of the context's GPU, in lane-operations per
 * second (one fused multiply-add = one operation): kind 0 FP64 FMA, 1 FP32 FMA, 2 INT32
 * multiply-add. A microbenchmark of about 30 ms (no counterpart in the reference); the
 * benchmark uses it as the denominator of pipe rooflines. */
int pc_debug_peak(pc_context* ctx, int kind, double* lane_ops_per_s);
int pc_debug_normals(pc_context* ctx, uint64_t seed, uint32_t root, uint64_t first_parent,
                     uint64_t count, float* z);
int pc_debug_tables(pc_context* ctx, uint32_t* k, uint32_t* w_bits, uint32_t* f_bits);

#ifdef __cplusplus
}
#endif

#endif /* PROCELL_H */
