/* Test infrastructure only: the CPU oracle for the proliferation path.
 *
 * This library is the CPU restatement that the GPU engine is compared against. Nothing in the
 * product (the procell library, its kernels or its CLI) links, loads or calls it; only
 * the test suite, the smoke check and the benchmark's CPU-baseline leg do.
 *
 * It restates, on the host and one tree node at a time, the reference's algorithm:
 *   - io::load_fluorescences / load_cell_types / save_fluorescences
 *     (src/io/parser.cu:68-217),
 *   - device::create_cell and the determine_* helpers (src/simulation/cell.cu:25-143),
 *   - device::proliferate and out_of_time (src/simulation/proliferation.cu:289-410),
 * with the reference's curand draws (src/utils/util.cu:143-169) replaced by the
 * engine's counter-based stream (Philox4x32-10 + a 128-layer FP32 ziggurat), which the
 * oracle implements independently of the product's sources.
 */
#ifndef PROCELL_ORACLE_H
#define PROCELL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_result oracle_result;

/* Simulate roots [root_begin, root_end) (root_end = UINT64_MAX for all roots) of the
 * histogram rows (values[i], freqs[i]) in file order and the cell types
 * (ratio, mean, sd) in file order. phi_given = 0 selects the reference's automatic
 * threshold (the smallest value with a nonzero frequency, parser.cu:80-96).
 * Returns NULL on invalid input (see oracle_last_error). */
oracle_result* oracle_simulate(const double* values, const uint64_t* freqs, uint64_t nrows,
                               const double* ratio, const double* mean, const double* sd,
                               uint32_t ntypes, double t_max, double phi, int phi_given,
                               uint64_t seed, uint64_t root_begin, uint64_t root_end,
                               int nthreads);
const char* oracle_last_error(void);
uint64_t oracle_result_nvalues(const oracle_result* r);
uint32_t oracle_result_ntypes(const oracle_result* r);
/* values[nvalues] ascending, totals[nvalues], per_type[nvalues*ntypes] (file order),
 * stats[6] = {roots, divisions, leaves_counted, leaves_uncounted, vanished, max_gen}. */
void oracle_result_copy(const oracle_result* r, double* values, uint64_t* totals,
                        uint64_t* per_type, uint64_t* stats);
void oracle_result_free(oracle_result* r);

/* Philox4x32-10 of one counter block. */
void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The FP32 ziggurat tables (k[256], w[256] as bits, f[257] as bits). */
void oracle_tables(uint32_t* k, uint32_t* w_bits, uint32_t* f_bits);
/* Standard normals drawn for the children of nodes: z[i] is the first-attempt variate of
 * child (i & 1) of parent node (first_parent + i/2) under root `root` (no truncation). */
void oracle_normals(uint64_t seed, uint32_t root, uint64_t first_parent, uint64_t count,
                    float* z);
/* The division time of child c of parent node n (truncated normal, tau > 0). */
double oracle_tau(uint64_t seed, uint32_t root, uint64_t parent, uint32_t child, double mean,
                  double sd);
/* The smoothed form (oracle/smooth_ref.py restated in C++, FP64, `nthreads` threads; 0 =
 * all): expected counts [ncand][V] and, with grad_expected [ncand][V], the gradient
 * [ncand][ntypes][3] of sum(grad_expected * expected) for params [ncand][ntypes][3]. V goes
 * to *nvalues; returns -1 (nothing computed) when V > nvalues_cap. */
int oracle_smooth(const double* values, const uint64_t* freqs, uint64_t nrows, double t_max, double phi,
                  int phi_given, double h, uint32_t paths, uint64_t seed, const double* params,
                  uint32_t ncand, uint32_t ntypes, const double* grad_expected, double* expected,
                  double* grad, uint64_t nvalues_cap, uint64_t* nvalues, int nthreads);
/* The FP32 exp/log helpers of the ziggurat's slow path. */
float oracle_expf(float x);
float oracle_logf(float u);

#ifdef __cplusplus
}
#endif

#endif
