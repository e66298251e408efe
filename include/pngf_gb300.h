/* pngf_gb300 — GB300 (sm_103a) implementation of the PNGF direct-binary-search
 * hot path: Woodbury tile-flip evaluation and the rank-k accept update over a
 * precomputed numerical Green's function (NGF) matrix G.
 *
 * C ABI. Every call returns a status code (PNGF_OK = 0); pngf_last_error()
 * gives a message for the last failure on a handle. A handle owns one CUDA
 * stream and all device memory for every frequency; it is not thread-safe.
 * Complex numbers are passed as interleaved (re, im) doubles.
 *
 * The reference is the header-only C++ class PNGF_Optimizer
 * (pngf-opt/pngfopt.hpp:18-679) driven by pngf-opt/main.cpp. Each entry point
 * names the reference member or code block it replaces.
 *
 * Algebra. With H = G - I, P the 0/1 design-edge indicator and C = I + P H
 * (the reference's C = (I-P) + P G, pngfopt.hpp:196-233), the handle keeps,
 * per frequency, the augmented matrix
 *     M = [ T  y    ]     T = H C^-1 (N x N),    y = T PEinc,
 *         [ R  Eobj ]     R = Gobj C^-1 (E x N), Eobj = R PEinc,
 * instead of C^-1 (pngfopt.hpp:240-249). A flip of the edge set s with signs
 * d (diag D) needs only gathers of M: its capacitance matrix is
 * K = I + T[s,s] D (the reference's I + V C^-1 U, pngfopt.hpp:435-455), and
 * newEobj = Eobj - R[:,s] D (Einc_s + K^-1 w), w = y_s - T[s,s] D Einc_s
 * (pngfopt.hpp:458-537). Accepting the flip is one rank-k update
 * M <- M - M[:,s] W with W = [D K^-1 T[s,:] , D (Einc_s + K^-1 w)]
 * (replaces update_C_inv, pngfopt.hpp:256-367, and compute_R_matrix(0)).
 */
#ifndef PNGF_GB300_H
#define PNGF_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PNGF_OK 0
#define PNGF_ERR_ARG 1         /* bad argument (null pointer, size, index) */
#define PNGF_ERR_CUDA 2        /* a CUDA runtime call failed */
#define PNGF_ERR_NOMEM 3       /* device or host allocation failed */
#define PNGF_ERR_IO 4          /* G file missing or short */
#define PNGF_ERR_SINGULAR 5    /* capacitance matrix K has a zero pivot */
#define PNGF_ERR_STATE 6       /* call out of order (e.g. accept before eval) */
#define PNGF_ERR_TIMEOUT 7     /* a bounded device wait ran out */
#define PNGF_ERR_UNSUPPORTED 8 /* configuration not supported by this build */
#define PNGF_ERR_NO_DEVICE 9   /* no usable CUDA device / kernel image */
#define PNGF_ERR_SCRATCH 10    /* request larger than the fixed scratch of pngf_accept_edges_noalloc */

/* ---- precision modes ---- */
#define PNGF_PREC_FP64 0 /* M in complex128, all arithmetic FP64 */
#define PNGF_PREC_C64 1  /* M in complex64, rank-k update on tensor cores;
                            capacitance LU, objective and accept test in FP64 */

#define PNGF_MAX_FREQ 16
#define PNGF_MAX_EOBJ 4

typedef struct pngf_handle pngf_handle;

/* Problem description. Mirrors the arguments of PNGF_Optimizer::init
 * (pngfopt.hpp:66-69) plus the constants pngf-opt/main.cpp fixes
 * (frequencies main.cpp:116-117, k0 main.cpp:162-164). */
typedef struct pngf_config {
  int tiles_x, tiles_y;  /* map_xsz, map_ysz */
  int cells_x, cells_y;  /* Yee cells per tile: tiles_yee_x, tiles_yee_y (3, 3) */
  int num_eobj;          /* E: rows of Gobj (1 port voltage + 2 NF2FF rows = 3) */
  int max_flips;         /* most tiles flipped by one candidate (4 for mirror mode) */
  double dx, dy, dz;     /* Yee cell size, metres */
  int num_freq;          /* frequencies handled by this handle */
  double freq_hz[PNGF_MAX_FREQ];
  int precision;         /* PNGF_PREC_FP64 or PNGF_PREC_C64 */
  int defer_rank;        /* C64: flush the deferred low-rank correction at this rank (0 = every accept) */
  int device;            /* CUDA device ordinal */
  int fp64_update;       /* PNGF_PREC_FP64: PNGF_F64_TENSOR (default) or PNGF_F64_SIMT */
  int c64_build;         /* PNGF_PREC_C64: PNGF_BUILD_FP64 (default) or PNGF_BUILD_C64, see below */
  int state_only;        /* 1: between calls the device holds only the state (see below) */
} pngf_config;

/* state_only = 1 (no reference counterpart): G comes from the built-in
 * synthetic generator (pngf_load_G_synth) and is regenerated on the device
 * whenever a build (pngf_prepare, pngf_refresh) or a drift check needs it,
 * instead of being kept; a PNGF_PREC_C64 handle also allocates its FP64
 * staging of M only for those calls. Device memory between calls is then the
 * state alone (complex64 T: 8 N^2 bytes per frequency), which is what lets many
 * large instances share one GPU. pngf_load_G / pngf_load_G_file return
 * PNGF_ERR_UNSUPPORTED on such a handle. */

/* How pngf_prepare builds the state of a PNGF_PREC_C64 handle for a design:
 * PNGF_BUILD_FP64 - in FP64 (as a PNGF_PREC_FP64 handle does), then T is
 *                   rounded to complex64;
 * PNGF_BUILD_C64  - directly in complex64: the design's edges are accepted in
 *                   chunks through the complex64 accept step (FP64 factor and
 *                   solves, 3xTF32 tensor-core update). Several times faster
 *                   and about as accurate as a run of complex64 accepts.
 * pngf_refresh always rebuilds in FP64. */
#define PNGF_BUILD_FP64 0
#define PNGF_BUILD_C64 1

/* How a PNGF_PREC_FP64 handle runs its rank-k accept update:
 * PNGF_F64_TENSOR - exact integer slices on the BF16 tensor cores, recombined
 *                   to FP64 accuracy (flip sets of up to 32 edges; larger ones
 *                   use the FP64 units);
 * PNGF_F64_SIMT   - FP64 fused multiply-adds on the FP64 units. */
#define PNGF_F64_TENSOR 0
#define PNGF_F64_SIMT 1

/* Fills a config with the reference's defaults (main.cpp:142-160):
 * 3x3 cells per tile, E = 3, dx = dy = 0.01/60 m, dz = 0.01/180 m, FP64. */
void pngf_config_default(pngf_config *cfg, int tiles_x, int tiles_y, int num_freq,
                         const double *freq_hz);

/* Number of design edges N for a tile map (pngfopt.hpp:86-94). */
long pngf_num_edges(int tiles_x, int tiles_y, int cells_x, int cells_y);

/* ---- G matrices (acmefdfd layout: (N+E-1)^2 complex128, column-major) ---- */

/* Synthetic complex-symmetric stand-in for an acmefdfd G: dyadic free-space
 * Green's function at k = 2 pi f sqrt(eps_r)/c between Yee edge centres,
 * edge-projected, scaled by dx*dy*dz; diagonal (0.3+0.05i) x row's largest
 * off-diagonal magnitude; seeded symmetric complex Gaussian relative
 * perturbation 1e-3. Writes N x N column-major with leading dimension ld. */
int pngf_synth_G(int tiles_x, int tiles_y, int cells_x, int cells_y, double dx, double dy,
                 double dz, double freq_hz, double eps_r, unsigned long long seed, double *out,
                 long ld);
/* NF2FF rows of the synthetic G (no reference counterpart; they stand in for
 * the far-field rows acmefdfd appends to G, acmefdfd/main.cpp:466-492): the
 * broadside far-field projection of the edge currents, row 1 (theta) over
 * the x-directed edges and row 2 (phi) over the y-directed ones, each entry
 * 32 eta0 dx dy dz times a seeded complex 1 + 1e-3 perturbation. Writes 2 x n
 * complex, row-major (the gobj_rows layout below). */
int pngf_synth_gobj(int tiles_x, int tiles_y, int cells_x, int cells_y, double dx, double dy, double dz,
                    unsigned long long seed, double *rows);
/* Writes / reads a G file (acmefdfd/main.cpp:533-538, pngfopt.hpp:163-180).
 * gobj_rows: (num_eobj-1) rows of n complex entries, row-major; NULL = zero. */
int pngf_write_G_file(const char *path, long n, int num_eobj, const double *G, long ldg,
                      const double *gobj_rows);
int pngf_read_G_file(const char *path, long n, int num_eobj, double *G, long ldg,
                     double *gobj_rows);

/* ---- handle lifecycle ---- */

/* Allocates device state for every frequency. Replaces the constructor and
 * the buffer sizing of PNGF_Optimizer::init (pngfopt.hpp:66-119). */
int pngf_create(const pngf_config *cfg, pngf_handle **out);
int pngf_destroy(pngf_handle *h);
/* Runs all later work on this CUDA stream (cudaStream_t); NULL = the handle's own. */
int pngf_set_stream(pngf_handle *h, void *cuda_stream);
const char *pngf_last_error(const pngf_handle *h);
/* N (edges) and the leading dimension of the device matrix M. */
int pngf_dims(const pngf_handle *h, long *n_edges, long *ld_m);

/* Loads frequency f's G from host memory (column-major, leading dimension
 * ldg) and the E-1 objective rows (row-major, may be NULL = zero). Replaces
 * the file read of PNGF_Optimizer::init (pngfopt.hpp:121-184). */
int pngf_load_G(pngf_handle *h, int f, const double *G, long ldg, const double *gobj_rows);
/* Same, from an acmefdfd G file. Missing or short file -> PNGF_ERR_IO. */
int pngf_load_G_file(pngf_handle *h, int f, const char *path);
/* No reference counterpart: frequency f's G is the synthetic G of
 * pngf_synth_G (same recipe, generated on the device; entries agree with
 * the host generator to ~1e-15 relative), with the synthetic NF2FF rows of
 * pngf_synth_gobj (from the same seed) as objective rows 1 and 2. */
int pngf_load_G_synth(pngf_handle *h, int f, unsigned long long seed, double eps_r);

/* Sets the design (PNGF_Optimizer::set_tile_map, pngfopt.hpp:669-674). */
int pngf_set_tile_map(pngf_handle *h, const int *tile_map);
int pngf_get_tile_map(const pngf_handle *h, int *tile_map);
/* Source port of x-directed edges (set_source_port, pngfopt.hpp:559-618);
 * an invalid y offset/size is PNGF_ERR_ARG (the reference exits). */
int pngf_set_source_port(pngf_handle *h, int tile_x, int tile_y, int y_offset, int y_size);
/* Builds M for the current design at every frequency. Replaces
 * compute_C_matrix + LinAlg::invertMatrix + compute_PEinc +
 * compute_R_matrix(1) (main.cpp:244-252; pngfopt.hpp:196-250, 542-552;
 * linalg.hpp:34-85). */
int pngf_prepare(pngf_handle *h);

/* Current Eobj (E complex) and the port constants Vinc, LN1inc, LN2inc
 * (3 complex) of frequency f: the members main.cpp reads (277-284). */
int pngf_get_eobj(pngf_handle *h, int f, double *eobj, double *vinc_ln);
/* Objective F = sum_f 200|S11|^2 + (15-D)^2 of the current design
 * (main.cpp:271-302). */
int pngf_objective(pngf_handle *h, double *F);
/* Copies frequency f's M ((N+E) x (N+1), row-major complex, leading
 * dimension ld >= N+1) to host memory, and Einc (N complex) if einc is not
 * NULL. The reference keeps its state in the public members C, R, S
 * (pngfopt.hpp:21-26); M holds the same information (see the top of this
 * header). */
int pngf_get_M(pngf_handle *h, int f, double *M, long ld, double *einc);

/* ---- hot path ---- */

/* Evaluates ncand candidates at every frequency. Candidate c flips tiles
 * tiles[c*max_flips .. + nflip[c]-1]. Outputs (host memory, either may be
 * NULL): new_eobj[(c*num_freq + f)*E] (complex) and F[c]. Also records the
 * batch so that pngf_accept can apply one of its candidates.
 * Replaces compute_updated_Eobj (pngfopt.hpp:379-539) and the objective loop
 * (main.cpp:401-420). */
int pngf_eval_candidates(pngf_handle *h, const int *tiles, const int *nflip, int ncand,
                         double *new_eobj, double *F);
/* Same with device pointers, asynchronous on the handle's stream. d_first,
 * if not NULL, receives the index of the first candidate with F < F_best
 * (-1 if none), the accept test of main.cpp:429. */
int pngf_eval_candidates_device(pngf_handle *h, const int *d_tiles, const int *d_nflip,
                                int ncand, double *d_new_eobj, double *d_F, double F_best,
                                int *d_first);
/* Accepts candidate `cand` of the last evaluated batch at every frequency:
 * rank-k update of M, then P and the tile map are committed. Replaces
 * update_C_inv + compute_PEinc + compute_R_matrix(0) (main.cpp:447-452). */
int pngf_accept(pngf_handle *h, int cand);

/* Accept step on caller-owned device memory that allocates nothing. No
 * counterpart in the reference. For callers that cannot allocate device
 * memory (a framework allocator that owns the GPU, an FFI host that cannot
 * free foreign allocations, a loop that cannot afford cudaMalloc's device
 * synchronisation). Applies the rank-k update M <- M - M[:,s] W for the
 * flip of edges s (k of them, signs d = +-1) to the augmented matrix M
 * ((N+E) x ldm row-major complex128, the layout pngf_get_M returns) with
 * Einc (N complex), all device pointers, asynchronously on `stream`
 * (cudaStream_t, NULL = default). Scratch lives in one fixed 8 MiB device
 * array: (N+E+ldm) k 16 + k^2 16 + 20 k bytes (plus alignment) must fit, and
 * k <= 104, else PNGF_ERR_SCRATCH / PNGF_ERR_ARG. The first call on a device
 * looks up that array's address (do it before any stream capture; the address
 * is not valid across cudaDeviceReset). Calls share the array: calls that
 * overlap on the GPU race. s must hold k distinct edges. *status (device int,
 * may be NULL) is cleared, then set on the device to PNGF_ERR_ARG if an index
 * of s is outside [0, n) or a sign of d is not +-1, or to PNGF_ERR_SINGULAR if
 * K is singular; in both cases M is left unchanged. */
int pngf_accept_edges_noalloc(double *M, long ldm, long n, int num_eobj, const double *Einc, const int *s,
                              const signed char *d, int k, int *status, void *stream);

/* Drift check of a PNGF_PREC_C64 handle: on `nrows` (1..8) sampled rows of T
 * at every frequency, the exact FP64 rows for the current design are formed
 * from G by iterative refinement (X <- X - (X C - H) C^-1 with
 * C^-1 = I - P T, two sweeps) and *max_rel = max |T_c64 - T| / max |T|. */
int pngf_drift_check(pngf_handle *h, int nrows, double *max_rel);
/* The same at frequency f only. */
int pngf_drift_check_freq(pngf_handle *h, int f, int nrows, double *max_rel);
/* Rebuilds M from G for the current design (drift refresh). */
int pngf_refresh(pngf_handle *h);

/* ---- measurement (no reference counterpart: the reference has wall timers only,
 * pngf-opt/acmetime.hpp:21-50) ---- */

/* Device time of the hot-path kernels, measured with CUDA events recorded on
 * the handle's stream around each launch group, and the algorithmic work
 * those launches did. */
typedef struct pngf_timing {
  double eval_ms;       /* edge lists + candidate kernel + score */
  long eval_launches;   /* candidate-kernel launches */
  double eval_cf;       /* candidate x frequency evaluations */
  double eval_bytes;    /* algorithmic gather bytes: per (cand, freq) s_M k^2 + 16 (E+2) k + 16 E */
  double eval_flop;     /* algorithmic FP64 flops: per (cand, freq) 8/3 k^3 + 8 k^2 (2 + ...) */
  double accept_ms;     /* whole accept step (factor, W solve, gather, update) */
  long accepts;         /* accept steps (one per frequency) */
  double update_ms;     /* rank-k update kernel alone */
  long update_launches;
  double update_flop;   /* 8 k (N+E)(N+1) per update */
  double update_bytes;  /* 2 s_M (N+E)(N+1) + 16 k ((N+E) + (N+1)) per update */
  long kernel_launches; /* every kernel this handle launched while timing was on */
  double h2d_bytes;     /* host-to-device bytes of candidate batches */
  double d2h_bytes;     /* device-to-host bytes of batch results */
} pngf_timing;

/* Turns event timing on (resets the counters) or off. */
int pngf_timing_enable(pngf_handle *h, int on);
/* Synchronizes the handle's stream and returns the accumulated counters. */
int pngf_timing_get(pngf_handle *h, pngf_timing *out);

/* Bounds-checked build (no reference counterpart; libpngf_gb300_bc.so, built
 * with python -m pngf_gb300.build --bounds-check): every data-dependent index
 * of the gathers of M, Einc and the state rows is checked against its extent
 * on the device; a violation is recorded and the access skipped, nothing
 * traps. *violations receives the number recorded since the last reset,
 * first[3] (may be NULL) the kind (1 T, 2 y, 3 R, 4 Einc, 5 state row), row
 * and column of one of the first; reset != 0 clears the record. The default
 * build returns PNGF_ERR_UNSUPPORTED. */
int pngf_bounds_check_report(long long *violations, long long *first, int reset);

/* ---- autotuning (no reference counterpart) ---- */

#define PNGF_TUNE_MAX 8
/* Forms of the candidate kernel: warps that work on one (candidate, frequency)
 * and candidates per CTA. Warp-per-candidate forms (1 warp) apply when a
 * candidate flips at most 32 edges. All forms return bit-identical results. */
typedef struct pngf_tune {
  int eval_form;                     /* chosen form */
  int eval_forms;                    /* forms listed below */
  int warps_per_cand[PNGF_TUNE_MAX];
  int cands_per_cta[PNGF_TUNE_MAX];
  double eval_us[PNGF_TUNE_MAX];     /* device time of one batch; -1 = form does not apply */
  int batch;                         /* candidates in the timed batch (every tile once) */
  int update_form;                   /* chosen complex64 update tile form for accepts (entry 0 or 1) */
  int update_forms;                  /* complex64: 4 entries, the two tile widths timed at the accept rank
                                        (min(k_max, 24)), then at the build chunk's rank (96); the widths
                                        chosen for each rank class are kept by the handle */
  int update_cols[PNGF_TUNE_MAX];    /* FP32 output columns per update tile */
  double update_us[PNGF_TUNE_MAX];   /* device time of one rank-update; -1 = not timed */
  int eval_form_small;               /* chosen candidate-kernel form for batches of at most 64 candidates */
  int batch_small;                   /* candidates in the small timed batch (the first 64 of the pass) */
  double eval_us_small[PNGF_TUNE_MAX]; /* device time of the small batch per form; -1 = form does not apply */
} pngf_tune;
/* Times every applicable form of the candidate kernel on a pass over every
 * tile and on the first 64 candidates of it (and, for PNGF_PREC_C64, the
 * update forms), keeps the fastest for each batch class for this handle and
 * reports the times. Call after pngf_prepare; the last evaluated batch is
 * discarded and M is left unchanged. */
int pngf_autotune(pngf_handle *h, pngf_tune *out);
/* Selects a candidate-kernel form by index for every batch size
 * (PNGF_ERR_UNSUPPORTED if it does not apply to this handle). */
int pngf_set_eval_form(pngf_handle *h, int form);
/* Failure test hook: records `code` in the handle's tensor-core error flag as
 * if an accept update's bounded wait had given up, without any device wait.
 * The next call that reads the flag (the next evaluation, or the device
 * loop's next decision) fails with PNGF_ERR_TIMEOUT and clears it. */
int pngf_inject_update_timeout(pngf_handle *h, int code);

/* ---- DBS driver (host, native): pngf-opt/main.cpp:181-459 ---- */

#define PNGF_DBS_SYMMETRIC 0 /* 4-fold mirror quarter hat, main.cpp:181, 343-392 */
#define PNGF_DBS_SINGLE 1    /* one tile per candidate over the whole map */
#define PNGF_INIT_EMPTY 0    /* main.cpp:107 */
#define PNGF_INIT_RANDOM 1   /* main.cpp:108, 187-208 */

typedef struct pngf_dbs_params {
  int mode;       /* PNGF_DBS_SYMMETRIC / PNGF_DBS_SINGLE */
  int init;       /* PNGF_INIT_EMPTY / PNGF_INIT_RANDOM */
  int seed;       /* MagicHat rng_seed (magichat.hpp:53-75); 0 is rejected */
  int run_index;
  long max_evals; /* stop after this many evaluations; 0 = run to convergence */
  int batch;      /* speculative candidates per launch: > 0 fixed; 0 = the whole remaining hat; < 0 adaptive,
                     -batch draws after an accept, doubling after each batch without an accept */
  int drift_every;   /* PNGF_PREC_C64: drift check every this many accepts (0 = never) */
  double drift_tol;  /* ... and rebuild M from G when the drift exceeds this (in complex64 for a
                        PNGF_BUILD_C64 handle, else in FP64) */
} pngf_dbs_params;

typedef struct pngf_dbs pngf_dbs;

typedef struct pngf_dbs_stats {
  long evals;          /* flip evaluations in reference order (main.cpp flip_count) */
  long accepts;
  long launched;       /* candidates evaluated on the GPU, speculative included */
  int converged;       /* hat ran out with no improving flip */
  double F_init, F_best;
  long drift_checks;   /* drift checks run */
  long refreshes;      /* rebuilds of M from G after a drift check */
  double drift_max;    /* largest drift seen, max |T_c64 - T| / max |T| */
  long prop_hits;      /* proposal steps whose top-k batch held an improving flip */
  long full_passes;    /* proposal steps that fell back to a full exact pass */
  long device_launches;   /* launches of the device-resident decision loop */
  long device_decisions;  /* decisions it took (each a batch evaluated and decided on the GPU) */
} pngf_dbs_stats;

/* Draws the initial design (rand_binary per tile, main.cpp:187-208), forces
 * the port tiles (main.cpp:215-219), sets the source port at the map centre
 * (main.cpp:241) and prepares every frequency. G must be loaded. */
int pngf_dbs_begin(pngf_handle *h, const pngf_dbs_params *p, pngf_dbs **out);
/* One DBS decision: evaluate draws in hat order until the first improving
 * flip (accepting it, main.cpp:429-456) or until the hat is empty. The
 * accept's launches are queued on the handle's stream and not waited for; a
 * tensor-core update that gave up waiting is reported (PNGF_ERR_TIMEOUT) by
 * the next step. */
int pngf_dbs_step(pngf_dbs *d, int *accepted);
/* Device-resident decisions (no reference counterpart): the hat's random
 * stream (std::mt19937 with std::uniform_int_distribution, restated for the
 * device and checked here against this C++ library's) lives on the GPU, and
 * one CUDA graph with a WHILE node draws, evaluates and decides batch after
 * batch without returning to the host until an accept, the end of the run,
 * or 1024 decisions; accepts then run on the host path. Flips, objectives and
 * log equal those of the host driver. Call before the first pngf_dbs_step;
 * not with learned proposals or in a group. enable = 0 turns it off again
 * (before the first step). PNGF_ERR_UNSUPPORTED when the library's stream
 * differs from the restatement. */
int pngf_dbs_set_device_loop(pngf_dbs *d, int enable);
int pngf_dbs_stats_get(const pngf_dbs *d, pngf_dbs_stats *out);
/* Log of every evaluation in reference order (Logger::record_flip,
 * logger.hpp:64-73): tile index tx+ty*tiles_x, accept bit, F, F_best and per
 * frequency (Re S11, Im S11, D). Arrays sized by the caller for `cap` rows;
 * returns the number of rows in *rows. Any pointer may be NULL. */
int pngf_dbs_log(const pngf_dbs *d, long cap, int *tile, int *accept, double *F, double *F_best,
                 double *perf, long *rows);
/* Writes the log in Logger::save's text format (logger.hpp:75-106). */
int pngf_dbs_save_log(const pngf_dbs *d, const char *path);
int pngf_dbs_end(pngf_dbs *d);

/* ---- many DBS runs at once (no reference counterpart: the reference runs
 * one design per process) ----
 * A group steps independent DBS runs, each on its own handle (so its own
 * stream and device state; sizes may differ), so that their batches and
 * accepts overlap on the GPU. One pngf_group_step draws every unfinished
 * member's next speculative batch and launches all their evaluations, as one
 * CUDA graph when use_graphs is set (captured once and replayed while every
 * member's batch size stays the same; a fixed pngf_dbs_params.batch keeps it
 * so), then takes each member's decision exactly as pngf_dbs_step would and
 * launches its accept without waiting. Each member's accepted flips,
 * objectives and log equal those of stepping it alone with pngf_dbs_step.
 * Members with an attached proposal network are refused.
 * If the members run device-resident decisions (pngf_dbs_set_device_loop,
 * all of them or none), the group holds one CUDA graph whose root nodes are
 * the members' decision loops (each a WHILE node: draw, evaluate, decide on
 * the device), captured once and rebuilt only when a member's buffers or
 * kernel forms change; one pngf_group_step launches it, every unfinished
 * member decides on the device until its next accept, and the group then
 * performs those accepts on the members' streams without waiting. */
typedef struct pngf_group pngf_group;
typedef struct pngf_group_stats {
  long rounds;          /* group steps that launched work */
  long graph_launches;  /* CUDA graph launches (use_graphs) */
  long captures;        /* graph (re)captures */
  long kernel_launches; /* kernels launched by group steps (graph kernels counted per replay) */
  long evals;           /* flip evaluations over all members */
  long accepts;         /* accepts taken in group steps */
} pngf_group_stats;
int pngf_group_create(pngf_dbs *const *members, int count, int use_graphs, pngf_group **out);
/* One round over the members; *active = members not finished afterwards. */
int pngf_group_step(pngf_group *g, int *active);
int pngf_group_stats_get(const pngf_group *g, pngf_group_stats *out);
/* Frees the group (not its members). */
int pngf_group_destroy(pngf_group *g);

/* ---- learned proposals (no reference counterpart) ----
 * A 4-layer 3x3 convolutional network over the tile map (3 input channels:
 * tile state, per-tile Woodbury sensitivity log mean |T_ee|, last exact gain;
 * C channels; BF16 weights, FP32 accumulation; hand-written forward, backward
 * and Adam kernels) predicts each single-tile flip's objective change. The
 * DBS driver uses it to order exact evaluations; every proposal is evaluated
 * exactly, and a full exact pass is the fallback. */
typedef struct pngf_prop pngf_prop;

int pngf_prop_create(pngf_handle *h, int channels, unsigned long long seed, pngf_prop **out);
int pngf_prop_destroy(pngf_prop *p);
long pngf_prop_num_params(const pngf_prop *p);
/* FP32 master parameters, layer by layer: weights (C_out x C_in x 3 x 3) then biases. */
int pngf_prop_get_params(const pngf_prop *p, float *params);
int pngf_prop_set_params(pngf_prop *p, const float *params);
/* Features (3 x tiles_y x tiles_x) of the handle's current design. */
int pngf_prop_features(pngf_prop *p, float *feat);
/* Records exact objective changes of single-tile flips at the current design
 * as one training sample (non-finite gains are skipped). */
int pngf_prop_record(pngf_prop *p, const int *tiles, const double *gains, int count);
long pngf_prop_num_samples(const pngf_prop *p);
/* Adam on random minibatches of recorded samples (masked mean squared error). */
int pngf_prop_train(pngf_prop *p, int steps, int batch, float lr, float *loss);
/* Predicted change (in gain-scale units) per tile; non-candidate tiles +inf. */
int pngf_prop_predict(pngf_prop *p, float *pred);
/* Forward + backward on given inputs (B x 3 x H x W), targets and masks
 * (B x H x W): output, mean masked squared error and parameter gradients. */
int pngf_prop_forward_backward(pngf_prop *p, const float *x, int B, const float *target, const float *mask,
                               float *out, float *grad, float *loss);
const char *pngf_prop_last_error(const pngf_prop *p);
/* Attaches a network to a single-tile DBS run. topk = 0: plain DBS that
 * records every exact evaluation as training data. topk > 0: each step
 * evaluates the top-k predicted flips exactly and accepts the best improving
 * one, else runs a full exact pass; every train_every steps, train_steps Adam
 * steps (batch train_batch, learning rate lr) on the recorded samples. */
int pngf_dbs_set_proposal(pngf_dbs *d, pngf_prop *p, int topk, int train_every, int train_steps, int train_batch,
                          float lr);
/* Which improving flip of an exactly evaluated proposal batch is accepted:
 * PNGF_PROP_BEST (default) the largest improvement, PNGF_PROP_FIRST the first
 * improving flip in the network's predicted order (a less greedy descent). */
#define PNGF_PROP_BEST 0
#define PNGF_PROP_FIRST 1
int pngf_dbs_set_proposal_rule(pngf_dbs *d, int rule);

#ifdef __cplusplus
}
#endif
#endif
