// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/pngf_gb300.h"
#include "hat_rng.h"

namespace pngf {

// NVTX range over a host call (tracing; no cost without a tool attached).
struct TraceRange {
  explicit TraceRange(const char *name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange &) = delete;
  TraceRange &operator=(const TraceRange &) = delete;
};

// Largest capacitance matrix a launch handles (edges flipped at once). The
// candidate kernel keeps K (kmax^2 complex128) in shared memory.
constexpr int kMaxK = 192;
// Largest k the candidate kernel supports (K must fit in shared memory).
constexpr int kMaxEvalK = 104;
// Edges accepted per chunk when M is built from G for a design.
constexpr int kInitChunk = 96;
// Edges per chunk when a complex64 state is built directly in complex64: the
// factor and W solve cost O(k^3) and O(k^2 N) in FP64, the tensor-core update
// O(1) passes over T, so mid-sized chunks are cheapest.
constexpr int kC64BuildChunk = 96;
// Largest pending rank of deferred complex64 updates.
constexpr int kMaxDeferRank = 256;
constexpr int kSmallBatch = 64;  // candidate batches up to this size use the small-batch kernel form
constexpr int kAccTuneRank = 24;  // updates of rank <= this use c64_cols, larger ones c64_cols_build

// Forms of the candidate kernel the autotuner chooses from: warps working on
// one (candidate, frequency) and candidates per CTA. Index 0 is the default.
struct EvalForm {
  int warps_per_cand, cands_per_cta;
};
constexpr int kEvalVariants = 6;
constexpr EvalForm kEvalForms[kEvalVariants] = {{4, 1}, {2, 1}, {8, 1}, {1, 2}, {1, 4}, {1, 8}};

// Batch gate of the edge-list and candidate kernels. With nc set, the batch
// size is read from *nc on the device (the launch grid covers the largest
// batch) and the launch does nothing unless lo < *nc <= hi: a CUDA graph can
// then replay one launch per kernel form for whatever batch the device drew.
struct Gate {
  const int *nc = nullptr;
  int lo = 0, hi = 0;
#ifdef __CUDACC__
  __device__ __forceinline__ bool open(int *ncand) const {
    if (!nc) return true;
    const int n = *nc;
    if (n <= lo || n > hi) return false;
    *ncand = n;
    return true;
  }
#endif
};

struct FreqConst {   // per-frequency scalars used by the objective
  double2 vinc, ln1, ln2;
  double k0;
  double pad;
};

struct Freq {
  double2 *G = nullptr;      // N x N column-major, as loaded (kept for refresh / drift check)
  double2 *gobj = nullptr;   // (E-1) x N row-major objective rows from the file
  double2 *Einc = nullptr;   // N
  double2 *M64 = nullptr;    // (N+E) x ldm row-major: the FP64 state (C64 mode: build staging)
  float2 *T32 = nullptr;     // C64 mode: T (N x ldm row-major, complex64)
  double2 *y64 = nullptr;    // C64 mode: y (N) in FP64
  double2 *R64 = nullptr;    // C64 mode: R and Eobj (E x ldm row-major, Eobj at column N) in FP64
  bool loaded = false;
  float2 *U = nullptr;       // C64 with deferred updates: pending factors, N x defer_cap each
  float2 *Vt = nullptr;      //   (T_true = T32 - U Vt^T over the first defer_rp columns)
  bool synth = false;        // G is the built-in synthetic G (generated on the device)
  unsigned long long synth_seed = 0;
  double synth_eps = 1.0;
};

// Accept scratch and stream of one frequency ("lane"). The frequencies of an
// accept, and of a design build, are independent: with one lane per frequency
// they run on their own streams and overlap on the GPU. A state_only handle
// has a single lane on the handle's stream (its frequencies run in turn).
struct Lane {
  cudaStream_t stream = nullptr;  // own stream (several lanes only)
  cudaEvent_t done = nullptr;
  cudaEvent_t upd = nullptr;      // after this lane's last persistent update (several lanes only)
  double2 *A = nullptr;           // (N+E) x acc_cap, column-major (ld = N+E)
  double2 *W = nullptr;           // acc_cap x ldm row-major
  double2 *LU = nullptr;          // acc_cap^2
  double2 *V = nullptr;           // acc_cap^2: -D K^-1 (column-major), the tensor-core W
  double2 *z = nullptr;           // acc_cap
  int *piv = nullptr;             // acc_cap
  float *Aop = nullptr;           // complex64 update operands: aop_rows x kt_cap fp32, K-major
  float *Bop = nullptr;           // bop_rows x kt_cap
  void *A16 = nullptr, *B16 = nullptr;  // FP64 tensor-core update: bf16 slices, a16_rows x f64tc_op_cols(),
                                        // b16_rows x f64tc_b_cols()
  int *eA = nullptr, *fB = nullptr;     // per-row / per-column power-of-two scales
  double2 *Xs = nullptr;  // rows s of the state as a dense block (acc_cap x ldm): deferred complex64 (T_true), and
                          //   FP64 accepts of more than 32 edges (the W refinement's residual)
  double2 *KD = nullptr;  // FP64 accepts of more than 32 edges: K D (acc_cap^2, column-major)
};

struct Handle {
  pngf_config cfg{};
  long n = 0;        // design edges
  int E = 3;
  long ldm = 0;      // leading dimension of M (elements)
  int map_sz = 0;
  int ex_xsz = 0, ex_ysz = 0, ey_xsz = 0, ey_ysz = 0;
  long nx = 0;       // number of Ex edges
  int kmax = 0;      // most edges one candidate flips
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::vector<Freq> f;
  FreqConst *d_fconst = nullptr;
  void *d_views = nullptr;     // device array of per-frequency state views (kernels_fp64.cu)
  int *d_iota = nullptr;       // 0, 1, ..., acc_cap - 1 (row indices of a dense block; deferred complex64)
  void **d_Eincs = nullptr;    // device array of per-frequency Einc pointers
  // per-frequency accept scratch and streams
  std::vector<Lane> lanes;
  cudaEvent_t ev_fork = nullptr;
  // tensor-core update operand shapes (kernels_c64.cu, kernels_f64tc.cu)
  int kt_cap = 0;
  long aop_rows = 0, bop_rows = 0;
  int *d_tc_err = nullptr;     // set by bounded waits in the tensor-core kernels
  long a16_rows = 0, b16_rows = 0;
  bool f64tc = false;                       // FP64 updates on tensor cores (pieces of f64tc_max_k() edges)
  int init_chunk = kInitChunk;
  int eval_variant = 0;                     // index into kEvalForms (set by the autotuner)
  int eval_variant_small = -1;              // the same for batches of at most kSmallBatch candidates (-1: eval_variant)
  int c64_cols = 128;                       // output tile width of the complex64 update (64 or 128)
  int c64_cols_build = 128;                 // the same for ranks above kAccTuneRank (build chunks, flushes)
  int defer_cap = 0;                        // C64: pending rank at which deferred updates are flushed (0 = off)
  int defer_rp = 0;                         //   rank pending now (same at every frequency)
  bool defer_now = false;                   //   accepts being launched are deferred (DBS accepts, not builds)
  bool defer_flush = false;                 //   the accept being launched flushes after appending
  std::vector<FreqConst> h_fconst;

  // design
  std::vector<int> tile_map;
  std::vector<signed char> P;
  std::vector<long> port;
  int *d_tile_map = nullptr;
  signed char *d_P = nullptr;
  bool have_map = false, have_port = false, prepared = false;

  // candidate batch
  int cand_cap = 0;
  int *d_tiles = nullptr, *d_nflip = nullptr;   // ncand x max_flips, ncand
  int *d_es = nullptr;                          // ncand x kmax edge indices
  signed char *d_ed = nullptr;                  // ncand x kmax signs
  int *d_ek = nullptr;                          // ncand
  double2 *d_new_eobj = nullptr;                // ncand x nf x E
  double *d_Ff = nullptr;                       // ncand x nf
  double *d_perf = nullptr;                     // ncand x nf x 3 (Re S11, Im S11, D)
  double *d_F = nullptr;                        // ncand
  int *d_first = nullptr;
  int *d_status = nullptr;                      // per-candidate LU status
  double2 *d_eval_LU = nullptr;                 // ncand x nf x kmax^2: each candidate's factored K (for its accept)
  int *d_eval_piv = nullptr;                    // ncand x nf x kmax
  double2 *d_eval_z = nullptr;                  // ncand x nf x kmax
  int acc_cand = -1;                            // candidate of the evaluated batch being accepted, else -1
  bool building = false;                        // inside a build of the state (prepare / refresh)
  int batch_n = 0;
  int launched_n = 0;      // batch enqueued by eval_launch, not yet collected
  int staged_n = 0;        // batch staged by eval_stage
  bool capturing = false;  // stream work is being captured into a CUDA graph (no timing events)
  double *h_fbest = nullptr, *d_fbest = nullptr;  // F_best of the staged batch (pinned / device)
  bool batch_valid = false;
  std::vector<int> batch_tiles, batch_nflip;
  std::vector<int> last_k, last_status;   // per-candidate edge count / status of the host-API batch

  // accept
  int acc_cap = 0;                  // columns of A / rows of W in each lane
  int *d_acc_s = nullptr;            // explicit edge list (init chunks)
  signed char *d_acc_d = nullptr;
  int *d_acc_status = nullptr;      // sticky: PNGF_ERR_SINGULAR from any lane
  unsigned long long *d_colmax = nullptr;  // N words of scratch for the synthetic G generator

  // host staging (pinned)
  int *h_tiles = nullptr, *h_nflip = nullptr;
  double *h_out = nullptr;
  size_t h_out_cap = 0;

  // measurement
  bool timing = false;
  pngf_timing tacc{};
  struct Pending {
    cudaEvent_t a, b;
    int cat;
    double x1, x2, x3;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> ev_pool;
  long nlaunch = 0;
  long state_version = 0;  // bumped whenever the stored state or the design changes (accept, build, flush)

  std::string err;
};

// The lane of frequency f and the stream its work goes to.
inline Lane &lane_of(Handle *h, int f) { return h->lanes[(size_t)f % h->lanes.size()]; }
inline cudaStream_t lane_stream(const Handle *h, int f) {
  return h->lanes.size() < 2 ? h->stream : h->lanes[(size_t)f % h->lanes.size()].stream;
}

// Timing categories.
enum { T_EVAL = 0, T_ACCEPT = 1, T_UPDATE = 2 };
// Records an event on stream s (the handle's stream when null) if timing is
// on (else nullptr).
cudaEvent_t timing_mark(Handle *h, cudaStream_t s = nullptr);
// Closes a span opened by timing_mark on the same stream: category and
// algorithmic work (T_EVAL: cand x freq, bytes, flops; T_ACCEPT: frequencies;
// T_UPDATE: flops, bytes).
void timing_close(Handle *h, cudaEvent_t start, int cat, double x1, double x2, double x3, cudaStream_t s = nullptr);

int set_error(Handle *h, int code, const std::string &msg);
int cuda_check(Handle *h, cudaError_t e, const char *what);
// Returns the library status of a failed CUDA call from the enclosing function.
#define PNGF_CUDA(h, call)                          \
  do {                                              \
    const int _rc = cuda_check((h), (call), #call); \
    if (_rc != PNGF_OK) return _rc;                 \
  } while (0)

// Host copy of one evaluated batch.
struct EvalOut {
  std::vector<double> F;         // ncand
  std::vector<double> perf;      // ncand x nf x 3
  std::vector<double> new_eobj;  // ncand x nf x E x 2
  std::vector<int> k;            // flipped-edge count per candidate (-1 = invalid)
  std::vector<int> status;       // ncand x nf
  int first = -1;                // first candidate with F < F_best
};
// Evaluates a batch of host tile lists (validated) and reads the results back.
int eval_batch(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best, EvalOut *out);
// The same in two phases: enqueue the batch and its result copies on the
// handle's stream, then wait for them and parse.
int eval_launch(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best);
int eval_collect(Handle *h, EvalOut *out);
// eval_launch split again: eval_stage validates the batch and copies it (and
// F_best) into pinned host staging; eval_enqueue issues the stream work
// (host-to-device copies from the staging, kernels, result copies), which a
// CUDA graph can capture and replay after a new eval_stage of the same size.
int eval_stage(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best);
int eval_enqueue(Handle *h);
// Applies candidate c (k flipped edges) of the last batch at every frequency.
int accept_cand(Handle *h, int c, int k);
// Same; with check_now = false nothing waits for the GPU (the tensor-core
// error flag is then reported by the next eval_collect).
int accept_cand_async(Handle *h, int c, int k, bool check_now);

// Makes room for batches of ncand candidates (device buffers only).
int reserve_candidates(Handle *h, int ncand);
// Marks the batch the device-resident loop evaluated (ncand candidates, left
// in the handle's device buffers) as the evaluated batch, so that candidate
// c (its tiles given for the host copy of the design) can be accepted.
int adopt_device_batch(Handle *h, int ncand, int c, const int *tiles_c, int nflip_c);

// ---- device-resident DBS decisions (dbs_device.cu) ----
struct DevLoopConfig {
  HatGeom geo;
  int hat_entries;
  int batch;             // pngf_dbs_params.batch
  long long max_evals;   // 0 = no budget
  unsigned seed;         // MagicHat seed
  long engine_used;      // engine outputs pngf_dbs_begin consumed (rand_binary)
  double F_best;
};
struct DevLoopResult {
  long long evals, accepts, launched;
  double F_best;
  int converged, done;
  int err;      // 1: an invalid candidate; 2: a tensor-core accept update gave up waiting (tc_code)
  int tc_code;
  int accepted, nc, j, k, nflip, tiles[4];  // the accept the host is to perform
  int decisions;                             // decisions taken by this launch
};
struct DevLoopLog {  // rows appended by devloop_run
  std::vector<int> &tile, &acc;
  std::vector<double> &F, &Fb, &perf;
};
struct DevLoop;
int devloop_create(Handle *h, const DevLoopConfig &cfg, DevLoop **out);
// Runs decisions on the device until an accept, the end of the run or a
// launch limit; appends the log rows and reports the state.
int devloop_run(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log);
// Many loops in one graph (groups): adds this loop's WHILE node to `graph`
// (its own launch graph is kept); devloop_prepare queues the per-launch reset
// on the handle's stream, and after `graph` has run devloop_collect reads
// the report as devloop_run does. devloop_key_current is false when the
// handle's buffers or kernel forms changed since the loop was captured.
int devloop_add_to_graph(Handle *h, DevLoop *L, cudaGraph_t graph);
int devloop_prepare(Handle *h, DevLoop *L);
int devloop_collect(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log);
int devloop_read(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log, size_t span1);
bool devloop_key_current(const Handle *h, const DevLoop *L);
// New F_best after the host changed it (drift refresh).
int devloop_set_fbest(Handle *h, DevLoop *L, double F_best);
void devloop_destroy(DevLoop *L);

// ---- kernels (kernels_fp64.cu) ----
// Builds M for P = 0 from G and the objective rows; computes Einc and the
// port constants (on the frequency's lane stream).
cudaError_t launch_init_M(Handle *h, int f);
// Per-candidate flipped-edge lists (sorted, deduplicated) from tile lists.
cudaError_t launch_edge_lists(Handle *h, int ncand, const int *d_tiles, const int *d_nflip, Gate gt = Gate{});
// Candidate evaluation + objective at every frequency, then the score
// against F_best (read from d_fbest when it is not null).
cudaError_t launch_eval(Handle *h, int ncand, double F_best, const double *d_fbest = nullptr);
// The candidate kernel alone in form kEvalForms[form], gated (no score).
cudaError_t launch_eval_form(Handle *h, int form, int ncand, Gate gt);
// Whether kEvalForms[v] applies to the handle (warp forms need kmax <= 32).
bool eval_variant_ok(const Handle *h, int v);
// Objective of the current design (from M's Eobj entries) into d_F[0].
cudaError_t launch_current_objective(Handle *h);
// Rank-k accept of an explicit edge list (device arrays s, d of length k) at
// frequency f, on the FP64 layout (M64) or the complex64 layout (layout =
// PNGF_PREC_C64: T32 on tensor cores, y64 / R64 in FP64), with the
// frequency's lane scratch, on its lane stream.
cudaError_t launch_accept_edges(Handle *h, int f, const int *d_s, const signed char *d_d, int k, int layout);
// Writes h->defer_rp into the device copies of the complex64 views (stream-ordered).
cudaError_t launch_set_pending_rank(Handle *h);
// Uploads the per-frequency state views for the handle's precision.
cudaError_t setup_views(Handle *h);
size_t view_bytes();
// ---- complex64 form (kernels_c64.cu) ----
// Splits the FP64 M of frequency f into T32 (complex64), y64 and R64 (on the
// frequency's lane stream).
cudaError_t launch_split_M(Handle *h, int f);
// After the accept prologue (A, W in FP64 in the frequency's lane): updates
// y64 and R64 in FP64 and T32 -= A W on the tensor cores (3xTF32 split
// products), on the lane's stream.
cudaError_t launch_c64_update(Handle *h, int f, int k);
// Deferred form of the update: y64 and R64 updated in FP64 now, the T part
// appended to the pending factors (U gets A's T rows, Vt gets W's T columns,
// in complex64); with h->defer_flush the pending rank-(defer_rp + k) product
// is then subtracted from T32 on the tensor cores.
cudaError_t launch_c64_defer(Handle *h, int f, int k);
// Subtracts the pending product U Vt^T (rank h->defer_rp) from T32 of frequency f.
cudaError_t launch_c64_flush(Handle *h, int f);
// Reassembles frequency f's M in FP64 (into M64) from T32, y64, R64.
cudaError_t launch_merge_M(Handle *h, int f);
// FP64 rows of T for the current design at rows d_rows (nr <= 8) by iterative
// refinement from T32 against G; d_out[0..1] receive (as double bits, atomic
// max) max |T32 - T| and max |T| over those rows. d_P: the set edges (np).
cudaError_t launch_drift_rows(Handle *h, int f, const int *d_rows, int nr, const int *d_P, int np, double2 *X,
                              double2 *PH, double2 *Rk, unsigned long long *d_out);
// ---- synthetic G on the device (synth.cu) ----
// Writes frequency f's synthetic G (n x n column-major, leading dimension ldg);
// colmax: n scratch words.
cudaError_t launch_synth_G(Handle *h, int f, double2 *G, long ldg, unsigned long long *colmax);
// Writes frequency f's synthetic NF2FF rows ((E-1) x n row-major) into rows.
cudaError_t launch_synth_gobj(Handle *h, int f, double2 *rows);
// Amplitude of the synthetic NF2FF rows: kappa eta0 dx dy dz with kappa = 32,
// the broadside far-field weight of one edge's current (see pngf_synth_gobj).
inline double synth_gobj_amplitude(double dx, double dy, double dz) {
  return 32.0 * 3.767303134118051e02 * dx * dy * dz;
}
// ---- FP64-accurate update on the tensor cores (kernels_f64tc.cu) ----
int f64tc_max_k();
size_t f64tc_op_cols();  // row pitch of the A slices (elements)
size_t f64tc_b_cols();   // row pitch of the B slices (elements)
long f64tc_b_rows(long n);  // rows of the B slices: 7 per output column, 32-column tiles stacked
// M -= A W for M ((N+E) x ldm complex128), A ((N+E) x k column-major), W (k x ldm),
// with frequency f's lane scratch and stream.
// Grid of a persistent update kernel (one CTA per SM) over ntiles tiles:
// during a build with several frequency lanes it leaves kReservedSMs SMs
// free, so that the other lanes' single-CTA capacitance LUs run beside it
// instead of waiting for it to end (an accept of an evaluated candidate has
// no LU to run: it starts from the evaluation's).
constexpr int kReservedSMs = 8;
inline int persistent_grid(const Handle *h, int ntiles, int nsm) {
  const int g = h->building && h->lanes.size() > 1 && nsm > 2 * kReservedSMs ? nsm - kReservedSMs : nsm;
  return ntiles < g ? ntiles : g;
}
// The frequency lanes' persistent M updates run one after another (each
// fills every SM and is HBM-bound, so running them side by side only makes
// them share the memory system, while their tiles' pipelines lose depth):
// before its update, lane f's stream waits for lane f-1's last update; the
// lanes' other kernels (factor, W, operand slicing) still overlap them.
// Design builds (h->building) keep the lanes' updates concurrent.
cudaError_t chain_update_wait(Handle *h, int f, cudaStream_t st);
cudaError_t chain_update_done(Handle *h, int f, cudaStream_t st);
cudaError_t launch_f64tc_update(Handle *h, int f, int k, double2 *M, const double2 *A, const double2 *W);
// W[:, 0:N] -= Vneg X[s, 0:N] on the tensor cores (FP64-accurate): Vneg k x k
// column-major, X rows s of the state (complex64 when x32, pitch ldx).
cudaError_t launch_f64tc_wgemm(Handle *h, int f, int k, const double2 *Vneg, const void *X, bool x32, long ldx,
                               const int *d_s, double2 *W);
// D[0:drows, 0:ncols) -= A B on the tensor cores (FP64-accurate), complex:
// A drows x k column-major (lda), B k x ncols row-major (ldb), D row-major
// (pitch ldd complex); the inner dimension in pieces of f64tc_max_k().
cudaError_t launch_f64tc_small(Handle *h, int f, int k, double2 *D, long drows, long ncols, long ldd,
                               const double2 *A, long lda, const double2 *B, long ldb);
// Commits P and the tile map on the device for candidate c of the batch.
cudaError_t launch_commit(Handle *h, int c);
// The accept kernels on caller-supplied buffers (no handle): scratch LU (k^2),
// piv (k), z (k), A ((n+E) x k), W (k x ldm), status (1, zero on entry). The
// factor kernel checks the edge list (indices in [0, n), signs +-1) and sets
// *status to PNGF_ERR_ARG, or to PNGF_ERR_SINGULAR for a singular K; the W,
// gather and update kernels then return without touching M.
cudaError_t launch_accept_raw(double2 *M, long ldm, long n, int E, const double2 *Einc, const int *d_s,
                              const signed char *d_d, int k, double2 *LU, int *piv, double2 *z, double2 *A,
                              double2 *W, int *status, cudaStream_t stream);

}  // namespace pngf
