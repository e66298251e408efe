// Device-resident DBS decisions (no reference counterpart; the decisions are
// those of pngf-opt/main.cpp:343-456).
//
// The host driver (dbs.cpp) draws each speculative batch on the CPU, reads
// its objectives back and decides there: one host round trip per decision.
// Here the MagicHat state lives in device memory and a CUDA graph with a
// WHILE conditional node repeats one decision per iteration:
//
//   k_dbs_draw     one thread draws the batch in hat order (MagicHat draws,
//                  skip rules and mirror images, hat_rng.h) into the
//                  candidate buffers; the batch size is the host driver's
//                  policy (fixed, whole hat or adaptive);
//   k_edge_lists,  the candidate kernels in the autotuned forms, gated on the
//   candidate      batch size the device drew (one launch per form: small
//   kernel(s)      batches and large ones);
//   k_dbs_decide   sums F over the frequencies in order, takes the first draw
//                  with F < F_best (the reference's accept, in draw order),
//                  appends the log rows and, on an accept, restores the
//                  engine to the start of the batch and replays it to just
//                  after the accepted draw (the hat is then refilled, as
//                  main.cpp:455 does). It sets the loop condition.
//
// The loop ends on an accept, when the run is over (hat exhausted or
// evaluation budget spent), when the device log is nearly full or after a
// set number of decisions; the host then reads the log and performs the
// accept on its usual path (the accept's kernel shapes depend on the flip's
// edge count). Runs of decisions without an accept -- most of them near
// convergence -- thus cost no host round trip. The flip sequence, objectives
// and log equal the host driver's.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <new>

#include "hat_rng.h"
#include "pngf_internal.h"

namespace pngf {

namespace {

struct DevScalars {
  long long evals, accepts, launched;
  double F_best;
  int left, last_tried, adapt_B;
  int nc, exhausted, converged, done, err;
  int iters, log_n, accepted;  // reset by the host before every launch (adjacent)
  int acc_j, acc_k, acc_nflip, acc_tiles[4];
  int tc_code;  // error code a tensor-core accept update left (its bounded waits gave up)
};

struct DevState {
  MtState mt;   // the hat's engine
  MtState mt0;  // the engine at the start of the batch being evaluated
};

// The report the host reads after a launch, one contiguous buffer: the
// scalars, then one record per logged evaluation (int tile, int accept,
// double F, double F_best, double perf[3 nf]), so that a launch's state and
// its first rows come back in one copy.
constexpr int kReportHead = 256;
static_assert(sizeof(DevScalars) <= kReportHead, "report head");
__host__ __device__ constexpr int log_rec_bytes(int nf) { return 24 + 24 * nf; }

struct DevConst {
  HatGeom geo;
  int hat_entries, batch, max_flips, nf, log_cap, max_iters;
  long long max_evals;
  const int *tc_err;  // the handle's tensor-core error flag (may be null)
  cudaGraphConditionalHandle cond;
};

constexpr int kLoopThreads = 256;
constexpr int kKeyLen = 8;
constexpr int kReportRows = 64;  // log rows read back with the scalars

__global__ void __launch_bounds__(kLoopThreads)
    k_dbs_draw(DevConst c, DevState *st, DevScalars *vs, int *__restrict__ entry, int *__restrict__ tiles,
               int *__restrict__ nflip, int *__restrict__ logidx, int *__restrict__ used, int *__restrict__ rval) {
  extern __shared__ unsigned char sh[];
  MtState *m = reinterpret_cast<MtState *>(sh);
  int *ent = reinterpret_cast<int *>(sh + sizeof(MtState));
  __shared__ int s_go;
  __shared__ long long s_budget;
  DevScalars &v = *vs;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_go = 0;
    v.nc = 0;
    if (!v.done && !v.err) {
      s_budget = c.max_evals > 0 ? c.max_evals - v.evals : LLONG_MAX;
      if (s_budget <= 0)
        v.done = 1;
      else
        s_go = 1;
    }
  }
  __syncthreads();
  if (!s_go) return;
  for (int i = tid; i < kMtN; i += blockDim.x) {
    m->x[i] = st->mt.x[i];
    st->mt0.x[i] = st->mt.x[i];
  }
  for (int i = tid; i < c.hat_entries; i += blockDim.x) ent[i] = entry[i];
  if (tid == 0) {
    m->i = st->mt.i;
    st->mt0.i = st->mt.i;
  }
  __syncthreads();
  if (tid == 0) {
    // batch > 0: fixed; 0: the whole remaining hat; < 0: adaptive
    if (c.batch < 0 && v.adapt_B <= 0) v.adapt_B = -c.batch;
    long long B = c.batch > 0 ? c.batch : c.batch < 0 ? v.adapt_B : max(1, v.left);
    B = min(B, s_budget);
    int n = 0, cnt = 0, ex = 0, left = v.left, last = v.last_tried;
    while (n < B) {
      const int r = hat_draw(m, ent, &left, &cnt);
      if (r < 0) {
        ex = 1;
        break;
      }
      int li = 0, nfl = 0, t[4] = {0, 0, 0, 0};
      if (!hat_candidate(c.geo, r, &last, &li, &nfl, t)) continue;
      for (int q = 0; q < c.max_flips; ++q) tiles[(size_t)n * c.max_flips + q] = q < nfl ? t[q] : 0;
      nflip[n] = nfl;
      logidx[n] = li;
      used[n] = cnt;
      rval[n] = r;
      ++n;
    }
    v.left = left;
    v.last_tried = last;
    v.nc = n;
    v.exhausted = ex;
    v.launched += n;
    if (n == 0) v.converged = v.done = 1;
  }
  __syncthreads();
  for (int i = tid; i < kMtN; i += blockDim.x) st->mt.x[i] = m->x[i];
  for (int i = tid; i < c.hat_entries; i += blockDim.x) entry[i] = ent[i];
  if (tid == 0) st->mt.i = m->i;
}

__global__ void __launch_bounds__(kLoopThreads)
    k_dbs_decide(DevConst c, DevState *st, DevScalars *vs, int *__restrict__ entry, const double *__restrict__ Ff,
                 double *__restrict__ F, int *__restrict__ first, const int *__restrict__ status,
                 const int *__restrict__ ek, const double *__restrict__ perf, const int *__restrict__ tiles,
                 const int *__restrict__ nflip, const int *__restrict__ logidx, const int *__restrict__ used,
                 const int *__restrict__ rval, unsigned char *__restrict__ logrec) {
  extern __shared__ unsigned char sh[];
  MtState *m = reinterpret_cast<MtState *>(sh);
  __shared__ int s_first, s_bad;
  DevScalars &v = *vs;
  const int tid = threadIdx.x, nc = v.nc, nf = c.nf;
  // an accept update that gave up waiting left M unusable: stop before deciding
  const int tc = c.tc_err ? *c.tc_err : 0;
  if (nc == 0 || tc != 0) {
    if (tid == 0) {
      if (tc != 0) {
        v.err = 2;
        v.tc_code = tc;
      }
      cudaGraphSetConditional(c.cond, 0);
    }
    return;
  }
  // every thread reads what thread 0 updates at the end before the first barrier
  const double Fb = v.F_best;
  const int row0 = v.log_n;
  if (tid == 0) {
    s_first = INT_MAX;
    s_bad = 0;
  }
  __syncthreads();
  for (int i = tid; i < nc; i += blockDim.x) {
    double acc = 0.0;
    for (int f = 0; f < nf; ++f) acc += Ff[(size_t)i * nf + f];
    F[i] = acc;
    if (acc < Fb) atomicMin(&s_first, i);  // a NaN F never passes
  }
  __syncthreads();
  const int j = s_first == INT_MAX ? -1 : s_first;
  const int rows = (j >= 0 ? j : nc - 1) + 1;
  for (int i = tid; i < rows * nf; i += blockDim.x)
    if (status[i] == PNGF_ERR_ARG) s_bad = 1;
  __syncthreads();
  if (s_bad) {
    if (tid == 0) {
      v.err = 1;
      cudaGraphSetConditional(c.cond, 0);
    }
    return;
  }
  const int pw = 3 * nf, rb = log_rec_bytes(nf);
  for (int i = tid; i < rows; i += blockDim.x) {
    unsigned char *r = logrec + (size_t)(row0 + i) * rb;
    reinterpret_cast<int *>(r)[0] = logidx[i];
    reinterpret_cast<int *>(r)[1] = i == j;
    reinterpret_cast<double *>(r)[1] = F[i];
    reinterpret_cast<double *>(r)[2] = Fb;
  }
  for (int x = tid; x < rows * pw; x += blockDim.x) {
    const int i = x / pw;
    reinterpret_cast<double *>(logrec + (size_t)(row0 + i) * rb)[3 + (x - i * pw)] = perf[x];
  }
  if (j >= 0) {
    // back to the start of the batch, then forward over the engine outputs
    // the draws up to and including draw j consumed; the hat is refilled
    for (int i = tid; i < kMtN; i += blockDim.x) m->x[i] = st->mt0.x[i];
    for (int i = tid; i < c.hat_entries; i += blockDim.x) entry[i] = i;
    if (tid == 0) m->i = st->mt0.i;
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < used[j]; ++q) mt_next(m);
    __syncthreads();
    for (int i = tid; i < kMtN; i += blockDim.x) st->mt.x[i] = m->x[i];
  }
  if (tid == 0) {
    *first = j;
    v.log_n += rows;
    v.evals += rows;
    ++v.iters;
    int cont;
    if (j >= 0) {
      st->mt.i = m->i;
      v.F_best = F[j];
      ++v.accepts;
      v.accepted = 1;
      v.acc_j = j;
      v.acc_k = ek[j];
      v.acc_nflip = nflip[j];
      for (int q = 0; q < 4; ++q) v.acc_tiles[q] = q < nflip[j] ? tiles[(size_t)j * c.max_flips + q] : 0;
      v.last_tried = rval[j];
      v.left = c.hat_entries;
      v.adapt_B = -c.batch;
      cont = 0;
    } else {
      if (c.batch < 0) v.adapt_B = (int)min(2LL * v.adapt_B, 1LL << 20);
      if (v.exhausted) v.converged = v.done = 1;
      if (c.max_evals > 0 && v.evals >= c.max_evals) v.done = 1;
      cont = !v.done && v.log_n + c.hat_entries <= c.log_cap && v.iters < c.max_iters;
    }
    cudaGraphSetConditional(c.cond, cont ? 1u : 0u);
  }
}

}  // namespace

struct DevLoop {
  DevConst c{};
  DevState *st = nullptr;
  int *entry = nullptr, *logidx = nullptr, *used = nullptr, *rval = nullptr;
  unsigned char *d_rep = nullptr;  // report: scalars, then log records
  unsigned char *h_rep = nullptr;  // its pinned host copy
  cudaStream_t cap = nullptr;  // capture stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uintptr_t key[kKeyLen] = {};  // handle buffers and kernel forms the graph was captured with
  int per_iter = 0;             // kernels one decision launches
  long long launched_seen = 0;  // candidates launched before the current graph launch
};

namespace {

void graph_release(DevLoop *L) {
  if (L->exec) cudaGraphExecDestroy(L->exec);
  if (L->graph) cudaGraphDestroy(L->graph);
  L->exec = nullptr;
  L->graph = nullptr;
}

void capture_key(const Handle *h, uintptr_t *key) {
  key[0] = reinterpret_cast<uintptr_t>(h->d_tiles);
  key[1] = reinterpret_cast<uintptr_t>(h->d_es);
  key[2] = reinterpret_cast<uintptr_t>(h->d_eval_LU);
  key[3] = reinterpret_cast<uintptr_t>(h->d_views);
  key[4] = reinterpret_cast<uintptr_t>(h->d_Ff);
  key[5] = (uintptr_t)h->cand_cap;
  key[6] = (uintptr_t)(unsigned)h->eval_variant;
  key[7] = (uintptr_t)(unsigned)h->eval_variant_small;
}

size_t draw_smem(const DevLoop *L) { return sizeof(MtState) + sizeof(int) * (size_t)L->c.hat_entries; }

// Adds to `graph` a WHILE node (on its own conditional handle, reset to 1 at
// every launch) whose body is one decision of this loop: draw, edge lists,
// candidate kernel(s), decide. L->c.cond is left at the new handle.
int loop_body_build(Handle *h, DevLoop *L, cudaGraph_t graph) {
  PNGF_CUDA(h, cudaGraphConditionalHandleCreate(&L->c.cond, graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = L->c.cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  PNGF_CUDA(h, cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  const int cap = L->c.hat_entries;
  const int small = std::min(cap, kSmallBatch);
  const int v_small = h->eval_variant_small >= 0 ? h->eval_variant_small : h->eval_variant;
  // the handle's launchers work on h->stream: point it at the capture stream
  cudaStream_t user = h->stream;
  h->stream = L->cap;
  h->capturing = true;
  cudaError_t e = cudaStreamBeginCaptureToGraph(L->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    DevScalars *vs = reinterpret_cast<DevScalars *>(L->d_rep);
    const int *nc = &vs->nc;
    const size_t sm = draw_smem(L);
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_dbs_draw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_dbs_draw<<<1, kLoopThreads, sm, L->cap>>>(L->c, L->st, vs, L->entry, h->d_tiles, h->d_nflip, L->logidx,
                                                L->used, L->rval);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_edge_lists(h, cap, h->d_tiles, h->d_nflip, Gate{nc, 0, INT_MAX});
    if (e == cudaSuccess) e = launch_eval_form(h, v_small, small, Gate{nc, 0, small});
    if (e == cudaSuccess && cap > small) e = launch_eval_form(h, h->eval_variant, cap, Gate{nc, small, INT_MAX});
    L->per_iter = cap > small ? 5 : 4;
    if (e == cudaSuccess) {
      k_dbs_decide<<<1, kLoopThreads, sizeof(MtState), L->cap>>>(
          L->c, L->st, vs, L->entry, h->d_Ff, h->d_F, h->d_first, h->d_status, h->d_ek, h->d_perf, h->d_tiles,
          h->d_nflip, L->logidx, L->used, L->rval, L->d_rep + kReportHead);
      e = cudaGetLastError();
    }
    cudaGraph_t out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(L->cap, &out);
    if (e == cudaSuccess) e = e2;
  }
  h->capturing = false;
  h->stream = user;
  PNGF_CUDA(h, e);
  return PNGF_OK;
}

int graph_build(Handle *h, DevLoop *L) {
  graph_release(L);
  PNGF_CUDA(h, cudaGraphCreate(&L->graph, 0));
  int rc = loop_body_build(h, L, L->graph);
  if (rc) return rc;
  PNGF_CUDA(h, cudaGraphInstantiate(&L->exec, L->graph, 0));
  capture_key(h, L->key);
  return PNGF_OK;
}

}  // namespace

void devloop_destroy(DevLoop *L) {
  if (!L) return;
  graph_release(L);
  if (L->cap) cudaStreamDestroy(L->cap);
  cudaFree(L->st);
  cudaFree(L->entry);
  cudaFree(L->logidx);
  cudaFree(L->used);
  cudaFree(L->rval);
  cudaFree(L->d_rep);
  if (L->h_rep) cudaFreeHost(L->h_rep);
  delete L;
}

int devloop_create(Handle *h, const DevLoopConfig &cfg, DevLoop **out) {
  *out = nullptr;
  int rc = reserve_candidates(h, cfg.hat_entries);
  if (rc) return rc;
  DevLoop *L = new (std::nothrow) DevLoop();
  if (!L) return PNGF_ERR_NOMEM;
  DevConst &c = L->c;
  c.geo = cfg.geo;
  c.hat_entries = cfg.hat_entries;
  c.batch = cfg.batch;
  c.max_flips = h->cfg.max_flips;
  c.nf = h->cfg.num_freq;
  c.log_cap = std::max(8 * cfg.hat_entries, 4096);
  c.max_iters = 1024;
  c.max_evals = cfg.max_evals;
  c.tc_err = h->d_tc_err;
  const size_t lc = (size_t)c.log_cap, ce = (size_t)cfg.hat_entries;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc(reinterpret_cast<void **>(&L->st), sizeof(DevState));
  alloc(reinterpret_cast<void **>(&L->entry), sizeof(int) * ce);
  alloc(reinterpret_cast<void **>(&L->logidx), sizeof(int) * ce);
  alloc(reinterpret_cast<void **>(&L->used), sizeof(int) * ce);
  alloc(reinterpret_cast<void **>(&L->rval), sizeof(int) * ce);
  const size_t rep_bytes = kReportHead + lc * log_rec_bytes(c.nf);
  alloc(reinterpret_cast<void **>(&L->d_rep), rep_bytes);
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void **>(&L->h_rep), rep_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    devloop_destroy(L);
    return cuda_check(h, e, "device DBS loop buffers");
  }
  // the hat as pngf_dbs_begin leaves it: seeded, rand_binary draws consumed, full
  DevState *hs = new (std::nothrow) DevState();
  std::vector<int> ent(ce);
  if (!hs) {
    devloop_destroy(L);
    return PNGF_ERR_NOMEM;
  }
  mt_seed(&hs->mt, cfg.seed);
  for (long i = 0; i < cfg.engine_used; ++i) mt_next(&hs->mt);
  hs->mt0 = hs->mt;
  DevScalars v;
  std::memset(&v, 0, sizeof(v));
  v.F_best = cfg.F_best;
  v.left = cfg.hat_entries;
  v.last_tried = -1;
  for (int i = 0; i < cfg.hat_entries; ++i) ent[i] = i;
  e = cudaMemcpy(L->st, hs, sizeof(DevState), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(L->d_rep, &v, sizeof(v), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(L->entry, ent.data(), sizeof(int) * ce, cudaMemcpyHostToDevice);
  delete hs;
  if (e != cudaSuccess) {
    devloop_destroy(L);
    return cuda_check(h, e, "device DBS loop state");
  }
  if ((rc = graph_build(h, L))) {
    devloop_destroy(L);
    return rc;
  }
  *out = L;
  return PNGF_OK;
}

int devloop_set_fbest(Handle *h, DevLoop *L, double F_best) {
  DevScalars *dv = reinterpret_cast<DevScalars *>(L->d_rep);
  PNGF_CUDA(h, cudaMemcpyAsync(&dv->F_best, &F_best, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  return PNGF_OK;
}

bool devloop_key_current(const Handle *h, const DevLoop *L) {
  uintptr_t key[kKeyLen];
  capture_key(h, key);
  return std::equal(key, key + kKeyLen, L->key);
}

int devloop_add_to_graph(Handle *h, DevLoop *L, cudaGraph_t graph) {
  const cudaGraphConditionalHandle own = L->c.cond;
  const int rc = loop_body_build(h, L, graph);
  L->c.cond = own;  // the loop's own graph keeps its handle
  if (rc == PNGF_OK) capture_key(h, L->key);
  return rc;
}

int devloop_prepare(Handle *h, DevLoop *L) {
  DevScalars *dv = reinterpret_cast<DevScalars *>(L->d_rep);
  PNGF_CUDA(h, cudaMemsetAsync(&dv->iters, 0, 3 * sizeof(int), h->stream));
  return PNGF_OK;
}

int devloop_collect(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log) { return devloop_read(h, L, r, log, 0); }

int devloop_run(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log) {
  pngf::TraceRange trace_("pngf device decisions");
  int rc;
  if (!devloop_key_current(h, L) && (rc = graph_build(h, L))) return rc;
  if ((rc = devloop_prepare(h, L))) return rc;
  // one timing span per launch: the decisions' draws, evaluations and scores
  cudaEvent_t t0 = timing_mark(h);
  PNGF_CUDA(h, cudaGraphLaunch(L->exec, h->stream));
  const size_t span = h->pending.size();
  timing_close(h, t0, T_EVAL, 0.0, 0.0, 0.0);
  return devloop_read(h, L, r, log, span + 1);
}

// Reads a launch's report (the scalars and the first rows in one copy, the
// rest in a second) and appends its log rows; span1 = index + 1 of the
// launch's timing span (0: none).
int devloop_read(Handle *h, DevLoop *L, DevLoopResult *r, DevLoopLog *log, size_t span1) {
  // the scalars and the first rows in one copy; the rest, if any, in a second
  const int rb = log_rec_bytes(L->c.nf);
  const int first_rows = std::min(L->c.log_cap, kReportRows);
  PNGF_CUDA(h, cudaMemcpyAsync(L->h_rep, L->d_rep, kReportHead + (size_t)first_rows * rb, cudaMemcpyDeviceToHost,
                               h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  const DevScalars &v = *reinterpret_cast<const DevScalars *>(L->h_rep);
  if (v.log_n > first_rows) {
    const size_t off = kReportHead + (size_t)first_rows * rb;
    PNGF_CUDA(h, cudaMemcpyAsync(L->h_rep + off, L->d_rep + off, (size_t)(v.log_n - first_rows) * rb,
                                 cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  if (span1 > 0 && h->pending.size() >= span1)
    h->pending[span1 - 1].x1 = (double)(v.launched - L->launched_seen) * L->c.nf;
  L->launched_seen = v.launched;
  h->nlaunch += (long)v.iters * L->per_iter;
  const int n = v.log_n, pw = 3 * L->c.nf;
  if (n > 0) {
    const size_t t0 = log->tile.size();
    log->tile.resize(t0 + n);
    log->acc.resize(t0 + n);
    log->F.resize(t0 + n);
    log->Fb.resize(t0 + n);
    log->perf.resize((t0 + n) * pw);
    for (int i = 0; i < n; ++i) {
      const unsigned char *r = L->h_rep + kReportHead + (size_t)i * rb;
      log->tile[t0 + i] = reinterpret_cast<const int *>(r)[0];
      log->acc[t0 + i] = reinterpret_cast<const int *>(r)[1];
      log->F[t0 + i] = reinterpret_cast<const double *>(r)[1];
      log->Fb[t0 + i] = reinterpret_cast<const double *>(r)[2];
      std::memcpy(log->perf.data() + (t0 + i) * pw, reinterpret_cast<const double *>(r) + 3, sizeof(double) * pw);
    }
  }
  r->evals = v.evals;
  r->accepts = v.accepts;
  r->launched = v.launched;
  r->F_best = v.F_best;
  r->converged = v.converged;
  r->done = v.done;
  r->err = v.err;
  r->tc_code = v.tc_code;
  r->accepted = v.accepted;
  r->nc = v.nc;
  r->j = v.acc_j;
  r->k = v.acc_k;
  r->nflip = v.acc_nflip;
  for (int q = 0; q < 4; ++q) r->tiles[q] = v.acc_tiles[q];
  r->decisions = v.iters;
  return PNGF_OK;
}

}  // namespace pngf
