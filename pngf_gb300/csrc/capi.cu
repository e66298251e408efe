// C ABI of the PNGF hot path: handle lifecycle, G loading, design setup,
// candidate evaluation and the accept step. See include/pngf_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "bounds.cuh"
#include "pngf_internal.h"

namespace pngf {

int set_error(Handle *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_check(Handle *h, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return PNGF_OK;
  return set_error(h, PNGF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

cudaEvent_t timing_mark(Handle *h, cudaStream_t s) {
  if (!h->timing) return nullptr;
  cudaEvent_t e;
  if (!h->ev_pool.empty()) {
    e = h->ev_pool.back();
    h->ev_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return nullptr;
  }
  cudaEventRecord(e, s ? s : h->stream);
  return e;
}

void timing_close(Handle *h, cudaEvent_t start, int cat, double x1, double x2, double x3, cudaStream_t s) {
  if (!start) return;
  cudaEvent_t stop = timing_mark(h, s);
  if (!stop) return;
  h->pending.push_back({start, stop, cat, x1, x2, x3});
}

// With one lane per frequency: every lane's stream waits for the work queued
// so far on the handle's stream (lanes_fork), and the handle's stream waits
// for everything queued on the lanes (lanes_join).
static int lanes_fork(Handle *h) {
  if (h->lanes.size() < 2) return PNGF_OK;
  cudaError_t e = cudaEventRecord(h->ev_fork, h->stream);
  for (size_t i = 0; i < h->lanes.size() && e == cudaSuccess; ++i)
    e = cudaStreamWaitEvent(h->lanes[i].stream, h->ev_fork, 0);
  return cuda_check(h, e, "fork onto the frequency streams");
}

cudaError_t chain_update_wait(Handle *h, int f, cudaStream_t st) {
  // builds keep their lanes concurrent: a chunk's update overlaps the other
  // lanes' capacitance LUs, and its narrower tile shapes (k = 32) gain from it
  if (h->building || h->lanes.size() < 2 || f <= 0 || (size_t)f >= h->lanes.size()) return cudaSuccess;
  return cudaStreamWaitEvent(st, h->lanes[f - 1].upd, 0);
}

cudaError_t chain_update_done(Handle *h, int f, cudaStream_t st) {
  if (h->building || h->lanes.size() < 2 || f < 0 || (size_t)f >= h->lanes.size()) return cudaSuccess;
  return cudaEventRecord(h->lanes[f].upd, st);
}

static int lanes_join(Handle *h) {
  if (h->lanes.size() < 2) return PNGF_OK;
  cudaError_t e = cudaSuccess;
  for (size_t i = 0; i < h->lanes.size() && e == cudaSuccess; ++i) {
    e = cudaEventRecord(h->lanes[i].done, h->lanes[i].stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, h->lanes[i].done, 0);
  }
  return cuda_check(h, e, "join of the frequency streams");
}

static void timing_collect(Handle *h) {
  for (auto &p : h->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    pngf_timing &t = h->tacc;
    if (p.cat == T_EVAL) {
      t.eval_ms += ms;
      t.eval_launches += 1;
      t.eval_cf += p.x1;
      t.eval_bytes += p.x2;
      t.eval_flop += p.x3;
    } else if (p.cat == T_ACCEPT) {
      t.accept_ms += ms;
      t.accepts += (long)p.x1;  // frequencies the accept covered
    } else {
      t.update_ms += ms;
      t.update_launches += 1;
      t.update_flop += p.x1;
      t.update_bytes += p.x2;
    }
    h->ev_pool.push_back(p.a);
    h->ev_pool.push_back(p.b);
  }
  h->pending.clear();
}


template <typename T> static int dalloc(Handle *h, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) return PNGF_OK;
  const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(h, PNGF_ERR_NOMEM,
                     std::string("cudaMalloc of ") + std::to_string(sizeof(T) * count) + " bytes: " +
                         cudaGetErrorString(e));
  }
  return PNGF_OK;
}

template <typename T> static void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

static int edges_per_tile(const pngf_config &c) {
  return c.cells_x * (c.cells_y + 1) + (c.cells_x + 1) * c.cells_y;
}

// compute_P_matrix (pngfopt.hpp:624-664): an edge is set when any owning tile is set.
static void compute_P(const Handle *h, const std::vector<int> &map, std::vector<signed char> &P) {
  const pngf_config &c = h->cfg;
  P.assign(h->n, 0);
  for (int t = 0; t < h->map_sz; ++t) {
    if (!map[t]) continue;
    const int ty = t / c.tiles_x, tx = t - ty * c.tiles_x;
    const long bx = (long)tx * c.cells_x + (long)ty * c.cells_y * h->ex_xsz;
    const long by = h->nx + (long)tx * c.cells_x + (long)ty * c.cells_y * h->ey_xsz;
    for (int jj = 0; jj < c.cells_y + 1; ++jj)
      for (int ii = 0; ii < c.cells_x; ++ii) P[bx + ii + (long)jj * h->ex_xsz] = 1;
    for (int jj = 0; jj < c.cells_y; ++jj)
      for (int ii = 0; ii < c.cells_x + 1; ++ii) P[by + ii + (long)jj * h->ey_xsz] = 1;
  }
}

static int ensure_cand_cap(Handle *h, int ncand) {
  if (ncand <= h->cand_cap) return PNGF_OK;
  const int cap = std::max(ncand, 2 * h->cand_cap);
  const int nf = h->cfg.num_freq;
  dfree(h->d_tiles);
  dfree(h->d_nflip);
  dfree(h->d_es);
  dfree(h->d_ed);
  dfree(h->d_ek);
  dfree(h->d_new_eobj);
  dfree(h->d_Ff);
  dfree(h->d_perf);
  dfree(h->d_F);
  dfree(h->d_status);
  dfree(h->d_eval_LU);
  dfree(h->d_eval_piv);
  dfree(h->d_eval_z);
  if (h->h_tiles) cudaFreeHost(h->h_tiles);
  if (h->h_nflip) cudaFreeHost(h->h_nflip);
  h->h_tiles = h->h_nflip = nullptr;
  h->cand_cap = 0;
  int rc;
  if ((rc = dalloc(h, &h->d_tiles, (size_t)cap * h->cfg.max_flips)) ||
      (rc = dalloc(h, &h->d_nflip, (size_t)cap)) || (rc = dalloc(h, &h->d_es, (size_t)cap * h->kmax)) ||
      (rc = dalloc(h, &h->d_ed, (size_t)cap * h->kmax)) || (rc = dalloc(h, &h->d_ek, (size_t)cap)) ||
      (rc = dalloc(h, &h->d_new_eobj, (size_t)cap * nf * h->E)) || (rc = dalloc(h, &h->d_Ff, (size_t)cap * nf)) ||
      (rc = dalloc(h, &h->d_perf, (size_t)cap * nf * 3)) || (rc = dalloc(h, &h->d_F, (size_t)cap)) ||
      (rc = dalloc(h, &h->d_status, (size_t)cap * nf)) ||
      (rc = dalloc(h, &h->d_eval_LU, (size_t)cap * nf * h->kmax * h->kmax)) ||
      (rc = dalloc(h, &h->d_eval_piv, (size_t)cap * nf * h->kmax)) ||
      (rc = dalloc(h, &h->d_eval_z, (size_t)cap * nf * h->kmax)))
    return rc;
  PNGF_CUDA(h, cudaMallocHost(&h->h_tiles, sizeof(int) * (size_t)cap * h->cfg.max_flips));
  PNGF_CUDA(h, cudaMallocHost(&h->h_nflip, sizeof(int) * (size_t)cap));
  h->cand_cap = cap;
  return PNGF_OK;
}

int reserve_candidates(Handle *h, int ncand) { return ensure_cand_cap(h, ncand); }

int adopt_device_batch(Handle *h, int ncand, int c, const int *tiles_c, int nflip_c) {
  if (c < 0 || c >= ncand || ncand > h->cand_cap || nflip_c < 0 || nflip_c > h->cfg.max_flips)
    return set_error(h, PNGF_ERR_STATE, "device batch out of range");
  const int mf = h->cfg.max_flips;
  h->batch_tiles.assign((size_t)ncand * mf, 0);
  h->batch_nflip.assign(ncand, 0);
  for (int i = 0; i < nflip_c; ++i) h->batch_tiles[(size_t)c * mf + i] = tiles_c[i];
  h->batch_nflip[c] = nflip_c;
  h->batch_n = ncand;
  h->batch_valid = true;
  return PNGF_OK;
}

static int ensure_host_out(Handle *h, size_t doubles) {
  if (doubles <= h->h_out_cap) return PNGF_OK;
  if (h->h_out) cudaFreeHost(h->h_out);
  h->h_out = nullptr;
  h->h_out_cap = 0;
  PNGF_CUDA(h, cudaMallocHost(&h->h_out, sizeof(double) * doubles));
  h->h_out_cap = doubles;
  return PNGF_OK;
}

static int check_tiles(Handle *h, const int *tiles, const int *nflip, int ncand) {
  for (int c = 0; c < ncand; ++c) {
    if (nflip[c] < 0 || nflip[c] > h->cfg.max_flips)
      return set_error(h, PNGF_ERR_ARG, "candidate " + std::to_string(c) + ": flip count out of range");
    for (int i = 0; i < nflip[c]; ++i) {
      const int t = tiles[(size_t)c * h->cfg.max_flips + i];
      if (t < 0 || t >= h->map_sz)
        return set_error(h, PNGF_ERR_ARG, "candidate " + std::to_string(c) + ": tile index out of range");
    }
  }
  return PNGF_OK;
}

// Evaluates a batch whose tile lists are already in h->d_tiles / h->d_nflip.
// The score reads F_best from d_fbest when it is given (the form a CUDA graph
// can replay with a new F_best), else takes it by value.
static int eval_resident(Handle *h, int ncand, double F_best, const double *d_fbest = nullptr) {
  cudaEvent_t t0 = h->capturing ? nullptr : timing_mark(h);
  PNGF_CUDA(h, launch_edge_lists(h, ncand, h->d_tiles, h->d_nflip));
  PNGF_CUDA(h, launch_eval(h, ncand, F_best, d_fbest));
  timing_close(h, t0, T_EVAL, (double)ncand * h->cfg.num_freq, 0.0, 0.0);
  h->batch_n = ncand;
  h->batch_valid = true;
  return PNGF_OK;
}

// Layout of the pinned result block of a batch of ncand: F, perf, new_eobj
// (as doubles), then ints: first, ek, status, and the tensor-core error flag
// (set by an earlier accept).
struct OutLayout {
  size_t nF, nperf, neo, nint;
  double *F, *perf, *eo;
  int *ints;
  OutLayout(const Handle *h, int ncand)
      : nF(ncand), nperf((size_t)ncand * h->cfg.num_freq * 3), neo((size_t)ncand * h->cfg.num_freq * h->E * 2),
        nint(2 + (size_t)ncand + (size_t)ncand * h->cfg.num_freq) {
    F = h->h_out;
    perf = F ? F + nF : nullptr;
    eo = F ? perf + nperf : nullptr;
    ints = F ? reinterpret_cast<int *>(eo + neo) : nullptr;
  }
  size_t doubles() const { return nF + nperf + neo + nint; }
};

int eval_stage(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best) {
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "pngf_prepare has not been called for this design");
  if (ncand <= 0) return set_error(h, PNGF_ERR_ARG, "ncand must be positive");
  int rc;
  if ((rc = check_tiles(h, tiles, nflip, ncand))) return rc;
  if ((rc = ensure_cand_cap(h, ncand))) return rc;
  if ((rc = ensure_host_out(h, OutLayout(h, ncand).doubles()))) return rc;
  const int mf = h->cfg.max_flips, nf = h->cfg.num_freq;
  std::memcpy(h->h_tiles, tiles, sizeof(int) * (size_t)ncand * mf);
  std::memcpy(h->h_nflip, nflip, sizeof(int) * (size_t)ncand);
  *h->h_fbest = F_best;
  h->batch_tiles.assign(tiles, tiles + (size_t)ncand * mf);
  h->batch_nflip.assign(nflip, nflip + ncand);
  const OutLayout o(h, ncand);
  o.ints[1 + ncand + (size_t)ncand * nf] = 0;
  h->staged_n = ncand;
  return PNGF_OK;
}

int eval_enqueue(Handle *h) {
  pngf::TraceRange trace_("pngf evaluate");
  const int ncand = h->staged_n, mf = h->cfg.max_flips, nf = h->cfg.num_freq;
  if (ncand <= 0) return set_error(h, PNGF_ERR_STATE, "no staged batch");
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_tiles, h->h_tiles, sizeof(int) * (size_t)ncand * mf, cudaMemcpyHostToDevice,
                               h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_nflip, h->h_nflip, sizeof(int) * (size_t)ncand, cudaMemcpyHostToDevice,
                               h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_fbest, h->h_fbest, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int rc;
  if ((rc = eval_resident(h, ncand, 0.0, h->d_fbest))) return rc;
  const OutLayout o(h, ncand);
  PNGF_CUDA(h, cudaMemcpyAsync(o.F, h->d_F, sizeof(double) * o.nF, cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(o.perf, h->d_perf, sizeof(double) * o.nperf, cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(o.eo, h->d_new_eobj, sizeof(double) * o.neo, cudaMemcpyDeviceToHost, h->stream));
  int *hint = o.ints;
  PNGF_CUDA(h, cudaMemcpyAsync(hint, h->d_first, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(hint + 1, h->d_ek, sizeof(int) * ncand, cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(hint + 1 + ncand, h->d_status, sizeof(int) * ncand * nf, cudaMemcpyDeviceToHost,
                               h->stream));
  if (h->d_tc_err)
    PNGF_CUDA(h, cudaMemcpyAsync(hint + 1 + ncand + (size_t)ncand * nf, h->d_tc_err, sizeof(int),
                                 cudaMemcpyDeviceToHost, h->stream));
  h->launched_n = ncand;
  return PNGF_OK;
}

int eval_launch(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best) {
  int rc = eval_stage(h, tiles, nflip, ncand, F_best);
  if (rc) return rc;
  return eval_enqueue(h);
}

int eval_collect(Handle *h, EvalOut *out) {
  const int ncand = h->launched_n, mf = h->cfg.max_flips, nf = h->cfg.num_freq;
  if (ncand <= 0) return set_error(h, PNGF_ERR_STATE, "no batch in flight");
  h->launched_n = 0;
  const OutLayout o(h, ncand);
  const size_t nF = o.nF, nperf = o.nperf, neo = o.neo, nint = o.nint;
  const double *hF = o.F, *hperf = o.perf, *heo = o.eo;
  const int *hint = o.ints;
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  const int tc = hint[1 + ncand + (size_t)ncand * nf];
  if (tc != 0) {
    cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->stream);
    h->batch_valid = false;
    return set_error(h, PNGF_ERR_TIMEOUT, "tensor-core update gave up waiting (code " + std::to_string(tc) + ")");
  }
  if (!out) return PNGF_OK;
  out->F.assign(hF, hF + nF);
  out->perf.assign(hperf, hperf + nperf);
  out->new_eobj.assign(heo, heo + neo);
  out->first = hint[0];
  out->k.assign(hint + 1, hint + 1 + ncand);
  out->status.assign(hint + 1 + ncand, hint + 1 + ncand + (size_t)ncand * nf);
  if (h->timing) {  // algorithmic work of this batch, from the actual flip sizes
    h->tacc.h2d_bytes += sizeof(int) * (double)ncand * (mf + 1);
    h->tacc.d2h_bytes += sizeof(double) * (double)(nF + nperf + neo) + sizeof(int) * (double)nint;
    const double sM = h->cfg.precision == PNGF_PREC_FP64 ? 16.0 : 8.0;
    for (int c = 0; c < ncand; ++c) {
      const double k = std::max(0, out->k[c]);
      h->tacc.eval_bytes += nf * (sM * (k * k + (h->E + 1) * k + h->E) + 21.0 * k);
      h->tacc.eval_flop += nf * (8.0 / 3.0 * k * k * k + 16.0 * k * k + 8.0 * h->E * k);
    }
  }
  return PNGF_OK;
}

int eval_batch(Handle *h, const int *tiles, const int *nflip, int ncand, double F_best, EvalOut *out) {
  int rc = eval_launch(h, tiles, nflip, ncand, F_best);
  if (rc) return rc;
  return eval_collect(h, out);
}

int accept_cand(Handle *h, int c, int k) { return accept_cand_async(h, c, k, true); }

int accept_cand_async(Handle *h, int c, int k, bool check_now) {
  pngf::TraceRange trace_("pngf accept");
  if (!h->batch_valid) return set_error(h, PNGF_ERR_STATE, "no evaluated batch to accept from");
  if (c < 0 || c >= h->batch_n) return set_error(h, PNGF_ERR_ARG, "candidate index outside the last batch");
  if (k < 0 || k > h->kmax) return set_error(h, PNGF_ERR_ARG, "invalid flipped-edge count");
  PNGF_CUDA(h, cudaMemsetAsync(h->d_acc_status, 0, sizeof(int), h->stream));
  ++h->state_version;
  // the frequencies' accepts are independent: one lane (stream + scratch) each
  cudaEvent_t t0 = timing_mark(h);
  int rc;
  if ((rc = lanes_fork(h))) return rc;
  // deferred complex64 updates: append this accept to the pending factors and
  // flush them to T when another accept might not fit
  h->defer_now = h->defer_cap > 0;
  h->defer_flush = h->defer_now && h->defer_rp + k + h->kmax > h->defer_cap;
  h->acc_cand = c;  // the accept starts from the factorization its evaluation left
  for (int f = 0; f < h->cfg.num_freq && rc == PNGF_OK; ++f)
    rc = cuda_check(h, launch_accept_edges(h, f, h->d_es + (size_t)c * h->kmax, h->d_ed + (size_t)c * h->kmax, k,
                                           h->cfg.precision), "accept");
  h->acc_cand = -1;
  h->defer_now = false;
  if (rc) return rc;
  if ((rc = lanes_join(h))) return rc;
  if (h->defer_cap > 0) {
    h->defer_rp = h->defer_flush ? 0 : h->defer_rp + k;
    PNGF_CUDA(h, launch_set_pending_rank(h));
  }
  timing_close(h, t0, T_ACCEPT, (double)h->cfg.num_freq, 0.0, 0.0);
  PNGF_CUDA(h, launch_commit(h, c));
  if (h->d_tc_err && check_now) {  // the tensor-core kernels' bounded waits report here (else at the next collect)
    int tc = 0;
    PNGF_CUDA(h, cudaMemcpyAsync(&tc, h->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
    if (tc != 0) {
      cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->stream);
      h->batch_valid = false;
      return set_error(h, PNGF_ERR_TIMEOUT, "tensor-core update gave up waiting (code " + std::to_string(tc) + ")");
    }
  }
  // host mirror of the design (update_C_inv commits the flip, pngfopt.hpp:360-366)
  const int mf = h->cfg.max_flips;
  for (int i = 0; i < h->batch_nflip[c]; ++i) h->tile_map[h->batch_tiles[(size_t)c * mf + i]] ^= 1;
  compute_P(h, h->tile_map, h->P);
  h->batch_valid = false;
  return PNGF_OK;
}

}  // namespace pngf

using namespace pngf;

static Handle *H(pngf_handle *p) { return reinterpret_cast<Handle *>(p); }
static const Handle *H(const pngf_handle *p) { return reinterpret_cast<const Handle *>(p); }

extern "C" {

void pngf_config_default(pngf_config *cfg, int tiles_x, int tiles_y, int num_freq, const double *freq_hz) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->tiles_x = tiles_x;
  cfg->tiles_y = tiles_y;
  cfg->cells_x = 3;
  cfg->cells_y = 3;
  cfg->num_eobj = 3;
  cfg->max_flips = 4;
  cfg->dx = 0.01 / 60.0;
  cfg->dy = 0.01 / 60.0;
  cfg->dz = 0.01 / 180.0;
  cfg->num_freq = num_freq;
  for (int i = 0; i < num_freq && i < PNGF_MAX_FREQ; ++i) cfg->freq_hz[i] = freq_hz ? freq_hz[i] : 30e9;
  cfg->precision = PNGF_PREC_FP64;
  cfg->defer_rank = 0;
  cfg->device = 0;
}

const char *pngf_last_error(const pngf_handle *h) { return h ? H(h)->err.c_str() : "null handle"; }

int pngf_destroy(pngf_handle *ph) {
  Handle *h = H(ph);
  if (!h) return PNGF_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (Freq &q : h->f) {
    dfree(q.G);
    dfree(q.gobj);
    dfree(q.Einc);
    dfree(q.M64);
    dfree(q.T32);
    dfree(q.y64);
    dfree(q.R64);
    dfree(q.U);
    dfree(q.Vt);
  }
  dfree(h->d_fconst);
  dfree(h->d_views);
  dfree(h->d_iota);
  dfree(h->d_Eincs);
  dfree(h->d_tc_err);
  for (Lane &L : h->lanes) {
    if (L.stream) cudaStreamSynchronize(L.stream);
    dfree(L.A);
    dfree(L.W);
    dfree(L.LU);
    dfree(L.z);
    dfree(L.piv);
    dfree(L.Aop);
    dfree(L.Bop);
    dfree(L.V);
    dfree(L.A16);
    dfree(L.B16);
    dfree(L.Xs);
    dfree(L.KD);
    dfree(L.eA);
    dfree(L.fB);
    if (L.done) cudaEventDestroy(L.done);
    if (L.upd) cudaEventDestroy(L.upd);
    if (L.stream) cudaStreamDestroy(L.stream);
  }
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  dfree(h->d_tile_map);
  dfree(h->d_P);
  dfree(h->d_tiles);
  dfree(h->d_nflip);
  dfree(h->d_es);
  dfree(h->d_ed);
  dfree(h->d_ek);
  dfree(h->d_new_eobj);
  dfree(h->d_Ff);
  dfree(h->d_perf);
  dfree(h->d_F);
  dfree(h->d_first);
  dfree(h->d_status);
  dfree(h->d_eval_LU);
  dfree(h->d_eval_piv);
  dfree(h->d_eval_z);
  dfree(h->d_acc_s);
  dfree(h->d_acc_d);
  dfree(h->d_acc_status);
  dfree(h->d_colmax);
  dfree(h->d_fbest);
  if (h->h_fbest) cudaFreeHost(h->h_fbest);
  if (h->h_tiles) cudaFreeHost(h->h_tiles);
  if (h->h_nflip) cudaFreeHost(h->h_nflip);
  if (h->h_out) cudaFreeHost(h->h_out);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return PNGF_OK;
}

int pngf_create(const pngf_config *cfg, pngf_handle **out) {
  if (!cfg || !out) return PNGF_ERR_ARG;
  *out = nullptr;
  const pngf_config &c = *cfg;
  if (c.tiles_x < 3 || c.tiles_y < 3 || c.cells_x < 1 || c.cells_y < 2 || c.num_eobj < 1 ||
      c.num_eobj > PNGF_MAX_EOBJ || c.num_freq < 1 || c.num_freq > PNGF_MAX_FREQ || c.max_flips < 1 ||
      c.max_flips > 8 || !(c.dx > 0) || !(c.dy > 0) || !(c.dz > 0))
    return PNGF_ERR_ARG;
  if (c.precision != PNGF_PREC_FP64 && c.precision != PNGF_PREC_C64) return PNGF_ERR_ARG;
  if (c.c64_build != PNGF_BUILD_FP64 && c.c64_build != PNGF_BUILD_C64) return PNGF_ERR_ARG;
  if (c.state_only != 0 && c.state_only != 1) return PNGF_ERR_ARG;
  const int kmax = c.max_flips * edges_per_tile(c);
  if (kmax > kMaxEvalK) return PNGF_ERR_UNSUPPORTED;
  // deferred updates (complex64): the pending rank must hold at least one accept
  const int defer_cap = c.precision == PNGF_PREC_C64 ? c.defer_rank : 0;
  if (defer_cap < 0 || (defer_cap > 0 && (defer_cap < kmax || defer_cap > kMaxDeferRank))) return PNGF_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c.device || c.device < 0) {
    cudaGetLastError();
    return PNGF_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(c.device) != cudaSuccess) return PNGF_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, c.device) != cudaSuccess || prop.major * 10 + prop.minor != 103)
    return PNGF_ERR_NO_DEVICE;  // this library carries sm_103a code only

  Handle *h = new (std::nothrow) Handle();
  if (!h) return PNGF_ERR_NOMEM;
  h->cfg = c;
  h->n = pngf_num_edges(c.tiles_x, c.tiles_y, c.cells_x, c.cells_y);
  h->E = c.num_eobj;
  h->ldm = (h->n + 1 + 15) / 16 * 16;
  h->map_sz = c.tiles_x * c.tiles_y;
  h->ex_xsz = c.tiles_x * c.cells_x;
  h->ex_ysz = c.tiles_y * c.cells_y + 1;
  h->ey_xsz = c.tiles_x * c.cells_x + 1;
  h->ey_ysz = c.tiles_y * c.cells_y;
  h->nx = (long)h->ex_xsz * h->ex_ysz;
  h->kmax = kmax;
  h->defer_cap = defer_cap;
  h->acc_cap = std::max(kmax, kInitChunk);
  h->f.resize(c.num_freq);
  h->h_fconst.resize(c.num_freq);
  h->tile_map.assign(h->map_sz, 0);
  h->P.assign(h->n, 0);
  auto fail = [&](int rc) {
    pngf_destroy(reinterpret_cast<pngf_handle *>(h));
    return rc;
  };
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(PNGF_ERR_CUDA);
  h->stream = h->own_stream;
  const long n = h->n, rows = n + h->E;
  int rc;
  const bool c64 = c.precision == PNGF_PREC_C64;
  std::vector<void *> einc(c.num_freq);
  for (int f = 0; f < c.num_freq; ++f) {
    Freq &q = h->f[f];
    // state_only: G (and a complex64 handle's FP64 staging of M) exist only while a build or check runs
    if ((!c.state_only && (rc = dalloc(h, &q.G, (size_t)n * n))) ||
        (rc = dalloc(h, &q.gobj, (size_t)std::max(1, h->E - 1) * n)) || (rc = dalloc(h, &q.Einc, (size_t)n)) ||
        (!(c.state_only && c64) && (rc = dalloc(h, &q.M64, (size_t)rows * h->ldm))))
      return fail(rc);
    if (c64 && ((rc = dalloc(h, &q.T32, (size_t)n * h->ldm)) || (rc = dalloc(h, &q.y64, (size_t)n)) ||
                (rc = dalloc(h, &q.R64, (size_t)h->E * h->ldm))))
      return fail(rc);
    if (defer_cap > 0 &&
        ((rc = dalloc(h, &q.U, (size_t)n * defer_cap)) || (rc = dalloc(h, &q.Vt, (size_t)n * defer_cap))))
      return fail(rc);
    einc[f] = q.Einc;
  }
  // Tensor-core operands: rows padded to the 128-row tile, zero outside what
  // each update writes. Complex64 updates (accepts and build chunks); FP64
  // updates (and the FP64 build of M) on the tensor cores, in pieces of
  // f64tc_max_k() edges, unless PNGF_F64_SIMT.
  if (c64) {
    h->kt_cap = (6 * std::max(std::max(kmax, kInitChunk), defer_cap) + 31) / 32 * 32;
    h->aop_rows = (n + 127) / 128 * 128;
    h->bop_rows = (2 * n + 127) / 128 * 128;
  }
  if (c.fp64_update != PNGF_F64_SIMT) {
    h->f64tc = true;
    h->init_chunk = f64tc_max_k();
    h->a16_rows = (rows + 127) / 128 * 128;
    h->b16_rows = f64tc_b_rows(n);
  }
  if ((rc = dalloc(h, &h->d_tc_err, 1))) return fail(rc);
  if (cudaMemset(h->d_tc_err, 0, sizeof(int)) != cudaSuccess) return fail(PNGF_ERR_CUDA);
  // One lane (stream + accept scratch) per frequency; one lane on the
  // handle's stream for a state_only handle, which keeps device memory to the state.
  h->lanes.resize(c.state_only ? 1 : c.num_freq);
  if (h->lanes.size() > 1 && cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess)
    return fail(PNGF_ERR_CUDA);
  for (Lane &L : h->lanes) {
    if (h->lanes.size() > 1 && (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess ||
                                cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming) != cudaSuccess ||
                                cudaEventCreateWithFlags(&L.upd, cudaEventDisableTiming) != cudaSuccess))
      return fail(PNGF_ERR_CUDA);
    if ((rc = dalloc(h, &L.A, (size_t)rows * h->acc_cap)) || (rc = dalloc(h, &L.W, (size_t)h->acc_cap * h->ldm)) ||
        (rc = dalloc(h, &L.LU, (size_t)h->acc_cap * h->acc_cap)) || (rc = dalloc(h, &L.V, (size_t)h->acc_cap * h->acc_cap)) ||
        (rc = dalloc(h, &L.piv, (size_t)h->acc_cap)) ||
        (rc = dalloc(h, &L.z, (size_t)h->acc_cap)))
      return fail(rc);
    if (c64) {
      if ((rc = dalloc(h, &L.Aop, (size_t)h->aop_rows * h->kt_cap)) ||
          (rc = dalloc(h, &L.Bop, (size_t)h->bop_rows * h->kt_cap)))
        return fail(rc);
      if (cudaMemset(L.Aop, 0, sizeof(float) * h->aop_rows * h->kt_cap) != cudaSuccess ||
          cudaMemset(L.Bop, 0, sizeof(float) * h->bop_rows * h->kt_cap) != cudaSuccess)
        return fail(PNGF_ERR_CUDA);
    }
    if (h->f64tc) {
      const size_t ca = (size_t)h->a16_rows * f64tc_op_cols(), cb = (size_t)h->b16_rows * f64tc_b_cols();
      if (cudaMalloc(&L.A16, 2 * ca) != cudaSuccess || cudaMalloc(&L.B16, 2 * cb) != cudaSuccess)
        return fail(PNGF_ERR_NOMEM);
      // one scale per output column, padded to the 32-column tiles
      if ((rc = dalloc(h, &L.eA, (size_t)h->a16_rows)) || (rc = dalloc(h, &L.fB, (size_t)(2 * (n + 1) + 127) / 128 * 128)))
        return fail(rc);
      if (cudaMemset(L.A16, 0, 2 * ca) != cudaSuccess || cudaMemset(L.B16, 0, 2 * cb) != cudaSuccess)
        return fail(PNGF_ERR_CUDA);
      // dense rows s: the deferred complex64 accept, and FP64 accepts of more than 32 edges (with K D)
      const bool big64 = !c64 && h->acc_cap > f64tc_max_k();
      if (((c64 && h->defer_cap > 0) || big64) && (rc = dalloc(h, &L.Xs, (size_t)h->acc_cap * h->ldm)))
        return fail(rc);
      if (big64 && (rc = dalloc(h, &L.KD, (size_t)h->acc_cap * h->acc_cap))) return fail(rc);
    }
  }
  if (c64 && h->defer_cap > 0 && h->f64tc) {
    std::vector<int> iota(h->acc_cap);
    for (int q = 0; q < h->acc_cap; ++q) iota[q] = q;
    if ((rc = dalloc(h, &h->d_iota, (size_t)h->acc_cap))) return fail(rc);
    if (cudaMemcpy(h->d_iota, iota.data(), sizeof(int) * h->acc_cap, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(PNGF_ERR_CUDA);
  }
  {
    void *v = nullptr;
    if (cudaMalloc(&v, view_bytes() * c.num_freq) != cudaSuccess) return fail(PNGF_ERR_NOMEM);
    h->d_views = v;
  }
  if ((rc = dalloc(h, &h->d_fconst, (size_t)c.num_freq)) || (rc = dalloc(h, &h->d_Eincs, (size_t)c.num_freq)) ||
      (rc = dalloc(h, &h->d_tile_map, (size_t)h->map_sz)) || (rc = dalloc(h, &h->d_P, (size_t)n)) ||
      (rc = dalloc(h, &h->d_first, 1)) || (rc = dalloc(h, &h->d_acc_s, (size_t)n)) ||
      (rc = dalloc(h, &h->d_acc_d, (size_t)n)) || (rc = dalloc(h, &h->d_acc_status, 1)) ||
      (rc = dalloc(h, &h->d_colmax, (size_t)n)) ||
      (rc = dalloc(h, &h->d_fbest, 1)))
    return fail(rc);
  if (cudaMemcpy(h->d_Eincs, einc.data(), sizeof(void *) * c.num_freq, cudaMemcpyHostToDevice) != cudaSuccess ||
      setup_views(h) != cudaSuccess)
    return fail(PNGF_ERR_CUDA);
  if ((rc = ensure_cand_cap(h, 64))) return fail(rc);
  if (cudaMallocHost(&h->h_fbest, sizeof(double)) != cudaSuccess) return fail(PNGF_ERR_NOMEM);
  *out = reinterpret_cast<pngf_handle *>(h);
  return PNGF_OK;
}

int pngf_set_stream(pngf_handle *ph, void *stream) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return PNGF_OK;
}

int pngf_dims(const pngf_handle *ph, long *n_edges, long *ld_m) {
  const Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (n_edges) *n_edges = h->n;
  if (ld_m) *ld_m = h->ldm;
  return PNGF_OK;
}

int pngf_load_G(pngf_handle *ph, int f, const double *G, long ldg, const double *gobj_rows) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (f < 0 || f >= h->cfg.num_freq || !G || ldg < h->n) return set_error(h, PNGF_ERR_ARG, "pngf_load_G: bad argument");
  if (h->cfg.state_only)
    return set_error(h, PNGF_ERR_UNSUPPORTED, "a state_only handle takes G from pngf_load_G_synth");
  Freq &q = h->f[f];
  const long n = h->n;
  PNGF_CUDA(h, cudaMemcpy2DAsync(q.G, sizeof(double2) * n, G, sizeof(double2) * ldg, sizeof(double2) * n, n,
                                 cudaMemcpyHostToDevice, h->stream));
  if (h->E > 1) {
    if (gobj_rows)
      PNGF_CUDA(h, cudaMemcpyAsync(q.gobj, gobj_rows, sizeof(double2) * (size_t)(h->E - 1) * n,
                                   cudaMemcpyHostToDevice, h->stream));
    else
      PNGF_CUDA(h, cudaMemsetAsync(q.gobj, 0, sizeof(double2) * (size_t)(h->E - 1) * n, h->stream));
  }
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  q.loaded = true;
  h->prepared = false;
  return PNGF_OK;
}

int pngf_load_G_synth(pngf_handle *ph, int f, unsigned long long seed, double eps_r) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (f < 0 || f >= h->cfg.num_freq || !(eps_r > 0.0))
    return set_error(h, PNGF_ERR_ARG, "pngf_load_G_synth: bad argument");
  Freq &q = h->f[f];
  q.synth = true;
  q.synth_seed = seed;
  q.synth_eps = eps_r;
  PNGF_CUDA(h, launch_synth_gobj(h, f, q.gobj));
  if (!h->cfg.state_only) PNGF_CUDA(h, launch_synth_G(h, f, q.G, h->n, h->d_colmax));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  q.loaded = true;
  h->prepared = false;
  return PNGF_OK;
}

// Streams one acmefdfd G file to the device (the reader of
// pngfopt.hpp:160-180 without its host copy of the whole matrix): the first N
// columns of the (N+E-1)^2 column-major file are read in panels of about
// 32 MB into two pinned buffers; while one panel's G block is copied
// (cudaMemcpy2DAsync, the N design rows of each column) the next is read.
// The E-1 objective rows (rows N.. of each column) are gathered on the host
// (E-1 values per column) and uploaded at the end. Host memory used: the two
// panels and the objective rows, never N^2. A missing or short file is
// PNGF_ERR_IO and leaves the frequency not loaded.
int pngf_load_G_file(pngf_handle *ph, int f, const char *path) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (f < 0 || f >= h->cfg.num_freq || !path) return set_error(h, PNGF_ERR_ARG, "pngf_load_G_file: bad argument");
  if (h->cfg.state_only)
    return set_error(h, PNGF_ERR_UNSUPPORTED, "a state_only handle takes G from pngf_load_G_synth");
  const long n = h->n, m = n + h->E - 1;
  const size_t colb = sizeof(double2) * (size_t)m;
  std::FILE *fp = std::fopen(path, "rb");
  if (!fp) return set_error(h, PNGF_ERR_IO, std::string("cannot open G file ") + path);
  if (std::fseek(fp, 0, SEEK_END) != 0 || std::ftell(fp) < (long)(colb * (size_t)n) || std::fseek(fp, 0, SEEK_SET)) {
    std::fclose(fp);
    return set_error(h, PNGF_ERR_IO, std::string("G file too short: ") + path);
  }
  const long P = std::max<long>(1, std::min<long>(n, (32l << 20) / (long)colb));  // columns per panel
  void *buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool used[2] = {false, false};
  std::vector<double2> gobj((size_t)std::max(1, h->E - 1) * n);
  int rc = PNGF_OK;
  std::string msg;
  Freq &q = h->f[f];
  for (int b = 0; b < 2 && rc == PNGF_OK; ++b)
    if (cudaHostAlloc(&buf[b], colb * P, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) != cudaSuccess) {
      rc = PNGF_ERR_NOMEM;
      msg = "pinned panel for the G file";
    }
  for (long j0 = 0, it = 0; j0 < n && rc == PNGF_OK; j0 += P, ++it) {
    const int b = (int)(it & 1);
    const long cols = std::min(P, n - j0);
    if (used[b] && cudaEventSynchronize(ev[b]) != cudaSuccess) {  // the panel's previous copy is done
      rc = PNGF_ERR_CUDA;
      msg = "G panel copy";
      break;
    }
    double2 *pb = static_cast<double2 *>(buf[b]);
    if (std::fread(pb, colb, (size_t)cols, fp) != (size_t)cols) {
      rc = PNGF_ERR_IO;
      msg = std::string("G file read failed: ") + path;
      break;
    }
    for (long c = 0; c < cols; ++c)
      for (int r = 0; r < h->E - 1; ++r) gobj[(size_t)r * n + j0 + c] = pb[(size_t)c * m + n + r];
    if (cudaMemcpy2DAsync(q.G + (size_t)j0 * n, sizeof(double2) * n, pb, colb, sizeof(double2) * n, (size_t)cols,
                          cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
        cudaEventRecord(ev[b], h->stream) != cudaSuccess) {
      rc = PNGF_ERR_CUDA;
      msg = "G panel copy";
      break;
    }
    used[b] = true;
  }
  std::fclose(fp);
  if (rc == PNGF_OK && h->E > 1 &&
      cudaMemcpyAsync(q.gobj, gobj.data(), sizeof(double2) * (size_t)(h->E - 1) * n, cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess) {
    rc = PNGF_ERR_CUDA;
    msg = "objective rows copy";
  }
  // every copy from the panels and the row vector completes before they are freed
  if (cudaStreamSynchronize(h->stream) != cudaSuccess && rc == PNGF_OK) {
    rc = PNGF_ERR_CUDA;
    msg = "G file load";
  }
  for (int b = 0; b < 2; ++b) {
    if (ev[b]) cudaEventDestroy(ev[b]);
    if (buf[b]) cudaFreeHost(buf[b]);
  }
  if (rc != PNGF_OK) {
    q.loaded = false;
    return set_error(h, rc, msg);
  }
  q.loaded = true;
  h->prepared = false;
  return PNGF_OK;
}

int pngf_set_tile_map(pngf_handle *ph, const int *tile_map) {
  Handle *h = H(ph);
  if (!h || !tile_map) return PNGF_ERR_ARG;
  for (int t = 0; t < h->map_sz; ++t) h->tile_map[t] = tile_map[t] ? 1 : 0;
  compute_P(h, h->tile_map, h->P);
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_tile_map, h->tile_map.data(), sizeof(int) * h->map_sz, cudaMemcpyHostToDevice,
                               h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_P, h->P.data(), h->n, cudaMemcpyHostToDevice, h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_map = true;
  h->prepared = false;
  h->batch_valid = false;
  return PNGF_OK;
}

int pngf_get_tile_map(const pngf_handle *ph, int *tile_map) {
  const Handle *h = H(ph);
  if (!h || !tile_map) return PNGF_ERR_ARG;
  std::copy(h->tile_map.begin(), h->tile_map.end(), tile_map);
  return PNGF_OK;
}

int pngf_set_source_port(pngf_handle *ph, int tile_x, int tile_y, int y_offset, int y_size) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  const pngf_config &c = h->cfg;
  if (y_offset < 0 || y_size < 1 || y_offset + y_size > c.cells_y)
    return set_error(h, PNGF_ERR_ARG, "set_source_port: invalid port y position and height parameters.");
  if (tile_x < 0 || tile_x >= c.tiles_x || tile_y < 0 || tile_y >= c.tiles_y)
    return set_error(h, PNGF_ERR_ARG, "set_source_port: port tile outside the map");
  h->port.clear();
  for (int jj = 0; jj < y_size; ++jj)
    for (int ii = 0; ii < c.cells_x; ++ii)
      h->port.push_back((long)(tile_x * c.cells_x + ii) + (long)(tile_y * c.cells_y + jj + y_offset) * h->ex_xsz);
  h->have_port = true;
  h->prepared = false;
  return PNGF_OK;
}

// Deferred complex64 updates: subtracts the pending factors from T at every
// frequency (before anything reads T32 directly).
static int flush_pending(Handle *h) {
  if (h->defer_rp == 0) return PNGF_OK;
  ++h->state_version;
  int rc = lanes_fork(h);
  for (int f = 0; f < h->cfg.num_freq && rc == PNGF_OK; ++f) rc = cuda_check(h, launch_c64_flush(h, f), "flush");
  const int rj = lanes_join(h);
  if (rc) return rc;
  if (rj) return rj;
  h->defer_rp = 0;
  PNGF_CUDA(h, launch_set_pending_rank(h));
  return PNGF_OK;
}

// state_only handles: frequency f's G (regenerated; need_G) and, for a
// complex64 handle, its FP64 staging of M (need_M64) exist on the device
// only between stage_in and stage_out. No-ops otherwise.
static int stage_in(Handle *h, int f, bool need_G, bool need_M64) {
  if (!h->cfg.state_only) return PNGF_OK;
  Freq &q = h->f[f];
  int rc;
  if (need_G) {
    if ((rc = dalloc(h, &q.G, (size_t)h->n * h->n))) return rc;
    PNGF_CUDA(h, launch_synth_G(h, f, q.G, h->n, h->d_colmax));
  }
  if (need_M64 && h->cfg.precision == PNGF_PREC_C64 &&
      (rc = dalloc(h, &q.M64, (size_t)(h->n + h->E) * h->ldm)))
    return rc;
  return PNGF_OK;
}

static void stage_out(Handle *h, int f) {
  if (!h->cfg.state_only) return;
  Freq &q = h->f[f];
  cudaStreamSynchronize(h->stream);
  dfree(q.G);
  if (h->cfg.precision == PNGF_PREC_C64) dfree(q.M64);
}

// Builds the state for the current design from G. fp64: in FP64 (then T is
// rounded for a complex64 handle); else directly in complex64.
static int prepare_impl(Handle *h, bool fp64) {
  for (int f = 0; f < h->cfg.num_freq; ++f)
    if (!h->f[f].loaded) return set_error(h, PNGF_ERR_STATE, "G not loaded for frequency " + std::to_string(f));
  if (!h->have_map) return set_error(h, PNGF_ERR_STATE, "tile map not set");
  if (!h->have_port) return set_error(h, PNGF_ERR_STATE, "source port not set");
  ++h->state_version;
  h->defer_rp = 0;  // a build starts from G: nothing is pending (build chunks are not deferred)
  PNGF_CUDA(h, launch_set_pending_rank(h));
  // Set edges of the design, ascending; M is built from P = 0 by accepting
  // them in chunks (every chunk is a +1 flip of those edges).
  std::vector<int> on;
  for (long e = 0; e < h->n; ++e)
    if (h->P[e]) on.push_back((int)e);
  std::vector<signed char> ones(on.size(), 1);
  if (!on.empty()) {
    PNGF_CUDA(h, cudaMemcpyAsync(h->d_acc_s, on.data(), sizeof(int) * on.size(), cudaMemcpyHostToDevice, h->stream));
    PNGF_CUDA(h, cudaMemcpyAsync(h->d_acc_d, ones.data(), on.size(), cudaMemcpyHostToDevice, h->stream));
  }
  PNGF_CUDA(h, cudaMemsetAsync(h->d_acc_status, 0, sizeof(int), h->stream));
  const bool c64 = h->cfg.precision == PNGF_PREC_C64;
  auto build = [&](int f) -> int {
    PNGF_CUDA(h, launch_init_M(h, f));
    if (c64 && !fp64) PNGF_CUDA(h, launch_split_M(h, f));
    const int chunk = fp64 ? h->init_chunk : kC64BuildChunk;
    // A complex64 build of a large state on a handle with deferred updates
    // pairs its chunks: the second chunk of a pair reads the first one's
    // update through the pending factors (dense rows and columns of T_true)
    // and one long-K flush of rank up to 2 x chunk applies both -- half the
    // passes over T. Measured: 16 % faster at N = 30504 (41x41, 4 frequencies),
    // 5-9 % slower at N = 8064 (21x21, 5 frequencies), where a pass over T
    // costs little more than the pending blocks.
    constexpr long kPairMinN = 16384;
    const bool pair = c64 && !fp64 && h->n >= kPairMinN && h->defer_cap >= 2 * chunk && h->d_iota &&
                      lane_of(h, f).Xs;
    int rp = 0;
    for (size_t c0 = 0; c0 < on.size(); c0 += chunk) {
      const int k = (int)std::min<size_t>(chunk, on.size() - c0);
      if (pair) {
        h->defer_rp = rp;
        h->defer_now = true;
        h->defer_flush = rp + k + chunk > h->defer_cap || c0 + k >= on.size();
      }
      PNGF_CUDA(h, launch_accept_edges(h, f, h->d_acc_s + c0, h->d_acc_d + c0, k,
                                       fp64 ? PNGF_PREC_FP64 : PNGF_PREC_C64));
      if (pair) rp = h->defer_flush ? 0 : rp + k;
    }
    h->defer_rp = 0;
    h->defer_now = h->defer_flush = false;
    if (c64 && fp64) PNGF_CUDA(h, launch_split_M(h, f));
    return PNGF_OK;
  };
  // frequencies build independently, one lane (stream + scratch) each
  int rc = lanes_fork(h);
  if (rc) return rc;
  h->building = true;
  for (int f = 0; f < h->cfg.num_freq && rc == PNGF_OK; ++f) {
    rc = stage_in(h, f, true, true);
    if (rc == PNGF_OK) rc = build(f);
    stage_out(h, f);
  }
  h->building = false;
  h->defer_rp = 0;  // a build that stopped early may have left a chunk pending
  h->defer_now = h->defer_flush = false;
  const int rj = lanes_join(h);
  if (rc) return rc;
  if (rj) return rj;
  int st = 0, tc = 0;
  PNGF_CUDA(h, cudaMemcpyAsync(&st, h->d_acc_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  if (h->d_tc_err) PNGF_CUDA(h, cudaMemcpyAsync(&tc, h->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(h->h_fconst.data(), h->d_fconst, sizeof(FreqConst) * h->cfg.num_freq,
                               cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  if (st != PNGF_OK) return set_error(h, st, "singular capacitance matrix while building M for the design");
  if (tc != 0) {
    cudaMemset(h->d_tc_err, 0, sizeof(int));
    return set_error(h, PNGF_ERR_TIMEOUT, "tensor-core update gave up waiting (code " + std::to_string(tc) + ")");
  }
  h->prepared = true;
  h->batch_valid = false;
  return PNGF_OK;
}

int pngf_prepare(pngf_handle *ph) {
  pngf::TraceRange trace_("pngf_prepare");
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  return prepare_impl(h, !(h->cfg.precision == PNGF_PREC_C64 && h->cfg.c64_build == PNGF_BUILD_C64));
}

int pngf_get_eobj(pngf_handle *ph, int f, double *eobj, double *vinc_ln) {
  Handle *h = H(ph);
  if (!h || f < 0 || f >= h->cfg.num_freq) return PNGF_ERR_ARG;
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "not prepared");
  if (eobj)
    for (int e = 0; e < h->E; ++e)
      PNGF_CUDA(h, cudaMemcpyAsync(eobj + 2 * e,
                                   h->cfg.precision == PNGF_PREC_C64
                                       ? h->f[f].R64 + (size_t)e * h->ldm + h->n
                                       : h->f[f].M64 + (size_t)(h->n + e) * h->ldm + h->n,
                                   sizeof(double2),
                                   cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  if (vinc_ln) {
    const FreqConst &c = h->h_fconst[f];
    const double v[6] = {c.vinc.x, c.vinc.y, c.ln1.x, c.ln1.y, c.ln2.x, c.ln2.y};
    std::memcpy(vinc_ln, v, sizeof(v));
  }
  return PNGF_OK;
}

int pngf_objective(pngf_handle *ph, double *F) {
  Handle *h = H(ph);
  if (!h || !F) return PNGF_ERR_ARG;
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "not prepared");
  PNGF_CUDA(h, launch_current_objective(h));
  PNGF_CUDA(h, cudaMemcpyAsync(F, h->d_F, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  h->batch_valid = false;  // d_F was reused
  return PNGF_OK;
}

int pngf_get_M(pngf_handle *ph, int f, double *M, long ld, double *einc) {
  Handle *h = H(ph);
  if (!h || !M || f < 0 || f >= h->cfg.num_freq || ld < h->n + 1) return PNGF_ERR_ARG;
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "not prepared");
  const long rows = h->n + h->E;
  int rc = flush_pending(h);
  if (rc) return rc;
  rc = stage_in(h, f, false, true);
  auto copy = [&]() -> int {
    if (h->cfg.precision == PNGF_PREC_C64) PNGF_CUDA(h, launch_merge_M(h, f));  // M64 is staging in this mode
    PNGF_CUDA(h, cudaMemcpy2DAsync(M, sizeof(double2) * ld, h->f[f].M64, sizeof(double2) * h->ldm,
                                   sizeof(double2) * (h->n + 1), rows, cudaMemcpyDeviceToHost, h->stream));
    if (einc)
      PNGF_CUDA(h, cudaMemcpyAsync(einc, h->f[f].Einc, sizeof(double2) * h->n, cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
    return PNGF_OK;
  };
  if (rc == PNGF_OK) rc = copy();
  stage_out(h, f);
  return rc;
}

int pngf_eval_candidates(pngf_handle *ph, const int *tiles, const int *nflip, int ncand, double *new_eobj,
                         double *F) {
  pngf::TraceRange trace_("pngf_eval_candidates");
  Handle *h = H(ph);
  if (!h || !tiles || !nflip) return PNGF_ERR_ARG;
  EvalOut o;
  const int rc = eval_batch(h, tiles, nflip, ncand, -std::numeric_limits<double>::infinity(), &o);
  if (rc) return rc;
  if (F) std::copy(o.F.begin(), o.F.end(), F);
  if (new_eobj) std::copy(o.new_eobj.begin(), o.new_eobj.end(), new_eobj);
  h->last_k = o.k;
  h->last_status = o.status;
  return PNGF_OK;
}

int pngf_eval_candidates_device(pngf_handle *ph, const int *d_tiles, const int *d_nflip, int ncand,
                                double *d_new_eobj, double *d_F, double F_best, int *d_first) {
  pngf::TraceRange trace_("pngf_eval_candidates_device");
  Handle *h = H(ph);
  if (!h || !d_tiles || !d_nflip || ncand <= 0) return PNGF_ERR_ARG;
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "not prepared");
  int rc;
  if ((rc = ensure_cand_cap(h, ncand))) return rc;
  const int mf = h->cfg.max_flips, nf = h->cfg.num_freq;
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_tiles, d_tiles, sizeof(int) * (size_t)ncand * mf, cudaMemcpyDeviceToDevice,
                               h->stream));
  PNGF_CUDA(h, cudaMemcpyAsync(h->d_nflip, d_nflip, sizeof(int) * ncand, cudaMemcpyDeviceToDevice, h->stream));
  if ((rc = eval_resident(h, ncand, F_best))) return rc;
  h->batch_tiles.clear();  // tile lists stay on the device; pngf_accept fetches them
  h->batch_nflip.clear();
  if (d_new_eobj)
    PNGF_CUDA(h, cudaMemcpyAsync(d_new_eobj, h->d_new_eobj, sizeof(double2) * (size_t)ncand * nf * h->E,
                                 cudaMemcpyDeviceToDevice, h->stream));
  if (d_F) PNGF_CUDA(h, cudaMemcpyAsync(d_F, h->d_F, sizeof(double) * ncand, cudaMemcpyDeviceToDevice, h->stream));
  if (d_first) PNGF_CUDA(h, cudaMemcpyAsync(d_first, h->d_first, sizeof(int), cudaMemcpyDeviceToDevice, h->stream));
  h->last_k.clear();
  h->last_status.clear();
  return PNGF_OK;
}

int pngf_accept(pngf_handle *ph, int cand) {
  pngf::TraceRange trace_("pngf_accept");
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (!h->batch_valid) return set_error(h, PNGF_ERR_STATE, "pngf_accept without a preceding evaluation");
  if (cand < 0 || cand >= h->batch_n) return set_error(h, PNGF_ERR_ARG, "candidate index outside the last batch");
  const int mf = h->cfg.max_flips, nf = h->cfg.num_freq;
  if (h->last_k.empty()) {  // device-pointer batch: fetch what the host needs
    int k = 0, nfl = 0;
    std::vector<int> st(nf), tl(mf);
    PNGF_CUDA(h, cudaMemcpyAsync(&k, h->d_ek + cand, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaMemcpyAsync(st.data(), h->d_status + (size_t)cand * nf, sizeof(int) * nf,
                                 cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaMemcpyAsync(&nfl, h->d_nflip + cand, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaMemcpyAsync(tl.data(), h->d_tiles + (size_t)cand * mf, sizeof(int) * mf,
                                 cudaMemcpyDeviceToHost, h->stream));
    PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
    h->batch_tiles.assign((size_t)h->batch_n * mf, 0);
    h->batch_nflip.assign(h->batch_n, 0);
    std::copy(tl.begin(), tl.end(), h->batch_tiles.begin() + (size_t)cand * mf);
    h->batch_nflip[cand] = nfl;
    for (int f = 0; f < nf; ++f)
      if (st[f] != PNGF_OK) return set_error(h, st[f], "candidate did not evaluate cleanly; not accepted");
    return accept_cand(h, cand, k);
  }
  for (int f = 0; f < nf; ++f)
    if (h->last_status[(size_t)cand * nf + f] != PNGF_OK)
      return set_error(h, h->last_status[(size_t)cand * nf + f], "candidate did not evaluate cleanly; not accepted");
  return accept_cand(h, cand, h->last_k[cand]);
}

}  // extern "C"

// Drift check over frequencies f0 .. f1-1.
static int drift_impl(Handle *h, int f0, int f1, int nrows, double *max_rel) {
  if (h->cfg.precision != PNGF_PREC_C64)
    return set_error(h, PNGF_ERR_UNSUPPORTED, "drift check applies to PNGF_PREC_C64 handles");
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "not prepared");
  if (nrows < 1 || nrows > 8) return set_error(h, PNGF_ERR_ARG, "drift check samples 1 to 8 rows");
  {
    const int rf = flush_pending(h);  // the check reads T32 directly
    if (rf) return rf;
  }
  const long n = h->n;
  std::vector<int> on, rows(nrows);
  for (long e = 0; e < n; ++e)
    if (h->P[e]) on.push_back((int)e);
  for (int r = 0; r < nrows; ++r) rows[r] = (int)(((2 * r + 1) * n) / (2 * nrows));
  double2 *X = nullptr, *PH = nullptr, *Rk = nullptr;
  int *d_rows = nullptr;
  unsigned long long *d_out = nullptr;
  int rc;
  auto release = [&]() {
    dfree(X);
    dfree(PH);
    dfree(Rk);
    dfree(d_rows);
    dfree(d_out);
  };
  if ((rc = dalloc(h, &X, (size_t)nrows * n)) || (rc = dalloc(h, &PH, (size_t)nrows * n)) ||
      (rc = dalloc(h, &Rk, (size_t)nrows * n)) || (rc = dalloc(h, &d_rows, (size_t)nrows)) ||
      (rc = dalloc(h, &d_out, 2 * (size_t)h->cfg.num_freq))) {
    release();
    return rc;
  }
  double worst = 0.0;
  cudaError_t e = cudaMemcpyAsync(d_rows, rows.data(), sizeof(int) * nrows, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess && !on.empty())
    e = cudaMemcpyAsync(h->d_acc_s, on.data(), sizeof(int) * on.size(), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long) * 2 * h->cfg.num_freq, h->stream);
  for (int f = f0; f < f1 && e == cudaSuccess; ++f) {
    if ((rc = stage_in(h, f, true, false))) {
      stage_out(h, f);
      release();
      return rc;
    }
    e = launch_drift_rows(h, f, d_rows, nrows, h->d_acc_s, (int)on.size(), X, PH, Rk, d_out + 2 * f);
    stage_out(h, f);
  }
  std::vector<unsigned long long> out(2 * h->cfg.num_freq);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out.data(), d_out, sizeof(unsigned long long) * out.size(), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  release();
  if (e != cudaSuccess) return cuda_check(h, e, "drift check");
  for (int f = f0; f < f1; ++f) {
    double dmax, xmax;
    std::memcpy(&dmax, &out[2 * f], sizeof(double));
    std::memcpy(&xmax, &out[2 * f + 1], sizeof(double));
    if (xmax > 0) worst = std::max(worst, dmax / xmax);
  }
  *max_rel = worst;
  return PNGF_OK;
}

extern "C" {

int pngf_drift_check(pngf_handle *ph, int nrows, double *max_rel) {
  Handle *h = H(ph);
  if (!h || !max_rel) return PNGF_ERR_ARG;
  return drift_impl(h, 0, h->cfg.num_freq, nrows, max_rel);
}

int pngf_drift_check_freq(pngf_handle *ph, int f, int nrows, double *max_rel) {
  pngf::TraceRange trace_("pngf_drift_check");
  Handle *h = H(ph);
  if (!h || !max_rel) return PNGF_ERR_ARG;
  if (f < 0 || f >= h->cfg.num_freq) return set_error(h, PNGF_ERR_ARG, "frequency index out of range");
  return drift_impl(h, f, f + 1, nrows, max_rel);
}

int pngf_refresh(pngf_handle *ph) {
  pngf::TraceRange trace_("pngf_refresh");
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  return prepare_impl(h, true);
}

int pngf_timing_enable(pngf_handle *ph, int on) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  timing_collect(h);
  h->tacc = pngf_timing{};
  h->nlaunch = 0;
  h->timing = on != 0;
  return PNGF_OK;
}

int pngf_timing_get(pngf_handle *ph, pngf_timing *out) {
  Handle *h = H(ph);
  if (!h || !out) return PNGF_ERR_ARG;
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  timing_collect(h);
  *out = h->tacc;
  out->kernel_launches = h->nlaunch;
  return PNGF_OK;
}

}  // extern "C"

// Times the complex64 update at each output tile width with zero operands
// (T, y and R are then left unchanged) and keeps the fastest.
static int tune_update(Handle *h, pngf_tune *out) {
  if (h->cfg.precision != PNGF_PREC_C64) return PNGF_OK;
  // widths for accepts (rank <= kAccTuneRank) and for build chunks / flushes
  const int widths[2] = {128, 64};
  const int ks[2] = {std::min(h->kmax, kAccTuneRank), kC64BuildChunk};
  const int k = std::max(ks[0], ks[1]);
  const long rows = h->n + h->E;
  int rc = lanes_fork(h);  // frequency 0's lane runs the timed updates
  if (rc) return rc;
  Lane &L = lane_of(h, 0);
  cudaStream_t st = lane_stream(h, 0);
  PNGF_CUDA(h, cudaMemsetAsync(L.A, 0, sizeof(double2) * rows * k, st));
  PNGF_CUDA(h, cudaMemsetAsync(L.W, 0, sizeof(double2) * k * h->ldm, st));
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return set_error(h, PNGF_ERR_CUDA, "event creation failed");
  }
  const long nl0 = h->nlaunch;
  const bool timing = h->timing;
  h->timing = false;
  const int reps = 3;
  double best[2] = {1e300, 1e300};
  int bi[2] = {0, 0};
  cudaError_t e = cudaSuccess;
  // entries 0, 1: the widths at the accept rank; 2, 3: at the build chunk rank
  for (int kc = 0; kc < 2 && e == cudaSuccess; ++kc)
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
      const int ent = 2 * kc + i;
      h->c64_cols = h->c64_cols_build = widths[i];
      out->update_cols[ent] = widths[i];
      out->update_us[ent] = -1.0;
      if ((e = launch_c64_update(h, 0, ks[kc])) != cudaSuccess) break;  // warm-up
      cudaEventRecord(a, st);
      for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch_c64_update(h, 0, ks[kc]);
      cudaEventRecord(b, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(b);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
      out->update_us[ent] = 1e3 * ms / reps;
      if (out->update_us[ent] < best[kc]) {
        best[kc] = out->update_us[ent];
        bi[kc] = i;
      }
    }
  h->timing = timing;
  h->nlaunch = nl0;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  h->c64_cols = widths[bi[0]];
  h->c64_cols_build = widths[bi[1]];
  out->update_form = bi[0];
  out->update_forms = 4;
  if (e != cudaSuccess) return cuda_check(h, e, "autotune (update)");
  if ((rc = lanes_join(h))) return rc;
  int tc = 0;
  PNGF_CUDA(h, cudaMemcpy(&tc, h->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (tc != 0) {
    cudaMemset(h->d_tc_err, 0, sizeof(int));
    return set_error(h, PNGF_ERR_TIMEOUT, "tensor-core update gave up waiting (code " + std::to_string(tc) + ")");
  }
  return PNGF_OK;
}

extern "C" {

int pngf_inject_update_timeout(pngf_handle *ph, int code) {
  Handle *h = H(ph);
  if (!h || code == 0) return PNGF_ERR_ARG;
  PNGF_CUDA(h, cudaStreamSynchronize(h->stream));
  PNGF_CUDA(h, cudaMemcpy(h->d_tc_err, &code, sizeof(int), cudaMemcpyHostToDevice));
  return PNGF_OK;
}

int pngf_set_eval_form(pngf_handle *ph, int form) {
  Handle *h = H(ph);
  if (!h) return PNGF_ERR_ARG;
  if (!eval_variant_ok(h, form)) return set_error(h, PNGF_ERR_UNSUPPORTED, "candidate-kernel form does not apply");
  h->eval_variant = h->eval_variant_small = form;
  return PNGF_OK;
}

int pngf_autotune(pngf_handle *ph, pngf_tune *out) {
  pngf::TraceRange trace_("pngf_autotune");
  Handle *h = H(ph);
  if (!h || !out) return PNGF_ERR_ARG;
  if (!h->prepared) return set_error(h, PNGF_ERR_STATE, "pngf_prepare has not been called for this design");
  std::memset(out, 0, sizeof(*out));
  // Every tile once as a single-tile candidate: the shape of a DBS pass.
  const int mf = h->cfg.max_flips, nc = h->map_sz;
  std::vector<int> tiles((size_t)nc * mf, 0), nfl(nc, 1);
  for (int i = 0; i < nc; ++i) tiles[(size_t)i * mf] = i;
  int rc = eval_batch(h, tiles.data(), nfl.data(), nc, 0.0, nullptr);
  if (rc) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return set_error(h, PNGF_ERR_CUDA, "event creation failed");
  }
  const int reps = 5;
  const long nl0 = h->nlaunch;
  cudaError_t e = cudaSuccess;
  // every form on the whole pass, then on the first kSmallBatch candidates of
  // it (the batches adaptive and proposal-driven decisions launch)
  const int nsmall = std::min(nc, kSmallBatch);
  int bestv[2] = {0, 0};
  h->eval_variant_small = -1;
  for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
    const int nb = pass == 0 ? nc : nsmall;
    double *us = pass == 0 ? out->eval_us : out->eval_us_small;
    double best = 1e300;
    for (int v = 0; v < kEvalVariants && e == cudaSuccess; ++v) {
      out->warps_per_cand[v] = kEvalForms[v].warps_per_cand;
      out->cands_per_cta[v] = kEvalForms[v].cands_per_cta;
      us[v] = -1.0;
      if (!eval_variant_ok(h, v)) continue;
      h->eval_variant = h->eval_variant_small = v;
      if ((e = launch_eval(h, nb, 0.0)) != cudaSuccess) break;  // warm-up
      cudaEventRecord(a, h->stream);
      for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch_eval(h, nb, 0.0);
      cudaEventRecord(b, h->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(b);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
      us[v] = 1e3 * ms / reps;
      if (us[v] < best) {
        best = us[v];
        bestv[pass] = v;
      }
    }
  }
  out->eval_forms = kEvalVariants;
  out->batch = nc;
  out->batch_small = nsmall;
  h->nlaunch = nl0;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  h->eval_variant = bestv[0];
  h->eval_variant_small = bestv[1];
  out->eval_form = bestv[0];
  out->eval_form_small = bestv[1];
  h->batch_valid = false;
  if (e != cudaSuccess) return cuda_check(h, e, "autotune");
  return tune_update(h, out);
}

}  // extern "C"

// Bounds-checked build only: the violations the data-dependent gathers
// recorded (see bounds.cuh), summed over the kernel files; first[3] = kind,
// row and column of one of the first. reset != 0 clears the records.
extern "C" int pngf_bounds_check_report(long long *violations, long long *first, int reset) {
#ifndef PNGF_BOUNDS_CHECK
  (void)violations;
  (void)first;
  (void)reset;
  return PNGF_ERR_UNSUPPORTED;
#else
  if (!violations) return PNGF_ERR_ARG;
  long long a[4], b[4];
  if (pngf::bounds_read_fp64(a, reset != 0) != cudaSuccess || pngf::bounds_read_f64tc(b, reset != 0) != cudaSuccess)
    return PNGF_ERR_CUDA;
  *violations = a[0] + b[0];
  if (first) {
    const long long *src = a[0] ? a : b;
    for (int q = 0; q < 3; ++q) first[q] = src[q + 1];
  }
  return PNGF_OK;
#endif
}
