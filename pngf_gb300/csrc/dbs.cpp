// Native DBS driver: the loop of pngf-opt/main.cpp:181-459 over the GPU hot
// path, with speculative batches.
//
// The reference evaluates one draw at a time and accepts the first improving
// one, then refills the hat (main.cpp:343-456). Here each launch evaluates the
// next B draws of the hat at once; the decisions are then taken in draw
// order against the same F_best, so the first improving draw of the batch is
// exactly the reference's next accept. Draws after it were speculative: the
// hat (engine state, entries, last_tried) is restored to its state at the
// start of the batch and replayed up to the accepted draw before being
// refilled, so the random sequence is the reference's.
//
// MagicHat (pngf-opt/magichat.hpp:32-111) uses std::mt19937 and
// std::uniform_int_distribution<>; its draws depend on the C++ library, so
// this driver stays in C++ and uses the same two standard components. The
// device-resident form of the loop (dbs_device.cu, pngf_dbs_set_device_loop)
// restates them (hat_rng.h) and is checked against them before it starts.
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <limits>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "pngf_internal.h"

namespace {

class Hat {
 public:
  Hat(int seed, int entries) : total_(entries), left_(entries), entry_(entries) {
    gen_.seed(seed);
    dis_ = std::uniform_int_distribution<>(0, entries - 1);
    for (int i = 0; i < entries; ++i) entry_[i] = i;
  }
  int rand_binary() {
    ++binary_draws_;
    return gen_() & 1;
  }
  long binary_draws() const { return binary_draws_; }
  // Whether the restated stream m (hat_rng.h), taken to this hat's engine
  // state, reproduces its bounded draws over every range a hat uses.
  bool restated_matches(const pngf::MtState &m0) const {
    std::mt19937 g = gen_;
    std::uniform_int_distribution<> d;
    pngf::MtState m = m0;
    int used = 0;
    for (int i = 0; i < 4096; ++i) {
      const int range = 1 + (int)((i * 7919L) % total_);
      d.param(std::uniform_int_distribution<int>::param_type(0, range - 1));
      if (d(g) != (int)pngf::mt_below(&m, (uint32_t)range, &used)) return false;
    }
    return true;
  }
  int draw() {
    if (left_ <= 0) return -1;
    dis_.param(std::uniform_int_distribution<int>::param_type(0, left_ - 1));
    const int idx = dis_(gen_);
    const int val = entry_[idx];
    entry_[idx] = entry_[left_ - 1];
    --left_;
    return val;
  }
  void reset() {
    for (int i = 0; i < total_; ++i) entry_[i] = i;
    left_ = total_;
  }
  int left() const { return left_; }

 private:
  int total_, left_;
  long binary_draws_ = 0;
  std::vector<int> entry_;
  std::mt19937 gen_;
  std::uniform_int_distribution<> dis_;
};

struct Cand {
  int log_index;  // tx + ty * tiles_x (what Logger::record_flip stores, main.cpp:426)
  int nflip;
  int tiles[4];
};

}  // namespace

struct pngf_dbs {
  pngf::Handle *h = nullptr;
  pngf_dbs_params p{};
  Hat hat{1, 1};
  int last_tried = -1;
  int hat_entries = 0;
  int mid_x = 0, mid_y = 0, qx = 0;
  bool converged = false, done = false;
  double F_init = 0.0, F_best = 0.0;
  std::vector<double> perf0;
  long evals = 0, accepts = 0, launched = 0;
  long drift_checks = 0, refreshes = 0;
  double drift_max = 0.0;
  std::vector<int> init_map;
  // log
  std::vector<int> lg_tile, lg_acc;
  std::vector<double> lg_F, lg_Fb, lg_perf;
  // learned proposals (optional)
  pngf_prop *prop = nullptr;
  int topk = 0, train_every = 0, train_steps = 0, train_batch = 32;
  int prop_rule = PNGF_PROP_BEST;  // which improving flip of an exact batch is accepted
  float train_lr = 1e-3f;
  long prop_steps = 0, prop_hits = 0, full_passes = 0;
  // the batch being evaluated: hat state at its start, its draws, staging
  Hat pend_hat{1, 1};
  int pend_last = -1;
  int adapt_B = 0;  // adaptive batch size (batch < 0)
  std::vector<Cand> pend;
  bool pend_exhausted = false;
  std::vector<int> tiles, nflip;
  // device-resident decisions (pngf_dbs_set_device_loop)
  pngf::DevLoop *dev = nullptr;
  long dev_launches = 0, dev_decisions = 0;
};

extern "C" {
int pngf_prop_record(pngf_prop *p, const int *tiles, const double *gains, int count);
int pngf_prop_predict(pngf_prop *p, float *pred);
int pngf_prop_train(pngf_prop *p, int steps, int batch, float lr, float *loss);
long pngf_prop_num_samples(const pngf_prop *p);
}

namespace {

pngf::HatGeom hat_geom(const pngf_dbs *d) {
  return pngf::HatGeom{d->h->cfg.tiles_x, d->h->cfg.tiles_y, d->qx, d->mid_x, d->mid_y,
                       d->p.mode == PNGF_DBS_SYMMETRIC ? 1 : 0};
}

// Draws the next valid candidate (main.cpp:343-392); false when the hat is empty.
bool next_candidate(pngf_dbs *d, Cand *c) {
  const pngf::HatGeom g = hat_geom(d);
  while (true) {
    const int r = d->hat.draw();
    if (r < 0) return false;
    if (pngf::hat_candidate(g, r, &d->last_tried, &c->log_index, &c->nflip, c->tiles)) return true;
  }
}

// Complex64 state: every drift_every accepts, an FP64 drift check of 4 sampled
// rows of T at one frequency (frequencies in turn); the state is rebuilt from
// G when the drift exceeds drift_tol -- in the handle's own build form (a
// complex64 build for PNGF_BUILD_C64, whose fresh state is within the drift
// tolerance and costs a fifth of an FP64 build), else in FP64.
int drift_after_accept(pngf_dbs *d) {
  pngf::Handle *h = d->h;
  if (h->cfg.precision != PNGF_PREC_C64 || d->p.drift_every <= 0 || d->accepts % d->p.drift_every != 0)
    return PNGF_OK;
  double rel = 0.0;
  pngf_handle *ph = reinterpret_cast<pngf_handle *>(h);
  int rc = pngf_drift_check_freq(ph, (int)(d->drift_checks % h->cfg.num_freq), 4, &rel);
  if (rc) return rc;
  ++d->drift_checks;
  d->drift_max = std::max(d->drift_max, rel);
  if (d->p.drift_tol > 0 && rel > d->p.drift_tol) {
    rc = h->cfg.c64_build == PNGF_BUILD_C64 ? pngf_prepare(ph) : pngf_refresh(ph);
    if (rc || (rc = pngf_objective(ph, &d->F_best))) return rc;
    ++d->refreshes;
  }
  return PNGF_OK;
}

void log_row(pngf_dbs *d, const Cand &c, int acc, double F, const double *perf, int nf) {
  d->lg_tile.push_back(c.log_index);
  d->lg_acc.push_back(acc);
  d->lg_F.push_back(F);
  d->lg_Fb.push_back(d->F_best);
  d->lg_perf.insert(d->lg_perf.end(), perf, perf + 3 * nf);
}

// Proposal-driven decision (no reference counterpart): the network's top-k
// single-tile flips are evaluated exactly and an improving one is accepted --
// the best (PNGF_PROP_BEST) or the first in predicted order (PNGF_PROP_FIRST);
// if none improves, an exact pass over every other candidate tile follows (in
// predicted order), and if that finds nothing either the design is a local
// minimum.
int proposal_step(pngf_dbs *d, int *accepted) {
  pngf::Handle *h = d->h;
  const int map_sz = h->map_sz, nf = h->cfg.num_freq, mf = h->cfg.max_flips;
  const int xsz = h->cfg.tiles_x;
  std::vector<int> elig;
  for (int t = 0; t < map_sz; ++t) {
    const int ty = t / xsz, tx = t - ty * xsz;
    if (ty == d->mid_y && (tx == d->mid_x || tx == d->mid_x - 1 || tx == d->mid_x + 1)) continue;
    elig.push_back(t);
  }
  // Evaluates `list` exactly, records the gains, logs the rows and returns the
  // index (into list) of the best improving flip, or -1.
  auto run_batch = [&](const std::vector<int> &list, pngf::EvalOut &o, int *best) -> int {
    const int n = (int)list.size();
    std::vector<int> tiles((size_t)n * mf, 0), nflip(n, 1);
    for (int i = 0; i < n; ++i) tiles[(size_t)i * mf] = list[i];
    int rc = pngf::eval_batch(h, tiles.data(), nflip.data(), n, d->F_best, &o);
    if (rc) return rc;
    d->launched += n;
    d->evals += n;
    std::vector<double> gains(n);
    for (int i = 0; i < n; ++i) gains[i] = o.F[i] - d->F_best;
    if ((rc = pngf_prop_record(d->prop, list.data(), gains.data(), n))) return rc;
    *best = -1;
    for (int i = 0; i < n; ++i)
      if (o.F[i] < d->F_best && (*best < 0 || (d->prop_rule == PNGF_PROP_BEST && o.F[i] < o.F[*best]))) *best = i;
    for (int i = 0; i < n; ++i) {
      Cand c{list[i], 1, {list[i], 0, 0, 0}};
      log_row(d, c, i == *best, o.F[i], o.perf.data() + (size_t)i * nf * 3, nf);
    }
    return PNGF_OK;
  };
  auto take = [&](const std::vector<int> &list, pngf::EvalOut &o, int best) -> int {
    // the tensor-core kernels' status is read at the next batch's collect
    int rc = pngf::accept_cand_async(h, best, o.k[best], false);
    if (rc) return rc;
    d->F_best = o.F[best];
    ++d->accepts;
    if (accepted) *accepted = 1;
    (void)list;
    return drift_after_accept(d);
  };
  int rc;
  ++d->prop_steps;
  if (d->train_every > 0 && d->prop_steps % d->train_every == 0 && pngf_prop_num_samples(d->prop) > 0) {
    float loss = 0.f;
    if ((rc = pngf_prop_train(d->prop, d->train_steps, d->train_batch, d->train_lr, &loss))) return rc;
  }
  pngf::EvalOut o;
  int best = -1;
  std::vector<int> full(elig);  // the fallback pass, in predicted order when there are predictions
  if (pngf_prop_num_samples(d->prop) > 0) {
    std::vector<float> pred(map_sz);
    if ((rc = pngf_prop_predict(d->prop, pred.data()))) return rc;
    std::stable_sort(full.begin(), full.end(), [&](int a, int b) { return pred[a] < pred[b]; });
    const int nt = std::min<int>(d->topk, (int)full.size());
    std::vector<int> order(full.begin(), full.begin() + nt);
    if ((rc = run_batch(order, o, &best))) return rc;
    if (best >= 0) {
      ++d->prop_hits;
      return take(order, o, best);
    }
    // none of them improves: the fallback pass takes the rest, in predicted
    // order (its best improving flip is the best of all eligible flips)
    full.erase(full.begin(), full.begin() + nt);
  }
  if (full.empty()) {  // the top k were every eligible flip
    d->converged = d->done = true;
    return PNGF_OK;
  }
  ++d->full_passes;
  if ((rc = run_batch(full, o, &best))) return rc;
  if (best >= 0) return take(full, o, best);
  d->converged = d->done = true;
  return PNGF_OK;
}

// First half of a DBS decision: draws the next speculative batch in hat
// order (main.cpp:343-392) and stages it on the handle (eval_stage).
// *have = false when the run is over (evaluation budget spent or hat empty).
int batch_draw(pngf_dbs *d, bool *have) {
  *have = false;
  if (d->done) return PNGF_OK;
  pngf::Handle *h = d->h;
  const int mf = h->cfg.max_flips;
  const long budget = d->p.max_evals > 0 ? d->p.max_evals - d->evals : std::numeric_limits<long>::max();
  if (budget <= 0) {
    d->done = true;
    return PNGF_OK;
  }
  d->pend_hat = d->hat;
  d->pend_last = d->last_tried;
  // batch > 0: fixed; 0: the whole remaining hat; < 0: adaptive, -batch draws
  // after an accept, doubling after every batch without one
  if (d->p.batch < 0 && d->adapt_B <= 0) d->adapt_B = -d->p.batch;
  int B = d->p.batch > 0 ? d->p.batch : d->p.batch < 0 ? d->adapt_B : std::max(1, d->hat.left());
  B = (int)std::min<long>(B, budget);
  d->pend.clear();
  d->pend_exhausted = false;
  while ((int)d->pend.size() < B) {
    Cand c;
    if (!next_candidate(d, &c)) {
      d->pend_exhausted = true;
      break;
    }
    d->pend.push_back(c);
  }
  if (d->pend.empty()) {
    d->converged = d->done = true;
    return PNGF_OK;
  }
  const int nc = (int)d->pend.size();
  d->tiles.assign((size_t)nc * mf, 0);
  d->nflip.resize(nc);
  for (int i = 0; i < nc; ++i) {
    d->nflip[i] = d->pend[i].nflip;
    for (int t = 0; t < d->pend[i].nflip; ++t) d->tiles[(size_t)i * mf + t] = d->pend[i].tiles[t];
  }
  const int rc = pngf::eval_stage(h, d->tiles.data(), d->nflip.data(), nc, d->F_best);
  if (rc) return rc;
  d->launched += nc;
  *have = true;
  return PNGF_OK;
}

// Second half: reads the batch's results and takes the reference's decisions
// in draw order against the same F_best (main.cpp:401-456): logs every draw
// up to the first improving one, accepts it, restores the hat to the start of
// the batch, replays it to just after that draw and refills it. Draws after it
// were speculative. With sync_accept = false the accept's launches are not
// waited for (their bounded-wait status is read with the next batch).
int batch_finish(pngf_dbs *d, int *accepted, bool sync_accept) {
  if (accepted) *accepted = 0;
  pngf::Handle *h = d->h;
  const int nf = h->cfg.num_freq;
  pngf::EvalOut o;
  int rc = pngf::eval_collect(h, &o);
  if (rc) return rc;
  const int nc = (int)d->pend.size();
  if (d->prop && d->p.mode == PNGF_DBS_SINGLE) {  // every exact evaluation is a training pair
    std::vector<int> tl(nc);
    std::vector<double> gains(nc);
    for (int i = 0; i < nc; ++i) {
      tl[i] = d->pend[i].tiles[0];
      gains[i] = o.F[i] - d->F_best;
    }
    if ((rc = pngf_prop_record(d->prop, tl.data(), gains.data(), nc))) return rc;
  }
  const int j = o.first;
  const int upto = j >= 0 ? j : nc - 1;
  for (int i = 0; i <= upto; ++i) {
    for (int f = 0; f < nf; ++f)
      if (o.status[(size_t)i * nf + f] == PNGF_ERR_ARG)
        return pngf::set_error(h, PNGF_ERR_ARG, "invalid candidate produced by the driver");
    log_row(d, d->pend[i], i == j, o.F[i], o.perf.data() + (size_t)i * nf * 3, nf);
  }
  d->evals += upto + 1;
  if (j >= 0) {
    if ((rc = pngf::accept_cand_async(h, j, o.k[j], sync_accept))) return rc;
    d->F_best = o.F[j];
    ++d->accepts;
    d->hat = d->pend_hat;  // replay to just after draw j, then refill (main.cpp:455)
    d->last_tried = d->pend_last;
    for (int i = 0; i <= j; ++i) {
      Cand c;
      next_candidate(d, &c);
    }
    d->hat.reset();
    if (accepted) *accepted = 1;
    d->adapt_B = -d->p.batch;
    return drift_after_accept(d);
  }
  if (d->p.batch < 0) d->adapt_B = (int)std::min<long>(2L * d->adapt_B, 1L << 20);
  if (d->pend_exhausted) d->converged = d->done = true;
  return PNGF_OK;
}

// One DBS decision on the device-resident loop: decisions without an accept
// run on the GPU; an accept is performed here as on the host path.
// Takes a device-loop launch's outcome: the counters and, on an accept, the
// accept itself on the host path (not waited for: the next launch's decide
// kernel reads the tensor-core error flag before it decides). *more = the
// run continues without an accept (another launch is due).
int device_after(pngf_dbs *d, const pngf::DevLoopResult &r, int *accepted, bool *more) {
  pngf::Handle *h = d->h;
  *more = false;
  d->evals = r.evals;
  d->accepts = r.accepts;
  d->launched = r.launched;
  d->F_best = r.F_best;
  d->converged = r.converged != 0;
  d->done = r.done != 0;
  ++d->dev_launches;
  d->dev_decisions += r.decisions;
  if (r.err == 2) {
    d->done = true;
    cudaMemsetAsync(h->d_tc_err, 0, sizeof(int), h->stream);
    return pngf::set_error(h, PNGF_ERR_TIMEOUT,
                           "tensor-core update gave up waiting (code " + std::to_string(r.tc_code) + ")");
  }
  if (r.err) {
    d->done = true;
    return pngf::set_error(h, PNGF_ERR_ARG, "invalid candidate produced by the driver");
  }
  if (r.accepted) {
    int rc;
    if ((rc = pngf::adopt_device_batch(h, r.nc, r.j, r.tiles, r.nflip)) ||
        (rc = pngf::accept_cand_async(h, r.j, r.k, false)))
      return rc;
    if (accepted) *accepted = 1;
    const double fb = d->F_best;
    if ((rc = drift_after_accept(d))) return rc;
    if (!(d->F_best == fb) && (rc = pngf::devloop_set_fbest(h, d->dev, d->F_best))) return rc;
    return PNGF_OK;
  }
  *more = !d->done;
  return PNGF_OK;
}

int device_step(pngf_dbs *d, int *accepted) {
  pngf::Handle *h = d->h;
  pngf::DevLoopLog lg{d->lg_tile, d->lg_acc, d->lg_F, d->lg_Fb, d->lg_perf};
  bool more = !d->done;
  while (more) {
    pngf::DevLoopResult r{};
    int rc = pngf::devloop_run(h, d->dev, &r, &lg);
    if (rc) return rc;
    if ((rc = device_after(d, r, accepted, &more))) return rc;
  }
  return PNGF_OK;
}

}  // namespace

extern "C" {

int pngf_dbs_set_device_loop(pngf_dbs *d, int enable) {
  if (!d) return PNGF_ERR_ARG;
  pngf::Handle *h = d->h;
  if (d->evals > 0 || d->launched > 0 || d->done)
    return pngf::set_error(h, PNGF_ERR_STATE, "the device loop is chosen before the first step");
  if (!enable) {
    pngf::devloop_destroy(d->dev);
    d->dev = nullptr;
    return PNGF_OK;
  }
  if (d->dev) return PNGF_OK;
  if (d->prop)
    return pngf::set_error(h, PNGF_ERR_UNSUPPORTED, "learned proposals run on the host driver");
  pngf::MtState m;
  pngf::mt_seed(&m, (uint32_t)d->p.seed);
  for (long i = 0; i < d->hat.binary_draws(); ++i) pngf::mt_next(&m);
  if (!d->hat.restated_matches(m))
    return pngf::set_error(h, PNGF_ERR_UNSUPPORTED,
                           "this C++ library's MagicHat stream differs from the device restatement");
  pngf::DevLoopConfig cfg{hat_geom(d), d->hat_entries, d->p.batch, d->p.max_evals, (unsigned)d->p.seed,
                          d->hat.binary_draws(), d->F_best};
  return pngf::devloop_create(h, cfg, &d->dev);
}

int pngf_dbs_set_proposal(pngf_dbs *d, pngf_prop *p, int topk, int train_every, int train_steps, int train_batch,
                          float lr) {
  if (!d) return PNGF_ERR_ARG;
  if (p && d->p.mode != PNGF_DBS_SINGLE)
    return pngf::set_error(d->h, PNGF_ERR_UNSUPPORTED, "proposals apply to single-tile candidates");
  if (p && d->dev)
    return pngf::set_error(d->h, PNGF_ERR_UNSUPPORTED, "learned proposals run on the host driver");
  d->prop = p;
  d->topk = topk;
  d->train_every = train_every;
  d->train_steps = train_steps;
  d->train_batch = train_batch > 0 ? train_batch : 32;
  d->train_lr = lr > 0 ? lr : 1e-3f;
  return PNGF_OK;
}

int pngf_dbs_set_proposal_rule(pngf_dbs *d, int rule) {
  if (!d || (rule != PNGF_PROP_BEST && rule != PNGF_PROP_FIRST)) return PNGF_ERR_ARG;
  d->prop_rule = rule;
  return PNGF_OK;
}

int pngf_dbs_begin(pngf_handle *ph, const pngf_dbs_params *p, pngf_dbs **out) {
  pngf::Handle *h = reinterpret_cast<pngf::Handle *>(ph);
  if (!h || !p || !out) return PNGF_ERR_ARG;
  *out = nullptr;
  if (p->seed == 0) return pngf::set_error(h, PNGF_ERR_ARG, "seed 0 (random seed) is not reproducible; pass one");
  if (p->mode != PNGF_DBS_SYMMETRIC && p->mode != PNGF_DBS_SINGLE) return PNGF_ERR_ARG;
  const int xsz = h->cfg.tiles_x, ysz = h->cfg.tiles_y;
  const int need_flips = p->mode == PNGF_DBS_SYMMETRIC ? 4 : 1;
  if (h->cfg.max_flips < need_flips)
    return pngf::set_error(h, PNGF_ERR_ARG, "handle max_flips too small for this candidate mode");
  pngf_dbs *d = new (std::nothrow) pngf_dbs();
  if (!d) return PNGF_ERR_NOMEM;
  d->h = h;
  d->p = *p;
  d->qx = (int)((xsz - 1) * 0.5 + 1);
  const int qy = (int)((ysz - 1) * 0.5 + 1);
  d->hat_entries = p->mode == PNGF_DBS_SYMMETRIC ? d->qx * qy - 1 : xsz * ysz;  // main.cpp:181
  d->hat = Hat(p->seed, d->hat_entries);
  std::vector<int> tm(xsz * ysz, 0);
  if (p->init == PNGF_INIT_RANDOM) {
    if (p->mode == PNGF_DBS_SYMMETRIC) {  // main.cpp:187-208
      for (int j = 0; j < (ysz - 1) * 0.5 + 1; j++)
        for (int i = 0; i < (xsz - 1) * 0.5 + 1; i++) {
          const int st = d->hat.rand_binary();
          tm[i + j * xsz] = st;
          if (i < (xsz - 1) * 0.5) tm[((xsz - 1) - i) + j * xsz] = st;
          if (j < (ysz - 1) * 0.5) {
            tm[i + ((ysz - 1) - j) * xsz] = st;
            if (i < (xsz - 1) * 0.5) tm[((xsz - 1) - i) + ((ysz - 1) - j) * xsz] = st;
          }
        }
    } else {
      for (int i = 0; i < xsz * ysz; ++i) tm[i] = d->hat.rand_binary();
    }
  }
  d->mid_x = (int)((xsz - 1) * 0.5);
  d->mid_y = (int)((ysz - 1) * 0.5);
  tm[d->mid_y * xsz + d->mid_x - 1] = 1;  // main.cpp:215-219
  tm[d->mid_y * xsz + d->mid_x + 1] = 1;
  tm[d->mid_y * xsz + d->mid_x] = 0;
  tm[(d->mid_y - 1) * xsz + d->mid_x] = 0;
  tm[(d->mid_y + 1) * xsz + d->mid_x] = 0;
  d->init_map = tm;
  int rc;
  if ((rc = pngf_set_tile_map(ph, tm.data())) || (rc = pngf_set_source_port(ph, d->mid_x, d->mid_y, 1, 2)) ||
      (rc = pngf_prepare(ph)) || (rc = pngf_objective(ph, &d->F_best))) {
    delete d;
    return rc;
  }
  d->perf0.resize(3 * h->cfg.num_freq);
  cudaMemcpy(d->perf0.data(), h->d_perf, sizeof(double) * d->perf0.size(), cudaMemcpyDeviceToHost);
  d->F_init = d->F_best;
  *out = d;
  return PNGF_OK;
}

int pngf_dbs_step(pngf_dbs *d, int *accepted) {
  pngf::TraceRange trace_("pngf_dbs_step");
  if (!d) return PNGF_ERR_ARG;
  if (accepted) *accepted = 0;
  if (d->prop && d->topk > 0) return d->done ? PNGF_OK : proposal_step(d, accepted);
  if (d->dev) return device_step(d, accepted);
  while (!d->done) {
    bool have = false;
    int rc = batch_draw(d, &have);
    if (rc || !have) return rc;
    if ((rc = pngf::eval_enqueue(d->h))) return rc;
    int acc = 0;
    // the accept is not waited for: the next batch queues behind it and its
    // read-back carries the tensor-core status
    if ((rc = batch_finish(d, &acc, false))) return rc;
    if (acc) {
      if (accepted) *accepted = 1;
      return PNGF_OK;
    }
  }
  return PNGF_OK;
}

int pngf_dbs_stats_get(const pngf_dbs *d, pngf_dbs_stats *out) {
  if (!d || !out) return PNGF_ERR_ARG;
  out->evals = d->evals;
  out->accepts = d->accepts;
  out->launched = d->launched;
  out->converged = d->converged ? 1 : 0;
  out->F_init = d->F_init;
  out->F_best = d->F_best;
  out->drift_checks = d->drift_checks;
  out->refreshes = d->refreshes;
  out->drift_max = d->drift_max;
  out->prop_hits = d->prop_hits;
  out->full_passes = d->full_passes;
  out->device_launches = d->dev_launches;
  out->device_decisions = d->dev_decisions;
  return PNGF_OK;
}

int pngf_dbs_log(const pngf_dbs *d, long cap, int *tile, int *accept, double *F, double *F_best, double *perf,
                 long *rows) {
  if (!d) return PNGF_ERR_ARG;
  const long n = (long)d->lg_tile.size();
  const long m = std::min(cap, n);
  const int nf = d->h->cfg.num_freq;
  if (tile) std::copy(d->lg_tile.begin(), d->lg_tile.begin() + m, tile);
  if (accept) std::copy(d->lg_acc.begin(), d->lg_acc.begin() + m, accept);
  if (F) std::copy(d->lg_F.begin(), d->lg_F.begin() + m, F);
  if (F_best) std::copy(d->lg_Fb.begin(), d->lg_Fb.begin() + m, F_best);
  if (perf) std::copy(d->lg_perf.begin(), d->lg_perf.begin() + (size_t)m * 3 * nf, perf);
  if (rows) *rows = n;
  return PNGF_OK;
}

// Logger::save's format (logger.hpp:75-106): "seed rows", initial map, one
// line per record (index, flip index, decision, perf...), final map. The
// first record is the starting point (main.cpp:328). The final map is the
// design after the last accept.
int pngf_dbs_save_log(const pngf_dbs *d, const char *path) {
  if (!d || !path) return PNGF_ERR_ARG;
  std::ofstream o(path);
  if (!o) return PNGF_ERR_IO;
  const int nf = d->h->cfg.num_freq;
  const long n = (long)d->lg_tile.size();
  o << d->p.seed << " " << n + 1 << std::endl;
  for (int v : d->init_map) o << (v ? "x" : ".");
  o << std::endl;
  o << 0 << " " << -1 << " " << -1 << " " << d->F_init << " " << d->F_init << " ";
  for (int i = 0; i < 3 * nf; ++i) o << d->perf0[i] << " ";
  o << std::endl;
  for (long r = 0; r < n; ++r) {
    o << r + 1 << " " << d->lg_tile[r] << " " << d->lg_acc[r] << " " << d->lg_F[r] << " " << d->lg_Fb[r] << " ";
    for (int i = 0; i < 3 * nf; ++i) o << d->lg_perf[(size_t)r * 3 * nf + i] << " ";
    o << std::endl;
  }
  for (int v : d->h->tile_map) o << (v ? "x" : ".");
  o << std::endl;
  return o ? PNGF_OK : PNGF_ERR_IO;
}

int pngf_dbs_end(pngf_dbs *d) {
  if (d) pngf::devloop_destroy(d->dev);
  delete d;
  return PNGF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Groups of independent DBS runs stepped together (no reference counterpart).
//
// A group step draws every unfinished member's next speculative batch on the
// host, then launches all their evaluations at once: with graphs on, as one
// CUDA graph (captured from the members' streams, forked from and joined to
// the group's stream) that is replayed while the members' batch sizes and
// staging buffers stay the same, else as each member's launches on its own
// stream. The group then reads every member's results and takes its decision
// exactly as pngf_dbs_step does, launching the accept without waiting, so the
// members' accept updates run concurrently on their streams while the host
// draws the next batches. A member's flips, objectives and log are therefore
// those of pngf_dbs_step on that member alone.

struct pngf_group {
  std::vector<pngf_dbs *> m;
  bool graphs = false;
  cudaStream_t s0 = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> ready, join;
  cudaGraphExec_t exec = nullptr;
  std::vector<long> key;  // per member: batch size and staging addresses the graph was captured with
  long graph_nodes_launches = 0;
  // device-resident members: one graph holding every member's decision loop
  bool device = false;
  cudaGraph_t dgraph = nullptr;
  cudaGraphExec_t dexec = nullptr;
  pngf_group_stats st{};
};

namespace {

void group_release(pngf_group *g) {
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->dexec) cudaGraphExecDestroy(g->dexec);
  if (g->dgraph) cudaGraphDestroy(g->dgraph);
  for (cudaEvent_t e : g->ready)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : g->join)
    if (e) cudaEventDestroy(e);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->s0) cudaStreamDestroy(g->s0);
  delete g;
}

int group_err(pngf_group *g, cudaError_t e, const char *what) {
  return pngf::cuda_check(g->m[0]->h, e, what);
}

// Captures the staged batches of the members marked in `on` into one graph.
int group_capture(pngf_group *g, const std::vector<char> &on) {
  if (g->exec) {
    cudaGraphExecDestroy(g->exec);
    g->exec = nullptr;
  }
  cudaError_t e = cudaStreamBeginCapture(g->s0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return group_err(g, e, "cudaStreamBeginCapture");
  int rc = PNGF_OK;
  long nl = 0;
  e = cudaEventRecord(g->fork, g->s0);
  for (size_t i = 0; i < g->m.size() && e == cudaSuccess && rc == PNGF_OK; ++i) {
    if (!on[i]) continue;
    pngf::Handle *h = g->m[i]->h;
    if ((e = cudaStreamWaitEvent(h->stream, g->fork, 0)) != cudaSuccess) break;
    const long l0 = h->nlaunch;
    h->capturing = true;
    rc = pngf::eval_enqueue(h);
    h->capturing = false;
    nl += h->nlaunch - l0;
    if (rc == PNGF_OK && (e = cudaEventRecord(g->join[i], h->stream)) == cudaSuccess)
      e = cudaStreamWaitEvent(g->s0, g->join[i], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(g->s0, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) return group_err(g, e, "graph capture of the members' batches");
  g->graph_nodes_launches = nl;
  ++g->st.captures;
  return PNGF_OK;
}

// Device-resident members: one graph whose root nodes are the members' WHILE
// loops (independent branches; each member draws, evaluates and decides on
// the device until its next accept), captured once and rebuilt only if a
// member's buffers or kernel forms change. A finished member's loop exits on
// its first iteration.
int group_device_build(pngf_group *g) {
  if (g->dexec) cudaGraphExecDestroy(g->dexec);
  if (g->dgraph) cudaGraphDestroy(g->dgraph);
  g->dexec = nullptr;
  g->dgraph = nullptr;
  cudaError_t e = cudaGraphCreate(&g->dgraph, 0);
  if (e != cudaSuccess) return group_err(g, e, "cudaGraphCreate");
  for (pngf_dbs *d : g->m) {
    const int rc = pngf::devloop_add_to_graph(d->h, d->dev, g->dgraph);
    if (rc) return rc;
  }
  if ((e = cudaGraphInstantiate(&g->dexec, g->dgraph, 0)) != cudaSuccess)
    return group_err(g, e, "instantiation of the members' decision loops");
  ++g->st.captures;
  return PNGF_OK;
}

int group_device_step(pngf_group *g, int *active) {
  const size_t nm = g->m.size();
  int rc, n_on = 0;
  bool stale = !g->dexec;
  for (pngf_dbs *d : g->m) {
    n_on += !d->done;
    stale = stale || !pngf::devloop_key_current(d->h, d->dev);
  }
  if (n_on > 0) {
    if (stale && (rc = group_device_build(g))) return rc;
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < nm && e == cudaSuccess; ++i) {  // after each member's earlier accepts
      pngf::Handle *h = g->m[i]->h;
      if ((rc = pngf::devloop_prepare(h, g->m[i]->dev))) return rc;
      if ((e = cudaEventRecord(g->ready[i], h->stream)) == cudaSuccess) e = cudaStreamWaitEvent(g->s0, g->ready[i], 0);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(g->dexec, g->s0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->s0);
    if (e != cudaSuccess) return group_err(g, e, "graph launch of the members' decision loops");
    ++g->st.rounds;
    ++g->st.graph_launches;
    for (size_t i = 0; i < nm; ++i) {  // outcomes and accepts, in member order
      pngf_dbs *d = g->m[i];
      if (d->done) continue;
      pngf::Handle *h = d->h;
      const long l0 = h->nlaunch;
      pngf::DevLoopLog lg{d->lg_tile, d->lg_acc, d->lg_F, d->lg_Fb, d->lg_perf};
      pngf::DevLoopResult r{};
      int acc = 0;
      bool more = false;
      if ((rc = pngf::devloop_collect(h, d->dev, &r, &lg)) || (rc = device_after(d, r, &acc, &more))) return rc;
      g->st.kernel_launches += h->nlaunch - l0;
      g->st.accepts += acc;
    }
  }
  int left = 0;
  for (size_t i = 0; i < nm; ++i) left += !g->m[i]->done;
  if (active) *active = left;
  return PNGF_OK;
}

}  // namespace

extern "C" {

int pngf_group_create(pngf_dbs *const *members, int count, int use_graphs, pngf_group **out) {
  if (!members || count <= 0 || !out) return PNGF_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    if (!members[i]) return PNGF_ERR_ARG;
    if (members[i]->prop && members[i]->topk > 0)
      return pngf::set_error(members[i]->h, PNGF_ERR_UNSUPPORTED, "proposal-driven runs are stepped on their own");
    if ((members[i]->dev != nullptr) != (members[0]->dev != nullptr))
      return pngf::set_error(members[i]->h, PNGF_ERR_UNSUPPORTED,
                             "a group's members all run device-resident decisions or none does");
    for (int j = 0; j < i; ++j)
      if (members[j]->h == members[i]->h)
        return pngf::set_error(members[i]->h, PNGF_ERR_ARG, "two group members share a handle");
  }
  pngf_group *g = new (std::nothrow) pngf_group();
  if (!g) return PNGF_ERR_NOMEM;
  g->m.assign(members, members + count);
  g->graphs = use_graphs != 0;
  g->device = members[0]->dev != nullptr;
  g->ready.assign(count, nullptr);
  g->join.assign(count, nullptr);
  cudaError_t e = cudaStreamCreateWithFlags(&g->s0, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  for (int i = 0; i < count && e == cudaSuccess; ++i) {
    e = cudaEventCreateWithFlags(&g->ready[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    const int rc = group_err(g, e, "group streams and events");
    group_release(g);
    return rc;
  }
  *out = g;
  return PNGF_OK;
}

int pngf_group_step(pngf_group *g, int *active) {
  pngf::TraceRange trace_("pngf_group_step");
  if (!g) return PNGF_ERR_ARG;
  if (g->device) return group_device_step(g, active);
  const size_t nm = g->m.size();
  std::vector<char> on(nm, 0);
  std::vector<long> key(3 * nm, 0);
  int rc, n_on = 0;
  for (size_t i = 0; i < nm; ++i) {  // draw and stage every unfinished member's batch
    bool have = false;
    if ((rc = batch_draw(g->m[i], &have))) return rc;
    on[i] = have;
    n_on += have;
    const pngf::Handle *h = g->m[i]->h;
    if (have) {
      key[3 * i] = h->staged_n;
      key[3 * i + 1] = reinterpret_cast<long>(h->h_tiles);
      key[3 * i + 2] = reinterpret_cast<long>(h->h_out);
    }
  }
  if (n_on > 0) {
    ++g->st.rounds;
    if (g->graphs) {
      if (key != g->key || !g->exec) {
        if ((rc = group_capture(g, on))) return rc;
        g->key = key;
      }
      cudaError_t e = cudaSuccess;
      for (size_t i = 0; i < nm && e == cudaSuccess; ++i) {  // after each member's earlier accepts
        if (!on[i]) continue;
        if ((e = cudaEventRecord(g->ready[i], g->m[i]->h->stream)) == cudaSuccess)
          e = cudaStreamWaitEvent(g->s0, g->ready[i], 0);
      }
      if (e == cudaSuccess) e = cudaGraphLaunch(g->exec, g->s0);
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->s0);
      if (e != cudaSuccess) return group_err(g, e, "graph launch of the members' batches");
      ++g->st.graph_launches;
      g->st.kernel_launches += g->graph_nodes_launches;
      for (size_t i = 0; i < nm; ++i) {  // the host-side effects of eval_enqueue, for the replay
        if (!on[i]) continue;
        pngf::Handle *h = g->m[i]->h;
        h->launched_n = h->batch_n = h->staged_n;
        h->batch_valid = true;
      }
    } else {
      for (size_t i = 0; i < nm; ++i) {
        if (!on[i]) continue;
        pngf::Handle *h = g->m[i]->h;
        const long l0 = h->nlaunch;
        if ((rc = pngf::eval_enqueue(h))) return rc;
        g->st.kernel_launches += h->nlaunch - l0;
      }
    }
    for (size_t i = 0; i < nm; ++i) {  // decisions, in member order
      if (!on[i]) continue;
      int acc = 0;
      pngf::Handle *h = g->m[i]->h;
      const long l0 = h->nlaunch;
      if ((rc = batch_finish(g->m[i], &acc, false))) return rc;
      g->st.kernel_launches += h->nlaunch - l0;
      g->st.accepts += acc;
    }
  }
  int left = 0;
  for (size_t i = 0; i < nm; ++i) left += !g->m[i]->done;
  if (active) *active = left;
  return PNGF_OK;
}

int pngf_group_stats_get(const pngf_group *g, pngf_group_stats *out) {
  if (!g || !out) return PNGF_ERR_ARG;
  *out = g->st;
  out->evals = 0;
  for (const pngf_dbs *d : g->m) out->evals += d->evals;
  return PNGF_OK;
}

int pngf_group_destroy(pngf_group *g) {
  if (!g) return PNGF_OK;
  for (pngf_dbs *d : g->m) cudaStreamSynchronize(d->h->stream);
  group_release(g);
  return PNGF_OK;
}

}  // extern "C"
