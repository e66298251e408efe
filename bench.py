#!/usr/bin/env python3
"""DBS flip-evaluation throughput of the PNGF hot path on GB300.

Workload (the plain wideband case): 21 x 21 tiles of 3 x 3 Yee cells
(N = 8064 design edges), 5 frequencies (27, 28.5, 30, 31.5, 33 GHz), one
synthetic complex128 G per frequency, single-tile candidates (441 per pass),
DBS from a 50%-fill random design drawn from seed 1, plain FP64 form.

A step is one DBS decision through the public C ABI (pngf_dbs_step): the
next draws of the hat are evaluated at every frequency in one speculative
launch, the first improving draw in hat order is accepted (rank-k update of
M at every frequency) and the hat is refilled -- exactly the reference's
sequence of evaluations and accepts. The metric counts flip evaluations in
the reference's sense (its flip_count), so speculative evaluations past the
accepted draw do not count.

  value  flip evals / device time of the hot-path kernels (CUDA events on the
         handle's stream around each launch group; G and M resident in HBM)
  e2e    flip evals / wall time of the same steps through the C ABI, host
         candidate lists in and results out every step

--impl reference times the reference algorithm (the oracle's C restatement
of pngf-opt/pngfopt.hpp on C^-1, OpenMP + OpenBLAS on every host core) on the
same workload, same steps.

Multi-GPU (--gpus N under torchrun): one independent DBS instance per GPU
(seed 1 + rank), no data-path exchange; weak scaling.
"""
from __future__ import annotations

import argparse
import json
import re
import os
import statistics
import subprocess
import sys
import tempfile
import time

# The CPU legs run OpenMP loops next to OpenBLAS's own thread pool; idle
# OpenMP threads must sleep rather than spin or the two pools fight for the
# cores (measured 4x slower). Set before any OpenMP runtime loads.
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FREQS = [27.0e9, 28.5e9, 30.0e9, 31.5e9, 33.0e9]
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "tc_update_f64_21x21.md")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--tiles", type=int, default=21)
    ap.add_argument("--mode", choices=["single", "sym"], default="single")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--batch", type=int, default=-16,
                    help="DBS speculative batch of the timed runs and of the plain convergence run: < 0 adaptive "
                         "(-batch draws after an accept, doubling after a batch without one), 0 = the whole "
                         "remaining hat, > 0 fixed; every size keeps the reference's evaluation order")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--device-loop", type=int, default=0,
                    help="1: DBS decisions without an accept run on the device (one CUDA graph with a WHILE node)")
    ap.add_argument("--forms", default="fp64,c64,c64d,sym",
                    help="forms to run (fp64 is the headline; c64, c64d: complex64 immediate / deferred; sym: the "
                         "4-fold mirror hat in FP64)")
    ap.add_argument("--nfreq", type=int, default=5, help="use the first NFREQ of the five frequencies")
    ap.add_argument("--no-converge", action="store_true",
                    help="skip the wall time to convergence, plain FP64 DBS against proposal + complex64 DBS")
    ap.add_argument("--no-group", action="store_true", help="skip the many-instance group run")
    ap.add_argument("--eval-probe", type=int, default=0,
                    help="profiling case for the candidate kernel: N passes of every tile at every frequency on a "
                         "state-only handle (G not kept), one JSON line; nothing else runs")
    ap.add_argument("--eval-form", type=int, default=1, help="--eval-probe: candidate-kernel form")
    ap.add_argument("--converge-seeds", type=int, default=5,
                    help="seeds of the 21x21 proposal + complex64 against plain FP64 comparison")
    ap.add_argument("--no-c5", action="store_true",
                    help="skip the reduced 41x41 x 4-frequency proposal comparison of the default run")
    ap.add_argument("--c5", action="store_true",
                    help="only the learned-proposal form at 41x41 tiles x 4 frequencies against plain FP64 DBS")
    ap.add_argument("--instances", type=int, default=64, help="group run: DBS instances")
    ap.add_argument("--group-evals", type=int, default=400, help="group run: flip evaluations per instance")
    ap.add_argument("--group-batch", type=int, default=64, help="group run: speculative batch per instance")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.2)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), power=float(f[3]), hw=f[5], hwt=f[6], swt=f[7],
                                 pcap=f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("pcap", "sw_power_cap")):
                if r[key].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "power_w_max": max(r["power"] for r in rows), "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_gemm_peak_tflops():
    """FP64 GEMM throughput of this GPU (cuBLAS DGEMM through torch, best of 5),
    the denominator for FP64-pipe-bound kernels (the measured-peaks file has
    no FP64 figure)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def make_Gs(tiles, freqs):
    """The workload's inputs, from the oracle's generator (oracle/synth.c, the
    same recipe as the library's): one synthetic G per frequency and the two
    NF2FF rows (broadside far-field projection), so that the objective's
    directivity term is live. Returns (Gs, rows)."""
    from oracle import synth
    return [synth.synth_G(tiles, tiles, f, seed=1) for f in freqs], synth.synth_gobj(tiles, tiles, seed=1)


def ldm_of(n):
    """Leading dimension of M on the device: N+1 rounded up to 16."""
    return (n + 1 + 15) // 16 * 16


METRIC = "DBS flip evals/s, 21x21 tiles x 5 frequencies, plain FP64 form"


def workload_config(a, n, nf, world):
    """The `config` object both arms print (identical for the same flags)."""
    return {
        "workload": "wideband %dx%d tiles x %d frequencies (27-33 GHz), N=%d edges, %s-tile DBS from a "
                    "50%%-fill random design (seed %d), synthetic complex-symmetric dyadic G with broadside NF2FF "
                    "rows" % (a.tiles, a.tiles, nf, n, a.mode, a.seed),
        "tiles": a.tiles, "freqs_ghz": [f / 1e9 for f in FREQS], "edges": n,
        "candidates_per_pass": a.tiles * a.tiles if a.mode == "single" else None,
        "precision": "fp64", "parallelism": "one DBS instance per GPU" if world > 1 else "single GPU",
        "l2": "inputs larger than L2: M is %.2f GB per frequency" % ((n + 3) * ldm_of(n) * 16 / 1e9),
        "step": "one DBS decision (evaluations in hat order until the first improving draw, which is accepted)",
    }


def cpu_baseline_sample(tiles, mode, seed, freq, gpu_evals, gpu_accepts, nf, budget_s=20.0):
    """The reference algorithm (C restatement, all host cores) on one of the
    frequencies: init, then DBS steps until ~budget_s of evaluation/accept work.
    Returns per-frequency eval and accept times and the modelled throughput on
    the GPU run's eval/accept mix at nf frequencies."""
    from oracle import synth
    from oracle.dbs import DbsRunner
    from oracle.port import threads
    G = synth.synth_G(tiles, tiles, freq, seed=1)
    gobj = synth.synth_gobj(tiles, tiles, seed=1)
    t0 = time.perf_counter()
    r = DbsRunner([G], [gobj], [freq], tiles, tiles, seed, sym=(mode == "sym"), algebra="port")
    t_init = time.perf_counter() - t0
    st = r.states[0]
    acc = {"eval": 0.0, "n_eval": 0, "accept": 0.0, "n_accept": 0}
    ev, ac = st.eval, st.accept

    def timed_eval(s, d):
        t = time.perf_counter()
        out = ev(s, d)
        acc["eval"] += time.perf_counter() - t
        acc["n_eval"] += 1
        return out

    def timed_accept(ne=None):
        t = time.perf_counter()
        ac(ne)
        acc["accept"] += time.perf_counter() - t
        acc["n_accept"] += 1

    st.eval, st.accept = timed_eval, timed_accept
    t0 = time.perf_counter()
    while not r.done and (acc["eval"] + acc["accept"]) < budget_s and (acc["n_accept"] < 8):
        r.step()
    wall = time.perf_counter() - t0
    te = acc["eval"] / max(1, acc["n_eval"])
    ta = acc["accept"] / max(1, acc["n_accept"])
    model_s = nf * (gpu_evals * te + gpu_accepts * ta)
    return {
        "value": gpu_evals / model_s if model_s > 0 else None,
        "unit": "flip_evals/s",
        "cores": threads(),
        "kind": "port",
        "sample": ("1 of %d frequencies at %dx%d (N=%d): init %.1f s, then %d evals and %d accepts of the same DBS "
                   "in %.1f s; per-frequency eval %.2f ms and accept %.0f ms, scaled x%d frequencies and applied to "
                   "the GPU run's %d evals / %d accepts") % (
                       nf, tiles, tiles, G.shape[0], t_init, acc["n_eval"], acc["n_accept"], wall, te * 1e3,
                       ta * 1e3, nf, gpu_evals, gpu_accepts),
        "eval_ms_per_freq": te * 1e3,
        "accept_ms_per_freq": ta * 1e3,
    }


def run_form(a, precision, Gs, rows, rank, local, dist, defer_rank=0):
    """Runs W + K DBS decisions of one precision form; returns its counters."""
    import torch
    from pngf_gb300 import lib
    t_setup = time.perf_counter()
    h = lib.Handle(a.tiles, a.tiles, FREQS, precision=precision, max_flips=1 if a.mode == "single" else 4,
                   device=local, defer_rank=defer_rank)
    for f, G in enumerate(Gs):
        h.load_G(f, G, rows)
    d = lib.Dbs(h, mode=lib.DBS_SINGLE if a.mode == "single" else lib.DBS_SYMMETRIC, init=lib.INIT_RANDOM,
                seed=a.seed + rank, batch=a.batch, device_loop=bool(a.device_loop))
    tune = h.autotune()  # kernel forms for this instance; the state is left unchanged
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    for _ in range(a.warmup):
        d.step()
    s0 = d.stats()
    sampler = ClockSampler(local)
    sampler.start()
    h.timing_enable(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        d.step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    tm = h.timing()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    s1 = d.stats()
    out = dict(evals=s1.evals - s0.evals, accepts=s1.accepts - s0.accepts, launched=s1.launched - s0.launched,
               wall=wall, dev_s=(tm["eval_ms"] + tm["accept_ms"]) * 1e-3, tm=tm, clocks=clocks, setup_s=setup_s,
               F_init=s1.F_init, F_best=s1.F_best, n=h.n, ldm=h.ldm, tune=tune)
    d.close()
    h.close()
    torch.cuda.empty_cache()
    return out


def isolated_update(a, precision, G0, rows, local, decisions=6):
    """The accept update alone: a one-frequency handle (one stream, nothing
    sharing the GPU with its launches), a few DBS decisions from the same
    design; returns the update kernel's mean launch time and bytes."""
    import torch
    from pngf_gb300 import lib
    h = lib.Handle(a.tiles, a.tiles, FREQS[:1], precision=precision, max_flips=1, device=local)
    h.load_G(0, G0, rows)
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=a.seed, batch=0)
    h.autotune()
    d.step()
    torch.cuda.synchronize()
    h.timing_enable(True)
    for _ in range(decisions):
        d.step()
    torch.cuda.synchronize()
    tm = h.timing()
    d.close()
    h.close()
    torch.cuda.empty_cache()
    nl = max(1, tm["update_launches"])
    return {"launch_ms": tm["update_ms"] / nl, "bytes_per_launch": tm["update_bytes"] / nl,
            "flop_per_launch": tm["update_flop"] / nl, "launches": tm["update_launches"]}


def autotune_on(h, mode_single=True):
    """Autotunes a handle's kernel forms on a throwaway random design (seed
    99), outside any timed region; the forms stay with the handle."""
    from pngf_gb300 import lib
    d = lib.Dbs(h, mode=lib.DBS_SINGLE if mode_single else lib.DBS_SYMMETRIC, init=lib.INIT_RANDOM, seed=99,
                max_evals=1)
    t = h.autotune()
    d.close()
    return t


def converge_compare(tiles, freqs, load_G, seed, local, train_seeds=(2, 3), train_evals=1500, train_steps=600,
                     topk=64, state_only=0, batch=0, device_loop=False, online_every=0, rule=0, defer_rank=0):
    """Wall time to the converged objective: plain FP64 DBS (reference order,
    run until the hat is empty) against the proposal + complex64 form, whose
    network is trained only on plain complex64 runs from other seeds. The
    proposal run stops once its objective is within 1e-3 relative of the plain
    run's final objective (or at its own convergence). load_G(handle) loads
    every frequency's G."""
    import torch
    from pngf_gb300 import lib
    out = {"tiles": tiles, "freqs_ghz": [f / 1e9 for f in freqs]}
    nfl = 1
    h = lib.Handle(tiles, tiles, freqs, precision=lib.PREC_FP64, max_flips=nfl, device=local, state_only=state_only)
    load_G(h)
    tune64 = autotune_on(h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=seed, batch=batch, device_loop=device_loop)
    torch.cuda.synchronize()
    t_prep = time.perf_counter() - t0
    # step by step, recording when each decision's F_best was known on the
    # host, so that the time to first reach the target is known afterwards
    trace = []
    while True:
        d.step()
        s = d.stats()
        trace.append((time.perf_counter() - t0, s.F_best, s.evals))
        if s.converged or s.evals >= 10 ** 7:
            break
    torch.cuda.synchronize()
    F_target = s.F_best * (1.0 + 1e-3)
    hit = next(((t, e) for t, F, e in trace if F <= F_target), (trace[-1][0], trace[-1][2]))
    out["plain_fp64"] = {"wall_s": time.perf_counter() - t0, "prepare_s": t_prep, "F_final": s.F_best,
                         "F_init": s.F_init,
                         "evals": s.evals, "accepts": s.accepts, "converged": bool(s.converged),
                         "wall_s_to_target": hit[0], "evals_to_target": hit[1],
                         "eval_form": tune64["eval_form"]}
    d.close()
    h.close()
    torch.cuda.empty_cache()
    # complex64 state built directly in complex64 on the tensor cores; accepts
    # deferred to pending factors, flushed at rank defer_rank (0: immediate)
    h = lib.Handle(tiles, tiles, freqs, precision=lib.PREC_C64, max_flips=nfl, device=local,
                   c64_build=lib.BUILD_C64, state_only=state_only, defer_rank=defer_rank)
    load_G(h)
    prop = lib.Proposal(h, channels=32, seed=1)
    t0 = time.perf_counter()
    pairs = 0
    for sd in train_seeds:  # training pairs from plain complex64 runs of other designs
        d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=sd, max_evals=train_evals)
        lib.dbs_set_proposal(d, prop, topk=0)
        pairs += d.run().launched  # every evaluated candidate is a (design, exact gain) pair
        d.close()
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = prop.train(train_steps, batch=32, lr=2e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    samples = prop.num_samples()
    tune32 = autotune_on(h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=seed, batch=0, drift_every=32, drift_tol=1e-4)
    # online_every > 0: 20 more training steps on the run's own exact pairs every
    # that many proposal steps (0: the network trained beforehand is kept)
    lib.dbs_set_proposal(d, prop, topk=topk, train_every=online_every, train_steps=20, train_batch=32, lr=1e-3,
                         rule=rule)
    torch.cuda.synchronize()
    t_prep = time.perf_counter() - t0
    h.timing_enable(True)
    t_reach = None
    while True:
        d.step()
        s = d.stats()
        if t_reach is None and s.F_best <= F_target:
            torch.cuda.synchronize()
            t_reach = time.perf_counter() - t0
            break
        if s.converged:
            break
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    tmp = h.timing()
    out["proposal_c64"] = {"wall_s_to_target": t_reach, "wall_s": wall, "prepare_s": t_prep,
                           "device_ms": {k: tmp[k] for k in ("eval_ms", "accept_ms", "update_ms")},
                           "F_final": s.F_best, "evals": s.evals,
                           "accepts": s.accepts, "prop_hits": s.prop_hits, "full_passes": s.full_passes,
                           "converged": bool(s.converged), "drift_max": s.drift_max,
                           "drift_checks": s.drift_checks, "refreshes": s.refreshes,
                           "eval_form": tune32["eval_form"], "update_cols": tune32["update"][tune32["update_form"]]["cols"],
                           "accept_rule": "first improving in predicted order" if rule else "best improving",
                           "defer_rank": defer_rank,
                           "reached_target": t_reach is not None,
                           "training": {"seeds": list(train_seeds), "collect_s": t_collect, "train_s": t_train,
                                        "samples": samples, "pairs": pairs, "final_loss": loss,
                                        "steps": train_steps,
                                        "online": ("20 steps every %d proposal steps" % online_every)
                                        if online_every > 0 else "none"}}
    out["F_target"] = F_target
    if t_reach:
        # headline: plain FP64 run to its converged objective against the
        # proposal form reaching that objective within 1e-3
        out["speedup_wall_to_objective"] = out["plain_fp64"]["wall_s"] / t_reach
        # both forms to the same target (plain FP64 also stops at its first
        # crossing of F_target)
        out["speedup_both_to_target"] = out["plain_fp64"]["wall_s_to_target"] / t_reach
        # with the network's offline data collection and training on the clock
        t_train_all = t_collect + t_train
        out["speedup_wall_to_objective_incl_training"] = out["plain_fp64"]["wall_s"] / (t_reach + t_train_all)
        out["speedup_both_to_target_incl_training"] = (out["plain_fp64"]["wall_s_to_target"] /
                                                       (t_reach + t_train_all))
    d.close()
    prop.close()
    h.close()
    torch.cuda.empty_cache()
    return out


FREQS_GROUP = [28.0e9, 30.0e9, 32.0e9]


def group_member(tiles, seed, max_evals, batch, local, device_loop=False, defer_rank=192):
    """One instance of the group workload: complex64 state built on the tensor
    cores, G generated on the device and not kept (state_only), accepts
    deferred to rank defer_rank (0: immediate), single-tile DBS from the
    50%-fill design of `seed`, its kernel forms autotuned; device_loop: its
    decisions drawn and taken on the device."""
    from pngf_gb300 import lib
    h = lib.Handle(tiles, tiles, FREQS_GROUP, precision=lib.PREC_C64, max_flips=1, device=local,
                   c64_build=lib.BUILD_C64, state_only=1, defer_rank=defer_rank)
    for f in range(len(FREQS_GROUP)):
        h.load_G_synth(f, seed=seed)
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=seed, max_evals=max_evals, batch=batch,
                device_loop=device_loop)
    h.autotune()
    return h, d


def group_bench(a, local, n_check=8):
    """Many independent DBS instances on one GPU: tile grids drawn uniformly
    from 11x11..31x31 (seeded), 3 frequencies, complex64, 50%-fill designs from
    seeds 1..I, each run for a fixed budget of flip evaluations. All instances
    step together as one group (one CUDA graph launch per round for every
    instance's batch; accepts run concurrently on the instances' streams).
    The first n_check instances are also run one after another with
    pngf_dbs_step, and their logs are compared with the group's (equivalence)
    and their times with a group of the same n_check (speed-up)."""
    import torch
    from pngf_gb300 import lib
    rng = np.random.default_rng(2024)
    sizes = [int(v) for v in rng.integers(11, 32, a.instances)]
    out = {"instances": a.instances, "tiles": sizes, "freqs_ghz": [f / 1e9 for f in FREQS_GROUP],
           "evals_per_instance": a.group_evals, "batch": a.group_batch}

    def logs_of(runs):
        return [(d.log(), d.stats().F_best) for _, d in runs]

    def close(runs):
        for h, d in runs:
            d.close()
            h.close()
        torch.cuda.empty_cache()

    # equivalence and speed-up on the first n_check instances
    nc = min(n_check, a.instances)
    runs = [group_member(sizes[i], i + 1, a.group_evals, a.group_batch, local) for i in range(nc)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _, d in runs:
        d.run()
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    seq_logs = logs_of(runs)
    close(runs)
    check = {"instances": nc, "sequential_s": t_seq}
    for mode, dev in (("host_drawn", False), ("device_resident", True)):
        runs = [group_member(sizes[i], i + 1, a.group_evals, a.group_batch, local, device_loop=dev)
                for i in range(nc)]
        g = lib.Group([d for _, d in runs], use_graphs=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.run()
        torch.cuda.synchronize()
        t_grp = time.perf_counter() - t0
        same = all(np.array_equal(l1["tile"], l0["tile"]) and np.array_equal(l1["accept"], l0["accept"]) and
                   np.array_equal(l1["F"].view(np.uint64), l0["F"].view(np.uint64)) and F1 == F0
                   for (l0, F0), (l1, F1) in zip(seq_logs, logs_of(runs)))
        st = g.stats()
        check[mode] = {"group_s": t_grp, "speedup": t_seq / t_grp, "logs_identical": bool(same),
                       "rounds": st["rounds"], "graph_captures": st["captures"]}
        g.close()
        close(runs)
    out["check"] = check
    # the whole group
    free0 = torch.cuda.mem_get_info(local)[0]
    t0 = time.perf_counter()
    runs = [group_member(sizes[i], i + 1, a.group_evals, a.group_batch, local, device_loop=True)
            for i in range(a.instances)]
    torch.cuda.synchronize()
    out["setup_s"] = time.perf_counter() - t0
    out["decisions"] = "device-resident: one graph of the instances' decision loops (draw, evaluate, decide)"
    out["accepts_form"] = "complex64, deferred to pending rank 192 (flushed by the long-K tensor-core kernel)"
    out["device_gb_held"] = (free0 - torch.cuda.mem_get_info(local)[0]) / 1e9
    out["edges_total"] = int(sum(h.n for h, _ in runs))
    g = lib.Group([d for _, d in runs], use_graphs=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = g.run()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    evals = sum(d.stats().evals for _, d in runs)
    accepts = sum(d.stats().accepts for _, d in runs)
    out.update({"wall_s": wall, "flip_evals": evals, "accepts": accepts, "flip_evals_per_s": evals / wall,
                "accepted_updates_per_s": accepts / wall, "rounds": st["rounds"],
                "graph_launches": st["graph_launches"], "graph_captures": st["captures"],
                "kernel_launches": st["kernel_launches"]})
    g.close()
    close(runs)
    return out


FREQS_C5 = [28.0e9, 29.33e9, 30.67e9, 32.0e9]


def c5_compare(a, local, reduced=True):
    """C5: 41x41 tiles (N = 30504), 4 frequencies, synthetic G and NF2FF rows
    generated on the device; plain FP64 DBS to convergence against proposal +
    complex64 DBS. The default run's reduced form trains the network on one
    other seed's 2000 plain complex64 evaluations (600 Adam steps); --c5 runs
    the full form (two seeds, 3000 evaluations each, 1000 steps)."""
    kw = dict(train_seeds=(2,), train_evals=2000, train_steps=600) if reduced else \
        dict(train_evals=3000, train_steps=1000)
    # deferred complex64 updates: at N = 30504 an update pass over T dominates an accept
    out = converge_compare(41, FREQS_C5, lambda h: [h.load_G_synth(f, seed=1) for f in range(len(FREQS_C5))],
                           a.seed, local, batch=a.batch, device_loop=bool(a.device_loop), online_every=8,
                           defer_rank=192, **kw)
    out["form"] = "reduced training (1 seed, 2000 evaluations)" if reduced else "full training"
    return out


def c5_run(a, local):
    """The learned-proposal form at 41x41 tiles (N = 30504), 4 frequencies,
    synthetic G generated on the device: wall time to the converged objective
    of plain FP64 DBS against proposal + complex64 DBS (network trained on
    plain complex64 runs of other seeds at this size). One JSON line."""
    import torch
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    out = c5_compare(a, local, reduced=False)
    print(json.dumps({"metric": "wall time to converged objective, 41x41 tiles x 4 frequencies, proposal + "
                                "complex64 vs plain FP64", "c5": out, "total_s": time.perf_counter() - t0}),
          flush=True)


def reduce_form(r, dist, device="cuda"):
    """Whole-job figures: sums of work over ranks, max of times over ranks
    (each rank runs its own DBS instance; the job ends with the slowest)."""
    import torch
    if not dist:
        return r["wall"], r["dev_s"], r["evals"], r["accepts"], r["launched"]
    vec = torch.tensor([r["wall"], r["dev_s"], r["evals"], r["accepts"], r["launched"]], dtype=torch.float64,
                       device=device)
    mx, sm = vec.clone(), vec.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return mx[0].item(), mx[1].item(), sm[2].item(), sm[3].item(), sm[4].item()


def gpu_arm(a, world, rank, local):
    import torch
    from pngf_gb300 import lib
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    peaks, peak_src = measured_peaks()
    fp64_peak = fp64_gemm_peak_tflops()
    nf = len(FREQS)
    Gs, rows = make_Gs(a.tiles, FREQS)
    forms = a.forms.split(",")
    r64 = r32 = None
    if "fp64" in forms:
        r64 = run_form(a, lib.PREC_FP64, Gs, rows, rank, local, dist)
        wall_m, dev_m, evals_t, accepts_t, launched_t = reduce_form(r64, dist)
    if "c64" in forms:
        r32 = run_form(a, lib.PREC_C64, Gs, rows, rank, local, dist)
        c64_red = reduce_form(r32, dist)
    r32d = None
    if "c64d" in forms:  # complex64 with the rank-k updates deferred to rank 192
        r32d = run_form(a, lib.PREC_C64, Gs, rows, rank, local, dist, defer_rank=192)
        c64d_red = reduce_form(r32d, dist)
    rsym = None
    if "sym" in forms and a.mode == "single":  # the reference's own 4-fold mirror hat, plain FP64, 10 decisions
        import copy
        asym = copy.copy(a)
        asym.mode, asym.steps = "sym", 10
        rsym = run_form(asym, lib.PREC_FP64, Gs, rows, rank, local, dist)
    iso64 = isolated_update(a, lib.PREC_FP64, Gs[0], rows, local) if r64 is not None and rank == 0 else None
    iso32 = isolated_update(a, lib.PREC_C64, Gs[0], rows, local) if r32 is not None and rank == 0 else None
    conv = None
    if not a.no_converge and rank == 0:
        # the complex64 form of the proposal run: deferred updates when this run
        # measured them faster than immediate ones at this size
        defer = 0
        if r32 is not None and r32d is not None:
            defer = 192 if reduce_form(r32d, None)[2] / reduce_form(r32d, None)[1] > \
                reduce_form(r32, None)[2] / reduce_form(r32, None)[1] else 0
        load = lambda h: [h.load_G(f, G, rows) for f, G in enumerate(Gs)]  # noqa: E731
        runs = []
        for sd in range(a.seed, a.seed + max(1, a.converge_seeds)):  # each run's network trains on two other seeds
            runs.append(converge_compare(a.tiles, FREQS, load, sd, local, train_seeds=(sd + 10, sd + 20),
                                         batch=a.batch, device_loop=bool(a.device_loop), defer_rank=defer))
        conv = runs[0]
        conv["complex64_form"] = ("deferred (rank 192): measured faster than immediate updates in this run"
                                  if defer else "immediate updates: measured faster than deferred in this run")
        keys = ("speedup_wall_to_objective", "speedup_both_to_target", "speedup_wall_to_objective_incl_training",
                "speedup_both_to_target_incl_training")
        conv["seeds"] = [dict({"seed": a.seed + i, "reached_target": r["proposal_c64"]["reached_target"],
                               "F_plain": r["plain_fp64"]["F_final"], "F_proposal": r["proposal_c64"]["F_final"],
                               "F_gap_rel": (r["proposal_c64"]["F_final"] - r["plain_fp64"]["F_final"]) /
                                            abs(r["plain_fp64"]["F_final"]),
                               "plain_wall_s": r["plain_fp64"]["wall_s"],
                               "proposal_wall_s": r["proposal_c64"]["wall_s"],
                               "proposal_accepts": r["proposal_c64"]["accepts"],
                               "proposal_full_passes": r["proposal_c64"]["full_passes"],
                               "proposal_refreshes": r["proposal_c64"]["refreshes"]},
                              **{k: r.get(k) for k in keys}) for i, r in enumerate(runs)]
        conv["reached_fraction"] = sum(x["reached_target"] for x in conv["seeds"]) / len(runs)
        reached = sorted(x["speedup_wall_to_objective"] for x in conv["seeds"] if x["reached_target"])
        conv["median_speedup_of_reached"] = reached[len(reached) // 2] if reached else None
    del Gs
    grp = group_bench(a, local) if (not a.no_group and rank == 0) else None
    c5 = c5_compare(a, local) if (not a.no_c5 and not a.no_converge and rank == 0) else None
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    if r64 is None:  # complex64 forms alone (profiling runs)
        print(json.dumps({name: {"counters": {k: v for k, v in r.items() if k != "tm"}, "timing": r["tm"]}
                          for name, r in (("c64", r32), ("c64d", r32d)) if r is not None}), flush=True)
        return
    tm, n = r64["tm"], r64["n"]
    upd_s = tm["update_ms"] * 1e-3
    achieved = tm["update_flop"] / upd_s / 1e12 if upd_s > 0 else None
    traffic = None
    if os.path.exists(PROFILE_SUMMARY):  # ncu capture summary: "dram_bytes_per_launch: <bytes>"
        with open(PROFILE_SUMMARY) as fh:
            m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", fh.read())
        traffic = float(m.group(1)) if m else None
    # Dominant kernel of the FP64 form: the accept update on the tensor cores
    # (k_tc_update_f64: exact 7-bit integer slices of A and W, BF16 MMAs into
    # FP32 TMEM accumulators, FP64 recombination). It streams M once in and
    # once out, so its bound is HBM; its FP64-equivalent rate is reported
    # against the measured DGEMM rate.
    upd_gbs = tm["update_bytes"] / upd_s / 1e9 if upd_s > 0 else None
    roofline = {
        "kernel": "k_tc_update_f64 (FP64-accurate complex rank-k update of M on tcgen05, accept step)",
        "bound": "hbm",
        "achieved": upd_gbs,
        "peak": peaks["hbm_gbs"],
        "unit": "GB/s",
        "frac": upd_gbs / peaks["hbm_gbs"] if upd_gbs else None,
        "peak_source": peak_src,
        "traffic": traffic,
        "algorithmic_bytes_per_launch": tm["update_bytes"] / max(1, tm["update_launches"]),
        "launch_ms": tm["update_ms"] / max(1, tm["update_launches"]),
        "fp64_view": {"achieved_tflops": achieved, "dgemm_peak_tflops": fp64_peak,
                      "frac": achieved / fp64_peak if achieved else None,
                      "algorithmic_flop_per_launch": tm["update_flop"] / max(1, tm["update_launches"]),
                      "peak_source": "cuBLAS DGEMM 4096^3 via torch on this GPU in this run, best of 5"},
        # the frequencies' updates of one accept run concurrently, one stream
        # each: launch_ms is a launch's own duration among them; the
        # aggregate counts every update byte over the accept steps' device
        # time (factor, solves and operand slicing included)
        "frequency_streams": nf,
        "aggregate_gbs_over_accept_time": tm["update_bytes"] / (tm["accept_ms"] * 1e-3) / 1e9
        if tm["accept_ms"] > 0 else None,
    }
    if iso64:  # the same kernel with the GPU to itself
        g = iso64["bytes_per_launch"] / (iso64["launch_ms"] * 1e-3) / 1e9
        roofline["isolated"] = {"what": "one-frequency handle, %d DBS decisions, one stream" % 6,
                                "launch_ms": iso64["launch_ms"], "achieved": g, "frac": g / peaks["hbm_gbs"],
                                "launches": iso64["launches"]}
    eval_s = tm["eval_ms"] * 1e-3
    # kernels (a)+(c): the candidate evaluation launch group (edge lists,
    # candidate kernel, scoring). Its work is a capacitance LU per (candidate,
    # frequency) in FP64 over gathers of k^2 + (E+1) k entries of M, so its
    # bound is the FP64 pipe; the HBM view is reported beside it.
    roofline_eval = {
        "kernel": "k_eval / k_eval_warp + k_edge_lists + k_score (candidate evaluation, FP64 capacitance LU)",
        "bound": "fp64",
        "achieved": tm["eval_flop"] / eval_s / 1e12 if eval_s > 0 else None,
        "peak": fp64_peak, "unit": "TFLOP/s",
        "frac": tm["eval_flop"] / eval_s / 1e12 / fp64_peak if eval_s > 0 else None,
        "peak_source": "cuBLAS DGEMM 4096^3 via torch on this GPU in this run, best of 5",
        "algorithmic_flop_per_cand_freq": tm["eval_flop"] / max(1.0, tm["eval_cf"]),
        "launch_ms": tm["eval_ms"] / max(1, tm["eval_launches"]),
        "cand_freq_per_launch": tm["eval_cf"] / max(1, tm["eval_launches"]),
        "hbm_view": {"achieved_gbs": tm["eval_bytes"] / eval_s / 1e9 if eval_s > 0 else None,
                     "peak_gbs": peaks["hbm_gbs"],
                     "frac": tm["eval_bytes"] / eval_s / 1e9 / peaks["hbm_gbs"] if eval_s > 0 else None,
                     "algorithmic_bytes_per_cand_freq": tm["eval_bytes"] / max(1.0, tm["eval_cf"])},
    }
    line = {
        "metric": METRIC,
        "value": evals_t / dev_m if dev_m > 0 else None,
        "unit": "flip_evals/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": wall_m / a.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(a, n, nf, world),
        "e2e": {"value": evals_t / wall_m, "unit": "flip_evals/s",
                "h2d_bytes_per_step": tm["h2d_bytes"] / a.steps, "d2h_bytes_per_step": tm["d2h_bytes"] / a.steps},
        "roofline": roofline,
        "roofline_eval": roofline_eval,
        "clocks": r64["clocks"],
        "gpu_launches": tm["kernel_launches"],
        "detail": {
            "evals": evals_t, "accepts": accepts_t, "launched_candidates": launched_t,
            "accepted_updates_per_s": accepts_t / wall_m,
            "cand_freq_evals_per_s_device": tm["eval_cf"] / eval_s if eval_s > 0 else None,
            "eval_kernel_gbs": tm["eval_bytes"] / eval_s / 1e9 if eval_s > 0 else None,
            "eval_kernel_fp64_tflops": tm["eval_flop"] / eval_s / 1e12 if eval_s > 0 else None,
            "eval_ms": tm["eval_ms"], "accept_ms": tm["accept_ms"], "update_ms": tm["update_ms"],
            "setup_s": r64["setup_s"], "F_init": r64["F_init"], "F_best": r64["F_best"],
            "speculation": "draws evaluated in speculative batches in hat order (batch %s); decisions, accepts and "
                           "the counted evaluations are the reference's" % (
                               "adaptive from %d" % -a.batch if a.batch < 0 else
                               "whole remaining hat" if a.batch == 0 else str(a.batch)),
            "value_timing": "sum of CUDA-event spans of the hot-path launch groups on the handle's stream",
            "fp64_gemm_tflops": fp64_peak, "autotune": r64["tune"],
        },
    }
    def c64_block(r32, c64_red, what):
        w32, d32, e32, acc32, l32 = c64_red
        t32 = r32["tm"]
        u32 = t32["update_ms"] * 1e-3
        return {
            "what": what,
            "value": e32 / d32 if d32 > 0 else None, "e2e": e32 / w32, "unit": "flip_evals/s",
            "evals": e32, "accepts": acc32, "F_init": r32["F_init"], "F_best": r32["F_best"],
            "F_best_rel_diff_vs_fp64": abs(r32["F_best"] - r64["F_best"]) / abs(r64["F_best"]),
            "eval_ms_fp64_form": tm["eval_ms"],
            "eval_ms": t32["eval_ms"], "accept_ms": t32["accept_ms"], "update_ms": t32["update_ms"],
            "roofline": {
                "kernel": "k_tc_update (tcgen05 complex rank-k update of T)",
                "bound": "hbm",
                "achieved": t32["update_bytes"] / u32 / 1e9 if u32 > 0 else None,
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": (t32["update_bytes"] / u32 / 1e9) / peaks["hbm_gbs"] if u32 > 0 else None,
                "peak_source": peak_src,
                "frequency_streams": nf,
                "aggregate_gbs_over_accept_time": t32["update_bytes"] / (t32["accept_ms"] * 1e-3) / 1e9
                if t32["accept_ms"] > 0 else None,
                "launch_ms": t32["update_ms"] / max(1, t32["update_launches"]),
                "algorithmic_bytes_per_launch": t32["update_bytes"] / max(1, t32["update_launches"]),
                # 3xTF32: the tensor pipe does 3 real products per complex-equivalent
                # flop counted in update_flop (8 r N^2 per launch of rank r)
                "tensor_view": {
                    "tf32_tflops": 3.0 * t32["update_flop"] / u32 / 1e12 if u32 > 0 else None,
                    "peak_tflops": peaks["bf16_tflops"] / 2.0,
                    "peak_source": "half the measured dense BF16 rate (TF32 runs at half the BF16 rate)",
                    "frac": 3.0 * t32["update_flop"] / u32 / 1e12 / (peaks["bf16_tflops"] / 2.0) if u32 > 0 else None,
                },
            },
            "clocks": r32["clocks"], "gpu_launches": t32["kernel_launches"], "setup_s": r32["setup_s"],
            "autotune": r32["tune"],
        }

    if r32 is not None:
        line["c64_form"] = c64_block(
            r32, c64_red, "T in complex64, rank-k update on tcgen05 tensor cores (kind::tf32, 3xTF32 split products, "
                          "FP32 accumulation in TMEM) at every accept; capacitance LU, y, R, Eobj, objective and accept "
                          "test in FP64; same workload and steps")
        if iso32:
            g = iso32["bytes_per_launch"] / (iso32["launch_ms"] * 1e-3) / 1e9
            line["c64_form"]["roofline"]["isolated"] = {
                "what": "one-frequency handle, 6 DBS decisions, one stream", "launch_ms": iso32["launch_ms"],
                "achieved": g, "frac": g / peaks["hbm_gbs"], "launches": iso32["launches"]}
    if r32d is not None:
        line["c64_deferred_form"] = c64_block(
            r32d, c64d_red, "the complex64 form with the T part of each accept appended to pending rank-k factors "
                            "(candidates and accepts read T minus the pending product) and flushed to T on the tensor "
                            "cores when the pending rank reaches 192 - 24: roofline per flush launch")
    if rsym is not None:
        ts = rsym["tm"]
        line["symmetric_form"] = {
            "what": "the reference's default candidate set: the 4-fold mirror quarter hat (flips of 1, 2 or 4 tiles, "
                    "up to 96 edges), plain FP64, same workload, 10 decisions",
            "value": rsym["evals"] / rsym["dev_s"] if rsym["dev_s"] > 0 else None,
            "e2e": rsym["evals"] / rsym["wall"], "unit": "flip_evals/s", "evals": rsym["evals"],
            "accepts": rsym["accepts"], "eval_ms": ts["eval_ms"], "accept_ms": ts["accept_ms"],
            "update_ms": ts["update_ms"], "update_launches": ts["update_launches"],
            "ms_per_accept": ts["accept_ms"] / max(1, rsym["accepts"]),
        }
    if conv is not None:
        line["converge"] = conv
    if grp is not None:
        line["group"] = grp
    if c5 is not None:
        line["c5"] = c5
    if world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(a.tiles, a.mode, a.seed, FREQS[0], r64["evals"],
                                                   r64["accepts"], nf)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def reference_arm(a, world, rank):
    if rank != 0:
        return
    from oracle.dbs import DbsRunner
    from oracle.port import threads
    nf = len(FREQS)
    t0 = time.perf_counter()
    Gs, rows = make_Gs(a.tiles, FREQS)
    n = Gs[0].shape[0]
    r = DbsRunner(Gs, [rows] * nf, FREQS, a.tiles, a.tiles, a.seed, sym=(a.mode == "sym"), algebra="port")
    del Gs
    setup_s = time.perf_counter() - t0
    for _ in range(a.warmup):
        r.step()
    e0 = r.log.evals
    t0 = time.perf_counter()
    for _ in range(a.steps):
        r.step()
    wall = time.perf_counter() - t0
    evals = r.log.evals - e0
    v = evals / wall
    line = {
        "metric": METRIC,
        "impl": "reference", "value": v, "unit": "flip_evals/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": wall / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a, n, nf, world),
        "cpu_baseline": {"value": v, "unit": "flip_evals/s", "cores": threads(), "kind": "port",
                         "sample": "%d DBS decisions (%d evals) after %d warm-up decisions, all %d frequencies; "
                                   "setup (G, LU inverse of C) %.1f s untimed" % (a.steps, evals, a.warmup, nf,
                                                                                  setup_s)},
        "e2e": {"value": v, "unit": "flip_evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def eval_probe(a, local):
    """The candidate kernel alone at the workload's full pass (every tile at
    every frequency: 441 x 5 (candidate, frequency) pairs at 21x21), on a
    state-only handle whose G is generated on the device and not kept (M only:
    about 1 GB per frequency). For ncu captures of one launch (-k regex:k_eval
    -c 1); also prints the CUDA-event time per launch."""
    import torch
    from pngf_gb300 import lib
    torch.cuda.set_device(local)
    h = lib.Handle(a.tiles, a.tiles, FREQS, precision=lib.PREC_FP64, max_flips=1, device=local, state_only=1)
    for f in range(len(FREQS)):
        h.load_G_synth(f, seed=1)
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=a.seed, max_evals=1)  # prepares the design
    h.set_eval_form(a.eval_form)
    cands = [[t] for t in range(a.tiles * a.tiles)]
    h.timing_enable(True)
    for _ in range(a.eval_probe):
        h.eval_candidates(cands)
    tm = h.timing()
    d.close()
    h.close()
    nl = max(1, tm["eval_launches"])
    print(json.dumps({"eval_probe": {"form": a.eval_form, "launches": tm["eval_launches"],
                                     "cand_freq_per_launch": tm["eval_cf"] / nl,
                                     "ms_per_launch_group": tm["eval_ms"] / nl,
                                     "fp64_tflops": tm["eval_flop"] / (tm["eval_ms"] * 1e-3) / 1e12
                                     if tm["eval_ms"] > 0 else None}}), flush=True)


def main():
    global FREQS
    a = parse()
    FREQS = FREQS[:max(1, min(a.nfreq, len(FREQS)))]
    world, rank, local = dist_env()
    if a.eval_probe:
        if rank == 0:
            eval_probe(a, local)
        return
    if a.c5:
        if rank == 0:
            c5_run(a, local)
        return
    if a.impl == "reference":
        reference_arm(a, world, rank)
    else:
        gpu_arm(a, world, rank, local)


if __name__ == "__main__":
    main()
