"""Many DBS runs at once, the device-side synthetic G and state-only handles.

- G generated on the device (pngf_load_G_synth) builds the same state as the
  host generator's G to 1e-12 relative (the generators differ only in the
  last bits of sqrt/exp/sin/cos/log).
- A state_only handle (G regenerated for every build and drift check, FP64
  staging of M allocated only while a build runs) gives bit-identical states,
  drift checks and DBS runs to a handle that keeps G.
- A group of runs of different sizes and precisions, stepped together (with
  and without CUDA graphs), reproduces every member's sequential run bit for
  bit: same accepted flips, same objectives, same log."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FREQS3 = [28e9, 30e9, 32e9]


def bits(x):
    return np.ascontiguousarray(x).view(np.uint64)


def design(a, seed):
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.integers(0, 2, a * a)]


def prepared(a, freqs, prec, synth, tm, **kw):
    from pngf_gb300 import lib
    h = lib.Handle(a, a, freqs, precision=prec, max_flips=1, **kw)
    for f, fr in enumerate(freqs):
        if synth:
            h.load_G_synth(f, seed=1)
        else:
            h.load_G(f, np.ascontiguousarray(lib.synth_G(a, a, fr, seed=1)), lib.synth_gobj(a, a, seed=1))
    mid = (a - 1) // 2
    h.set_tile_map(tm)
    h.set_source_port(mid, mid, 1, 2)
    h.prepare()
    return h


def test_device_synth_G_matches_host(built_lib):
    from pngf_gb300 import lib
    a = 9
    tm = design(a, 4)
    hh = prepared(a, FREQS3[:2], lib.PREC_FP64, False, tm)
    hd = prepared(a, FREQS3[:2], lib.PREC_FP64, True, tm)
    for f in range(2):
        Mh, eh = hh.get_M(f)
        Md, ed = hd.get_M(f)
        assert np.abs(Md - Mh).max() <= 1e-12 * np.abs(Mh).max()
        assert np.abs(ed - eh).max() <= 1e-12 * np.abs(eh).max()
    assert abs(hd.objective() - hh.objective()) <= 1e-12 * abs(hh.objective())
    hh.close()
    hd.close()


@pytest.mark.parametrize("build", [0, 1])
def test_state_only_handle_matches_full_handle(build, built_lib):
    from pngf_gb300 import lib
    a = 9
    tm = design(a, 6)
    hf = prepared(a, FREQS3, lib.PREC_C64, True, tm, c64_build=build)
    hs = prepared(a, FREQS3, lib.PREC_C64, True, tm, c64_build=build, state_only=1)
    for f in range(3):
        assert np.array_equal(bits(hs.get_M(f)[0]), bits(hf.get_M(f)[0]))
    assert hs.drift_check(2) == hf.drift_check(2)
    with pytest.raises(lib.PngfError):
        hs.load_G(0, np.zeros((hs.n, hs.n), dtype=np.complex128), None)
    logs = []
    for h in (hf, hs):
        d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=5, max_evals=400, batch=64,
                    drift_every=8, drift_tol=1e-12)  # tolerance forces refreshes: regenerated G on hs
        s = d.run()
        assert s.refreshes > 0
        logs.append((d.log(), s.F_best))
        d.close()
    (l0, F0), (l1, F1) = logs
    assert F0 == F1
    for k in ("tile", "accept"):
        assert np.array_equal(l0[k], l1[k])
    assert np.array_equal(bits(l0["F"]), bits(l1["F"]))
    hf.close()
    hs.close()


# (tiles, precision, mode, seed, batch, state_only)
MEMBERS = [(7, 0, 0, 1, 16, 0), (9, 1, 1, 2, 32, 1), (11, 0, 1, 3, 32, 0), (9, 0, 0, 4, 8, 0), (11, 1, 1, 5, 48, 0)]


def member_runs(built_lib, device_loop=False):
    from pngf_gb300 import lib
    runs = []
    for a, prec, mode, seed, batch, so in MEMBERS:
        h = lib.Handle(a, a, FREQS3, precision=prec, max_flips=4 if mode == 0 else 1, state_only=so)
        for f in range(3):
            h.load_G_synth(f, seed=seed)
        d = lib.Dbs(h, mode=lib.DBS_SYMMETRIC if mode == 0 else lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=seed,
                    max_evals=700, batch=batch, drift_every=16 if prec == 1 else 0, drift_tol=1e-4,
                    device_loop=device_loop)
        runs.append((h, d))
    return runs


@pytest.mark.parametrize("graphs,device_loop", [(True, False), (False, False), (True, True)])
def test_group_equals_sequential_runs(graphs, device_loop, built_lib):
    """Host-drawn groups (one graph of the members' batches per round) and
    device-resident groups (one graph of the members' decision loops,
    captured once) reproduce every member's sequential host-driver run."""
    from pngf_gb300 import lib
    seq = []
    for h, d in member_runs(built_lib):
        s = d.run()
        seq.append((d.log(), s.F_best, s.accepts))
        d.close()
        h.close()
    runs = member_runs(built_lib, device_loop=device_loop)
    g = lib.Group([d for _, d in runs], use_graphs=graphs)
    st = g.run()
    assert st["rounds"] > 0 and st["accepts"] > 0
    if graphs:
        assert st["graph_launches"] == st["rounds"] and st["captures"] < st["rounds"]
    if device_loop:
        assert st["captures"] == 1
    for (h, d), (log0, F0, acc0) in zip(runs, seq):
        s = d.stats()
        log1 = d.log()
        assert s.F_best == F0 and s.accepts == acc0
        for k in ("tile", "accept"):
            assert np.array_equal(log1[k], log0[k])
        assert np.array_equal(bits(log1["F"]), bits(log0["F"]))
        assert np.array_equal(bits(log1["perf"]), bits(log0["perf"]))
    g.close()
    for h, d in runs:
        d.close()
        h.close()
