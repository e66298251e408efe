"""GPU FP64 path against the reference's golden logs and the CPU oracle.

Bar (the plain FP64 form): identical flip sequence, accept decisions and
final design as the reference on the same G and seed, and every logged
objective value within 1e-10 relative (S11 / D within 1e-10 relative or
1e-12 absolute near zero).
"""
import numpy as np
import pytest

from conftest import case_G, force_port_tiles, free_tiles, golden_log

pytestmark = pytest.mark.gpu

RTOL = 1e-10
ATOL = 1e-12


def gpu_dbs(c, Gs, gobj, batch=0):
    from pngf_gb300 import lib
    h = lib.Handle(c["tiles"], c["tiles"], c["freqs"], max_flips=4 if c["mode"] == "sym" else 1)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    d = lib.Dbs(h, mode=lib.DBS_SYMMETRIC if c["mode"] == "sym" else lib.DBS_SINGLE,
                init=lib.INIT_RANDOM if c["init"] == "random" else lib.INIT_EMPTY, seed=c["seed"],
                max_evals=c["max_evals"], batch=batch)
    s = d.run()
    return h, d, s


def compare_log(d, h, ref, s):
    lg = d.log()
    assert len(lg["tile"]) == len(ref["rows"])
    for i, r in enumerate(ref["rows"]):
        assert lg["tile"][i] == r[1], "flip index differs at eval %d" % i
        assert lg["accept"][i] == r[2], "accept differs at eval %d" % i
        assert abs(lg["F"][i] - r[3]) <= RTOL * abs(r[3]), (i, lg["F"][i], r[3])
        assert abs(lg["F_best"][i] - r[4]) <= RTOL * abs(r[4])
        np.testing.assert_allclose(lg["perf"][i], r[5], rtol=RTOL, atol=ATOL)
    assert abs(s.F_init - ref["start"][0]) <= RTOL * abs(ref["start"][0])
    assert list(h.tile_map()) == ref["final_map"]
    assert bool(s.converged) == bool(ref["end"]["converged"])


@pytest.mark.parametrize("name", ["sym_7x7_f1_seed1", "sym_7x7_f5_empty", "single_7x7_f2_seed1",
                                  "sym_9x9_f2_seed3", "single_11x11_f3_seed2"])
def test_dbs_matches_reference(name, cases, built_lib):
    c = cases[name]
    Gs, gobj = case_G(c, built_lib)
    h, d, s = gpu_dbs(c, Gs, gobj)
    ref = golden_log(name)
    # every case carries the synthetic NF2FF rows: D is nonzero in every row
    assert c.get("gobj") == "synth" and all(abs(v) > 1e-3 for r in ref["rows"] for v in r[5][2::3])
    compare_log(d, h, ref, s)


def test_dbs_matches_reference_at_benchmark_size(cases, built_lib):
    """The benchmarked workload itself -- 21x21 tiles (N = 8064), five
    frequencies 27-33 GHz, single-tile hat, seed 1, NF2FF rows live -- driven
    exactly as bench.py drives it (adaptive speculative batches from 16):
    the first 120 evaluations of the reference's run, flip for flip."""
    c = cases["single_21x21_f5_seed1"]
    assert c["tiles"] == 21 and len(c["freqs"]) == 5 and c.get("gobj") == "synth"
    Gs, gobj = case_G(c, built_lib)
    h, d, s = gpu_dbs(c, Gs, gobj, batch=-16)
    ref = golden_log(c["name"])
    assert any(abs(r[5][2]) > 0.1 for r in ref["rows"])  # the directivity term is live
    compare_log(d, h, ref, s)
    d.close()
    h.close()


def test_dbs_matches_reference_at_benchmark_size_symmetric(cases, built_lib):
    """The same size in the reference's default candidate set, the 4-fold
    mirror hat (flips of 1, 2 or 4 tiles, up to 96 edges: the FP64 accepts of
    more than 32 edges take the refined tensor-core W and the update in
    pieces): the first 40 evaluations of the reference's run, flip for flip."""
    c = cases["sym_21x21_f5_seed1"]
    assert c["tiles"] == 21 and c["mode"] == "sym" and len(c["freqs"]) == 5
    Gs, gobj = case_G(c, built_lib)
    h, d, s = gpu_dbs(c, Gs, gobj, batch=-16)
    ref = golden_log(c["name"])
    assert sum(r[2] for r in ref["rows"]) >= 5  # several accepts
    compare_log(d, h, ref, s)
    d.close()
    h.close()


@pytest.mark.parametrize("batch", [1, 5, -2, -16])
def test_dbs_batch_size_does_not_change_sequence(batch, cases, built_lib):
    """Speculative batches of any size replay the hat to the reference's order
    (negative: adaptive, |batch| draws after an accept, doubling after each
    batch without one)."""
    c = cases["single_7x7_f2_seed1"]
    Gs, gobj = case_G(c, built_lib)
    h, d, s = gpu_dbs(c, Gs, gobj, batch=batch)
    compare_log(d, h, golden_log(c["name"]), s)
    assert s.launched >= s.evals


def test_eval_and_accept_match_oracle(cases, built_lib):
    """Random candidates on a random design: newEobj and F against the
    reference algebra on C^-1, then Eobj after an accept."""
    from oracle.dbs import DX, DY, DZ
    from oracle.geometry import Geometry, port_setup
    from oracle.refalg import C0, RefState, objective
    from pngf_gb300 import lib
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    geo = Geometry(a, a)
    rng = np.random.default_rng(5)
    tm = force_port_tiles(rng.integers(0, 2, a * a), a, a)
    mid = (a - 1) // 2
    P = geo.compute_P(tm)
    port = geo.port_indices(mid, mid, 1, 2)
    h = lib.Handle(a, a, c["freqs"], max_flips=4)
    refs, consts = [], []
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
        Gobj, Einc, vinc, ln1, ln2 = port_setup(G, gobj[f], port)
        refs.append(RefState(G, Gobj, Einc, P))
        consts.append((vinc, ln1, ln2, 2 * np.pi * c["freqs"][f] / C0))
    h.set_tile_map(tm)
    h.set_source_port(mid, mid, 1, 2)
    h.prepare()
    for f in range(len(Gs)):
        e, v = h.eobj(f)
        np.testing.assert_allclose(e, refs[f].Eobj, rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(v, consts[f][:3], rtol=1e-13, atol=1e-16)
    pool = free_tiles(a, a)
    cands = [[int(t) for t in rng.choice(pool, size=rng.integers(1, 5), replace=False)] for _ in range(40)]
    eo, F = h.eval_candidates(cands)
    for i, cand in enumerate(cands):
        s, d = geo.flip_set(tm, P, cand)
        Fr = 0.0
        for f in range(len(Gs)):
            ne = refs[f].eval(s, d)
            np.testing.assert_allclose(eo[i, f], ne, rtol=1e-10, atol=1e-13)
            Fr += objective(ne, *consts[f], DX, DY, DZ)[0]
        assert abs(F[i] - Fr) <= RTOL * abs(Fr)
    # accept candidate 7 and compare the new state
    s, d = geo.flip_set(tm, P, cands[7])
    news = [refs[f].eval(s, d) for f in range(len(Gs))]
    h.accept(7)
    for f in range(len(Gs)):
        refs[f].accept(news[f])
        e, _ = h.eobj(f)
        np.testing.assert_allclose(e, refs[f].Eobj, rtol=1e-10, atol=1e-13)
    for t in cands[7]:
        tm[t] ^= 1
    assert list(h.tile_map()) == tm


def test_prepared_M_matches_oracle(cases, built_lib):
    """M built on the GPU from G (chunked accepts of the design's edges)
    against the oracle's M algebra and against H C^-1 from a direct inverse."""
    from oracle.geometry import Geometry, port_setup
    from oracle.refalg import MState
    from pngf_gb300 import lib
    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    geo = Geometry(7, 7)
    tm = list(np.random.default_rng(3).integers(0, 2, 49))
    P = geo.compute_P(tm)
    Gobj, Einc, _, _, _ = port_setup(Gs[0], gobj[0], geo.port_indices(3, 3, 1, 2))
    h = lib.Handle(7, 7, c["freqs"], max_flips=4)
    h.load_G(0, Gs[0], gobj[0])
    h.set_tile_map(tm)
    h.set_source_port(3, 3, 1, 2)
    h.prepare()
    M, e = h.get_M(0)
    np.testing.assert_allclose(e, Einc, rtol=1e-14, atol=0)
    ref = MState.build(Gs[0], Gobj, Einc, P).M
    scale = np.abs(ref).max()
    assert np.abs(M - ref).max() <= 1e-11 * scale
    n = Gs[0].shape[0]
    C = np.eye(n, dtype=complex)
    C[P.astype(bool)] = Gs[0][P.astype(bool)]
    T = (Gs[0] - np.eye(n)) @ np.linalg.inv(C)
    assert np.abs(M[:n, :n] - T).max() <= 1e-10 * np.abs(T).max()


def test_api_errors(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    h = lib.Handle(7, 7, [30e9], max_flips=4)
    h.load_G(0, Gs[0], gobj[0])
    with pytest.raises(lib.PngfError) as e:
        h.prepare()  # no tile map / port yet
    assert e.value.code == 6
    h.set_tile_map([0] * 49)
    with pytest.raises(lib.PngfError) as e:
        h.set_source_port(3, 3, 2, 2)  # y offset + size beyond the tile (the reference exits)
    assert e.value.code == 1
    h.set_source_port(3, 3, 1, 2)
    h.prepare()
    with pytest.raises(lib.PngfError) as e:
        h.accept(0)  # nothing evaluated
    assert e.value.code == 6
    with pytest.raises(lib.PngfError) as e:
        h.eval_candidates([[49]])  # tile index out of range
    assert e.value.code == 1
    with pytest.raises(lib.PngfError) as e:
        h.load_G_file(0, "/nonexistent/G.bin")
    assert e.value.code == 4
