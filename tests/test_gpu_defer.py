"""Deferred complex64 updates (defer_rank > 0): the T part of each accept is
appended to pending factors and flushed to T on the tensor cores when the
pending rank would pass the cap; candidates and accepts read T minus the
pending product (summed in FP32).

Against the same complex64 form without deferral: candidate objectives
within 1e-6 relative and T (after the flush a state read forces) within
5e-6 of max|T| over a run of accepts that crosses several flushes; a DBS run
ends within 1e-3 relative of the plain FP64 run's objective."""
import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu


def make(c, Gs, gobj, tm, prec, defer_rank=0):
    from pngf_gb300 import lib
    a = c["tiles"]
    mid = (a - 1) // 2
    h = lib.Handle(a, a, c["freqs"], precision=prec, max_flips=1, defer_rank=defer_rank)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    h.set_tile_map(tm)
    h.set_source_port(mid, mid, 1, 2)
    h.prepare()
    return h


@pytest.mark.parametrize("cap", [48, 192])
def test_deferred_accepts_match_immediate(cap, cases, built_lib):
    """cap 48: a flush every accept or two (k <= 24); cap 192: nothing flushed
    until the state is read. Both complex64 forms are compared with the FP64
    form: deferral may not make the complex64 error more than twice larger."""
    from pngf_gb300 import lib
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    rng = np.random.default_rng(21)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    h64 = make(c, Gs, gobj, tm, lib.PREC_FP64)
    h0 = make(c, Gs, gobj, tm, lib.PREC_C64)
    h1 = make(c, Gs, gobj, tm, lib.PREC_C64, defer_rank=cap)
    mid = (a - 1) // 2
    pool = [t for t in range(a * a) if t not in (mid * a + mid, mid * a + mid - 1, mid * a + mid + 1)]
    for step in range(7):
        cands = [[int(t)] for t in rng.choice(pool, size=30, replace=False)]
        _, F64 = h64.eval_candidates(cands)
        _, F0 = h0.eval_candidates(cands)
        _, F1 = h1.eval_candidates(cands)
        np.testing.assert_allclose(F1, F0, rtol=1e-6)
        np.testing.assert_allclose(F1, F64, rtol=1e-6)
        pick = int(np.nanargmin(F64))
        for h in (h64, h0, h1):
            h.accept(pick)
    n = h0.n
    for f in range(len(Gs)):
        M64, _ = h64.get_M(f)
        M0, _ = h0.get_M(f)
        M1, _ = h1.get_M(f)  # flushes what is pending
        scale = np.abs(M64[:n, :n]).max()
        e0 = np.abs(M0[:n, :n] - M64[:n, :n]).max()
        e1 = np.abs(M1[:n, :n] - M64[:n, :n]).max()
        assert e1 <= 2.0 * e0 + 1e-6 * scale, (f, e0 / scale, e1 / scale)
        np.testing.assert_allclose(M1[n:], M64[n:], rtol=0, atol=1e-5 * np.abs(M64[n:]).max())
    assert abs(h1.objective() - h64.objective()) <= 1e-6 * abs(h64.objective())
    for h in (h64, h0, h1):
        h.close()


def test_deferred_dbs_reaches_fp64_objective(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    F = []
    for prec, defer in ((lib.PREC_FP64, 0), (lib.PREC_C64, 192)):
        h = lib.Handle(a, a, c["freqs"], precision=prec, max_flips=1, defer_rank=defer)
        for f, G in enumerate(Gs):
            h.load_G(f, G, gobj[f])
        d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=c["seed"], drift_every=32, drift_tol=1e-4)
        s = d.run()
        assert s.converged
        F.append(s.F_best)
        d.close()
        h.close()
    assert abs(F[1] - F[0]) <= 1e-3 * abs(F[0])


def test_defer_rank_below_one_accept_is_refused(built_lib):
    from pngf_gb300 import lib
    with pytest.raises(lib.PngfError):
        lib.Handle(7, 7, [30e9], precision=lib.PREC_C64, max_flips=1, defer_rank=8)
