"""Complex64 form (T in complex64, rank-k accept update on tcgen05 tensor
cores with 3xTF32 split products; capacitance LU, y, R, Eobj, objective and
accept test in FP64) against the plain FP64 form on the same G and design.

Tolerances: the prepared state differs only by the complex64 rounding of T
(relative 2^-24); tensor-core accepts keep T within 5e-6 of max|T|;
newEobj within 1e-5 relative, F within 1e-7 relative (1e-4 after accepts:
the flip undoing an accept cancels in its NF2FF outputs); a DBS run's
objective within 1e-3 relative of the FP64 run's."""
import numpy as np
import pytest

from conftest import case_G, force_port_tiles, free_tiles

pytestmark = pytest.mark.gpu


def handles(c, Gs, gobj, tm, max_flips):
    from pngf_gb300 import lib
    a = c["tiles"]
    mid = (a - 1) // 2
    out = []
    for prec in (lib.PREC_FP64, lib.PREC_C64):
        h = lib.Handle(a, a, c["freqs"], precision=prec, max_flips=max_flips)
        for f, G in enumerate(Gs):
            h.load_G(f, G, gobj[f])
        h.set_tile_map(tm)
        h.set_source_port(mid, mid, 1, 2)
        h.prepare()
        out.append(h)
    return out


@pytest.mark.parametrize("max_flips", [1, 4])
def test_c64_eval_and_tensor_core_accept_match_fp64(max_flips, cases, built_lib):
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    rng = np.random.default_rng(7)
    tm = force_port_tiles(rng.integers(0, 2, a * a), a, a)
    h64, h32 = handles(c, Gs, gobj, tm, max_flips)
    n = h64.n
    for f in range(len(Gs)):
        M64, _ = h64.get_M(f)
        M32, _ = h32.get_M(f)
        scale = np.abs(M64[:n, :n]).max()
        assert np.abs(M32[:n, :n] - M64[:n, :n]).max() <= 2e-7 * scale
        # R and Eobj stay FP64; the two handles build them with different chunkings
        np.testing.assert_allclose(M32[n:], M64[n:], rtol=0, atol=1e-11 * np.abs(M64[n:]).max())
    # DBS never flips the source tile or its forced neighbours (main.cpp:358-359)
    pool = free_tiles(a, a)
    cands = [[int(t) for t in rng.choice(pool, size=max_flips, replace=False)] for _ in range(40)]
    eo64, F64 = h64.eval_candidates(cands)
    eo32, F32 = h32.eval_candidates(cands)
    np.testing.assert_allclose(eo32, eo64, rtol=1e-5, atol=1e-5 * np.abs(eo64).max())
    np.testing.assert_allclose(F32, F64, rtol=1e-7)
    for pick in (3, 11):  # two tensor-core accepts in a row
        h64.accept(pick)
        h32.accept(pick)
        for f in range(len(Gs)):
            M64, _ = h64.get_M(f)
            M32, _ = h32.get_M(f)
            scale = np.abs(M64[:n, :n]).max()
            err = np.abs(M32[:n, :n] - M64[:n, :n]).max()
            # complex64 rounding of T (6e-8) reaches the update through K^-1:
            # ~1e-6 for 4-tile flips (k up to 96), below 1e-7 for single tiles
            assert err <= 5e-6 * scale, (pick, f, err / scale)
            e64, _ = h64.eobj(f)
            e32, _ = h32.eobj(f)
            np.testing.assert_allclose(e32, e64, rtol=1e-5, atol=1e-5 * np.abs(e64).max())
        eo64, F64 = h64.eval_candidates(cands)
        eo32, F32 = h32.eval_candidates(cands)
        # after accepts T carries ~1e-6 of max|T| (complex64 rounding through K^-1
        # and the 3xTF32 products); the flip that undoes an accept cancels in its
        # NF2FF outputs (measured: 2e-5 relative in F on this case)
        np.testing.assert_allclose(F32, F64, rtol=1e-4)


def test_drift_check_measures_complex64_error(cases, built_lib):
    """The drift check's FP64 rows (refined from G) reproduce the FP64 state's
    rows, so the reported drift equals the true complex64 error on them."""
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    rng = np.random.default_rng(4)
    tm = force_port_tiles(rng.integers(0, 2, a * a), a, a)
    h64, h32 = handles(c, Gs, gobj, tm, 1)
    n = h64.n
    pool = free_tiles(a, a)
    for step in range(3):
        cands = [[int(t)] for t in rng.choice(pool, size=8, replace=False)]
        h64.eval_candidates(cands)
        h32.eval_candidates(cands)
        h64.accept(step)
        h32.accept(step)
    rows = [((2 * r + 1) * n) // 8 for r in range(4)]
    true = 0.0
    for f in range(len(Gs)):
        T64 = h64.get_M(f)[0][rows, :n]
        T32 = h32.get_M(f)[0][rows, :n]
        true = max(true, np.abs(T32 - T64).max() / np.abs(T64).max())
    drift = h32.drift_check(4)
    assert 1e-9 < drift < 1e-5
    assert abs(drift - true) <= 0.05 * true + 1e-12


def test_c64_dbs_reaches_fp64_objective(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    res = {}
    for prec in (lib.PREC_FP64, lib.PREC_C64):
        h = lib.Handle(11, 11, c["freqs"], precision=prec, max_flips=1)
        for f, G in enumerate(Gs):
            h.load_G(f, G, gobj[f])
        d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=c["seed"], max_evals=600,
                    drift_every=16, drift_tol=1e-4)
        res[prec] = d.run()
    F64, F32 = res[lib.PREC_FP64].F_best, res[lib.PREC_C64].F_best
    assert abs(F32 - F64) <= 1e-3 * abs(F64)
    s32 = res[lib.PREC_C64]
    assert s32.drift_checks >= 1 and 0 < s32.drift_max < 1e-2
    # a drift above the tolerance rebuilt the state from G
    assert s32.drift_max <= 1e-4 or s32.refreshes >= 1
