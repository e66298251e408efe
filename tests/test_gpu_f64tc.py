"""FP64-accurate rank-k update on the tensor cores (exact BF16 integer slices,
FP32 accumulation of integers below 2^24 in TMEM, integer recombination)
against the FP64 fused multiply-add update on the FP64 units.

Both are FP64-accurate, so after building M for a design and after several
accepts their M agree to 1e-12 of max|M| (the reference-parity tests in
test_gpu_parity.py run on the tensor-core update, the default)."""
import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu


def make(c, Gs, gobj, tm, fp64_update, max_flips=1):
    from pngf_gb300 import lib
    a = c["tiles"]
    mid = (a - 1) // 2
    h = lib.Handle(a, a, c["freqs"], max_flips=max_flips, fp64_update=fp64_update)
    for f, G in enumerate(Gs):
        h.load_G(f, G, gobj[f])
    h.set_tile_map(tm)
    h.set_source_port(mid, mid, 1, 2)
    h.prepare()
    return h


def test_tensor_update_matches_fp64_units(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    rng = np.random.default_rng(21)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    ht = make(c, Gs, gobj, tm, lib.F64_TENSOR)
    hs = make(c, Gs, gobj, tm, lib.F64_SIMT)

    def check(tag):
        for f in range(len(Gs)):
            Mt, _ = ht.get_M(f)
            Ms, _ = hs.get_M(f)
            err = np.abs(Mt - Ms).max() / np.abs(Ms).max()
            assert err <= 1e-12, (tag, f, err)

    check("prepared")
    mid = (a - 1) // 2
    pool = [t for t in range(a * a) if t != mid * a + mid]
    cands = [[int(t)] for t in rng.choice(pool, size=30, replace=False)]
    for pick in (0, 5, 9, 17):
        et, Ft = ht.eval_candidates(cands)
        es, Fs = hs.eval_candidates(cands)
        np.testing.assert_allclose(Ft, Fs, rtol=1e-12)
        ht.accept(pick)
        hs.accept(pick)
        check("after accept %d" % pick)


def test_tensor_update_in_pieces_matches_fp64_units(cases, built_lib):
    """Accepts of four-tile flips (up to 96 edges, as the 4-fold symmetric
    mode makes): the tensor-core update runs in pieces of 32 edges, each
    rounded once into M (W from FP64 triangular solves above 32 edges). Both
    paths are held against T = (G - I) C^-1 from a direct FP64 inverse for
    each new design. The tensor-core state's floor is the slices' truncation
    (2^-50 of the row and column scales, about 15x the FP64-unit path's
    error here); the bar is 1e-12 of max|T|, two orders inside the parity
    tolerance."""
    from oracle.geometry import Geometry
    from pngf_gb300 import lib
    c = cases["sym_9x9_f2_seed3"]
    Gs, gobj = case_G(c, built_lib)
    a = c["tiles"]
    geo = Geometry(a, a)
    rng = np.random.default_rng(5)
    tm = [int(v) for v in (rng.random(a * a) < 0.2)]
    ht = make(c, Gs, gobj, tm, lib.F64_TENSOR, max_flips=4)
    hs = make(c, Gs, gobj, tm, lib.F64_SIMT, max_flips=4)
    mid = (a - 1) // 2
    pool = [t for t in range(a * a) if t != mid * a + mid]
    n = Gs[0].shape[0]
    ks, errs = [], []
    for size in (1, 1, 4, 4):
        cands = [[int(t) for t in rng.choice(pool, size=size, replace=False)] for _ in range(12)]
        et, Ft = ht.eval_candidates(cands)
        es, Fs = hs.eval_candidates(cands)
        np.testing.assert_allclose(Ft, Fs, rtol=1e-10)
        P = geo.compute_P(tm)
        sizes = [len(geo.flip_set(tm, P, cd)[0]) for cd in cands]
        pick = int(np.argmax(sizes))
        ks.append(sizes[pick])
        ht.accept(pick)
        hs.accept(pick)
        for t in cands[pick]:
            tm[t] ^= 1
        on = geo.compute_P(tm).astype(bool)
        for f, G in enumerate(Gs):
            C = np.eye(n, dtype=complex)
            C[on] = G[on]
            T = (G - np.eye(n)) @ np.linalg.inv(C)
            scale = np.abs(T).max()
            errs.append((np.abs(ht.get_M(f)[0][:n, :n] - T).max() / scale,
                         np.abs(hs.get_M(f)[0][:n, :n] - T).max() / scale))
    assert max(ks) > 64  # three pieces
    assert max(e[0] for e in errs) <= 1e-12, errs
    assert max(e[1] for e in errs) <= 1e-13, errs
    print("ranks", ks, "max relative error against the direct inverse: tensor %.2e, FP64 units %.2e"
          % (max(e[0] for e in errs), max(e[1] for e in errs)))
