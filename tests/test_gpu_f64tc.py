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


def make(c, Gs, gobj, tm, fp64_update):
    from pngf_gb300 import lib
    a = c["tiles"]
    mid = (a - 1) // 2
    h = lib.Handle(a, a, c["freqs"], max_flips=1, fp64_update=fp64_update)
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
