"""Failures made on the host, none of which faults or traps the GPU.

A singular capacitance matrix: from the empty design, flipping a tile on
gives K = G[s, s] over the tile's edges s, so a G whose row for one of those
edges is zero makes K exactly singular (elimination keeps that row zero).
The reference passes LAPACK's info by (pngfopt.hpp:493-510) and its F is
NaN/inf, which never passes the accept test; here the candidate kernel also
reports PNGF_ERR_SINGULAR for it, the accept refuses it, and the other
candidates of the batch are unaffected."""
import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu


def test_singular_capacitance_is_reported(cases, built_lib):
    from oracle.geometry import Geometry
    from pngf_gb300 import lib
    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    geo = Geometry(7, 7)
    tm = [0] * 49
    P = geo.compute_P(tm)
    bad, good = 10, 40
    s_bad, _ = geo.flip_set(tm, P, [bad])
    s_good, _ = geo.flip_set(tm, P, [good])
    assert not set(s_bad) & set(s_good)
    G = Gs[0].copy()
    G[s_bad[0], :] = 0.0
    h = lib.Handle(7, 7, c["freqs"][:1], max_flips=1)
    h.load_G(0, G, gobj[0])
    h.set_tile_map(tm)
    h.set_source_port(3, 3, 1, 2)
    h.prepare()
    eo, F = h.eval_candidates([[bad], [good]])
    assert not np.isfinite(F[0])
    assert np.isfinite(F[1])
    with pytest.raises(lib.PngfError) as e:
        h.accept(0)
    assert e.value.code == 5  # PNGF_ERR_SINGULAR
    assert list(h.tile_map()) == tm
    h.eval_candidates([[bad], [good]])
    h.accept(1)
    tm[good] = 1
    assert list(h.tile_map()) == tm
