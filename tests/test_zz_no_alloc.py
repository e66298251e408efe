"""pngf_accept_edges_noalloc: the accept step for callers that cannot
allocate device memory (it keeps its scratch in a fixed device array).

Through the C ABI, on device buffers the test owns (torch tensors), two
accepts in a row must give the same M as the handle's own accept
(pngf_accept), within 1e-10 of max|M|. This file sorts last so that a run
stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_noalloc_accept_matches_handle_accept(cases, built_lib):
    import torch

    from oracle.geometry import Geometry
    from pngf_gb300 import lib

    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    a = 7
    geo = Geometry(a, a)
    rng = np.random.default_rng(11)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    h = lib.Handle(a, a, c["freqs"], max_flips=4)
    h.load_G(0, Gs[0], gobj[0])
    h.set_tile_map(tm)
    h.set_source_port(3, 3, 1, 2)
    h.prepare()
    n, E, ldm = h.n, h.E, h.ldm
    M0, einc = h.get_M(0)
    Md = torch.zeros((n + E, ldm), dtype=torch.complex128, device="cuda")
    Md[:, :n + 1] = torch.from_numpy(M0).cuda()
    einc_d = torch.from_numpy(einc).cuda()
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    L = built_lib

    for tiles in ([10, 38], [16, 18, 30, 32]):  # two accepts in a row
        P = geo.compute_P(tm)
        s, d = geo.flip_set(tm, P, tiles)
        h.eval_candidates([tiles])
        h.accept(0)
        ref, _ = h.get_M(0)
        s_d = torch.from_numpy(s.astype(np.int32)).cuda()
        d_d = torch.from_numpy(d.astype(np.int8)).cuda()
        rc = L.pngf_accept_edges_noalloc(C.c_void_p(Md.data_ptr()), ldm, n, E, C.c_void_p(einc_d.data_ptr()),
                                         C.c_void_p(s_d.data_ptr()), C.c_void_p(d_d.data_ptr()), len(s),
                                         C.c_void_p(status.data_ptr()), C.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        got = Md[:, :n + 1].cpu().numpy()
        assert np.abs(got - ref).max() <= TOL * np.abs(ref).max()
        for t in tiles:
            tm[t] ^= 1

    # sizes beyond the fixed scratch are refused before any device work
    huge_ldm = 1 << 22
    rc = L.pngf_accept_edges_noalloc(C.c_void_p(Md.data_ptr()), huge_ldm, n, E, C.c_void_p(einc_d.data_ptr()),
                                     C.c_void_p(s_d.data_ptr()), C.c_void_p(d_d.data_ptr()), len(s), None,
                                     C.c_void_p(stream))
    assert rc == 10  # PNGF_ERR_SCRATCH
    rc = L.pngf_accept_edges_noalloc(C.c_void_p(Md.data_ptr()), ldm, n, E, C.c_void_p(einc_d.data_ptr()),
                                     C.c_void_p(s_d.data_ptr()), C.c_void_p(d_d.data_ptr()), 105, None,
                                     C.c_void_p(stream))
    assert rc == 1  # PNGF_ERR_ARG
