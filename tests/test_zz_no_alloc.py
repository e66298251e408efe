"""pngf_accept_edges_noalloc: the accept step for callers that cannot
allocate device memory (it keeps its scratch in a fixed device array).

Through the C ABI, on device buffers the test owns (torch tensors):
  * two accepts in a row give the same M as the oracle's M-algebra accept
    (oracle/refalg.py MState, numpy on the CPU) and as the handle's own accept
    (pngf_accept), within 1e-10 of max|M|;
  * an accept with no status pointer (the status word inside the scratch
    array) does the same;
  * the largest flip the fixed scratch admits at 11x11 tiles (k = 104 edges)
    matches the oracle;
  * an edge index outside [0, n) is refused on the device with PNGF_ERR_ARG
    and a singular capacitance matrix with PNGF_ERR_SINGULAR, M left
    bit-for-bit unchanged in both cases;
  * sizes beyond the fixed scratch are refused before any device work.
This file sorts last so that a run stopping at the first failure has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu

TOL = 1e-10
ERR_ARG, ERR_SINGULAR, ERR_SCRATCH = 1, 5, 10


def _prepared(lib, a, freqs, G, gobj, tm, max_flips=4):
    h = lib.Handle(a, a, freqs, max_flips=max_flips)
    h.load_G(0, G, gobj)
    h.set_tile_map(tm)
    h.set_source_port(a // 2, a // 2, 1, 2)
    h.prepare()
    return h


def _device_M(h):
    import torch
    n, E, ldm = h.n, h.E, h.ldm
    M0, einc = h.get_M(0)
    Md = torch.zeros((n + E, ldm), dtype=torch.complex128, device="cuda")
    Md[:, :n + 1] = torch.from_numpy(M0).cuda()
    return M0, einc, Md, torch.from_numpy(einc).cuda()


def _call(L, Md, ldm, n, E, einc_d, s, d, status, k=None, stream=None):
    import torch
    s_d = torch.from_numpy(np.asarray(s, dtype=np.int32)).cuda()
    d_d = torch.from_numpy(np.asarray(d, dtype=np.int8)).cuda()
    st = C.c_void_p(status.data_ptr()) if status is not None else None
    rc = L.pngf_accept_edges_noalloc(C.c_void_p(Md.data_ptr()), ldm, n, E, C.c_void_p(einc_d.data_ptr()),
                                     C.c_void_p(s_d.data_ptr()), C.c_void_p(d_d.data_ptr()),
                                     len(s) if k is None else k, st,
                                     C.c_void_p(stream or torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc


def _oracle_accept(M, einc, s, d):
    from oracle.refalg import MState
    st = MState(M.copy(), einc)
    st.eval(np.asarray(s), np.asarray(d, dtype=np.int64))
    st.accept()
    return st.M


def test_noalloc_accept_matches_oracle_and_handle(cases, built_lib):
    import torch

    from oracle.geometry import Geometry
    from pngf_gb300 import lib

    c = cases["sym_7x7_f1_seed1"]
    Gs, gobj = case_G(c, built_lib)
    a = 7
    geo = Geometry(a, a)
    rng = np.random.default_rng(11)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    h = _prepared(lib, a, c["freqs"], Gs[0], gobj[0], tm)
    n, E, ldm = h.n, h.E, h.ldm
    M_host, einc, Md, einc_d = _device_M(h)
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    L = built_lib

    for i, tiles in enumerate(([10, 38], [16, 18, 30, 32])):  # two accepts in a row
        P = geo.compute_P(tm)
        s, d = geo.flip_set(tm, P, tiles)
        M_host = _oracle_accept(M_host, einc, s, d)
        h.eval_candidates([tiles])
        h.accept(0)
        ref, _ = h.get_M(0)
        # the second call keeps its status word inside the scratch array
        rc = _call(L, Md, ldm, n, E, einc_d, s, d, status if i == 0 else None)
        assert rc == 0
        if i == 0:
            assert int(status.item()) == 0
        got = Md[:, :n + 1].cpu().numpy()
        scale = np.abs(M_host).max()
        assert np.abs(got - M_host).max() <= TOL * scale
        assert np.abs(got - ref).max() <= TOL * scale
        for t in tiles:
            tm[t] ^= 1

    # an index outside [0, n): refused on the device, M untouched
    before = Md.clone()
    bad = np.array(s, dtype=np.int64)
    bad[-1] = n
    status.fill_(-7)
    assert _call(L, Md, ldm, n, E, einc_d, bad, d, status) == 0
    assert int(status.item()) == ERR_ARG
    assert torch.equal(Md, before)
    bad[-1] = -3
    status.fill_(-7)
    assert _call(L, Md, ldm, n, E, einc_d, bad, d, status) == 0
    assert int(status.item()) == ERR_ARG
    assert torch.equal(Md, before)
    # a sign that is not +-1
    dd = np.array(d, dtype=np.int64)
    dd[0] = 2
    status.fill_(-7)
    assert _call(L, Md, ldm, n, E, einc_d, s, dd, status) == 0
    assert int(status.item()) == ERR_ARG
    assert torch.equal(Md, before)

    # a singular capacitance matrix: adding edge e with T[e,e] = -1 gives K = 0
    P = geo.compute_P(tm)
    e = int(np.nonzero(P == 0)[0][0])
    Md[e, e] = -1.0
    before = Md.clone()
    status.fill_(-7)
    assert _call(L, Md, ldm, n, E, einc_d, [e], [1], status) == 0
    assert int(status.item()) == ERR_SINGULAR
    assert torch.equal(Md, before)

    # sizes beyond the fixed scratch are refused before any device work
    huge_ldm = 1 << 22
    assert _call(L, Md, huge_ldm, n, E, einc_d, s, d, None) == ERR_SCRATCH
    assert _call(L, Md, ldm, n, E, einc_d, s, d, None, k=105) == ERR_ARG
    h.close()


def test_noalloc_largest_flip_matches_oracle(built_lib):
    """k = 104 edges at 11x11 tiles (N = 2244): the largest flip the header
    admits, with its A and W within the fixed scratch."""
    import torch

    from oracle.geometry import Geometry
    from pngf_gb300 import lib

    a, f = 11, 30e9
    geo = Geometry(a, a)
    G = np.ascontiguousarray(lib.synth_G(a, a, f, seed=5))
    gobj = np.zeros((2, G.shape[0]), dtype=np.complex128)
    rng = np.random.default_rng(3)
    tm = [int(v) for v in rng.integers(0, 2, a * a)]
    h = _prepared(lib, a, [f], G, gobj, tm)
    n, E, ldm = h.n, h.E, h.ldm
    M_host, einc, Md, einc_d = _device_M(h)
    P = geo.compute_P(tm)
    s = np.sort(rng.choice(n, size=104, replace=False))
    d = np.where(P[s] == 0, 1, -1)
    want = _oracle_accept(M_host, einc, s, d)
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    assert _call(built_lib, Md, ldm, n, E, einc_d, s, d, status) == 0
    assert int(status.item()) == 0
    got = Md[:, :n + 1].cpu().numpy()
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    h.close()
