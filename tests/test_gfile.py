"""G matrices: the synthetic generator against an independent numpy
restatement, the golden checksums, and the acmefdfd file layout round trip."""
import os

import numpy as np
import pytest

from pngf_gb300 import lib


def numpy_synth_G(tx, ty, f, eps_r=2.25, dx=0.01 / 60, dy=0.01 / 60, dz=0.01 / 180):
    """Dyadic Green's function recipe restated with numpy, without the
    seeded perturbation (which the comparison divides out)."""
    from oracle.geometry import Geometry
    g = Geometry(tx, ty)
    pos, dirs = [], []
    for iy in range(g.ex_ysz):
        for ix in range(g.ex_xsz):
            pos.append(((ix + 0.5) * dx, iy * dy))
            dirs.append((1.0, 0.0))
    for iy in range(g.ey_ysz):
        for ix in range(g.ey_xsz):
            pos.append((ix * dx, (iy + 0.5) * dy))
            dirs.append((0.0, 1.0))
    pos, dirs = np.array(pos), np.array(dirs)
    k = 2 * np.pi * f * np.sqrt(eps_r) / 2.997924579998211e8
    Rv = pos[:, None, :] - pos[None, :, :]
    R = np.sqrt((Rv ** 2).sum(-1))
    np.fill_diagonal(R, 1.0)
    Rh = Rv / R[..., None]
    kr = k * R
    a = 1 + 1j / kr - 1 / kr ** 2
    b = -1 - 3j / kr + 3 / kr ** 2
    ui = (Rh * dirs[:, None, :]).sum(-1)
    uj = (Rh * dirs[None, :, :]).sum(-1)
    dd = (dirs[:, None, :] * dirs[None, :, :]).sum(-1)
    G = 1j * 2 * np.pi * f * 1.25663706127e-6 * dx * dy * dz * np.exp(1j * kr) / (4 * np.pi * R) * (a * dd + b * ui * uj)
    np.fill_diagonal(G, 0)
    G[np.diag_indices_from(G)] = (0.3 + 0.05j) * np.abs(G).max(axis=1)
    return G


def test_synth_matches_numpy(built_lib):
    from oracle import synth
    for G in (lib.synth_G(3, 3, 30e9), synth.synth_G(3, 3, 30e9)):
        Gn = numpy_synth_G(3, 3, 30e9)
        pert = G / Gn - 1.0
        # the seeded perturbation is 1e-3 relative, symmetric, complex Gaussian
        assert np.abs(pert).max() < 1e-2
        assert 5e-4 < np.abs(pert).std() * np.sqrt(2) < 2e-3
        np.testing.assert_allclose(pert, pert.T, atol=1e-15)
        np.testing.assert_allclose(G, G.T, rtol=0, atol=0)


@pytest.mark.parametrize("tiles,freq", [(3, 30e9), (7, 28e9), (11, 33e9)])
def test_library_generator_matches_oracle(tiles, freq, built_lib):
    """The library's G and NF2FF rows equal the oracle's (oracle/synth.c):
    G to rounding (the two evaluate the complex products in different
    orders), the rows bit for bit."""
    from oracle import synth
    Gl, Go = lib.synth_G(tiles, tiles, freq), synth.synth_G(tiles, tiles, freq)
    assert np.abs(Gl - Go).max() <= 1e-15 * np.abs(Go).max()
    np.testing.assert_array_equal(lib.synth_gobj(tiles, tiles), synth.synth_gobj(tiles, tiles))


def test_nf2ff_rows_recipe(built_lib):
    """Row 1 weights the x-directed edges, row 2 the y-directed ones, at
    32 eta0 dV (1 + 1e-3 q)."""
    from oracle import synth
    from oracle.geometry import Geometry
    geo = Geometry(5, 5)
    rows = synth.synth_gobj(5, 5)
    amp = 32 * 3.767303134118051e02 * (0.01 / 60) ** 2 * (0.01 / 180)
    isx = np.arange(geo.n) < geo.nx
    assert np.all(rows[0, ~isx] == 0) and np.all(rows[1, isx] == 0)
    q = np.concatenate([rows[0, isx], rows[1, ~isx]]) / amp - 1.0
    assert np.abs(q).max() < 1e-2 and 5e-4 < np.abs(q).std() * np.sqrt(2) < 2e-3


def test_synth_reproduces_golden_checksums(cases, built_lib):
    from oracle import synth
    for name in ("sym_7x7_f1_seed1", "single_11x11_f3_seed2", "single_21x21_f5_seed1"):
        c = cases[name]
        for f, s in zip(c["freqs"], c["g_checksums"]):
            gens = [synth.synth_G] + ([lib.synth_G] if c["tiles"] <= 11 else [])  # the library's at small sizes
            for G in (gen(c["tiles"], c["tiles"], f, seed=c["g_seed"]) for gen in gens):
                np.testing.assert_allclose(G.real.sum(), s["sum_re"], rtol=1e-12)
                np.testing.assert_allclose(G.imag.sum(), s["sum_im"], rtol=1e-12)
                np.testing.assert_allclose((abs(G) ** 2).sum(), s["sumsq"], rtol=1e-12)
        if c.get("gobj") == "synth":
            r = synth.synth_gobj(c["tiles"], c["tiles"], seed=c["g_seed"])
            np.testing.assert_allclose((abs(r) ** 2).sum(), c["gobj_checksum"]["sumsq"], rtol=1e-12)
            np.testing.assert_allclose(r.real.sum(), c["gobj_checksum"]["sum_re"], rtol=1e-12)


def test_file_roundtrip_and_errors(tmp_path, built_lib):
    import ctypes as C
    from oracle import synth
    G = lib.synth_G(3, 3, 30e9)
    n = G.shape[0]
    gobj = (np.arange(2 * n) * (1 + 2j)).reshape(2, n)
    p = str(tmp_path / "g.bin")
    lib.write_G_file(p, G, gobj)
    assert os.path.getsize(p) == (n + 2) ** 2 * 16
    raw = np.fromfile(p, dtype=np.complex128).reshape(n + 2, n + 2, order="F")
    np.testing.assert_array_equal(raw[:n, :n], G)
    np.testing.assert_array_equal(raw[n:, :n], gobj)
    # the oracle's writer (used for the golden logs) writes the same bytes
    p2 = str(tmp_path / "g2.bin")
    synth.write_G_file(p2, G, gobj)
    assert open(p, "rb").read() == open(p2, "rb").read()
    G2 = np.zeros((n, n), dtype=np.complex128, order="F")
    go2 = np.zeros((2, n), dtype=np.complex128)
    L = lib.load()
    assert L.pngf_read_G_file(p.encode(), n, 3, G2.ctypes.data_as(C.c_void_p), n, go2.ctypes.data_as(C.c_void_p)) == 0
    np.testing.assert_array_equal(G2, G)
    np.testing.assert_array_equal(go2, gobj)
    # short file: an error, not silently zero-filled
    with open(p, "r+b") as fh:
        fh.truncate(16 * n * 10)
    assert L.pngf_read_G_file(p.encode(), n, 3, G2.ctypes.data_as(C.c_void_p), n, None) == 4
    assert L.pngf_read_G_file(str(tmp_path / "missing.bin").encode(), n, 3, G2.ctypes.data_as(C.c_void_p), n,
                              None) == 4
