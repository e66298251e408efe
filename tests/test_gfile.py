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
    G = lib.synth_G(3, 3, 30e9)
    Gn = numpy_synth_G(3, 3, 30e9)
    pert = G / Gn - 1.0
    # the seeded perturbation is 1e-3 relative, symmetric, complex Gaussian
    assert np.abs(pert).max() < 1e-2
    assert 5e-4 < np.abs(pert).std() * np.sqrt(2) < 2e-3
    np.testing.assert_allclose(pert, pert.T, atol=1e-15)
    np.testing.assert_allclose(G, G.T, rtol=0, atol=0)


def test_synth_reproduces_golden_checksums(cases, built_lib):
    c = cases["sym_7x7_f1_seed1"]
    G = lib.synth_G(c["tiles"], c["tiles"], c["freqs"][0], seed=c["g_seed"])
    s = c["g_checksums"][0]
    np.testing.assert_allclose(G.real.sum(), s["sum_re"], rtol=1e-12)
    np.testing.assert_allclose(G.imag.sum(), s["sum_im"], rtol=1e-12)
    np.testing.assert_allclose((abs(G) ** 2).sum(), s["sumsq"], rtol=1e-12)


def test_file_roundtrip_and_errors(tmp_path, built_lib):
    import ctypes as C
    G = lib.synth_G(3, 3, 30e9)
    n = G.shape[0]
    gobj = (np.arange(2 * n) * (1 + 2j)).reshape(2, n)
    p = str(tmp_path / "g.bin")
    lib.write_G_file(p, G, gobj)
    assert os.path.getsize(p) == (n + 2) ** 2 * 16
    raw = np.fromfile(p, dtype=np.complex128).reshape(n + 2, n + 2, order="F")
    np.testing.assert_array_equal(raw[:n, :n], G)
    np.testing.assert_array_equal(raw[n:, :n], gobj)
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
