"""ctypes binding of synth.c: the synthetic G and NF2FF rows every oracle run
uses (test infrastructure only).

``synth_G`` and ``synth_gobj`` return the stand-in for one acmefdfd G file
(the N x N design block and the two NF2FF rows; recipe in synth.c). The
tests, tests/golden/make_golden.py and the CPU legs of bench.py take their
inputs from here, so that no oracle run loads the library under test.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpngf_synth.so")
DX = DY = 0.01 / 60   # pngf-opt/main.cpp:142-160
DZ = 0.01 / 180
_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE, "synth"], check=True)
    L = C.CDLL(LIB)
    I, D, P, Lg, U = C.c_int, C.c_double, C.c_void_p, C.c_long, C.c_ulonglong
    L.synth_num_edges.restype = Lg
    L.synth_num_edges.argtypes = [I, I, I, I]
    L.synth_G.restype = Lg
    L.synth_G.argtypes = [I, I, I, I, D, D, D, D, D, U, P, Lg]
    L.synth_gobj.restype = Lg
    L.synth_gobj.argtypes = [I, I, I, I, D, D, D, U, P]
    _lib = L
    return L


def num_edges(tiles_x, tiles_y, cells=3):
    return int(load().synth_num_edges(tiles_x, tiles_y, cells, cells))


def synth_G(tiles_x, tiles_y, freq_hz, seed=1, eps_r=2.25, cells=3, dx=DX, dy=DY, dz=DZ):
    """N x N complex128 G (C-contiguous, G[i, j] = entry (i, j))."""
    L = load()
    n = num_edges(tiles_x, tiles_y, cells)
    out = np.empty((n, n), dtype=np.complex128, order="F")
    rc = L.synth_G(tiles_x, tiles_y, cells, cells, dx, dy, dz, float(freq_hz), eps_r, seed,
                   out.ctypes.data_as(C.c_void_p), n)
    if rc != n:
        raise ValueError("synth_G: bad arguments")
    return np.ascontiguousarray(out)


def synth_gobj(tiles_x, tiles_y, seed=1, cells=3, dx=DX, dy=DY, dz=DZ):
    """The two NF2FF rows, 2 x N complex128."""
    L = load()
    n = num_edges(tiles_x, tiles_y, cells)
    rows = np.empty((2, n), dtype=np.complex128)
    rc = L.synth_gobj(tiles_x, tiles_y, cells, cells, dx, dy, dz, seed, rows.ctypes.data_as(C.c_void_p))
    if rc != n:
        raise ValueError("synth_gobj: bad arguments")
    return rows


def write_G_file(path, G, gobj_rows=None, num_eobj=3):
    """One G file in acmefdfd's layout (acmefdfd/main.cpp:533-538, read by
    pngf-opt/pngfopt.hpp:163-180): an (N+E-1) x (N+E-1) complex128 matrix in
    column-major order, G in the top-left N x N block and the E-1 objective
    rows below it; the remaining entries are zero. Written column by column
    block so that no second N^2 array is held."""
    n = G.shape[0]
    m = n + num_eobj - 1
    with open(path, "wb") as fh:
        step = max(1, (1 << 26) // max(1, m))
        for j0 in range(0, m, step):
            j1 = min(m, j0 + step)
            blk = np.zeros((j1 - j0, m), dtype=np.complex128)  # row b = column j0 + b of the file
            jj = min(j1, n)
            if j0 < n:
                blk[:jj - j0, :n] = G[:, j0:jj].T
                if gobj_rows is not None:
                    blk[:jj - j0, n:] = np.asarray(gobj_rows)[:, j0:jj].T
            blk.tofile(fh)
