"""Yee-edge geometry of the PNGF design region (test infrastructure only).

Restates pngf-opt/pngfopt.hpp:
  * edge numbering, pngfopt.hpp:86-94: Ex edges first on a (tx*cx) x (ty*cy+1)
    grid, x fastest; then Ey edges on a (tx*cx+1) x (ty*cy) grid;
  * compute_P_matrix, pngfopt.hpp:624-664: an edge is a design unknown (P=1)
    when any tile that owns it is set; shared tile-boundary edges count once;
  * set_source_port, pngfopt.hpp:559-618: the port is a cx-wide, y_size-high
    block of Ex edges starting y_offset cells into the port tile.
"""
from __future__ import annotations

import numpy as np


class Geometry:
    def __init__(self, tiles_x: int, tiles_y: int, cells_x: int = 3, cells_y: int = 3):
        self.tx, self.ty, self.cx, self.cy = tiles_x, tiles_y, cells_x, cells_y
        self.ex_xsz = tiles_x * cells_x
        self.ex_ysz = tiles_y * cells_y + 1
        self.ey_xsz = tiles_x * cells_x + 1
        self.ey_ysz = tiles_y * cells_y
        self.nx = self.ex_xsz * self.ex_ysz
        self.n = self.nx + self.ey_xsz * self.ey_ysz
        self.map_sz = tiles_x * tiles_y
        self.tile_edges = [self._edges_of(t) for t in range(self.map_sz)]

    def _edges_of(self, index: int) -> np.ndarray:
        """Edges set by tile `index` (pngfopt.hpp:637-661), ascending."""
        ty = index // self.tx
        tx = index - ty * self.tx
        base_x = tx * self.cx + ty * self.cy * self.ex_xsz
        base_y = self.nx + tx * self.cx + ty * self.cy * self.ey_xsz
        ex = [base_x + ii + jj * self.ex_xsz for jj in range(self.cy + 1) for ii in range(self.cx)]
        ey = [base_y + ii + jj * self.ey_xsz for jj in range(self.cy) for ii in range(self.cx + 1)]
        return np.array(sorted(ex + ey), dtype=np.int64)

    def compute_P(self, tile_map) -> np.ndarray:
        P = np.zeros(self.n, dtype=np.int8)
        for t in range(self.map_sz):
            if tile_map[t]:
                P[self.tile_edges[t]] = 1
        return P

    def flip_set(self, tile_map, P, tiles):
        """Edges whose P changes when `tiles` are flipped, ascending, with the
        change d = P_new - P_old (pngfopt.hpp:384-418)."""
        m = np.array(tile_map, dtype=np.int8).copy()
        for t in tiles:
            m[t] ^= 1
        Pn = self.compute_P(m)
        dP = Pn.astype(np.int64) - P.astype(np.int64)
        s = np.nonzero(dP)[0]
        return s, dP[s]

    def port_indices(self, tile_x: int, tile_y: int, y_offset: int, y_size: int) -> np.ndarray:
        if y_offset + y_size > self.cy:
            raise ValueError("set_source_port: invalid port y position and height parameters.")
        idx = []
        for jj in range(y_size):
            for ii in range(self.cx):
                idx.append((tile_x * self.cx + ii) + (tile_y * self.cy + jj + y_offset) * self.ex_xsz)
        return np.array(idx, dtype=np.int64)


def port_setup(G: np.ndarray, gobj_rows: np.ndarray, port: np.ndarray):
    """Gobj row 0, Einc, Vinc, LN1inc, LN2inc (pngfopt.hpp:572-617).

    G: N x N complex, gobj_rows: (E-1) x N. Sums run in port order, as the
    reference accumulates them."""
    n = G.shape[0]
    E = 1 + gobj_rows.shape[0]
    Gobj = np.zeros((E, n), dtype=np.complex128)
    Gobj[1:] = gobj_rows
    Einc = np.zeros(n, dtype=np.complex128)
    ln1 = 0j
    ln2 = 0j
    for p in port:
        Gobj[0] += G[p, :]
        Einc += G[:, p]
        if E > 1:
            ln1 += Gobj[1, p]
            ln2 += Gobj[2, p]
    vinc = 0j
    for p in port:
        vinc += Einc[p]
    return Gobj, Einc, vinc, ln1, ln2
