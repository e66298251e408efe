"""Numpy restatements of the two algebras (test infrastructure only).

``RefState`` follows the reference optimizer on C^-1:
  compute_C_matrix  pngf-opt/pngfopt.hpp:196-233   C = (I-P) + P G
  invertMatrix      pngf-opt/linalg.hpp:34-85      C <- C^-1 (LU)
  compute_PEinc     pngfopt.hpp:542-552            PEinc = -P Einc
  compute_R_matrix  pngfopt.hpp:237-250            R = Gobj C^-1, S = C^-1 PEinc
  compute_updated_Eobj pngfopt.hpp:379-539         Woodbury candidate evaluation
  update_C_inv      pngfopt.hpp:256-367            rank-k Woodbury update of C^-1

``MState`` is the formulation the GPU implements. With H = G - I it keeps
    M = [[T, y], [R, Eobj]],  T = H C^-1,  y = T PEinc,
so that a candidate needs only gathers of M and accepting it is one rank-k
update of M (derivation in the library header include/pngf_gb300.h).
``MState.build`` starts from P = 0 (T = H, R = Gobj, y = 0, Eobj = 0) and
accepts the design's set edges in chunks, which is how the GPU initialises.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

C0 = 2.997924579998211e8   # main.cpp:101
ETA0 = 3.767303134118051e02  # main.cpp:102


def objective(eobj, vinc, ln1, ln2, k0, dx, dy, dz):
    """One frequency's term of F (main.cpp:277-289 and 407-413).

    Returns (F_f, S11, D)."""
    zin = -(eobj[0] + vinc) * dx * 0.5 / (2.0 * dy * dz)
    s11 = (zin - 50.0) / (zin + 50.0)
    a = eobj[1] + ln1 if len(eobj) > 1 else 0j
    b = eobj[2] + ln2 if len(eobj) > 2 else 0j
    D = (k0 * k0 / (32 * np.pi * np.pi * ETA0)) * (np.conj(a) * a + np.conj(b) * b).real
    D = 4.0 * np.pi * D / (-(eobj[0] + vinc) * dx * 0.5 * (2.0 * dy * dz) * 0.5).real
    m = abs(s11)
    return 200.0 * m * m + (15.0 - D) * (15.0 - D), s11, D


class RefState:
    """The reference's per-frequency optimizer state on C^-1."""

    def __init__(self, G, Gobj, Einc, P):
        n = G.shape[0]
        self.G, self.Gobj, self.Einc = G, Gobj, Einc
        self.P = P.astype(np.int8).copy()
        p = self.P.astype(bool)
        C = np.eye(n, dtype=np.complex128)
        C[p, :] = G[p, :]
        self.Cinv = np.linalg.inv(C)
        self._refresh(compute_eobj=True)

    def _refresh(self, compute_eobj):
        self.PEinc = np.where(self.P.astype(bool), -self.Einc, 0)
        self.R = self.Gobj @ self.Cinv
        self.S = self.Cinv @ self.PEinc
        if compute_eobj:
            self.Eobj = self.R @ self.PEinc

    def eval(self, s, d):
        n = self.G.shape[0]
        k = len(s)
        V = self.G[s, :].copy()
        V[np.arange(k), s] -= 1.0
        K = V @ self.Cinv[:, s] * d[None, :] + np.eye(k)
        Snew = self.S - self.Cinv[:, s] @ (self.Einc[s] * d)
        VS = V @ Snew
        lu = sla.lu_factor(K)
        x = sla.lu_solve(lu, VS)
        RU = self.R[:, s] * d[None, :]
        new = self.Gobj @ Snew - RU @ x
        self._last = (s, d, V, K)
        return new

    def accept(self, new_eobj):
        s, d, V, K = self._last
        CinvU = self.Cinv[:, s] * d[None, :]
        self.Cinv = self.Cinv - CinvU @ (np.linalg.inv(K) @ (V @ self.Cinv))
        self.P[s] += d.astype(np.int8)
        self._refresh(compute_eobj=False)
        self.Eobj = new_eobj


class MState:
    """The GPU path's per-frequency state, M = [[T, y], [R, Eobj]]."""

    def __init__(self, M, Einc):
        self.M, self.Einc = M, Einc
        self.n = M.shape[1] - 1

    @classmethod
    def build(cls, G, Gobj, Einc, P, chunk=96):
        n = G.shape[0]
        E = Gobj.shape[0]
        M = np.zeros((n + E, n + 1), dtype=np.complex128)
        M[:n, :n] = G - np.eye(n)
        M[n:, :n] = Gobj
        st = cls(M, Einc)
        on = np.nonzero(P)[0]
        for c0 in range(0, len(on), chunk):
            s = on[c0:c0 + chunk]
            d = np.ones(len(s), dtype=np.int64)
            st.eval(s, d)
            st.accept()
        return st

    @property
    def Eobj(self):
        return self.M[self.n:, self.n]

    def eval(self, s, d):
        n = self.n
        M = self.M
        Tss = M[np.ix_(s, s)]
        K = np.eye(len(s)) + Tss * d[None, :]
        w = M[s, n] - Tss @ (d * self.Einc[s])
        lu = sla.lu_factor(K)
        x = sla.lu_solve(lu, w)
        z = d * (self.Einc[s] + x)
        self._last = (s, d, lu, z)
        return M[n:, n] - M[n:, s] @ z

    def accept(self):
        s, d, lu, z = self._last
        n = self.n
        A = self.M[:, s].copy()
        W = np.empty((len(s), n + 1), dtype=np.complex128)
        W[:, :n] = d[:, None] * sla.lu_solve(lu, self.M[s, :n])
        W[:, n] = z
        self.M -= A @ W
