"""The DBS loop of pngf-opt/main.cpp:181-459, restated (test infrastructure only).

Two candidate modes:
  * ``sym``    - the reference's 4-fold mirror-symmetric quarter hat
                 (main.cpp:181, 187-208, 343-392);
  * ``single`` - one tile per candidate over the whole map; the source tile
                 and both forced-metal port neighbours are skipped; a random
                 initial design draws one rand_binary() per tile in order.

``run_dbs`` drives per-frequency states that provide ``eval(s, d) -> newEobj``
and ``accept(newEobj)`` (``refalg.RefState``) or ``accept()``
(``refalg.MState``), and returns the log in the same row format as the
reference build's driver (oracle/ref_driver.cpp).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .geometry import Geometry, port_setup
from .magichat import MagicHat
from .refalg import C0, MState, RefState, objective

DX = 0.01 / 60.0   # main.cpp:157-160
DY = 0.01 / 60.0
DZ = 0.01 / 180.0


def initial_design(geo: Geometry, hat: MagicHat, sym: bool, random_init: bool):
    xsz, ysz = geo.tx, geo.ty
    tm = [0] * (xsz * ysz)
    if random_init:
        if sym:
            for j in range(int((ysz - 1) * 0.5 + 1)):
                for i in range(int((xsz - 1) * 0.5 + 1)):
                    st = hat.rand_binary()
                    tm[i + j * xsz] = st
                    if i < (xsz - 1) * 0.5:
                        tm[((xsz - 1) - i) + j * xsz] = st
                    if j < (ysz - 1) * 0.5:
                        tm[i + ((ysz - 1) - j) * xsz] = st
                        if i < (xsz - 1) * 0.5:
                            tm[((xsz - 1) - i) + ((ysz - 1) - j) * xsz] = st
        else:
            for i in range(xsz * ysz):
                tm[i] = hat.rand_binary()
    mx, my = int((xsz - 1) * 0.5), int((ysz - 1) * 0.5)
    tm[my * xsz + mx - 1] = 1
    tm[my * xsz + mx + 1] = 1
    tm[my * xsz + mx] = 0
    tm[(my - 1) * xsz + mx] = 0
    tm[(my + 1) * xsz + mx] = 0
    return tm


def hat_size(geo: Geometry, sym: bool) -> int:
    if sym:
        return int(((geo.tx - 1) * 0.5 + 1) * ((geo.ty - 1) * 0.5 + 1)) - 1
    return geo.tx * geo.ty


def next_candidate(geo: Geometry, hat: MagicHat, sym: bool, last_tried: int):
    """Draws until a valid candidate (main.cpp:343-392). Returns
    (log_index, tiles, last_tried) or None when the hat is empty."""
    xsz, ysz = geo.tx, geo.ty
    mx, my = int((xsz - 1) * 0.5), int((ysz - 1) * 0.5)
    qx = int((xsz - 1) * 0.5 + 1)
    while True:
        r = hat.draw()
        if r < 0:
            return None
        if sym:
            ty = r // qx
            tx = r - ty * qx
        else:
            ty = r // xsz
            tx = r - ty * xsz
        if r == last_tried:
            continue
        if tx == mx and ty == my:
            continue
        if tx == mx - 1 and ty == my:
            continue
        if not sym and tx == mx + 1 and ty == my:
            continue
        if not sym:
            tiles = [tx + ty * xsz]
        elif tx == mx:
            tiles = [tx + ty * xsz, tx + ((ysz - 1) - ty) * xsz]
        elif ty == my:
            tiles = [tx + ty * xsz, ((xsz - 1) - tx) + ty * xsz]
        else:
            tiles = [tx + ty * xsz, ((xsz - 1) - tx) + ty * xsz,
                     tx + ((ysz - 1) - ty) * xsz, ((xsz - 1) - tx) + ((ysz - 1) - ty) * xsz]
        return tx + ty * xsz, tiles, r


@dataclass
class DbsLog:
    init_map: list
    start_F: float
    start_perf: list
    rows: list = field(default_factory=list)   # (eval, tile, accept, F, F_best, perf[3*nf])
    final_map: list = field(default_factory=list)
    evals: int = 0
    accepts: int = 0
    converged: bool = False


class DbsRunner:
    """DBS on per-frequency CPU states, one decision per ``step()``.

    Gs: list of N x N complex G per frequency; algebra: "ref" (numpy on C^-1),
    "port" (the C restatement on C^-1) or "m" (numpy on M)."""

    def __init__(self, Gs, gobj_rows, freqs, tiles_x, tiles_y, seed, sym=True, random_init=True,
                 max_evals=0, algebra="ref", run_index=0):
        self.geo = geo = Geometry(tiles_x, tiles_y)
        self.sym, self.max_evals, self.algebra = sym, max_evals, algebra
        self.hat = MagicHat(seed, run_index, hat_size(geo, sym))
        self.tm = initial_design(geo, self.hat, sym, random_init)
        self.P = geo.compute_P(self.tm)
        mx, my = int((tiles_x - 1) * 0.5), int((tiles_y - 1) * 0.5)
        port = geo.port_indices(mx, my, 1, 2)
        self.states, self.consts = [], []
        for f, G in enumerate(Gs):
            Gobj, Einc, vinc, ln1, ln2 = port_setup(G, gobj_rows[f], port)
            if algebra == "ref":
                st = RefState(G, Gobj, Einc, self.P)
            elif algebra == "port":
                from .port import PortState
                st = PortState(G, Gobj, Einc, self.P, kmax=96 if sym else 24)
            else:
                st = MState.build(G, Gobj, Einc, self.P)
            self.states.append(st)
            self.consts.append((vinc, ln1, ln2, 2.0 * np.pi * freqs[f] / C0))
        self.F_best, perf0 = self.score([st.Eobj for st in self.states])
        self.log = DbsLog(init_map=list(self.tm), start_F=self.F_best, start_perf=perf0)
        self.last = -1
        self.done = False

    def score(self, eobjs):
        F, perf = 0.0, []
        for f, eo in enumerate(eobjs):
            vinc, ln1, ln2, k0 = self.consts[f]
            Ff, s11, D = objective(eo, vinc, ln1, ln2, k0, DX, DY, DZ)
            F += Ff
            perf += [s11.real, s11.imag, D]
        return F, perf

    def step(self):
        """Evaluates draws until the first improving flip (accepted) or the
        end of the hat / evaluation cap. Returns True if a flip was accepted."""
        log = self.log
        while not self.done:
            if self.max_evals and log.evals >= self.max_evals:
                self.done = True
                break
            c = next_candidate(self.geo, self.hat, self.sym, self.last)
            if c is None:
                log.converged = self.done = True
                break
            idx, tiles, self.last = c
            s, d = self.geo.flip_set(self.tm, self.P, tiles)
            news = [st.eval(s, d) for st in self.states]
            F, perf = self.score(news)
            acc = F < self.F_best
            log.rows.append((log.evals, idx, int(acc), F, self.F_best, perf))
            log.evals += 1
            if acc:
                self.F_best = F
                for st, ne in zip(self.states, news):
                    if self.algebra in ("ref", "port"):
                        st.accept(ne)
                    else:
                        st.accept()
                for t in tiles:
                    self.tm[t] ^= 1
                self.P = self.geo.compute_P(self.tm)
                self.hat.reset()
                log.accepts += 1
                return True
        return False


def run_dbs(Gs, gobj_rows, freqs, tiles_x, tiles_y, seed, sym=True, random_init=True,
            max_evals=0, algebra="ref", run_index=0):
    """Runs DBS to convergence (or the evaluation cap) and returns the log."""
    r = DbsRunner(Gs, gobj_rows, freqs, tiles_x, tiles_y, seed, sym, random_init, max_evals, algebra, run_index)
    while not r.done:
        r.step()
    r.log.final_map = list(r.tm)
    return r.log


def parse_ref_log(path):
    """Reads a log written by oracle/ref_driver.cpp."""
    rows, init_map, final_map, start = [], None, None, None
    end = {}
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if not t or t[0] == "#":
                continue
            if t[0] == "init_map":
                init_map = [1 if ch == "x" else 0 for ch in t[1]]
            elif t[0] == "final_map":
                final_map = [1 if ch == "x" else 0 for ch in t[1]]
            elif t[0] == "start":
                start = (float(t[1]), [float(v) for v in t[2:]])
            elif t[0] == "eval":
                rows.append((int(t[1]), int(t[2]), int(t[3]), float(t[4]), float(t[5]),
                             [float(v) for v in t[6:]]))
            elif t[0] == "end":
                it = iter(t[1:])
                end = {k: float(v) for k, v in zip(it, it)}
    return dict(rows=rows, init_map=init_map, final_map=final_map, start=start, end=end)
