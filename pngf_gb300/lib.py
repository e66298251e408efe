"""ctypes binding of libpngf_gb300.so (the C ABI in include/pngf_gb300.h).

The library is loaded from this package directory. There is no fallback: if
the shared object is missing, or no sm_103a device is present when a handle
is created, these calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PNGF_BOUNDS_CHECK=1 selects the bounds-checked build (libpngf_gb300_bc.so)
LIB_PATH = os.path.join(HERE, "libpngf_gb300_bc.so" if os.environ.get("PNGF_BOUNDS_CHECK") == "1"
                        else "libpngf_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "pngf_gb300.h")

PNGF_OK = 0
ERRORS = {1: "PNGF_ERR_ARG", 2: "PNGF_ERR_CUDA", 3: "PNGF_ERR_NOMEM", 4: "PNGF_ERR_IO", 5: "PNGF_ERR_SINGULAR",
          6: "PNGF_ERR_STATE", 7: "PNGF_ERR_TIMEOUT", 8: "PNGF_ERR_UNSUPPORTED", 9: "PNGF_ERR_NO_DEVICE",
          10: "PNGF_ERR_SCRATCH"}
PREC_FP64, PREC_C64 = 0, 1
F64_TENSOR, F64_SIMT = 0, 1
DBS_SYMMETRIC, DBS_SINGLE = 0, 1
PROP_BEST, PROP_FIRST = 0, 1
INIT_EMPTY, INIT_RANDOM = 0, 1
MAX_FREQ = 16
TUNE_MAX = 8
BUILD_FP64, BUILD_C64 = 0, 1


class PngfError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Config(C.Structure):
    _fields_ = [("tiles_x", C.c_int), ("tiles_y", C.c_int), ("cells_x", C.c_int), ("cells_y", C.c_int),
                ("num_eobj", C.c_int), ("max_flips", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
                ("dz", C.c_double), ("num_freq", C.c_int), ("freq_hz", C.c_double * MAX_FREQ),
                ("precision", C.c_int), ("defer_rank", C.c_int), ("device", C.c_int), ("fp64_update", C.c_int),
                ("c64_build", C.c_int), ("state_only", C.c_int)]


class DbsParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("init", C.c_int), ("seed", C.c_int), ("run_index", C.c_int),
                ("max_evals", C.c_long), ("batch", C.c_int), ("drift_every", C.c_int), ("drift_tol", C.c_double)]


class DbsStats(C.Structure):
    _fields_ = [("evals", C.c_long), ("accepts", C.c_long), ("launched", C.c_long), ("converged", C.c_int),
                ("F_init", C.c_double), ("F_best", C.c_double), ("drift_checks", C.c_long),
                ("refreshes", C.c_long), ("drift_max", C.c_double), ("prop_hits", C.c_long),
                ("full_passes", C.c_long), ("device_launches", C.c_long), ("device_decisions", C.c_long)]


class Timing(C.Structure):
    _fields_ = [("eval_ms", C.c_double), ("eval_launches", C.c_long), ("eval_cf", C.c_double),
                ("eval_bytes", C.c_double), ("eval_flop", C.c_double), ("accept_ms", C.c_double),
                ("accepts", C.c_long), ("update_ms", C.c_double), ("update_launches", C.c_long),
                ("update_flop", C.c_double), ("update_bytes", C.c_double), ("kernel_launches", C.c_long),
                ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tune(C.Structure):
    _fields_ = [("eval_form", C.c_int), ("eval_forms", C.c_int), ("warps_per_cand", C.c_int * TUNE_MAX),
                ("cands_per_cta", C.c_int * TUNE_MAX), ("eval_us", C.c_double * TUNE_MAX), ("batch", C.c_int),
                ("update_form", C.c_int), ("update_forms", C.c_int), ("update_cols", C.c_int * TUNE_MAX),
                ("update_us", C.c_double * TUNE_MAX), ("eval_form_small", C.c_int), ("batch_small", C.c_int),
                ("eval_us_small", C.c_double * TUNE_MAX)]

    def as_dict(self):
        ne, nu = self.eval_forms, self.update_forms
        return {"eval_form": self.eval_form, "batch": self.batch,
                "eval": [{"warps_per_cand": self.warps_per_cand[i], "cands_per_cta": self.cands_per_cta[i],
                          "us": self.eval_us[i]} for i in range(ne)],
                "eval_form_small": self.eval_form_small, "batch_small": self.batch_small,
                "eval_small": [{"us": self.eval_us_small[i]} for i in range(ne)],
                "update_form": self.update_form,
                "update": [{"cols": self.update_cols[i], "us": self.update_us[i]} for i in range(nu)]}


_lib = None


def load():
    """Loads the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libpngf_gb300.so not built (run __graft_entry__.build() or python -m pngf_gb300.build)")
    L = C.CDLL(LIB_PATH)
    P, I, D, L_, V = C.c_void_p, C.c_int, C.c_double, C.c_long, None
    sig = {
        "pngf_config_default": (V, [P, I, I, I, P]),
        "pngf_num_edges": (L_, [I, I, I, I]),
        "pngf_synth_G": (I, [I, I, I, I, D, D, D, D, D, C.c_ulonglong, P, L_]),
        "pngf_synth_gobj": (I, [I, I, I, I, D, D, D, C.c_ulonglong, P]),
        "pngf_write_G_file": (I, [C.c_char_p, L_, I, P, L_, P]),
        "pngf_read_G_file": (I, [C.c_char_p, L_, I, P, L_, P]),
        "pngf_create": (I, [P, P]),
        "pngf_destroy": (I, [P]),
        "pngf_set_stream": (I, [P, P]),
        "pngf_last_error": (C.c_char_p, [P]),
        "pngf_dims": (I, [P, P, P]),
        "pngf_load_G": (I, [P, I, P, L_, P]),
        "pngf_load_G_file": (I, [P, I, C.c_char_p]),
        "pngf_load_G_synth": (I, [P, I, C.c_ulonglong, D]),
        "pngf_set_tile_map": (I, [P, P]),
        "pngf_get_tile_map": (I, [P, P]),
        "pngf_set_source_port": (I, [P, I, I, I, I]),
        "pngf_prepare": (I, [P]),
        "pngf_get_eobj": (I, [P, I, P, P]),
        "pngf_objective": (I, [P, P]),
        "pngf_get_M": (I, [P, I, P, L_, P]),
        "pngf_eval_candidates": (I, [P, P, P, I, P, P]),
        "pngf_eval_candidates_device": (I, [P, P, P, I, P, P, D, P]),
        "pngf_accept": (I, [P, I]),
        "pngf_drift_check": (I, [P, I, P]),
        "pngf_drift_check_freq": (I, [P, I, I, P]),
        "pngf_autotune": (I, [P, P]),
        "pngf_bounds_check_report": (I, [P, P, I]),
        "pngf_set_eval_form": (I, [P, I]),
        "pngf_accept_edges_noalloc": (I, [P, L_, L_, I, P, P, P, I, P, P]),
        "pngf_refresh": (I, [P]),
        "pngf_timing_enable": (I, [P, I]),
        "pngf_timing_get": (I, [P, P]),
        "pngf_dbs_begin": (I, [P, P, P]),
        "pngf_dbs_step": (I, [P, P]),
        "pngf_dbs_set_device_loop": (I, [P, I]),
        "pngf_inject_update_timeout": (I, [P, I]),
        "pngf_dbs_stats_get": (I, [P, P]),
        "pngf_dbs_log": (I, [P, L_, P, P, P, P, P, P]),
        "pngf_dbs_save_log": (I, [P, C.c_char_p]),
        "pngf_dbs_end": (I, [P]),
        "pngf_group_create": (I, [P, I, I, P]),
        "pngf_group_step": (I, [P, P]),
        "pngf_group_stats_get": (I, [P, P]),
        "pngf_group_destroy": (I, [P]),
        "pngf_prop_create": (I, [P, I, C.c_ulonglong, P]),
        "pngf_prop_destroy": (I, [P]),
        "pngf_prop_num_params": (L_, [P]),
        "pngf_prop_get_params": (I, [P, P]),
        "pngf_prop_set_params": (I, [P, P]),
        "pngf_prop_features": (I, [P, P]),
        "pngf_prop_record": (I, [P, P, P, I]),
        "pngf_prop_num_samples": (L_, [P]),
        "pngf_prop_train": (I, [P, I, I, C.c_float, P]),
        "pngf_prop_predict": (I, [P, P]),
        "pngf_prop_forward_backward": (I, [P, P, I, P, P, P, P, P]),
        "pngf_prop_last_error": (C.c_char_p, [P]),
        "pngf_dbs_set_proposal": (I, [P, P, I, I, I, I, C.c_float]),
        "pngf_dbs_set_proposal_rule": (I, [P, I]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def header_symbols(path: str = HEADER):
    """Function names declared in the public header."""
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    return sorted(set(re.findall(r"\b(pngf_[A-Za-z0-9_]+)\s*\(", src)))


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def num_edges(tiles_x, tiles_y, cells_x=3, cells_y=3):
    return load().pngf_num_edges(tiles_x, tiles_y, cells_x, cells_y)


def synth_G(tiles_x, tiles_y, freq_hz, seed=1, eps_r=2.25, cells=3, dx=0.01 / 60, dy=0.01 / 60, dz=0.01 / 180):
    """Synthetic complex-symmetric G (N x N, complex128, column-major)."""
    n = num_edges(tiles_x, tiles_y, cells, cells)
    G = np.empty((n, n), dtype=np.complex128, order="F")
    rc = load().pngf_synth_G(tiles_x, tiles_y, cells, cells, dx, dy, dz, freq_hz, eps_r, seed, _ptr(G), n)
    if rc:
        raise PngfError(rc, "pngf_synth_G")
    return G


def synth_gobj(tiles_x, tiles_y, seed=1, cells=3, dx=0.01 / 60, dy=0.01 / 60, dz=0.01 / 180):
    """The synthetic G's two NF2FF rows (2 x N complex128, row-major)."""
    n = num_edges(tiles_x, tiles_y, cells, cells)
    rows = np.empty((2, n), dtype=np.complex128)
    rc = load().pngf_synth_gobj(tiles_x, tiles_y, cells, cells, dx, dy, dz, seed, _ptr(rows))
    if rc:
        raise PngfError(rc, "pngf_synth_gobj")
    return rows


def write_G_file(path, G, gobj_rows=None, num_eobj=3):
    G = np.asfortranarray(G, dtype=np.complex128)
    go = None if gobj_rows is None else np.ascontiguousarray(gobj_rows, dtype=np.complex128)
    rc = load().pngf_write_G_file(path.encode(), G.shape[0], num_eobj, _ptr(G), G.shape[0], _ptr(go))
    if rc:
        raise PngfError(rc, "pngf_write_G_file " + path)


class Handle:
    """Owns one pngf_handle (all frequencies of one DBS instance)."""

    def __init__(self, tiles_x, tiles_y, freqs, precision=PREC_FP64, max_flips=4, num_eobj=3, defer_rank=0,
                 device=0, fp64_update=0, c64_build=0, state_only=0):
        L = load()
        self.L = L
        cfg = Config()
        fa = (C.c_double * MAX_FREQ)(*freqs)
        L.pngf_config_default(C.byref(cfg), tiles_x, tiles_y, len(freqs), fa)
        cfg.max_flips = max_flips
        cfg.num_eobj = num_eobj
        cfg.precision = precision
        cfg.defer_rank = defer_rank
        cfg.device = device
        cfg.fp64_update = fp64_update
        cfg.c64_build = c64_build
        cfg.state_only = state_only
        self.cfg = cfg
        self.nf = len(freqs)
        self.E = num_eobj
        self.max_flips = max_flips
        self.map_sz = tiles_x * tiles_y
        h = C.c_void_p()
        rc = L.pngf_create(C.byref(cfg), C.byref(h))
        if rc:
            raise PngfError(rc, "pngf_create")
        self.h = h
        n, ld = C.c_long(), C.c_long()
        L.pngf_dims(h, C.byref(n), C.byref(ld))
        self.n, self.ldm = n.value, ld.value

    def _chk(self, rc, what):
        if rc:
            raise PngfError(rc, "%s: %s" % (what, self.L.pngf_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.L.pngf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def timing_enable(self, on=True):
        self._chk(self.L.pngf_timing_enable(self.h, 1 if on else 0), "pngf_timing_enable")

    def timing(self):
        t = Timing()
        self._chk(self.L.pngf_timing_get(self.h, C.byref(t)), "pngf_timing_get")
        return t.as_dict()

    def set_stream(self, stream_ptr):
        self._chk(self.L.pngf_set_stream(self.h, C.c_void_p(stream_ptr)), "pngf_set_stream")

    def load_G(self, f, G, gobj_rows=None):
        G = np.asfortranarray(G, dtype=np.complex128)
        go = None if gobj_rows is None else np.ascontiguousarray(gobj_rows, dtype=np.complex128)
        self._chk(self.L.pngf_load_G(self.h, f, _ptr(G), G.shape[0], _ptr(go)), "pngf_load_G")

    def load_G_synth(self, f, seed=1, eps_r=2.25):
        """Frequency f's G from the built-in synthetic generator, on the device."""
        self._chk(self.L.pngf_load_G_synth(self.h, f, seed, eps_r), "pngf_load_G_synth")

    def load_G_file(self, f, path):
        self._chk(self.L.pngf_load_G_file(self.h, f, path.encode()), "pngf_load_G_file")

    def set_tile_map(self, tm):
        a = np.ascontiguousarray(tm, dtype=np.int32)
        self._chk(self.L.pngf_set_tile_map(self.h, _ptr(a)), "pngf_set_tile_map")

    def tile_map(self):
        a = np.zeros(self.map_sz, dtype=np.int32)
        self._chk(self.L.pngf_get_tile_map(self.h, _ptr(a)), "pngf_get_tile_map")
        return a

    def set_source_port(self, tx, ty, yoff=1, ysz=2):
        self._chk(self.L.pngf_set_source_port(self.h, tx, ty, yoff, ysz), "pngf_set_source_port")

    def prepare(self):
        self._chk(self.L.pngf_prepare(self.h), "pngf_prepare")

    def eobj(self, f):
        e = np.zeros(self.E, dtype=np.complex128)
        v = np.zeros(3, dtype=np.complex128)
        self._chk(self.L.pngf_get_eobj(self.h, f, _ptr(e), _ptr(v)), "pngf_get_eobj")
        return e, v

    def get_M(self, f):
        """(M, Einc) of frequency f: M is (N+E) x (N+1) complex128."""
        M = np.zeros((self.n + self.E, self.n + 1), dtype=np.complex128)
        e = np.zeros(self.n, dtype=np.complex128)
        self._chk(self.L.pngf_get_M(self.h, f, _ptr(M), self.n + 1, _ptr(e)), "pngf_get_M")
        return M, e

    def objective(self):
        F = np.zeros(1)
        self._chk(self.L.pngf_objective(self.h, _ptr(F)), "pngf_objective")
        return float(F[0])

    def pack(self, cands):
        t = np.zeros((len(cands), self.max_flips), dtype=np.int32)
        nfl = np.zeros(len(cands), dtype=np.int32)
        for i, c in enumerate(cands):
            t[i, :len(c)] = c
            nfl[i] = len(c)
        return t, nfl

    def eval_candidates(self, cands):
        t, nfl = self.pack(cands)
        eo = np.zeros((len(cands), self.nf, self.E), dtype=np.complex128)
        F = np.zeros(len(cands))
        self._chk(self.L.pngf_eval_candidates(self.h, _ptr(t), _ptr(nfl), len(cands), _ptr(eo), _ptr(F)),
                  "pngf_eval_candidates")
        return eo, F

    def accept(self, c):
        self._chk(self.L.pngf_accept(self.h, c), "pngf_accept")

    def drift_check(self, nrows=4, f=None):
        r = C.c_double()
        if f is None:
            self._chk(self.L.pngf_drift_check(self.h, nrows, C.byref(r)), "pngf_drift_check")
        else:
            self._chk(self.L.pngf_drift_check_freq(self.h, f, nrows, C.byref(r)), "pngf_drift_check_freq")
        return r.value

    def refresh(self):
        """Rebuilds the state for the current design from G in FP64."""
        self._chk(self.L.pngf_refresh(self.h), "pngf_refresh")

    def autotune(self):
        """Times the kernel forms at the current design and keeps the fastest;
        returns the chosen forms and the measured times (microseconds)."""
        t = Tune()
        self._chk(self.L.pngf_autotune(self.h, C.byref(t)), "pngf_autotune")
        return t.as_dict()

    def set_eval_form(self, form):
        self._chk(self.L.pngf_set_eval_form(self.h, form), "pngf_set_eval_form")

    def inject_update_timeout(self, code=21):
        """Failure test hook: the tensor-core error flag as a timed-out update leaves it."""
        self._chk(self.L.pngf_inject_update_timeout(self.h, code), "pngf_inject_update_timeout")


class Dbs:
    """The native DBS driver over a prepared-able handle (G loaded)."""

    def __init__(self, handle: Handle, mode=DBS_SYMMETRIC, init=INIT_RANDOM, seed=1, max_evals=0, batch=0,
                 run_index=0, drift_every=0, drift_tol=0.0, device_loop=False):
        self.hd = handle
        self.max_evals = max_evals
        p = DbsParams(mode, init, seed, run_index, max_evals, batch, drift_every, drift_tol)
        d = C.c_void_p()
        handle._chk(handle.L.pngf_dbs_begin(handle.h, C.byref(p), C.byref(d)), "pngf_dbs_begin")
        self.d = d
        if device_loop:
            self.set_device_loop(True)

    def set_device_loop(self, enable=True):
        """Decisions without an accept run on the GPU (pngf_dbs_set_device_loop)."""
        self.hd._chk(self.hd.L.pngf_dbs_set_device_loop(self.d, 1 if enable else 0), "pngf_dbs_set_device_loop")

    def step(self):
        a = C.c_int()
        self.hd._chk(self.hd.L.pngf_dbs_step(self.d, C.byref(a)), "pngf_dbs_step")
        return bool(a.value)

    def stats(self):
        s = DbsStats()
        self.hd._chk(self.hd.L.pngf_dbs_stats_get(self.d, C.byref(s)), "pngf_dbs_stats_get")
        return s

    def run(self):
        """Steps until the hat runs out (or the evaluation cap is reached)."""
        while True:
            self.step()
            s = self.stats()
            if s.converged or (0 < self.max_evals <= s.evals):
                return s

    def log(self):
        L, nf = self.hd.L, self.hd.nf
        rows = C.c_long()
        L.pngf_dbs_log(self.d, 0, None, None, None, None, None, C.byref(rows))
        n = rows.value
        tile = np.zeros(n, dtype=np.int32)
        acc = np.zeros(n, dtype=np.int32)
        F = np.zeros(n)
        Fb = np.zeros(n)
        perf = np.zeros((n, 3 * nf))
        L.pngf_dbs_log(self.d, n, _ptr(tile), _ptr(acc), _ptr(F), _ptr(Fb), _ptr(perf), C.byref(rows))
        return dict(tile=tile, accept=acc, F=F, F_best=Fb, perf=perf)

    def save_log(self, path):
        self.hd._chk(self.hd.L.pngf_dbs_save_log(self.d, path.encode()), "pngf_dbs_save_log")

    def close(self):
        if getattr(self, "d", None):
            self.hd.L.pngf_dbs_end(self.d)
            self.d = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GroupStats(C.Structure):
    _fields_ = [("rounds", C.c_long), ("graph_launches", C.c_long), ("captures", C.c_long),
                ("kernel_launches", C.c_long), ("evals", C.c_long), ("accepts", C.c_long)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Group:
    """Independent DBS runs (each on its own handle) stepped together."""

    def __init__(self, runs, use_graphs=True):
        self.runs = list(runs)
        self.L = self.runs[0].hd.L
        arr = (C.c_void_p * len(self.runs))(*[r.d.value for r in self.runs])
        g = C.c_void_p()
        self.runs[0].hd._chk(self.L.pngf_group_create(arr, len(self.runs), int(bool(use_graphs)), C.byref(g)),
                             "pngf_group_create")
        self.g = g

    def step(self):
        """One round; returns the number of members still running."""
        a = C.c_int()
        self.runs[0].hd._chk(self.L.pngf_group_step(self.g, C.byref(a)), "pngf_group_step")
        return a.value

    def run(self, max_rounds=None):
        r = 0
        while self.step() > 0:
            r += 1
            if max_rounds is not None and r >= max_rounds:
                break
        return self.stats()

    def stats(self):
        s = GroupStats()
        self.runs[0].hd._chk(self.L.pngf_group_stats_get(self.g, C.byref(s)), "pngf_group_stats_get")
        return s.as_dict()

    def close(self):
        if getattr(self, "g", None):
            self.L.pngf_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Proposal:
    """The learned flip-proposal network attached to a handle."""

    def __init__(self, handle: Handle, channels=32, seed=1):
        self.hd = handle
        self.L = handle.L
        p = C.c_void_p()
        rc = self.L.pngf_prop_create(handle.h, channels, seed, C.byref(p))
        if rc:
            raise PngfError(rc, "pngf_prop_create")
        self.p = p
        self.H = handle.cfg.tiles_y
        self.W = handle.cfg.tiles_x

    def _chk(self, rc, what):
        if rc:
            raise PngfError(rc, "%s: %s" % (what, self.L.pngf_prop_last_error(self.p).decode()))

    def num_params(self):
        return self.L.pngf_prop_num_params(self.p)

    def params(self):
        w = np.zeros(self.num_params(), dtype=np.float32)
        self._chk(self.L.pngf_prop_get_params(self.p, _ptr(w)), "get_params")
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._chk(self.L.pngf_prop_set_params(self.p, _ptr(w)), "set_params")

    def features(self):
        f = np.zeros((3, self.H, self.W), dtype=np.float32)
        self._chk(self.L.pngf_prop_features(self.p, _ptr(f)), "features")
        return f

    def record(self, tiles, gains):
        t = np.ascontiguousarray(tiles, dtype=np.int32)
        g = np.ascontiguousarray(gains, dtype=np.float64)
        self._chk(self.L.pngf_prop_record(self.p, _ptr(t), _ptr(g), len(t)), "record")

    def num_samples(self):
        return self.L.pngf_prop_num_samples(self.p)

    def train(self, steps, batch=32, lr=1e-3):
        loss = C.c_float()
        self._chk(self.L.pngf_prop_train(self.p, steps, batch, lr, C.byref(loss)), "train")
        return loss.value

    def predict(self):
        out = np.zeros(self.H * self.W, dtype=np.float32)
        self._chk(self.L.pngf_prop_predict(self.p, _ptr(out)), "predict")
        return out

    def forward_backward(self, x, target=None, mask=None):
        x = np.ascontiguousarray(x, dtype=np.float32)
        B = x.shape[0]
        out = np.zeros((B, self.H, self.W), dtype=np.float32)
        grad = np.zeros(self.num_params(), dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        t = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        self._chk(self.L.pngf_prop_forward_backward(self.p, _ptr(x), B, _ptr(t), _ptr(m), _ptr(out), _ptr(grad),
                                                    _ptr(loss)), "forward_backward")
        return out, grad, float(loss[0])

    def close(self):
        if getattr(self, "p", None):
            self.L.pngf_prop_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dbs_set_proposal(dbs: Dbs, prop, topk=64, train_every=0, train_steps=0, train_batch=32, lr=1e-3, rule=PROP_BEST):
    dbs.hd._chk(dbs.hd.L.pngf_dbs_set_proposal(dbs.d, prop.p if prop else None, topk, train_every, train_steps,
                                              train_batch, lr), "pngf_dbs_set_proposal")
    dbs.hd._chk(dbs.hd.L.pngf_dbs_set_proposal_rule(dbs.d, rule), "pngf_dbs_set_proposal_rule")
