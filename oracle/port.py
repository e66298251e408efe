"""ctypes binding of the C restatement (pngf_port.c) -- test infrastructure only.

``PortState`` has the interface of ``refalg.RefState`` (eval / accept) so
``oracle.dbs.run_dbs(..., algebra="port")`` runs the reference algorithm at
full sizes. LAPACK/BLAS come from scipy's bundled OpenBLAS through the
function pointers scipy.linalg.cython_lapack / cython_blas export.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpngf_port.so")
_lib = None


def _capsule_ptr(capsule):
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype = C.c_char_p
    get_name.argtypes = [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = C.c_void_p
    get_ptr.argtypes = [C.py_object, C.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    L = C.CDLL(LIB)
    P, I, L_ = C.c_void_p, C.c_int, C.c_long
    L.port_set_lapack.argtypes = [P, P, P, P]
    L.port_create.restype = P
    L.port_create.argtypes = [L_, I, I, P, P, P, P]
    L.port_destroy.argtypes = [P]
    L.port_eval.argtypes = [P, P, P, I, P]
    L.port_accept.argtypes = [P]
    L.port_eobj.argtypes = [P, P]
    L.port_threads.restype = I
    import scipy.linalg.cython_blas as cb
    import scipy.linalg.cython_lapack as cl
    L.port_set_lapack(_capsule_ptr(cl.__pyx_capi__["zgetrf"]), _capsule_ptr(cl.__pyx_capi__["zgetri"]),
                      _capsule_ptr(cl.__pyx_capi__["zgetrs"]), _capsule_ptr(cb.__pyx_capi__["zgemm"]))
    _lib = L
    return L


def threads() -> int:
    return load().port_threads()


class PortState:
    def __init__(self, G, Gobj, Einc, P, kmax=96):
        L = load()
        self.L = L
        self.E = Gobj.shape[0]
        G = np.asfortranarray(G, dtype=np.complex128)
        Gobj = np.asfortranarray(Gobj, dtype=np.complex128)
        Einc = np.ascontiguousarray(Einc, dtype=np.complex128)
        P = np.ascontiguousarray(P, dtype=np.int8)
        self.kmax = kmax
        self.p = L.port_create(G.shape[0], self.E, kmax, G.ctypes.data, Gobj.ctypes.data, Einc.ctypes.data,
                               P.ctypes.data)
        if not self.p:
            raise RuntimeError("port_create failed (LU of C)")

    @property
    def Eobj(self):
        e = np.zeros(self.E, dtype=np.complex128)
        self.L.port_eobj(self.p, e.ctypes.data)
        return e

    def eval(self, s, d):
        s = np.ascontiguousarray(s, dtype=np.int32)
        d = np.ascontiguousarray(d, dtype=np.int32)
        out = np.zeros(self.E, dtype=np.complex128)
        self.L.port_eval(self.p, s.ctypes.data, d.ctypes.data, len(s), out.ctypes.data)
        return out

    def accept(self, new_eobj=None):
        self.L.port_accept(self.p)

    def __del__(self):
        if getattr(self, "p", None):
            self.L.port_destroy(self.p)
            self.p = None
