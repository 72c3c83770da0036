"""ctypes binding of the host DMR oracle (oracle/dmr_oracle.cpp) -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product never does.  Parity status: unpinned (the reference
has no golden vectors and cannot run without a GPU); see dmr_oracle.cpp.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "dmr_oracle.cpp")):
        subprocess.check_call(["sh", os.path.join(_HERE, "build_oracle.sh")])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [I, I, I, P, P, P, I, I, I]
        L.oracle_destroy.argtypes = [P]
        L.oracle_set_threads.argtypes = [I]
        L.oracle_max_threads.restype = I
        L.oracle_solve.restype = D
        L.oracle_solve.argtypes = [P, I, P, P, D, I, P, P, P, P]
        L.oracle_cycle_log.restype = I
        L.oracle_cycle_log.argtypes = [P, P, I]
        L.oracle_cycle_ms.restype = I
        L.oracle_cycle_ms.argtypes = [P, P, I]
        L.oracle_cycle_info.restype = I
        L.oracle_cycle_info.argtypes = [P, P, P, I]
        L.oracle_get_Z.argtypes = [P, P]
        L.oracle_set_Z.argtypes = [P, P]
        L.oracle_ls.argtypes = [I, I, P, P, P]
        L.oracle_svd.argtypes = [I, I, P, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """Host DMR solver over a CSR operator, complex128 (precision='c128') or an
    emulation of the reference's complex64 arithmetic (precision='c64')."""

    def __init__(self, A, m: int, k: int, precision: str = "c128", compat_eye: bool = True,
                 fuse_deflation: bool = False, threads: int = 0):
        L = lib()
        if threads:
            L.oracle_set_threads(int(threads))
        self.n, self.m, self.k = A.n, m, k
        self._indptr = np.ascontiguousarray(A.indptr, dtype=np.int32)
        self._indices = np.ascontiguousarray(A.indices, dtype=np.int32)
        self._vals = np.ascontiguousarray(A.data, dtype=np.complex128)
        h = L.oracle_create(A.n, m, k, _ptr(self._indptr), _ptr(self._indices), _ptr(self._vals),
                            0 if precision == "c128" else 1, int(compat_eye), int(fuse_deflation))
        if not h:
            raise ValueError("oracle_create rejected the sizes")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_destroy(self._h)
            self._h = None

    def solve(self, b, x0=None, mode: int = 0, tol: float = 1e-10, mat_rank: int = 2000) -> dict:
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros(self.n, np.complex128) if x0 is None else np.array(x0, dtype=np.complex128)
        its, cycles, status = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        mv = ctypes.c_long()
        ret = lib().oracle_solve(self._h, int(mode), _ptr(b), _ptr(x), float(tol), int(mat_rank),
                                 ctypes.byref(its), ctypes.byref(cycles), ctypes.byref(status), ctypes.byref(mv))
        nlog = max(cycles.value, 1)
        log = np.zeros(nlog)
        got = lib().oracle_cycle_log(self._h, _ptr(log), log.size)
        restart = np.zeros(nlog, np.int32)
        broken = np.zeros(nlog, np.int32)
        lib().oracle_cycle_info(self._h, _ptr(restart), _ptr(broken), nlog)
        ms = np.zeros(nlog)
        lib().oracle_cycle_ms(self._h, _ptr(ms), nlog)
        c = min(got, cycles.value)
        return dict(x=x, ret=ret, its=its.value, cycles=cycles.value, status=status.value,
                    matvecs=mv.value, rho=log[:c], restart=restart[:c], breakdown=broken[:c], cycle_ms=ms[:c])

    def get_Z(self) -> np.ndarray:
        out = np.zeros((self.k, self.n), np.complex128)
        lib().oracle_get_Z(self._h, _ptr(out))
        return out

    def set_Z(self, Z) -> None:
        Z = np.ascontiguousarray(Z, dtype=np.complex128).reshape(self.k, self.n)
        lib().oracle_set_Z(self._h, _ptr(Z))


def ls(H: np.ndarray, g: np.ndarray) -> np.ndarray:
    H = np.asfortranarray(H, dtype=np.complex128)
    g = np.ascontiguousarray(g, dtype=np.complex128)
    y = np.zeros(H.shape[1], np.complex128)
    lib().oracle_ls(H.shape[0], H.shape[1], _ptr(H), _ptr(g), _ptr(y))
    return y


def svd(A: np.ndarray):
    """Returns (sigma descending, V) with A = U diag(sigma) V^H."""
    A = np.asfortranarray(A, dtype=np.complex128)
    s = np.zeros(A.shape[1])
    V = np.zeros((A.shape[1], A.shape[1]), np.complex128, order="F")
    lib().oracle_svd(A.shape[0], A.shape[1], _ptr(A), _ptr(s), _ptr(V))
    return s, V
