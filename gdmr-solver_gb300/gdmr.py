"""Python binding of libgDMR (GB300 build) over its C ABI (ctypes).

Mirrors the reference's plugin interface (gDMRC.h: initLS / imp*LS / exp*LS /
solveLS / linOptLS / impSVDMR / expSVDMR) with the same names and argument
meaning, plus the complex128 twins and the context API of gdmr_ext.h.  There
is no fallback: if the CUDA library is missing or no GPU is visible, calls
raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgDMR.so.1")

# Every C entry point declared in include/*.h, with its ctypes signature.
P, I, F, D, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_longlong
SIGNATURES = {
    # gDMR.h
    "initDMR": (None, [I, I, P, I, I, I, I, P]),
    "freeDMR": (None, []),
    "solverDMR": (F, [I, P, P, P, I, F, I, P]),
    "impSVDMR": (None, [P]),
    "expSVDMR": (None, [P]),
    # gDMRC.h
    "initLS": (None, [I, I, I, I, P, I, I, I]),
    "freeLS": (None, []),
    "impImgLS": (None, [P]), "expImgLS": (None, [P]),
    "impSrcLS": (None, [P]), "expSrcLS": (None, [P]),
    "impOptLS": (None, [P]), "expOptLS": (None, [P]),
    "solveLS": (F, [I, F, I, P]),
    "linOptLS": (None, []),
    # gdmr_ext.h
    "gdmrLastStatus": (I, []),
    "gdmrLastError": (ctypes.c_char_p, []),
    "gdmrVersion": (ctypes.c_char_p, []),
    "gdmrLastStats": (None, [P]),
    "gdmrLastHistory": (I, [P, I]),
    "gdmrWaitLimit": (D, [D]),
    "gdmrInjectAllocFailure": (None, [I]),
    "initDMR_z": (None, [I, I, P, I, I, I, I, P]),
    "freeDMR_z": (None, []),
    "solverDMR_z": (D, [I, P, P, P, I, D, I, P]),
    "impSVDMR_z": (None, [P]), "expSVDMR_z": (None, [P]),
    "impCsrLS": (I, [I, P, P, P]),
    "initLS_z": (None, [I, I, I, I, P, I, I, I]),
    "freeLS_z": (None, []),
    "impImgLS_z": (None, [P]), "expImgLS_z": (None, [P]),
    "impSrcLS_z": (None, [P]), "expSrcLS_z": (None, [P]),
    "impOptLS_z": (None, [P]),
    "impCsrLS_z": (I, [I, P, P, P]),
    "solveLS_z": (D, [I, D, I, P]),
    "linOptLS_z": (None, []),
    "gdmrKernelLaunches": (LL, []),
    "gdmrProfile": (None, [I]),
    "gdmrProfileReset": (None, []),
    "gdmrProfileRead": (I, [I, P, P, P]),
    "gdmrTune": (None, [I]),
    "gdmrTuneReport": (ctypes.c_char_p, []),
    "gdmrTuneForce": (None, [I, I]),
    "gdmrGridOperator": (None, [I]),
    "gdmrGridBatch": (None, [I]),
    "gdmrCombineGroup": (None, [I]),
    "gdmrOverlapResidual": (I, [I]),
    "gdmr_csr_grid_form": (I, [I, P, P, P, P]),
    "gdmrAsyncTimeouts": (ctypes.c_uint, []),
    "gdmr_hessenberg_svd": (I, [I, I, P, P, P, P]),
    "gdmr_shared_basis_check": (I, [I, I, I, P, P, P, P, P]),
    "gdmr_system_set_stencil": (I, [P, I, I, I, P]),
    "gdmr_system_clear_stencil": (I, [P]),
    "gdmr_system_create": (I, [P, I, P, P, P, I, I, I, I, I]),
    "gdmr_system_destroy": (I, [P]),
    "gdmr_system_bytes": (LL, [P]),
    "gdmr_system_svd_sweeps": (I, [P]),
    "gdmr_system_set_graphs": (I, [P, I]),
    "gdmr_system_set_fused": (I, [P, I]),
    "gdmr_system_grid": (I, [P, P]),
    "gdmr_system_set_compat_eye": (I, [P, I]),
    "gdmr_solve": (I, [P, I, P, P, D, I, I, P]),
    "gdmr_solve_batch": (I, [P, I, P, P, P, I, I, P]),
    "gdmr_true_residual": (I, [P, I, P, P, I, P]),
    "gdmr_multi_solve": (I, [I, P, P, P, P, P, I, P]),
    "gdmrMultiTail": (I, [I]),
    "gdmr_true_residual_noalloc": (I, [P, I, P, P, P, P]),
    "gdmr_export_deflation": (I, [P, P]),
    "gdmr_import_deflation": (I, [P, P]),
    "gdmr_drop_deflation": (I, [P]),
    "gdmr_deflation_write": (I, [ctypes.c_char_p, I, I, P]),
    "gdmr_deflation_read": (I, [ctypes.c_char_p, I, I, P]),
    "gdmr_save_deflation": (I, [P, ctypes.c_char_p]),
    "gdmr_load_deflation": (I, [P, ctypes.c_char_p]),
    "gdmr_server_create": (I, [P, LL, I]),
    "gdmr_server_create_multi": (I, [P, LL, P, I]),
    "gdmr_server_operator_device": (I, [P, I]),
    "gdmr_place_operator": (I, [I, P, P, LL, LL, I, P]),
    "gdmr_server_add_operator": (I, [P, I, P, P, P, I, I, I, I, P]),
    "gdmr_server_slot_bytes": (LL, [I, I, I]),
    "gdmr_server_operator_capacity": (I, [P, I]),
    "gdmr_server_bytes": (LL, [P]),
    "gdmr_server_start": (I, [P]),
    "gdmr_server_submit": (I, [P, I, P, P, D, I, P]),
    "gdmr_server_wait": (I, [P, LL, D, P]),
    "gdmr_server_poll": (I, [P, P, P, I]),
    "gdmr_server_destroy": (I, [P]),
}

STATUS = {0: "GDMR_OK", 1: "GDMR_EINVAL", 2: "GDMR_ENOMEM", 3: "GDMR_ENOCONV", 4: "GDMR_ERUNAWAY",
          5: "GDMR_ECUDA", 6: "GDMR_ENOTINIT", 7: "GDMR_EBREAKDOWN", 8: "GDMR_ETIMEOUT", 9: "GDMR_ENONFINITE"}


class Stats(ctypes.Structure):
    _fields_ = [("cycles", I), ("its", I), ("matvecs", LL), ("rel_res", D), ("true_rel_res", D),
                ("status", I), ("breakdowns", I), ("latency_ms", D)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Cycle(ctypes.Structure):
    _fields_ = [("rho", D), ("rel_res", D), ("kk", I), ("restart", I), ("breakdown", I), ("stagnated", I)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def last_history() -> list:
    """Per restart cycle of the last reference-semantics solve: rho, rel_res, kk, restart (0 or the
    [W V] storage index of the mid-Krylov restart vector), breakdown step, stagnated flag."""
    L = load()
    cnt = int(L.gdmrLastHistory(None, 0))
    buf = (Cycle * max(cnt, 1))()
    L.gdmrLastHistory(buf, cnt)
    return [buf[i].as_dict() for i in range(cnt)]


def wait_limit(ms: float = -1.0) -> float:
    """Bound (ms at 2.07 GHz) of the kernels' stage waits and grid barriers; sets it when ms >= 0
    and returns the previous value."""
    return float(load().gdmrWaitLimit(float(ms)))


def inject_alloc_failure(nth: int) -> None:
    """Failure-path testing: the nth engine allocation from now on fails (0 disarms)."""
    load().gdmrInjectAllocFailure(int(nth))


KERNEL_CLASSES = ["projection", "update", "operator", "combine", "deflation_update", "residual64",
                  "least_squares", "svd", "other"]


def kernel_launches() -> int:
    return int(load().gdmrKernelLaunches())


def profile(on: bool) -> None:
    load().gdmrProfile(1 if on else 0)


def profile_reset() -> None:
    load().gdmrProfileReset()


def tune_report() -> str:
    return load().gdmrTuneReport().decode()


def tune(on: bool) -> None:
    load().gdmrTune(1 if on else 0)


def async_timeouts() -> int:
    """Bounded mbarrier waits of the pipelined kernels that ran out since load (0 when healthy)."""
    return int(load().gdmrAsyncTimeouts())


def tune_force(projection: int = -1, update: int = -1) -> None:
    """Pins the Gram-Schmidt variants (index as in tune_report; -1 hands back to the tuner)."""
    load().gdmrTuneForce(int(projection), int(update))


def grid_operator(enable: bool) -> None:
    """Structured-grid operator kernel for matrices with a grid form (on by default); off sends
    the products launched afterwards to the SELL-32 kernels."""
    load().gdmrGridOperator(1 if enable else 0)


def grid_batch(systems_per_thread: int) -> None:
    """Batched operator products on the grid kernel with 1, 2 or 4 systems a thread; 0 (the
    default) keeps them on the SELL-32 kernel."""
    load().gdmrGridBatch(int(systems_per_thread))


def combine_group(enable: bool) -> None:
    """Cycle-end combinations of batches four systems a CTA (on by default) or one."""
    load().gdmrCombineGroup(1 if enable else 0)


def overlap_residual(ctas_per_sm: int = -1) -> int:
    """gdmrOverlapResidual: the refined solves' FP64 residual beside the next cycle's deflation
    loop, on its own stream with its grid capped at about ctas_per_sm CTAs an SM, or before the
    loop (0, the default); -1 only reads.  Returns the previous setting."""
    return int(load().gdmrOverlapResidual(int(ctas_per_sm)))


def csr_grid_form(A):
    """(nx, ny, nz) if the CSR matrix A (n, indptr, indices, data) has the structured-grid form
    of the grid operator kernel, else None.  Host-only."""
    indptr = np.ascontiguousarray(A.indptr, dtype=np.int32)
    indices = np.ascontiguousarray(A.indices, dtype=np.int32)
    vals = np.ascontiguousarray(np.asarray(A.data, dtype=np.complex128).view(np.float64))
    dims = np.zeros(3, dtype=np.int32)
    _check(load().gdmr_csr_grid_form(int(A.n), _ptr(indptr), _ptr(indices), _ptr(vals), _ptr(dims)),
           "gdmr_csr_grid_form")
    return tuple(int(d) for d in dims) if dims[0] > 0 else None


def hessenberg_svd(H: np.ndarray, k: int, with_sweeps: bool = False):
    """The deflation update's SVD of a (m+1) x m complex Hessenberg (gdmr_hessenberg_svd):
    the m singular values in descending order and, as the columns of an m x k array, the right
    singular vectors of the k smallest (column t belongs to the (m-k+t)-th largest value);
    with_sweeps adds (FP32 sweeps, double-float sweeps)."""
    H = np.asarray(H, dtype=np.complex128)
    rows, m = H.shape
    if rows != m + 1:
        raise ValueError("H must be (m+1) x m")
    Hc = np.ascontiguousarray(H.T)                   # column-major: column j contiguous
    sigma = np.empty(m, dtype=np.float64)
    vs = np.empty((k, m), dtype=np.complex128)
    sw = ctypes.c_int(0)
    _check(load().gdmr_hessenberg_svd(int(m), int(k), _ptr(Hc), _ptr(sigma), _ptr(vs), ctypes.byref(sw)),
           "gdmr_hessenberg_svd")
    if with_sweeps:
        return sigma, vs.T.copy(), (sw.value // 1000, sw.value % 1000)
    return sigma, vs.T.copy()


def shared_basis_check(W, Y, c):
    """The batched shared-basis tensor-core kernels on their own (gdmr_shared_basis_check):
    W (k, n) and Y (nsys, n) complex64, c (nsys, k) complex128.  Returns (coef, P): coef (nsys, k)
    complex128 with coef[s, p] = <W_p, Y_s>, and P (nsys, n) complex64 with P[s] = sum_p c[s, p] W_p."""
    W = np.ascontiguousarray(W, dtype=np.complex64)
    Y = np.ascontiguousarray(Y, dtype=np.complex64)
    c = np.ascontiguousarray(c, dtype=np.complex128)
    k, n = W.shape
    nsys = Y.shape[0]
    coef = np.empty((nsys, k), np.complex128)
    P = np.empty((nsys, n), np.complex64)
    _check(load().gdmr_shared_basis_check(n, k, nsys, _ptr(W), _ptr(Y), _ptr(c), _ptr(coef), _ptr(P)),
           "gdmr_shared_basis_check")
    return coef, P


def profile_read() -> dict:
    """Per kernel class: algorithmic bytes, CUDA-event milliseconds, launches."""
    out = {}
    for i, name in enumerate(KERNEL_CLASSES):
        b, ms, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        load().gdmrProfileRead(i, ctypes.byref(b), ctypes.byref(ms), ctypes.byref(n))
        out[name] = {"bytes": b.value, "ms": ms.value, "launches": n.value}
    return out


class GDMRError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Loads the library, building it first if it is missing (`build.py` rebuilds a stale one)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location("gdmr_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def place_operator(budget, used, fixed_bytes: int, per_slot_bytes: int, capacity: int = 0):
    """Host-only placement rule of the server (gdmr_place_operator): (device index or -1,
    capacity granted) for an operator on devices with the given budgets and used bytes."""
    b = np.ascontiguousarray(budget, dtype=np.int64)
    u = np.ascontiguousarray(used, dtype=np.int64)
    cap = ctypes.c_int(0)
    d = load().gdmr_place_operator(len(b), _ptr(b), _ptr(u), int(fixed_bytes), int(per_slot_bytes), int(capacity),
                                   ctypes.byref(cap))
    return int(d), int(cap.value)


def write_deflation(path: str, Z) -> None:
    """Host-only: write a k x n complex128 deflation space in the versioned on-disk format."""
    Z = np.ascontiguousarray(Z, dtype=np.complex128)
    _check(load().gdmr_deflation_write(os.fsencode(path), Z.shape[1], Z.shape[0], _ptr(Z)), "gdmr_deflation_write")


def read_deflation(path: str, k: int, n: int) -> np.ndarray:
    Z = np.zeros((k, n), np.complex128)
    _check(load().gdmr_deflation_read(os.fsencode(path), n, k, _ptr(Z)), "gdmr_deflation_read")
    return Z


def last_error() -> str:
    return load().gdmrLastError().decode()


def last_stats() -> dict:
    s = Stats()
    load().gdmrLastStats(ctypes.byref(s))
    return s.as_dict()


def _check(rc: int, what: str):
    if rc != 0:
        raise GDMRError(rc, f"{what}: {last_error()}")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _csr_arrays(A):
    indptr = np.ascontiguousarray(A.indptr, dtype=np.int32)
    indices = np.ascontiguousarray(A.indices, dtype=np.int32)
    return indptr, indices


class LinearSystem:
    """The reference's plugin (gDMRC.h) in complex64 ('c64', the reference's
    precision) or complex128 ('c128', the *_z entry points).  One instance per
    precision may be live at a time: the plugin, like the reference's, is
    process-global."""

    def __init__(self, n: int, basis: int, deflat: int, precision: str = "c64", device: int = 0,
                 blocks: int = 32, threads: int = 512, devices=(0,)):
        self.L = load()
        self.n, self.m, self.k = n, basis, deflat
        self.z = precision == "c128"
        self.cdt = np.complex128 if self.z else np.complex64
        devs = (ctypes.c_int * len(devices))(*devices)
        init = self.L.initLS_z if self.z else self.L.initLS
        init(blocks, threads, device, n, devs, len(devices), basis, deflat)
        if self.L.gdmrLastStatus() != 0:
            raise GDMRError(self.L.gdmrLastStatus(), last_error())
        self._live = True

    def _fn(self, name):
        return getattr(self.L, name + ("_z" if self.z else ""))

    def imp_img(self, b):
        b = np.ascontiguousarray(b, dtype=self.cdt)
        self._fn("impImgLS")(_ptr(b))

    def exp_img(self):
        out = np.zeros(self.n, self.cdt)
        self._fn("expImgLS")(_ptr(out))
        return out

    def imp_src(self, x):
        x = np.ascontiguousarray(x, dtype=self.cdt)
        self._fn("impSrcLS")(_ptr(x))

    def exp_src(self):
        out = np.zeros(self.n, self.cdt)
        self._fn("expSrcLS")(_ptr(out))
        return out

    def imp_opt(self, dense):
        """Dense operator, (n, n) array; stored column-major as the reference does."""
        a = np.asfortranarray(dense, dtype=self.cdt)
        self._fn("impOptLS")(_ptr(a.reshape(-1, order="F")))

    def imp_csr(self, A):
        indptr, indices = _csr_arrays(A)
        vals = np.ascontiguousarray(A.data, dtype=self.cdt)
        _check(self._fn("impCsrLS")(int(A.nnz), _ptr(indptr), _ptr(indices), _ptr(vals)), "impCsrLS")

    def lin_opt(self):
        self._fn("linOptLS")()

    def solve(self, mode: int, tol: float, mat_rank: int):
        its = ctypes.c_int()
        r = self._fn("solveLS")(int(mode), float(tol), int(mat_rank), ctypes.byref(its))
        return float(r), its.value

    def imp_sv(self, Z):
        Z = np.ascontiguousarray(Z, dtype=self.cdt).reshape(-1)
        (self.L.impSVDMR_z if self.z else self.L.impSVDMR)(_ptr(Z))

    def exp_sv(self):
        out = np.zeros(self.k * self.n, self.cdt)
        (self.L.expSVDMR_z if self.z else self.L.expSVDMR)(_ptr(out))
        return out.reshape(self.k, self.n)

    def close(self):
        if self._live:
            self._fn("freeLS")()
            self._live = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class System:
    """Context API (gdmr_ext.h): a resident CSR operator plus a solver engine of
    `capacity` systems sharing one recycled deflation space.
    precision: 'fp64' (plain complex128 iteration), 'fp64e' (the same iteration in
    double-float arithmetic on the FP32 pipes, about 48 significant bits) or 'mixed'
    (complex64 inner iteration inside FP64 refinement)."""

    def __init__(self, A, basis: int, deflat: int, capacity: int = 1, precision: str = "fp64", device: int = 0):
        self.L = load()
        self.n, self.m, self.k, self.capacity = A.n, basis, deflat, capacity
        indptr, indices = _csr_arrays(A)
        vals = np.ascontiguousarray(A.data, dtype=np.complex128)
        h = ctypes.c_void_p()
        prec = {"fp64": 0, "mixed": 1, "fp64e": 2}[precision]
        _check(self.L.gdmr_system_create(ctypes.byref(h), A.n, _ptr(indptr), _ptr(indices), _ptr(vals),
                                         basis, deflat, capacity, prec, device), "gdmr_system_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.L.gdmr_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_graphs(self, on: bool) -> None:
        _check(self.L.gdmr_system_set_graphs(self._h, 1 if on else 0), "gdmr_system_set_graphs")

    def set_fused(self, on: bool) -> None:
        """One small system: run the Krylov loop as one cooperative kernel (default) or step by step."""
        _check(self.L.gdmr_system_set_fused(self._h, 1 if on else 0), "gdmr_system_set_fused")

    def set_compat_eye(self, on: bool) -> None:
        """The reference's breakdown identity tail (default) or the standard one (see gdmr_ext.h)."""
        _check(self.L.gdmr_system_set_compat_eye(self._h, 1 if on else 0), "gdmr_system_set_compat_eye")

    def grid_shape(self):
        """(nx, ny, nz) if the CSR operator has the structured-grid form, else None."""
        dims = np.zeros(3, dtype=np.int32)
        _check(self.L.gdmr_system_grid(self._h, _ptr(dims)), "gdmr_system_grid")
        return tuple(int(d) for d in dims) if dims[0] > 0 else None

    def set_stencil(self, shape, d, wx, wy, wz=0.0) -> None:
        """Matrix-free inner operator: the constant-coefficient stencil on a grid of `shape`
        (2 or 3 edge lengths, first fastest).  Checked in FP64 against the system's CSR
        operator; raises GDMRError if it does not reproduce it."""
        nx, ny = int(shape[0]), int(shape[1])
        nz = int(shape[2]) if len(shape) > 2 else 1
        coef = np.array([d, wx, wy, wz], dtype=np.complex128)
        _check(self.L.gdmr_system_set_stencil(self._h, nx, ny, nz, _ptr(coef)), "gdmr_system_set_stencil")

    def clear_stencil(self) -> None:
        _check(self.L.gdmr_system_clear_stencil(self._h), "gdmr_system_clear_stencil")

    def svd_sweeps(self) -> dict:
        v = int(self.L.gdmr_system_svd_sweeps(self._h))
        return {"fp32": v // 1000, "fp64": v % 1000}

    @property
    def device_bytes(self) -> int:
        return int(self.L.gdmr_system_bytes(self._h))

    def solve(self, b, x0=None, mode: int = 0, tol: float = 1e-10, mat_rank: int = 2000):
        """Reference-semantics solve of one right-hand side; returns (x, stats)."""
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros(self.n, np.complex128) if x0 is None else np.array(x0, dtype=np.complex128)
        st = Stats()
        rc = self.L.gdmr_solve(self._h, int(mode), _ptr(b), _ptr(x), float(tol), int(mat_rank), 0, ctypes.byref(st))
        if rc not in (0, 3, 4):
            _check(rc, "gdmr_solve")
        return x, st.as_dict()

    def solve_batch(self, B, X0=None, tol=1e-10, max_cycles: int = 5000):
        """FP64-refined batched solve; B is (nrhs, n).  Returns (X, [stats])."""
        B = np.ascontiguousarray(B, dtype=np.complex128)
        nrhs = B.shape[0]
        X = np.zeros_like(B) if X0 is None else np.array(X0, dtype=np.complex128)
        tols = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (nrhs,)))
        stats = (Stats * nrhs)()
        rc = self.L.gdmr_solve_batch(self._h, nrhs, _ptr(B), _ptr(X), _ptr(tols), int(max_cycles), 0, stats)
        if rc not in (0, 3, 4):
            _check(rc, "gdmr_solve_batch")
        return X, [s.as_dict() for s in stats]

    def solve_batch_device(self, b_ptr: int, x_ptr: int, nrhs: int, tol, max_cycles: int = 5000):
        """Same on device buffers (raw pointers to complex128 arrays of nrhs*n)."""
        tols = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (nrhs,)))
        stats = (Stats * nrhs)()
        rc = self.L.gdmr_solve_batch(self._h, nrhs, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), _ptr(tols),
                                     int(max_cycles), 1, stats)
        if rc not in (0, 3, 4):
            _check(rc, "gdmr_solve_batch")
        return [s.as_dict() for s in stats]

    def true_residual(self, B, X):
        B = np.ascontiguousarray(np.atleast_2d(B), dtype=np.complex128)
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.complex128)
        out = np.zeros(B.shape[0])
        _check(self.L.gdmr_true_residual(self._h, B.shape[0], _ptr(B), _ptr(X), 0, _ptr(out)), "gdmr_true_residual")
        return out

    def true_residual_noalloc(self, b_ptr: int, x_ptr: int, out_ptr: int, nrhs: int, stream: int = 0):
        """gdmr_true_residual_noalloc on caller-owned device buffers (raw pointers); enqueued on
        `stream` without synchronising; allocates nothing."""
        _check(self.L.gdmr_true_residual_noalloc(self._h, int(nrhs), ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr),
                                                 ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream)),
               "gdmr_true_residual_noalloc")

    def export_deflation(self):
        Z = np.zeros((self.k, self.n), np.complex128)
        _check(self.L.gdmr_export_deflation(self._h, _ptr(Z)), "gdmr_export_deflation")
        return Z

    def import_deflation(self, Z):
        Z = np.ascontiguousarray(Z, dtype=np.complex128)
        _check(self.L.gdmr_import_deflation(self._h, _ptr(Z)), "gdmr_import_deflation")

    def save_deflation(self, path: str) -> None:
        _check(self.L.gdmr_save_deflation(self._h, os.fsencode(path)), "gdmr_save_deflation")

    def load_deflation(self, path: str) -> None:
        _check(self.L.gdmr_load_deflation(self._h, os.fsencode(path)), "gdmr_load_deflation")

    def drop_deflation(self):
        _check(self.L.gdmr_drop_deflation(self._h), "gdmr_drop_deflation")


def multi_tail(systems: int = -1) -> int:
    """gdmrMultiTail: systems in flight at or below which multi_solve finishes on the systems'
    own batched cycles (default 48; 0: lockstep to the end); returns the previous value."""
    return int(load().gdmrMultiTail(int(systems)))


def multi_solve(systems, Bs, tol=1e-10, max_cycles: int = 5000):
    """gdmr_multi_solve: the refined batched solves of several systems at once, their restart
    cycles in lockstep and the Krylov loops of every right-hand side in flight in one launch a
    cycle.  systems: System objects of one precision; Bs[o]: (nrhs_o, n_o) right-hand sides;
    tol: one value or one per system.  Returns [(X_o, [stats])]."""
    L = load()
    nops = len(systems)
    Bs = [np.ascontiguousarray(np.atleast_2d(B), dtype=np.complex128) for B in Bs]
    Xs = [np.zeros_like(B) for B in Bs]
    tols = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (nops,)))
    stats = [(Stats * max(B.shape[0], 1))() for B in Bs]
    hs = (ctypes.c_void_p * nops)(*[s._h.value for s in systems])
    nr = (ctypes.c_int * nops)(*[B.shape[0] for B in Bs])
    bp = (ctypes.c_void_p * nops)(*[B.ctypes.data for B in Bs])
    xp = (ctypes.c_void_p * nops)(*[X.ctypes.data for X in Xs])
    sp_ = (ctypes.c_void_p * nops)(*[ctypes.addressof(st) for st in stats])
    rc = L.gdmr_multi_solve(nops, hs, nr, bp, xp, _ptr(tols), int(max_cycles), sp_)
    if rc not in (0, 3, 4):
        _check(rc, "gdmr_multi_solve")
    return [(Xs[o], [stats[o][i].as_dict() for i in range(Bs[o].shape[0])]) for o in range(nops)]


class Server:
    """Serving layer (gdmr_server_*): resident operators with their deflation spaces,
    continuous batching of requests, admission bounded by a device-memory budget."""

    def __init__(self, budget_bytes: int, device: int = 0, devices=None):
        """budget_bytes per device; devices: a list of CUDA ordinals (operators are placed across
        them by budget; an ordinal may repeat), default [device]."""
        self.L = load()
        h = ctypes.c_void_p()
        devs = list(devices) if devices is not None else [int(device)]
        arr = (ctypes.c_int * len(devs))(*devs)
        _check(self.L.gdmr_server_create_multi(ctypes.byref(h), int(budget_bytes), arr, len(devs)),
               "gdmr_server_create_multi")
        self._h = h
        self.devices = devs
        self._keep = {}          # ticket -> (b, x) buffers that must outlive the request
        self.n = {}

    def add_operator(self, A, basis: int, deflat: int, capacity: int = 0, precision: str = "mixed") -> int:
        indptr, indices = _csr_arrays(A)
        vals = np.ascontiguousarray(A.data, dtype=np.complex128)
        op = ctypes.c_int()
        _check(self.L.gdmr_server_add_operator(self._h, A.n, _ptr(indptr), _ptr(indices), _ptr(vals), basis, deflat,
                                               capacity, {"fp64": 0, "mixed": 1}[precision], ctypes.byref(op)),
               "gdmr_server_add_operator")
        self.n[op.value] = A.n
        return op.value

    def capacity(self, op: int) -> int:
        return int(self.L.gdmr_server_operator_capacity(self._h, op))

    def device_of(self, op: int) -> int:
        """Index into `devices` of the device the operator was placed on."""
        return int(self.L.gdmr_server_operator_device(self._h, op))

    @property
    def device_bytes(self) -> int:
        return int(self.L.gdmr_server_bytes(self._h))

    def start(self):
        _check(self.L.gdmr_server_start(self._h), "gdmr_server_start")

    def submit(self, op: int, b, tol: float = 1e-10, max_cycles: int = 5000) -> int:
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        t = ctypes.c_longlong()
        _check(self.L.gdmr_server_submit(self._h, op, _ptr(b), _ptr(x), float(tol), int(max_cycles),
                                         ctypes.byref(t)), "gdmr_server_submit")
        self._keep[t.value] = (b, x)
        return t.value

    def wait(self, ticket: int, timeout: float = 0.0):
        st = Stats()
        _check(self.L.gdmr_server_wait(self._h, int(ticket), float(timeout), ctypes.byref(st)), "gdmr_server_wait")
        b, x = self._keep.pop(ticket)
        return x, st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self.L.gdmr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
