"""ctypes binding of the FP64 CPU oracle (oracle/p2de_oracle.cpp).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py as the checker and the timed CPU restatement. It takes the same
descriptors (p2de_param / p2de_mesh) as the GPU library. PARITY UNPINNED: the
reference ships no golden vectors for this path (see the header of p2de_oracle.cpp).
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, byref, c_double, c_int, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libp2de_oracle.so"

_LIB = None


def build(force: bool = False) -> Path:
    import fcntl

    src = HERE / "p2de_oracle.cpp"
    hdr = HERE.parent / "include" / "p2de.h"
    (HERE / "_build").mkdir(exist_ok=True)
    with open(HERE / "_build" / ".lock", "w") as lk:  # one builder at a time across processes
        fcntl.flock(lk, fcntl.LOCK_EX)
        stale = not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime)
        if force or stale:
            subprocess.run(["make", "-C", str(HERE), "-B" if force else "all"], check=True, capture_output=True)
        fcntl.flock(lk, fcntl.LOCK_UN)
    return LIB_PATH


def load(path=None):
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    import sys

    sys.path.insert(0, str(HERE.parent / "p2de.jl_gb300"))
    from p2de import abi  # struct definitions shared with the product ABI

    p = Path(path) if path else build()
    lib = ctypes.CDLL(str(p))
    sig = [
        ("oracle_create", [POINTER(abi.P2deParam), POINTER(abi.P2deMesh), c_int, POINTER(c_void_p)]),
        ("oracle_destroy", [c_void_p]),
        ("oracle_set_Uq", [c_void_p, POINTER(c_double)]),
        ("oracle_rhs", [c_void_p, c_double, c_double, c_int, POINTER(c_double)]),
        ("oracle_ssp33_step", [c_void_p, POINTER(c_double), POINTER(c_double)]),
        ("oracle_ssp33", [c_void_p, POINTER(c_double), POINTER(c_int64), POINTER(c_double)]),
        ("oracle_get_field", [c_void_p, c_int, c_int, POINTER(c_double)]),
        ("oracle_get_operator", [c_void_p, c_int, POINTER(c_double), POINTER(c_int64)]),
        ("oracle_nnz_counts", [c_void_p, POINTER(c_int64), POINTER(c_int64)]),
        ("oracle_fS", [c_double, POINTER(c_double), POINTER(c_double), POINTER(c_double)]),
        ("oracle_fluxes", [c_double, POINTER(c_double), POINTER(c_double)]),
    ]
    for name, args in sig:
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = c_int
    lib.oracle_logmean.argtypes = [c_double, c_double]
    lib.oracle_logmean.restype = c_double
    lib.oracle_num_threads.argtypes = []
    lib.oracle_num_threads.restype = c_int
    if path is None:
        _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(POINTER(c_double))


class Oracle:
    """One FP64 CPU solve built from a p2de Descriptor."""

    def __init__(self, desc, nthreads: int = 0):
        self.lib = load()
        self.desc = desc
        h = c_void_p()
        st = self.lib.oracle_create(byref(desc.param), byref(desc.mesh), nthreads, byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_create failed with status {st}")
        self.h = h
        self.N, self.K = desc.N, desc.K
        self.N1D = self.N + 1
        eqn = getattr(desc.param, "equation", 0)
        self.dim1 = eqn == 2  # CompressibleEulerIdealGas{Dim1}
        self.Nq = self.N1D if self.dim1 else self.N1D**2
        self.Nfp = 2 if self.dim1 else 4 * self.N1D

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def count(self, field: int) -> int:
        n, Nq, Nfp, K = self.N1D, self.Nq, self.Nfp, self.K
        eqn = getattr(self.desc.param, "equation", 0)
        c = {1: 1, 2: 3}.get(eqn, 4)  # KPP: one component; Dim1: (rho, rhou, E)
        d = 1 if self.dim1 else 2
        return {0: c * Nq * K, 1: c * Nq * K, 2: c * Nq * K, 3: c * Nq * K, 4: d * c * Nq * K, 5: d * c * Nq * K,
                6: d * c * Nfp * K, 7: d * c * Nfp * K, 8: (Nq + n) * d * K, 9: c * Nq * K, 10: K, 11: Nfp * K,
                12: (Nq + n) * d * K * c, 13: (Nq + n) * d * K * c}[field]

    def set_Uq(self, Uq):
        U = np.ascontiguousarray(Uq, dtype=np.float64).ravel()
        assert U.size == self.count(0)
        self.lib.oracle_set_Uq(self.h, _dp(U))

    def get_field(self, field: int, nstage: int = 1) -> np.ndarray:
        out = np.empty(self.count(field))
        st = self.lib.oracle_get_field(self.h, field, nstage, _dp(out))
        if st != 0:
            raise RuntimeError(f"oracle_get_field {field}: {st}")
        return out

    def rhs(self, t: float, dt: float, nstage: int) -> float:
        out = c_double()
        self.lib.oracle_rhs(self.h, t, dt, nstage, byref(out))
        return out.value

    def step(self, t: float) -> tuple[float, float]:
        tt, dt = c_double(t), c_double()
        self.lib.oracle_ssp33_step(self.h, byref(tt), byref(dt))
        return tt.value, dt.value

    def run(self) -> tuple[float, int, float]:
        t, n, dt = c_double(), c_int64(), c_double()
        self.lib.oracle_ssp33(self.h, byref(t), byref(n), byref(dt))
        return t.value, n.value, dt.value

    def operator(self, which: int) -> np.ndarray:
        n = c_int64()
        self.lib.oracle_get_operator(self.h, which, None, byref(n))
        out = np.empty(n.value)
        self.lib.oracle_get_operator(self.h, which, _dp(out), byref(n))
        return out

    def nnz_counts(self) -> tuple[int, int]:
        a, b = c_int64(), c_int64()
        self.lib.oracle_nnz_counts(self.h, byref(a), byref(b))
        return a.value, b.value


def fS(gamma: float, UL, UR) -> np.ndarray:
    lib = load()
    a = np.ascontiguousarray(UL, dtype=np.float64)
    b = np.ascontiguousarray(UR, dtype=np.float64)
    out = np.empty(8)
    lib.oracle_fS(gamma, _dp(a), _dp(b), _dp(out))
    return out


def fluxes(gamma: float, U) -> np.ndarray:
    lib = load()
    a = np.ascontiguousarray(U, dtype=np.float64)
    out = np.empty(8)
    lib.oracle_fluxes(gamma, _dp(a), _dp(out))
    return out


def logmean(aL: float, aR: float) -> float:
    return load().oracle_logmean(aL, aR)


def num_threads() -> int:
    return load().oracle_num_threads()
