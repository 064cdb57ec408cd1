"""Batches of independent solves and the continuous-batching server (libp2de_gpu.so).

Batch: solves of any mesh size and degree advanced together, one persistent launch per
RK stage. Server: a native worker thread admitting submitted solves by HBM budget,
stepping the batch and retiring solves at their final time.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int32, c_int64, c_size_t, c_void_p
from dataclasses import dataclass

import numpy as np

from . import abi
from .solver import Descriptor


def solve_bytes(desc: Descriptor) -> int:
    lib = abi.load_library()
    out = c_size_t()
    abi.check(lib, lib.p2de_batch_solve_bytes(byref(desc.param), desc.mesh.nI, desc.mesh.nS, byref(out)))
    return out.value


class Batch:
    def __init__(self, pool_bytes: int, max_solves: int = 64, precision: str = "fp64", device: int = 0):
        self.lib = abi.load_library()
        h = c_void_p()
        st = self.lib.p2de_batch_create(device, abi.PRECISIONS[precision], pool_bytes, max_solves, byref(h))
        abi.check(self.lib, st, None)
        self.h = h
        self.max_solves = max_solves
        self.members: dict[int, Descriptor] = {}

    def _check(self, st):
        if st != 0:
            buf = ctypes.create_string_buffer(512)
            self.lib.p2de_batch_last_error(self.h, buf, len(buf))
            raise abi.P2deError(st, buf.value.decode())

    def add(self, desc: Descriptor, U0: np.ndarray) -> int:
        U = np.ascontiguousarray(U0, dtype=np.float64)
        slot = c_int32()
        self._check(self.lib.p2de_batch_add(self.h, byref(desc.param), byref(desc.mesh), abi.dptr(U), byref(slot)))
        self.members[slot.value] = desc
        return slot.value

    def remove(self, slot: int) -> None:
        self._check(self.lib.p2de_batch_remove(self.h, slot))
        self.members.pop(slot, None)

    def step(self, nsteps: int) -> None:
        self._check(self.lib.p2de_batch_step(self.h, nsteps))

    def states(self) -> np.ndarray:
        out = np.zeros((self.max_solves, 4))
        self._check(self.lib.p2de_batch_states(self.h, abi.dptr(out)))
        return out

    def run_to_end(self, chunk: int = 50, max_steps: int = 10**7) -> int:
        steps = 0
        while steps < max_steps:
            st = self.states()
            live = [s for s in self.members if st[s, 2] == 0.0]
            if not live:
                return steps
            self.step(chunk)
            steps += chunk
        return steps

    def Uq(self, slot: int) -> np.ndarray:
        d = self.members[slot]
        out = np.empty(4 * d.Nq * d.K)
        self._check(self.lib.p2de_batch_get_Uq(self.h, slot, abi.dptr(out)))
        return out

    def memory(self) -> tuple[int, int]:
        u, c = c_size_t(), c_size_t()
        self._check(self.lib.p2de_batch_memory(self.h, byref(u), byref(c)))
        return u.value, c.value

    def launch_count(self) -> int:
        c = c_int64()
        self._check(self.lib.p2de_batch_launch_count(self.h, byref(c)))
        return c.value

    def elements_per_block(self, N: int) -> tuple[int, int]:
        e, m = c_int32(), c_int32()
        self._check(self.lib.p2de_batch_get_elements_per_block(self.h, N, byref(e), byref(m)))
        return e.value, m.value

    def set_elements_per_block(self, N: int, epb: int) -> None:
        self._check(self.lib.p2de_batch_set_elements_per_block(self.h, N, int(epb)))

    def layout(self, N: int) -> int:
        v = c_int32()
        self._check(self.lib.p2de_batch_get_layout(self.h, N, byref(v)))
        return v.value

    def set_layout(self, N: int, layout: int) -> None:
        self._check(self.lib.p2de_batch_set_layout(self.h, N, int(layout)))

    def autotune(self) -> dict[int, int]:
        """Fastest elements-per-block per degree present; {N: epb}."""
        out = (c_int32 * 5)()
        self._check(self.lib.p2de_batch_autotune(self.h, out))
        return {N: out[N - 1] for N in range(1, 6) if out[N - 1] > 0}

    def close(self):
        if getattr(self, "h", None):
            self.lib.p2de_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class RequestInfo:
    state: int
    latency_s: float
    t_final: float
    steps: int


class Server:
    QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, hbm_budget_bytes: int, max_active: int = 64, steps_per_tick: int = 8, precision: str = "fp64",
                 device: int = 0):
        self.lib = abi.load_library()
        h = c_void_p()
        st = self.lib.p2de_server_create(device, abi.PRECISIONS[precision], hbm_budget_bytes, max_active,
                                         steps_per_tick, byref(h))
        abi.check(self.lib, st, None)
        self.h = h
        self.sizes: dict[int, int] = {}

    def submit(self, desc: Descriptor, U0: np.ndarray) -> int:
        U = np.ascontiguousarray(U0, dtype=np.float64)
        rid = c_int64()
        abi.check(self.lib, self.lib.p2de_server_submit(self.h, byref(desc.param), byref(desc.mesh), abi.dptr(U), byref(rid)))
        self.sizes[rid.value] = U.size
        return rid.value

    def poll(self, rid: int) -> RequestInfo:
        s, lat, tf, n = c_int32(), c_double(), c_double(), c_int64()
        abi.check(self.lib, self.lib.p2de_server_poll(self.h, rid, byref(s), byref(lat), byref(tf), byref(n)))
        return RequestInfo(s.value, lat.value, tf.value, n.value)

    def wait(self, rid: int, timeout_s: float = 60.0) -> int:
        s = c_int32()
        abi.check(self.lib, self.lib.p2de_server_wait(self.h, rid, timeout_s, byref(s)))
        return s.value

    def result(self, rid: int) -> np.ndarray:
        out = np.empty(self.sizes.pop(rid))
        abi.check(self.lib, self.lib.p2de_server_result(self.h, rid, abi.dptr(out)))
        return out

    def stats(self) -> dict:
        out = np.zeros(8)
        abi.check(self.lib, self.lib.p2de_server_stats(self.h, abi.dptr(out)))
        keys = ["completed", "failed", "active", "queued", "pool_used", "pool_capacity", "ticks", "busy_s"]
        return dict(zip(keys, out.tolist()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.p2de_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
