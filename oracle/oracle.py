"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, by __graft_entry__.smoke() (as the checker) and by bench.py's
CPU-baseline leg.  The product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from ndspmhd_gb300.abi import (NdsphDt, NdsphParticles, alloc_state, copy_state,
                               make_opts, make_particles)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libndsph_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ndsph_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(type(make_opts.__annotations__) if False else C.c_char), C.c_int]
        L.orc_create.argtypes = None
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_message.restype = C.c_char_p
        L.orc_message.argtypes = [C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, C.POINTER(NdsphParticles)]
        L.orc_get_state.argtypes = [C.c_void_p, C.POINTER(NdsphParticles)]
        L.orc_get_dt.argtypes = [C.c_void_p, C.POINTER(NdsphDt)]
        L.orc_set_dt.argtypes = [C.c_void_p, C.c_double, C.c_double]
        for f in ("orc_derivs", "orc_iterate_density", "orc_get_rates", "orc_primitive2conservative"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_step.restype = C.c_int
        L.orc_polyk.restype = C.c_double
        L.orc_polyk.argtypes = [C.c_void_p]
        L.orc_kernel_tables.argtypes = [C.c_int, C.POINTER(C.c_double)]
        L.orc_interp.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.orc_neighbour_csr.restype = C.c_long
        L.orc_neighbour_csr.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_long), C.POINTER(C.c_int32),
                                        C.c_long]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


class Oracle:
    """One oracle simulation: reference-layout host arrays in ``self.state``."""

    def __init__(self, opts: dict, state: dict):
        self.opts = dict(opts)
        self.ndim = opts["ndim"]
        self.n = state["x"].shape[0]
        self._o = make_opts(opts)
        L = lib()
        L.orc_create.argtypes = [C.POINTER(type(self._o)), C.c_int]
        self.h = C.c_void_p(L.orc_create(C.byref(self._o), self.n))
        self.state = alloc_state(self.n, self.ndim)
        for k, v in state.items():
            self.state[k][...] = v
        self._push()

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _push(self):
        self._p = make_particles(self.state)
        lib().orc_set_state(self.h, C.byref(self._p))

    def _pull(self):
        lib().orc_get_state(self.h, C.byref(self._p))

    def _check(self, rc: int):
        if rc != 0:
            raise OracleError(rc, lib().orc_message(self.h).decode())

    def set_state(self, state: dict):
        for k, v in state.items():
            self.state[k][...] = v
        self._push()

    def primitive2conservative(self):
        self._check(lib().orc_primitive2conservative(self.h))
        self._pull()
        self.opts["polyk"] = lib().orc_polyk(self.h)

    def derivs(self):
        self._check(lib().orc_derivs(self.h))
        self._pull()

    def iterate_density(self):
        self._check(lib().orc_iterate_density(self.h))
        self._pull()

    def get_rates(self):
        self._check(lib().orc_get_rates(self.h))
        self._pull()

    def step(self, nsteps: int = 1):
        self._check(lib().orc_step(self.h, nsteps))
        self._pull()

    def set_dt(self, dt: float, time: float = 0.0):
        lib().orc_set_dt(self.h, dt, time)

    def dts(self) -> dict:
        d = NdsphDt()
        lib().orc_get_dt(self.h, C.byref(d))
        return d.as_dict()

    def neighbours(self, mode: int):
        """CSR of 1-based neighbour indices (self excluded)."""
        offs = np.zeros(self.n + 1, dtype=np.int64)
        cap = int(self.n * 200)
        while True:
            neigh = np.zeros(cap, dtype=np.int32)
            r = lib().orc_neighbour_csr(self.h, mode, offs.ctypes.data_as(C.POINTER(C.c_long)),
                                        neigh.ctypes.data_as(C.POINTER(C.c_int32)), cap)
            if r >= 0:
                return offs, neigh[:r]
            cap = -r

    def snapshot(self) -> dict:
        return copy_state(self.state)


def kernel_tables(ndim: int) -> np.ndarray:
    out = np.zeros(5 * 4001)
    lib().orc_kernel_tables(ndim, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(5, 4001)


def interp(ndim: int, q2: np.ndarray):
    q2 = np.ascontiguousarray(q2, dtype=np.float64)
    w = np.zeros_like(q2)
    gw = np.zeros_like(q2)
    P = C.POINTER(C.c_double)
    lib().orc_interp(ndim, len(q2), q2.ctypes.data_as(P), w.ctypes.data_as(P), gw.ctypes.data_as(P))
    return w, gw
