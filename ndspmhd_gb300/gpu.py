"""Python host binding of libndsph_gpu.so (the C-ABI of include/ndsph.h).

``GpuSPH`` mirrors the reference's hot-path subroutines on one set of host
arrays in Fortran module layout (see ``ndspmhd_gb300.configs``):

=================================  =========================================
reference (file:line)              method
=================================  =========================================
set_linklist  linkND.f90:45        ``set_linklist()``
iterate_density iterate_density.f90:43  ``iterate_density()``
conservative2primitive :42         ``conservative2primitive()``
get_rates  ratesND_mhd.f90:29      ``get_rates()``
derivs  derivs.f90:27              ``derivs()``
step  stepND_leapfrog_mhd.f90:31   ``step()`` / ``dev_step()``
primitive2conservative :478        ``primitive2conservative()``
=================================  =========================================

Errors come back as :class:`NdsphError` carrying the library's status code,
as the reference would ``call quit``.  There is no CPU fallback: importing the
binding without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (NdsphDt, NdsphOpts, NdsphParticles, NdsphTiming, NdsphTuning, alloc_state, make_opts,
                  make_particles)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libndsph_gpu.so")

ERRORS = {
    1: "bad argument", 2: "CUDA error", 3: "h <= 0", 4: "rho <= 0", 5: "density not converged",
    6: "MHD signal-speed determinant < 0", 7: "non-finite value", 8: "cell grid invalid",
    9: "coincident particles", 10: "capacity exceeded", 11: "thermal energy < 0",
}

_lib = None


class NdsphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ndsph error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the in-tree CUDA library (never a fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc sm_103a) first")
    L = C.CDLL(LIB_PATH)
    P, PP = C.c_void_p, C.POINTER(C.c_void_p)
    parts = C.POINTER(NdsphParticles)
    dtp = C.POINTER(NdsphDt)
    L.ndsph_init.argtypes = [PP, C.POINTER(NdsphOpts), C.c_int32]
    L.ndsph_finalize.argtypes = [P]
    L.ndsph_last_error.argtypes = [P]
    L.ndsph_last_error.restype = C.c_char_p
    for name in ("ndsph_set_linklist", "ndsph_iterate_density", "ndsph_get_rates", "ndsph_derivs",
                 "ndsph_step", "ndsph_primitive2conservative"):
        getattr(L, name).argtypes = [P, parts, C.c_int32, dtp]
    L.ndsph_conservative2primitive.argtypes = [P, parts, C.c_int32]
    L.ndsph_dev_upload.argtypes = [P, parts, C.c_int32]
    L.ndsph_dev_download.argtypes = [P, parts, dtp]
    L.ndsph_dev_step.argtypes = [P, C.c_int32, dtp]
    L.ndsph_dev_derivs.argtypes = [P, dtp]
    L.ndsph_dev_set_time.argtypes = [P, C.c_double, C.c_double, C.c_int32]
    L.ndsph_neighbour_csr.argtypes = [P, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int64]
    L.ndsph_kernel_tables.argtypes = [C.c_int32, C.POINTER(C.c_double)]
    L.ndsph_get_timing.argtypes = [P, C.POINTER(NdsphTiming)]
    L.ndsph_set_profiling.argtypes = [P, C.c_int32]
    L.ndsph_set_learning.argtypes = [P, C.c_float, C.c_int32, C.c_int32]
    L.ndsph_batch_upload.argtypes = [P, parts, C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_int32]
    L.ndsph_batch_step.argtypes = [P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ndsph_batch_download.argtypes = [P, parts]
    L.ndsph_batch_set_kdrag.argtypes = [P, C.c_int32, C.POINTER(C.c_double)]
    L.ndsph_set_tuning.argtypes = [P, C.POINTER(NdsphTuning)]
    L.ndsph_get_tuning.argtypes = [P, C.POINTER(NdsphTuning)]
    _lib = L
    return L


def kernel_tables(ndim: int) -> np.ndarray:
    out = np.zeros(5 * 4001)
    rc = lib().ndsph_kernel_tables(ndim, out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc:
        raise NdsphError(rc, "kernel tables")
    return out.reshape(5, 4001)


class GpuSPH:
    """One device context (one CUDA stream) plus the host arrays it serves."""

    def __init__(self, opts: dict, state: dict | None = None, n: int | None = None, nmax: int = 0):
        self.opts = dict(opts)
        self.ndim = opts["ndim"]
        if state is None:
            state = alloc_state(int(n), self.ndim)
        self.state = state
        self.n = state["x"].shape[0]
        self._o = make_opts(opts)
        self._h = C.c_void_p()
        rc = lib().ndsph_init(C.byref(self._h), C.byref(self._o), max(nmax, self.n))
        if rc:
            raise NdsphError(rc, lib().ndsph_last_error(None).decode())
        self._p = make_particles(self.state)
        self.dt = NdsphDt()

    def close(self):
        if self._h:
            lib().ndsph_finalize(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc:
            raise NdsphError(rc, lib().ndsph_last_error(self._h).decode())

    def rebind(self, state: dict):
        """Point the context at another host array set of the same size."""
        self.state = state
        self._p = make_particles(state)

    # ---- drop-in entry points ------------------------------------------------
    def set_linklist(self):
        self._check(lib().ndsph_set_linklist(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    def iterate_density(self):
        self._check(lib().ndsph_iterate_density(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    def conservative2primitive(self):
        self._check(lib().ndsph_conservative2primitive(self._h, C.byref(self._p), self.n))

    def get_rates(self):
        self._check(lib().ndsph_get_rates(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    def derivs(self):
        self._check(lib().ndsph_derivs(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    def step(self):
        self._check(lib().ndsph_step(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    def primitive2conservative(self):
        self._check(lib().ndsph_primitive2conservative(self._h, C.byref(self._p), self.n, C.byref(self.dt)))

    # ---- device-resident form ---------------------------------------------------
    def dev_upload(self):
        self._check(lib().ndsph_dev_upload(self._h, C.byref(self._p), self.n))

    def dev_step(self, nsteps: int = 1):
        self._check(lib().ndsph_dev_step(self._h, nsteps, C.byref(self.dt)))

    def dev_derivs(self):
        self._check(lib().ndsph_dev_derivs(self._h, C.byref(self.dt)))

    def dev_download(self):
        self._check(lib().ndsph_dev_download(self._h, C.byref(self._p), C.byref(self.dt)))

    def set_dt(self, dt: float, time: float = 0.0, nsteps: int = 0):
        self.dt.dt = dt
        self.dt.time = time
        self.dt.nsteps = nsteps
        self._check(lib().ndsph_dev_set_time(self._h, dt, time, nsteps))

    # ---- batched form ---------------------------------------------------------------
    def batch_upload(self, sim: np.ndarray, nsim: int, initialise: bool = True):
        self._sim = np.ascontiguousarray(sim, dtype=np.int32)
        self.nsim = nsim
        self._check(lib().ndsph_batch_upload(self._h, C.byref(self._p), self.n,
                                             self._sim.ctypes.data_as(C.POINTER(C.c_int32)), nsim,
                                             1 if initialise else 0))

    def batch_step(self, nsteps: int = 1):
        dt = np.zeros(self.nsim)
        t = np.zeros(self.nsim)
        self._check(lib().ndsph_batch_step(self._h, nsteps, dt.ctypes.data_as(C.POINTER(C.c_double)),
                                           t.ctypes.data_as(C.POINTER(C.c_double))))
        return dt, t

    def set_host_access(self, mode: int):
        self._check(lib().ndsph_set_host_access(self._h, int(mode)))

    def batch_set_kdrag(self, kdrag):
        """Per-simulation drag constants K; call before batch_upload so the
        initialising derivs use them."""
        k = np.ascontiguousarray(kdrag, dtype=np.float64)
        self._check(lib().ndsph_batch_set_kdrag(self._h, len(k), k.ctypes.data_as(C.POINTER(C.c_double))))

    def batch_set_graph(self, mode: int):
        self._check(lib().ndsph_batch_set_graph(self._h, int(mode)))

    def batch_download(self):
        self._check(lib().ndsph_batch_download(self._h, C.byref(self._p)))

    # ---- diagnostics --------------------------------------------------------------
    def dts(self) -> dict:
        return self.dt.as_dict()

    def neighbours(self, mode: int):
        offs = np.zeros(self.n + 1, dtype=np.int64)
        cap = int(self.n) * 64
        while True:
            neigh = np.zeros(max(cap, 1), dtype=np.int32)
            rc = lib().ndsph_neighbour_csr(self._h, mode, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                           neigh.ctypes.data_as(C.POINTER(C.c_int32)), cap)
            if rc == 10:
                cap = int(offs[-1])
                continue
            self._check(rc)
            return offs, neigh[: offs[-1]]

    def set_learning(self, lr: float = 2e-3, iters_per_step: int = 4, batch: int = 16384):
        self._check(lib().ndsph_set_learning(self._h, lr, iters_per_step, batch))

    def get_tuning(self) -> dict:
        t = NdsphTuning()
        self._check(lib().ndsph_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        """Change tuning knobs (nl_skin, nl_reuse, nl_grow,
        graph_cell_margin, stencil, step_pieces); the others keep their
        values."""
        t = NdsphTuning()
        self._check(lib().ndsph_get_tuning(self._h, C.byref(t)))
        for k, v in kw.items():
            if k not in dict(NdsphTuning._fields_):
                raise KeyError(k)
            setattr(t, k, v)
        self._check(lib().ndsph_set_tuning(self._h, C.byref(t)))

    def set_profiling(self, on: bool = True):
        self._check(lib().ndsph_set_profiling(self._h, 1 if on else 0))

    def timing(self) -> dict:
        t = NdsphTiming()
        self._check(lib().ndsph_get_timing(self._h, C.byref(t)))
        return t.as_dict()
