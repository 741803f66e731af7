"""ctypes mirror of include/ndsph.h (structs and the C-ABI entry points).

The library is plain C-ABI: pointers and sizes only.  This module owns the
ctypes layouts so that the package, the tests and the bench all bind the same
shapes.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

from .configs import ALLOC_FIELDS_SCALAR, ALLOC_FIELDS_VEC3

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int32)


class NdsphOpts(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("ibound", C.c_int32 * 3),
        ("xmin", C.c_double * 3), ("xmax", C.c_double * 3),
        ("hfact", C.c_double), ("tolh", C.c_double), ("psep", C.c_double),
        ("maxdensits", C.c_int32), ("imhd", C.c_int32), ("imagforce", C.c_int32),
        ("iener", C.c_int32), ("iav", C.c_int32), ("iavlim", C.c_int32 * 3),
        ("alphamin", C.c_double), ("alphaumin", C.c_double), ("alphaBmin", C.c_double),
        ("beta", C.c_double), ("avdecayconst", C.c_double), ("gamma", C.c_double),
        ("polyk", C.c_double), ("idust", C.c_int32), ("idrag_nature", C.c_int32),
        ("Kdrag", C.c_double), ("C_cour", C.c_double), ("C_force", C.c_double),
        ("precision", C.c_int32), ("learned_h", C.c_int32),
    ]


PARTICLE_FIELDS = [
    ("x", "d"), ("vel", "d"), ("Bevol", "d"), ("en", "d"), ("hh", "d"), ("pmass", "d"),
    ("alpha", "d"), ("itype", "i"), ("ireal", "i"),
    ("rho", "d"), ("rhoalt", "d"), ("drhodt", "d"), ("dhdt", "d"), ("gradh", "d"),
    ("gradhn", "d"), ("gradgradh", "d"), ("numneigh", "i"),
    ("dens", "d"), ("uu", "d"), ("pr", "d"), ("spsound", "d"), ("Bfield", "d"),
    ("force", "d"), ("dBevoldt", "d"), ("dudt", "d"), ("dendt", "d"), ("daldt", "d"),
    ("divB", "d"), ("curlB", "d"), ("del2u", "d"), ("graddivv", "d"),
]


class NdsphParticles(C.Structure):
    _fields_ = [(name, c_double_p if t == "d" else c_int_p) for name, t in PARTICLE_FIELDS]


class NdsphDt(C.Structure):
    _fields_ = [
        ("dtcourant", C.c_double), ("dtforce", C.c_double), ("dtav", C.c_double),
        ("dtdrag", C.c_double), ("dtvisc", C.c_double), ("vsigmax", C.c_double),
        ("stressmax", C.c_double), ("hhmax", C.c_double), ("dt", C.c_double),
        ("time", C.c_double), ("its", C.c_int32), ("ncalctotal", C.c_int32),
        ("nsteps", C.c_int32), ("nrelink", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class NdsphTiming(C.Structure):
    _fields_ = [
        ("link_ms", C.c_float), ("density_ms", C.c_float), ("density_pass1_ms", C.c_float),
        ("eos_ms", C.c_float), ("rates_ms", C.c_float), ("post_ms", C.c_float),
        ("step_ms", C.c_float), ("total_ms", C.c_float), ("density_passes", C.c_int32),
        ("launches", C.c_int32), ("pairs_density", C.c_int64), ("pairs_rates", C.c_int64),
        ("mlp_loss", C.c_float), ("mlp_ms", C.c_float), ("mlp_updates", C.c_int32), ("nl_builds", C.c_int32),
        ("graph_steps", C.c_int32), ("graph_redos", C.c_int32), ("nl_reused", C.c_int32),
        ("fused_steps", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class NdsphTuning(C.Structure):
    """ndsph_tuning: neighbour-search knobs (include/ndsph.h)."""
    _fields_ = [("nl_skin", C.c_float), ("nl_reuse", C.c_int32), ("nl_grow", C.c_float),
                ("graph_cell_margin", C.c_float), ("stencil", C.c_int32), ("step_pieces", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def make_opts(d: dict) -> NdsphOpts:
    o = NdsphOpts()
    for name, ctype in NdsphOpts._fields_:
        v = d[name]
        if isinstance(v, (list, tuple)):
            arr = getattr(o, name)
            for k in range(3):
                arr[k] = v[k] if k < len(v) else 0
        else:
            setattr(o, name, v)
    return o


def alloc_state(n: int, ndim: int) -> dict:
    """Zeroed host arrays for every ndsph_particles field."""
    s = {"x": np.zeros((n, ndim))}
    for k in ALLOC_FIELDS_SCALAR:
        s[k] = np.zeros(n)
    for k in ALLOC_FIELDS_VEC3:
        s[k] = np.zeros((n, 3))
    s["pmass"] = np.zeros(n)
    s["itype"] = np.zeros(n, np.int32)
    s["ireal"] = np.zeros(n, np.int32)
    s["numneigh"] = np.zeros(n, np.int32)
    return s


def make_particles(state: dict) -> NdsphParticles:
    """Point an NdsphParticles at the numpy arrays of ``state`` (kept alive by
    the caller).  Arrays must be C-contiguous float64 / int32."""
    p = NdsphParticles()
    for name, t in PARTICLE_FIELDS:
        a = state[name]
        if t == "d":
            assert a.dtype == np.float64 and a.flags.c_contiguous, name
            setattr(p, name, a.ctypes.data_as(c_double_p))
        else:
            assert a.dtype == np.int32 and a.flags.c_contiguous, name
            setattr(p, name, a.ctypes.data_as(c_int_p))
    return p


def copy_state(s: dict) -> dict:
    return {k: v.copy() for k, v in s.items()}
