"""The allocation-free entry point ndsph_density_noalloc.

It serves callers that may not allocate device memory when they call (device
memory owned by another runtime's pool, real-time loops that must not take
cudaMalloc's implicit synchronisation, applications that reserve all device
memory up front): they hand in device buffers, and the entry point's only
other memory is a fixed file-scope device array.

This file checks, through the C-ABI, that two calls in a row give the same
rho, gradh, drhodt and numneigh as the allocating path
(ndsph_iterate_density with maxdensits = 0, i.e. one density pass with every
particle treated as converged) and as the oracle, within the 1e-12 tolerance
of the other parity tests -- in 1D (a Brio-Wu tube with fixed ends, whose
fixed particles' outputs the call leaves alone), 2D and 3D, on the legacy
stream and on a caller's stream -- and that sizes above the fixed maximum,
bounding boxes that would need too many cells, non-finite positions,
unsupported boundaries and h <= 0 / rho <= 0 are refused with a status and a
message in ndsph_last_error(NULL).  It is collected last so that a failure
here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import field_err

pytestmark = pytest.mark.gpu

NOALLOC_MAX_N = 1 << 18


def _bind(lib):
    from ndspmhd_gb300.abi import NdsphOpts
    f = lib.ndsph_density_noalloc
    f.argtypes = [C.POINTER(NdsphOpts)] + [C.c_void_p] * 5 + [C.c_int32] + [C.c_void_p] * 4 + [C.c_void_p]
    f.restype = C.c_int
    return f


def _reference(o, st):
    """The allocating path: one density pass, every particle converged."""
    from ndspmhd_gb300.gpu import GpuSPH
    o0 = dict(o)
    o0["maxdensits"] = 0
    g = GpuSPH(o0, {k: v.copy() for k, v in st.items()})
    g.iterate_density()
    out = {k: g.state[k].copy() for k in ("rho", "gradh", "drhodt", "numneigh")}
    g.close()
    return out


def _noalloc(f, o, st, stream=None, fill=0.0, expect=0):
    """One call on device copies of the state; outputs start at `fill`.
    `stream`: a torch.cuda.Stream the call runs on (None: the legacy stream)."""
    import torch
    from ndspmhd_gb300.abi import make_opts
    dev = torch.device("cuda:0")
    n = st["x"].shape[0]
    x = torch.from_numpy(np.ascontiguousarray(st["x"])).to(dev)
    hh = torch.from_numpy(st["hh"].copy()).to(dev)
    pm = torch.from_numpy(st["pmass"].copy()).to(dev)
    vel = torch.from_numpy(np.ascontiguousarray(st["vel"])).to(dev)
    it = torch.from_numpy(st["itype"].copy()).to(dev)
    rho = torch.full((n,), fill, dtype=torch.float64, device=dev)
    drhodt = torch.full((n,), fill, dtype=torch.float64, device=dev)
    gradh = torch.full((n,), fill, dtype=torch.float64, device=dev)
    nn = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    oo = make_opts(o)
    sh = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = f(C.byref(oo), x.data_ptr(), hh.data_ptr(), pm.data_ptr(), vel.data_ptr(), it.data_ptr(), n,
           rho.data_ptr(), drhodt.data_ptr(), gradh.data_ptr(), nn.data_ptr(), sh)
    assert rc == expect, (rc, _last_error())
    torch.cuda.synchronize()
    return {"rho": rho.cpu().numpy(), "gradh": gradh.cpu().numpy(), "drhodt": drhodt.cpu().numpy(),
            "numneigh": nn.cpu().numpy()}


def _last_error():
    from ndspmhd_gb300.gpu import lib
    return lib().ndsph_last_error(None).decode()


def _oracle(o, st):
    """The oracle's iterate_density with maxdensits = 0 (one pass, every
    particle converged)."""
    from oracle.oracle import Oracle
    orc = Oracle(dict(o, maxdensits=0), {k: v.copy() for k, v in st.items()})
    orc.iterate_density()
    return {k: orc.state[k].copy() for k in ("rho", "gradh", "drhodt", "numneigh")}


def _check(got, ref, st, mask=None):
    sel = np.ones(len(ref["rho"]), bool) if mask is None else mask
    for k in ("rho", "gradh"):
        assert field_err(got[k][sel], ref[k][sel]) <= 1e-12, (k, field_err(got[k][sel], ref[k][sel]))
    scale = float(np.mean(ref["rho"][sel])) * max(float(np.sqrt(np.mean((st["vel"] ** 2).sum(1)))), 1e-30) \
        / float(np.mean(st["hh"]))
    assert field_err(got["drhodt"][sel], ref["drhodt"][sel], scale) <= 1e-12
    assert np.array_equal(got["numneigh"], ref["numneigh"])


def _state(maker):
    from oracle.oracle import Oracle
    o, p = maker()
    orc = Oracle(o, configs.full_state(p, o["ndim"]))
    orc.primitive2conservative()
    st = orc.snapshot()
    rng = np.random.default_rng(7)
    st["hh"] *= 1.0 + 0.03 * rng.uniform(-1, 1, size=st["hh"].shape)
    return o, st


def test_noalloc_matches_allocating_path_two_calls(gpulib):
    f = _bind(gpulib)
    cases = [_state(lambda: configs.mhd_box_3d(16, seed=11)),
             _state(lambda: configs.orszag_tang_2d(40))]
    for o, st in cases:          # two calls in a row on the shared scratch
        ref = _reference(o, st)
        got = _noalloc(f, o, st)
        for k in ("rho", "gradh"):
            assert field_err(got[k], ref[k]) <= 1e-12, (k, field_err(got[k], ref[k]))
        scale = float(np.mean(ref["rho"])) * max(float(np.sqrt(np.mean((st["vel"] ** 2).sum(1)))), 1e-30) \
            / float(np.mean(st["hh"]))
        assert field_err(got["drhodt"], ref["drhodt"], scale) <= 1e-12
        assert np.array_equal(got["numneigh"], ref["numneigh"])


def test_noalloc_matches_oracle_1d_2d_3d_and_a_stream(gpulib):
    """Against the oracle (one density pass, maxdensits = 0): a 1D Brio-Wu
    tube with 6 fixed particles per end, the 2D Orszag-Tang lattice and a 3D
    box, each on a caller's CUDA stream.  Fixed particles' rho, gradh and
    drhodt are left as they were (the caller copies them from their sources);
    numneigh is compared for every particle."""
    import torch
    f = _bind(gpulib)
    s = torch.cuda.Stream()
    cases = [_state(lambda: configs.brio_wu_tube(400)),
             _state(lambda: configs.orszag_tang_2d(40)),
             _state(lambda: configs.mhd_box_3d(16, seed=11))]
    for o, st in cases:
        ref = _oracle(o, st)
        got = _noalloc(f, o, st, stream=s, fill=-7.0)
        fixed = (st["itype"] == 1) | (st["itype"] == 12)
        _check(got, ref, st, ~fixed)
        for k in ("rho", "gradh", "drhodt"):
            assert np.all(got[k][fixed] == -7.0), k
        if o["ndim"] == 1:
            assert fixed.sum() == 12


def test_noalloc_refuses_sizes_above_maximum(gpulib):
    f = _bind(gpulib)
    from ndspmhd_gb300.abi import make_opts
    o, _ = configs.mhd_box_3d(4)
    oo = make_opts(o)
    rc = f(C.byref(oo), None, None, None, None, None, NOALLOC_MAX_N + 1, None, None, None, None, None)
    assert rc == 10      # NDSPH_E_CAPACITY
    assert "fixed maximum" in _last_error()


def test_noalloc_refusals(gpulib):
    """Bad inputs come back as a status with a message, before any cell index
    is formed: a bounding box that needs more cells than the fixed maximum
    (12 particles spread over 1000 units with h = 0.01 in an open 3D box), a
    non-finite position, an unsupported boundary (reflective ghosts), h = 0,
    and zero masses (rho = 0)."""
    f = _bind(gpulib)
    o, st = _state(lambda: configs.mhd_box_3d(8, seed=3))
    # open box, two clusters 1000 apart: ~5e4 cells a side
    wide = {k: v[:12].copy() for k, v in st.items()}
    wide["x"][:6] = 0.5 + 0.001 * np.arange(18).reshape(6, 3)
    wide["x"][6:] = 1000.0 + 0.001 * np.arange(18).reshape(6, 3)
    wide["hh"][:] = 0.01
    _noalloc(f, dict(o, ibound=[0, 0, 0]), wide, expect=10)
    assert "cells above the fixed maximum" in _last_error()
    bad = {k: v.copy() for k, v in st.items()}
    bad["x"][5, 2] = np.nan
    _noalloc(f, o, bad, expect=7)
    assert "non-finite" in _last_error()
    _noalloc(f, dict(o, ibound=[2, 2, 2]), st, expect=1)
    assert "ibound" in _last_error()
    bad = {k: v.copy() for k, v in st.items()}
    bad["hh"][17] = 0.0
    _noalloc(f, o, bad, expect=3)
    assert "h <= 0" in _last_error()
    bad = {k: v.copy() for k, v in st.items()}
    bad["pmass"][:] = 0.0
    _noalloc(f, o, bad, expect=4)
    assert "rho <= 0" in _last_error()
    # and the next call works
    got = _noalloc(f, o, st)
    _check(got, _oracle(o, st), st)
