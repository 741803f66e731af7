"""The allocation-free entry point ndsph_density_noalloc.

It serves callers that may not allocate device memory when they call (device
memory owned by another runtime's pool, real-time loops that must not take
cudaMalloc's implicit synchronisation, applications that reserve all device
memory up front): they hand in device buffers, and the entry point's only
other memory is a fixed file-scope device array.

This file checks, through the C-ABI, that two calls in a row give the same
rho, gradh, drhodt and numneigh as the allocating path
(ndsph_iterate_density with maxdensits = 0, i.e. one density pass with every
particle treated as converged), within the 1e-12 tolerance of the other
parity tests, and that sizes above the fixed maximum are refused.  It is
collected last so that a failure here cannot hide the other tests.
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


def _noalloc(f, o, st):
    import torch
    from ndspmhd_gb300.abi import make_opts
    dev = torch.device("cuda:0")
    n = st["x"].shape[0]
    x = torch.from_numpy(np.ascontiguousarray(st["x"])).to(dev)
    hh = torch.from_numpy(st["hh"].copy()).to(dev)
    pm = torch.from_numpy(st["pmass"].copy()).to(dev)
    vel = torch.from_numpy(np.ascontiguousarray(st["vel"])).to(dev)
    it = torch.from_numpy(st["itype"].copy()).to(dev)
    rho = torch.zeros(n, dtype=torch.float64, device=dev)
    drhodt = torch.zeros(n, dtype=torch.float64, device=dev)
    gradh = torch.zeros(n, dtype=torch.float64, device=dev)
    nn = torch.zeros(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    oo = make_opts(o)
    rc = f(C.byref(oo), x.data_ptr(), hh.data_ptr(), pm.data_ptr(), vel.data_ptr(), it.data_ptr(), n,
           rho.data_ptr(), drhodt.data_ptr(), gradh.data_ptr(), nn.data_ptr(), None)
    assert rc == 0, rc
    return {"rho": rho.cpu().numpy(), "gradh": gradh.cpu().numpy(), "drhodt": drhodt.cpu().numpy(),
            "numneigh": nn.cpu().numpy()}


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


def test_noalloc_refuses_sizes_above_maximum(gpulib):
    f = _bind(gpulib)
    from ndspmhd_gb300.abi import make_opts
    o, _ = configs.mhd_box_3d(4)
    oo = make_opts(o)
    rc = f(C.byref(oo), None, None, None, None, None, NOALLOC_MAX_N + 1, None, None, None, None, None)
    assert rc == 10      # NDSPH_E_CAPACITY
