"""The CUDA path against the committed golden fixtures (tests/golden/), with
no oracle in the loop: the start arrays of each fixture go through the C-ABI
and the outputs are compared with the stored oracle outputs.

Tolerances, as |d| / max(|ref|, rms(ref), physical scale):
* plain FP64 form: derivs 1e-12, numneigh and the Newton-Raphson pass count
  exact, state after the leapfrog steps 1e-9;
* FP32 pair form: rho, h, gradh, force, du/dt, dB/dt, div B, curl B 1e-5;
  drhodt, dalpha/dt 1e-4 (small residuals of large pair sums); the state
  after the leapfrog steps 1e-5.
"""
import numpy as np
import pytest

from tests.golden import make_golden as G
from tests.helpers import compare_fields

pytestmark = pytest.mark.gpu

FLOAT_DERIVS = [k for k in G.DERIVS_FIELDS if k != "numneigh"]
FP32_TIGHT = ["rho", "hh", "gradh", "force", "dudt", "dBevoldt", "divB", "curlB"]


@pytest.mark.parametrize("name", list(G.cases()))
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_matches_fixture(name, prec, gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    o, arr = G.load(name)
    o["precision"] = prec
    start = G.section(arr, "start")
    want = dict(start, **G.section(arr, "derivs"))
    g = GpuSPH(o, {k: v.copy() for k, v in start.items()})
    g.derivs()
    if prec == 0:
        errs, bad = compare_fields(g.state, want, FLOAT_DERIVS, 1e-12)
        assert not bad, (name, errs)
        assert np.array_equal(g.state["numneigh"], want["numneigh"]), name
        d = g.dts()
        got = np.array([float(d[k]) for k in G.DT_KEYS])
        np.testing.assert_allclose(got, want["dts"], rtol=1e-12, atol=0)
    else:
        errs, bad = compare_fields(g.state, want, FP32_TIGHT, 1e-5)
        assert not bad, (name, errs)
        errs, bad = compare_fields(g.state, want, ["drhodt", "daldt"], 1e-4)
        assert not bad, (name, errs)
    g.close()
    g = GpuSPH(o, {k: v.copy() for k, v in start.items()})
    g.dev_upload()
    g.set_dt(0.0)
    g.dev_step(G.NSTEPS)
    g.dev_download()
    ws = dict(start, **G.section(arr, "steps"))
    tol = 1e-9 if prec == 0 else 1e-5
    errs, bad = compare_fields(g.state, ws, ["x", "vel", "Bevol", "en", "hh", "rho", "alpha", "force"], tol)
    assert not bad, (name, prec, errs)
    assert abs(g.dts()["dt"] - ws["dt"][0]) <= tol * ws["dt"][0]
    g.close()
