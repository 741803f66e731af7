"""The oracle against its committed golden fixtures (tests/golden/).

The reference ships no golden vectors; the fixtures freeze the oracle's
outputs on small seeded particle sets (generated by
tests/golden/make_golden.py).  Re-running the oracle from each fixture's start
arrays must reproduce them: derivs to 1e-13 of max(|ref|, rms(ref), physical
scale) -- bit-identical on one machine, the margin covers libm differences
between x86-64 and aarch64 -- with numneigh and the Newton-Raphson pass count
exact, and the state after the leapfrog steps to 1e-11.
"""
import numpy as np
import pytest

from tests.golden import make_golden as G
from tests.helpers import compare_fields

FLOAT_DERIVS = [k for k in G.DERIVS_FIELDS if k != "numneigh"]


@pytest.mark.parametrize("name", list(G.cases()))
def test_oracle_reproduces_fixture(name):
    from oracle.oracle import Oracle
    o, arr = G.load(name)
    start = G.section(arr, "start")
    want = dict(start, **G.section(arr, "derivs"))
    ref = Oracle(o, start)
    ref.derivs()
    errs, bad = compare_fields(ref.state, want, FLOAT_DERIVS, 1e-13)
    assert not bad, (name, errs)
    assert np.array_equal(ref.state["numneigh"], want["numneigh"]), name
    d = ref.dts()
    got_dts = np.array([float(d[k]) for k in G.DT_KEYS])
    np.testing.assert_allclose(got_dts, want["dts"], rtol=1e-13, atol=0)
    ref = Oracle(o, start)
    ref.set_dt(0.0, 0.0)
    ref.step(G.NSTEPS)
    ws = dict(start, **G.section(arr, "steps"))
    errs, bad = compare_fields(ref.state, ws, G.STEP_FIELDS, 1e-11)
    assert not bad, (name, errs)
    assert abs(ref.dts()["dt"] - ws["dt"][0]) <= 1e-11 * ws["dt"][0]


def test_fixtures_cover_every_workload_family():
    # 1D with fixed particles, 2D periodic MHD, 3D periodic MHD (B/rho and B),
    # two-fluid dust, isothermal turbulent box
    fams = set()
    for name in G.cases():
        o, arr = G.load(name)
        fams.add((o["ndim"], o["imhd"], o["idust"], o["iener"], tuple(o["ibound"][:o["ndim"]])))
    assert len(fams) == 6
