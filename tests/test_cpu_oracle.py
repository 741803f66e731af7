"""CPU tests of the oracle (no GPU): analytic invariants that pin the
restatement in the absence of reference outputs."""
import math

import numpy as np
import pytest

from ndspmhd_gb300 import configs
from oracle import oracle as O


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_kernel_table_normalisation(ndim):
    # integral of W over the support ~ 1; exact up to the truncated pi and the
    # 1D constant 0.66666666666 the reference uses (kernelND.f90:4149-4156)
    t = O.kernel_tables(ndim)
    q2 = np.linspace(0, 4, 4001)
    q = np.sqrt(q2)
    w = t[0]
    fine = np.linspace(0, 2, 200001)
    wf = np.interp(fine ** 2, q2, w)
    if ndim == 1:
        integ = 2 * np.trapezoid(wf, fine)
    elif ndim == 2:
        integ = np.trapezoid(wf * 2 * np.pi * fine, fine)
    else:
        integ = np.trapezoid(wf * 4 * np.pi * fine ** 2, fine)
    assert abs(integ - 1.0) < 2e-6


def test_kernel_table_values():
    t = O.kernel_tables(3)
    pi_t = 3.141592653589
    assert t[0][0] == pytest.approx(1.0 / pi_t, rel=1e-15)
    assert t[0][4000] == 0.0 and t[1][4000] == 0.0
    # q = 1 boundary (q2 = 1 at index 1000): W = 0.25/pi
    assert t[0][1000] == pytest.approx(0.25 / pi_t, rel=1e-14)
    # drag kernel 41 vanishes at q = 0 and q = 2
    assert t[3][0] == 0.0 and t[3][4000] == 0.0


def test_interpolation_matches_reference_lerp():
    t = O.kernel_tables(2)
    q2 = np.array([0.0, 0.0005, 0.999, 1.0, 2.5, 3.9999, 4.0, 5.0])
    w, gw = O.interp(2, q2)
    dq2 = 4.0 / 4000.0
    idx = np.minimum((q2 * (1.0 / dq2)).astype(int), 4000)
    i1 = np.minimum(idx + 1, 4000)
    expect = t[0][idx] + (t[0][i1] - t[0][idx]) * (1.0 / dq2) * (q2 - idx * dq2)
    np.testing.assert_allclose(w, expect, rtol=0, atol=1e-15)


def test_lattice_density_uniform():
    o, p = configs.orszag_tang_2d(32)
    orc = O.Oracle(o, configs.full_state(p, 2))
    orc.primitive2conservative()
    rho = orc.state["rho"]
    assert rho.std() / rho.mean() < 1e-12
    assert abs(rho.mean() / (25 / (36 * math.pi)) - 1) < 5e-3


@pytest.mark.parametrize("maker", [lambda: configs.mhd_box_3d(10, seed=2),
                                   lambda: configs.orszag_tang_2d(24),
                                   lambda: configs.dust_gas_box_3d(8, eps=0.3, tstop=0.05)])
def test_pairwise_momentum_conservation(maker):
    o, p = maker()
    orc = O.Oracle(o, configs.full_state(p, o["ndim"]))
    orc.primitive2conservative()
    s = orc.state
    mf = s["pmass"][:, None] * s["force"]
    net = np.abs(mf.sum(0))
    scale = np.abs(mf).sum(0) + 1e-300
    assert np.all(net / scale < 1e-12)


def test_neighbour_list_vs_brute_force():
    # check_neighbourlist.f90:27-182: link-list neighbours == O(N^2) scan
    o, p = configs.mhd_box_3d(8, seed=9)
    orc = O.Oracle(o, configs.full_state(p, 3))
    orc.primitive2conservative()
    x, h = orc.state["x"], orc.state["hh"]
    L = 1.0
    offs, neigh = orc.neighbours(1)
    for i in range(0, len(x), 37):
        d = x[i] - x
        d -= L * np.round(d / L)
        r2 = (d ** 2).sum(1)
        ok = (r2 < 4 * h[i] ** 2) | (r2 < 4 * h ** 2)
        ok[i] = False
        brute = np.sort(np.nonzero(ok)[0] + 1)
        got = np.sort(neigh[offs[i]:offs[i + 1]])
        assert np.array_equal(brute, got), i


def test_energy_conservation_short_run():
    o, p = configs.orszag_tang_2d(24)
    orc = O.Oracle(o, configs.full_state(p, 2))
    orc.primitive2conservative()

    def etot(s):
        b2 = (s["Bfield"] ** 2).sum(1)
        return np.sum(s["pmass"] * (0.5 * (s["vel"] ** 2).sum(1) + s["uu"] + 0.5 * b2 / s["rho"]))

    e0 = etot(orc.state)
    orc.step(10)
    e1 = etot(orc.state)
    assert abs(e1 - e0) / e0 < 1e-3


def test_error_status_propagates():
    o, p = configs.orszag_tang_2d(16)
    st = configs.full_state(p, 2)
    orc = O.Oracle(o, st)
    orc.primitive2conservative()
    bad = orc.snapshot()
    bad["hh"][3] = 0.0
    o2 = O.Oracle(o, bad)
    with pytest.raises(O.OracleError) as e:
        o2.iterate_density()
    assert e.value.code == 3
