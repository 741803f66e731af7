"""Conservation over 100 leapfrog steps, GPU against the oracle.

The reference scatters each pair to both particles, so its momentum is
conserved to round-off; the GPU gathers each side separately, so its
conservation rests on the pair terms being antisymmetric term by term.  Both
codes run 100 steps (device-resident, FP64 form) from the same state, and the
GPU's drift of total momentum and total energy (kinetic + thermal + magnetic,
as evwrite_mhd.f90:27-320 sums them) must stay at the oracle's level:
momentum to 1e-12 of sum(m |v|), energy drift within 1.5x the oracle's plus
1e-12 of E.  The FP32 form is held to 1e-6 (momentum) and 2x the oracle's
energy drift plus 1e-7 of E.
"""
import numpy as np
import pytest

from ndspmhd_gb300 import configs

pytestmark = pytest.mark.gpu

NSTEPS = 100


def _totals(st: dict, o: dict):
    m = st["pmass"]
    mom = (m[:, None] * st["vel"]).sum(0)
    if o["imhd"] == 0:
        emag = 0.0
    elif o["imhd"] > 10:
        emag = 0.5 * np.sum(m * (st["Bevol"] ** 2).sum(1) / st["rho"])
    else:
        emag = 0.5 * np.sum(m * (st["Bevol"] ** 2).sum(1) * st["rho"])
    e = np.sum(m * (0.5 * (st["vel"] ** 2).sum(1) + st["uu"])) + emag
    return mom, e, np.sum(m * np.sqrt((st["vel"] ** 2).sum(1)))


def _uu(st, o):
    # thermal energy from the evolved variable (iener=2: en = u)
    return st["en"]


@pytest.mark.parametrize("case", ["ot2d", "box3d"])
@pytest.mark.parametrize("precision", [0, 1])
def test_conservation_100_steps(gpulib, case, precision):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p = configs.orszag_tang_2d(32) if case == "ot2d" else configs.mhd_box_3d(12, seed=7)
    orc = Oracle(o, configs.full_state(p, o["ndim"]))
    orc.primitive2conservative()
    st0 = orc.snapshot()
    o = dict(o, polyk=orc.opts["polyk"])

    def totals(st):
        s = dict(st)
        s["uu"] = _uu(st, o)
        return _totals(s, o)

    p0, e0, scale = totals(st0)
    ref = Oracle(o, {k: v.copy() for k, v in st0.items()})
    ref.step(NSTEPS)
    pr, er, _ = totals(ref.state)

    og = dict(o, precision=precision)
    g = GpuSPH(og, {k: v.copy() for k, v in st0.items()})
    g.dev_upload()
    g.set_dt(0.0)
    g.dev_step(NSTEPS)
    g.dev_download()
    pg, eg, _ = totals(g.state)
    g.close()

    dp_ref = np.abs(pr - p0).max() / scale
    dp_gpu = np.abs(pg - p0).max() / scale
    de_ref = abs(er - e0) / abs(e0)
    de_gpu = abs(eg - e0) / abs(e0)
    if precision == 0:
        assert dp_gpu <= 1e-12, (dp_gpu, dp_ref)
        assert de_gpu <= 1.5 * de_ref + 1e-12, (de_gpu, de_ref)
    else:
        assert dp_gpu <= 1e-6, (dp_gpu, dp_ref)
        assert de_gpu <= 2.0 * de_ref + 1e-7, (de_gpu, de_ref)
