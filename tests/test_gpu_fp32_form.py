"""Error of the FP32 form against the FP64 form on the same particle sets.

The FP32 form takes separations from FP32 cell-relative coordinates, FP32
kernel tables and pair terms, compensated FP32 accumulation; the state, the
integration and the NR residual stay FP64.  Bound: 1e-5 of
max(|ref|, rms(ref), physical scale) for density, h and the force /
induction / energy rates; 1e-4 for drhodt and dalpha/dt (small residuals of
large pair sums in the turbulent box).
"""
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import compare_fields

pytestmark = pytest.mark.gpu

CASES = {
    "box3d": lambda: configs.mhd_box_3d(24, seed=2),
    "ot2d": lambda: configs.orszag_tang_2d(48),
    "dust3d": lambda: configs.dust_gas_box_3d(12, eps=0.5, tstop=0.05),
    "isothermal": lambda: configs.turbulent_box_3d(24),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp32_form_error(name, gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = CASES[name]()
    st = configs.full_state(p, o["ndim"])
    g = GpuSPH(o, st)
    g.primitive2conservative()
    base = {k: v.copy() for k, v in g.state.items()}
    g.close()
    res = {}
    for prec in (0, 1):
        o2 = dict(o)
        o2["precision"] = prec
        g = GpuSPH(o2, {k: v.copy() for k, v in base.items()})
        g.derivs()
        res[prec] = g.state
        g.close()
    errs, bad = compare_fields(res[1], res[0], ["rho", "hh", "gradh", "force", "dudt", "dBevoldt",
                                                "divB", "curlB"], 1e-5)
    assert not bad, (name, errs)
    errs2, bad2 = compare_fields(res[1], res[0], ["drhodt", "daldt"], 1e-4)
    assert not bad2, (name, errs2)
