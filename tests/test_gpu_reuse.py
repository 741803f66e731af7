"""Neighbour-row reuse across steps (FP32 form, one simulation).

A step may keep the slot order, cells and rows of the previous link when
every particle satisfies h + dmax <= skin * h_build (dmax: the largest
displacement since the rows were built).  The pairs summed are then the same
as after a fresh link, so results agree with the relink-every-step run within
the FP32 form's rounding: |d| / max(|ref|, rms(ref), physical scale) <= 1e-5
after a few steps.  A row missing a neighbour inside the kernel support
would move that particle's density by ~1/60 and its force by far more than
that bound.  (numneigh is not compared: the reference defines it by the
union criterion in the first Newton-Raphson pass and by q_i < 2 in later
ones, so a particle converging one pass earlier in one run reports the other
count.)

The runs use tolh = 1e-6.  At the default 1e-3 a particle whose
Newton-Raphson residual sits at the threshold converges one pass earlier in
one run than in the other (the two differ by rounding), which legitimately
moves its h by up to ~tolh and its neighbours' forces by ~1e-4 -- the same
happens between the FP32 and FP64 forms; a tight tolerance puts every h at
the root, so the comparison sees the pair sums alone.
"""
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import compare_fields

pytestmark = pytest.mark.gpu

FIELDS = ["x", "vel", "hh", "rho", "en", "Bevol", "force"]


def _initial(case):
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = case()
    o = dict(o)
    o["precision"] = 1
    o["tolh"] = 1e-6
    g = GpuSPH(o, configs.full_state(p, o["ndim"]))
    g.primitive2conservative()
    st = {k: v.copy() for k, v in g.state.items()}
    g.close()
    return o, st


def _device_run(o, st, nsteps, **tuning):
    from ndspmhd_gb300.gpu import GpuSPH
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.set_tuning(**tuning)
    g.dev_upload()
    g.set_dt(0.0)
    for _ in range(nsteps):
        g.dev_step(1)
    g.dev_download()
    out = {k: v.copy() for k, v in g.state.items()}
    tim, dts = g.timing(), g.dts()
    g.close()
    return out, tim, dts


@pytest.mark.parametrize("skin", [1.1, 1.2])
def test_device_steps_with_reuse_match_relinking(skin, gpulib):
    o, st = _initial(lambda: configs.mhd_box_3d(24, seed=4))
    nsteps = 12
    a, ta, da = _device_run(o, st, nsteps, nl_reuse=1, nl_skin=skin)
    b, tb, db = _device_run(o, st, nsteps, nl_reuse=0, nl_skin=skin)
    assert ta["nl_reused"] >= nsteps // 2, ta
    assert tb["nl_reused"] == 0
    assert ta["nl_builds"] < tb["nl_builds"], (ta["nl_builds"], tb["nl_builds"])
    errs, bad = compare_fields(a, b, FIELDS, 1e-5)
    assert not bad, errs
    assert abs(da["time"] - db["time"]) <= 1e-6 * db["time"]


def test_host_steps_with_reuse_same_pairs(gpulib):
    """ndsph_step with host arrays: a context that keeps its link across calls
    and one that relinks on every call take the same inputs at every step."""
    from ndspmhd_gb300.gpu import GpuSPH
    o, st = _initial(lambda: configs.mhd_box_3d(20, seed=9))
    ga = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    ga.set_tuning(nl_reuse=1)
    ga.set_dt(0.0)
    cur = {k: v.copy() for k, v in st.items()}
    dt, t = 0.0, 0.0
    for step in range(8):
        ga.rebind({k: v.copy() for k, v in cur.items()})
        ga.dt.dt, ga.dt.time, ga.dt.nsteps = dt, t, step
        ga.step()
        gb = GpuSPH(o, {k: v.copy() for k, v in cur.items()})
        gb.set_tuning(nl_reuse=0)
        gb.dt.dt, gb.dt.time, gb.dt.nsteps = dt, t, step
        gb.step()
        errs, bad = compare_fields(ga.state, gb.state, ["rho", "hh", "force", "dudt", "dBevoldt"], 1e-5)
        assert not bad, (step, errs)
        cur = {k: v.copy() for k, v in gb.state.items()}
        dt, t = gb.dt.dt, gb.dt.time
        gb.close()
    reused = ga.timing()["nl_reused"]
    ga.close()
    assert reused >= 4, reused


def test_reuse_check_falls_back_to_relink(gpulib):
    """Supersonic flow, thin skin and no room left for Newton-Raphson growth
    of h: the check fails on some steps (a fresh link), and rows can go stale
    during the iteration of a step that kept the link (a relink there);
    results still match the relinking run."""
    o, st = _initial(lambda: configs.turbulent_box_3d(24))
    nsteps = 10
    a, ta, _ = _device_run(o, st, nsteps, nl_reuse=1, nl_skin=1.05, nl_grow=1.0)
    b, tb, _ = _device_run(o, st, nsteps, nl_reuse=0, nl_skin=1.05, nl_grow=1.0)
    assert ta["nl_reused"] < nsteps
    errs, bad = compare_fields(a, b, ["x", "vel", "hh", "rho", "force"], 1e-5)
    assert not bad, errs


def test_stencils_agree(gpulib):
    """5-wide stencils of half-size cells (the FP32 default) and 3-wide
    stencils of full cells find the same pairs: device runs agree within the
    FP32 form's rounding."""
    o, st = _initial(lambda: configs.mhd_box_3d(24, seed=6))
    a, ta, _ = _device_run(o, st, 6, stencil=5)
    b, tb, _ = _device_run(o, st, 6, stencil=3)
    errs, bad = compare_fields(a, b, FIELDS, 1e-5)
    assert not bad, errs


def test_tuning_rejects_out_of_range(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH, NdsphError
    o, p = configs.mhd_box_3d(10, seed=1)
    g = GpuSPH(o, configs.full_state(p, 3))
    t0 = g.get_tuning()
    assert t0["nl_reuse"] == 1 and abs(t0["nl_skin"] - 1.1) < 1e-6
    assert t0["stencil"] == 5 and t0["step_pieces"] == 8
    for bad in ({"nl_skin": 0.9}, {"nl_skin": 2.5}, {"nl_grow": 0.99}, {"graph_cell_margin": 0.5},
                {"nl_reuse": 2}, {"stencil": 4}, {"step_pieces": 0}, {"step_pieces": 9}):
        with pytest.raises(NdsphError):
            g.set_tuning(**bad)
    assert g.get_tuning() == t0
    g.close()


@pytest.mark.parametrize("precision,pieces", [(1, 3), (1, 7), (1, 8), (0, 3)])
def test_host_step_streamed_outputs_identical(precision, pieces, gpulib):
    """ndsph_step on 110,592 particles: with the rates sweep in pieces (each
    chunk of the host arrays copied back while the later pieces run) every
    array the step returns is bit-identical to the single-sweep step (7
    pieces: chunks of 15,799 and a last one of 15,798)."""
    import numpy as np
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.mhd_box_3d(48, seed=6)
    o = dict(o)
    o["precision"] = precision
    g0 = GpuSPH(o, configs.full_state(p, 3))
    g0.primitive2conservative()
    st = {k: v.copy() for k, v in g0.state.items()}
    g0.close()
    runs = []
    for k in (1, pieces):
        g = GpuSPH(o, {key: v.copy() for key, v in st.items()})
        g.set_tuning(step_pieces=k)
        g.dt.dt, g.dt.time, g.dt.nsteps = 0.0, 0.0, 0
        for _ in range(4):
            g.step()
        runs.append(({key: v.copy() for key, v in g.state.items()}, g.dt.dt, g.dt.time))
        g.close()
    (a, dta, ta), (b, dtb, tb) = runs
    assert dta == dtb and ta == tb
    differ = [key for key in a if not np.array_equal(a[key], b[key])]
    assert not differ, differ


def test_host_step_streamed_skips_null_outputs(gpulib):
    """Outputs the caller passes as null are not written (the rest streams as
    usual and matches a step that returns everything)."""
    import numpy as np
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.mhd_box_3d(48, seed=7)
    o = dict(o)
    o["precision"] = 1
    g0 = GpuSPH(o, configs.full_state(p, 3))
    g0.primitive2conservative()
    st = {k: v.copy() for k, v in g0.state.items()}
    g0.close()
    dropped = ("del2u", "graddivv", "curlB", "divB")
    runs = []
    for drop in (False, True):
        s = {k: v.copy() for k, v in st.items()}
        if drop:
            for k in dropped:
                s[k][...] = -7.0
        g = GpuSPH(o, s)
        if drop:
            for k in dropped:
                setattr(g._p, k, None)
        g.dt.dt, g.dt.time, g.dt.nsteps = 0.0, 0.0, 0
        for _ in range(3):
            g.step()
        runs.append({k: v.copy() for k, v in g.state.items()})
        g.close()
    full, part = runs
    for k in dropped:
        assert np.all(part[k] == -7.0), k
    differ = [k for k in full if k not in dropped and not np.array_equal(full[k], part[k])]
    assert not differ, differ


# outputs the Fortran shim's gpu_step leaves on the host between the steps
# whose results output/evwrite read (gpu_step_all_outputs = .false.)
INFO_ONLY = ("rho", "rhoalt", "drhodt", "gradh", "gradhn", "gradgradh", "numneigh", "dens", "uu", "pr",
             "spsound", "Bfield", "dudt", "divB", "curlB", "del2u", "graddivv")


@pytest.mark.parametrize("precision", [1, 0])
def test_host_step_integrator_outputs_only(precision, gpulib):
    """ndsph_step with every info-only output null (what gpu_step passes
    between output steps): the next step reads only x, vel, Bevol, en, hh,
    alpha and their rates, so three steps give bitwise the particles of three
    steps that return everything, and the null arrays stay untouched."""
    import numpy as np
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.mhd_box_3d(48, seed=7)
    o = dict(o, precision=precision)
    g0 = GpuSPH(o, configs.full_state(p, 3))
    g0.primitive2conservative()
    st = {k: v.copy() for k, v in g0.state.items()}
    g0.close()
    runs = []
    for drop in (False, True):
        s = {k: v.copy() for k, v in st.items()}
        if drop:
            for k in INFO_ONLY:
                s[k][...] = -7
        g = GpuSPH(o, s)
        if drop:
            for k in INFO_ONLY:
                setattr(g._p, k, None)
        g.dt.dt, g.dt.time, g.dt.nsteps = 0.0, 0.0, 0
        for _ in range(3):
            g.step()
        runs.append(({k: v.copy() for k, v in g.state.items()}, g.dts()))
        g.close()
    (full, dfull), (part, dpart) = runs
    for k in INFO_ONLY:
        assert np.all(part[k] == -7), k
    differ = [k for k in full if k not in INFO_ONLY and not np.array_equal(full[k], part[k])]
    assert not differ, differ
    assert dfull["dt"] == dpart["dt"] and dfull["time"] == dpart["time"]


@pytest.mark.parametrize("precision", [1, 0])
def test_device_steps_in_one_call_identical(precision, gpulib):
    """Several device-resident steps in one call (the corrector and the next
    predictor fused between them) leave the state bit-identical to the same
    steps taken one call at a time."""
    import numpy as np
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.mhd_box_3d(20, seed=5)
    o = dict(o)
    o["precision"] = precision
    g0 = GpuSPH(o, configs.full_state(p, 3))
    g0.primitive2conservative()
    st = {k: v.copy() for k, v in g0.state.items()}
    g0.close()
    runs = []
    for split in (False, True):
        g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
        g.dev_upload()
        g.set_dt(0.0)
        if split:
            for _ in range(6):
                g.dev_step(1)
        else:
            g.dev_step(6)
        g.dev_download()
        runs.append(({k: v.copy() for k, v in g.state.items()}, g.dt.dt, g.dt.time))
        g.close()
    (a, dta, ta), (b, dtb, tb) = runs
    assert dta == dtb and ta == tb
    differ = [k for k in a if not np.array_equal(a[k], b[k])]
    assert not differ, differ
