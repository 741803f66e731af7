"""GPU parity of the plain FP64 form against the CPU oracle.

Every case starts both codes from the same particle arrays (the oracle's
primitive2conservative output) and compares through the C-ABI.  Tolerances:

* neighbour sets: bit-exact (sorted index lists per particle);
* numneigh and NR pass counts: exact;
* FP64 fields: |d| / max(|ref|, rms(ref)) <= 1e-12 (summation order differs:
  the GPU gathers each particle's sum, the reference scatters pairs);
* after several leapfrog steps: <= 1e-9 (round-off grows through the
  Newton-Raphson iteration and the integrator).
"""
import numpy as np
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import compare_fields, csr_sets

pytestmark = pytest.mark.gpu

DENS_FIELDS = ["rho", "hh", "gradh", "gradhn", "gradgradh", "drhodt", "dhdt", "rhoalt"]
RATE_FIELDS = ["force", "dBevoldt", "dudt", "dendt", "daldt", "divB", "curlB", "del2u", "graddivv",
               "pr", "spsound", "Bfield"]


def _cases():
    return {
        "ot2d": lambda: configs.orszag_tang_2d(32),
        "box3d": lambda: configs.mhd_box_3d(14, seed=3),
        "box3d_B": lambda: configs.mhd_box_3d(12, seed=5, imhd=11),
        "briowu": lambda: configs.brio_wu_tube(400),
        "dust3d": lambda: configs.dust_gas_box_3d(10, eps=0.5, tstop=0.05),
        "isothermal": lambda: configs.turbulent_box_3d(16),
    }


def _init(name):
    from oracle.oracle import Oracle
    o, p = _cases()[name]()
    st = configs.full_state(p, o["ndim"])
    orc = Oracle(o, st)
    orc.primitive2conservative()
    return o, orc


@pytest.fixture(scope="module", params=list(_cases().keys()))
def initialised(request, gpulib):
    o, orc = _init(request.param)
    o = dict(o)
    o["polyk"] = orc.opts["polyk"]
    return request.param, o, orc


def test_neighbour_sets_bit_exact(initialised):
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    g = GpuSPH(o, orc.snapshot())
    g.set_linklist()
    for mode in (0, 1):
        go, gn = g.neighbours(mode)
        oo, on = orc.neighbours(mode)
        gs, os_ = csr_sets(go, gn), csr_sets(oo, on)
        bad = [i for i in range(len(gs)) if not np.array_equal(gs[i], os_[i])]
        assert not bad, f"{name} mode {mode}: {len(bad)} particles differ, first {bad[:5]}"
    g.close()


def test_neighbour_sets_fp32_contexts(initialised):
    """An FP32-form context links on its own cells (5^ndim stencils of cells
    of hmax x skin where the box allows it); ndsph_neighbour_csr decides in
    exact FP64 over that stencil, so the sets must still equal the
    oracle's."""
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    g = GpuSPH(dict(o, precision=1), orc.snapshot())
    g.set_linklist()
    for mode in (0, 1):
        go, gn = g.neighbours(mode)
        oo, on = orc.neighbours(mode)
        gs, os_ = csr_sets(go, gn), csr_sets(oo, on)
        bad = [i for i in range(len(gs)) if not np.array_equal(gs[i], os_[i])]
        assert not bad, f"{name} mode {mode}: {len(bad)} particles differ, first {bad[:5]}"
    g.close()


def test_iterate_density(initialised):
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    st = orc.snapshot()
    # perturb h so that the NR loop takes several passes
    rng = np.random.default_rng(1)
    st["hh"] *= 1.0 + 0.05 * rng.uniform(-1, 1, size=st["hh"].shape)
    from oracle.oracle import Oracle
    ref = Oracle(o, st)
    ref.iterate_density()
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.iterate_density()
    assert g.dts()["its"] == ref.dts()["its"], (name, g.dts(), ref.dts())
    got = g.state
    errs, bad = compare_fields(got, ref.state, DENS_FIELDS, 1e-12)
    assert not bad, f"{name}: {errs}"
    nd = np.nonzero(got["numneigh"] != ref.state["numneigh"])[0]
    assert len(nd) == 0, (name, nd[:10], got["numneigh"][nd[:10]], ref.state["numneigh"][nd[:10]])
    g.close()


def test_derivs(initialised):
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    st = orc.snapshot()
    from oracle.oracle import Oracle
    ref = Oracle(o, st)
    ref.derivs()
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.derivs()
    errs, bad = compare_fields(g.state, ref.state, DENS_FIELDS + RATE_FIELDS, 1e-12)
    assert not bad, f"{name}: {errs}"
    assert np.array_equal(g.state["numneigh"], ref.state["numneigh"]), name
    gd, rd = g.dts(), ref.dts()
    for k in ("dtcourant", "dtforce", "dtav", "vsigmax", "stressmax"):
        assert abs(gd[k] - rd[k]) <= 1e-12 * max(abs(rd[k]), 1e-300), (name, k, gd[k], rd[k])
    if o["idust"]:
        assert abs(gd["dtdrag"] - rd["dtdrag"]) <= 1e-12 * rd["dtdrag"]
    g.close()


def test_leapfrog_steps(initialised):
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    st = orc.snapshot()
    from oracle.oracle import Oracle
    ref = Oracle(o, st)
    nsteps = 4
    ref.step(nsteps)
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.dev_upload()
    g.set_dt(0.0)
    g.dev_step(nsteps)
    g.dev_download()
    assert g.dts()["nsteps"] == nsteps
    assert abs(g.dts()["time"] - ref.dts()["time"]) <= 1e-10 * max(ref.dts()["time"], 1e-300)
    errs, bad = compare_fields(g.state, ref.state, ["x", "vel", "hh", "en", "Bevol", "rho", "force", "alpha"], 1e-9)
    assert not bad, f"{name}: {errs}"
    g.close()


def test_host_buffer_step(initialised):
    """ndsph_step: one leapfrog step per call with the state in host arrays
    (the reference-facing form the bench's e2e number times)."""
    from ndspmhd_gb300.gpu import GpuSPH
    name, o, orc = initialised
    st = orc.snapshot()
    from oracle.oracle import Oracle
    ref = Oracle(o, st)
    ref.step(3)
    host = {k: v.copy() for k, v in st.items()}
    if 1 not in list(o["ibound"])[:o["ndim"]]:
        # arrays the step only writes: garbage in them must not matter
        for k in ("rhoalt", "drhodt", "gradh", "gradhn", "gradgradh", "dens", "uu", "pr", "spsound", "Bfield",
                  "dudt", "divB", "curlB", "del2u", "graddivv"):
            host[k][...] = np.nan
        host["numneigh"][...] = -7
    g = GpuSPH(o, host)
    g.set_dt(0.0)
    for _ in range(3):
        g.step()
    assert g.dts()["nsteps"] == 3
    errs, bad = compare_fields(g.state, ref.state, ["x", "vel", "hh", "en", "Bevol", "rho", "force", "alpha"], 1e-9)
    assert not bad, f"{name}: {errs}"
    g.close()


def test_host_access_modes_identical(gpulib):
    """ndsph_step reading and writing the caller's arrays in place (pageable
    numpy arrays, and pinned buffers) gives bitwise the same particles as
    staging them through device copies."""
    import torch
    from ndspmhd_gb300.gpu import GpuSPH
    o, orc = _init("box3d")
    o = dict(o, polyk=orc.opts["polyk"])
    st0 = orc.snapshot()
    out = {}
    for mode, pinned in ((0, False), (1, False), (1, True)):
        st = {k: v.copy() for k, v in st0.items()}
        keep = []
        if pinned:
            for k, v in list(st.items()):
                t = torch.from_numpy(v).pin_memory()
                keep.append(t)
                st[k] = t.numpy()
        g = GpuSPH(o, st)
        g.set_host_access(mode)
        g.set_dt(0.0)
        for _ in range(2):
            g.step()
        out[(mode, pinned)] = {k: v.copy() for k, v in g.state.items()}
        g.close()
    ref = out[(0, False)]
    for key in ((1, False), (1, True)):
        for k, v in ref.items():
            assert np.array_equal(out[key][k], v), (key, k)
