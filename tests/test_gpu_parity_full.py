"""GPU parity against the oracle on the benchmark workloads at their own sizes.

The small-case parity tests (test_gpu_parity.py) cover every option path; this
file repeats the checks on the particle sets the throughput figures are quoted
on, so that bit-exact neighbour sets and the 1e-12 / 1e-9 bounds hold there
too:

* 2D Orszag-Tang vortex, 256 x 296 = 75,776 particles (the reference's own CPU
  case): neighbour sets bit-exact (both criteria), one derivs at 1e-12 with
  numneigh exact, four leapfrog steps at 1e-9, and the FP32 form's derivs
  within its 1e-5 bound;
* 3D MHD box: 64^3 neighbour sets bit-exact; at 128^3 = 2,097,152 particles
  one derivs at 1e-12 with numneigh exact (so every particle's neighbour count
  over both criteria agrees) and the FP32 form's derivs within 1e-5 (at the
  workload's tolh, bar the few particles whose convergence pass differs);
* a 1,600-particle Brio-Wu tube with fixed ends (the largest tube of the
  batched workload): neighbour sets, derivs, four steps;
* the two-fluid dust box at 2 x 24^3 (every gas-dust drag pair): derivs and
  four steps; at its own size, 2 x 96^3, one derivs in both forms; and the
  batch of its 8 settings (14.2 M particles) against each setting run alone.

Both codes start from the same state (primitive2conservative of the GPU
FP64 form for the 128^3 box, whose oracle set-up would take half a minute;
the oracle's own for the others).  Tolerances as test_gpu_parity.py:
|d| / max(|ref|, rms(ref), physical scale).
"""
import numpy as np
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import compare_fields

pytestmark = pytest.mark.gpu

DENS_FIELDS = ["rho", "hh", "gradh", "gradhn", "gradgradh", "drhodt", "dhdt", "rhoalt"]
RATE_FIELDS = ["force", "dBevoldt", "dudt", "dendt", "daldt", "divB", "curlB", "del2u", "graddivv",
               "pr", "spsound", "Bfield"]
STEP_FIELDS = ["x", "vel", "hh", "en", "Bevol", "rho", "force", "alpha"]
FP32_FIELDS = ["rho", "hh", "gradh", "force", "dudt", "dBevoldt", "divB", "curlB"]


def _sorted_csr(offs, neigh):
    """Per-row sorted neighbour ids, as one flat array (rows in order)."""
    counts = np.diff(offs)
    rows = np.repeat(np.arange(len(counts)), counts)
    order = np.lexsort((neigh, rows))
    return counts, neigh[order]


def _check_neighbour_sets(g, orc, name):
    for mode in (0, 1):
        gc, gn = _sorted_csr(*g.neighbours(mode))
        oc, on = _sorted_csr(*orc.neighbours(mode))
        bad = np.nonzero(gc != oc)[0]
        assert len(bad) == 0, f"{name} mode {mode}: {len(bad)} counts differ, first {bad[:5]}"
        assert np.array_equal(gn, on), f"{name} mode {mode}: neighbour ids differ"


def _oracle_start(o, p):
    from oracle.oracle import Oracle
    orc = Oracle(o, configs.full_state(p, o["ndim"]))
    orc.primitive2conservative()
    return dict(o, polyk=orc.opts["polyk"]), orc.snapshot()


def _derivs_pair(o, st):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    ref = Oracle(o, {k: v.copy() for k, v in st.items()})
    ref.derivs()
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.derivs()
    return g, ref


def _check_derivs(g, ref, o, name):
    errs, bad = compare_fields(g.state, ref.state, DENS_FIELDS + RATE_FIELDS, 1e-12)
    assert not bad, f"{name}: {errs}"
    nd = np.nonzero(g.state["numneigh"] != ref.state["numneigh"])[0]
    assert len(nd) == 0, (name, len(nd), nd[:5])
    gd, rd = g.dts(), ref.dts()
    assert gd["its"] == rd["its"], (name, gd["its"], rd["its"])
    for k in ("dtcourant", "dtforce", "dtav", "vsigmax", "stressmax"):
        assert abs(gd[k] - rd[k]) <= 1e-12 * max(abs(rd[k]), 1e-300), (name, k, gd[k], rd[k])
    if o["idust"]:
        assert abs(gd["dtdrag"] - rd["dtdrag"]) <= 1e-12 * rd["dtdrag"], (name, gd["dtdrag"], rd["dtdrag"])


def _check_fp32(o, st, ref, name):
    from ndspmhd_gb300.gpu import GpuSPH
    g = GpuSPH(dict(o, precision=1), {k: v.copy() for k, v in st.items()})
    g.derivs()
    errs, bad = compare_fields(g.state, ref.state, FP32_FIELDS, 1e-5)
    assert not bad, f"{name} FP32 form: {errs}"
    g.close()


def _check_fp32_many(o, st, ref, name):
    """The FP32 form on a set of millions of particles.  At the workload's
    tolh (1e-3) a particle whose Newton-Raphson residual sits within the FP32
    form's ~5e-7 density error of the tolerance stops one pass earlier or
    later than in the FP64 arithmetic, and its h then differs by up to
    ~tolh: against the oracle, those particles (a few per million) and their
    neighbours are allowed up to tolh, every other particle 1e-5.  At tolh
    1e-6 no decision differs and every particle holds 1e-5, checked against
    the FP64 form (itself within 1e-12 of the oracle, above)."""
    from ndspmhd_gb300.gpu import GpuSPH
    from tests.helpers import field_scales
    g = GpuSPH(dict(o, precision=1), {k: v.copy() for k, v in st.items()})
    g.derivs()
    sc = field_scales(ref.state)
    dh = np.abs(g.state["hh"] - ref.state["hh"]) / ref.state["hh"]
    flipped = dh > 1e-5
    assert flipped.sum() <= 1e-5 * len(dh) + 2, (name, int(flipped.sum()))
    assert dh.max() <= 1.05 * o["tolh"], (name, float(dh.max()))
    for k in FP32_FIELDS:
        a, b = g.state[k], ref.state[k]
        rms = float(np.sqrt(np.mean(b ** 2)))
        e = np.abs(a - b) / np.maximum(np.abs(b), max(rms, sc.get(k, 0.0)))
        e = e.max(axis=1) if e.ndim > 1 else e
        assert np.mean(e > 1e-5) <= 1e-3, (name, k, float(np.mean(e > 1e-5)))
        assert e.max() <= 2.0 * o["tolh"], (name, k, float(e.max()))
    g.close()
    res = {}
    for prec in (0, 1):
        g = GpuSPH(dict(o, precision=prec, tolh=1e-6), {k: v.copy() for k, v in st.items()})
        g.derivs()
        res[prec] = g.state
        g.close()
    errs, bad = compare_fields(res[1], res[0], FP32_FIELDS, 1e-5)
    assert not bad, f"{name} FP32 form at tolh 1e-6: {errs}"


def _check_steps(o, st, name, nsteps=4):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    ref = Oracle(o, {k: v.copy() for k, v in st.items()})
    ref.step(nsteps)
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.dev_upload()
    g.set_dt(0.0)
    g.dev_step(nsteps)
    g.dev_download()
    assert g.dts()["nsteps"] == nsteps
    assert abs(g.dts()["time"] - ref.dts()["time"]) <= 1e-10 * max(ref.dts()["time"], 1e-300)
    errs, bad = compare_fields(g.state, ref.state, STEP_FIELDS, 1e-9)
    assert not bad, f"{name}: {errs}"
    g.close()


@pytest.fixture(scope="module")
def ot_full():
    o, p = configs.orszag_tang_2d(256)
    assert p["x"].shape[0] == 75776
    return _oracle_start(o, p)


def test_orszag_tang_full_neighbour_sets(gpulib, ot_full):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, st = ot_full
    orc = Oracle(o, {k: v.copy() for k, v in st.items()})
    for prec in (0, 1):
        g = GpuSPH(dict(o, precision=prec), {k: v.copy() for k, v in st.items()})
        g.set_linklist()
        _check_neighbour_sets(g, orc, f"ot2d 256x296 prec {prec}")
        g.close()


def test_orszag_tang_full_derivs(gpulib, ot_full):
    o, st = ot_full
    g, ref = _derivs_pair(o, st)
    _check_derivs(g, ref, o, "ot2d 256x296")
    g.close()
    _check_fp32(o, st, ref, "ot2d 256x296")


def test_orszag_tang_full_steps(gpulib, ot_full):
    o, st = ot_full
    _check_steps(o, st, "ot2d 256x296")


def test_mhd_box_64_neighbour_sets(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p = configs.mhd_box_3d(64, seed=1234)
    o, st = _oracle_start(o, p)
    orc = Oracle(o, {k: v.copy() for k, v in st.items()})
    for prec in (0, 1):
        g = GpuSPH(dict(o, precision=prec), {k: v.copy() for k, v in st.items()})
        g.set_linklist()
        _check_neighbour_sets(g, orc, f"box 64^3 prec {prec}")
        g.close()


def test_mhd_box_128_derivs(gpulib):
    """The headline workload itself: one derivs of the 128^3 box, FP64 form
    against the oracle at 1e-12 (numneigh exact for all 2,097,152 particles),
    and the FP32 form within 1e-5 of the oracle."""
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.mhd_box_3d(128, seed=1234)
    assert o["iener"] == 2   # polyk plays no part
    g = GpuSPH(o, configs.full_state(p, 3))
    g.primitive2conservative()
    st = {k: v.copy() for k, v in g.state.items()}
    g.close()
    g, ref = _derivs_pair(o, st)
    _check_derivs(g, ref, o, "box 128^3")
    g.close()
    _check_fp32_many(o, st, ref, "box 128^3")


def test_brio_wu_1600_tube(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p = configs.brio_wu_tube(1600)
    o, st = _oracle_start(o, p)
    orc = Oracle(o, {k: v.copy() for k, v in st.items()})
    g = GpuSPH(o, {k: v.copy() for k, v in st.items()})
    g.set_linklist()
    _check_neighbour_sets(g, orc, "brio-wu 1600")
    g.close()
    g, ref = _derivs_pair(o, st)
    _check_derivs(g, ref, o, "brio-wu 1600")
    g.close()
    _check_steps(o, st, "brio-wu 1600")


def test_dust_box_full_2x96(gpulib):
    """The dust workload at its own size (2 x 96^3 = 1,769,472 particles, one
    of its settings): one derivs, FP64 form against the oracle at 1e-12 with
    numneigh exact and dtdrag, the FP32 form within its stated bounds."""
    from ndspmhd_gb300.gpu import GpuSPH
    o, p = configs.dust_gas_box_3d(96, eps=0.3, tstop=0.02, seed=77)
    g = GpuSPH(o, configs.full_state(p, 3))
    g.primitive2conservative()
    st = {k: v.copy() for k, v in g.state.items()}
    g.close()
    g, ref = _derivs_pair(o, st)
    _check_derivs(g, ref, o, "dust 2x96^3")
    g.close()
    _check_fp32_many(o, st, ref, "dust 2x96^3")


def test_dust_batch_full_8_settings(gpulib):
    """The batched dust workload at its own size: 8 (eps, t_s) settings of
    2 x 96^3 in one periodic batch (14,155,776 particles), FP32 form.  After
    two steps every setting agrees with the same setting run alone (FP32 form)
    within 1e-5: the batch's shared cells change only the order of each pair
    sum.  At tolh 1e-6, as in _check_fp32_many: at the workload's 1e-3 a few
    particles per million sit within rounding of the tolerance and stop one
    Newton-Raphson pass apart in the two orders, which moves their h by up to
    tolh."""
    from ndspmhd_gb300.gpu import GpuSPH
    rng = np.random.default_rng(99)
    eps = np.exp(rng.uniform(np.log(0.01), np.log(1.0), 8))
    ts = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), 8))
    runs = [configs.dust_gas_box_3d(96, eps=float(eps[k]), tstop=float(ts[k]), seed=77 + k) for k in range(8)]
    parts = [q for _, q in runs]
    cat = {k: np.concatenate([q[k] for q in parts], axis=0) for k in parts[0]}
    sim = np.concatenate([np.full(q["x"].shape[0], s, np.int32) for s, q in enumerate(parts)])
    runs = [(dict(o, tolh=1e-6), q) for o, q in runs]
    o0 = dict(runs[0][0], precision=1)
    g = GpuSPH(o0, configs.full_state(cat, 3))
    g.batch_set_kdrag([o["Kdrag"] for o, _ in runs])
    g.batch_upload(sim, 8, initialise=True)
    _, t = g.batch_step(2)
    g.batch_download()
    out = {k: g.state[k].copy() for k in STEP_FIELDS}
    g.close()
    start = 0
    for k, (o, q) in enumerate(runs):
        n = q["x"].shape[0]
        a = GpuSPH(dict(o, precision=1), configs.full_state(q, 3))
        a.primitive2conservative()
        a.dev_upload()
        a.set_dt(0.0)
        a.dev_step(2)
        a.dev_download()
        assert abs(a.dts()["time"] - t[k]) <= 1e-6 * t[k], (k, a.dts()["time"], t[k])
        errs, bad = compare_fields({f: out[f][start:start + n] for f in STEP_FIELDS}, a.state, STEP_FIELDS, 1e-5)
        assert not bad, (k, errs)
        a.close()
        start += n


def test_dust_box_2x24(gpulib):
    o, p = configs.dust_gas_box_3d(24, eps=0.5, tstop=0.05)
    o, st = _oracle_start(o, p)
    g, ref = _derivs_pair(o, st)
    _check_derivs(g, ref, o, "dust 2x24^3")
    g.close()
    _check_fp32(o, st, ref, "dust 2x24^3")
    _check_steps(o, st, "dust 2x24^3")
