"""Batched form with periodic boundaries: two-fluid dust + gas boxes, each in
its own periodic unit cube with its own dust-to-gas ratio, drag constant K
and lattice jitter, in one device state.  Each box must evolve as it does
run alone through the oracle (one reference run per input file):

* the initialising derivs (primitive2conservative, then link, density
  iteration, EOS, rates with the gas-dust drag of ratesND_mhd.f90:1074-1169)
  at 1e-12 with numneigh exact, and four leapfrog steps at 1e-9 with each
  box's own dt (dtdrag from its own K) and clock;
* boxes of different resolution (8^3, 10^3, 12^3 pairs) in one batch, so the
  shared cells are sized by the coarsest box while each box keeps its own
  ghosts' hhmax (ghostND_mhd.f90:218) and relinks;
* the FP32 form of the batch within its 1e-5 bound of the oracle, and after
  six steps within 1e-5 of the same boxes run one at a time in the FP32 form
  (the batch's cells differ, so only the order of each pair sum does);
* a 2D periodic batch (Orszag-Tang at two resolutions) against the oracle.
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


def _boxes(settings):
    """(opts, particles) per setting (n1d, eps, t_s, seed), their
    concatenation, the simulation index of every particle and the K's."""
    runs = [configs.dust_gas_box_3d(n1d, eps=eps, tstop=ts, seed=seed) for n1d, eps, ts, seed in settings]
    parts = [p for _, p in runs]
    cat = {k: np.concatenate([q[k] for q in parts], axis=0) for k in parts[0]}
    sim = np.concatenate([np.full(q["x"].shape[0], s, np.int32) for s, q in enumerate(parts)])
    kd = np.array([o["Kdrag"] for o, _ in runs])
    # one option set for the batch: the drag constants go per simulation;
    # psep (only the density iteration's fallback step reads it) is the finest
    o = dict(runs[0][0], psep=min(o["psep"] for o, _ in runs))
    return runs, o, cat, sim, kd


def _batch(o, cat, sim, kd, nsim, prec, nsteps):
    from ndspmhd_gb300.gpu import GpuSPH
    g = GpuSPH(dict(o, precision=prec), configs.full_state(cat, 3))
    g.batch_set_kdrag(kd)
    g.batch_upload(sim, nsim, initialise=True)
    g.batch_download()
    first = {k: v.copy() for k, v in g.state.items()}
    dt = t = None
    if nsteps:
        dt, t = g.batch_step(nsteps)
        g.batch_download()
    out = {k: v.copy() for k, v in g.state.items()}
    tm = g.timing()
    g.close()
    return first, out, dt, t, tm


def _slices(runs):
    start = 0
    for o, p in runs:
        n = p["x"].shape[0]
        yield o, p, slice(start, start + n)
        start += n


def _oracle_derivs(o, p):
    from oracle.oracle import Oracle
    orc = Oracle(o, configs.full_state(p, 3))
    orc.primitive2conservative()
    orc.derivs()
    return orc


def _oracle_steps(o, p, nsteps):
    from oracle.oracle import Oracle
    orc = Oracle(o, configs.full_state(p, 3))
    orc.primitive2conservative()
    orc.step(nsteps)
    return orc


def test_dust_batch_two_settings_match_oracle(gpulib):
    settings = [(10, 0.5, 0.05, 77), (10, 0.02, 0.3, 78)]
    runs, o, cat, sim, kd = _boxes(settings)
    assert kd[0] != kd[1]
    nsteps = 4
    first, out, dt, t, tm = _batch(o, cat, sim, kd, len(settings), 0, nsteps)
    assert tm["graph_steps"] == 0 and tm["fused_steps"] == 0
    for k, (ok, pk, sl) in enumerate(_slices(runs)):
        ref = _oracle_derivs(ok, pk)
        got = {f: first[f][sl] for f in DENS_FIELDS + RATE_FIELDS + ["numneigh"]}
        errs, bad = compare_fields(got, ref.state, DENS_FIELDS + RATE_FIELDS, 1e-12)
        assert not bad, (k, errs)
        nd = np.nonzero(got["numneigh"] != ref.state["numneigh"])[0]
        assert len(nd) == 0, (k, len(nd), nd[:5])
        orc = _oracle_steps(ok, pk, nsteps)
        got = {f: out[f][sl] for f in STEP_FIELDS}
        errs, bad = compare_fields(got, orc.state, STEP_FIELDS, 1e-9)
        assert not bad, (k, errs)
        d = orc.dts()
        assert abs(t[k] - d["time"]) <= 1e-10 * d["time"], (k, t[k], d["time"])
        assert abs(dt[k] - d["dt"]) <= 1e-9 * d["dt"], (k, dt[k], d["dt"])


def test_dust_batch_uneven_resolutions_match_oracle(gpulib):
    settings = [(8, 1.0, 0.01, 80), (12, 0.1, 0.2, 81), (10, 0.03, 1.0, 82)]
    runs, o, cat, sim, kd = _boxes(settings)
    nsteps = 3
    _, out, dt, t, _ = _batch(o, cat, sim, kd, len(settings), 0, nsteps)
    for k, (ok, pk, sl) in enumerate(_slices(runs)):
        orc = _oracle_steps(ok, pk, nsteps)
        got = {f: out[f][sl] for f in STEP_FIELDS}
        errs, bad = compare_fields(got, orc.state, STEP_FIELDS, 1e-9)
        assert not bad, (k, errs)
        d = orc.dts()
        assert abs(t[k] - d["time"]) <= 1e-10 * d["time"], (k, t[k], d["time"])


def test_dust_batch_fp32_form(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    settings = [(12, 0.5, 0.05, 90), (12, 0.05, 0.5, 91)]
    runs, o, cat, sim, kd = _boxes(settings)
    nsteps = 6
    first, out, _, t, _ = _batch(o, cat, sim, kd, len(settings), 1, nsteps)
    for k, (ok, pk, sl) in enumerate(_slices(runs)):
        ref = _oracle_derivs(ok, pk)
        got = {f: first[f][sl] for f in FP32_FIELDS}
        errs, bad = compare_fields(got, ref.state, FP32_FIELDS, 1e-5)
        assert not bad, (k, errs)
        # the same box alone in the FP32 form
        g = GpuSPH(dict(ok, precision=1), configs.full_state(pk, 3))
        g.primitive2conservative()
        g.dev_upload()
        g.set_dt(0.0)
        g.dev_step(nsteps)
        g.dev_download()
        assert abs(g.dts()["time"] - t[k]) <= 1e-6 * t[k], (k, g.dts()["time"], t[k])
        got = {f: out[f][sl] for f in STEP_FIELDS}
        errs, bad = compare_fields(got, g.state, STEP_FIELDS, 1e-5)
        assert not bad, (k, errs)
        g.close()


def test_orszag_tang_2d_batch_match_oracle(gpulib):
    """A 2D periodic batch (the grids stacked along y): the Orszag-Tang vortex
    at two resolutions (32 x 36 and 48 x 56 particles on their own hcp
    lattices), MHD, against two oracle runs after 3 steps."""
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    runs = [configs.orszag_tang_2d(nx) for nx in (32, 48)]
    parts = [q for _, q in runs]
    cat = {k: np.concatenate([q[k] for q in parts], axis=0) for k in parts[0]}
    sim = np.concatenate([np.full(q["x"].shape[0], s, np.int32) for s, q in enumerate(parts)])
    o = dict(runs[0][0], psep=min(r[0]["psep"] for r in runs))
    g = GpuSPH(o, configs.full_state(cat, 2))
    g.batch_upload(sim, 2, initialise=True)
    dt, t = g.batch_step(3)
    g.batch_download()
    start = 0
    for k, (ok, pk) in enumerate(runs):
        n = pk["x"].shape[0]
        orc = Oracle(ok, configs.full_state(pk, 2))
        orc.primitive2conservative()
        orc.step(3)
        got = {f: g.state[f][start:start + n] for f in STEP_FIELDS}
        errs, bad = compare_fields(got, orc.state, STEP_FIELDS, 1e-9)
        assert not bad, (k, errs)
        d = orc.dts()
        assert abs(t[k] - d["time"]) <= 1e-10 * d["time"], (k, t[k], d["time"])
        start += n
    g.close()


def test_batch_refuses_mixed_boundaries(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH, NdsphError
    runs, o, cat, sim, kd = _boxes([(6, 0.5, 0.05, 1), (6, 0.5, 0.05, 2)])
    g = GpuSPH(dict(o, ibound=[3, 3, 0]), configs.full_state(cat, 3))
    with pytest.raises(NdsphError) as e:
        g.batch_upload(sim, 2, initialise=True)
    assert e.value.code == 1
    g.close()
    g = GpuSPH(o, configs.full_state(cat, 3))
    with pytest.raises(NdsphError):
        g.batch_set_kdrag(np.array([1.0, -1.0]))
    g.close()


def test_sweep_of_dust_infiles_batches_the_drag_constants(gpulib, tmp_path):
    """The sweep driver batches runs whose options files differ only in the
    drag constant (one periodic batch, one K per run) and each run evolves as
    the oracle runs its file."""
    from ndspmhd_gb300.infile import read_infile, run_sweep, write_infile
    from oracle.oracle import Oracle
    settings = [(8, 0.5, 0.05, 60), (8, 0.1, 0.3, 61)]
    runs = []
    for k, (n1d, eps, ts, seed) in enumerate(settings):
        o, p = configs.dust_gas_box_3d(n1d, eps=eps, tstop=ts, seed=seed)
        path = tmp_path / f"dust{k}.in"
        write_infile(str(path), o)
        runs.append((read_infile(str(path), 3, base=o), configs.full_state(p, 3)))
    assert runs[0][0]["Kdrag"] != runs[1][0]["Kdrag"]
    out = run_sweep(runs, 3, precision=0)
    for k, (o, st) in enumerate(runs):
        orc = Oracle(o, configs.full_state({f: st[f] for f in st}, 3))
        orc.primitive2conservative()
        orc.step(3)
        got, t, dt = out[k]
        errs, bad = compare_fields({f: got[f] for f in ("x", "vel", "hh", "en", "rho")}, orc.state,
                                   ["x", "vel", "hh", "en", "rho"], 1e-9)
        assert not bad, (k, errs)
        assert abs(t - orc.dts()["time"]) <= 1e-10 * orc.dts()["time"]


def test_batch_full_pass_rule_per_simulation(gpulib):
    """A Newton-Raphson pass is full while every particle of the run is
    unconverged (iterate_density.f90:129-133), which decides the union
    criterion of numneigh and the particle set of the pass.  In a batch whose
    first box starts 8 % off in h (no particle of it converges in the first
    pass) and whose second starts converged, the second pass is full for the
    first box only: both boxes must match their oracle runs, numneigh
    included."""
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    states, opts = [], None
    for k in range(2):
        o, p = configs.mhd_box_3d(10, seed=40 + k)
        g = GpuSPH(o, configs.full_state(p, 3))
        g.primitive2conservative()
        states.append({f: v.copy() for f, v in g.state.items()})
        g.close()
        opts = o
    states[0]["hh"] *= 1.08
    cat = {f: np.concatenate([s[f] for s in states], axis=0) for f in states[0]}
    sim = np.concatenate([np.full(s["x"].shape[0], k, np.int32) for k, s in enumerate(states)])
    g = GpuSPH(opts, cat)
    g.batch_upload(sim, 2, initialise=False)
    g.batch_step(1)
    g.batch_download()
    start = 0
    for k, s in enumerate(states):
        n = s["x"].shape[0]
        orc = Oracle(opts, {f: v.copy() for f, v in s.items()})
        orc.step(1)
        got = {f: g.state[f][start:start + n] for f in STEP_FIELDS + ["numneigh"]}
        errs, bad = compare_fields(got, orc.state, STEP_FIELDS, 1e-9)
        assert not bad, (k, errs)
        nd = np.nonzero(got["numneigh"] != orc.state["numneigh"])[0]
        assert len(nd) == 0, (k, len(nd), nd[:5])
        start += n
    g.close()
