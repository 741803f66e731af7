"""Batched form: many independent Brio-Wu tubes in one device state must
evolve exactly as each tube run alone through the oracle (per-tube dt,
per-tube stressmax and timestep reductions, fixed end particles)."""
import numpy as np
import pytest

from ndspmhd_gb300 import configs
from tests.helpers import compare_fields

pytestmark = pytest.mark.gpu


def test_batched_tubes_match_independent_oracle_runs(gpulib):
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p, sim, counts = configs.brio_wu_batch(ntubes=5, nmin=200, nmax=700, seed=5)
    st = configs.full_state(p, 1)
    g = GpuSPH(o, st)
    g.batch_upload(sim, len(counts), initialise=True)
    nsteps = 4
    dt, t = g.batch_step(nsteps)
    g.batch_download()
    start = 0
    for k, c in enumerate(counts):
        ok, pk = configs.brio_wu_tube(int(_npart_arg(c)))
        assert pk["x"].shape[0] == c
        orc = Oracle(ok, configs.full_state(pk, 1))
        orc.primitive2conservative()
        orc.step(nsteps)
        ref = orc.state
        got = {f: g.state[f][start:start + c] for f in ("x", "vel", "hh", "en", "Bevol", "rho", "force")}
        errs, bad = compare_fields(got, ref, list(got), 1e-9)
        assert not bad, (k, errs)
        d = orc.dts()
        assert abs(t[k] - d["time"]) <= 1e-10 * d["time"], (k, t[k], d["time"])
        assert abs(dt[k] - d["dt"]) <= 1e-9 * d["dt"], (k, dt[k], d["dt"])
        start += c
    g.close()


def _npart_arg(c):
    # brio_wu_tube rounds npart to 9 n_R; c is already such a count
    return int(c)


def test_sweep_from_infiles_matches_oracle(gpulib, tmp_path):
    """Sweep driver: three tube runs given by options files, two sharing
    their options (one batched launch) and one with another gamma."""
    from ndspmhd_gb300.infile import read_infile, run_sweep, write_infile
    from oracle.oracle import Oracle
    runs = []
    for k, (npart, gamma) in enumerate([(270, 2.0), (450, 2.0), (360, 1.4)]):
        o, p = configs.brio_wu_tube(npart)
        o = dict(o, gamma=gamma)
        p["uu"][:] = np.where(p["dens"] == 1.0, 1.0, 0.1) / ((gamma - 1.0) * p["dens"])
        path = tmp_path / f"tube{k}.in"
        write_infile(str(path), o)
        runs.append((read_infile(str(path), 1, base=o), configs.full_state(p, 1)))
    nsteps = 3
    out = run_sweep(runs, nsteps, precision=0)
    for k, (o, st) in enumerate(runs):
        orc = Oracle(o, configs.full_state({f: st[f] for f in st}, 1))
        orc.primitive2conservative()
        orc.step(nsteps)
        got, t, dt = out[k]
        errs, bad = compare_fields({f: got[f] for f in ("x", "vel", "hh", "en", "rho")},
                                   orc.state, ["x", "vel", "hh", "en", "rho"], 1e-9)
        assert not bad, (k, errs)
        assert abs(t - orc.dts()["time"]) <= 1e-10 * orc.dts()["time"]


def _batch_run(o, p, sim, nsim, mode, nsteps):
    from ndspmhd_gb300.gpu import GpuSPH
    g = GpuSPH(o, configs.full_state(p, 1))
    g.batch_upload(sim, nsim, initialise=True)
    g.batch_set_graph(mode)
    dt, t = g.batch_step(nsteps)
    g.batch_download()
    out = ({f: v.copy() for f, v in g.state.items()}, dt, t, g.timing())
    g.close()
    return out


FIELDS = ["x", "vel", "hh", "en", "Bevol", "rho", "force"]


def test_graph_step_matches_eager_step(gpulib):
    """Captured steps (one CUDA graph launch each, Newton-Raphson passes under
    a device-driven WHILE node) against the eager host loop on the same tubes,
    FP64 form.  The captured link uses wider cells, so only the order of each
    particle's neighbour sum differs: 1e-11 after 12 steps."""
    o, p, sim, counts = configs.brio_wu_batch(ntubes=24, nmin=200, nmax=900, seed=9)
    eager = _batch_run(o, p, sim, len(counts), 0, 12)
    graph = _batch_run(o, p, sim, len(counts), 2, 12)
    assert eager[3]["graph_steps"] == 0
    assert graph[3]["graph_steps"] >= 12
    assert graph[3]["graph_redos"] <= graph[3]["graph_steps"]
    errs, bad = compare_fields(graph[0], eager[0], FIELDS, 1e-11)
    assert not bad, errs
    np.testing.assert_allclose(graph[1], eager[1], rtol=1e-11)
    np.testing.assert_allclose(graph[2], eager[2], rtol=1e-11)


def test_graph_step_fp32_error_unchanged(gpulib):
    """FP32 form: the captured step's cells differ from the eager step's, so
    the FP32 cell-relative coordinates round differently; its error against
    the FP64 eager run must stay at the eager FP32 run's level (within 2x)."""
    o, p, sim, counts = configs.brio_wu_batch(ntubes=24, nmin=200, nmax=900, seed=9)
    ref = _batch_run(o, p, sim, len(counts), 0, 3)
    o32 = dict(o, precision=1)
    eager = _batch_run(o32, p, sim, len(counts), 0, 3)
    graph = _batch_run(o32, p, sim, len(counts), 2, 3)
    e_eager, _ = compare_fields(eager[0], ref[0], FIELDS, 1.0)
    e_graph, _ = compare_fields(graph[0], ref[0], FIELDS, 1.0)
    for f in FIELDS:
        assert e_graph[f] <= 2.0 * e_eager[f] + 1e-7, (f, e_graph, e_eager)


def test_fused_tube_step_matches_eager_step(gpulib):
    """The fused per-tube step (one block per tube runs the tube's whole step,
    candidates from the tube's x order instead of cells and rows) against the
    eager host loop, FP64 form: only the order of each particle's neighbour
    sums differs, 1e-11 after 12 steps; dt and time per tube likewise."""
    o, p, sim, counts = configs.brio_wu_batch(ntubes=24, nmin=200, nmax=900, seed=9)
    eager = _batch_run(o, p, sim, len(counts), 0, 12)
    fused = _batch_run(o, p, sim, len(counts), 1, 12)
    assert eager[3]["fused_steps"] == 0
    assert fused[3]["fused_steps"] == 12 and fused[3]["graph_steps"] == 0
    errs, bad = compare_fields(fused[0], eager[0], FIELDS, 1e-11)
    assert not bad, errs
    np.testing.assert_allclose(fused[1], eager[1], rtol=1e-11)
    np.testing.assert_allclose(fused[2], eager[2], rtol=1e-11)


def test_fused_tube_step_fp32_error(gpulib):
    """FP32 form of the fused step: its error against the FP64 eager run stays
    at the eager FP32 run's level (within 2x)."""
    o, p, sim, counts = configs.brio_wu_batch(ntubes=24, nmin=200, nmax=900, seed=9)
    ref = _batch_run(o, p, sim, len(counts), 0, 3)
    o32 = dict(o, precision=1)
    eager = _batch_run(o32, p, sim, len(counts), 0, 3)
    fused = _batch_run(o32, p, sim, len(counts), 1, 3)
    assert fused[3]["fused_steps"] == 3
    e_eager, _ = compare_fields(eager[0], ref[0], FIELDS, 1.0)
    e_fused, _ = compare_fields(fused[0], ref[0], FIELDS, 1.0)
    for f in FIELDS:
        assert e_fused[f] <= 2.0 * e_eager[f] + 1e-7, (f, e_fused, e_eager)


def test_fused_tube_step_out_of_order_particles(gpulib):
    """Tubes whose particles are not in x order in their slots (two interior
    particles of each tube with their positions exchanged, so index order and
    x order disagree inside a cell): the fused step ranks the tube by x and
    still matches independent oracle runs at 1e-9 after 4 steps."""
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p, sim, counts = configs.brio_wu_batch(ntubes=4, nmin=200, nmax=500, seed=13)
    start = np.concatenate([[0], np.cumsum(counts)])
    tubes = []
    for k, c in enumerate(counts):
        ok, pk = configs.brio_wu_tube(int(c))
        a = c // 3
        pk["x"][[a, a + 1]] = pk["x"][[a + 1, a]]
        p["x"][start[k] + a], p["x"][start[k] + a + 1] = pk["x"][a].copy(), pk["x"][a + 1].copy()
        tubes.append((ok, pk))
    g = GpuSPH(o, configs.full_state(p, 1))
    g.batch_upload(sim, len(counts), initialise=True)
    nsteps = 4
    dt, t = g.batch_step(nsteps)
    assert g.timing()["fused_steps"] == nsteps
    g.batch_download()
    for k, (ok, pk) in enumerate(tubes):
        orc = Oracle(ok, configs.full_state(pk, 1))
        orc.primitive2conservative()
        orc.step(nsteps)
        c0, c1 = start[k], start[k + 1]
        got = {f: g.state[f][c0:c1] for f in ("x", "vel", "hh", "en", "Bevol", "rho", "force")}
        errs, bad = compare_fields(got, orc.state, list(got), 1e-9)
        assert not bad, (k, errs)
        assert abs(t[k] - orc.dts()["time"]) <= 1e-10 * orc.dts()["time"]
    g.close()
