#!/usr/bin/env python
"""Benchmark of the NDSPMHD per-step hot path on GB300.

Workload (one "step" = one leapfrog step of the whole box: link, all
Newton-Raphson density passes, EOS, rates, predictor/corrector, dt):
the 3D MHD uniform box, 128^3 = 2,097,152 particles in a periodic unit cube,
jittered cubic lattice (seed 1234), rho = 1, v ~ N(0, 0.1^2), B = (0.1, 0, 0)
plus a 1% transverse perturbation, gamma = 5/3, cubic-spline kernel,
hfact = 1.2, tolh = 1e-3.  Synthetic data generated in-process.

Metric: particle-updates/s = N x steps / device time of the step loop.
``value`` is the chosen form -- FP32 pair sums with the learned h predictor
in front of the Newton-Raphson iteration -- with the state resident in HBM;
``fp32_predictor`` the FP32 form with the reference's own predictor;
``fp64`` the plain FP64 form (the parity form) on the same workload;
``fp32_error_vs_fp64`` the FP32 forms' error against the FP64 form (tolh 1e-3
and 1e-6, with the speed ratio at 1e-6); ``e2e`` times the reference-facing
C-ABI call ndsph_step with the state in pinned host buffers (H2D of the state
and D2H of the result every step).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
(N>1 under torchrun: independent replicas, one box per rank, weak scaling.)
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N1D = int(os.environ.get("NDSPH_BENCH_N1D", "128"))
CPU_SAMPLE_N1D = 48          # CPU baseline sample: 48^3 box, 2 steps
CPU_SAMPLE_STEPS = 2
METRIC = "SPH particle-updates/s on 1 GB300: FP32+learned-h vs plain FP64 at stated error"
UNIT = "particle-updates/s"

# algorithmic bytes per particle of the rates sweep: reads x(3) v(3) m h rho P
# c_s u gradh B(3) alpha(3) Bevol(3) drhodt dhdt (26 doubles) and writes
# force(3) dBevol/dt(3) du/dt de/dt dalpha/dt(3) divB curlB(3) del2u
# graddivv(3) drhodt dhdt (21 doubles) once each
RATES_BYTES_PER_PARTICLE = (26 + 21) * 8
# ncu of one k_rates<3,FP32> launch of the 64^3 box (profiles/k_rates_mhd_box3d_64cubed_fp32.md):
# DRAM bytes read + written, warp instructions issued, and the ratios that explain it
RATES_DRAM_BYTES_64 = 148.6e6
RATES_WARP_INSTR_64 = 253.8e6
RATES_NCU_64 = {"issue_active_frac": 0.601, "threads_per_instruction": 29.7, "warps_active_frac": 0.223,
                "fma_pipe_frac": 0.402, "top_stalls_per_issue": {"wait": 1.55, "long_scoreboard": 1.28}}
SMS, SMSP_PER_SM = 152, 4
# density pass: reads x(3) h m v(3) (8 doubles) writes rho rhoalt drhodt dhdt
# gradh gradhn gradgradh h (8 doubles) + numneigh (4 B)
DENSITY_BYTES_PER_PARTICLE = 16 * 8 + 4


def _load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def max_over_ranks(x: float, dist, device: str) -> float:
    """Largest value over the ranks (the slowest replica's time); the value
    itself without a process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job particle-updates/s of `world` independent replicas of an
    n-particle box, timed by the slowest (weak scaling)."""
    return world * n_per_rank / (ms_max * 1e-3)


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._first = threading.Event()
        self._proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                if self._stop.is_set():
                    break
                self.samples.append(parts)
                self._first.set()

    def wait_first(self, timeout: float = 3.0):
        """Block until nvidia-smi delivered its first sample (its start-up
        takes longer than a short timed region)."""
        self._first.wait(timeout)

    def stop(self) -> dict:
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                smax = float(s[1])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if s[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_problem(n1d: int, precision: int):
    from ndspmhd_gb300 import configs
    o, p = configs.mhd_box_3d(n1d, seed=1234)
    o["precision"] = precision
    return o, configs.full_state(p, 3)


def init_state(o, st):
    """primitive2conservative on the GPU (untimed set-up)."""
    from ndspmhd_gb300.gpu import GpuSPH
    g = GpuSPH(o, st)
    g.primitive2conservative()
    return g


def tune(o, st):
    """Search settings for this workload from the project autotuner (timed
    trials on copies of the initial state; the timed run starts afresh)."""
    from ndspmhd_gb300 import autotune
    g = init_state(o, st)
    st0 = {k: v.copy() for k, v in g.state.items()}
    g.close()
    return autotune.tune_device(o, st0, steps=8, warmup=3)


def run_device(o, st, steps: int, warmup: int, dist=None, tuning=None):
    """Device-resident timing: returns (ms_per_step, timing dict, dts, clocks)."""
    import torch
    g = init_state(o, st)
    if tuning:
        g.set_tuning(**tuning)
    g.dev_upload()
    g.set_dt(0.0)
    g.dev_step(warmup)
    g.set_profiling(False)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    kept0, builds0 = g.timing()["nl_reused"], g.timing()["nl_builds"]
    clk.start()
    clk.wait_first()
    g.dev_step(steps)              # bracketed by CUDA events on the library's stream
    torch.cuda.synchronize()
    clocks = clk.stop()
    t_timed = g.timing()
    t_timed["kept_link_steps"] = t_timed["nl_reused"] - kept0
    t_timed["row_builds"] = t_timed["nl_builds"] - builds0
    total_ms = t_timed["total_ms"]
    launches = t_timed["launches"]
    # kernel breakdown on one extra profiled step (not part of the timed loop)
    g.set_profiling(True)
    g.dev_step(1)
    tim = g.timing()
    tim["launches_timed"] = launches
    tim["kept_link_steps"] = t_timed["kept_link_steps"]
    tim["row_builds"] = t_timed["row_builds"]
    dts = g.dts()
    g.close()
    return total_ms / steps, tim, dts, clocks


# outputs of ndsph_step that no later step reads: the Fortran shim's gpu_step
# passes them as null between the steps whose results output/evwrite read
INFO_ONLY = ("rho", "rhoalt", "drhodt", "gradh", "gradhn", "gradgradh", "numneigh", "dens", "uu", "pr",
             "spsound", "Bfield", "dudt", "divB", "curlB", "del2u", "graddivv")


def run_e2e(o, steps: int, warmup: int, tuning=None):
    """Reference-facing C-ABI call with pinned host buffers: ndsph_step, one
    leapfrog step per call, every input uploaded and every result copied back
    inside the timed loop.  Two output sets: the integrator's (x, vel, Bevol,
    en, hh, alpha and their rates: what the next step reads, and what the
    Fortran shim's gpu_step returns between output steps) and all 47.5
    doubles a particle ndsph_step can return (the shim's output steps).
    Returns {set: (value, h2d bytes, d2h bytes, per-call ms min/median/max)}
    and the in-place-access rate."""
    import numpy as np
    import torch
    from ndspmhd_gb300.gpu import GpuSPH
    # the caller's form (precision, learned h) on the same particle set
    o2 = dict(o)
    _, st = make_problem(N1D, o["precision"])
    g0 = init_state(o2, st)
    g0.close()
    n = st["x"].shape[0]
    # pinned host copies of every array ndsph_step reads and writes
    pinned = {}
    for k, v in st.items():
        t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32, pin_memory=True)
        a = t.numpy()
        a[...] = v
        pinned[k] = (t, a)
    host = {k: a for k, (t, a) in pinned.items()}

    def timed(mode, drop):
        # mode 0 (the library default): staging copies on a copy stream,
        # overlapped with the layout kernels and, for outputs final before the
        # rates sweep, with the sweep; 1: the layout kernels read and write
        # the pinned arrays in place over the CPU-GPU link
        for k, (t, a) in pinned.items():
            a[...] = st[k]
        g = GpuSPH(o2, host)
        if drop:
            for k in INFO_ONLY:
                setattr(g._p, k, None)
        if tuning:
            g.set_tuning(**tuning)
        g.set_host_access(mode)
        g.set_dt(0.0)
        g.dt.dt, g.dt.time, g.dt.nsteps = 0.0, 0.0, 0
        for _ in range(warmup):
            g.step()
        torch.cuda.synchronize()
        # no Python garbage collection inside the timed loop (a collection of
        # the earlier legs' objects stalled single steps); each call returns
        # with its results in the host arrays, so the per-call times add up
        # to the loop's
        gc.collect()
        gc.disable()
        kept0 = g.timing()["nl_reused"]
        try:
            t0 = time.perf_counter()
            tk = [t0]
            its, relinks = [], []
            for _ in range(steps):
                g.step()
                tk.append(time.perf_counter())
                its.append(g.dt.its)
                relinks.append(g.dt.nrelink)
            torch.cuda.synchronize()
            r = n * steps / (time.perf_counter() - t0)
        finally:
            gc.enable()
        kept = g.timing()["nl_reused"] - kept0
        g.close()
        dts = sorted((b - a) * 1e3 for a, b in zip(tk, tk[1:]))
        step_ms = {"min": round(dts[0], 3), "median": round(statistics.median(dts), 3), "max": round(dts[-1], 3),
                   "calls_keeping_the_link": kept, "calls": steps,
                   "newton_raphson_passes": {str(k): its.count(k) for k in sorted(set(its))},
                   "calls_relinking_inside_the_iteration": sum(1 for x in relinks if x > 0)}
        return r, step_ms

    # bytes per particle: ndsph_step uploads the step's inputs x(3) v(3) Bevol(3)
    # en hh pmass alpha(3) dhdt force(3) dBevoldt(3) dendt daldt(3) + itype
    d_up = (3 + 3 + 3 + 1 + 1 + 1 + 3 + 1 + 3 + 3 + 1 + 3) * 8 + 4
    # integrator set: x v Bevol en hh alpha dhdt force dBevoldt dendt daldt
    d_dn_int = (3 + 3 + 3 + 1 + 1 + 3 + 1 + 3 + 3 + 1 + 3) * 8
    # every output: the above plus rho rhoalt drhodt gradh gradhn gradgradh,
    # dens uu pr spsound Bfield(3), dudt divB curlB(3) del2u graddivv(3) + numneigh
    d_dn_all = d_dn_int + (6 + 4 + 3 + 1 + 1 + 3 + 1 + 3) * 8 + 4
    ri, si = timed(0, True)
    ra, sa = timed(0, False)
    out = {"integrator": (ri, d_up * n, d_dn_int * n, si),
           "all": (ra, d_up * n, d_dn_all * n, sa)}
    return out, timed(1, False)[0]


def run_batched(steps: int, warmup: int, ntubes: int = 4096):
    """Batched form: 4096 independent 1D Brio-Wu tubes, 200-1600 particles
    each (seeded), one device state, per-tube dt; FP32 pair sums.  `steps`
    timed steps of the fused per-tube kernel (one launch per step, one block
    per tube), then the same problem as captured CUDA graphs of the per-kernel
    step (one graph launch per step, search settings from the autotuner) and
    on the eager host loop, for comparison."""
    from ndspmhd_gb300 import autotune, configs
    from ndspmhd_gb300.gpu import GpuSPH
    o, p, sim, counts = configs.brio_wu_batch(ntubes)
    o["precision"] = 1
    n = int(counts.sum())
    cands = [{"graph_cell_margin": m, "nl_skin": sk} for m in (1.02, 1.05, 1.1) for sk in (1.05, 1.1)]
    tuned = autotune.tune_batched(o, configs.full_state(p, 1), sim, len(counts), candidates=cands,
                                  steps=20, warmup=3)
    out = {}
    for mode, nst in ((1, steps), (2, max(steps // 4, 20)), (0, max(steps // 4, 5))):
        g = GpuSPH(o, configs.full_state(p, 1))
        g.set_tuning(**tuned["tuning"])
        g.batch_upload(sim, len(counts), initialise=True)
        g.batch_set_graph(mode)
        g.batch_step(warmup)
        g.batch_step(nst)
        tim = g.timing()
        ms = tim["total_ms"]
        g.close()
        out[mode] = {"value": round(n * nst / (ms * 1e-3), 1), "ms_per_step": round(ms / nst, 3), "steps": nst,
                     "launches_per_step": round(tim["launches"] / nst, 1),
                     "fused_steps": tim["fused_steps"], "graph_steps": tim["graph_steps"],
                     "graph_redos": tim["graph_redos"]}
    res = dict(out[1])
    res.update({"unit": UNIT, "config": f"{ntubes} Brio-Wu tubes, {n} particles, FP32 pairs, per-tube dt, "
                                        f"one fused launch per step (one block per tube)",
                "captured_graph": out[2], "eager": out[0], "graph_search_tuning": tuned["tuning"],
                "autotune_trials": [[t["tuning"], t["ms_per_step"]] for t in tuned["trials"]]})
    return res


def _fp32_vs_fp64(st0, o64, steps: int, tolh: float, timed_steps: int = 0):
    """The FP32 forms (reference predictor; learned h) against the FP64 form
    from the same FP64 state, `steps` device-resident steps each (each form
    takes its own dt); then, if timed_steps, that many more steps timed.  Per
    field: max |fp32 - fp64| / max(max |fp64|, rms fp64), and the 99.99th
    percentile of the same per-particle ratio."""
    import numpy as np
    from ndspmhd_gb300.gpu import GpuSPH
    fields = ("x", "vel", "hh", "rho", "en", "Bevol", "force", "dudt", "dBevoldt")
    forms = {"fp64": dict(precision=0, learned_h=0), "fp32": dict(precision=1, learned_h=0),
             "fp32_learned_h": dict(precision=1, learned_h=1)}
    out, ms = {}, {}
    for key, f in forms.items():
        g = GpuSPH(dict(o64, tolh=tolh, **f), {k: v.copy() for k, v in st0.items()})
        g.dev_upload()
        g.set_dt(0.0)
        g.dev_step(steps)
        g.dev_download()
        out[key] = {k: g.state[k].copy() for k in fields}
        if timed_steps:
            g.dev_step(timed_steps)
            ms[key] = g.timing()["total_ms"] / timed_steps
        g.close()
    res = {"steps": steps, "tolh": tolh}
    for key in ("fp32", "fp32_learned_h"):
        r = {}
        for k in fields:
            ref = out["fp64"][k]
            scale = max(float(np.max(np.abs(ref))), float(np.sqrt(np.mean(ref * ref))))
            d = np.abs(out[key][k] - ref)
            if d.ndim > 1:
                d = d.max(axis=1)
            r[k] = float(d.max() / scale) if scale > 0 else 0.0
            r[k + "_p9999"] = float(np.quantile(d, 0.9999) / scale) if scale > 0 else 0.0
        # particles whose h differs by more than 1e-5 relative: those whose
        # Newton-Raphson residual sat at the tolerance and converged one pass
        # apart (or, with learned h, from another starting point)
        dh = np.abs(out[key]["hh"] - out["fp64"]["hh"]) / out["fp64"]["hh"]
        r["particles_h_differ_1e-5"] = int(np.sum(dh > 1e-5))
        res[key] = r
    if ms:
        res["ms_per_step"] = {k: round(v, 3) for k, v in ms.items()}
        res["ms_per_step"]["timed_steps"] = timed_steps
        res["ms_per_step"]["speedup_fp32_over_fp64"] = round(ms["fp64"] / ms["fp32"], 2)
        res["ms_per_step"]["speedup_fp32_learned_h_over_fp64"] = round(ms["fp64"] / ms["fp32_learned_h"], 2)
    return res


def fp32_error(steps: int = 4):
    """Error of the FP32 forms against the FP64 (parity) form on the headline
    workload, at two Newton-Raphson tolerances (the same in every form):

    * tolh 1e-3, the headline's: a particle whose residual sits within the
      FP32 form's ~5e-7 density error of the tolerance converges one pass
      apart in the two forms (with learned h the starting point differs as
      well), and its h then differs by up to ~tolh; the max error is set by
      those few particles (counted) and their neighbours, the 99.99th
      percentile by the arithmetic;
    * tolh 1e-6: the decisions agree closely enough that the error is the
      arithmetic's own (<= 1e-5); the forms are also timed there, so the
      FP32/FP64 speed ratio is quoted at a tolerance where that bound holds.
    """
    o64, st64 = make_problem(N1D, 0)
    g = init_state(o64, st64)
    st0 = {k: v.copy() for k, v in g.state.items()}
    g.close()
    return {"metric": "max |fp32 - fp64| / max(max |fp64|, rms fp64), per field (and its 99.99th percentile)",
            "at_headline_tolh": _fp32_vs_fp64(st0, o64, steps, 1e-3),
            "at_tolh_1e-6": _fp32_vs_fp64(st0, o64, steps, 1e-6, timed_steps=4)}


def run_learned(n1d: int, steps: int, warmup: int):
    """Learned-h workload: isothermal log-normal turbulent box, tolh = 1e-4,
    FP32 pairs; NR density work and step rate with the reference's predictor
    vs the learned predictor (trained online from step 0)."""
    from ndspmhd_gb300 import autotune, configs
    from ndspmhd_gb300.gpu import GpuSPH
    out = {}
    o, p = configs.turbulent_box_3d(n1d)
    # search settings from the autotuner on this workload (reference predictor),
    # the same for both runs
    g = GpuSPH(dict(o, precision=1, learned_h=0), configs.full_state(p, 3))
    g.primitive2conservative()
    st0 = {k: v.copy() for k, v in g.state.items()}
    g.close()
    tuned = autotune.tune_device(dict(o, precision=1, learned_h=0), st0, steps=6, warmup=3)
    for learned in (0, 1):
        o2 = dict(o)
        o2["precision"] = 1
        o2["learned_h"] = learned
        g = GpuSPH(o2, configs.full_state(p, 3))
        g.set_tuning(**tuned["tuning"])
        g.primitive2conservative()
        g.dev_upload()
        g.set_dt(0.0)
        g.dev_step(warmup)
        work, passes = [], []
        tot = 0.0
        for _ in range(steps):
            g.dev_step(1)
            d = g.dts()
            work.append(d["ncalctotal"] / g.n)
            passes.append(d["its"])
            tot += g.timing()["total_ms"]
        key = "learned" if learned else "predictor"
        out[key] = {"particle_passes_per_step": round(sum(work) / len(work), 4),
                    "nr_passes_per_step": round(sum(passes) / len(passes), 3),
                    "value": round(g.n * steps / (tot * 1e-3), 1), "ms_per_step": round(tot / steps, 3)}
        g.close()
    out["config"] = f"isothermal turbulent box {n1d}^3, tolh 1e-4, FP32 pairs, {warmup} warm-up steps then {steps} timed"
    out["search_tuning"] = tuned["tuning"]
    out["work_reduction"] = round(1 - out["learned"]["particle_passes_per_step"] /
                                  out["predictor"]["particle_passes_per_step"], 4)
    return out


def run_ot2d(steps: int = 50, cpu_steps: int = 10):
    """The reference's own CPU case: the 2D Orszag-Tang vortex, 256 x 296
    particles on the close-packed lattice, FP64, 50 leapfrog steps from the
    initial conditions (plus the FP32 form), and the 1-core oracle on the
    first `cpu_steps` steps of the same run."""
    from ndspmhd_gb300 import configs
    from ndspmhd_gb300.gpu import GpuSPH
    from oracle.oracle import Oracle
    o, p = configs.orszag_tang_2d(256)
    n = p["x"].shape[0]
    out = {"config": f"2D Orszag-Tang, {n} particles (256 x 296 hcp), periodic, {steps} leapfrog steps"}
    for prec, key in ((0, "fp64"), (1, "fp32")):
        o2 = dict(o, precision=prec)
        g = GpuSPH(o2, configs.full_state(p, 2))
        g.primitive2conservative()
        g.dev_upload()
        g.set_dt(0.0)
        g.dev_step(steps)
        ms = g.timing()["total_ms"]
        d = g.dts()
        g.close()
        out[key] = {"value": round(n * steps / (ms * 1e-3), 1), "ms_per_step": round(ms / steps, 3),
                    "time_reached": d["time"]}
    orc = Oracle(o, configs.full_state(p, 2))
    orc.primitive2conservative()
    orc.set_dt(0.0, 0.0)
    t0 = time.perf_counter()
    orc.step(cpu_steps)
    el = time.perf_counter() - t0
    out["cpu_oracle_1core"] = {"value": round(n * cpu_steps / el, 1), "sample": f"first {cpu_steps} steps, {el:.1f} s"}
    return out


def run_dust(n1d: int, steps: int, warmup: int, nset: int = 8, serial: bool = True):
    """Two-fluid dust + gas MHD box (2 x n1d^3, periodic), a batch of `nset`
    (dust-to-gas ratio, stopping time) settings in one device state: each
    setting keeps its own periodic box, drag constant K, dt and clock
    (ndsph_batch_upload with periodic boundaries, ndsph_batch_set_kdrag).
    FP32 pair sums, FP64 integration.  `serial` also times the settings one
    after another in their own contexts, for comparison."""
    import numpy as np
    from ndspmhd_gb300 import autotune, configs
    from ndspmhd_gb300.gpu import GpuSPH
    rng = np.random.default_rng(99)
    eps = np.exp(rng.uniform(np.log(0.01), np.log(1.0), nset))
    ts = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), nset))
    runs = [configs.dust_gas_box_3d(n1d, eps=float(eps[k]), tstop=float(ts[k]), seed=77 + k) for k in range(nset)]
    o0 = dict(runs[0][0], precision=1)
    # search settings tuned on the first setting alone, kept for the batch
    g = GpuSPH(o0, configs.full_state(runs[0][1], 3))
    g.primitive2conservative()
    st0 = {kk: v.copy() for kk, v in g.state.items()}
    g.close()
    tuning = autotune.tune_device(o0, st0, steps=6, warmup=3)["tuning"]
    parts = [p for _, p in runs]
    cat = {k: np.concatenate([q[k] for q in parts], axis=0) for k in parts[0]}
    sim = np.concatenate([np.full(q["x"].shape[0], s, np.int32) for s, q in enumerate(parts)])
    kd = np.array([o["Kdrag"] for o, _ in runs])
    n = cat["x"].shape[0]
    g = GpuSPH(o0, configs.full_state(cat, 3))
    g.set_tuning(**tuning)
    g.batch_set_kdrag(kd)
    g.batch_upload(sim, nset, initialise=True)
    g.batch_step(warmup)
    _, t = g.batch_step(steps)
    tim = g.timing()
    ms = tim["total_ms"]
    g.close()
    out = {"value": round(n * steps / (ms * 1e-3), 1), "unit": UNIT,
           "ms_per_step": round(ms / steps, 3), "ms_per_step_per_setting": round(ms / (steps * nset), 3),
           "particles": n, "launches_per_step": round(tim["launches"] / steps, 1),
           "config": f"gas+dust box 2x{n1d}^3 x {nset} (eps, t_s) settings in one device state (periodic "
                     f"boxes side by side in the cell grid), eps in [0.01,1], t_s in [1e-3,1], FP32 pairs",
           "search_tuning": tuning, "time_range": [float(t.min()), float(t.max())]}
    if serial:
        tot_ms, tot_upd = 0.0, 0
        for o, p in runs:
            g = GpuSPH(dict(o, precision=1), configs.full_state(p, 3))
            g.set_tuning(**tuning)
            g.primitive2conservative()
            g.dev_upload()
            g.set_dt(0.0)
            g.dev_step(warmup)
            g.dev_step(steps)
            tot_ms += g.timing()["total_ms"]
            tot_upd += g.n * steps
            g.close()
        out["serial"] = {"value": round(tot_upd / (tot_ms * 1e-3), 1),
                         "ms_per_step_per_setting": round(tot_ms / (steps * nset), 3),
                         "form": "the same settings one after another, each in its own context"}
    return out


def cpu_baseline(n1d: int = CPU_SAMPLE_N1D, steps: int = CPU_SAMPLE_STEPS, warmup: int = 0) -> dict:
    """The oracle (single-threaded C restatement of the reference) on a
    bounded sample of the same workload: a n1d^3 box, `warmup` untimed then
    `steps` timed leapfrog steps."""
    from ndspmhd_gb300 import configs
    from oracle.oracle import Oracle
    o, p = configs.mhd_box_3d(n1d, seed=1234)
    orc = Oracle(o, configs.full_state(p, 3))
    orc.primitive2conservative()
    orc.set_dt(0.0, 0.0)
    if warmup > 0:
        orc.step(warmup)
    t0 = time.perf_counter()
    orc.step(steps)
    el = time.perf_counter() - t0
    n = n1d ** 3
    return {"value": n * steps / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n1d}^3 box ({n} particles), {steps} leapfrog steps, FP64 oracle, 1 thread, "
                      f"{el:.1f} s"}


def _cpu_worker(args):
    n1d, steps, warmup = args
    return cpu_baseline(n1d, steps, warmup)["value"]


def _cpu_tube_worker(args):
    """One host process: the oracle on each of its Brio-Wu tubes in turn,
    `warmup` untimed then `steps` timed steps from the initial conditions;
    returns (particle-updates, seconds in the timed steps)."""
    counts, steps, warmup = args
    from ndspmhd_gb300 import configs
    from oracle.oracle import Oracle
    upd, el = 0, 0.0
    for c in counts:
        o, p = configs.brio_wu_tube(int(c))
        orc = Oracle(o, configs.full_state(p, 1))
        orc.primitive2conservative()
        orc.set_dt(0.0, 0.0)
        if warmup > 0:
            orc.step(warmup)
        t0 = time.perf_counter()
        orc.step(steps)
        el += time.perf_counter() - t0
        upd += p["x"].shape[0] * steps
    return upd, el


def cpu_batched_baseline(counts, steps: int, warmup: int, ntubes: int = 1024) -> dict:
    """The batched workload on the host: the reference is serial, so the
    tubes are spread over all host cores as independent processes (spawned:
    the parent already holds a CUDA context).  Bounded sample: the first
    `ntubes` tubes of the same seeded batch, the same steps as the GPU run."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    sample = [int(c) for c in counts[:ntubes]]
    work = [(sample[w::cores], steps, warmup) for w in range(cores)]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_tube_worker, work)
    wall = time.perf_counter() - t0
    upd = sum(r[0] for r in res)
    el = max(r[1] for r in res)
    return {"value": round(upd / el, 1), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {len(sample)} tubes ({upd // steps} particles), {warmup} + {steps} steps each, "
                      f"FP64 oracle, {cores} processes, slowest process {el:.1f} s in the timed steps, "
                      f"wall {wall:.1f} s"}


def reference_arm(args):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle port; the Fortran reference cannot be built here) on all host
    cores as independent replicas of the bounded sample (the reference is
    serial, so one simulation per core)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    # every core runs its own replica of the sample: `warmup` untimed steps,
    # then `steps` timed ones (the reference is serial)
    steps = max(1, args.steps)
    warmup = max(0, args.warmup)
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        vals = pool.map(_cpu_worker, [(CPU_SAMPLE_N1D, steps, warmup)] * cores)
    el = time.perf_counter() - t0
    value = float(sum(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": warmup,
        "ms_per_step": 1e3 * (CPU_SAMPLE_N1D ** 3) / (value / cores) if value > 0 else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 3D MHD box)",
        "config": {"workload": f"3D MHD box, sample {CPU_SAMPLE_N1D}^3 per core", "n1d": CPU_SAMPLE_N1D,
                   "parallelism": f"{cores} independent serial replicas"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} x ({CPU_SAMPLE_N1D}^3 box, {warmup} + {steps} steps), wall {el:.1f} s"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form measurement")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and learned-h workloads")
    ap.add_argument("--only", choices=["batched", "dust", "learned", "ot2d"],
                    help="run one secondary workload alone and print its JSON (for profiling it)")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.only:
        import torch
        torch.cuda.set_device(0)
        if args.only == "batched":
            r = run_batched(args.steps, max(args.warmup, 3))
        elif args.only == "dust":
            r = run_dust(96 if N1D >= 128 else 32, args.steps, max(args.warmup, 3), serial=False)
        elif args.only == "learned":
            r = run_learned(min(N1D, 128), args.steps, 40)
        else:
            r = run_ot2d()
        print(json.dumps({"workload": args.only, **r}), flush=True)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist
    else:
        torch.cuda.set_device(0)
    warmup = max(args.warmup, 3)

    # CPU baseline first (before heavy GPU work; rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline()

    o32, st32 = make_problem(N1D, 1)
    n = st32["x"].shape[0]
    tuned = tune(o32, st32)
    tuning = tuned["tuning"]
    # the headline form: FP32 pairs + the learned h predictor in front of the
    # Newton-Raphson iteration (the form the metric names), then the same
    # workload with the reference's own predictor; same tolh, same search
    # settings (tuned on the reference predictor)
    o32l = dict(o32, learned_h=1)
    ms32, tim32, dts32, clocks = run_device(o32l, st32, args.steps, warmup, dist, tuning)
    msp, timp, dtsp, _ = run_device(o32, st32, args.steps, warmup, dist, tuning)
    # the host-buffer step next, before the FP64 form (whose seconds of FP64
    # sweeps were followed by slower first e2e calls in some runs), with the
    # clocks sampled over it
    clk_e2e = ClockSampler(torch.cuda.current_device())
    clk_e2e.start()
    clk_e2e.wait_first()
    e2e_sets, e2e_inplace = run_e2e(o32l, max(3, args.steps), 3, tuning)
    clocks_e2e = clk_e2e.stop()
    e2e_val, h2d, d2h, e2e_step_ms = e2e_sets["integrator"]
    ms64 = tim64 = None
    if not args.no_fp64:
        o64, st64 = make_problem(N1D, 0)
        ms64, tim64, _, _ = run_device(o64, st64, max(2, args.steps // 2), 3, dist)

    # max over ranks
    ms32 = max_over_ranks(ms32, dist, "cuda")
    value = replica_value(n, world, ms32)

    peak, peak_kind = _load_peaks()
    rates_ms = tim32["rates_ms"]
    achieved = RATES_BYTES_PER_PARTICLE * n / (rates_ms * 1e-3) / 1e9 if rates_ms > 0 else 0.0
    # DRAM bytes of one k_rates<3,FP32> launch from an ncu capture of the 64^3 box
    # (129.8 MB read + 18.8 MB written), scaled by the particle count
    traffic = round(RATES_DRAM_BYTES_64 * n / 64 ** 3)
    # the sweep's issue rate, live: warp instructions of one launch (the 64^3
    # capture scaled by N) over the slots of 152 SMs x 4 schedulers at the
    # clock sampled during the timed steps
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    warp_instr = RATES_WARP_INSTR_64 * n / 64 ** 3
    issue_frac = warp_instr / (rates_ms * 1e-3 * SMS * SMSP_PER_SM * sm_mhz * 1e6) if rates_ms > 0 else 0.0
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic, "traffic_note": "ncu dram bytes of the 64^3 launch x N/64^3",
                "kernel": "k_rates<3,FP32> (rates sweep)",
                "issue_view": dict(RATES_NCU_64, **{
                    "issue_frac_live": round(issue_frac, 4),
                    "issue_note": "the sweep is bound by FP32 instruction issue: issue_frac_live = warp instructions "
                                  "per launch / (rates time x 152 SMs x 4 schedulers x SM clock); the other "
                                  "figures from ncu --set full of the 64^3 launch"}),
                "note": f"peak of {peak_kind} (MEASURED_PEAKS.json hbm_gbs); algorithmic bytes "
                        f"{RATES_BYTES_PER_PARTICLE} B/particle x {n}; the sweep is FP32-issue bound"}
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": round(ms32, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pairs / f64 state",
        "data": "synthetic (seeded jittered 128^3 MHD box, generated in-process)",
        "config": {"workload": f"3D MHD box {N1D}^3 = {n} particles, periodic, full leapfrog step",
                   "form": "FP32 pair sums (compensated), FP64 state/integration, learned h predictor "
                           "(MLP, trained online) in front of the Newton-Raphson iteration at tolh 1e-3",
                   "l2": "inputs larger than L2 (state slab ~1.3 GB)", "parallelism": f"replicas x{world}",
                   "nr_passes_per_step": tim32["density_passes"],
                   "steps_keeping_the_link": tim32["kept_link_steps"], "row_builds": tim32["row_builds"],
                   "search_tuning": tuning,
                   "autotune_trials": [[t["tuning"], t["ms_per_step"]] for t in tuned["trials"]]},
        "gpu_launches": None,
        "kernels_ms_per_step": {"rates": round(tim32["rates_ms"], 3), "density_all_passes": round(tim32["density_ms"], 3),
                                "link": round(tim32["link_ms"], 3), "mlp": round(tim32["mlp_ms"], 3),
                                "step_total": round(tim32["step_ms"], 3)},
        "particle_passes_last_step": round(dts32["ncalctotal"] / n, 4),
        "roofline": roofline,
        "clocks": clocks,
        "e2e": {"value": round(e2e_val, 1), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "call": "ndsph_step with pinned host buffers (staging copies overlapped with the kernels), "
                        "returning the integrator's arrays (x, vel, Bevol, en, hh, alpha and their rates) as "
                        "the Fortran shim's gpu_step does between output steps",
                "step_ms": dict(e2e_step_ms, note="host wall time of each call; the link is kept on every "
                                                  "other step and rebuilt on the others"),
                "clocks": clocks_e2e,
                "all_outputs": {"value": round(e2e_sets["all"][0], 1), "h2d_bytes_per_step": e2e_sets["all"][1],
                                "d2h_bytes_per_step": e2e_sets["all"][2], "step_ms": e2e_sets["all"][3],
                                "call": "the same, returning all 47.5 doubles a particle (output steps)"},
                "in_place_access_value": round(e2e_inplace, 1)},
    }
    msp = max_over_ranks(msp, dist, "cuda")
    line["fp32_predictor"] = {
        "value": round(replica_value(n, world, msp), 1), "ms_per_step": round(msp, 4),
        "form": "FP32 pairs with the reference's predictor h + dt dh/dt (stepND_leapfrog_mhd.f90:152-153)",
        "particle_passes_last_step": round(dtsp["ncalctotal"] / n, 4), "nr_passes_last_step": dtsp["its"],
        "kernels_ms_per_step": {"rates": round(timp["rates_ms"], 3), "density_all_passes": round(timp["density_ms"], 3),
                                "link": round(timp["link_ms"], 3), "step_total": round(timp["step_ms"], 3)},
        "learned_speedup": round(msp / ms32, 4)}
    if ms64 is not None:
        line["fp64"] = {"value": round(n / (ms64 * 1e-3), 1), "ms_per_step": round(ms64, 3),
                        "rates_ms": round(tim64["rates_ms"], 3), "density_ms": round(tim64["density_ms"], 3),
                        "speedup_fp32_over_fp64": round(ms64 / ms32, 2)}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if not args.no_fp64 and world == 1:
        line["fp32_error_vs_fp64"] = fp32_error()
    if not args.no_extra and world == 1:
        line["batched"] = run_batched(200, 3)
        if not args.no_cpu:
            from ndspmhd_gb300 import configs
            line["batched"]["cpu_baseline"] = cpu_batched_baseline(configs.brio_wu_batch(4096)[3], 200, 3)
        line["learned_h"] = run_learned(min(N1D, 128), 20, 40)
        line["dust"] = run_dust(96 if N1D >= 128 else 32, 5, 3)
        line["orszag_tang_2d"] = run_ot2d()
    # kernel launches the library issued inside the timed step loop (counted
    # at every launch site)
    line["gpu_launches"] = tim32["launches_timed"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
