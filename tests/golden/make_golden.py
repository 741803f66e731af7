"""Generates the golden fixtures of tests/golden/ from the CPU oracle.

The reference (serial Fortran 90) ships no tests, fixtures or stored outputs
and cannot be compiled on these machines (no Fortran compiler), so its own
outputs cannot be captured.  These fixtures freeze the oracle's outputs -- the
oracle restates the reference routines and is itself pinned by the analytic
invariants of tests/test_cpu_oracle.py -- on small seeded particle sets, so
that

* tests/test_cpu_golden.py re-runs the oracle and must reproduce them (any
  change of the restatement shows up as a fixture mismatch), and
* tests/test_gpu_golden.py runs the CUDA path from the same start arrays and
  compares with the stored outputs, with no oracle in the loop.

Each fixture ``<case>.npz`` holds

* ``opts`` (JSON text): the options the runs use (polyk as set by
  primitive2conservative);
* ``start/<field>``: the state after primitive2conservative (the input of
  both runs);
* ``derivs/<field>``: outputs of one derivs (link, iterate_density,
  conservative2primitive, get_rates) from the start state, plus
  ``derivs/dts`` (dtcourant, dtforce, dtav, dtdrag, vsigmax, stressmax, its);
* ``steps/<field>``: the state after NSTEPS leapfrog steps from the start state
  with dt = 0 on the first step, plus ``steps/dt``.

Usage:  python tests/golden/make_golden.py      (rewrites every fixture)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NSTEPS = 3
START_FIELDS = ["x", "vel", "Bevol", "en", "hh", "pmass", "alpha", "itype", "ireal", "rho", "rhoalt",
                "drhodt", "dhdt", "gradh", "gradhn", "gradgradh", "numneigh", "dens", "uu", "pr", "spsound",
                "Bfield", "force", "dBevoldt", "dudt", "dendt", "daldt", "divB", "curlB", "del2u", "graddivv"]
DERIVS_FIELDS = ["rho", "hh", "gradh", "gradhn", "gradgradh", "drhodt", "dhdt", "rhoalt", "numneigh", "pr",
                 "spsound", "Bfield", "force", "dBevoldt", "dudt", "dendt", "daldt", "divB", "curlB", "del2u",
                 "graddivv"]
STEP_FIELDS = ["x", "vel", "Bevol", "en", "hh", "rho", "alpha", "force", "dudt"]
DT_KEYS = ["dtcourant", "dtforce", "dtav", "dtdrag", "vsigmax", "stressmax", "its"]


def cases() -> dict:
    from ndspmhd_gb300 import configs
    return {
        "ot2d_16": lambda: configs.orszag_tang_2d(16),
        "box3d_8": lambda: configs.mhd_box_3d(8, seed=7),
        "box3d_B_8": lambda: configs.mhd_box_3d(8, seed=8, imhd=11),
        "briowu_200": lambda: configs.brio_wu_tube(200),
        "dust3d_8": lambda: configs.dust_gas_box_3d(8, eps=0.3, tstop=0.02),
        "isothermal_10": lambda: configs.turbulent_box_3d(10),
    }


def make_case(name: str) -> dict:
    from ndspmhd_gb300 import configs
    from oracle.oracle import Oracle
    o, p = cases()[name]()
    orc = Oracle(o, configs.full_state(p, o["ndim"]))
    orc.primitive2conservative()
    o = dict(o)
    o["polyk"] = orc.opts["polyk"]
    start = orc.snapshot()
    out = {"opts": np.array(json.dumps(o))}
    for k in START_FIELDS:
        out[f"start/{k}"] = start[k]
    ref = Oracle(o, start)
    ref.derivs()
    d = ref.dts()
    for k in DERIVS_FIELDS:
        out[f"derivs/{k}"] = ref.state[k]
    out["derivs/dts"] = np.array([float(d[k]) for k in DT_KEYS])
    ref = Oracle(o, start)
    ref.set_dt(0.0, 0.0)
    ref.step(NSTEPS)
    for k in STEP_FIELDS:
        out[f"steps/{k}"] = ref.state[k]
    out["steps/dt"] = np.array([float(ref.dts()["dt"])])
    return out


def load(name: str) -> tuple[dict, dict]:
    """(opts, arrays) of a committed fixture."""
    with np.load(os.path.join(HERE, f"{name}.npz")) as z:
        arrays = {k: z[k] for k in z.files}
    return json.loads(str(arrays.pop("opts"))), arrays


def section(arrays: dict, prefix: str) -> dict:
    p = prefix + "/"
    return {k[len(p):]: v.copy() for k, v in arrays.items() if k.startswith(p)}


def main():
    for name in cases():
        out = make_case(name)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path)} bytes, n = {out['start/x'].shape[0]}")


if __name__ == "__main__":
    main()
