"""The reference's run-time options file (``<run>.in``) and its sweep driver.

Format (utils_infiles.f90:83-283, read_infile readwrite_infile.f90:130-290):
one ``name = value   ! description`` per line, ``#`` comment lines, blank
lines; reals in any Fortran form (``1.0``, ``1.e-3``, ``1.0d0``), logicals as
``T``/``F``.  Options not in the file keep the defaults of defaults.f90.

``read_infile`` maps the file onto this library's option dict (the fields of
``ndsph_opts``); ``write_infile`` writes one back in the reference's layout.
``run_sweep`` is the batched replacement of running one simulation per input
file (ndspmhd.f90:312-359, multi/multirun.f90, scripts/domulti.pl): input files
with identical hot-path options go into one batched launch.
"""
from __future__ import annotations

import re

from .configs import default_opts

# names of the reference's options that map onto ndsph_opts fields
_MAP = {
    "psep": "psep", "C_cour": "C_cour", "C_force": "C_force", "maxdensits": "maxdensits",
    "hfact": "hfact", "tolh": "tolh", "iener": "iener", "gamma": "gamma", "polyk": "polyk",
    "iav": "iav", "alphamin": "alphamin", "alphaumin": "alphaumin", "alphaBmin": "alphaBmin",
    "beta": "beta", "avdecayconst": "avdecayconst", "imhd": "imhd", "imagforce": "imagforce",
    "idust": "idust", "idrag_nature": "idrag_nature", "Kdrag": "Kdrag",
}
# options the hot path implements only at their default value (defaults.f90)
_FIXED = {
    "icty": 0, "ihvar": 2, "ikernel": 0, "ikernav": 3, "iprterm": 0, "idivbzero": 0, "iresist": 0,
    "igravity": 0, "ixsph": 0, "iexternal_force": 0, "iambipolar": 0, "iuse_exact_derivs": 0,
    "ind_timesteps": 0, "damp": 0.0, "iquantum": 0, "usenumdens": False, "ibiascorrection": 0,
}
_ORDER = [
    ("# options affecting setup", [("psep", "particle separation")]),
    ("# options affecting timestepping/output", [("C_cour", "Courant factor on timestep"),
                                                 ("C_force", "Factor in force timestep condition")]),
    ("# options affecting density calculation", [("maxdensits", "maximum number of density iterations"),
                                                 ("hfact", "h in units of mean particle spacing"),
                                                 ("tolh", "tolerance on h-rho iterations")]),
    ("# options affecting equation of state, energy equation", [("iener", "type of energy equation"),
                                                               ("gamma", "adiabatic index"),
                                                               ("polyk", "polytropic constant if iener=0")]),
    ("# options affecting momentum equation and shock-capturing terms",
     [("iav", "type of artificial viscosity"), ("alphamin", "minimum alpha (viscosity)"),
      ("alphaumin", "minimum alphau (conductivity)"), ("alphaBmin", "minimum alphaB (resistivity)"),
      ("beta", "beta in artificial viscosity"), ("iavlim", "use viscosity switch"),
      ("iavlimu", "use conductivity switch"), ("iavlimB", "use resistivity switch"),
      ("avdecayconst", "decay constant in av switch (0.1-0.2)")]),
    ("# options affecting magnetic fields", [("imhd", "MHD (0:no 1-10:B/rho >10:B <0:A -3:GEPs)"),
                                             ("imagforce", "MHD force type(1:vector 2:tensor)")]),
    ("# options affecting dust", [("idust", "dust (0:off 1:one-f 2:two-f)"),
                                  ("idrag_nature", "drag type (0=none 1=const K 2=const ts 3=Epstein)"),
                                  ("Kdrag", "drag coefficient")]),
]


def _parse_value(v: str):
    v = v.strip()
    if v.upper() in ("T", ".TRUE.", "TRUE"):
        return True
    if v.upper() in ("F", ".FALSE.", "FALSE"):
        return False
    if re.fullmatch(r"[+-]?\d+", v):
        return int(v)
    try:
        return float(v.lower().replace("d", "e"))
    except ValueError:
        return v


def parse_infile(text: str) -> dict:
    """All ``name = value`` pairs of an input file (later entries win)."""
    out = {}
    for line in text.splitlines():
        s = line.split("!", 1)[0].strip()
        if not s or s.startswith("#") or "=" not in s:
            continue
        name, val = s.split("=", 1)
        out[name.strip()] = _parse_value(val)
    return out


def read_infile(path: str, ndim: int, base: dict | None = None) -> dict:
    """Options of ``path`` on top of the reference defaults (or ``base``).

    Raises ValueError for options the GPU path implements only at their
    default (e.g. icty /= 0): running them there would silently differ."""
    with open(path) as f:
        raw = parse_infile(f.read())
    o = dict(base) if base is not None else default_opts(ndim)
    for name, val in raw.items():
        if name in _MAP:
            o[_MAP[name]] = val
        elif name in ("iavlim", "iavlimu", "iavlimB"):
            lim = list(o["iavlim"])
            lim[{"iavlim": 0, "iavlimu": 1, "iavlimB": 2}[name]] = int(val)
            o["iavlim"] = lim
        elif name in _FIXED and val != _FIXED[name]:
            raise ValueError(f"{path}: {name} = {val} is outside the options the GPU path implements")
    return o


def _strip_zeros(s: str, keep: int) -> str:
    dot = s.rfind(".")
    if dot < 0:
        return s
    end = len(s)
    while end > dot + keep + 1 and s[end - 1] == "0":
        end -= 1
    return s[:end]


def _fmt_real(v: float) -> str:
    """write_inopt_real8 (utils_infiles.f90:210-237): es10.3 outside
    [1e-3, 1e4), else 9-13 significant digits with trailing zeros stripped."""
    a = abs(v)
    if (a < 1.0e-3 and a > 0.0) or a >= 1.0e4:
        m, e = f"{v:.3e}".split("e")
        return f"{m}E{int(e):+03d}".rjust(10)
    if a < 1.0e-1:
        s = _strip_zeros(f"{v:.13f}", 3)
    else:
        whole = len(str(int(a))) if a >= 1.0 else 0
        s = _strip_zeros(f"{v:.{max(9 - whole, 0) if a >= 1.0 else 9}f}", 0 if a >= 10.0 else 3)
    return s.rjust(10) if len(s) <= 10 else s


def _fmt(val) -> str:
    if isinstance(val, bool):
        return f"{'T' if val else 'F':>10s}"
    if isinstance(val, int):
        return f"{val:10d}"
    return _fmt_real(float(val))


def write_infile(path: str, opts: dict) -> None:
    """Write the hot-path options in the reference's layout (write_inopt)."""
    lines = ["# input file for ndspmhd, options not present assume default values"]
    for header, items in _ORDER:
        lines.append("")
        lines.append(header)
        for name, desc in items:
            if name.startswith("iavlim"):
                val = int(opts["iavlim"][{"iavlim": 0, "iavlimu": 1, "iavlimB": 2}[name]])
            else:
                val = opts[_MAP[name]]
            lines.append(f"{name:>20s} =  {_fmt(val)}    ! {desc}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _key(o: dict) -> tuple:
    # psep and the drag constant may differ inside a batch (the drag
    # constant goes per simulation)
    return tuple((k, tuple(v) if isinstance(v, list) else v) for k, v in sorted(o.items())
                 if k not in ("psep", "Kdrag"))


def run_sweep(runs, nsteps: int, precision: int = 1):
    """Run ``runs`` = [(opts, particles), ...] (open or fixed boundaries, or
    periodic in every dimension): runs whose hot-path options agree (psep and
    the drag constant K aside) share one batched launch, each with its own K.
    Returns the final particle dicts and per-run (time, dt), in input order."""
    import numpy as np
    from .configs import full_state
    from .gpu import GpuSPH
    groups: dict = {}
    for k, (o, p) in enumerate(runs):
        groups.setdefault(_key(o), []).append(k)
    results = [None] * len(runs)
    for _, idx in groups.items():
        o0 = dict(runs[idx[0]][0])
        o0["precision"] = precision
        o0["psep"] = max(runs[k][0]["psep"] for k in idx)
        parts, sims, counts = [], [], []
        start = 0
        for s, k in enumerate(idx):
            p = dict(runs[k][1])
            n = p["x"].shape[0]
            p["ireal"] = np.where(p["ireal"] > 0, p["ireal"] + start, 0).astype(np.int32)
            parts.append(p)
            sims.append(np.full(n, s, np.int32))
            counts.append(n)
            start += n
        cat = {f: np.concatenate([q[f] for q in parts], axis=0) for f in parts[0]}
        g = GpuSPH(o0, full_state(cat, o0["ndim"]))
        g.batch_set_kdrag([runs[k][0].get("Kdrag", 0.0) for k in idx])
        g.batch_upload(np.concatenate(sims), len(idx), initialise=True)
        dt, t = g.batch_step(nsteps)
        g.batch_download()
        start = 0
        for s, k in enumerate(idx):
            c = counts[s]
            results[k] = ({f: v[start:start + c].copy() for f, v in g.state.items()}, float(t[s]), float(dt[s]))
            start += c
        g.close()
    return results
