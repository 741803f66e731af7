"""Shared comparison helpers for the parity tests."""
import numpy as np


def field_scales(st: dict) -> dict:
    """Physical magnitude of each field, used as the floor of the relative
    error's denominator.  Near-uniform or divergence-free flows make drhodt,
    net forces, div B ... small residuals (down to round-off) of pair sums
    whose terms are of these sizes; an error measured against the residual
    alone would be noise against noise."""
    rho = float(np.mean(np.abs(st["rho"]))) or 1.0
    h = float(np.mean(st["hh"]))
    cs = float(np.sqrt(np.mean(st["spsound"] ** 2))) if "spsound" in st else 0.0
    vrms = float(np.sqrt(np.mean((st["vel"] ** 2).sum(1))))
    v = max(vrms, cs, 1e-30)
    B = float(np.sqrt(np.mean((st["Bfield"] ** 2).sum(1)))) if "Bfield" in st else 0.0
    B = max(B, 1e-30)
    u = float(np.mean(np.abs(st["uu"]))) if "uu" in st else 0.0
    return {
        "rho": rho, "rhoalt": float(np.mean(np.abs(st["rhoalt"]))) or 1.0, "hh": h,
        "gradh": 1.0, "gradhn": float(np.mean(np.abs(st["gradhn"]))) or 1.0,
        "gradgradh": float(np.mean(np.abs(st["gradgradh"]))) or 1.0,
        "drhodt": rho * v / h, "dhdt": v, "force": v * v / h, "dudt": v ** 3 / h, "dendt": v ** 3 / h,
        "dBevoldt": B * v / h / min(rho, 1.0), "divB": B / h, "curlB": B / h, "daldt": v / h,
        "del2u": max(u, v * v) / (h * h), "graddivv": v / h, "pr": 0.0, "spsound": 0.0, "Bfield": 0.0,
        "x": 1.0, "vel": v, "en": max(u, 1e-30), "Bevol": B / min(rho, 1.0), "alpha": 1.0,
    }


def field_err(got: np.ndarray, ref: np.ndarray, floor: float = 0.0) -> float:
    """max |got - ref| / max(|ref|, rms(ref), floor) over particles and components."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if not ref.size:
        return 0.0
    rms = float(np.sqrt(np.mean(ref ** 2)))
    den = np.maximum(np.abs(ref), max(rms, floor))
    den = np.where(den > 0, den, 1.0)
    return float(np.max(np.abs(got - ref) / den))


def compare_fields(got: dict, ref: dict, names, tol: float):
    sc = field_scales(ref)
    errs = {k: field_err(got[k], ref[k], sc.get(k, 0.0)) for k in names}
    bad = {k: v for k, v in errs.items() if not (v <= tol)}
    return errs, bad


def csr_sets(offs, neigh):
    return [np.sort(neigh[offs[i]:offs[i + 1]]) for i in range(len(offs) - 1)]
