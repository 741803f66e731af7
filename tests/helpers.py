"""Shared comparison helpers for the parity tests."""
import numpy as np


def field_err(got: np.ndarray, ref: np.ndarray) -> float:
    """max |got - ref| / max(|ref|, rms(ref)) over particles (and components).

    Near-uniform boxes make net forces small residuals of large pair terms, so
    a plain relative error is ill-defined near zero; the field's RMS is the
    floor of the denominator."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    rms = float(np.sqrt(np.mean(ref ** 2))) if ref.size else 0.0
    den = np.maximum(np.abs(ref), rms)
    den = np.where(den > 0, den, 1.0)
    return float(np.max(np.abs(got - ref) / den)) if ref.size else 0.0


def compare_fields(got: dict, ref: dict, names, tol: float):
    errs = {k: field_err(got[k], ref[k]) for k in names}
    bad = {k: v for k, v in errs.items() if not (v <= tol)}
    return errs, bad


def csr_sets(offs, neigh):
    return [np.sort(neigh[offs[i]:offs[i + 1]]) for i in range(len(offs) - 1)]
