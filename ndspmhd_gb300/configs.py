"""Synthetic particle sets for the NDSPMHD hot-path workloads.

The reference sets its problems up in Fortran setup routines; these generators
restate the ones the workloads need, in numpy, so that the GPU path and the CPU
oracle start from bit-identical particle arrays:

* ``orszag_tang_2d``  -- non-symmetric branch of setup_orszagtang2D_mhd.f90:55-200
  on the close-packed lattice of set_uniform_distributionND.f90:122-330
  (``idist=2``, ``fill`` default), in a periodic [-0.5,0.5]^2 box.
* ``mhd_box_3d``       -- the 128^3 jittered periodic MHD box (seeded).
* ``brio_wu_tube``     -- one 1D Brio-Wu tube with equal masses (spacing ~ 1/rho)
  and 6 fixed particles per end (setup_shock1DND_mhd2.f90:60-215,
  set_fixedbound.f90:43-56).
* ``turbulent_box_3d`` -- isothermal log-normal density box for the learned-h
  workload (seeded Gaussian random fields).
* ``dust_gas_box_3d``  -- interleaved gas/dust lattices (two-fluid drag).

Every generator returns ``(opts_dict, particles)`` where ``particles`` maps the
reference's array names to numpy arrays in Fortran module layout: ``x`` is
``(n, ndim)``, vectors are ``(n, 3)``, scalars ``(n,)``; ``itype``/``ireal`` are
int32 (``ireal`` 1-based, 0 = none).  Inputs are ``x, vel, pmass, itype, ireal,
dens, uu, Bfield, alpha`` (the primitive variables a setup produces).
"""
from __future__ import annotations

import math
import numpy as np

ITYPE_GAS, ITYPE_BND, ITYPE_DUST = 0, 1, 2


def default_opts(ndim: int) -> dict:
    """Reference defaults (defaults.f90:29-120) for the fields of ndsph_opts."""
    return dict(
        ndim=ndim, ibound=[0, 0, 0], xmin=[0.0, 0.0, 0.0], xmax=[1.0, 1.0, 1.0],
        hfact=1.2, tolh=1.0e-3, psep=0.01, maxdensits=250, imhd=0, imagforce=2,
        iener=2, iav=2, iavlim=[2, 1, 0], alphamin=0.1, alphaumin=0.0,
        alphaBmin=1.0, beta=2.0, avdecayconst=0.1, gamma=5.0 / 3.0, polyk=1.0,
        idust=0, idrag_nature=0, Kdrag=0.0, C_cour=0.3, C_force=0.25,
        precision=0, learned_h=0,
    )


def _empty(n: int, ndim: int) -> dict:
    return dict(
        x=np.zeros((n, ndim)), vel=np.zeros((n, 3)), pmass=np.zeros(n),
        itype=np.zeros(n, np.int32), ireal=np.zeros(n, np.int32),
        dens=np.zeros(n), uu=np.zeros(n), Bfield=np.zeros((n, 3)),
        alpha=np.zeros((n, 3)),
    )


def _set_alpha(p: dict, o: dict) -> None:
    # initialiseND_mhd.f90:243-245
    p["alpha"][:, 0] = o["alphamin"]
    p["alpha"][:, 1] = o["alphaumin"]
    p["alpha"][:, 2] = o["alphaBmin"]


def hcp_lattice_2d(psep: float, xmin, xmax, periodic_y: bool = True) -> np.ndarray:
    """Close-packed 2D lattice, set_uniform_distributionND.f90:122-330 (idist=2)."""
    deltax = psep
    deltay = 0.5 * math.sqrt(3.0) * psep
    fac = 1.0 - np.finfo(np.float64).eps
    npartx = int(fac * (xmax[0] - xmin[0]) / deltax) + 1
    nparty = int(fac * (xmax[1] - xmin[1]) / deltay) + 1
    if periodic_y:
        nparty = 2 * int(nparty / 2)
    # fill=.true. default: adjust deltas so the particles fill the box
    deltax = (xmax[0] - xmin[0]) / float(npartx)
    deltay = (xmax[1] - xmin[1]) / float(nparty)
    pts = np.empty((npartx * nparty, 2))
    k = 0
    for j in range(1, nparty + 1):
        ystart = deltay / 6.0
        xstart = 0.25 * deltax
        if j % 2 == 0:
            xstart = xstart + 0.5 * deltax
        i = np.arange(1, npartx + 1, dtype=np.float64)
        pts[k:k + npartx, 0] = xmin[0] + (i - 1) * deltax + xstart
        pts[k:k + npartx, 1] = xmin[1] + (j - 1) * deltay + ystart
        k += npartx
    return pts


def orszag_tang_2d(nx: int = 256) -> tuple[dict, dict]:
    """2D Orszag-Tang vortex: psep = 1/nx on a close-packed lattice.

    nx=256 gives 256 x 296 = 75,776 particles.  v = (-sin 2pi y', sin 2pi x'),
    B = (-sin 2pi y', sin 4pi x')/sqrt(4 pi), x' = x - xmin; rho = 25/(36 pi),
    P = 5/(12 pi), gamma = 5/3, equal masses.
    """
    o = default_opts(2)
    o.update(ibound=[3, 3, 0], xmin=[-0.5, -0.5, 0.0], xmax=[0.5, 0.5, 0.0],
             imhd=1, psep=1.0 / nx)
    pts = hcp_lattice_2d(1.0 / nx, o["xmin"], o["xmax"])
    n = len(pts)
    p = _empty(n, 2)
    p["x"][:] = pts
    const = 4.0 * math.pi
    betazero, machzero, vzero = 10.0 / 3.0, 1.0, 1.0
    bzero = 1.0 / math.sqrt(const)
    przero = 0.5 * bzero ** 2 * betazero
    denszero = o["gamma"] * przero * machzero
    uuzero = przero / ((o["gamma"] - 1.0) * denszero)
    totmass = denszero * 1.0
    xs = pts[:, 0] - o["xmin"][0]
    ys = pts[:, 1] - o["xmin"][1]
    p["vel"][:, 0] = -vzero * np.sin(2.0 * math.pi * ys)
    p["vel"][:, 1] = vzero * np.sin(2.0 * math.pi * xs)
    p["dens"][:] = denszero
    p["pmass"][:] = totmass / float(n)
    p["uu"][:] = uuzero
    p["Bfield"][:, 0] = -bzero * np.sin(2.0 * math.pi * ys)
    p["Bfield"][:, 1] = bzero * np.sin(4.0 * math.pi * xs)
    _set_alpha(p, o)
    return o, p


def mhd_box_3d(n1d: int = 128, seed: int = 1234, imhd: int = 1) -> tuple[dict, dict]:
    """3D periodic MHD box: n1d^3 particles on a cubic lattice in [0,1)^3.

    Positions (i+1/2)dx jittered by U(-0.1,0.1)dx; rho = 1 (equal masses);
    v_i ~ N(0, 0.1^2) iid per particle and component; B = (0.1, dBy, dBz) with
    a 1% transverse perturbation dBy = 0.001 cos(2 pi x + phi_y),
    dBz = 0.001 cos(2 pi x + phi_z) (divergence free, seeded phases);
    gamma = 5/3, u = 1.5 so that P = 1.
    """
    rng = np.random.default_rng(seed)
    o = default_opts(3)
    o.update(ibound=[3, 3, 3], xmin=[0.0, 0.0, 0.0], xmax=[1.0, 1.0, 1.0],
             imhd=imhd, psep=1.0 / n1d)
    dx = 1.0 / n1d
    g = (np.arange(n1d, dtype=np.float64) + 0.5) * dx
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    n = n1d ** 3
    p = _empty(n, 3)
    p["x"][:, 0] = xx.ravel()
    p["x"][:, 1] = yy.ravel()
    p["x"][:, 2] = zz.ravel()
    p["x"] += rng.uniform(-0.1, 0.1, size=(n, 3)) * dx
    p["vel"][:] = rng.normal(0.0, 0.1, size=(n, 3))
    phy, phz = rng.uniform(0.0, 2.0 * math.pi, size=2)
    p["Bfield"][:, 0] = 0.1
    p["Bfield"][:, 1] = 0.001 * np.cos(2.0 * math.pi * p["x"][:, 0] + phy)
    p["Bfield"][:, 2] = 0.001 * np.cos(2.0 * math.pi * p["x"][:, 0] + phz)
    p["dens"][:] = 1.0
    p["pmass"][:] = 1.0 / n
    p["uu"][:] = 1.0 / ((o["gamma"] - 1.0) * 1.0)
    _set_alpha(p, o)
    return o, p


def brio_wu_tube(npart: int, nbpts: int = 6, imhd: int = 1) -> tuple[dict, dict]:
    """One 1D Brio-Wu tube on [-0.5, 0.5] with equal masses.

    Left (rho, P, By) = (1, 1, 1), right (0.125, 0.1, -1), Bx = 0.75,
    gamma = 2.  Particle spacing ~ 1/rho: with n_R right particles the left
    holds 8 n_R, so npart is rounded to a multiple of 9.  The first and last
    ``nbpts`` particles are fixed (itype = 1) and copy their state from the
    first/last free particle (ireal, 1-based), as set_fixedbound.f90:43-56.
    """
    nR = max(npart // 9, 2)
    nL = 8 * nR
    n = nL + nR
    massp = 0.5 / nL
    psepL = massp / 1.0
    psepR = massp / 0.125
    o = default_opts(1)
    o.update(ibound=[1, 0, 0], xmin=[-0.5, 0.0, 0.0], xmax=[0.5, 0.0, 0.0],
             imhd=imhd, gamma=2.0, psep=psepR)
    p = _empty(n, 1)
    xl = -0.5 + (np.arange(nL) + 0.5) * psepL
    xr = 0.0 + (np.arange(nR) + 0.5) * psepR
    p["x"][:, 0] = np.concatenate([xl, xr])
    left = np.arange(n) < nL
    p["dens"][:] = np.where(left, 1.0, 0.125)
    pr = np.where(left, 1.0, 0.1)
    p["uu"][:] = pr / ((o["gamma"] - 1.0) * p["dens"])
    p["pmass"][:] = massp
    p["Bfield"][:, 0] = 0.75
    p["Bfield"][:, 1] = np.where(left, 1.0, -1.0)
    p["itype"][:nbpts] = ITYPE_BND
    p["itype"][n - nbpts:] = ITYPE_BND
    p["ireal"][:nbpts] = nbpts + 1
    p["ireal"][n - nbpts:] = n - nbpts
    _set_alpha(p, o)
    return o, p


def _gaussian_field(n1d: int, rng, kmin: float, kmax: float, slope: float) -> np.ndarray:
    """Real Gaussian random field on an n1d^3 grid with P(k) ~ k^slope in
    [kmin, kmax] (k in units of the box wavenumber), zero mean, unit variance."""
    k = np.fft.fftfreq(n1d, d=1.0 / n1d)
    kz, ky, kx = np.meshgrid(k, k, np.fft.rfftfreq(n1d, d=1.0 / n1d), indexing="ij")
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    amp = np.zeros_like(kk)
    band = (kk >= kmin) & (kk <= kmax)
    amp[band] = kk[band] ** (slope / 2.0)
    noise = rng.normal(size=kk.shape) + 1j * rng.normal(size=kk.shape)
    f = np.fft.irfftn(noise * amp, s=(n1d, n1d, n1d), axes=(0, 1, 2))
    f -= f.mean()
    s = f.std()
    return f / s if s > 0 else f


def turbulent_box_3d(n1d: int = 128, seed1: int = 11, seed2: int = 12,
                     sigma_lnrho: float = 1.0, mach: float = 2.0) -> tuple[dict, dict]:
    """Isothermal (gamma = 1.0001, iener = 0) log-normal density box.

    ln rho is a Gaussian random field (sigma = 1, P(k) ~ k^-2 for 2 <= k <= 32)
    imposed by mass-weighted lattice displacement: particles keep equal masses
    and are moved along the gradient of the displacement potential that maps
    the uniform lattice density onto rho (Zel'dovich-style, one step, so the
    realised field is an approximation of the target).  The velocity is a
    solenoidal Gaussian field (same band) scaled to rms Mach 2 with c_s = 1.
    """
    rng1 = np.random.default_rng(seed1)
    rng2 = np.random.default_rng(seed2)
    o = default_opts(3)
    o.update(ibound=[3, 3, 3], xmin=[0.0, 0.0, 0.0], xmax=[1.0, 1.0, 1.0],
             imhd=0, iener=0, gamma=1.0001, tolh=1.0e-4, psep=1.0 / n1d)
    n = n1d ** 3
    dx = 1.0 / n1d
    lnrho = sigma_lnrho * _gaussian_field(n1d, rng1, 2.0, 32.0, -2.0)
    delta = np.exp(lnrho - lnrho.mean())
    delta = delta / delta.mean() - 1.0
    # displacement s with div s = -delta  (continuity to first order)
    k = 2.0 * np.pi * np.fft.fftfreq(n1d, d=dx)
    kz, ky, kx = np.meshgrid(k, k, 2.0 * np.pi * np.fft.rfftfreq(n1d, d=dx), indexing="ij")
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    k2[0, 0, 0] = 1.0
    dk = np.fft.rfftn(delta)
    phi = dk / k2                       # s = grad(phi) ... div s = -k2 phi = -delta
    sx = np.fft.irfftn(1j * kx * phi, s=(n1d,) * 3, axes=(0, 1, 2))
    sy = np.fft.irfftn(1j * ky * phi, s=(n1d,) * 3, axes=(0, 1, 2))
    sz = np.fft.irfftn(1j * kz * phi, s=(n1d,) * 3, axes=(0, 1, 2))
    smax = 0.45 * dx * 4.0
    scale = min(1.0, smax / max(np.abs(sx).max(), np.abs(sy).max(), np.abs(sz).max(), 1e-30))
    g = (np.arange(n1d, dtype=np.float64) + 0.5) * dx
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    p = _empty(n, 3)
    p["x"][:, 0] = np.mod(xx.ravel() + scale * sx.ravel(), 1.0)
    p["x"][:, 1] = np.mod(yy.ravel() + scale * sy.ravel(), 1.0)
    p["x"][:, 2] = np.mod(zz.ravel() + scale * sz.ravel(), 1.0)
    # solenoidal velocity: curl of a random vector potential
    ax = _gaussian_field(n1d, rng2, 2.0, 32.0, -2.0)
    ay = _gaussian_field(n1d, rng2, 2.0, 32.0, -2.0)
    az = _gaussian_field(n1d, rng2, 2.0, 32.0, -2.0)
    fx, fy, fz = np.fft.rfftn(ax), np.fft.rfftn(ay), np.fft.rfftn(az)
    vx = np.fft.irfftn(1j * (ky * fz - kz * fy), s=(n1d,) * 3, axes=(0, 1, 2))
    vy = np.fft.irfftn(1j * (kz * fx - kx * fz), s=(n1d,) * 3, axes=(0, 1, 2))
    vz = np.fft.irfftn(1j * (kx * fy - ky * fx), s=(n1d,) * 3, axes=(0, 1, 2))
    vrms = math.sqrt(np.mean(vx ** 2 + vy ** 2 + vz ** 2))
    cs = 1.0
    f = mach * cs / vrms if vrms > 0 else 0.0
    p["vel"][:, 0] = f * vx.ravel()
    p["vel"][:, 1] = f * vy.ravel()
    p["vel"][:, 2] = f * vz.ravel()
    p["pmass"][:] = 1.0 / n
    p["dens"][:] = 1.0 + delta.ravel() * 0.0   # initial h guess from the mean density
    # isothermal: polyk = 2/3 u (primitive2conservative, gamma <= 1.0001) and
    # c_s^2 = gamma polyk rho^(gamma-1) ~ 1  ->  u = 1.5/gamma
    p["uu"][:] = 1.5 / o["gamma"]
    o["polyk"] = 2.0 / 3.0 * p["uu"][0]
    _set_alpha(p, o)
    return o, p


def dust_gas_box_3d(n1d: int = 96, eps: float = 0.1, tstop: float = 0.01,
                    seed: int = 77) -> tuple[dict, dict]:
    """Two-fluid dust + gas MHD box: 2 x n1d^3 particles, periodic unit cube.

    Gas on a jittered cubic lattice, dust on the same lattice offset by dx/2
    in every direction.  rho_gas = 1, rho_dust = eps; K set so that the
    stopping time t_s = rho_g rho_d / (K (rho_g + rho_d)) equals ``tstop``
    (dust.f90:91, idrag_nature = 1).  Gas velocity 1e-2 sin(2 pi x) in x,
    dust at rest; B = (0.05, 0, 0) on the gas; gamma = 5/3, P_gas = 1.
    """
    rng = np.random.default_rng(seed)
    o = default_opts(3)
    kdrag = 1.0 * eps / (tstop * (1.0 + eps))
    o.update(ibound=[3, 3, 3], xmin=[0.0, 0.0, 0.0], xmax=[1.0, 1.0, 1.0],
             imhd=1, idust=2, idrag_nature=1, Kdrag=kdrag, psep=1.0 / n1d)
    dx = 1.0 / n1d
    g = (np.arange(n1d, dtype=np.float64) + 0.25) * dx
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    ng = n1d ** 3
    n = 2 * ng
    p = _empty(n, 3)
    base = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)
    p["x"][:ng] = base + rng.uniform(-0.1, 0.1, size=(ng, 3)) * dx
    p["x"][ng:] = base + 0.5 * dx + rng.uniform(-0.1, 0.1, size=(ng, 3)) * dx
    p["itype"][ng:] = ITYPE_DUST
    p["vel"][:ng, 0] = 1.0e-2 * np.sin(2.0 * math.pi * p["x"][:ng, 0])
    p["pmass"][:ng] = 1.0 / ng
    p["pmass"][ng:] = eps / ng
    p["dens"][:ng] = 1.0
    p["dens"][ng:] = eps
    p["uu"][:ng] = 1.0 / ((o["gamma"] - 1.0) * 1.0)
    p["Bfield"][:ng, 0] = 0.05
    _set_alpha(p, o)
    return o, p


def brio_wu_batch(ntubes: int = 4096, nmin: int = 200, nmax: int = 1600, seed: int = 2024):
    """Batched workload: ``ntubes`` independent 1D Brio-Wu tubes with particle
    counts drawn from a seeded uniform integer range [nmin, nmax] (uneven),
    concatenated.  Returns (opts, particles, sim, counts) where sim[i] is the
    tube of particle i; ireal stays 1-based over the concatenation."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(nmin, nmax + 1, size=ntubes)
    parts, sims, o0 = [], [], None
    start = 0
    psep = 0.0
    real_counts = []
    for t, c in enumerate(counts):
        o, p = brio_wu_tube(int(c))
        n = p["x"].shape[0]
        p["ireal"] = np.where(p["ireal"] > 0, p["ireal"] + start, 0).astype(np.int32)
        parts.append(p)
        sims.append(np.full(n, t, np.int32))
        real_counts.append(n)
        psep = max(psep, o["psep"])
        start += n
        o0 = o
    o0 = dict(o0)
    o0["psep"] = psep
    cat = {k: np.concatenate([p[k] for p in parts], axis=0) for k in parts[0]}
    return o0, cat, np.concatenate(sims), np.array(real_counts)


ALLOC_FIELDS_SCALAR = ("en", "hh", "rho", "rhoalt", "drhodt", "dhdt", "gradh", "gradhn",
                       "gradgradh", "dens", "uu", "pr", "spsound", "dudt", "dendt", "divB", "del2u")
ALLOC_FIELDS_VEC3 = ("vel", "Bevol", "alpha", "Bfield", "force", "dBevoldt", "daldt", "curlB", "graddivv")


def full_state(p: dict, ndim: int) -> dict:
    """Complete ndsph_particles-shaped array set (missing fields zeroed)."""
    n = p["x"].shape[0]
    out = {}
    out["x"] = np.ascontiguousarray(p["x"], dtype=np.float64).reshape(n, ndim).copy()
    for k in ALLOC_FIELDS_SCALAR:
        out[k] = np.ascontiguousarray(p[k], dtype=np.float64).copy() if k in p else np.zeros(n)
    for k in ALLOC_FIELDS_VEC3:
        out[k] = np.ascontiguousarray(p[k], dtype=np.float64).copy() if k in p else np.zeros((n, 3))
    out["pmass"] = np.ascontiguousarray(p["pmass"], dtype=np.float64).copy()
    out["itype"] = np.ascontiguousarray(p["itype"], dtype=np.int32).copy()
    out["ireal"] = np.ascontiguousarray(p["ireal"], dtype=np.int32).copy()
    out["numneigh"] = np.zeros(n, np.int32)
    return out
