"""The reference's dump files (readwrite_dumps.f90:32-440).

A dump is a Fortran unformatted sequential file (gfortran: every record is
framed by 4-byte little-endian length markers).  Record 1 is the header
``t, npart, nprint, gamma, hfact, ndim, ndimV, ncolumns, iformat,
ibound(1:ndim), xmin(1:ndim), xmax(1:ndim), len(geom), geom``; then one
record per column, each column a whole array over the particles
(write_dump :94-190): x(ndim), vel(ndimV), h, dens, u, m and, with MHD,
alpha(3), B(ndimV), psi, then the information-only pr, -drho/dt/rho, div B,
curl B(ndimV), gradh, force(ndimV); without MHD alpha(2), pr, -drho/dt/rho,
gradh, force(ndimV); finally itype.  Cartesian geometry, no one-fluid dust
(the hot path's subset).

``write_dump`` writes that layout from a particle dict; ``read_dump`` reads
it back into the dict the library takes, so GPU runs, oracle runs and a
Fortran build of the reference exchange identical particle sets.
"""
from __future__ import annotations

import struct

import numpy as np

NDIMV = 3


def _rec(f, payload: bytes) -> None:
    n = struct.pack("<i", len(payload))
    f.write(n)
    f.write(payload)
    f.write(n)


def _read_rec(f) -> bytes:
    head = f.read(4)
    if len(head) < 4:
        raise EOFError("truncated dump")
    (n,) = struct.unpack("<i", head)
    data = f.read(n)
    (m,) = struct.unpack("<i", f.read(4))
    if m != n or len(data) != n:
        raise ValueError("corrupt record framing")
    return data


def ncolumns(ndim: int, imhd: int) -> tuple[int, int]:
    """ncolumns and iformat as write_dump computes them (cartesian, no dust)."""
    nc = ndim + 2 * NDIMV + 4
    if imhd != 0:
        nc += 8 + 2 * NDIMV
        iformat = 2
    else:
        nc += 5
        iformat = 1
    return nc, iformat


def write_dump(path: str, t: float, st: dict, opts: dict, geom: str = "cartesian") -> None:
    ndim = opts["ndim"]
    n = st["x"].shape[0]
    nc, iformat = ncolumns(ndim, opts["imhd"])
    g = geom.ljust(12)[:12].encode()
    head = struct.pack("<dii", t, n, n) + struct.pack("<dd", opts["gamma"], opts["hfact"])
    head += struct.pack("<iiii", ndim, NDIMV, nc, iformat)
    head += struct.pack(f"<{ndim}i", *[int(v) for v in opts["ibound"][:ndim]])
    head += struct.pack(f"<{ndim}d", *opts["xmin"][:ndim]) + struct.pack(f"<{ndim}d", *opts["xmax"][:ndim])
    head += struct.pack("<i", len(g)) + g
    d = lambda a: np.ascontiguousarray(a, dtype="<f8").tobytes()
    x = np.asarray(st["x"]).reshape(n, ndim)
    with open(path, "wb") as f:
        _rec(f, head)
        for k in range(ndim):
            _rec(f, d(x[:, k]))
        for k in range(NDIMV):
            _rec(f, d(st["vel"][:, k]))
        _rec(f, d(st["hh"]))
        _rec(f, d(st["dens"]))
        _rec(f, d(st["uu"]))
        _rec(f, d(st["pmass"]))
        rho = np.where(st["rho"] != 0, st["rho"], 1.0)
        if opts["imhd"] != 0:
            for k in range(3):
                _rec(f, d(st["alpha"][:, k]))
            for k in range(NDIMV):
                _rec(f, d(st["Bfield"][:, k]))
            _rec(f, d(st.get("psi", np.zeros(n))))
            _rec(f, d(st["pr"]))
            _rec(f, d(-st["drhodt"] / rho))
            _rec(f, d(st["divB"]))
            for k in range(NDIMV):
                _rec(f, d(st["curlB"][:, k]))
            _rec(f, d(st["gradh"]))
            for k in range(NDIMV):
                _rec(f, d(st["force"][:, k]))
        else:
            for k in range(2):
                _rec(f, d(st["alpha"][:, k]))
            _rec(f, d(st["pr"]))
            _rec(f, d(-st["drhodt"] / rho))
            _rec(f, d(st["gradh"]))
            for k in range(NDIMV):
                _rec(f, d(st["force"][:, k]))
        _rec(f, np.ascontiguousarray(st["itype"], dtype="<i4").tobytes())


def read_dump(path: str) -> tuple[float, dict, dict]:
    """Returns (t, header, columns) with columns in the library's dict layout."""
    with open(path, "rb") as f:
        h = _read_rec(f)
        t, npart, nprint = struct.unpack_from("<dii", h, 0)
        gamma, hfact = struct.unpack_from("<dd", h, 16)
        ndim, ndimv, nc, iformat = struct.unpack_from("<iiii", h, 32)
        off = 48
        ibound = list(struct.unpack_from(f"<{ndim}i", h, off)); off += 4 * ndim
        xmin = list(struct.unpack_from(f"<{ndim}d", h, off)); off += 8 * ndim
        xmax = list(struct.unpack_from(f"<{ndim}d", h, off)); off += 8 * ndim
        (lg,) = struct.unpack_from("<i", h, off); off += 4
        geom = h[off:off + lg].decode().strip()
        n = nprint
        col = lambda: np.frombuffer(_read_rec(f), dtype="<f8").astype(np.float64)
        st = {}
        st["x"] = np.stack([col() for _ in range(ndim)], axis=1)
        st["vel"] = np.stack([col() for _ in range(ndimv)], axis=1)
        st["hh"] = col()
        st["dens"] = col()
        st["uu"] = col()
        st["pmass"] = col()
        if iformat in (2, 4):
            st["alpha"] = np.stack([col() for _ in range(3)], axis=1)
            st["Bfield"] = np.stack([col() for _ in range(ndimv)], axis=1)
            st["psi"] = col()
            st["pr"] = col()
            st["divv"] = col()
            st["divB"] = col()
            st["curlB"] = np.stack([col() for _ in range(ndimv)], axis=1)
            st["gradh"] = col()
            st["force"] = np.stack([col() for _ in range(ndimv)], axis=1)
        else:
            a = [col() for _ in range(2)]
            st["alpha"] = np.stack(a + [np.zeros(n)], axis=1)
            st["pr"] = col()
            st["divv"] = col()
            st["gradh"] = col()
            st["force"] = np.stack([col() for _ in range(ndimv)], axis=1)
        st["itype"] = np.frombuffer(_read_rec(f), dtype="<i4").astype(np.int32)
    header = dict(t=t, npart=npart, nprint=nprint, gamma=gamma, hfact=hfact, ndim=ndim, ndimV=ndimv,
                  ncolumns=nc, iformat=iformat, ibound=ibound, xmin=xmin, xmax=xmax, geom=geom)
    return t, header, st
