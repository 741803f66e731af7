"""Options files and dumps in the reference's formats (CPU only)."""
import struct

import numpy as np
import pytest

from ndspmhd_gb300 import configs
from ndspmhd_gb300.dumps import ncolumns, read_dump, write_dump
from ndspmhd_gb300.infile import parse_infile, read_infile, write_infile


def test_parse_fortran_forms():
    text = """# comment line
                psep =   1.000E-02    ! particle separation
               gamma =  1.4d0    ! adiabatic index
          maxdensits =         250    ! maximum number of density iterations
          usenumdens =           F    ! Use number density formulation of gradh

              iavlimu =          1    ! use conductivity switch
"""
    d = parse_infile(text)
    assert d["psep"] == 0.01 and d["gamma"] == 1.4 and d["maxdensits"] == 250
    assert d["usenumdens"] is False and d["iavlimu"] == 1


def test_infile_round_trip(tmp_path):
    o, _ = configs.orszag_tang_2d(16)
    o = dict(o)
    o.update(gamma=1.4, alphaBmin=0.5, iavlim=[2, 1, 1], idust=2, idrag_nature=1, Kdrag=12.5)
    path = tmp_path / "run.in"
    write_infile(str(path), o)
    lines = path.read_text().splitlines()
    # write_inopt layout: name right-justified in 20 columns, ' = ', value, '! description'
    g = [ln for ln in lines if ln.strip().startswith("gamma")][0]
    assert g.index("=") == 21 and "!" in g
    back = read_infile(str(path), 2, base=o)
    for k in ("gamma", "alphaBmin", "idust", "idrag_nature", "Kdrag", "hfact", "tolh", "C_cour"):
        assert back[k] == pytest.approx(o[k], rel=1e-8), k
    assert list(back["iavlim"]) == [2, 1, 1]


def test_sweep_groups_runs_that_differ_only_in_psep_or_drag(tmp_path):
    """The sweep driver's batch key: options files that differ only in psep
    or the drag constant K share a batch (K goes per simulation); any other
    difference splits them."""
    from ndspmhd_gb300.infile import _key
    o1, _ = configs.dust_gas_box_3d(8, eps=0.5, tstop=0.05)
    o2, _ = configs.dust_gas_box_3d(8, eps=0.1, tstop=0.3)
    assert o1["Kdrag"] != o2["Kdrag"]
    assert _key(o1) == _key(o2)
    assert _key(o1) == _key(dict(o1, psep=0.5))
    assert _key(o1) != _key(dict(o1, gamma=1.4))
    assert _key(o1) != _key(dict(o1, idrag_nature=2))


def test_infile_rejects_unsupported_option(tmp_path):
    path = tmp_path / "bad.in"
    path.write_text("icty = 1 ! continuity by time derivative\n")
    with pytest.raises(ValueError):
        read_infile(str(path), 1)
    path.write_text("icty = 0\nikernel = 0\n")
    assert read_infile(str(path), 1)["hfact"] == 1.2


@pytest.mark.parametrize("imhd", [0, 1])
def test_dump_round_trip_and_layout(tmp_path, imhd):
    o, p = configs.orszag_tang_2d(8)
    o = dict(o, imhd=imhd)
    st = configs.full_state(p, 2)
    rng = np.random.default_rng(3)
    n = st["x"].shape[0]
    for k in ("hh", "rho", "drhodt", "pr", "gradh", "divB"):
        st[k] = rng.random(n) + 0.5
    for k in ("force", "curlB"):
        st[k] = rng.random((n, 3))
    path = tmp_path / "run_00001.dat"
    write_dump(str(path), 0.125, st, o)
    t, h, back = read_dump(str(path))
    nc, iformat = ncolumns(2, imhd)
    assert t == 0.125 and h["npart"] == n and h["ndim"] == 2 and h["ndimV"] == 3
    assert h["ncolumns"] == nc and h["iformat"] == iformat and h["geom"] == "cartesian"
    assert h["ibound"] == o["ibound"][:2] and h["xmin"] == o["xmin"][:2]
    # one record per column plus the header and itype
    nrec = 0
    raw = path.read_bytes()
    off = 0
    while off < len(raw):
        (m,) = struct.unpack_from("<i", raw, off)
        off += 8 + m
        nrec += 1
    assert off == len(raw)
    assert nrec == 1 + nc + 1
    np.testing.assert_array_equal(back["x"], st["x"])
    np.testing.assert_array_equal(back["vel"], st["vel"])
    for k in ("hh", "dens", "uu", "pmass", "pr", "gradh"):
        np.testing.assert_array_equal(back[k], st[k])
    np.testing.assert_array_equal(back["divv"], -st["drhodt"] / st["rho"])
    np.testing.assert_array_equal(back["itype"], st["itype"])
    if imhd:
        np.testing.assert_array_equal(back["Bfield"], st["Bfield"])
        np.testing.assert_array_equal(back["divB"], st["divB"])
        np.testing.assert_array_equal(back["alpha"], st["alpha"])
    else:
        np.testing.assert_array_equal(back["alpha"][:, :2], st["alpha"][:, :2])
