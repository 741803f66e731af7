"""CPU tests of the C-ABI library: it loads without a GPU and exports every
entry point include/ndsph.h declares; host-only calls agree with the oracle."""
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "ndsph.h")).read()
    return sorted(set(re.findall(r"NDSPH_API\s+[\w\s\*]+?\b(ndsph_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from ndspmhd_gb300 import gpu
    lib = gpu.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", gpu.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ndsph_\w+)", out))
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        assert hasattr(lib, s)


def test_kernel_tables_match_oracle():
    from ndspmhd_gb300 import gpu
    from oracle import oracle as O
    for ndim in (1, 2, 3):
        a = gpu.kernel_tables(ndim)
        b = O.kernel_tables(ndim)
        np.testing.assert_array_equal(a, b)


def test_default_opts_match_reference_defaults():
    import ctypes as C
    from ndspmhd_gb300 import gpu
    from ndspmhd_gb300.abi import NdsphOpts
    from ndspmhd_gb300.configs import default_opts
    o = NdsphOpts()
    gpu.lib().ndsph_default_opts.argtypes = [C.POINTER(NdsphOpts), C.c_int32]
    gpu.lib().ndsph_default_opts(C.byref(o), 3)
    d = default_opts(3)
    for k in ("hfact", "tolh", "maxdensits", "imagforce", "iener", "iav", "alphamin", "alphaumin",
              "alphaBmin", "beta", "avdecayconst", "C_cour", "C_force"):
        assert getattr(o, k) == d[k], k
    assert list(o.iavlim) == d["iavlim"]


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the public structs have the header's sizes and
    field offsets (a C program built against include/ndsph.h prints them)."""
    import ctypes as C
    import shutil
    from ndspmhd_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    pairs = [("ndsph_opts", abi.NdsphOpts), ("ndsph_particles", abi.NdsphParticles), ("ndsph_dt", abi.NdsphDt),
             ("ndsph_timing", abi.NdsphTiming), ("ndsph_tuning", abi.NdsphTuning)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ndsph.h"', 'int main(void) {']
    for cname, py in pairs:
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln.strip():
            a, b, c = ln.split()
            got[(a, b)] = int(c)
    for cname, py in pairs:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def _c_struct_fields(txt, name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), txt, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for m in re.finditer(r"\b(int32_t|int64_t|double|float)\s*(\*?)\s*(\w+)\s*(?:\[(\d+)\])?\s*;", body):
        kind = "ptr" if m.group(2) else m.group(1)
        out.append((m.group(3).lower(), kind, int(m.group(4) or 1)))
    return out


def _f_type_fields(txt, name):
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)\n\s*end type" % name, txt, re.S).group(1)
    kinds = {"integer(c_int32_t)": "int32_t", "integer(c_int64_t)": "int64_t", "real(c_double)": "double",
             "real(c_float)": "float", "type(c_ptr)": "ptr"}
    out = []
    for line in body.split("\n"):
        line = line.split("!")[0].strip()
        if not line:
            continue
        decl, names = [x.strip() for x in line.split("::")]
        for m in re.finditer(r"(\w+)\s*(?:\((\d+)\))?", names):
            out.append((m.group(1).lower(), kinds[decl.replace(" ", "")], int(m.group(2) or 1)))
    return out


def test_fortran_shim_types_match_the_header():
    """The bind(C) derived types of the Fortran shim list the header's fields
    in the same order with the matching C kinds (the shim is not compiled
    here, so its layout is checked against the declarations as text)."""
    c = open(os.path.join(ROOT, "include", "ndsph.h")).read()
    f = open(os.path.join(ROOT, "ndspmhd_gb300", "fortran", "gpu_sph.f90")).read()
    for cname in ("ndsph_opts", "ndsph_particles", "ndsph_dt", "ndsph_tuning"):
        cf, ff = _c_struct_fields(c, cname), _f_type_fields(f, cname + "_t")
        assert cf and cf == ff, (cname, cf, ff)


# option sets the reference supports but the device path does not take: each is
# refused by ndsph_init with NDSPH_E_ARG before any CUDA call
_OUT_OF_SCOPE = [
    (dict(ndim=4), "ndim"),
    (dict(ibound=[2, 0, 0]), "ibound"),
    (dict(ibound=[3, 0, 0], xmin=[1.0, 0.0, 0.0], xmax=[1.0, 1.0, 1.0]), "xmax <= xmin"),
    (dict(imhd=2), "imhd"),
    (dict(imhd=1, imagforce=1), "imagforce"),
    (dict(iener=1), "iener"),
    (dict(iav=1), "iav"),
    (dict(idust=1), "idust"),
    (dict(idust=2, idrag_nature=2), "idrag_nature"),
    (dict(iavlim=[3, 1, 0]), "iavlim"),
    (dict(iavlim=[2, 1, 1]), "iavlim"),
    (dict(precision=7), "precision"),
]


def test_out_of_scope_options_are_refused():
    import pytest
    from ndspmhd_gb300 import gpu
    from ndspmhd_gb300.configs import default_opts
    for change, word in _OUT_OF_SCOPE:
        o = default_opts(3)
        o.update(change)
        with pytest.raises(gpu.NdsphError) as e:
            gpu.GpuSPH(o, n=64)
        assert e.value.code == 1, (change, str(e.value))
        assert word in str(e.value), (change, str(e.value))


def test_without_a_gpu_the_context_fails_loudly():
    """A valid option set on a machine without a GPU ends in NDSPH_E_CUDA from
    ndsph_init: there is no host fallback behind the C-ABI."""
    import pytest
    import torch
    from ndspmhd_gb300 import gpu
    from ndspmhd_gb300.configs import default_opts
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    for ndim in (1, 2, 3):
        with pytest.raises(gpu.NdsphError) as e:
            gpu.GpuSPH(default_opts(ndim), n=64)
        assert e.value.code == 2, str(e.value)


def test_kernel_tables_refuse_bad_dimension():
    import ctypes as C
    from ndspmhd_gb300 import gpu
    out = np.zeros(5 * 4001)
    ptr = out.ctypes.data_as(C.POINTER(C.c_double))
    for ndim in (0, 4):
        assert gpu.lib().ndsph_kernel_tables(ndim, ptr) == 1
    assert gpu.lib().ndsph_kernel_tables(3, None) == 1
