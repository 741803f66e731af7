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
