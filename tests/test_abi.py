"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/*.h declares
(no compute calls: runs without a GPU)."""
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fpde_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib_path():
    from fpde_hpc_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = _declared()
    assert "fpde_l1_sum" in names and "fpde_line_run" in names and "fpde_tridiag_solve" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], stdout=subprocess.PIPE, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = sorted(_declared() - exported)
    assert not missing, missing


def test_library_loads_and_binds_every_symbol(lib_path):
    from fpde_hpc_gb300 import _lib
    lib = _lib.load(lib_path)
    for name in _declared():
        assert hasattr(lib, name), name
    assert set(_lib.exported_symbols()) <= _declared()


def test_host_functions_without_gpu(lib_path):
    """Pure host entry points (weights, Gamma, coefficients) need no device."""
    import math
    import numpy as np
    import fpde_hpc_gb300 as fp
    import oracle
    t = oracle.time_points(np.full(40, 1e-3))
    for n in (0, 1, 7, 39):
        kb, k0 = fp.weights_l1(0.7, t, n)
        kb2, k02 = oracle.l1_weights(0.7, t, n)
        np.testing.assert_allclose(kb, kb2, rtol=1e-15)
        assert abs(k0 - k02) <= 1e-15 * k02
    b = fp.weights_l1_lags(0.7, 100)
    assert b[0] == 1.0
    j = np.arange(1, 100)
    np.testing.assert_allclose(b[1:], (j + 1.0) ** 0.3 - j ** 0.3, rtol=1e-12)
    assert abs(fp.gamma(0.3) - math.gamma(0.3)) <= 1e-15 * math.gamma(0.3)
    k = 1.0 + np.random.default_rng(0).random(11)
    A, B, R = fp.line_coefs(k, np.full(11, 0.1))
    A2, B2, R2 = oracle.line_coefs(k, np.ones(11), np.full(11, 0.1))
    np.testing.assert_array_equal(A[1:10], A2[1:10])
    np.testing.assert_array_equal(B[1:10], B2[1:10])
    np.testing.assert_array_equal(R[1:10], R2[1:10])


def test_errors_are_codes_not_exits(lib_path):
    """Bad arguments return FPDE_ERR_ARG with a message (the reference exits the process)."""
    import ctypes as C
    import fpde_hpc_gb300 as fp
    lib = fp.load()
    rc = lib.fpde_weights_l1(1.5, None, 3, None, None)
    assert rc == 1
    assert b"alpha" in lib.fpde_last_error_string() or b"bad" in lib.fpde_last_error_string()
    out = C.c_double()
    assert lib.fpde_gamma(-1.0, C.byref(out)) == 1


def test_do_weights_match_oracle(lib_path):
    """fpde_do_weights (host) fuses the per-order L1 weights like the oracle, and its c[0]
    is the local weight b0 of fr_do's eq_init for the reference's own orders and weights."""
    import numpy as np
    import fgv
    import oracle
    import do_cases
    import fpde_hpc_gb300 as fp
    from conftest import golden_path
    g = fgv.load(golden_path("frdo_eq_ex0"))
    Na = len(g["WA"])
    aq, qw, gq = do_cases.orders(Na), do_cases.quad_weights(g["WA"]), do_cases.gammas(Na)
    for tau, n in ((g["tau"], 64), (1e-4, 5000)):
        c = fp.do_weights(aq, qw, tau, n, gq)
        c_or = oracle.do_fused_weights(aq, qw, gq, tau, n)
        assert np.max(np.abs(c - c_or) / np.abs(c_or)) <= 1e-14
    c = fp.do_weights(aq, qw, g["tau"], 4, gq)
    assert abs(c[0] - g["b0"]) <= 1e-13 * g["b0"]
    c2 = fp.do_weights(aq, qw, g["tau"], 4)          # normalisers computed by the library
    assert np.allclose(c2, c, rtol=1e-14, atol=0)
    with pytest.raises(fp.FpdeError):
        fp.do_weights([1.5], [1.0], 0.1, 3)


def test_python_binding_covers_every_declared_symbol():
    """Every entry point of include/*.h has a ctypes signature in the Python layer."""
    from fpde_hpc_gb300 import _lib
    missing = sorted(_declared() - set(_lib._SIGS))
    assert not missing, missing
