"""The reference's printed known answer on the GPU: its column (mode 3, BS 1, NB 3, M 3, K 1000,
analytic problem 2, alpha 0.8, tau 1e-3, 1,000 steps) reports the squared error 0.014446 against
the exact solution. The library's 3D LOD runs the same column from the rebuilt per-step inputs:
  * FP64: the reference's final grid within 2e-12 (the closed-form weights differ from the
    reference's EPS-1e-15 series by up to 1.5e-13) and its error within 1e-8 relative;
  * the exact three-slice split (far history on the tensor cores, 15 blocks of 64 steps): within
    1e-7 of the FP64 grid and the error within 1e-6 relative."""
import numpy as np
import pytest

import kat_case
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def case():
    return kat_case.load()


def _run(ctx, c, precision):
    import fpde_hpc_gb300 as fp
    g = c["g"]
    lod = fp.Lod3D(ctx, c["dims"], float(g["alpha"]), float(g["tau"]), float(g["Da"]), *c["coefs"], g["U0"],
                   c["steps"], source=c["src"], bc=c["bc"], precision=precision)
    lod.run(c["steps"])
    U = lod.state()
    lod.close()
    return U


def test_known_answer_fp64(ctx, case):
    g = case["g"]
    U = _run(ctx, case, 0)
    err = kat_case.analytic_sq_err(U, case)
    print(f"K=1000 column, 1000 steps: grid vs reference {relmax(U, g['U_final']):.2e}, "
          f"analytic squared error {err:.8g} (reference {float(g['analytic_sq_err']):.8g})")
    assert relmax(U, g["U_final"]) <= 2e-12
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])


def test_known_answer_split(ctx, case):
    g = case["g"]
    U64 = _run(ctx, case, 0)
    U3 = _run(ctx, case, 3)
    err = kat_case.analytic_sq_err(U3, case)
    print(f"split x3: vs FP64 {relmax(U3, U64):.2e}, analytic squared error {err:.8g}")
    assert relmax(U3, U64) <= 1e-7
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-6 * float(g["analytic_sq_err"])


def test_reference_known_answer_3d_generalized_kernel(ctx):
    """gpu_test.sh's error_tests parameters at 20 x 20 x 20 with g(t) = t^0.8 (the reference prints
    0.0472441): the 3D LOD's variable-step time loop with the reference's weight rows reproduces its
    final grid to 1e-12 and that error."""
    import fpde_hpc_gb300 as fp
    c = kat_case.load("fpde_lod3d_kat")
    g = c["g"]
    lod = fp.Lod3D(ctx, c["dims"], float(g["alpha"]), float(g["tau"]), float(g["Da"]), *c["coefs"], g["U0"],
                   c["steps"], source=c["src"], bc=c["bc"], time_steps=g["tau_steps"], weight_rows=c["rows"])
    lod.run(c["steps"])
    U = lod.state()
    lod.close()
    assert relmax(U, g["U_final"]) <= 1e-12
    err = kat_case.analytic_sq_err(U, c)
    print(f"3D known answer: squared error {err:.6g} (reference {float(g['analytic_sq_err']):.6g})")
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])
    assert f"{err:.6g}" == "0.0472441"
