"""Edge cases of the device time loops against the oracle: the smallest grids and lines the
library accepts (two intervals per axis), single steps, a one-column ensemble, and the split
path across a block boundary on them."""
import numpy as np
import pytest

import oracle
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("precision,steps,tol", [(0, 1, 1e-13), (0, 70, 1e-12), (3, 70, 1e-7)])
def test_smallest_lod_grid(ctx, precision, steps, tol):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=2, steps=steps)
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, steps, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN, precision=precision)
    lod.run(steps)
    got = lod.state()
    lod.close()
    ref = oracle.lod_run(p.dims, p.u0, steps, p.tau, p.alpha, p.Da, cA, cB, cR, None, None, p.left_kind,
                         p.right_kind, p.dLN)
    assert relmax(got, ref) <= tol


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (3, 1e-7)])
def test_shortest_line(ctx, precision, tol):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    steps = 70
    p = problems.config2(N=2, steps=steps)
    A, B, R = p.coefs()
    line = fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, steps, precision=precision)
    line.run(steps)
    got = line.state()
    line.close()
    ref, _ = oracle.line_run(p.u0, steps, p.tau, p.alpha, p.Da, A, B, R)
    assert relmax(got, ref) <= tol


def test_one_column_ensemble_one_step(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=2, steps=1)
    A, B, R = p.coefs()
    col = dict(N=p.N, alpha=p.alpha, tau=p.tau, Da=p.Da, A=A, B=B, Rlap=R, u0=p.u0)
    b = fp.Batch(ctx, [col], 1)
    b.run(1)
    got = b.state(0)
    b.close()
    ref, _ = oracle.line_run(p.u0, 1, p.tau, p.alpha, p.Da, A, B, R)
    assert relmax(got, ref) <= 1e-13


def test_variable_step_lod_single_step(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=2, steps=1)
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, 1, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN, time_steps=[p.tau])
    lod.run(1)
    got = lod.state()
    lod.close()
    ref = oracle.lod_run(p.dims, p.u0, 1, p.tau, p.alpha, p.Da, cA, cB, cR, None, None, p.left_kind,
                         p.right_kind, p.dLN)
    assert relmax(got, ref) <= 1e-13
