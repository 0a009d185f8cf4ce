"""Autotuner (fpde_line_autotune): it returns launch parameters inside the documented ranges,
and a line created with them computes the same solution as the built-in partition (up to the
rounding that a different order of the scans' operations gives: 1e-12, or 4x the oracle's
one-ulp envelope on a long line)."""
import numpy as np
import pytest
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("N,steps,prec,tol", [(1000, 160, 0, 1e-12), (20000, 160, 0, 1e-9),
                                              (20000, 200, 3, 1e-9), (65536, 192, 3, 3e-9),
                                              (16384, 768, 3, 3e-9)])
def test_autotuned_line_matches_default(ctx, N, steps, prec, tol):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=N, steps=steps)
    A, B, R = p.coefs()
    t = fp.autotune_line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, steps, precision=prec)
    print(f"N={N} prec={prec}: solve_sp={t.solve_sp} chunks={t.chunks} far_splits={t.far_splits} "
          f"gemv_splits={t.gemv_splits} far_super={t.far_super} ms/step={t.ms_per_step:.4f}")
    assert t.solve_sp in (1, 2, 4, 8) and 1 <= t.chunks <= ctx.sm_count and t.ms_per_step > 0
    assert 0 <= t.far_splits <= 4 and 0 <= t.gemv_splits <= 64
    if prec == 3 and steps >= 512:                  # the super-block depth is timed, not left at 0
        assert t.far_super in (1, 2, 4)
    out = []
    for tuning in (None, t):
        line = fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, steps, precision=prec, tuning=tuning)
        line.run(steps)
        out.append(line.state())
        line.close()
    assert relmax(out[1], out[0]) <= tol


def test_bad_tuning_is_rejected(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=4000, steps=10)
    A, B, R = p.coefs()
    t = fp.LineTuning(solve_sp=3)
    with pytest.raises(fp.FpdeError):
        fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, 10, tuning=t)
