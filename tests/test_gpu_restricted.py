"""Restricted summing in the line solve (the reference's sum_alg 1, time_summing
fpde_hpc_1d.cpp:4117-4131: newest first, the history stops before the first lag whose kb is
below sum_param): a line with restrict_eps against the oracle's general line run with the lag
weights from that lag on set to zero.

Windows: empty (only the local term), shorter than a 64-step block, exactly one block, one
that starts mid-tile in the far contraction, and one longer than the run (no truncation); FP64
to 1e-12 and the three-slice split to 1e-7, over 300 steps (five blocks).
"""
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


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (3, 1e-7)])
@pytest.mark.parametrize("max_lag", [0, 5, 63, 64, 100, 1000])
def test_restricted_line_vs_oracle(ctx, precision, tol, max_lag):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=4096, steps=300)
    A, B, R = p.coefs()
    b = fp.weights_l1_lags(p.alpha, p.steps + 2)       # b[j]: lag j (b[0] the local weight)
    kkk0 = p.tau ** (1 - p.alpha) / (1 - p.alpha)
    kb = kkk0 * b                                      # kb of lag j
    # a threshold between lag max_lag and the next one: the rule keeps lags 1..max_lag
    eps = 0.5 * (kb[max_lag] + kb[max_lag + 1]) if max_lag < p.steps else 0.5 * kb[p.steps + 1]
    line = fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, p.steps, precision=precision, restrict_eps=eps)
    line.run(p.steps)
    u = line.state()
    line.close()
    w = np.zeros(p.steps + 1)
    keep = min(max_lag, p.steps)
    w[:keep + 1] = p.Da * kb[:keep + 1] / p.tau
    uref, _ = oracle.line_run_general(p.u0, p.steps, w, 0.0, A, B, R)
    err = relmax(u, uref)
    print(f"precision {precision}, window {max_lag} lags: {err:.2e}")
    assert err <= tol


def test_restricted_two_term_split_is_unsupported(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config1(steps=10)
    A, B, R = p.coefs()
    with pytest.raises(fp.FpdeError) as e:
        fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, 10, precision=1, restrict_eps=0.01)
    assert e.value.code == 6


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (3, 1e-7)])
def test_restricted_do_line_vs_oracle(ctx, precision, tol):
    """Restricted summing on the distributed-order line (fused lag weights, theta = 1): the
    window comes from kb = w tau / Da of the fused weights; 200 steps, a 90-lag window."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config3(N=3000, steps=200)
    A, B, R = p.coefs()
    c = fp.do_weights(p.orders, p.qw, p.tau, p.steps + 1, p.gnorm)      # kb of lag l (Da = 1)
    keep = 90
    eps = 0.5 * (abs(c[keep]) + abs(c[keep + 1]))
    assert fp.restricted_lags(c[1:], eps) == keep
    line = fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, p.steps, lag_weights=c / p.tau, theta=1.0,
                   precision=precision, restrict_eps=eps)
    line.run(p.steps)
    u = line.state()
    line.close()
    w = c / p.tau
    w[keep + 1:] = 0.0
    uref, _ = oracle.line_run_general(p.u0, p.steps, w, 1.0, A, B, R)
    # the explicit half makes this line ill-conditioned: FP64 is held to 4x the oracle's own
    # movement under one-ulp changes of its inputs (as the unrestricted FP64 DO test)
    rng = np.random.default_rng(0)
    pert = lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))
    u2, _ = oracle.line_run_general(p.u0, p.steps, pert(w), 1.0, pert(A), pert(B), pert(R))
    env = relmax(u2, uref)
    err = relmax(u, uref)
    print(f"DO line restricted to {keep} lags, precision {precision}: {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(tol, 4 * env)
