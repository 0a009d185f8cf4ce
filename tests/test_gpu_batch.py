"""Ensembles of columns (fpde_batch_*) on the GPU against the oracle, column by column.

Columns of very different lengths (2 .. 5000 intervals, around the 512-thread segment
boundaries), orders and boundary kinds share one history sum and one solve kernel per step;
each must equal the oracle's own run of that column to 1e-12, or to 4x the oracle's one-ulp
rounding envelope where the column is long and ill-conditioned.
"""
import math

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


def _col(prob, left=(0, 0.0), right=(0, 0.0)):
    A, B, R = prob.coefs()
    return dict(N=prob.N, alpha=prob.alpha, tau=prob.tau, Da=prob.Da, A=A, B=B, Rlap=R, u0=prob.u0,
                left=left, right=right, dLN=1.0 / prob.N)


def _oracle(c, steps, pert=None):
    f = pert or (lambda x: x)
    u, _ = oracle.line_run(c["u0"], steps, c["tau"], c["alpha"], c["Da"], f(c["A"]), f(c["B"]), f(c["Rlap"]),
                           c["left"][0], c["left"][1], c["right"][0], c["right"][1], c["dLN"])
    return u


def _check(ctx, cols, steps):
    import fpde_hpc_gb300 as fp
    b = fp.Batch(ctx, cols, steps)
    b.run(steps)
    worst = 0.0
    for i, c in enumerate(cols):
        u = b.state(i)
        uref = _oracle(c, steps)
        rng = np.random.default_rng(i)
        env = relmax(_oracle(c, steps, lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))), uref)
        err = relmax(u, uref)
        worst = float(np.maximum(worst, err))
        assert err <= max(1e-12, 4 * env), (i, c["N"], err, env)
    b.close()
    return worst


def test_batch_mixed_columns_vs_oracle(ctx):
    from fpde_hpc_gb300 import problems
    rng = np.random.default_rng(11)
    sizes = [2, 3, 17, 255, 256, 257, 511, 512, 513, 1000, 1025, 2049, 5000, 40, 700, 1300]
    cols = []
    for j, N in enumerate(sizes):
        p = problems.config2(N=N, steps=90)
        p.alpha = float(rng.uniform(0.5, 0.95))
        p.tau = 1e-3
        left = (1, 0.0) if j % 3 == 1 else (0, 0.0)
        right = (1, 0.0) if j % 4 == 2 else (0, 0.0)
        cols.append(_col(p, left, right))
    worst = _check(ctx, cols, 90)
    print(f"mixed ensemble of {len(cols)} columns, 90 steps: max rel vs oracle {worst:.2e}")


def test_batch_config5_sample_vs_oracle(ctx):
    """A 24-column draw of the ensemble benchmark's distribution (N up to 4096), 100 steps."""
    from fpde_hpc_gb300 import problems
    cols = [_col(p) for p in problems.config5(n_cols=24, steps=100, n_max=4096)]
    worst = _check(ctx, cols, 100)
    print(f"config-5 sample, 24 columns, 100 steps: max rel vs oracle {worst:.2e}")


def test_batch_pieces_reset_and_host_call(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    cols = [_col(p) for p in problems.config5(n_cols=6, steps=40, n_max=1500)]
    b = fp.Batch(ctx, cols, 40)
    b.run(25)
    b.run(15)
    two = [b.state(i) for i in range(len(cols))]
    b.reset()
    b.run(40)
    again = [b.state(i) for i in range(len(cols))]
    u0 = b.pack([c["u0"] for c in cols])
    out = np.zeros_like(u0)
    b.solve_host(u0, 40, out)
    host = b.unpack(out)
    b.close()
    for x, y, z in zip(two, again, host):
        assert np.array_equal(x, y) and np.array_equal(x, z)


@pytest.mark.parametrize("steps,tol", [(64, 1e-11), (200, 1e-7)])
def test_batch_split_history_vs_fp64(ctx, steps, tol):
    """Split path of the ensemble (per-column weight tiles in one tensor-core contraction, FP64
    near history, work-queue solve) against the FP64 ensemble: within the first block the same
    up to rounding, across blocks within 1e-7, column by column."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    cols = [_col(p) for p in problems.config5(n_cols=20, steps=steps, n_max=3000)]
    res = []
    for prec in (0, 3):
        b = fp.Batch(ctx, cols, steps, precision=prec)
        b.run(steps)
        res.append([b.state(i) for i in range(len(cols))])
        b.close()
    worst = max(relmax(x, y) for x, y in zip(res[1], res[0]))
    print(f"ensemble of {len(cols)} columns, {steps} steps, split x3 vs FP64: max rel {worst:.2e}")
    assert worst <= tol


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (3, 1e-7)])
def test_batch_restricted_summing_vs_oracle(ctx, precision, tol):
    """Restricted summing per column (restrict_eps, the reference's sum_alg 1): columns with
    windows of 0, 5, 63, 64 and 100 lags and one untruncated share the ensemble; each equals the
    oracle's general line run with its lag weights from the window on set to zero."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    steps = 200
    cols, refs = [], []
    for j, (N, max_lag) in enumerate([(300, 0), (1000, 5), (2049, 63), (700, 64), (4096, 100), (513, 1000)]):
        p = problems.config2(N=N, steps=steps)
        p.alpha = 0.6 + 0.05 * j
        A, B, R = p.coefs()
        b = fp.weights_l1_lags(p.alpha, steps + 2)
        kkk0 = p.tau ** (1 - p.alpha) / (1 - p.alpha)
        kb = kkk0 * b
        eps = 0.5 * (kb[max_lag] + kb[max_lag + 1]) if max_lag < steps else 0.5 * kb[steps + 1]
        c = dict(N=p.N, alpha=p.alpha, tau=p.tau, Da=p.Da, A=A, B=B, Rlap=R, u0=p.u0, restrict_eps=eps)
        cols.append(c)
        w = np.zeros(steps + 1)
        keep = min(max_lag, steps)
        w[:keep + 1] = p.Da * kb[:keep + 1] / p.tau
        refs.append(oracle.line_run_general(p.u0, steps, w, 0.0, A, B, R)[0])
    bt = fp.Batch(ctx, cols, steps, precision=precision)
    bt.run(steps)
    for i, uref in enumerate(refs):
        err = relmax(bt.state(i), uref)
        print(f"precision {precision}, column {i}: {err:.2e}")
        assert err <= tol, (i, err)
    bt.close()
