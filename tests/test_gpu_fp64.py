"""Parity of the plain FP64 GPU path with the CPU oracle (and the reference's golden runs).

Tolerance: 1e-12 relative to the maximum magnitude of the reference value (normwise), the
parity bar of the FP64 path. All calls go through the C ABI.
"""
import numpy as np
import pytest

import fgv
import oracle
from conftest import golden_path
from conftest import relmax

pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def test_history_sum_matches_oracle(ctx):
    import fpde_hpc_gb300 as fp
    rng = np.random.default_rng(3)
    nodes, steps = 3001, 150
    snaps = np.cumsum(rng.standard_normal((steps + 1, nodes)) * 1e-2, axis=0) + 1.0
    h = fp.History(ctx, nodes, steps)
    for s in snaps:
        h.append(s)
    assert len(h) == steps
    kb = rng.random(steps) + 0.1
    tau = rng.random(steps) * 1e-3 + 1e-4
    S = h.l1_sum(kb, tau, scale=0.37)
    D = np.diff(snaps, axis=0)
    Sref = 0.37 * oracle.l1_sum(D, steps, kb, tau)
    assert relmax(S, Sref) <= RTOL
    h.close()


def test_sum_snapshots_matches_reference_golden(ctx):
    """The reference's Sum contract (snapshots + kb_3_cache + tau) on the reference's own run."""
    g = fgv.load(golden_path("fpde_column_a2"))
    U = g["U"]
    n = U.shape[0] - 1
    old = np.concatenate([g["U0"][None], U[:n]]).reshape(n + 1, -1)
    off = g["kb_off"].astype(int)
    kb = g["kb_flat"][off[n]:off[n + 1]]
    S = ctx.sum_snapshots(old, kb, g["tau"])
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    mask = np.zeros(g["U0"].shape, dtype=bool)
    mask[1:K + 1, 1:M, 1:sN] = True
    Sref = g["S"][n].reshape(-1)[mask.reshape(-1)]
    assert relmax(S[mask.reshape(-1)], Sref) <= RTOL


@pytest.mark.parametrize("lk,rk", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_batched_thomas_matches_oracle(ctx, lk, rk):
    rng = np.random.default_rng(10 + 2 * lk + rk)
    n_lines, N = 37, 50
    a = rng.random((n_lines, N + 1)) + 0.5
    b = rng.random((n_lines, N + 1)) + 0.5
    r = a + b + rng.random((n_lines, N + 1)) + 0.1
    om = rng.standard_normal((n_lines, N + 1))
    u = rng.standard_normal((n_lines, N + 1))
    lv = rng.standard_normal(n_lines)
    rv = rng.standard_normal(n_lines)
    dLN = 0.02
    ref = np.stack([oracle.thomas_line(a[l], b[l], r[l], om[l], lk, lv[l], rk, rv[l], dLN, u[l])
                    for l in range(n_lines)])
    # lines stored with stride_line = N+1, stride_elem = 1 (host path) ...
    out = u.copy()
    ctx.tridiag_solve(a, b, r, om, out, n_lines, N, 1, N + 1, lk, lv, rk, rv, dLN)
    assert relmax(out, ref) <= RTOL
    # ... and transposed on the device: element stride n_lines, line stride 1
    import torch
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    ud = T(u)
    ctx.tridiag_solve(T(a), T(b), T(r), T(om), ud, n_lines, N, n_lines, 1, lk, torch.from_numpy(lv).cuda(),
                      rk, torch.from_numpy(rv).cuda(), dLN)
    assert relmax(ud.cpu().numpy().T, ref) <= RTOL


def _run_line(ctx, prob, steps, left=(0, 0.0), right=(0, 0.0), dLN=0.0):
    import fpde_hpc_gb300 as fp
    A, B, R = prob.coefs()
    line = fp.Line(ctx, prob.N, prob.alpha, prob.tau, prob.Da, A, B, R, prob.u0, steps, left=left,
                   right=right, dLN=dLN)
    line.run(steps)
    u = line.state()
    line.close()
    uref, _ = oracle.line_run(prob.u0, steps, prob.tau, prob.alpha, prob.Da, A, B, R,
                              left[0], left[1], right[0], right[1], dLN)
    return u, uref


def rounding_envelope(prob, steps, left=(0, 0.0), right=(0, 0.0), dLN=0.0):
    """How far the oracle's own result moves when its coefficients change by one ulp (random
    signs). Long fine lines are ill-conditioned (Laplacian ~k/h^2 >> local term), so any
    reordering of FP64 operations (FMA, scans) moves the result by about this much."""
    A, B, R = prob.coefs()
    rng = np.random.default_rng(0)
    pert = lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))
    u1, _ = oracle.line_run(prob.u0, steps, prob.tau, prob.alpha, prob.Da, A, B, R,
                            left[0], left[1], right[0], right[1], dLN)
    u2, _ = oracle.line_run(prob.u0, steps, prob.tau, prob.alpha, prob.Da, pert(A), pert(B), pert(R),
                            left[0], left[1], right[0], right[1], dLN)
    return relmax(u2, u1)


def test_line_config1_full_matches_oracle(ctx):
    """Config 1 at full size: N=1000, 1000 steps, alpha 0.8 (single-CTA solve)."""
    from fpde_hpc_gb300 import problems
    p = problems.config1()
    u, uref = _run_line(ctx, p, p.steps)
    assert relmax(u, uref) <= RTOL


@pytest.mark.parametrize("N,steps", [(20000, 120), (65536, 48)])
def test_line_multi_cta_matches_oracle(ctx, N, steps):
    """Long lines: the Thomas solve spans many CTAs (grid-wide affine scans). Tolerance:
    1e-12, or 4x the oracle's own one-ulp rounding envelope where that is larger (the
    65,536-node line moves by ~2e-10 under a one-ulp change of its coefficients)."""
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=N, steps=steps)
    u, uref = _run_line(ctx, p, steps)
    env = rounding_envelope(p, steps)
    err = relmax(u, uref)
    print(f"N={N}: rel err {err:.3e}, oracle one-ulp envelope {env:.3e}")
    assert err <= max(RTOL, 4 * env)


def test_line_flux_boundaries_match_oracle(ctx):
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=3000, steps=100, tau=1e-3)
    h = 1.0 / p.N
    u, uref = _run_line(ctx, p, 100, left=(1, 0.02), right=(1, -0.5), dLN=h)
    assert relmax(u, uref) <= RTOL


def test_line_host_entry_and_restart(ctx):
    """fpde_line_solve_host (upload, run, download) equals run-from-reset, and runs split
    into pieces equal one run."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config1(steps=300)
    A, B, R = p.coefs()
    line = fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, 300)
    out = np.zeros(p.N + 1)
    line.solve_host(p.u0, 300, out)
    line.reset(p.u0)
    line.run(100)
    line.run(200)
    u2 = line.state()
    np.testing.assert_array_equal(out, u2)
    line.close()
