"""Distributed-order path on the GPU against the reference's golden output and the oracle.

  * fr_do's equation (eq_solve, eq_ex 0 and 1) run as a line with fused DO lag weights,
    theta = 1 and per-step sources: every time level equals the reference's C to 1e-12;
  * the DO line of the benchmark form (variable k, 16-node Gauss-Legendre orders) against the
    oracle: FP64 within the rounding envelope, the exact three-slice split within 1e-7;
  * fpde_do_derivative (the DOC/Sum kernels' operator) against the oracle's DO_Cder restatement
    and the reference's DF of F = x^2, including the t0/j0/maxt windows eq_solve uses.
"""
import ctypes as C

import numpy as np
import pytest

import do_cases
import fgv
import oracle
from conftest import golden_path
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _do_weights(aq, qw, gq, tau, n):
    import fpde_hpc_gb300 as fp
    return fp.do_weights(aq, qw, tau, n, gq)


@pytest.mark.parametrize("name", ["frdo_eq_ex0", "frdo_eq_ex1", "frdo_eq_ex0_kat"])
def test_do_equation_every_level_matches_fr_do(ctx, name):
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path(name))
    u0, A, B, Rl, w, theta, src, steps = do_cases.line_problem(g, _do_weights)
    N = len(u0) - 1
    line = fp.Line(ctx, N, 0.5, g["tau"], 1.0, A, B, Rl, u0, steps, lag_weights=w, theta=theta, source=src)
    worst = 0.0
    for n in range(1, steps + 1):
        line.run(1)
        worst = max(worst, relmax(line.state(), g["C"][:, n]))
    line.close()
    print(f"{name}: max rel over {steps} levels {worst:.2e}")
    assert worst <= 1e-12


def _do_line(ctx, p, steps, precision):
    import fpde_hpc_gb300 as fp
    A, B, R = p.coefs()
    c = fp.do_weights(p.orders, p.qw, p.tau, steps + 1, p.gnorm)
    line = fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, steps, lag_weights=c / p.tau, theta=1.0,
                   precision=precision)
    line.run(steps)
    u = line.state()
    line.close()
    return u, c


def _envelope(p, steps, c):
    """How far the oracle's own result moves under a one-ulp change (random signs) of its
    coefficients and weights. The explicit half of the space operator (k/h^2 ~ 4e8 at
    N=20000) and the near-singular implicit half make long fine lines ill-conditioned, so any
    reordering of FP64 operations moves the result by about this much."""
    A, B, R = p.coefs()
    rng = np.random.default_rng(0)
    pert = lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))
    u1, _ = oracle.line_run_general(p.u0, steps, c / p.tau, 1.0, A, B, R)
    u2, _ = oracle.line_run_general(p.u0, steps, pert(c / p.tau), 1.0, pert(A), pert(B), pert(R))
    return u1, relmax(u2, u1)


@pytest.mark.parametrize("N,steps", [(1500, 300), (20000, 200)])
def test_do_line_fp64_vs_oracle(ctx, N, steps):
    """Tolerance 1e-12, or 4x the oracle's one-ulp envelope where that is larger."""
    from fpde_hpc_gb300 import problems
    p = problems.config3(N=N, steps=steps)
    u, c = _do_line(ctx, p, steps, 0)
    uref, env = _envelope(p, steps, c)
    err = relmax(u, uref)
    print(f"DO line N={N} {steps} steps FP64 vs oracle: {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(1e-12, 4 * env)


def test_do_line_split_x3_vs_oracle(ctx):
    from fpde_hpc_gb300 import problems
    p = problems.config3(N=4096, steps=700)
    u, c = _do_line(ctx, p, p.steps, 3)
    A, B, R = p.coefs()
    uref, _ = oracle.line_run_general(p.u0, p.steps, c / p.tau, 1.0, A, B, R)
    err = relmax(u, uref)
    print(f"DO line N=4096 700 steps bf16x3 split vs oracle: {err:.2e}")
    assert err <= 1e-7


@pytest.mark.parametrize("sp,chunks,theta,right", [
    (1, 0, 1.0, (0, 0.0)),      # one node per solver thread, built-in chunks
    (2, 30, 0.5, (1, 0.0)),     # ragged chunks of 200 nodes (idle solver threads), flux end
    (4, 13, 1.0, (1, 0.3)),     # four nodes per thread, 116 of 128 threads busy, boundary flux
])
def test_do_line_split_explicit_partitions_vs_oracle(ctx, sp, chunks, theta, right):
    """The speculative block solve with an explicit part (theta != 0): its right-hand side
    takes the neighbours' zero-carry results inside each chunk, the previous chunk's carry
    at the chunk's first node and the carry-out at its last, under every partition shape
    (nodes per thread, ragged chunks, idle threads) and both right-end kinds, with per-step
    sources, against the oracle to 1e-7 over 300 steps (5 blocks)."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config3(N=6000, steps=300)
    A, B, R = p.coefs()
    c = fp.do_weights(p.orders, p.qw, p.tau, p.steps + 1, p.gnorm)
    rng = np.random.default_rng(11)
    src = 0.1 * rng.standard_normal((40, p.N + 1))
    tuning = fp.LineTuning(solve_sp=sp, chunks=chunks, far_splits=0, gemv_splits=0)
    line = fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, p.steps, right=right, dLN=1.0 / p.N,
                   lag_weights=c / p.tau, theta=theta, source=src, precision=3, tuning=tuning)
    line.run(p.steps)
    u = line.state()
    line.close()
    uref, _ = oracle.line_run_general(p.u0, p.steps, c / p.tau, theta, A, B, R, src, rtype=right[0],
                                      gN=right[1], dLN=1.0 / p.N)
    err = relmax(u, uref)
    print(f"DO line N=6000 300 steps bf16x3, sp={sp} chunks={chunks} theta={theta} right={right}: {err:.2e}")
    assert err <= 1e-7

def _derivative(ctx, F, tau, c, t0=1, j0=0, maxt=-1, DF0=None, append=0):
    import torch
    import fpde_hpc_gb300 as fp
    nodes, ntau = F.shape
    Fd = torch.from_numpy(np.ascontiguousarray(F)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(c)).cuda()
    DF = torch.from_numpy(np.zeros_like(F) if DF0 is None else DF0.copy()).cuda()
    rc = ctx.lib.fpde_do_derivative(ctx.h, C.c_void_p(Fd.data_ptr()), nodes, ntau, ntau, tau,
                                    C.c_void_p(cd.data_ptr()), t0, j0, maxt, C.c_void_p(DF.data_ptr()), ntau, append)
    fp.check(rc, "fpde_do_derivative")
    ctx.synchronize()                      # the kernel runs on the context's stream
    return DF.cpu().numpy()


@pytest.mark.parametrize("name", ["frdo_derivative", "frdo_derivative_kat"])
def test_do_derivative_matches_reference_and_oracle(ctx, name):
    g = fgv.load(golden_path(name))
    n, tau = int(g["N"]), g["tau"]
    Na = len(g["WA"])
    F = (np.arange(n) * tau) ** 2
    c = _do_weights(do_cases.orders(Na), do_cases.quad_weights(g["WA"]), g["gs"], tau, n)
    DF = _derivative(ctx, F[None, :], tau, c)[0]
    assert relmax(DF[1:], g["DF_do"][1:]) <= 1e-12
    DFo = oracle.do_derivative(F, tau, g["WA"], g["gs"])
    assert relmax(DF[1:], DFo[1:]) <= 1e-12
    if "analytic" in g:                        # fr_do's default run prints DOerr 0.000375753
        err = float(np.sqrt(np.sum((g["analytic"][1:] - DF[1:]) ** 2) / n))
        assert f"{err:.6g}" == "0.000375753"


@pytest.mark.parametrize("t0,j0,maxt", [(1, 0, -1), (32, 0, 31), (40, 31, 39), (8, -1, 7)])
def test_do_derivative_windows_many_nodes(ctx, t0, j0, maxt):
    rng = np.random.default_rng(t0 + 10 * (maxt + 1))
    nodes, ntau, tau, Na = 300, 48, 0.01, 16
    F = np.cumsum(rng.standard_normal((nodes, ntau)) * 0.1, axis=1)
    WA = rng.uniform(0.5, 1.5, Na) / (Na - 1)
    gs = do_cases.gammas(Na)
    c = _do_weights(do_cases.orders(Na), do_cases.quad_weights(WA), gs, tau, ntau)
    DF0 = rng.standard_normal((nodes, ntau))
    DF = _derivative(ctx, F, tau, c, t0, j0, maxt, DF0=DF0, append=1)
    ref = DF0.copy()
    for pt in range(nodes):
        d = oracle.do_derivative(F[pt], tau, WA, gs, maxt, t0, j0)
        ref[pt, t0:] += d[t0:]
    assert relmax(DF[:, t0:] - DF0[:, t0:], ref[:, t0:] - DF0[:, t0:]) <= 1e-12
    assert np.array_equal(DF[:, :t0], DF0[:, :t0])


def test_do_line_split_in_pieces(ctx):
    """The speculative solve with the explicit half restarted mid-block: a run split into
    pieces of 37, 64, 99 and 50 steps (launches that start inside a 64-step block, with the
    edge states taken from the stored state) against one run of all 250 steps. A restarted
    launch sums its first history rows in another float-float order, so the states agree to
    rounding, and both stay within 1e-7 of the oracle."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config3(N=3000, steps=250)
    A, B, R = p.coefs()
    c = fp.do_weights(p.orders, p.qw, p.tau, p.steps + 1, p.gnorm) / p.tau
    mk = lambda: fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, p.steps, lag_weights=c, theta=1.0, precision=3)
    line = mk()
    line.run(p.steps)
    u_one = line.state()
    line.close()
    line = mk()
    for m in (37, 64, 99, 50):
        line.run(m)
    u_pieces = line.state()
    line.close()
    uref, _ = oracle.line_run_general(p.u0, p.steps, c, 1.0, A, B, R)
    print(f"DO line in pieces: vs one run {relmax(u_pieces, u_one):.2e}, vs oracle {relmax(u_pieces, uref):.2e}")
    assert relmax(u_pieces, u_one) <= 1e-9
    assert relmax(u_pieces, uref) <= 1e-7
