"""Generalized-kernel L1 weights on the device (fpde_weights_g) against 40-digit values, the
oracle's quadrature and the closed form of the linear kernel:

  * the six reference time grids (g(t) = sqrt(t), t^2, t^1.5; uniform and variable steps),
    every weight of 40 steps in one call, to 2e-15 of the exact integrals;
  * sweeps of p (0.5 .. 3) and alpha (0 .. 1, including the reference's alpha = 1 rule) on a
    variable-step grid with rows up to 300 steps, to 1e-14 of the oracle;
  * p = 1 equals the L1 closed form; host and device buffers agree; bad arguments are
    reported as FPDE_ERR_ARG.
"""
import numpy as np
import pytest

import fgv
import oracle
from conftest import golden_path

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("fk,p,suf", [(1, 0.5, ""), (1, 0.5, "_vartau"), (2, 2.0, ""), (2, 2.0, "_vartau"),
                                      (3, 1.5, ""), (3, 1.5, "_vartau")])
def test_weights_g_vs_exact(ctx, fk, p, suf):
    ex = fgv.load(golden_path("fpde_weights_g_exact"))
    time, rows = ex[f"fk{fk}{suf}_time"], ex[f"fk{fk}{suf}_rows"]
    alpha = fgv.load(golden_path(f"fpde_weights_fk{fk}{suf}"))["alpha"]
    ns = rows.shape[0]
    W = ctx.weights_g(p, alpha, time, 0, ns - 1)
    mask = np.tril(np.ones((ns, ns), dtype=bool))
    err = np.max(np.abs(W[mask] - rows[mask]) / rows[mask])
    print(f"fk{fk}{suf}: max rel vs 40-digit values {err:.2e}")
    assert err <= 2e-15


@pytest.mark.parametrize("p", [0.5, 1.0, 1.5, 2.0, 3.0])
@pytest.mark.parametrize("alpha", [0.0, 0.05, 0.5, 0.9, 1.0])
def test_weights_g_vs_oracle(ctx, p, alpha):
    rng = np.random.default_rng(int(p * 10 + alpha * 100))
    time = oracle.time_points(1e-3 * (0.3 + rng.random(301)))
    n0, n1 = 250, 299
    W = ctx.weights_g(p, alpha, time, n0, n1)
    worst = 0.0
    for n in (n0, n0 + 7, n1):
        kb, k0 = oracle.weights_g(p, alpha, time, n)
        ref = np.append(kb, k0)
        got = W[n - n0, :n + 1]
        if alpha == 1.0:
            np.testing.assert_array_equal(got, ref)
            continue
        worst = float(np.maximum(worst, float(np.max(np.abs(got - ref) / np.abs(ref)))))
    assert worst <= 1e-14, worst
    assert np.all(W[0, n0 + 1:] == 0.0)                  # entries past t = n untouched


def test_weights_g_linear_kernel_and_device_buffers(ctx):
    import torch
    rng = np.random.default_rng(8)
    time = oracle.time_points(1e-3 * (0.5 + rng.random(1025)))
    Wh = ctx.weights_g(1.0, 0.7, time, 0, 1023)
    for n in (0, 1, 100, 1023):
        kc, kc0 = oracle.l1_weights(0.7, time, n)
        got = Wh[n, :n + 1]
        ref = np.append(kc, kc0)
        assert np.max(np.abs(got - ref) / ref) <= 1e-14
    Wd = ctx.weights_g(1.0, 0.7, torch.from_numpy(time).cuda(), 0, 1023)
    np.testing.assert_array_equal(Wd.cpu().numpy(), Wh)


FPDE_ERR_ARG = 1


def test_weights_g_bad_arguments(ctx):
    time = np.linspace(0.0, 1.0, 12)
    out = np.zeros((3, 11))
    lib = ctx.lib
    import ctypes as C
    p_t, p_o = time.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)
    assert lib.fpde_weights_g(ctx.h, 0.0, 0.5, p_t, 8, 10, p_o, 11, 0) == FPDE_ERR_ARG      # p <= 0
    assert lib.fpde_weights_g(ctx.h, 1.0, 1.5, p_t, 8, 10, p_o, 11, 0) == FPDE_ERR_ARG      # alpha > 1
    assert lib.fpde_weights_g(ctx.h, 1.0, 0.5, p_t, 8, 10, p_o, 10, 0) == FPDE_ERR_ARG      # ld < n1 + 1
    assert lib.fpde_weights_g(ctx.h, 1.0, 0.5, p_t, 9, 8, p_o, 11, 0) == FPDE_ERR_ARG       # n1 < n0


@pytest.mark.parametrize("p", [0.5, 1.5, 3.0])
def test_weights_g_rows_sum_to_the_beta_integral(ctx, p):
    """Every row (a step's weights and its local weight) covers [0, T]: the row sums equal
    T^(1 - p alpha) B(1/p, 1 - alpha) / p, for 200 rows of a random variable-step grid."""
    from scipy.special import beta
    rng = np.random.default_rng(int(10 * p))
    time = oracle.time_points(1e-2 * (0.2 + rng.random(201)))
    alpha = 0.7
    W = ctx.weights_g(p, alpha, time, 0, 199)
    T = time[1:201]
    exact = T ** (1.0 - p * alpha) * beta(1.0 / p, 1.0 - alpha) / p
    err = np.max(np.abs(W.sum(axis=1) - exact) / exact)
    assert err <= 1e-14, err
