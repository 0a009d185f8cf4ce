"""3D LOD path (fpde_lod3d_*) on the GPU against the reference's own run and the oracle.

  * replay of the reference's mode-3 run (fixture fpde_lod3d_a2: 6 x 4 x 8 intervals,
    alpha 0.85, 16 steps, the analytic test's Rp and boundary grids per step): every step's
    grid equals the reference's to 1e-12;
  * the benchmark form (lognormal k, zero-flux sides, Dirichlet top and bottom) on cubic and
    non-cubic grids against the oracle's LOD restatement: 1e-12 or 4x the oracle's one-ulp
    rounding envelope.
"""
import numpy as np
import pytest

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


def test_lod_replays_reference_run(ctx):
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_lod3d_a2"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    cA = np.stack([g["coefA_pass%d" % p] for p in range(3)])
    cB = np.stack([g["coefB_pass%d" % p] for p in range(3)])
    cR = np.stack([g["coefRlap_pass%d" % p] for p in range(3)])
    taus = g["tau"]
    assert np.all(taus == taus[0])
    steps = len(taus)
    lod = fp.Lod3D(ctx, dims, g["alpha"], taus[0], g["Da"], cA, cB, cR, g["U0"], steps,
                   source=g["Rp"], bc=g["BC"])
    worst = 0.0
    for n in range(steps):
        lod.run(1)
        worst = max(worst, relmax(lod.state(), g["U"][n]))
    lod.close()
    print(f"LOD replay 6x4x8, {steps} steps: max rel {worst:.2e}")
    assert worst <= 1e-12


def _envelope(p, cA, cB, cR):
    rng = np.random.default_rng(0)
    pert = lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))
    args = (None, None, p.left_kind, p.right_kind, p.dLN)
    u1 = oracle.lod_run(p.dims, p.u0, p.steps, p.tau, p.alpha, p.Da, cA, cB, cR, *args)
    u2 = oracle.lod_run(p.dims, p.u0, p.steps, p.tau, p.alpha, p.Da, pert(cA), pert(cB), pert(cR), *args)
    return u1, relmax(u2, u1)


@pytest.mark.parametrize("dims,steps", [((20, 20, 20), 40), ((24, 12, 18), 33)])
def test_lod_benchmark_form_vs_oracle(ctx, dims, steps):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    base = problems.config4(n=max(dims), steps=steps)
    sN, M, K = dims
    p = problems.LodProblem("lod", dims, base.alpha, base.tau, steps, base.k[:K + 2, :M + 2, :sN + 2].copy(),
                            base.u0[:K + 2, :M + 2, :sN + 2].copy(), base.left_kind, base.right_kind)
    p.u0[K:] = 0.0
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, steps, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN)
    lod.run(steps)
    u = lod.state()
    lod.close()
    uref, env = _envelope(p, cA, cB, cR)
    err = relmax(u, uref)
    print(f"LOD {dims} {steps} steps vs oracle: {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(1e-12, 4 * env)


def test_lod_runs_in_pieces_and_solve_host(ctx):
    """Two runs of 10 steps equal one of 20; the host end-to-end call equals both."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=16, steps=20)
    cA, cB, cR = p.coefs()
    kw = dict(left_kind=p.left_kind, right_kind=p.right_kind, dLN=p.dLN)
    lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, 20, **kw)
    lod.run(10)
    lod.run(10)
    u_two = lod.state()
    out = np.zeros_like(p.u0)
    lod.solve_host(p.u0, 20, out)
    lod.close()
    assert np.array_equal(u_two, out)


@pytest.mark.parametrize("steps,tol", [(64, 1e-12), (230, 1e-7)])
def test_lod_split_history_vs_fp64(ctx, steps, tol):
    """Split path (far history as exact bf16 slices on the tensor cores, near history and
    passes in FP64): equal to the FP64 path within one block, within 1e-7 across blocks."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=20, steps=steps)
    cA, cB, cR = p.coefs()
    kw = dict(left_kind=p.left_kind, right_kind=p.right_kind, dLN=p.dLN)
    out = []
    for prec in (0, 3):
        lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, steps, precision=prec, **kw)
        lod.run(steps)
        out.append(lod.state())
        lod.close()
    err = relmax(out[1], out[0])
    print(f"LOD 20^3 {steps} steps, split x3 vs FP64: max rel {err:.2e}")
    assert err <= tol


@pytest.mark.parametrize("dims,steps", [((129, 6, 5), 12), ((141, 5, 7), 10)])
def test_lod_long_lines_vs_oracle(ctx, dims, steps):
    """Lines of exactly 4 x 32 interior nodes (the segmented pass at its limit) and longer lines
    (the one-thread-per-line pass) in the same grid as short ones: every pass against the
    oracle's LOD restatement, 1e-12 or 4x its one-ulp rounding envelope."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    base = problems.config4(n=max(dims), steps=steps)
    sN, M, K = dims
    p = problems.LodProblem("lod", dims, base.alpha, base.tau, steps, base.k[:K + 2, :M + 2, :sN + 2].copy(),
                            base.u0[:K + 2, :M + 2, :sN + 2].copy(), base.left_kind, base.right_kind)
    p.u0[K:] = 0.0
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, steps, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN)
    lod.run(steps)
    u = lod.state()
    lod.close()
    uref, env = _envelope(p, cA, cB, cR)
    err = relmax(u, uref)
    print(f"LOD {dims} {steps} steps vs oracle: {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(1e-12, 4 * env)


def test_lod_restricted_replays_reference_run(ctx):
    """The reference's own mode-3 column run with restricted summing (sum_alg 1, sum_param
    0.05: the 8 newest lags) replayed by the GPU LOD with restrict_eps = 0.05, every level to
    1e-12. The run is the column problem of fpde_column_a2 (coefficient grids, sources and
    boundary values recorded there)."""
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_column_alg1"))
    a2 = fgv.load(golden_path("fpde_column_a2"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    cA = np.stack([a2["coefA_pass%d" % p] for p in range(3)])
    cB = np.stack([a2["coefB_pass%d" % p] for p in range(3)])
    cR = np.stack([a2["coefRlap_pass%d" % p] for p in range(3)])
    taus = g["tau"]
    steps = len(taus)
    lod = fp.Lod3D(ctx, dims, g["alpha"], taus[0], a2["Da"], cA, cB, cR, g["U0"], steps, source=a2["Rp"],
                   bc=a2["BC"], restrict_eps=g["sum_param"])
    worst = 0.0
    for n in range(steps):
        lod.run(1)
        worst = max(worst, relmax(lod.state(), g["U"][n]))
    lod.close()
    print(f"LOD restricted replay (sum_alg 1), {steps} steps: max rel {worst:.2e}")
    assert worst <= 1e-12


@pytest.mark.parametrize("max_lag", [0, 10, 70])
def test_lod_restricted_split_vs_fp64(ctx, max_lag):
    """The three-slice split LOD with a history window against the FP64 LOD with the same
    window (far contraction from the first tile the window reaches), 150 steps."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=24, steps=150)
    cA, cB, cR = p.coefs()
    b = fp.weights_l1_lags(p.alpha, p.steps + 2)
    kkk0 = p.tau ** (1 - p.alpha) / (1 - p.alpha)
    eps = 0.5 * kkk0 * (b[max_lag] + b[max_lag + 1])
    out = []
    for prec in (0, 3):
        lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, p.steps, left_kind=p.left_kind,
                       right_kind=p.right_kind, dLN=p.dLN, precision=prec, restrict_eps=eps)
        lod.run(p.steps)
        out.append(lod.state())
        lod.close()
    err = relmax(out[1], out[0])
    print(f"LOD 24^3 restricted to {max_lag} lags: split vs FP64 {err:.2e}")
    assert err <= 1e-7


def test_lod_series_replays_reference_run(ctx):
    """The reference's own mode-3 column run with the series expansion (sum_alg 2, 16 moments)
    replayed by the GPU LOD with series_terms = 16 (moments carried on the device, the step's
    coefficients in closed form for g(t) = t), every level to 1e-12. The run is the column
    problem of fpde_column_a2 (coefficient grids, sources and boundary values recorded there)."""
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_column_alg2"))
    a2 = fgv.load(golden_path("fpde_column_a2"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    cA = np.stack([a2["coefA_pass%d" % p] for p in range(3)])
    cB = np.stack([a2["coefB_pass%d" % p] for p in range(3)])
    cR = np.stack([a2["coefRlap_pass%d" % p] for p in range(3)])
    taus = g["tau"]
    steps = len(taus)
    lod = fp.Lod3D(ctx, dims, g["alpha"], taus[0], a2["Da"], cA, cB, cR, g["U0"], steps, source=a2["Rp"],
                   bc=a2["BC"], series_terms=int(g["sum_param"]))
    worst = 0.0
    for n in range(steps):
        lod.run(1)
        worst = max(worst, relmax(lod.state(), g["U"][n]))
    lod.close()
    print(f"LOD series replay (sum_alg 2), {steps} steps: max rel {worst:.2e}")
    assert worst <= 1e-12


def test_lod_series_runs_in_pieces(ctx):
    """A series-expansion LOD run in one call equals the same run in pieces (the moments
    persist across graphs) and after a reset (the moments restart from zero)."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=20, steps=30)
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, p.steps, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN, series_terms=12)
    lod.run(30)
    u_one = lod.state()
    lod.reset(p.u0)
    for m in (7, 13, 10):
        lod.run(m)
    np.testing.assert_array_equal(lod.state(), u_one)
    lod.close()


@pytest.mark.parametrize("segments", [(4, 4, 4), (8, 8, 8), (16, 16, 16), (32, 32, 32), (4, 16, 32)])
def test_lod_segment_counts_vs_oracle(ctx, segments):
    """Every segment count of the Thomas passes (fpde_lod3d_desc.segments) gives the oracle's run
    (the segments join by exact affine scans; only the rounding order differs)."""
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    dims, steps = (24, 12, 18), 33
    base = problems.config4(n=max(dims), steps=steps)
    sN, M, K = dims
    p = problems.LodProblem("lod", dims, base.alpha, base.tau, steps, base.k[:K + 2, :M + 2, :sN + 2].copy(),
                            base.u0[:K + 2, :M + 2, :sN + 2].copy(), base.left_kind, base.right_kind)
    p.u0[K:] = 0.0
    cA, cB, cR = p.coefs()
    lod = fp.Lod3D(ctx, dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, steps, left_kind=p.left_kind,
                   right_kind=p.right_kind, dLN=p.dLN, segments=segments)
    lod.run(steps)
    u = lod.state()
    lod.close()
    uref, env = _envelope(p, cA, cB, cR)
    err = relmax(u, uref)
    print(f"LOD {dims} segments {segments}: {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(1e-12, 4 * env)


def test_lod_autotune_and_bad_segments(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=40, steps=40)
    cA, cB, cR = p.coefs()
    seg, ms = fp.autotune_lod3d(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, 40, 40, left_kind=p.left_kind,
                                right_kind=p.right_kind, dLN=p.dLN, precision=fp.FPDE_PREC_SPLIT_BF16X3)
    print(f"LOD 40^3 autotune: segments {seg}, {ms:.4f} ms per step")
    assert all(s in (0, 4, 8, 16, 32) for s in seg) and ms > 0
    for bad in ((3, 0, 0), (0, 0, 64), (1, 1, 1)):
        with pytest.raises(fp.FpdeError) as e:
            fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, 8, left_kind=p.left_kind,
                     right_kind=p.right_kind, dLN=p.dLN, segments=bad)
        assert e.value.code == 1
    shape = (6, 6, 202)                               # 4 segments of more than 32 nodes: 200 intervals
    z = np.zeros((3,) + shape)
    with pytest.raises(fp.FpdeError) as e:
        fp.Lod3D(ctx, (200, 4, 4), p.alpha, p.tau, p.Da, z, z, z, np.zeros(shape), 2, segments=(4, 0, 0))
    assert e.value.code == 1
