"""The fully implicit 3D space-fractional scheme on the GPU (fpde_sf3d_matvec, fpde_sf3d_solve and the
LOD with space_frac.implicit3d) against the reference's own runs and the oracle.

The product forms every output with the reference's operations in its order (vmul_T_3d,
fpde_hpc_1d.cpp:6801-8722), so it equals the reference's bit for bit. The solve with exact dot
products adds every dot product in index order on one thread, as solve_mln<1> does, so its iterates,
iteration count and solution are the reference's bit for bit; the fast form sums its dot products in
a fixed tree and its Toeplitz terms as fused multiply-adds, and is compared within the reference's own
sensitivity: ten times how far the oracle (bitwise the reference) moves when the right-hand side
changes by 1e-15."""
import numpy as np
import pytest

import oracle
import sf3d_cases
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_matvec_bitwise_vs_reference(ctx, name):
    c = sf3d_cases.load(name)
    g = c["g"]
    r = ctx.sf3d_matvec(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["mv_x"], iw=c["iw3"],
                        space_der=c["space_der"])
    assert np.array_equal(r, g["mv_r"])


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_exact_solve_bitwise_vs_reference(ctx, name):
    c = sf3d_cases.load(name)
    g = c["g"]
    x, it = ctx.sf3d_solve(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["sys_last_om"], g["solve_x0"],
                           c["thr"], c["maxiter"], iw=c["iw3"], space_der=c["space_der"], exact=True)
    assert it == c["solve_iters"]
    assert np.array_equal(x, g["solve_sol"])


def _solve_envelope(c, B, x0, rel):
    g = c["g"]
    x, _ = oracle.sf3d_solve(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], B * (1.0 + rel), x0, c["thr"],
                             c["maxiter"], iw=c["iw3"], space_der=c["space_der"])
    return relmax(x, g["solve_sol"])


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_fast_solve_vs_reference(ctx, name):
    c = sf3d_cases.load(name)
    g = c["g"]
    B, x0 = g["sys_last_om"], g["solve_x0"]
    env = max(_solve_envelope(c, B, x0, 1e-15), _solve_envelope(c, B, x0, -1e-15))
    x, it = ctx.sf3d_solve(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], B, x0, c["thr"], c["maxiter"],
                           iw=c["iw3"], space_der=c["space_der"])
    assert it >= 1
    assert relmax(x, g["solve_sol"]) <= max(10.0 * env, 1e-12), env


def _random_system(dims, seed, sd):
    """A diagonally dominant 7-diagonal part, Mcoefs of second differences with random weights, iw
    in [1, 1.5], decaying Toeplitz rows."""
    sN, M, K = dims
    V = (sN + 2) * (M + 2) * (K + 2) + 1
    rng = np.random.default_rng(seed)
    mat = np.zeros((7, V))
    off = [0, 2, 3, 4, 5, 6]
    for d in off:
        mat[d] = 0.5 + rng.random(V)
    mat[1] = -(mat[off].sum(axis=0) + 20.0 + 10.0 * rng.random(V))
    mc = np.zeros((9, V))
    for cax in range(3):
        lo, hi = 0.5 + rng.random(V), 0.5 + rng.random(V)
        mc[3 * cax], mc[3 * cax + 2], mc[3 * cax + 1] = lo, hi, -(lo + hi)
    iw = 1.0 + 0.5 * rng.random((3, V))
    Tm = []
    for nl in dims:
        t = np.zeros(nl + 1)
        k = np.arange(2, nl + 1)
        t[2:] = 0.2 * (k ** 0.3 - (k - 1) ** 0.3)
        Tm.append(t)
    x = rng.standard_normal(V)
    B = rng.standard_normal(V)
    return mat, mc, Tm, iw, x, B


@pytest.mark.parametrize("sd", [0, 1])
@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 5, 6), (5, 2, 7), (6, 5, 2), (5, 3, 7), (24, 20, 28)])
def test_random_bitwise_vs_oracle(ctx, dims, sd):
    """Grids with an axis of 1 or 2 intervals (that axis's neighbours and Toeplitz term are skipped,
    :6859-6876) and a larger one: product and exact solve bit for bit against the oracle, the fast
    solve to 1e-10 of the converged solution."""
    mat, mc, Tm, iw, x, B = _random_system(dims, 11 * sum(dims) + sd, sd)
    r = ctx.sf3d_matvec(dims, mat, mc, Tm, x, iw=iw, space_der=sd)
    ro = oracle.sf3d_matvec(dims, mat, mc, Tm, x, iw=iw, space_der=sd)
    assert np.array_equal(r, ro)
    xe, ite = ctx.sf3d_solve(dims, mat, mc, Tm, B, x, 1e-26, 200, iw=iw, space_der=sd, exact=True)
    xo, ito = oracle.sf3d_solve(dims, mat, mc, Tm, B, x, 1e-26, 200, iw=iw, space_der=sd)
    assert ite == ito and np.array_equal(xe, xo)
    xf, itf = ctx.sf3d_solve(dims, mat, mc, Tm, B, x, 1e-26, 200, iw=iw, space_der=sd)
    assert itf >= 1 and relmax(xf, xo) <= 1e-10


def test_row_scaling_and_device_buffers(ctx):
    import torch
    dims = (7, 6, 9)
    mat, mc, Tm, iw, x, B = _random_system(dims, 5, 1)
    rs = 1.0 + np.random.default_rng(6).random(x.size)
    r_host = ctx.sf3d_matvec(dims, mat, mc, Tm, x, iw=iw, rs=rs, space_der=1)
    assert np.array_equal(r_host, oracle.sf3d_matvec(dims, mat, mc, Tm, x, iw=iw, rs=rs, space_der=1))
    t = lambda a: torch.tensor(a, device="cuda")
    r_dev = ctx.sf3d_matvec(dims, t(mat), t(mc), [t(v) for v in Tm], t(x), iw=t(iw), rs=t(rs), space_der=1)
    assert np.array_equal(r_dev.cpu().numpy(), r_host)
    xd, itd = ctx.sf3d_solve(dims, t(mat), t(mc), [t(v) for v in Tm], t(B), t(x), 1e-24, 100, iw=t(iw), space_der=1,
                             exact=True)
    xh, ith = ctx.sf3d_solve(dims, mat, mc, Tm, B, x, 1e-24, 100, iw=iw, space_der=1, exact=True)
    assert itd == ith and np.array_equal(xd.cpu().numpy(), xh)


@pytest.mark.parametrize("exact", [False, True])
def test_breakdown_is_bounded_and_reported(ctx, exact):
    """A zero operator makes solve_mln<1> restart for ever (c[1] = 0 every time); the solve stops after
    max_iter restarts in a row and reports FPDE_ERR_NUMERIC; a zero right-hand side is solved at once."""
    import fpde_hpc_gb300 as fp
    dims = (3, 3, 3)
    V = 5 * 5 * 5 + 1
    z7, z9, zT = np.zeros((7, V)), np.zeros((9, V)), [np.zeros(4)] * 3
    with pytest.raises(fp.FpdeError) as e:
        ctx.sf3d_solve(dims, z7, z9, zT, np.ones(V), np.zeros(V), 1e-12, 5, exact=exact)
    assert e.value.code == 7
    x, it = ctx.sf3d_solve(dims, z7, z9, zT, np.zeros(V), np.zeros(V), 1e-12, 5, exact=exact)
    assert it == 1


def test_bad_arguments_are_errors(ctx):
    import fpde_hpc_gb300 as fp
    dims = (3, 3, 3)
    V = 5 * 5 * 5 + 1
    with pytest.raises(ValueError):
        ctx.sf3d_matvec(dims, np.zeros((7, V - 1)), np.zeros((9, V)), [np.zeros(4)] * 3, np.zeros(V))
    with pytest.raises(fp.FpdeError) as e:
        ctx.sf3d_matvec(dims, np.zeros((7, V)), np.zeros((9, V)), [np.zeros(4)] * 3, np.zeros(V), space_der=2)
    assert e.value.code == 1


def _lod(ctx, c, exact):
    import fpde_hpc_gb300 as fp
    g = c["g"]
    sf = dict(space_der=c["space_der"], tol=c["thr"], max_iter=c["maxiter"], Tm=[c["Tm"][p] for p in range(3)],
              mc=[c["mc"][p] for p in range(3)], iw=[c["iw"][p] for p in range(3)], implicit3d=1,
              exact=1 if exact else 0)
    ends = {} if c["rkind"] is None else dict(right_kind=c["rkind"], dLN=c["dLN"])
    return fp.Lod3D(ctx, c["dims"], float(g["alpha"]), float(g["tau"][0]), c["Da"], c["coefA"], c["coefB"],
                    c["coefRlap"], g["U0"], c["steps"], source=g["Rp"], bc=g["BC"], space_frac=sf, **ends)


def _lod_envelope(c, rel):
    """How far the reference's implicit3d run moves when its source is scaled by 1 + rel (the oracle
    replays it bit for bit)."""
    g = c["g"]
    U = g["U0"].reshape(-1).copy()
    hist = np.zeros((c["steps"], c["G"]))
    ue, worst = 0.0, 0.0
    for n in range(c["steps"]):
        ue, *_ = oracle.lod_step_sf3d(c["dims"], U, ue, hist, n, c["kb_rows"][n], g["tau"], c["Da"],
                                      float(g["kkk0"][n]), c["coefA"], c["coefB"], c["coefRlap"], c["mc"], c["iw"],
                                      c["Tm"], c["space_der"], c["thr"], c["maxiter"], g["Rp"][n] * (1.0 + rel),
                                      g["BC"][n], rkind=c["rkind"], dLN=c["dLN"])
        worst = max(worst, relmax(U, g["U"][n].reshape(-1)))
    return worst


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_lod_implicit3d_vs_reference(ctx, name, exact):
    """The whole run: the GPU's history sum and its uniform-step kkk0 differ from the reference's in the
    last bits and the solver carries that, so the bar is ten times the reference's own response to a
    1e-15 change of its source, and 1e-12."""
    c = sf3d_cases.load(name)
    g = c["g"]
    env = max(_lod_envelope(c, 1e-15), _lod_envelope(c, -1e-15))
    lod = _lod(ctx, c, exact)
    worst = 0.0
    for n in range(c["steps"]):
        lod.run(1)
        worst = max(worst, relmax(lod.state().reshape(-1), g["U"][n].reshape(-1)))
    assert lod.sf_iterations() >= c["steps"]
    lod.close()
    assert worst <= max(10.0 * env, 1e-12), (worst, env)


@pytest.mark.parametrize("sd", [0, 1])
def test_lod_implicit3d_larger_grid_vs_oracle(ctx, sd):
    """16 x 12 x 20 cells, 6 steps, tight threshold: the GPU's fast solves against the oracle's
    replay (bitwise the reference's scheme) within ten times the oracle's 1e-15 response."""
    import fpde_hpc_gb300 as fp
    from test_gpu_spacefrac import _synthetic
    dims, alpha, tau, steps, thr, mx = (16, 12, 20), 0.7, 1e-3, 6, 1e-24, 400
    coefA, coefB, coefR, mc, iw, Tm, rp, u0 = _synthetic(dims, 0.75, 21 + sd)
    Da = 1.0 / fp.gamma(1.0 - alpha)
    sf = dict(space_der=sd, tol=thr, max_iter=mx, Tm=list(Tm), mc=list(mc), iw=list(iw), implicit3d=1)
    lod = fp.Lod3D(ctx, dims, alpha, tau, Da, coefA, coefB, coefR, u0, steps, source=rp, space_frac=sf)
    t = oracle.time_points(np.full(steps, tau))
    bc = np.zeros_like(u0)
    G = u0.size

    def oracle_run(scale):
        U = u0.reshape(-1).copy()
        hist = np.zeros((steps, G))
        out = []
        for n in range(steps):
            kb, k0 = oracle.l1_weights(alpha, t, n)
            oracle.lod_step_sf3d(dims, U, 0.0, hist, n, kb, np.full(steps, tau), Da, k0, coefA, coefB, coefR, mc, iw,
                                 Tm, sd, thr, mx, rp * scale, bc)
            out.append(U.copy())
        return out

    ref = oracle_run(1.0)
    env = max(max(relmax(a, b) for a, b in zip(oracle_run(1.0 + 1e-15), ref)),
              max(relmax(a, b) for a, b in zip(oracle_run(1.0 - 1e-15), ref)))
    worst = 0.0
    for n in range(steps):
        lod.run(1)
        worst = max(worst, relmax(lod.state().reshape(-1), ref[n]))
    lod.close()
    assert worst <= max(10.0 * env, 1e-12), (worst, env)


@pytest.mark.parametrize("exact", [False, True])
def test_lod_implicit3d_graph_replay(ctx, exact):
    """A run of 130 steps is captured as a CUDA graph (the cooperative solve inside it); it must equal
    130 single-step runs (enqueued directly) bit for bit: the dot products are deterministic."""
    import fpde_hpc_gb300 as fp
    from test_gpu_spacefrac import _synthetic
    dims, alpha, tau, steps = (8, 6, 10), 0.75, 1e-3, 130
    coefA, coefB, coefR, mc, iw, Tm, rp, u0 = _synthetic(dims, 0.7, 5)
    Da = 1.0 / fp.gamma(1.0 - alpha)
    sf = dict(space_der=1, tol=1e-20, max_iter=300, Tm=list(Tm), mc=list(mc), iw=list(iw), implicit3d=1,
              exact=1 if exact else 0)
    out = []
    for chunk in (steps, 1):
        lod = fp.Lod3D(ctx, dims, alpha, tau, Da, coefA, coefB, coefR, u0, steps, source=rp, space_frac=sf)
        for _ in range(steps // chunk):
            lod.run(chunk)
        out.append((lod.state(), lod.sf_iterations()))
        lod.close()
    assert out[0][1] == out[1][1] and out[0][1] >= steps
    assert np.array_equal(out[0][0], out[1][0])
