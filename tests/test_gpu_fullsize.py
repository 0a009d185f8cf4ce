"""Parity at the benchmark configurations' own spatial sizes, at 8 checkpoints.

Each benchmark configuration runs at its full size in space with a truncated step count that
still crosses several 64-step blocks (and, on the split paths, the 256-step super-blocks of the
far history):
  config 2: 1D line, N = 65,536, 512 steps;
  config 3: distributed-order line, N = 16,384, 256 steps;
  config 4: 3D LOD, 128^3, 130 steps;
  config 5: all 512 columns of the ensemble, 130 steps.
The run is taken in eight pieces; after each piece (the checkpoints) the state is compared
  * FP64 path vs the oracle: 1e-12, or 4x the oracle's one-ulp rounding envelope where that is
    larger (long fine lines are ill-conditioned: a one-ulp change of the coefficients moves the
    oracle's own result by ~2e-10 at N = 65,536); both numbers are printed;
  * split bf16x3 path vs the FP64 path and vs the oracle: 1e-7 (max relative, normwise), with
    the RMS relative error printed beside it.
"""
import numpy as np
import pytest

import oracle
from conftest import relmax

pytestmark = pytest.mark.gpu
RTOL, SPLIT_TOL = 1e-12, 1e-7


def relrms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.max(np.abs(b)), 1e-300))


def checkpoints(steps):
    return [int(round((k + 1) * steps / 8)) for k in range(8)]


def states_from_increments(u0, hist, cps):
    """Oracle states at the checkpoints from its increment rows, added in step order."""
    u, out, t = np.array(u0, dtype=np.float64), [], 0
    for c in cps:
        for r in range(t, c):
            u += hist[r, :len(u)]
        t = c
        out.append(u.copy())
    return out


def pert(rng):
    return lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _pieces(obj, cps, state):
    out, t = [], 0
    for c in cps:
        obj.run(c - t)
        t = c
        out.append(state())
    return out


def _report(name, cps, fp64, split, ora, env):
    worst_f, worst_s, worst_so = 0.0, 0.0, 0.0
    for k, c in enumerate(cps):
        ef, es, eso = relmax(fp64[k], ora[k]), relmax(split[k], fp64[k]), relmax(split[k], ora[k])
        print(f"{name} step {c:4d}: FP64 vs oracle {ef:.2e} (envelope {env[k]:.2e}); split vs FP64 {es:.2e} "
              f"(rms {relrms(split[k], fp64[k]):.2e}), split vs oracle {eso:.2e}")
        assert ef <= max(RTOL, 4 * env[k]), (c, ef, env[k])
        assert es <= SPLIT_TOL and eso <= SPLIT_TOL, (c, es, eso)
        worst_f, worst_s, worst_so = max(worst_f, ef), max(worst_s, es), max(worst_so, eso)
    print(f"{name}: worst FP64 vs oracle {worst_f:.2e}, split vs FP64 {worst_s:.2e}, split vs oracle {worst_so:.2e}")


def test_config2_line_65536_nodes(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    S = 512
    p = problems.config2(N=65536, steps=S)
    A, B, R = p.coefs()
    cps = checkpoints(S)
    runs = []
    for prec in (0, 3):
        line = fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, S, precision=prec)
        runs.append(_pieces(line, cps, line.state))
        line.close()
    _, hist = oracle.line_run(p.u0, S, p.tau, p.alpha, p.Da, A, B, R)
    ora = states_from_increments(p.u0, hist, cps)
    f = pert(np.random.default_rng(0))
    _, hist2 = oracle.line_run(p.u0, S, p.tau, p.alpha, p.Da, f(A), f(B), f(R))
    env = [relmax(x, y) for x, y in zip(states_from_increments(p.u0, hist2, cps), ora)]
    _report("config 2 (N=65536)", cps, runs[0], runs[1], ora, env)


def test_config3_do_line_16384_nodes(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    S = 256
    p = problems.config3(N=16384, steps=S)
    A, B, R = p.coefs()
    c = fp.do_weights(p.orders, p.qw, p.tau, S + 1, p.gnorm)
    cps = checkpoints(S)
    runs = []
    for prec in (0, 3):
        line = fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, S, lag_weights=c / p.tau, theta=1.0,
                       precision=prec)
        runs.append(_pieces(line, cps, line.state))
        line.close()
    _, hist = oracle.line_run_general(p.u0, S, c / p.tau, 1.0, A, B, R)
    ora = states_from_increments(p.u0, hist, cps)
    f = pert(np.random.default_rng(0))
    _, hist2 = oracle.line_run_general(p.u0, S, f(c / p.tau), 1.0, f(A), f(B), f(R))
    env = [relmax(x, y) for x, y in zip(states_from_increments(p.u0, hist2, cps), ora)]
    _report("config 3 (DO, N=16384)", cps, runs[0], runs[1], ora, env)


def _lod_oracle(p, cA, cB, cR, S, cps):
    U = p.u0.copy()
    G = U.shape
    hist = np.zeros((S,) + G)
    taus = np.full(S + 1, p.tau)
    tp = oracle.time_points(taus)
    bc = np.zeros(G)
    out = []
    for n in range(S):
        kb, k0 = oracle.l1_weights(p.alpha, tp, n)
        oracle.lod_step(p.dims, U, hist, n, kb if n else np.zeros(1), taus, p.Da, k0, cA, cB, cR, None, bc,
                        p.left_kind, p.right_kind, p.dLN)
        if n + 1 in cps:
            out.append(U.copy())
    return out


def test_config4_lod_128_cubed(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    S = 130
    p = problems.config4(n=128, steps=S)
    cA, cB, cR = p.coefs()
    cps = checkpoints(S)
    runs = []
    for prec in (0, 3):
        lod = fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, S, left_kind=p.left_kind,
                       right_kind=p.right_kind, dLN=p.dLN, precision=prec)
        runs.append(_pieces(lod, cps, lod.state))
        lod.close()
    ora = _lod_oracle(p, cA, cB, cR, S, cps)
    f = pert(np.random.default_rng(0))
    env = [relmax(x, y) for x, y in zip(_lod_oracle(p, f(cA), f(cB), f(cR), S, cps), ora)]
    _report("config 4 (128^3)", cps, runs[0], runs[1], ora, env)


def test_config5_ensemble_512_columns(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    S = 130
    probs = problems.config5(n_cols=512, steps=S)
    cols = []
    for q in probs:
        A, B, R = q.coefs()
        cols.append(dict(N=q.N, alpha=q.alpha, tau=q.tau, Da=q.Da, A=A, B=B, Rlap=R, u0=q.u0, left=(0, 0.0),
                         right=(0, 0.0), dLN=1.0 / q.N))
    cps = checkpoints(S)
    runs = []
    for prec in (0, 3):
        b = fp.Batch(ctx, cols, S, precision=prec)
        runs.append(_pieces(b, cps, lambda: [b.state(i) for i in range(len(cols))]))
        b.close()
    ora = [[] for _ in cps]
    env = [[] for _ in cps]
    rng = np.random.default_rng(0)
    for i, c in enumerate(cols):
        _, hist = oracle.line_run(c["u0"], S, c["tau"], c["alpha"], c["Da"], c["A"], c["B"], c["Rlap"])
        f = pert(rng)
        _, hist2 = oracle.line_run(c["u0"], S, c["tau"], c["alpha"], c["Da"], f(c["A"]), f(c["B"]), f(c["Rlap"]))
        for k, (x, y) in enumerate(zip(states_from_increments(c["u0"], hist, cps),
                                       states_from_increments(c["u0"], hist2, cps))):
            ora[k].append(x)
            env[k].append(relmax(y, x))
    # per column and checkpoint; the report gives the worst column of each checkpoint
    worst = {"f": [0.0] * 8, "s": [0.0] * 8, "so": [0.0] * 8}
    for k in range(8):
        for i in range(len(cols)):
            ef = relmax(runs[0][k][i], ora[k][i])
            assert ef <= max(RTOL, 4 * env[k][i]), (k, i, cols[i]["N"], ef, env[k][i])
            es, eso = relmax(runs[1][k][i], runs[0][k][i]), relmax(runs[1][k][i], ora[k][i])
            assert es <= SPLIT_TOL and eso <= SPLIT_TOL, (k, i, es, eso)
            worst["f"][k], worst["s"][k], worst["so"][k] = (max(worst["f"][k], ef), max(worst["s"][k], es),
                                                            max(worst["so"][k], eso))
        print(f"config 5 (512 columns) step {cps[k]:4d}: FP64 vs oracle {worst['f'][k]:.2e} (largest column "
              f"envelope {max(env[k]):.2e}); split vs FP64 {worst['s'][k]:.2e}, split vs oracle {worst['so'][k]:.2e}")
