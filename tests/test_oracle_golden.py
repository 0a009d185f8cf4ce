"""Pins the CPU oracle to the reference's own FP64 code.

The fixtures in tests/golden were produced by running the reference (fpde_hpc_1d.cpp,
fr_do.cpp) through the harnesses in oracle/ref_pin (regenerate with
tests/golden/make_golden.py). Tolerances: 1e-12 relative wherever the oracle is given
the reference's own weights (identical arithmetic up to operation order), and 1e-12 for
the closed-form weights against the reference's series at EPS 1e-15.
"""
import os
import subprocess

import numpy as np
import pytest

import fgv
import oracle
from conftest import ROOT, golden_path
from conftest import relmax as _relmax

RTOL = 1e-12


def _weights_of(g, n):
    off = g["kb_off"].astype(int)
    return g["kb_flat"][off[n]:off[n + 1]]


@pytest.mark.parametrize("name", ["fpde_weights_long", "fpde_weights_vartau", "fpde_column_a2",
                                  "fpde_column_a5", "fpde_lod3d_a2"])
def test_l1_weights_closed_form_matches_reference_series(name):
    g = fgv.load(golden_path(name))
    alpha = g["alpha"]
    time = oracle.time_points(g["tau"])
    nsteps = len(g["tau"])
    worst = 0.0
    for n in range(nsteps):
        kb_ref = _weights_of(g, n)
        assert len(kb_ref) == n
        kb, k0 = oracle.l1_weights(alpha, time, n)
        if n:
            worst = float(np.maximum(worst, float(np.max(np.abs(kb - kb_ref) / np.abs(kb_ref)))))
        worst = float(np.maximum(worst, abs(k0 - g["kkk0"][n]) / g["kkk0"][n]))
    assert worst <= RTOL, worst


def _grids(g):
    G = g["U0"].shape
    cA = np.stack([g["coefA_pass%d" % p] for p in range(3)])
    cB = np.stack([g["coefB_pass%d" % p] for p in range(3)])
    cR = np.stack([g["coefRlap_pass%d" % p] for p in range(3)])
    return G, cA, cB, cR


@pytest.mark.parametrize("name", ["fpde_column_a2", "fpde_column_a5", "fpde_lod3d_a2"])
@pytest.mark.parametrize("weights", ["reference", "closed_form"])
def test_lod_replay_matches_reference_run(name, weights):
    """Replays the reference's mode-3 LOD steps (history sum + three Thomas passes)."""
    g = fgv.load(golden_path(name))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    G, cA, cB, cR = _grids(g)
    taus = g["tau"]
    time = oracle.time_points(taus)
    Da = g["Da"]
    U = g["U0"].copy()
    nsteps = len(taus)
    hist = np.zeros((nsteps,) + G)
    sN, M, K = dims
    for n in range(nsteps):
        if weights == "reference":
            kb, k0 = _weights_of(g, n), g["kkk0"][n]
        else:
            kb, k0 = oracle.l1_weights(g["alpha"], time, n)
        S = oracle.lod_step_dirichlet(dims, U, hist, n, kb if n else np.zeros(1), taus, Da, k0,
                                      cA, cB, cR, g["Rp"][n], g["BC"][n], want_S=True)
        # history sums on the K-pass nodes
        sl = (slice(1, K + 1), slice(1, M), slice(1, sN))
        if n:
            # S is an intermediate with cancellation (a weighted sum of increments of
            # O(1) values): closed-form weights, which differ from the reference's series
            # by ~1e-13, move it by up to a few 1e-12 of its maximum.
            tol_s = RTOL if weights == "reference" else 1e-11
            assert _relmax(S[sl], g["S"][n][sl]) <= tol_s, (n, _relmax(S[sl], g["S"][n][sl]))
        assert _relmax(U, g["U"][n]) <= RTOL, (n, _relmax(U, g["U"][n]))


def test_l1_sum_snapshot_form_equals_increment_form():
    g = fgv.load(golden_path("fpde_column_a2"))
    U = g["U"]
    n = U.shape[0] - 1
    old = np.concatenate([g["U0"][None], U[:n]]).reshape(n + 1, -1)
    kb = _weights_of(g, n)
    S1 = oracle.l1_sum_snapshots(old, kb, g["tau"])
    D = np.diff(old, axis=0)
    S2 = oracle.l1_sum(D, n, kb, g["tau"])
    np.testing.assert_array_equal(S1, S2)
    Sref = g["S"][n].reshape(-1)
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    grid = np.zeros(g["U0"].shape, dtype=bool)
    grid[1:K + 1, 1:M, 1:sN] = True
    assert _relmax(S1[grid.reshape(-1)], Sref[grid.reshape(-1)]) <= RTOL


@pytest.mark.parametrize("name", ["frdo_derivative", "frdo_derivative_kat"])
def test_do_derivative_matches_fr_do(name):
    """fr_do's DO derivative of t^2 (DO_Cder); frdo_derivative_kat is its main's default run (N 1000,
    aN 32), which prints DOerr 0.000375753: the oracle's derivative gives the same error."""
    g = fgv.load(golden_path(name))
    n, tau = int(g["N"]), g["tau"]
    x = np.arange(n) * tau
    F = x * x
    DF = oracle.do_derivative(F, tau, g["WA"], g["gs"])
    assert _relmax(DF[1:], g["DF_do"][1:]) <= RTOL
    if "analytic" in g:
        err = float(np.sqrt(np.sum((g["analytic"][1:] - DF[1:]) ** 2) / n))
        assert f"{err:.6g}" == f"{float(g['DOerr']):.6g}" == "0.000375753"
    from math import gamma
    DC = oracle.caputo_derivative(F, tau, 0.5, gamma(1.5))
    assert _relmax(DC[1:], g["DF_caputo05"][1:]) <= RTOL


@pytest.mark.parametrize("name", ["frdo_eq_ex0", "frdo_eq_ex1", "frdo_eq_ex0_kat"])
def test_do_equation_matches_fr_do(name):
    g = fgv.load(golden_path(name))
    ex, Nx, Nt = int(g["ex"]), int(g["Nx"]), int(g["Nt"])
    h = g["h"]
    x = np.arange(Nx) * h
    C0 = np.zeros(Nx) if ex == 0 else x * (1.0 - x)
    from math import gamma
    Na = int(g["Na"])
    gs = np.array([gamma(2.0 - (i / (Na - 1))) for i in range(Na)])
    Cm, b0 = oracle.do_eq_solve(ex, C0, Nt, int(g["tblock"]), h, g["tau"], g["D"], g["WA"], gs)
    assert abs(b0 - g["b0"]) <= RTOL * abs(g["b0"])
    assert _relmax(Cm, g["C"]) <= RTOL, _relmax(Cm, g["C"])
    err = np.sqrt(np.mean((Cm[:, -1] - g["analytic_last"]) ** 2))
    assert abs(err - g["err"]) <= 1e-9 * max(g["err"], 1e-300) + 1e-15
    if name.endswith("_kat"):                  # fr_do -1 (its defaults) prints err 0.0117073
        assert f"{err:.6g}" == "0.0117073"


@pytest.mark.parametrize("name", ["frdo_eq_ex0", "frdo_eq_ex1", "frdo_eq_ex0_kat"])
def test_do_equation_as_general_line_run(name):
    """fr_do's eq_solve, restated as a line run with fused DO lag weights, theta = 1 and a
    per-step source (the form the GPU line path runs), meets the reference's own output."""
    import do_cases
    g = fgv.load(golden_path(name))
    u0, A, B, Rl, w, theta, src, steps = do_cases.line_problem(g, oracle.do_fused_weights)
    assert abs(w[0] * g["tau"] - g["b0"]) <= 1e-12 * g["b0"]
    Cref = g["C"]
    U = u0.copy()
    for n in range(1, steps + 1):            # compare every time level
        U, _ = oracle.line_run_general(u0, n, w, theta, A, B, Rl, src)
        assert _relmax(U, Cref[:, n]) <= RTOL, (n, _relmax(U, Cref[:, n]))


def _interior(g):
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    m = np.zeros(g["U0"].shape, dtype=bool)
    m[1:K + 1, 1:M, 1:sN] = True
    return m.reshape(-1)


def test_sum_restricted_matches_reference_run():
    """sum_alg 1 (time_summing's restricted summing, threshold 0.05: the 8 newest lags) on the
    reference's own column run: every step's history sum, bit for bit. Step 0 has no history
    and the reference leaves its b_Utimesum unwritten, so it is skipped."""
    g = fgv.load(golden_path("fpde_column_alg1"))
    U, m = g["U"], _interior(g)
    off = g["kb_off"].astype(int)
    for n in range(1, U.shape[0]):
        old = np.concatenate([g["U0"][None], U[:n]]).reshape(n + 1, -1)
        S = oracle.sum_restricted(old, g["kb_flat"][off[n]:off[n + 1]], g["tau"], g["sum_param"], 0)
        np.testing.assert_array_equal(S[m], g["S"][n].reshape(-1)[m])


def test_sum_series_matches_reference_run():
    """sum_alg 2 (16-term series expansion) on the reference's own column run: the moments are
    carried from step to step from zero, every step's history sum bit for bit."""
    g = fgv.load(golden_path("fpde_column_alg2"))
    U, m = g["U"], _interior(g)
    H = np.zeros((U.shape[1] * U.shape[2] * U.shape[3], int(g["sum_param"])))
    for n in range(1, U.shape[0]):
        prev = (g["U0"] if n == 1 else U[n - 2]).reshape(-1)
        S = oracle.sum_series(prev, U[n - 1].reshape(-1), H, g["row2"][n], g["gt"][n], g["gtj"][n], g["alpha"],
                              g["tau"][n])
        np.testing.assert_array_equal(S[m], g["S"][n].reshape(-1)[m])


def test_sum_restricted_chunk_rule():
    """The GPU kernel's chunked rule (BS terms at a time, stop after the first all-small chunk)
    against the window it implies, on weights decreasing with lag."""
    rng = np.random.default_rng(3)
    nt, nodes = 50, 9
    old = rng.standard_normal((nt + 1, nodes))
    tau = 0.5 + rng.random(nt)
    kb = 1.0 / (1.0 + np.arange(nt)[::-1])          # kb[t] for lag nt - t: 1, 1/2, 1/3, ...
    thr = 1.0 / 7.5                                  # lags 1..7 are >= thr
    def window(L):
        return sum(kb[t] * (old[t + 1] - old[t]) / tau[t] for t in range(nt - 1, nt - 1 - L, -1))
    np.testing.assert_allclose(oracle.sum_restricted(old, kb, tau, thr, 0), window(7), rtol=1e-14)
    for bs, L in ((1, 8), (4, 12), (7, 14), (8, 16), (64, 50)):
        np.testing.assert_allclose(oracle.sum_restricted(old, kb, tau, thr, bs), window(L), rtol=1e-14,
                                   err_msg=f"bs={bs}")


WG_SCENARIOS = [(1, 0.5, ""), (1, 0.5, "_vartau"), (2, 2.0, ""), (2, 2.0, "_vartau"), (3, 1.5, ""), (3, 1.5, "_vartau")]


@pytest.mark.parametrize("fk,p,suf", WG_SCENARIOS)
def test_weights_g_matches_reference_series(fk, p, suf):
    """Generalized kernels g(t) = t^p (func_in_kernel 1-3), uniform and variable steps: the
    oracle's quadrature against the reference's own series weights on every interval that
    does not start at t = 0 (there the reference's series for (g^-1)' is expanded at the edge
    of its convergence disc and is off the exact integral by up to 2e-2 for p = 2, 1.5; those
    entries are pinned by the 40-digit values of the next test)."""
    g = fgv.load(golden_path(f"fpde_weights_fk{fk}{suf}"))
    alpha = g["alpha"]
    time = oracle.time_points(g["tau"])
    worst = 0.0
    for n in range(1, len(g["tau"])):
        kb, k0 = oracle.weights_g(p, alpha, time, n)
        ref = _weights_of(g, n)
        if n > 1:
            worst = float(np.maximum(worst, float(np.max(np.abs(kb[1:] - ref[1:]) / np.abs(ref[1:])))))
        worst = float(np.maximum(worst, abs(k0 - g["kkk0"][n]) / g["kkk0"][n]))
        if p == 0.5:
            worst = float(np.maximum(worst, abs(kb[0] - ref[0]) / ref[0]))
    assert worst <= 3e-13, worst


@pytest.mark.parametrize("fk,p,suf", WG_SCENARIOS)
def test_weights_g_matches_exact_values(fk, p, suf):
    ex = fgv.load(golden_path("fpde_weights_g_exact"))
    time, rows = ex[f"fk{fk}{suf}_time"], ex[f"fk{fk}{suf}_rows"]
    alpha = fgv.load(golden_path(f"fpde_weights_fk{fk}{suf}"))["alpha"]
    worst = 0.0
    for n in range(rows.shape[0]):
        kb, k0 = oracle.weights_g(p, alpha, time, n)
        got = np.append(kb, k0)
        worst = float(np.maximum(worst, float(np.max(np.abs(got - rows[n, :n + 1]) / rows[n, :n + 1]))))
    assert worst <= 2e-15, worst


def test_weights_g_linear_kernel_is_the_l1_closed_form():
    rng = np.random.default_rng(4)
    time = oracle.time_points(1e-3 * (0.5 + rng.random(80)))
    for alpha in (0.1, 0.5, 0.85):
        for n in (0, 1, 9, 79):
            kb, k0 = oracle.weights_g(1.0, alpha, time, n)
            kc, kc0 = oracle.l1_weights(alpha, time, n)
            assert abs(k0 - kc0) / kc0 <= 2e-15
            if n:
                assert np.max(np.abs(kb - kc) / kc) <= 2e-15


def test_lod_restricted_replay_matches_reference_run():
    """The reference's mode-3 column run with restricted summing (sum_alg 1, sum_param 0.05)
    replayed step by step by the oracle: the same column problem as fpde_column_a2 (its
    coefficient grids, sources and boundary values), each step's history cut by time_summing's
    rule on the reference's own kb_3_cache."""
    g = fgv.load(golden_path("fpde_column_alg1"))
    a2 = fgv.load(golden_path("fpde_column_a2"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    assert dims == (int(a2["sN"]), int(a2["M"]), int(a2["K"])) and g["alpha"] == a2["alpha"]
    assert np.array_equal(g["tau"], a2["tau"])
    G, cA, cB, cR = _grids(a2)
    taus = g["tau"]
    U = g["U0"].copy()
    hist = np.zeros((len(taus),) + G)
    for n in range(len(taus)):
        kb = _weights_of(g, n).copy()
        for t in range(n - 1, -1, -1):                 # newest first: stop at the first small weight
            if abs(kb[t]) < g["sum_param"]:
                kb[:t + 1] = 0.0
                break
        oracle.lod_step_dirichlet(dims, U, hist, n, kb if n else np.zeros(1), taus, a2["Da"], a2["kkk0"][n],
                                  cA, cB, cR, a2["Rp"][n], a2["BC"][n])
        assert _relmax(U, g["U"][n]) <= RTOL, (n, _relmax(U, g["U"][n]))


def test_restricted_window_rule_matches_reference_run():
    """fpde_restricted_lags (host, the rule the line and LOD set-up apply to their weights) on
    the reference's own sum_alg 1 run: at every step the window it gives from that step's
    kb_3_cache is the one the reference summed (the replayed history sums match bit for bit),
    and the Caputo lag weights kkk0 b_l give the same 8 lags."""
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_column_alg1"))
    U = g["U"]
    m = _interior(g)
    off = g["kb_off"].astype(int)
    eps = g["sum_param"]
    for n in range(1, U.shape[0]):
        kb = g["kb_flat"][off[n]:off[n + 1]]
        L = fp.restricted_lags(kb[::-1], eps)          # kb[t] is the weight of lag n - t
        old = np.concatenate([g["U0"][None], U[:n]]).reshape(n + 1, -1)
        S = sum(kb[t] * (old[t + 1] - old[t]) / g["tau"][t] for t in range(n - 1, n - 1 - L, -1)) if L else 0.0 * old[0]
        np.testing.assert_allclose(S[m], g["S"][n].reshape(-1)[m], rtol=0, atol=1e-13 * np.abs(g["S"][n]).max())
    b = fp.weights_l1_lags(g["alpha"], 40)
    kkk0 = g["tau"][0] ** (1 - g["alpha"]) / (1 - g["alpha"])
    assert fp.restricted_lags(kkk0 * b[1:], eps) == 8
    assert fp.restricted_lags(kkk0 * b[1:], 0.0) == 39 and fp.restricted_lags(kkk0 * b[1:], 10.0) == 0


@pytest.mark.parametrize("p", [0.5, 1.0, 1.5, 2.0, 3.0])
@pytest.mark.parametrize("alpha", [0.05, 0.4, 0.8, 0.95])
def test_weights_g_sum_to_the_beta_integral(p, alpha):
    """A step's weights and its local weight cover [0, T]: sum_t kb_t + kkk0 =
    int_0^T (T^p - s^p)^-alpha ds = T^(1 - p alpha) B(1/p, 1 - alpha) / p, on random time grids."""
    from scipy.special import beta
    rng = np.random.default_rng(int(100 * p + 1000 * alpha))
    time = oracle.time_points(1e-2 * (0.2 + rng.random(60)))
    for n in (0, 1, 7, 59):
        kb, k0 = oracle.weights_g(p, alpha, time, n)
        T = time[n + 1]
        exact = T ** (1.0 - p * alpha) * beta(1.0 / p, 1.0 - alpha) / p
        assert abs((kb.sum() + k0) - exact) <= 1e-14 * exact, (n, (kb.sum() + k0) / exact - 1)


def test_gamma_matches_reference_gamma():
    """fpde_gamma against the reference's own Gamma (fpde_hpc_1d.cpp:70-252, exp(LogGamma) with
    its series and asymptotic branches), recorded by the pin harness at the orders the
    configurations use (1 - alpha for Da, 2 - a for the distributed-order normalisers) and over
    (0, 4]: the C library's tgamma and the reference's evaluation agree to a few ulps, far inside
    the 1e-12 parity bar they feed."""
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_gamma"))
    mine = np.array([fp.gamma(v) for v in g["x"]])
    rel = np.abs(mine - g["gamma"]) / np.abs(g["gamma"])
    assert rel.max() <= 4e-15, (rel.max(), g["x"][np.argmax(rel)])
    assert rel[:24].max() <= 4e-15          # the configurations' orders come first


@pytest.mark.parametrize("kform", [1, 2])
def test_richards_lod_replays_reference_run(kform):
    """The reference's Richards problem (analytic_test 0: van Genuchten-Mualem water content,
    k_form 1 VGM or 2 Averianov conductivity, no irrigation, zero-flux bottom and sides) in its 3D
    LOD mode with the history, 40 steps on 6^3 cells: the oracle forms every line's coefficients
    from the grid as the reference's A_/B/R do (fpde_hpc_1d.cpp:3095-3142 with KK/inv_dw_dh
    :2493-2657) and the surface condition from the step's evaporation rate, and replays every
    grid - bit for bit for k_form 2; for k_form 1 one value of step 10 rounds one ulp apart,
    4e-16 at most over the run."""
    g = fgv.load(golden_path(f"fpde_richards_k{kform}"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    U = g["U0"].copy()
    steps = len(g["tau"])
    hist = np.zeros((steps,) + U.shape)
    off = g["kb_off"].astype(int)
    worst = 0.0
    for n in range(steps):
        kb = g["kb_flat"][off[n]:off[n + 1]]
        S = oracle.lod_step_richards(dims, U, hist, n, kb if n else np.zeros(1), g["tau"], g["Da"], g["kkk0"][n],
                                     g["sZ"], g["sdL"], g["dLx"], g["dLy"], kform, g["k_sat"], g["E"][n], g["Rp"][n],
                                     want_S=True)
        worst = float(np.maximum(worst, float(np.max(np.abs(U - g["U"][n])) / np.max(np.abs(g["U"][n])))))
        if n > 0:                                   # the history sums on the K-pass nodes
            sl = (slice(1, dims[2] + 1), slice(1, dims[1]), slice(1, dims[0]))
            assert np.allclose(S[sl], g["S"][n][sl], rtol=1e-13, atol=1e-13 * np.max(np.abs(g["S"][n][sl])))
    assert worst <= (0.0 if kform == 2 else 1e-14), worst


def _salt_case():
    g = fgv.load(golden_path("fpde_richards_ct"))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    cA = np.stack([g[f"eq1_A_pass{p}"] for p in range(3)])
    cB = np.stack([g[f"eq1_B_pass{p}"] for p in range(3)])
    cR = np.stack([g[f"eq1_R_pass{p}"] for p in range(3)])
    return g, dims, cA, cB, cR


def test_richards_salt_lod_replays_reference_run():
    """The reference's Richards run with the salt concentration C (equation 1: chemical osmosis in
    the H equation, the H-driven and osmotic terms in C's, C's own history) replayed by the oracle
    bit for bit, H and C at every step (6^3 cells, 24 steps, k_form 1)."""
    g, dims, cA, cB, cR = _salt_case()
    U, C = g["U0"].copy(), g["C0"].copy()
    steps = g["U"].shape[0]
    hist, histC = np.zeros((steps,) + U.shape), np.zeros((steps,) + U.shape)
    kbo = g["kb_off"].astype(np.int64)
    for n in range(steps):
        kb = g["kb_flat"][kbo[n]:kbo[n + 1]]
        oracle.lod_step_richards_salt(dims, U, hist, n, kb if n else np.zeros(1), g["tau"], float(g["Da"]),
                                      float(g["kkk0"][n]), g["sZ"], g["sdL"], g["dLx"], g["dLy"], int(g["k_form"]),
                                      float(g["k_sat"]), float(g["E"][n]), C, histC, cA, cB, cR, float(g["nu"]),
                                      float(g["sigma"]))
        assert np.array_equal(U, g["U"][n]), f"H at step {n}"
        assert np.array_equal(C, g["C"][n]), f"C at step {n}"
    assert np.abs(C - g["C0"])[1:-1, 1:-1, 1:-1].max() > 0.05      # the concentration moved


def test_salt_coefficients_match_the_reference_formula():
    """Equation 1's constant coefficients (A_/B/R :3099-3136 with Dg = kb = 1, Da = 0) from D, sigma
    and the steps, as the device forms them, equal the reference's recorded grids."""
    g, dims, cA, cB, cR = _salt_case()
    sN, M, K = dims
    D, sigma = float(g["D"]), float(g["sigma"])
    for p, (dl, nl) in enumerate(((g["sdL"], sN), (g["dLx"], M), (g["dLy"], K))):
        ref = (cA[p], cB[p], cR[p])
        ax = 2 - p                                   # grid axis of the pass (k, j, i order)
        for q in range(1, nl):
            a = (D * (1.0 / (dl[q] * dl[q - 1]))) / sigma
            b = (D * (1.0 / (dl[q] * dl[q]))) / sigma
            r = (D * ((1.0 / (dl[q] * dl[q])) + (1.0 / (dl[q] * dl[q - 1])))) / sigma
            sl = [slice(1, -1)] * 3
            sl[ax] = q
            for got, want in zip((a, b, r), ref):
                vals = np.unique(want[tuple(sl)])
                vals = vals[vals != 0]                   # nodes off the pass's lines hold 0
                assert vals.size == 1 and vals[0] == got, (p, q)


@pytest.mark.parametrize("name", ["fpde_lod3d_vartau", "fpde_lod3d_fk3_vartau"])
def test_variable_step_lod_replays_reference_run(name):
    """The reference's 3D LOD with variable steps (its varT step sequence, g(t) = t and the
    generalized kernel t^1.5) replayed by the oracle from its recorded weight rows, bit for bit."""
    g = fgv.load(golden_path(name))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    cA, cB, cR = (np.stack([g[f"{k}_pass{p}"] for p in range(3)]) for k in ("coefA", "coefB", "coefRlap"))
    U = g["U0"].copy()
    steps = g["U"].shape[0]
    hist = np.zeros((steps,) + U.shape)
    kbo = g["kb_off"].astype(np.int64)
    assert np.ptp(g["tau"]) > 0                           # the steps do vary
    for n in range(steps):
        kb = g["kb_flat"][kbo[n]:kbo[n + 1]]
        oracle.lod_step_dirichlet(dims, U, hist, n, kb if n else np.zeros(1), g["tau"], float(g["Da"]),
                                  float(g["kkk0"][n]), cA, cB, cR, g["Rp"][n], g["BC"][n])
        assert np.array_equal(U, g["U"][n]), f"step {n}"


def test_reference_known_answer_column_k1000():
    """The reference's printed known answer for its column K = 1000, alpha 0.8, 1,000 steps
    (analytic squared error 0.014446): the oracle, from the rebuilt per-step inputs, reproduces the
    reference's final grid (to 2e-12: its closed-form weights differ from the reference's EPS-1e-15
    series by up to 1.5e-13, and 1,000 steps of this column carry that) and that error."""
    import kat_case
    c = kat_case.load()
    g = c["g"]
    U = g["U0"].copy()
    taus = np.full(c["steps"], float(g["tau"]))
    hist = np.zeros((c["steps"],) + U.shape)
    t = oracle.time_points(taus)
    for n in range(c["steps"]):
        kb, k0 = oracle.l1_weights(float(g["alpha"]), t, n)
        oracle.lod_step_dirichlet(c["dims"], U, hist, n, kb if n else np.zeros(1), taus, float(g["Da"]), k0,
                                  *c["coefs"], c["src"][n], c["bc"][n])
    assert _relmax(U, g["U_final"]) <= 2e-12
    err = kat_case.analytic_sq_err(U, c)
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])   # printed: 6 digits
    assert abs(float(g["analytic_sq_err"]) - 0.014446) < 5e-7        # the value the reference prints


def test_reference_known_answer_3d_generalized_kernel():
    """gpu_test.sh's error_tests parameters at 20 x 20 x 20 (analytic problem 2, alpha 0.8,
    g(t) = t^0.8, 40 steps): the reference prints the squared error 0.0472441. The oracle, from the
    rebuilt inputs and the reference's own weight rows (its series at EPS 1e-5), reproduces the final
    grid and that error."""
    import kat_case
    c = kat_case.load("fpde_lod3d_kat")
    g = c["g"]
    U = _replay_kat3d(c)
    assert _relmax(U, g["U_final"]) <= 1e-12
    err = kat_case.analytic_sq_err(U, c)
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])
    assert f"{err:.6g}" == "0.0472441"


def _replay_kat3d(c):
    """Step the oracle's LOD through a recorded 3D known-answer run: from the reference's weight
    rows (sum_alg 0), or (sum_alg 2) with the series sums formed from the oracle's own grids
    (fo_sum_series with the recorded row2_precalc rows and g(t) at each step's ends; the moments are
    carried from zero). Returns the final grid."""
    g = c["g"]
    U = g["U0"].copy()
    taus = g["tau_steps"]
    hist = np.zeros((c["steps"],) + U.shape)
    series = int(g.get("sum_alg", 0)) == 2
    H = np.zeros((U.size, int(g["sum_param"]))) if series else None
    grids = [U.copy()]
    for n in range(c["steps"]):
        if series:
            S = np.zeros(U.size)
            if n:
                S = oracle.sum_series(grids[n - 1].reshape(-1), grids[n].reshape(-1), H, g["row2"][n], g["gt"][n],
                                      g["gtj"][n], float(g["alpha"]), taus[n])
            oracle.lod_step_dirichlet_sum(c["dims"], U, hist, n, taus, float(g["Da"]), float(g["kkk0"][n]),
                                          *c["coefs"], c["src"][n], c["bc"][n], S)
        else:
            kb = c["rows"][n, :n]
            oracle.lod_step_dirichlet(c["dims"], U, hist, n, kb if n else np.zeros(1), taus, float(g["Da"]),
                                      float(c["rows"][n, n]), *c["coefs"], c["src"][n], c["bc"][n])
        grids.append(U.copy())
    return U


def test_reference_known_answer_3d_series_history():
    """The 20 x 20 x 20 known answer with the 16-term series history (sum_alg 2 sum_param 16,
    otherwise as above): the reference prints 0.0733568. The oracle, with the series sums formed from
    its own grids, reproduces the final grid and that error."""
    import kat_case
    c = kat_case.load("fpde_lod3d_kat_alg2")
    g = c["g"]
    assert int(g["sum_alg"]) == 2 and int(g["sum_param"]) == 16
    U = _replay_kat3d(c)
    assert _relmax(U, g["U_final"]) <= 1e-12
    err = kat_case.analytic_sq_err(U, c)
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])
    assert f"{err:.6g}" == "0.0733568"

PIN_FPDE = os.path.join(ROOT, "oracle", "_ref", "pin_fpde")


@pytest.fixture(scope="module")
def kat40_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("kat40")
    subprocess.run([PIN_FPDE, "kat40", str(d)], cwd=d, check=True, timeout=300)
    return d


@pytest.mark.skipif(not os.access(PIN_FPDE, os.X_OK),
                    reason="the reference harness is built only where the reference sources are")
@pytest.mark.parametrize("name,printed", [("fpde_lod3d_kat40", "0.403897"), ("fpde_lod3d_kat40_alg2", "0.600943"),
                                          ("fpde_lod3d_kat40_alg2_p32", "0.474818"),
                                          ("fpde_lod3d_kat40_alg2_p48", "0.437075"),
                                          ("fpde_lod3d_kat40_alg2_p64", "0.421276")])
def test_reference_known_answer_3d_error_tests_40(kat40_dir, name, printed):
    """gpu_test.sh's error_tests as the script runs them (NB M K 4: 40 x 40 x 40 cells, otherwise
    as the 20 x 20 x 20 case), with sum_alg 0 and with the 16-term series, and its bs_tests (the
    series with 32, 48 and 64 terms): the reference prints 0.403897, 0.600943, 0.474818, 0.437075 and
    0.421276. The harness writes the runs' inputs (8 MB each, so not kept as fixtures)
    into a temporary folder; the oracle replays them, reproduces the final grids and prints the same
    errors."""
    import kat_case
    c = kat_case.load(path=str(kat40_dir / (name + ".fgv")))
    g = c["g"]
    assert c["dims"] == (40, 40, 40)
    U = _replay_kat3d(c)
    assert _relmax(U, g["U_final"]) <= 1e-12
    err = kat_case.analytic_sq_err(U, c)
    assert abs(err - float(g["analytic_sq_err"])) <= 1e-8 * float(g["analytic_sq_err"])
    assert f"{err:.6g}" == printed
