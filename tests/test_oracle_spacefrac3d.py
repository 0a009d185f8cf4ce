"""The oracle's fully implicit 3D space-fractional scheme against the reference's own runs.

fo_sf3d_matvec restates vmul_T_3d (fpde_hpc_1d.cpp:6801-8722, toeplitz_mult_alg 0, equation 0),
fo_sf3d_solve solve_mln<1> over the G + 1 values and fo_lod_step_sf3d the implicit3d 1 step
(calc_step :5160-5716: the lines' implicit2_gen systems added into Mat_3d / Om, the time term and
history in the K pass only). All keep the reference's operation order and build without
contracted multiply-adds, so the products, the assembled systems, the iterates and the whole run
must equal the reference's bit for bit."""
import numpy as np
import pytest

import oracle
import sf3d_cases


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_matvec_bitwise(name):
    c = sf3d_cases.load(name)
    g = c["g"]
    r = oracle.sf3d_matvec(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["mv_x"], iw=c["iw3"],
                           space_der=c["space_der"])
    assert np.array_equal(r, g["mv_r"])


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_solve_bitwise_with_count(name):
    c = sf3d_cases.load(name)
    g = c["g"]
    x, it = oracle.sf3d_solve(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["sys_last_om"], g["solve_x0"],
                              c["thr"], c["maxiter"], iw=c["iw3"], space_der=c["space_der"])
    assert it == c["solve_iters"]
    assert np.array_equal(x, g["solve_sol"])


@pytest.mark.parametrize("name", sf3d_cases.NAMES)
def test_lod_replay_bitwise(name):
    c = sf3d_cases.load(name)
    g = c["g"]
    U = g["U0"].reshape(-1).copy()
    hist = np.zeros((c["steps"], c["G"]))
    mask = sf_mask(c)
    ue = 0.0
    for n in range(c["steps"]):
        ue, it, mat, om, S = oracle.lod_step_sf3d(c["dims"], U, ue, hist, n, c["kb_rows"][n], g["tau"], c["Da"],
                                                  float(g["kkk0"][n]), c["coefA"], c["coefB"], c["coefRlap"], c["mc"],
                                                  c["iw"], c["Tm"], c["space_der"], c["thr"], c["maxiter"], g["Rp"][n],
                                                  g["BC"][n], want_system=True, rkind=c["rkind"], dLN=c["dLN"])
        assert it >= 1
        if n == 0:
            assert np.array_equal(mat, g["sys_first_mat"]) and np.array_equal(om, g["sys_first_om"])
        if n == c["steps"] - 1:
            assert np.array_equal(mat, g["sys_last_mat"]) and np.array_equal(om, g["sys_last_om"])
            assert it == c["solve_iters"]
        assert np.array_equal(U, g["U"][n].reshape(-1)), f"step {n}"
        if n > 0:
            assert np.array_equal(S[mask], g["S"][n].reshape(-1)[mask]), f"step {n}"
    assert ue == float(g["U_end"])


def sf_mask(c):
    sN, M, K = c["dims"]
    m = np.zeros((K + 2, M + 2, sN + 2), dtype=bool)
    m[1:K, 1:M, 1:sN] = True
    return m.reshape(-1)


def test_axis_terms_are_read():
    """Each axis's Toeplitz term and the space_der switch change the product (planted in the oracle's
    inputs: a zeroed row or the other switch value must move the result off the reference's)."""
    c = sf3d_cases.load("fpde_sf3d_sd1")
    g = c["g"]
    base = dict(iw=c["iw3"], space_der=1)
    r = oracle.sf3d_matvec(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["mv_x"], **base)
    assert np.array_equal(r, g["mv_r"])
    for ax in range(3):
        rows = [t.copy() for t in c["Tm3"]]
        rows[ax][:] = 0.0
        r2 = oracle.sf3d_matvec(c["dims"], g["sys_last_mat"], c["mc3d"], rows, g["mv_x"], **base)
        assert not np.array_equal(r2, g["mv_r"]), f"axis {ax}"
    r0 = oracle.sf3d_matvec(c["dims"], g["sys_last_mat"], c["mc3d"], c["Tm3"], g["mv_x"], iw=c["iw3"], space_der=0)
    assert not np.array_equal(r0, g["mv_r"])


def test_flux_rows_are_read():
    """The flux fixture's first step needs the flux rows: replayed with Dirichlet far ends it moves."""
    c = sf3d_cases.load("fpde_sf3d_flux")
    g = c["g"]
    out = []
    for rk in (c["rkind"], None):
        U = g["U0"].reshape(-1).copy()
        hist = np.zeros((c["steps"], c["G"]))
        oracle.lod_step_sf3d(c["dims"], U, 0.0, hist, 0, c["kb_rows"][0], g["tau"], c["Da"], float(g["kkk0"][0]),
                             c["coefA"], c["coefB"], c["coefRlap"], c["mc"], c["iw"], c["Tm"], c["space_der"], c["thr"],
                             c["maxiter"], g["Rp"][0], g["BC"][0], rkind=rk, dLN=c["dLN"])
        out.append(U)
    assert np.array_equal(out[0], g["U"][0].reshape(-1)) and not np.array_equal(out[1], out[0])
