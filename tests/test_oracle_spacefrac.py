"""The oracle's implicit space-fractional operator against the reference's own runs.

fo_sf_matvec restates vmul_T (fpde_hpc_1d.cpp:6618-6747, toeplitz_mult_alg 0), fo_sf_solve
solve_mln<1> (:812-1157) and fo_lod_step_sf the impl-2 LOD step (implicit2_gen :4630-4663, U1
:4769-4791). All three keep the reference's operation order and build without contracted
multiply-adds, so they must reproduce the reference's numbers bit for bit."""
import numpy as np
import pytest

import oracle
import sf_cases


@pytest.mark.parametrize("name", sf_cases.NAMES)
@pytest.mark.parametrize("p", [0, 1, 2])
def test_matvec_and_solve_bitwise(name, p):
    c = sf_cases.load(name)
    lc = sf_cases.line_case(c, p)
    r = oracle.sf_matvec(lc["mat"], lc["mc"], lc["Tm"], lc["x"], iw=lc["iw"], space_der=c["space_der"])
    assert np.array_equal(r, lc["r"])
    x, it = oracle.sf_solve(lc["mat"], lc["mc"], lc["Tm"], lc["B"], lc["x0"], c["thr"], c["maxiter"],
                            iw=lc["iw"], space_der=c["space_der"])
    assert it >= 1
    assert np.array_equal(x, lc["sol"])


@pytest.mark.parametrize("name", sf_cases.NAMES)
def test_lod_replay_bitwise(name):
    c = sf_cases.load(name)
    g = c["g"]
    U = g["U0"].copy()
    hist = np.zeros((c["steps"],) + U.shape)
    mask = sf_cases.interior(c["dims"])
    for n in range(c["steps"]):
        S, it = oracle.lod_step_sf(c["dims"], U, hist, n, c["kb_rows"][n], g["tau"], c["Da"], float(g["kkk0"][n]),
                                   c["coefA"], c["coefB"], c["coefRlap"], c["mc"], c["iw"], c["Tm"],
                                   c["space_der"], c["thr"], c["maxiter"], g["Rp"][n], g["BC"][n], want_S=True,
                                   rkind=c["rkind"], dLN=c["dLN"])
        assert it > 0
        assert np.array_equal(U, g["U"][n]), f"step {n}"
        if n > 0:      # at step 0 there is no history and the reference leaves its buffer untouched
            assert np.array_equal(S[mask], g["S"][n][mask]), f"step {n}"


def test_two_sided_differs_from_one_sided():
    """The space_der switch changes the product (a planted check that it is read)."""
    c = sf_cases.load("fpde_sf_sd1")
    lc = sf_cases.line_case(c, 2)
    r1 = oracle.sf_matvec(lc["mat"], lc["mc"], lc["Tm"], lc["x"], iw=lc["iw"], space_der=1)
    r0 = oracle.sf_matvec(lc["mat"], lc["mc"], lc["Tm"], lc["x"], iw=lc["iw"], space_der=0)
    assert np.array_equal(r1, lc["r"]) and not np.array_equal(r0, lc["r"])


def test_flux_rows_are_read():
    """The flux fixture's first step needs the flux rows: replayed with Dirichlet far ends it moves."""
    c = sf_cases.load("fpde_sf_flux")
    g = c["g"]
    out = []
    for rk in (c["rkind"], None):
        U = g["U0"].copy()
        hist = np.zeros((c["steps"],) + U.shape)
        oracle.lod_step_sf(c["dims"], U, hist, 0, c["kb_rows"][0], g["tau"], c["Da"], float(g["kkk0"][0]), c["coefA"],
                           c["coefB"], c["coefRlap"], c["mc"], c["iw"], c["Tm"], c["space_der"], c["thr"],
                           c["maxiter"], g["Rp"][0], g["BC"][0], rkind=rk, dLN=c["dLN"])
        out.append(U)
    assert np.array_equal(out[0], g["U"][0]) and not np.array_equal(out[1], out[0])
