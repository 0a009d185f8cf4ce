"""fpde_sf_toeplitz_row (host) against the Toeplitz rows the reference filled for its runs
(fpde_hpc_1d.cpp:3670-3694); no GPU needed."""
import numpy as np
import pytest

import sf_cases


@pytest.mark.parametrize("name", sf_cases.NAMES)
def test_toeplitz_row_matches_reference(name):
    import fpde_hpc_gb300 as fp
    c = sf_cases.load(name)
    g = c["g"]
    gam = float(g["gamma"])
    for p, nl in enumerate(c["dims"]):
        Tm = fp.sf_toeplitz_row(gam, g[f"Z_pass{p}"], nl)
        ref = g[f"Tm_pass{p}"]
        # entries 2..Nl-1 are the ones the product reads; C tgamma stands in for the reference's Gamma
        np.testing.assert_allclose(Tm[2:nl], ref[2:nl], rtol=4e-15, atol=0)
