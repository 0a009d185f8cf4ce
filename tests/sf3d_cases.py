"""The fully implicit 3D space-fractional fixtures (fpde_sf3d_*.fgv.gz) as the arrays a replay needs.

Each fixture is one run of the reference's implicit3d 1 scheme (impl 2, TMA 0, analytic problem 2):
every step assembles Mat_3d / Mcoefs_3d / Om from the lines of the three passes and runs one
solve_mln<1> with vmul_T_3d over the G + 1 values (fpde_hpc_1d.cpp:5160-5716, :6801-8722). Recorded:
the per-pass coefficient grids, Mcoefs, inv_dw_dh and Toeplitz rows (as in the line-solve fixtures),
per step the grid, history sum, Rp and line ends, the assembled system of the first and last step,
Mcoefs_3d at the nodes the product reads, one product of a fixed vector and the last step's solve
repeated with its product count (tests/golden/make_golden.py --only spacefrac3d). fpde_sf3d_flux has flux
rows at the lines' far ends (the reference's bottom_cond 0)."""
import numpy as np

import sf_cases

NAMES = ["fpde_sf3d_sd0", "fpde_sf3d_sd1", "fpde_sf3d_tight", "fpde_sf3d_flux"]


def load(name):
    c = sf_cases.load(name)
    g = c["g"]
    sN, M, K = c["dims"]
    G = (sN + 2) * (M + 2) * (K + 2)
    V = G + 1
    c["G"], c["V"] = G, V
    rows = []
    for p in range(3):
        t = g[f"Tm_pass{p}"].copy()
        t[:2] = 0.0                      # entries 0 and 1 are never read by vmul_T_3d
        rows.append(t)
    c["Tm3"] = rows
    iw3 = np.zeros((3, V))
    for p in range(3):
        iw3[p, :G] = g[f"iw_pass{p}"].reshape(-1)
    c["iw3"] = iw3
    c["mc3d"] = g["mc3d"]
    # solve_mln counts two products per start, three per iteration and one final check
    c["solve_iters"] = (int(g["solve_products"]) - 3) // 3
    return c
