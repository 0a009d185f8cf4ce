"""The implicit space-fractional fixtures (fpde_sf_*.fgv.gz) as the arrays a replay needs.

Each fixture is one run of the reference's LOD (impl 2, TMA 0, analytic problem 2): the per-pass
coefficient grids, the Mcoefs diagonals and inv_dw_dh of every line node, the Toeplitz rows
Tm[pass], and per step the grid, the history sum, Rp and the line ends; plus one product vmul_T
and one solve_mln<1> on the first line of each pass (tests/golden/make_golden.py --only
spacefrac). fpde_sf_flux has flux rows at the lines' far ends (the reference's bottom_cond 0)."""
import numpy as np

import fgv
from conftest import golden_path

NAMES = ["fpde_sf_sd0", "fpde_sf_sd1", "fpde_sf_col", "fpde_sf_flux"]


def load(name):
    g = fgv.load(golden_path(name))
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    c = dict(g=g, dims=(sN, M, K), space_der=int(g["space_der"]), thr=float(g["impl_err"]),
             maxiter=int(g["impl_niter"]), Da=float(g["Da"]))
    c["coefA"] = np.stack([g[f"coefA_pass{p}"] for p in range(3)])
    c["coefB"] = np.stack([g[f"coefB_pass{p}"] for p in range(3)])
    c["coefRlap"] = np.stack([g[f"coefRlap_pass{p}"] for p in range(3)])
    c["mc"] = np.stack([np.stack([g[f"mc{q}_pass{p}"] for q in range(3)]) for p in range(3)])
    c["iw"] = np.stack([g[f"iw_pass{p}"] for p in range(3)])
    ldt = max(sN, M, K) + 2
    Tm = np.zeros((3, ldt))
    for p in range(3):
        t = g[f"Tm_pass{p}"]
        Tm[p, 2:t.size] = t[2:]          # entries 0 and 1 are never read by vmul_T
    c["Tm"] = Tm
    kbo = g["kb_off"].astype(np.int64)
    c["kb_rows"] = [g["kb_flat"][kbo[n]:kbo[n + 1]] for n in range(len(kbo) - 1)]
    c["steps"] = g["U"].shape[0]
    # bottom_cond 0: every line's far end is the flux row U[N] - U[N-1] = bcN dL[N-1]
    if "bottom_cond" in g:
        c["rkind"] = (1, 1, 1)
        c["dLN"] = tuple(float(g[f"dLN_pass{p}"]) for p in range(3))
    else:
        c["rkind"], c["dLN"] = None, None
    return c


def line_case(c, p):
    """The recorded product and solve on the first line of pass p."""
    g = c["g"]
    Tm = g[f"mv{p}_Tm"].copy()
    Tm[:2] = 0.0
    return dict(mat=g[f"mv{p}_mat"], mc=g[f"mv{p}_mc"], Tm=Tm, iw=g[f"mv{p}_iw"], x=g[f"mv{p}_x"],
                r=g[f"mv{p}_r"], B=g[f"mv{p}_B"], x0=g[f"mv{p}_x0"], sol=g[f"mv{p}_sol"])


def interior(dims):
    """Mask of the nodes every pass updates (the reference's S is stale elsewhere)."""
    sN, M, K = dims
    m = np.zeros((K + 2, M + 2, sN + 2), dtype=bool)
    m[1:K, 1:M, 1:sN] = True
    return m
