"""The reference's known answers. Its column (fixture fpde_column_kat: mode 3, BS 1, NB 3, M 3,
K 1000, analytic problem 2, alpha 0.8, tau 1e-3, 1,000 steps): its run prints the squared error
0.014446 against the exact solution (analytic_compare). The fixture keeps the inputs in separated
form (source S1 - p2(t), line ends V + vt(t)); this module rebuilds the per-step grids."""
import numpy as np

import fgv
from conftest import golden_path


def load(name="fpde_column_kat", path=None):
    """The column KAT (fpde_column_kat) or the 3D one (fpde_lod3d_kat: gpu_test.sh's error_tests
    parameters at 20 x 20 x 20, g(t) = t^0.8, 40 steps; its run prints 0.0472441, and it carries the
    reference's weight rows of every step in `rows`). path: a fixture file written elsewhere (the
    harness's 40 x 40 x 40 run)."""
    g = fgv.load(path or golden_path(name))
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    sN, M, K = dims
    steps = g["p2"].size
    shape = g["U0"].shape
    # line-end nodes of the three passes (record_step_inputs)
    mask = np.zeros(shape, dtype=bool)
    mask[0, 1:M, 1:sN] = mask[K, 1:M, 1:sN] = True           # K lines (i, j) at k = 0, K
    mask[1:K, 0, 1:sN] = mask[1:K, M, 1:sN] = True           # _M lines (i, k) at j = 0, M
    mask[1:K, 1:M, 0] = mask[1:K, 1:M, sN] = True            # sN lines (j, k) at i = 0, sN
    V = np.where(mask, g["BC0"] - g["vt"][0], 0.0)
    interior = np.zeros(shape, dtype=bool)
    interior[1:K, 1:M, 1:sN] = True
    src = np.where(interior[None], g["S1"][None] - g["p2"][:, None, None, None], 0.0)
    bc = np.where(mask[None], V[None] + g["vt"][:, None, None, None], 0.0)
    coefs = [np.stack([g[f"{k}_pass{p}"] for p in range(3)]) for k in ("coefA", "coefB", "coefRlap")]
    c = dict(g=g, dims=dims, steps=steps, src=src, bc=bc, coefs=coefs, interior=interior)
    if "kb_off" in g and int(g.get("sum_alg", 0)) != 2:   # the reference's weight rows (row n: kb_3_cache, kkk0);
                                                          # its series mode keeps none
        kbo = g["kb_off"].astype(np.int64)
        rows = np.zeros((steps, steps + 1))
        for n in range(steps):
            rows[n, :n] = g["kb_flat"][kbo[n]:kbo[n + 1]]
            rows[n, n] = g["kkk0"][n]
        c["rows"] = rows
    return c


def analytic_sq_err(U, c):
    """analytic_compare: the sum over interior nodes of (U - exact)^2 at the final time."""
    d = (U - c["g"]["exact_final"])[c["interior"]]
    return float(np.sum(d * d))
