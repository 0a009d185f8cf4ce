"""The tensor-core far-history contraction (fpde_far_contract) against an FP64 product of the
same 16-bit operands.

The kernel multiplies exactly representable fp16/bf16 values (products are exact), sums
them in FP32 for 256 columns at a time and folds those chunks in float-float, so it must
equal the FP64 product of the split operands to ~1e-6 of the result's magnitude
(tolerance 2e-6, normwise), and the unsplit FP64 product to the split's representation
error (fp16 pairs ~2^-22, bf16 pairs ~2^-17).
"""
import ctypes as C

import numpy as np
import pytest
from conftest import relmax

pytestmark = pytest.mark.gpu


def split16(x, fmt):
    import torch
    t = torch.from_numpy(x.astype(np.float32))
    dt = torch.float16 if fmt == "f16" else torch.bfloat16
    hi = t.to(dt)
    lo = (torch.from_numpy(x) - hi.double()).float().to(dt)
    return hi, lo


@pytest.mark.parametrize("fmt", ["f16", "bf16"])
@pytest.mark.parametrize("rows,k,splits", [(256, 64, 1), (1024, 768, 1), (1024, 832, 3), (4096, 2048, 4)])
def test_far_contract_matches_fp64(fmt, rows, k, splits):
    import torch
    import fpde_hpc_gb300 as fp
    lib = fp.load()
    rng = np.random.default_rng(rows + k)
    lda = ((k + 63) // 64) * 64 + 64        # pitch larger than K
    A = rng.standard_normal((rows, lda)) * (1000.0 if fmt == "f16" else 1e-3)
    W = rng.standard_normal((64, lda)) * 4.0
    Ah, Al = split16(A, fmt)
    Wh, Wl = split16(W, fmt)
    dev = [x.contiguous().cuda() for x in (Ah, Al, Wh, Wl)]
    Cout = torch.full((splits, 64, rows), np.nan, dtype=torch.float64, device="cuda")
    with fp.Context(0) as ctx:
        rc = lib.fpde_far_contract(ctx.h, *(C.c_void_p(x.data_ptr()) for x in dev[:2]), rows, lda,
                                   *(C.c_void_p(x.data_ptr()) for x in dev[2:]), lda, k, 1 if fmt == "bf16" else 0,
                                   0.5, C.c_void_p(Cout.data_ptr()), splits)
        fp.check(rc, "fpde_far_contract")
    got = Cout.sum(dim=0).cpu().numpy().T             # (rows, 64)
    a_h, a_l = Ah.double().numpy()[:, :k], Al.double().numpy()[:, :k]
    w_h, w_l = Wh.double().numpy()[:, :k], Wl.double().numpy()[:, :k]
    ref_split = 0.5 * (a_h @ w_h.T + a_h @ w_l.T + a_l @ w_h.T)
    ref_exact = 0.5 * (A[:, :k] @ W[:, :k].T)
    e1 = relmax(got, ref_split)
    e2 = relmax(got, ref_exact)
    print(f"{fmt} rows={rows} k={k} splits={splits}: vs split-FP64 {e1:.2e}, vs exact {e2:.2e}")
    assert np.isfinite(got).all()
    assert e1 <= 2e-6
    assert e2 <= (5e-6 if fmt == "f16" else 1e-4)


def slice3_host(X, per_row_blocks=True):
    """Host restatement of the three-slice split: per (row, 64-column block) exponent p with
    max|x| < 2^(p+8); x 2^-p = a0 + a1/256 + a2/65536 with integer a0, a1, a2 (round half even)."""
    rows, cols = X.shape
    nb = cols // 64
    m = np.abs(X).reshape(rows, nb, 64).max(axis=2)
    f, e = np.frexp(m)                          # m = f 2^e, f in [0.5, 1)
    p = np.where(m > 0, e - 8, 0).astype(np.int64)
    sc = np.repeat(np.ldexp(1.0, -p), 64, axis=1)
    x = X * sc
    a0 = np.rint(x)
    r1 = (x - a0) * 256.0
    a1 = np.rint(r1)
    a2 = np.rint((r1 - a1) * 256.0)
    back = (a0 + a1 / 256.0 + a2 / 65536.0) * np.repeat(np.ldexp(1.0, p), 64, axis=1)
    return [a0, a1 / 256.0, a2 / 65536.0], p.astype(np.int8), back


@pytest.mark.parametrize("rows,k,splits", [(256, 64, 1), (1024, 832, 3), (4096, 2048, 2)])
def test_far_contract3_exact_leading_product(rows, k, splits):
    import torch
    import fpde_hpc_gb300 as fp
    lib = fp.load()
    rng = np.random.default_rng(7 + rows + k)
    lda = ((k + 63) // 64) * 64 + 64
    # magnitudes varying by orders of magnitude across rows and column blocks
    A = rng.standard_normal((rows, lda)) * 10.0 ** rng.uniform(-6, 1, (rows, 1)) \
        * np.repeat(10.0 ** rng.uniform(-3, 0, (1, lda // 64)), 64, axis=1)
    W = np.abs(rng.standard_normal((64, lda))) * 30.0 + 0.1
    sa, pa, Aback = slice3_host(A)
    sw, pw, Wback = slice3_host(W)
    bf = lambda x: torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).contiguous().cuda()
    ad = [bf(x) for x in sa]
    wd = [bf(x) for x in sw]
    for x, ref in zip(ad + wd, sa + sw):          # the slices are exact in bf16
        assert np.array_equal(x.float().cpu().numpy().astype(np.float64), ref)
    pa_d = torch.from_numpy(np.ascontiguousarray(pa)).cuda()
    pw_d = torch.from_numpy(np.ascontiguousarray(pw)).cuda()
    Cout = torch.full((splits, 64, rows), np.nan, dtype=torch.float64, device="cuda")
    AP = (C.c_void_p * 3)(*[x.data_ptr() for x in ad])
    WP = (C.c_void_p * 3)(*[x.data_ptr() for x in wd])
    with fp.Context(0) as ctx:
        rc = lib.fpde_far_contract3(ctx.h, AP, rows, lda, WP, lda, k, C.c_void_p(pa_d.data_ptr()),
                                    C.c_void_p(pw_d.data_ptr()), lda // 64, C.c_void_p(Cout.data_ptr()), splits)
        fp.check(rc, "fpde_far_contract3")
    got = Cout.sum(dim=0).cpu().numpy().T
    # the six slice products the kernel forms (levels s + t <= 2), in FP64
    sA = [x * np.repeat(np.ldexp(1.0, pa.astype(np.int64)), 64, axis=1) for x in sa]
    sW = [x * np.repeat(np.ldexp(1.0, pw.astype(np.int64)), 64, axis=1) for x in sw]
    ref_kept = sum(sA[s][:, :k] @ sW[t][:, :k].T for s in range(3) for t in range(3) if s + t <= 2)
    ref_exact = A[:, :k] @ W[:, :k].T
    e1, e2 = relmax(got, ref_kept), relmax(got, ref_exact)
    print(f"x3 rows={rows} k={k} splits={splits}: vs kept-products FP64 {e1:.2e}, vs exact {e2:.2e}")
    assert np.isfinite(got).all()
    assert e1 <= 1e-8          # leading products exact; the 2^-8-smaller rest in FP32
    assert e2 <= 5e-7          # dropped slice products and representation, ~2^-24 each
