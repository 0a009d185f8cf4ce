"""The reference's Sum kernel in its other history modes (fpde_sum) on the GPU:

  * sum_alg 1 (restricted summing) and sum_alg 2 (series expansion) replay the reference's
    own column runs (golden vectors of time_summing) to 1e-13 at every step; the GPU path
    forms kb/tau once per weight and sums with FMAs, the reference with separate roundings,
    hence not bit for bit;
  * windowed sums are checked per node against 1e-13 x the sum of the terms' magnitudes (the
    scale of any summation-order difference: FP64's own sequential bound is n 2^-53 of it);
  * against the oracle on larger seeded cases: windows longer than a 256-term chunk, the
    GPU kernel's chunk rule for several BS, no truncation and an empty window; moment counts
    from 1 to 128, node counts that leave a partial CTA, non-finite coefficients;
  * sum_alg 0 equals fpde_sum_snapshots; host and device buffers give the same result.
"""
import numpy as np
import pytest

import fgv
import oracle
from conftest import golden_path
from conftest import relmax

pytestmark = pytest.mark.gpu
RTOL = 1e-13


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _interior(g):
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    m = np.zeros(g["U0"].shape, dtype=bool)
    m[1:K + 1, 1:M, 1:sN] = True
    return m.reshape(-1)


def test_restricted_replays_reference_run(ctx):
    import torch
    g = fgv.load(golden_path("fpde_column_alg1"))
    U, m = g["U"], _interior(g)
    off = g["kb_off"].astype(int)
    worst = 0.0
    for n in range(1, U.shape[0]):
        old = torch.from_numpy(np.concatenate([g["U0"][None], U[:n]]).reshape(n + 1, -1)).cuda()
        kb = torch.from_numpy(g["kb_flat"][off[n]:off[n + 1]].copy()).cuda()
        tau = torch.from_numpy(g["tau"][:n].copy()).cuda()
        S = ctx.sum_alg(1, old, tau, kb=kb, sum_param=g["sum_param"]).cpu().numpy()
        worst = max(worst, relmax(S[m], g["S"][n].reshape(-1)[m]))
    print(f"sum_alg 1 vs the reference's run: max rel {worst:.2e}")
    assert worst <= RTOL


def test_series_replays_reference_run(ctx):
    """Moments stay on the device from step to step, as the reference's Htmp buffer."""
    import torch
    g = fgv.load(golden_path("fpde_column_alg2"))
    U, m = g["U"], _interior(g)
    P = int(g["sum_param"])
    G = U.shape[1] * U.shape[2] * U.shape[3]
    H = torch.zeros((G, P), dtype=torch.float64, device="cuda")
    tau = torch.from_numpy(g["tau"].copy()).cuda()
    worst = 0.0
    for n in range(1, U.shape[0]):
        prev = g["U0"] if n == 1 else U[n - 2]
        old = torch.from_numpy(np.stack([prev.reshape(-1), U[n - 1].reshape(-1)])).cuda()
        row2 = torch.from_numpy(g["row2"][n].copy()).cuda()
        S = ctx.sum_alg(2, old, tau, sum_param=g["sum_param"], Htmp=H, row2=row2, gtj=g["gtj"][n], gt=g["gt"][n],
                        alpha=g["alpha"], tstep=n).cpu().numpy()
        worst = max(worst, relmax(S[m], g["S"][n].reshape(-1)[m]))
    print(f"sum_alg 2 vs the reference's run: max rel {worst:.2e}")
    assert worst <= RTOL


@pytest.mark.parametrize("nt,nodes,thr,bs", [
    (700, 3001, 0.0, 0),          # no truncation: every term (three 256-term chunks)
    (700, 3001, 5e-4, 0),         # time_summing's rule, window of 564 terms (three chunks)
    (700, 3001, 5e-4, 16),        # the GPU kernel's rule, BS = 16
    (700, 3001, 5e-4, 256),
    (700, 3001, 5e-4, 300),       # BS not a divisor of the window
    (40, 257, 10.0, 0),           # the newest weight is already below: empty window, S = 0
    (1, 100, 0.0, 0),             # one term
])
def test_restricted_vs_oracle(ctx, nt, nodes, thr, bs):
    rng = np.random.default_rng(nt + nodes + bs)
    old = np.cumsum(0.01 * rng.standard_normal((nt + 1, nodes)), axis=0) + 1.0
    lag = nt - np.arange(nt)
    kb = 1.0 / lag ** 1.2
    tau = 1e-3 * (1.0 + 0.3 * rng.random(nt))
    ref = oracle.sum_restricted(old, kb, tau, thr, bs)
    # the same window over |increments|: the sum of the terms' magnitudes per node
    mag = oracle.sum_restricted(np.concatenate([[np.zeros(nodes)], np.cumsum(np.abs(np.diff(old, axis=0)), axis=0)]),
                                kb, tau, thr, bs)
    S = ctx.sum_alg(1, old, tau, kb=kb, sum_param=thr, bs=bs)
    if np.max(np.abs(ref)) == 0.0:
        assert np.max(np.abs(S)) == 0.0
    else:
        err = np.abs(S - ref)
        print(f"nt={nt} thr={thr} bs={bs}: max err / sum|terms| {np.max(err / np.maximum(mag, 1e-300)):.2e}")
        assert np.all(err <= RTOL * mag)


def test_full_mode_equals_sum_snapshots(ctx):
    rng = np.random.default_rng(5)
    old = rng.standard_normal((300, 1000))
    kb = rng.random(299)
    tau = 1e-3 + rng.random(299) * 1e-3
    S0 = ctx.sum_alg(0, old, tau, kb=kb)
    S1 = ctx.sum_snapshots(old, kb, tau)
    assert relmax(S0, S1) <= RTOL


@pytest.mark.parametrize("P,nodes", [(1, 129), (7, 1000), (16, 65536 + 77), (75, 5000), (128, 300)])
def test_series_vs_oracle(ctx, P, nodes):
    """Five steps carried in the moments; host buffers (the entry copies them each call)."""
    rng = np.random.default_rng(P * 7 + nodes)
    alpha = 0.7
    H = np.zeros((nodes, P))
    Href = np.zeros((nodes, P))
    u = rng.standard_normal(nodes)
    tau = np.full(10, 2e-3)
    for n in range(1, 6):
        un = u + 0.01 * rng.standard_normal(nodes)
        gt, gtj = n * 2e-3, (n + 1) * 2e-3
        row2 = 1.0 / (np.arange(P) + 1.0) * (1.0 - (gt / gtj) ** (np.arange(P) + 1.0))
        ref = oracle.sum_series(u, un, Href, row2, gt, gtj, alpha, tau[n])
        S = ctx.sum_alg(2, np.stack([u, un]), tau, sum_param=P, Htmp=H, row2=row2, gtj=gtj, gt=gt, alpha=alpha,
                        tstep=n)
        assert relmax(S, ref) <= RTOL, n
        assert relmax(H, Href) <= RTOL, n
        u = un


def test_series_truncates_fractional_sum_param(ctx):
    """sum_param = 16.5 keeps 16 moments, as the reference's (int)sum_param (time_summing :4137,
    Sum kernel :1462-1474): the same sums and moments as sum_param = 16."""
    rng = np.random.default_rng(5)
    nodes, alpha, tau = 2000, 0.6, np.full(4, 1e-3)
    u, un = rng.standard_normal(nodes), rng.standard_normal(nodes)
    row2 = 1.0 / np.arange(1.0, 17.0)
    H1, H2 = np.zeros((nodes, 16)), np.zeros((nodes, 16))
    S1 = ctx.sum_alg(2, np.stack([u, un]), tau, sum_param=16, Htmp=H1, row2=row2, gtj=0.003, gt=0.002,
                     alpha=alpha, tstep=2)
    S2 = ctx.sum_alg(2, np.stack([u, un]), tau, sum_param=16.5, Htmp=H2, row2=row2, gtj=0.003, gt=0.002,
                     alpha=alpha, tstep=2)
    np.testing.assert_array_equal(S1, S2)
    np.testing.assert_array_equal(H1, H2)


def test_series_guards_and_device_buffers(ctx):
    """A non-finite row2 entry counts as 0 (the GPU kernel's guard, also in the oracle);
    device buffers give the same moments and sums as host buffers."""
    import torch
    rng = np.random.default_rng(9)
    nodes, P = 1000, 16
    prev, cur = rng.standard_normal(nodes), rng.standard_normal(nodes)
    row2 = rng.random(P)
    row2[3] = np.nan
    row2[9] = np.inf
    Hh = rng.standard_normal((nodes, P))
    Href = Hh.copy()
    tau = np.array([1e-3, 2e-3])
    ref = oracle.sum_series(prev, cur, Href, row2, 0.01, 0.012, 0.6, tau[1])
    assert np.isfinite(ref).all()
    Hd = torch.from_numpy(Hh.copy()).cuda()
    Sd = ctx.sum_alg(2, torch.from_numpy(np.stack([prev, cur])).cuda(), torch.from_numpy(tau).cuda(), sum_param=P,
                     Htmp=Hd, row2=torch.from_numpy(row2).cuda(), gtj=0.012, gt=0.01, alpha=0.6, tstep=1)
    Sh = ctx.sum_alg(2, np.stack([prev, cur]), tau, sum_param=P, Htmp=Hh, row2=row2, gtj=0.012, gt=0.01, alpha=0.6,
                     tstep=1)
    assert relmax(Sh, ref) <= RTOL and relmax(Hh, Href) <= RTOL
    np.testing.assert_array_equal(Sd.cpu().numpy(), Sh)
    np.testing.assert_array_equal(Hd.cpu().numpy(), Hh)


def test_series_first_step_has_no_history(ctx):
    H = np.ones((50, 4))
    S = ctx.sum_alg(2, np.ones((1, 50)), np.ones(3), sum_param=4, Htmp=H, row2=np.ones(4), gtj=1.0, gt=1.0,
                    alpha=0.5, tstep=0)
    assert np.all(S == 0.0) and np.all(H == 1.0)


def test_stream_ordered_mode(ctx):
    """on_device = 2 returns after launching; after the context's stream drains the results equal
    the synchronous call's (restricted window found on the device in both)."""
    import torch
    rng = np.random.default_rng(12)
    nt, nodes = 600, 4000
    old = torch.from_numpy(rng.standard_normal((nt + 1, nodes))).cuda()
    kb = torch.from_numpy(1.0 / (nt - np.arange(nt)) ** 1.1).cuda()
    tau = torch.from_numpy(1e-3 * (1 + rng.random(nt))).cuda()
    S1 = ctx.sum_alg(1, old, tau, kb=kb, sum_param=1e-3, bs=32)
    S2 = torch.empty_like(S1)
    ctx.sum_alg(1, old, tau, kb=kb, sum_param=1e-3, bs=32, out=S2, sync=False)
    ctx.synchronize()
    assert torch.equal(S1, S2)


def test_snapshot_pitch_larger_than_nodes(ctx):
    """Snapshots with a row pitch OS above the node count (the reference rounds ocl_sol_size up
    to its block size): only the first `nodes` entries of each row are read and written."""
    rng = np.random.default_rng(21)
    nt, nodes, OS = 90, 1000, 1024
    old = rng.standard_normal((nt + 1, OS))
    kb = 1.0 / (nt - np.arange(nt)) ** 0.9
    tau = np.full(nt, 1e-3)
    S = ctx.sum_alg(1, old, tau, kb=kb, sum_param=0.02, nodes=nodes)
    ref = oracle.sum_restricted(old[:, :nodes], kb, tau, 0.02, 0)
    assert S.shape == (nodes,) and relmax(S, ref) <= RTOL
    H = np.zeros((nodes, 8))
    Href = np.zeros((nodes, 8))
    row2 = 1.0 / np.arange(1.0, 9.0)
    S2 = ctx.sum_alg(2, old[:2], tau, sum_param=8, Htmp=H, row2=row2, gtj=0.02, gt=0.01, alpha=0.5, tstep=3,
                     nodes=nodes)
    ref2 = oracle.sum_series(old[0, :nodes], old[1, :nodes], Href, row2, 0.01, 0.02, 0.5, tau[3])
    assert relmax(S2, ref2) <= RTOL and relmax(H, Href) <= RTOL
