"""The algebra of the speculative block solve (k_line_block_spec), checked in numpy against
direct time stepping (no GPU).

Per step the line solves A U_{i-1} - R U_i + B U_{i+1} = Om_i by Thomas (the reference's al1 /
bt1 / U1 form). The kernel splits the line into chunks, sweeps each chunk from zero carries and
finishes with u = ub + c_in GG + u_b CB (c_in: the forward value at the node before the chunk,
u_b: the state at the node after it). Because every step is linear, step t+1's right-hand side
is known up to step t's two carries:
    Om^{t+1} = Omega0 + c_in E1 + u_b E2,
so the sweeps of step t+1 run on Omega0 while the carries are exchanged and are corrected
afterwards with the chunk-local responses to E1 and E2. With an explicit part (theta != 0:
Om -= theta (A u_{i-1} - Rlap u_i + B u_{i+1}) on the state before the step) the neighbours'
zero-carry results enter Omega0, the term of node a on u_{a-1} = al_{a-1} u_a + c_in folds into
node a's own coefficient, and E1, E2 carry the neighbours' GG, CB. This test builds exactly
those quantities and steps a ragged chunking speculatively against the direct solve.
"""
import numpy as np
import pytest


def _setup(N, chunk, theta, seed):
    rng = np.random.default_rng(seed)
    A = np.zeros(N + 1)
    B = np.zeros(N + 1)
    A[1:N] = rng.uniform(1, 2, N - 1)
    B[1:N] = rng.uniform(1, 2, N - 1)
    Rl = A + B + rng.uniform(0.01, 0.1, N + 1)
    lam = 0.7
    Al = np.zeros(N + 2)
    for i in range(1, N):
        Al[i + 1] = B[i] / ((Rl[i] + lam) - A[i] * Al[i])
    al = Al[1:N + 1]
    g = np.zeros(N)
    g[1:] = Al[2:N + 1] / B[1:N]
    Ah = np.zeros(N)
    Ah[1:] = A[1:N]
    chunks = [(a, min(a + chunk, N)) for a in range(0, N, chunk)]
    GG, CB = np.zeros(N), np.zeros(N)
    for a, b in chunks:
        pr, cf = 1.0, np.zeros(N)
        for i in range(a, b):
            pr *= g[i] * Ah[i]
            cf[i] = pr
        cb, gg = 1.0, 0.0
        for i in range(b - 1, a - 1, -1):
            cb *= al[i]
            CB[i] = cb
            gg = al[i] * gg + cf[i]
            GG[i] = gg
    return dict(N=N, A=A, B=B, Rl=Rl, lam=lam, al=al, g=g, Ah=Ah, chunks=chunks, GG=GG, CB=CB,
                klam=lam - theta * Rl, eA=theta * A, eB=theta * B)


def _local(s, om):
    """Zero-carry forward (y) and backward (ub) sweeps inside every chunk."""
    N = s["N"]
    y, ub = np.zeros(N), np.zeros(N)
    for a, b in s["chunks"]:
        yl = 0.0
        for i in range(a, b):
            yl = 0.0 if i == 0 else s["g"][i] * (s["Ah"][i] * yl - om[i])
            y[i] = yl
        ul = 0.0
        for i in range(b - 1, a - 1, -1):
            ul = s["al"][i] * ul + y[i]
            ub[i] = ul
    return y, ub


def _thomas(s, om):
    N = s["N"]
    Bt = np.zeros(N + 2)
    for i in range(1, N):
        Bt[i + 1] = s["g"][i] * (s["Ah"][i] * Bt[i] - om[i])
    U = np.zeros(N + 1)
    for i in range(N - 1, -1, -1):
        U[i] = s["al"][i] * U[i + 1] + Bt[i + 1]
    return U, Bt


def _carries(s, U, Bt):
    N = s["N"]
    cin, ub = np.zeros(N), np.zeros(N)
    for a, b in s["chunks"]:
        cin[a:b] = Bt[a] if a > 0 else 0.0      # forward value at node a - 1
        ub[a:b] = U[b]                          # state at node b
    return cin, ub


def _expl(s, u):
    N = s["N"]
    e = np.zeros(N)
    e[1:N] = s["eA"][1:N] * u[0:N - 1] + s["eB"][1:N] * u[2:N + 1]
    return e


@pytest.mark.parametrize("theta", [0.0, 0.5, 1.0])
@pytest.mark.parametrize("chunk", [64, 37])
def test_speculative_steps_equal_direct_steps(theta, chunk):
    N, steps = 300, 16
    s = _setup(N, chunk, theta, seed=int(7 + 10 * theta + chunk))
    w = np.concatenate([[s["lam"]], 0.5 / (1 + np.arange(1, 64)) ** 1.3])   # w[0] local, w[l] lag l
    klam, GG, CB, al = s["klam"][:N], s["GG"], s["CB"], s["al"]
    u0 = np.concatenate([np.sin(np.linspace(0, 3, N)), [0.0]])
    u0[0] = 0.0
    # direct stepping: Om = -klam u + sum_{r<t} w[t-r] D_r - explicit(u)
    Ud, D = u0.copy(), []
    for t in range(steps):
        S = sum(w[t - r] * D[r][:N] for r in range(t)) if t else np.zeros(N)
        Un, _ = _thomas(s, -klam * Ud[:N] + S - _expl(s, Ud))
        D.append(Un - Ud)
        Ud = Un
    # E1, E2 and the neighbour coefficients of Omega0 (the host preparation of the kernel)
    w1 = w[1]
    E1, E2 = (w1 - klam) * GG, (w1 - klam) * CB
    XA, XB, fold = np.zeros(N), np.zeros(N), np.zeros(N)
    for a, b in s["chunks"]:
        for i in range(max(a, 1), b):
            eA, eB = s["eA"][i], s["eB"][i]
            if i > a:
                E1[i] -= eA * GG[i - 1]
                E2[i] -= eA * CB[i - 1]
                XA[i] = -eA
            else:
                E1[i] -= eA * (al[a - 1] * GG[a] + 1.0)
                E2[i] -= eA * al[a - 1] * CB[a]
                fold[i] = -eA * al[a - 1]
            if i < b - 1:
                E1[i] -= eB * GG[i + 1]
                E2[i] -= eB * CB[i + 1]
                XB[i] = -eB
            else:
                E2[i] -= eB
    _, RB1 = _local(s, E1)
    _, RB2 = _local(s, E2)

    def omega0(ubc, u, dm1, H):
        om = (w1 - klam + fold) * ubc - w1 * u + w[2] * dm1 + H
        om[1:] += XA[1:] * ubc[:-1]
        om[:-1] += XB[:-1] * ubc[1:]
        return om

    # speculative stepping from step 0: the prologue solves step 0 from its full right-hand side
    u = u0[:N].copy()
    ring = []
    # history of step t' from the rows D_0 .. D_{t'-1-skip} (skip = 1: all but the newest row,
    # which the true right-hand side adds as w1 D_{t'-1}; skip = 2: Omega0's H, without D_{t'-2})
    hist = lambda tp, skip: sum(w[tp - r] * ring[r] for r in range(tp - skip)) if tp > skip else np.zeros(N)
    om = -klam * u - _expl(s, u0)
    _, ubc = _local(s, om)
    Ut, Bt = _thomas(s, om)
    cin, ubv = _carries(s, Ut, Bt)
    dm1 = np.zeros(N)
    for t in range(steps):
        if t > 0:
            un = ubprev + cin * GG + ubv * CB              # step t-1's state from its carries
            ring.append(un - u)
            dm1, u = un - u, un
            ubc = ubp + cin * RB1 + ubv * RB2              # corrected zero-carry result of step t
            U_t, Bt = _thomas(s, -klam * u + hist(t, 1) + w1 * dm1 - _expl(s, np.append(u, 0.0)))
            cin, ubv = _carries(s, U_t, Bt)                # the exchange of step t
        if t + 1 < steps:
            _, ubp = _local(s, omega0(ubc, u, dm1, hist(t + 1, 2)))
        ubprev = ubc
    u_final = ubprev + cin * GG + ubv * CB
    err = np.max(np.abs(u_final - Ud[:N])) / np.max(np.abs(Ud))
    assert err <= 1e-12, err
