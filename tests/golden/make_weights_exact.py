"""Exact (40-digit) generalized-kernel L1 weights for the time grids of the reference's
weights fixtures fpde_weights_fk{1,2,3}[_vartau] (g(t) = t^p with p = 0.5, 2, 1.5):

    kb_t(n) = int_{time[t]}^{time[t+1]} (T^p - s^p)^-alpha ds,  T = time[n+1],  t = 0..n

(t = n is kkk0). Evaluated with mpmath's tanh-sinh quadrature in the variable delta = T - s,
T^p - s^p formed as -T^p expm1(p log1p(-delta/T)); on the newest interval the factor
delta^-alpha is integrated analytically on its last 1/16 (delta = h y^(1/(1-alpha))).
The reference's own series (_kb_row/_kb_row2) is off on the intervals that start at t = 0
for p = 2 and 1.5, so these values pin the weights there. Needs mpmath (not needed by the
tests, which read the committed output fpde_weights_g_exact.fgv.gz).

    python tests/golden/make_weights_exact.py
"""
import gzip
import os
import struct

import mpmath as mp
import numpy as np

import fgv

HERE = os.path.dirname(os.path.abspath(__file__))
SCENARIOS = [(1, 0.5), (2, 2.0), (3, 1.5)]


def exact(alpha, p, s0, s1, T):
    T, p, alpha = mp.mpf(T), mp.mpf(p), mp.mpf(alpha)
    G = T ** p
    f = lambda d: (-G * mp.expm1(p * mp.log1p(-d / T))) ** (-alpha)
    if mp.mpf(s1) == T:
        wd = T - mp.mpf(s0)
        hw = wd / 16
        q = 1 / (1 - alpha)

        def R(y):
            d = hw * y ** q
            return (-G * mp.expm1(p * mp.log1p(-d / T)) / d) ** (-alpha) if d > 0 else (p * T ** (p - 1)) ** (-alpha)
        return mp.re(hw ** (1 - alpha) / (1 - alpha) * mp.quad(R, [0, 0.5, 0.9, 1]) + mp.quad(f, [hw, wd]))
    return mp.re(mp.quad(f, [T - mp.mpf(s1), T - mp.mpf(s0)]))


def put(f, name, arr):
    arr = np.ascontiguousarray(arr, dtype="<f8")
    nb = name.encode()
    f.write(struct.pack("<I", len(nb)) + nb + struct.pack("<I", arr.ndim))
    for d in arr.shape:
        f.write(struct.pack("<Q", d))
    f.write(arr.tobytes())


def main():
    mp.mp.dps = 40
    out = os.path.join(HERE, "fpde_weights_g_exact.fgv.gz")
    with gzip.GzipFile(out, "wb", 9, mtime=0) as f:
        f.write(b"FGV1")
        for fk, p in SCENARIOS:
            for suf in ("", "_vartau"):
                g = fgv.load(os.path.join(HERE, f"fpde_weights_fk{fk}{suf}.fgv.gz"))
                alpha = float(g["alpha"])
                tau = g["tau"]
                time = np.zeros(len(tau) + 1)
                for i, t in enumerate(tau):       # the reference accumulates Time[n+1] = Time[n] + tau
                    time[i + 1] = time[i] + t
                ns = len(tau)
                rows = np.zeros((ns, ns))
                for n in range(ns):
                    T = time[n + 1]
                    for t in range(n + 1):
                        rows[n, t] = float(exact(alpha, p, time[t], time[t + 1], T))
                put(f, f"fk{fk}{suf}_time", time)
                put(f, f"fk{fk}{suf}_rows", rows)
                print(f"fk{fk}{suf}: {ns} rows")
    print("wrote", out)


if __name__ == "__main__":
    main()
