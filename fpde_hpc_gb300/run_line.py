"""Run one line solve of the benchmark family from the command line (for profiling runs and as a
usage example):

    python -m fpde_hpc_gb300.run_line N STEPS [PRECISION] [--sp SP --chunks G --far-splits S --far-super B] [--do]

builds the lognormal-k, 8-Gaussian line of N intervals (problems.config2; with --do the
distributed-order line of problems.config3: fused 16-order weights, the explicit half of the
space operator), advances it STEPS time steps with fpde_line_* on cuda:0 (PRECISION: 0 FP64,
1 bf16, 2 fp16, 3 exact three-slice bf16; default 3) and prints the largest |u| of the final
state.
"""
import argparse

import numpy as np

from . import api, problems


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("N", type=int)
    ap.add_argument("steps", type=int)
    ap.add_argument("precision", type=int, nargs="?", default=3)
    ap.add_argument("--sp", type=int, default=0, help="nodes per solver thread (0: built-in rule)")
    ap.add_argument("--chunks", type=int, default=0, help="CTAs of the block solve (0: built-in rule)")
    ap.add_argument("--far-splits", type=int, default=0, help="K splits of the far contraction (0: built-in)")
    ap.add_argument("--far-super", type=int, default=0, help="64-step blocks per far super-block (0: built-in)")
    ap.add_argument("--do", action="store_true", help="the distributed-order line (theta = 1)")
    a = ap.parse_args(argv)
    p = problems.config3(N=a.N, steps=a.steps) if a.do else problems.config2(N=a.N, steps=a.steps)
    A, B, R = p.coefs()
    tuning = None
    if a.sp or a.chunks or a.far_splits or a.far_super:
        tuning = api.LineTuning(solve_sp=a.sp, chunks=a.chunks, far_splits=a.far_splits, gemv_splits=0,
                                far_super=a.far_super)
    with api.Context(0) as ctx:
        if a.do:
            c = api.do_weights(p.orders, p.qw, p.tau, a.steps + 1, p.gnorm)
            line = api.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, a.steps, precision=a.precision,
                            tuning=tuning, lag_weights=c / p.tau, theta=1.0)
        else:
            line = api.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, a.steps, precision=a.precision,
                            tuning=tuning)
        line.run(a.steps)
        u = line.state()
        line.close()
    print(f"N={a.N} steps={a.steps} precision={a.precision}: max |u| = {float(np.max(np.abs(u))):.6e}")


if __name__ == "__main__":
    main()
