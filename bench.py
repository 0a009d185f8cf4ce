"""Benchmark of the hot path: implicit fractional time stepping with the full L1 history.

Default workload (the headline, config 2): one bench step = one full solve of a
65,536-interval 1D Caputo line, 8,192 implicit time steps (alpha 0.7, tau 1e-4, seeded
lognormal k and 8-Gaussian H0), i.e. 65,535 x 8,192 = 5.37e8 node-steps, each with the full
L1 history sum and a Thomas solve. Other workloads of the same operator:
  config3  distributed-order line, N=16,384, 4,096 steps, 16-node Gauss-Legendre orders
  config4  3D LOD 128^3, 1,024 steps, alpha 0.85 (history in the K pass, three Thomas passes)
  config5  ensemble of 512 columns, N log-uniform [256, 16384], alpha U[0.5, 0.95], 2,048 steps
  sum1     the Sum kernel contract with restricted summing (sum_alg 1) over config 4's 130^3
           grid: 1,024 stored snapshots, a threshold that keeps the 256 newest lags
  sum2     the Sum kernel contract with the series expansion (sum_alg 2, 16 moments per point)
           over config 4's 130^3 grid
  weights  every L1 weight row of a 4,096-step run with the generalized kernel g(t) = t^1.5 and
           variable steps (fpde_weights_g: 8.4 M weights per call)
  sf3d     3D 64^3, 32 steps with the implicit space-fractional operator (gamma 0.7): the LOD's
           line solves (vmul_T + solve_mln<1>), or with --implicit3d 1 the fully implicit scheme
           (one vmul_T_3d solve over the grid per step); --space-der 1 two-sided, --sf-exact the
           reference's operation order (else tree dot products and fused multiply-adds)
`value` is measured with inputs resident in HBM (CUDA events on the library's stream, the
run replayed from a captured CUDA graph, no probes); `e2e` goes through the C ABI with host
buffers (the *_solve_host calls: upload the initial state, solve, download the state).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config3|config4|config5|sum1|sum2|weights|sf3d]
                    [--precision auto|fp64|bf16|f16|bf16x3] [--implicit3d 0|1] [--space-der 0|1] [--sf-exact]

--impl reference times the reference algorithm on the host cores: the CPU restatement of the
reference's FP64 path (oracle/), on all host threads, on a bounded sample of the same workload
(the first S1 and S2 time steps at full size), extrapolated with t(S) = a S + b S^2 (the history
term makes the cost quadratic in the step count).
Multi-GPU: nothing here shards (a line couples all its nodes; the ensemble could shard by column
but runs on one GPU), so N GPUs run N independent replicas (weak scaling).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2",
                    choices=["config2", "config3", "config4", "config5", "sum1", "sum2", "weights", "sf3d"])
    ap.add_argument("--space-der", type=int, default=0, choices=[0, 1],
                    help="sf3d: one-sided (0) or two-sided (1) space-fractional operator")
    ap.add_argument("--implicit3d", type=int, default=0, choices=[0, 1],
                    help="sf3d: line solves per pass (0) or the fully implicit scheme, one 3D solve per step (1)")
    ap.add_argument("--sf-exact", action="store_true",
                    help="sf3d: the reference's operation order (sequential dot products, separate roundings)")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "bf16", "f16", "bf16x3"])
    ap.add_argument("--time-steps", type=int, default=None, help="override the workload's step count")
    ap.add_argument("--nodes", type=int, default=None, help="override the workload's size")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-arm", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="built-in launch rules instead of fpde_line_autotune")
    ap.add_argument("--max-lag", type=int, default=0,
                    help="config2: restricted summing (the reference's sum_alg 1) keeping the newest MAX_LAG lags")
    return ap.parse_args()


def max_over_ranks(x, device):
    """The largest value of x over all ranks of the process group (the slowest replica's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "of fallback 6.8 TB/s"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workloads

def cpu_fit(samples, S):
    """Least-squares fit of t(s) = a s + b s^2 to timed samples [(s, seconds), ...] (the history
    term makes the cost quadratic in the step count) and its extrapolation to S steps. Returns
    (T(S), a, b, relative rms residual of the samples)."""
    s = np.array([x for x, _ in samples], dtype=np.float64)
    t = np.array([y for _, y in samples], dtype=np.float64)
    M = np.stack([s, s * s], axis=1)
    (a, b), *_ = np.linalg.lstsq(M / t[:, None], np.ones_like(t), rcond=None)   # relative residuals
    if b < 0:                                   # timing noise: linear model
        a, b = float(np.sum(t * s) / np.sum(s * s)), 0.0
    fit = a * s + b * s * s
    resid = float(np.sqrt(np.mean(((fit - t) / t) ** 2)))
    return float(a * S + b * S * S), float(a), float(b), resid


def cpu_record(wl, samples, threads):
    """cpu_baseline / reference-arm record from timed samples of the workload's CPU oracle."""
    T, a, b, resid = cpu_fit(samples, wl.steps)
    scale = getattr(wl, "sample_scale", 1.0)
    T *= scale
    lens = sorted({s for s, _ in samples})
    return {"value": wl.node_steps / T, "unit": "node-steps/s", "cores": threads, "kind": "port",
            "sample": wl.sample_desc(lens), "extrapolated": True,
            "fit": {"model": "t(S) = a S + b S^2 (seconds)", "a": a, "b": b, "relative_rms_residual": resid,
                    "samples": [{"steps": int(s), "seconds": float(t)} for s, t in samples],
                    "extrapolated_to_steps": wl.steps, "scale": scale, "seconds_per_solve": T},
            "seconds_timed": float(sum(t for _, t in samples))}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.load()
    return oracle


class LineWorkload:
    """1D lines: config2 (Caputo) and config3 (distributed order)."""

    def __init__(self, name, args):
        from fpde_hpc_gb300 import problems
        self.name = name
        if name == "config2":
            kw = {}
            if args.nodes:
                kw["N"] = args.nodes
            if args.time_steps:
                kw["steps"] = args.time_steps
            self.p = problems.config2(**kw)
            self.do = False
            self.metric = f"node-steps/s (1D Caputo L1 history sum + Thomas, N={self.p.N}, {self.p.steps} steps)"
            self.desc = (f"1D Caputo line N={self.p.N}, {self.p.steps} steps, alpha 0.7, tau 1e-4, lognormal k "
                         "(sigma 0.5, ell 0.01), 8-Gaussian H0 (config 2)")
            self.restrict_eps = 0.0
            if args.max_lag:
                # threshold between the kb of lags max_lag and max_lag + 1 (kb_l = kkk0 b_l)
                import fpde_hpc_gb300 as fp
                b = fp.weights_l1_lags(self.p.alpha, args.max_lag + 2)
                kkk0 = self.p.tau ** (1 - self.p.alpha) / (1 - self.p.alpha)
                self.restrict_eps = 0.5 * kkk0 * (b[args.max_lag] + b[args.max_lag + 1])
                self.metric = self.metric[:-1] + f", restricted summing: newest {args.max_lag} lags)"
                self.desc += (f"; restricted summing (the reference's sum_alg 1) with sum_param "
                              f"{self.restrict_eps:.6g}: the newest {args.max_lag} lags")
        else:
            kw = {}
            if args.nodes:
                kw["N"] = args.nodes
            if args.time_steps:
                kw["steps"] = args.time_steps
            self.p = problems.config3(**kw)
            self.do = True
            self.metric = (f"node-steps/s (1D distributed-order L1 history sum + Crank-Nicolson Thomas, "
                           f"N={self.p.N}, {self.p.steps} steps)")
            self.desc = (f"distributed-order line N={self.p.N}, {self.p.steps} steps, w(a)=6a(1-a), 16-node "
                         "Gauss-Legendre, tau 1e-4, lognormal k (seed 3), 8-Gaussian H0 (seed 4) (config 3)")
        self.node_steps = self.p.node_steps

    def weights(self, n):
        import fpde_hpc_gb300 as fp
        return fp.do_weights(self.p.orders, self.p.qw, self.p.tau, n, self.p.gnorm) / self.p.tau

    def build(self, ctx, prec, tuning=None):
        import fpde_hpc_gb300 as fp
        p = self.p
        A, B, R = p.coefs()
        if self.do:
            return fp.Line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, p.steps, precision=prec,
                           lag_weights=self.weights(p.steps + 1), theta=1.0, tuning=tuning)
        return fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, p.steps, precision=prec, tuning=tuning,
                       restrict_eps=self.restrict_eps)

    def autotune(self, ctx, prec):
        """fpde_line_autotune for this line (partition of the solve, far split depth, GEMV splits)."""
        import fpde_hpc_gb300 as fp
        p = self.p
        A, B, R = p.coefs()
        if self.do:
            return fp.autotune_line(ctx, p.N, 0.5, p.tau, 1.0, A, B, R, p.u0, p.steps, precision=prec,
                                    lag_weights=self.weights(p.steps + 1), theta=1.0)
        return fp.autotune_line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, p.steps, precision=prec)

    @property
    def u0(self):
        return self.p.u0

    @property
    def steps(self):
        return self.p.steps

    def sample_lengths(self):
        """Step counts of the timed CPU samples (the first steps of the full-size line)."""
        S = self.p.steps
        return [max(1, min(256, S // 8)), max(2, min(512, S // 4)), max(3, min(1024, S // 2))]

    def run_sample(self, s, threads):
        """Seconds for the oracle to run the first s steps at full size on `threads` host threads."""
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        p = self.p
        A, B, R = p.coefs()
        w = self.weights_host(s + 1) if self.do else None
        t0 = time.perf_counter()
        if self.do:
            oracle.line_run_general(p.u0, s, w, 1.0, A, B, R)
        else:
            oracle.line_run(p.u0, s, p.tau, p.alpha, p.Da, A, B, R)
        return time.perf_counter() - t0

    def sample_desc(self, lens):
        return (f"the first {', '.join(map(str, lens))} steps of the {self.p.N}-node line (full history), "
                f"least-squares fit t(S) = aS + bS^2, extrapolated to {self.p.steps} steps")

    def weights_host(self, n):
        oracle = _oracle()
        return oracle.do_fused_weights(self.p.orders, self.p.qw, self.p.gnorm, self.p.tau, n) / self.p.tau

    def bytes_io(self):
        return 8 * (self.p.N + 1), 8 * (self.p.N + 1)


class LodWorkload:
    def __init__(self, args):
        from fpde_hpc_gb300 import problems
        n = args.nodes or 128
        self.p = problems.config4(n=n, steps=args.time_steps or 1024)
        self.name = "config4"
        self.node_steps = self.p.node_steps
        self.metric = (f"node-steps/s (3D LOD: L1 history sum + three Thomas passes, {n}^3, "
                       f"{self.p.steps} steps)")
        self.desc = (f"3D LOD {n}^3, {self.p.steps} steps, alpha 0.85, tau 1e-3, lognormal k (sigma 0.4, seed 5), "
                     "Gaussian blob, zero-flux sides, Dirichlet top/bottom (config 4)")

    def build(self, ctx, prec, segments=(0, 0, 0)):
        import fpde_hpc_gb300 as fp
        p = self.p
        cA, cB, cR = p.coefs()
        return fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, p.steps, left_kind=p.left_kind,
                        right_kind=p.right_kind, dLN=p.dLN, precision=prec, segments=segments)

    def autotune(self, ctx, prec):
        """fpde_lod3d_autotune over the first min(steps, 128) steps: the passes' segment counts."""
        import fpde_hpc_gb300 as fp
        p = self.p
        cA, cB, cR = p.coefs()
        s = min(p.steps, 128)
        return fp.autotune_lod3d(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, s, s, left_kind=p.left_kind,
                                 right_kind=p.right_kind, dLN=p.dLN, precision=prec)

    @property
    def u0(self):
        return self.p.u0

    @property
    def steps(self):
        return self.p.steps

    def sample_lengths(self):
        S = self.p.steps
        return [max(1, min(16, S // 8)), max(2, min(32, S // 4)), max(3, min(64, S // 2))]

    def run_sample(self, s, threads):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        p = self.p
        cA, cB, cR = p.coefs()
        t0 = time.perf_counter()
        oracle.lod_run(p.dims, p.u0, s, p.tau, p.alpha, p.Da, cA, cB, cR, None, None, p.left_kind,
                       p.right_kind, p.dLN)
        return time.perf_counter() - t0

    def sample_desc(self, lens):
        return (f"the first {', '.join(map(str, lens))} steps of the {self.p.dims[0]}^3 grid, least-squares "
                f"fit t(S) = aS + bS^2, extrapolated to {self.p.steps} steps")

    def bytes_io(self):
        return 8 * self.p.u0.size, 8 * self.p.u0.size


class SfWorkload(LodWorkload):
    """The 3D LOD with the reference's implicit space-fractional line solves (impl 2, TMA 0): every
    line of every pass solved by solve_mln<1> with vmul_T (problems.sf3d)."""

    def __init__(self, args):
        from fpde_hpc_gb300 import problems
        n = args.nodes or 64
        self.impl3d = bool(args.implicit3d)
        self.exact = bool(args.sf_exact)
        self.p = problems.sf3d(n=n, steps=args.time_steps or 32, space_der=args.space_der)
        self.name = "sf3d_implicit3d" if self.impl3d else "sf3d"
        self.node_steps = self.p.node_steps
        side = "two-sided" if args.space_der else "one-sided"
        form = ("the reference's operation order" if self.exact
                else "tree dot products, fused multiply-adds")
        if self.impl3d:
            self.metric = (f"node-steps/s (fully implicit 3D space-fractional scheme, vmul_T_3d + solve_mln<1> over "
                           f"the grid, {n}^3, {self.p.steps} steps)")
            scheme = f"fully implicit (implicit3d 1: one 3D solve per step; {form})"
        else:
            self.metric = (f"node-steps/s (3D LOD with implicit space-fractional line solves, vmul_T + "
                           f"solve_mln<1>, {n}^3, {self.p.steps} steps)")
            scheme = f"LOD (line solves per pass; {form})"
        self.desc = (f"3D {scheme} {n}^3, {self.p.steps} steps, alpha 0.8, gamma {self.p.gamma} {side}, tau 1e-3, "
                     "lognormal k (sigma 0.4, seed 11), Gaussian blob and source, Dirichlet 0 line ends, "
                     "solver threshold 1e-9 / 5000 iterations (the reference's defaults)")
        self._ops = None

    def operands(self):
        if self._ops is None:
            p = self.p
            cA, cB, cR = p.coefs()
            Tm, mc, iw = p.sf_operands()
            self._ops = (cA, cB, cR, Tm, mc, iw, p.source())
        return self._ops

    def build(self, ctx, prec):
        import fpde_hpc_gb300 as fp
        p = self.p
        cA, cB, cR, Tm, mc, iw, src = self.operands()
        sf = dict(space_der=p.space_der, tol=p.tol, max_iter=p.max_iter, Tm=list(Tm), mc=list(mc), iw=list(iw),
                  implicit3d=1 if self.impl3d else 0, exact=1 if self.exact else 0)
        return fp.Lod3D(ctx, p.dims, p.alpha, p.tau, p.Da, cA, cB, cR, p.u0, p.steps, source=src, precision=prec,
                        space_frac=sf)

    def sample_lengths(self):
        S = self.p.steps
        if self.impl3d:                  # the oracle's 3D solve is one thread's work: seconds per step at 64^3
            return [1, 2, 3]
        return [max(1, S // 8), max(2, S // 4), max(3, S // 2)]

    def run_sample(self, s, threads):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        p = self.p
        cA, cB, cR, Tm, mc, iw, src = self.operands()
        taus = np.full(p.steps, p.tau)
        t = oracle.time_points(taus)
        U = p.u0.copy()
        hist = np.zeros((s,) + U.shape)
        bc = np.zeros_like(U)
        t0 = time.perf_counter()
        for n in range(s):
            kb, k0 = oracle.l1_weights(p.alpha, t, n)
            if self.impl3d:
                oracle.lod_step_sf3d(p.dims, U.reshape(-1), 0.0, hist.reshape(s, -1), n, kb, taus, p.Da, k0, cA, cB,
                                     cR, mc, iw, Tm, p.space_der, p.tol, p.max_iter, src, bc)
            else:
                oracle.lod_step_sf(p.dims, U, hist, n, kb, taus, p.Da, k0, cA, cB, cR, mc, iw, Tm, p.space_der,
                                   p.tol, p.max_iter, src, bc)
        return time.perf_counter() - t0

    def grid_iteration_ops(self):
        """FP64 flops of one iteration of the 3D solve over V = (n+2)^3 + 1 values: three products
        vmul_T_3d (seven diagonals 13 per value; Bt 5 per interior node and axis; per interior node and
        axis the Toeplitz sum, 2 per term: n-2 terms two-sided, (n-2)/2 on average one-sided, plus the
        iw product and the add), five dot products (2 per value) and the vector updates (11 per value)."""
        n = self.p.dims[0]
        V = (n + 2) ** 3 + 1
        inner = (n - 1) ** 3
        terms = (n - 2) if self.p.space_der else (n - 2) / 2.0
        mv = 13 * V + 3 * inner * (5 + 2 * terms + 2)
        return 3 * mv + 10 * V + 11 * V

    def line_iteration_ops(self):
        """FP64 flops (multiplies and adds) of one solver iteration on a line
        of n intervals: three products vmul_T (bt 5(n-1), tridiagonal 5(n-1)+6, Toeplitz
        (n-1)(n-2) one-sided or twice that two-sided, iw 2(n-1)), five dot products (2 (n+1)
        each) and the vector updates (11 (n+1))."""
        n = self.p.dims[0]
        toe = (n - 1) * (n - 2) * (2 if self.p.space_der else 1)
        mv = 5 * (n - 1) + 5 * (n - 1) + 6 + toe + 2 * (n - 1)
        return 3 * mv + 10 * (n + 1) + 11 * (n + 1)


class BatchWorkload:
    def __init__(self, args):
        from fpde_hpc_gb300 import problems
        self.cols = problems.config5(n_cols=args.nodes or 512, steps=args.time_steps or 2048)
        self.name = "config5"
        self._steps = self.cols[0].steps
        self.node_steps = sum(c.node_steps for c in self.cols)
        self.metric = (f"node-steps/s (ensemble of {len(self.cols)} 1D Caputo columns, N log-uniform "
                       f"[256,16384], {self._steps} steps)")
        self.desc = (f"ensemble of {len(self.cols)} columns, N log-uniform [256, 16384] "
                     f"(sum N = {sum(c.N for c in self.cols)}), alpha U[0.5, 0.95], tau 1e-3, {self._steps} steps, "
                     "seeds 6.. (config 5)")
        self._b = None

    def build(self, ctx, prec):
        import fpde_hpc_gb300 as fp
        cols = []
        for c in self.cols:
            A, B, R = c.coefs()
            cols.append(dict(N=c.N, alpha=c.alpha, tau=c.tau, Da=c.Da, A=A, B=B, Rlap=R, u0=c.u0))
        self._b = fp.Batch(ctx, cols, self._steps, precision=prec)
        return self._b

    @property
    def u0(self):
        return self._b.pack([c.u0 for c in self.cols])

    @property
    def steps(self):
        return self._steps

    SAMPLE_COLS = 16

    def _sample_idx(self):
        return np.linspace(0, len(self.cols) - 1, self.SAMPLE_COLS).astype(int)

    @property
    def sample_scale(self):
        """Total nodes over the sampled columns' nodes (the fit is per sampled column set)."""
        return sum(c.N for c in self.cols) / sum(self.cols[i].N for i in self._sample_idx())

    def sample_lengths(self):
        S = self._steps
        return [max(1, min(64, S // 8)), max(2, min(128, S // 4)), max(3, min(256, S // 2))]

    def run_sample(self, s, threads):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        t0 = time.perf_counter()
        for i in self._sample_idx():
            c = self.cols[i]
            A, B, R = c.coefs()
            oracle.line_run(c.u0, s, c.tau, c.alpha, c.Da, A, B, R)
        return time.perf_counter() - t0

    def sample_desc(self, lens):
        return (f"{self.SAMPLE_COLS} of the {len(self.cols)} columns, the first {', '.join(map(str, lens))} steps, "
                f"least-squares fit t(S) = aS + bS^2, extrapolated to {self._steps} steps and scaled by total nodes")

    def bytes_io(self):
        n = 8 * sum(c.N + 1 for c in self.cols)
        return n, n


class SumWorkload:
    """The reference's Sum kernel contract in its other history modes (fpde_sum) over the
    grid of config 4 (130^3 points with ghosts, as the reference's Sum runs over the whole
    snapshot). One bench step = `calls` consecutive time steps (one Sum call each)."""

    def __init__(self, args):
        self.alg = 1 if args.workload == "sum1" else 2
        self.name = args.workload
        n = args.nodes or 130
        self.points = n ** 3
        self.calls = 64
        self.alpha, self.tau = 0.85, 1e-3
        self.node_steps = self.points * self.calls
        if self.alg == 1:
            self.nt = args.time_steps or 1024          # stored increments at the timed steps
            self.window = 256
            import fpde_hpc_gb300 as fp
            b = fp.weights_l1_lags(self.alpha, self.nt + 1)
            kkk0 = self.tau ** (1 - self.alpha) / (1 - self.alpha)
            lagw = kkk0 * b                                # kb of lag l = kkk0 b[l-1]
            self.kb = np.ascontiguousarray(lagw[:self.nt][::-1])          # kb[t], t = 0..nt-1 (lag nt-t)
            self.thr = 0.5 * (lagw[self.window - 1] + lagw[self.window])  # keeps lags 1..window
            self.metric = (f"node-steps/s (Sum kernel, restricted summing: newest {self.window} of {self.nt} lags, "
                           f"{n}^3 points)")
            self.desc = (f"Sum contract sum_alg 1 over {n}^3 points (config 4's grid), {self.nt} stored snapshots, "
                         f"L1 weights alpha {self.alpha}, tau {self.tau}, threshold keeping the newest {self.window} "
                         f"lags (time_summing's rule), {self.calls} calls per step")
            self.bytes_per_point = 8.0 * (self.window + 1) + 8.0
        else:
            self.P = 16
            self.metric = f"node-steps/s (Sum kernel, series expansion with {self.P} moments, {n}^3 points)"
            self.desc = (f"Sum contract sum_alg 2 over {n}^3 points (config 4's grid), {self.P} moments per point "
                         f"(the reference's GPU default), alpha {self.alpha}, tau {self.tau}, {self.calls} calls "
                         "per step")
            self.bytes_per_point = 16.0 * self.P + 16.0 + 8.0

    def series_inputs(self, n):
        """row2, gt, gtj of time step n (g(t) = t): the normalised interval moments."""
        t0, t1, t2 = (n - 1) * self.tau, n * self.tau, (n + 1) * self.tau
        j = np.arange(self.P) + 1.0
        return (1.0 - (t0 / t1) ** j) / j, t1, t2

    def cpu_rate(self, threads):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        rng = np.random.default_rng(1)
        m = min(1 << 16 if self.alg == 1 else 1 << 18, self.points)
        if self.alg == 1:
            old = rng.standard_normal((self.nt + 1, m))
            t0 = time.perf_counter()
            oracle.sum_restricted(old, self.kb, np.full(self.nt, self.tau), self.thr, 0)
            dt = time.perf_counter() - t0
        else:
            H = np.zeros((m, self.P))
            prev, cur = rng.standard_normal(m), rng.standard_normal(m)
            row2, gt, gtj = self.series_inputs(100)
            t0 = time.perf_counter()
            reps = 8
            for _ in range(reps):
                oracle.sum_series(prev, cur, H, row2, gt, gtj, self.alpha, self.tau)
            dt = (time.perf_counter() - t0) / reps
        return {"value": m / dt, "sample_seconds": dt,
                "sample": f"one call over {m} of the {self.points} points (the oracle's restatement, "
                          f"{threads} threads)"}


def run_sum(args, wl):
    """Our arm for the Sum-contract workloads: device-resident calls timed with CUDA events on
    the context's stream (stream-ordered mode), and end to end as the reference drives its
    kernel: upload the newest snapshot, one synchronous call, read S back."""
    import torch
    import fpde_hpc_gb300 as fp
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    ctx = fp.Context(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    lib = ctx.lib
    dev = "cuda"
    G = wl.points
    S = torch.empty(G, dtype=torch.float64, device=dev)
    if wl.alg == 1:
        old = torch.rand((wl.nt + 1, G), dtype=torch.float64, device=dev)
        kb = torch.from_numpy(wl.kb).to(dev)
        tau = torch.full((wl.nt,), wl.tau, dtype=torch.float64, device=dev)
        call = lambda c, sync=False: ctx.sum_alg(1, old, tau, kb=kb, sum_param=wl.thr, out=S, sync=sync)
    else:
        old = torch.rand((2, G), dtype=torch.float64, device=dev)
        H = torch.zeros((G, wl.P), dtype=torch.float64, device=dev)
        tau = torch.full((wl.calls + 2,), wl.tau, dtype=torch.float64, device=dev)
        ins = [wl.series_inputs(100 + c) for c in range(wl.calls)]
        row2 = torch.from_numpy(np.stack([r for r, _, _ in ins])).to(dev)

        def call(c, sync=False):
            _, gt, gtj = ins[c]
            return ctx.sum_alg(2, old, tau, sum_param=wl.P, Htmp=H, row2=row2[c], gtj=gtj, gt=gt, alpha=wl.alpha,
                               tstep=c + 1, out=S, sync=sync)

    def step():
        for c in range(wl.calls):
            call(c)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = lib.fpde_kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = lib.fpde_kernel_launch_count() - launches0
    clk = clocks.stop()
    value = wl.node_steps * world / (ms / 1e3)
    per_call_ms = ms / wl.calls

    # end to end: newest snapshot up (pinned), one synchronous call, S down (pinned)
    snap_h = torch.rand(G, dtype=torch.float64).pin_memory()
    S_h = torch.empty(G, dtype=torch.float64).pin_memory()
    dst = old[-1]

    def e2e_step():
        for c in range(wl.calls):
            dst.copy_(snap_h, non_blocking=True)
            call(c, sync=True)
            S_h.copy_(S, non_blocking=True)
            torch.cuda.current_stream().synchronize()
    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    nb = 8 * G * wl.calls
    e2e = {"value": wl.node_steps / e2e_s, "unit": "node-steps/s", "h2d_bytes_per_step": nb,
           "d2h_bytes_per_step": nb, "ms_per_step": e2e_s * 1e3}

    peak, peak_src = measured_peaks()
    alg_bytes = wl.bytes_per_point * G
    gbs = alg_bytes / (per_call_ms / 1e3) / 1e9
    kname = "k_sum_window (+ k_window_len)" if wl.alg == 1 else "k_sum_series"
    fp64_per_point = 2 * (wl.window) + 1 if wl.alg == 1 else 2 * wl.P + 1
    roof = {"kernel": kname, "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": peak_src, "traffic": None, "ms_per_call": per_call_ms,
            "algorithmic_bytes_per_call": alg_bytes,
            "fp64_ops_per_point": fp64_per_point,
            "limiter": "fp64 pipe (GB300 issues ~1.7 FP64 lane-ops/clk/SM); see the profile"}
    out = {"metric": wl.metric, "value": value, "unit": "node-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded snapshots; no dataset exists)",
           "config": bench_config(wl, world), "path": f"sum_alg {wl.alg}",
           "e2e": e2e, "gpu_launches": int(launches), "clocks": clk, "roofline": roof}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = wl.cpu_rate(os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": cb["value"], "unit": "node-steps/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": cb["sample"]}
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


class WeightsWorkload:
    """All weight rows of a run with the generalized kernel g(t) = t^p and variable steps."""

    def __init__(self, args):
        self.name = "weights"
        self.steps = args.time_steps or 4096
        self.p, self.alpha = 1.5, 0.85
        rng = np.random.default_rng(7)
        tau = 1e-3 * (1.0 + 0.5 * np.sin(0.7 * np.arange(self.steps)) + 0.1 * rng.random(self.steps))
        self.time = np.concatenate([[0.0], np.cumsum(tau)])
        self.node_steps = self.steps * (self.steps + 1) // 2          # weights per call
        self.metric = f"weights/s (generalized L1 kernel g(t)=t^{self.p}, variable steps, all rows of {self.steps} steps)"
        self.desc = (f"fpde_weights_g rows 0..{self.steps - 1}: g(t) = t^{self.p}, alpha {self.alpha}, tau 1e-3 x "
                     "(1 + 0.5 sin(0.7 n) + 0.1 U[0,1)) (seed 7), one call per step")

    def cpu_rate(self, threads, rows=24):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle = _oracle()
        ns = list(range(self.steps - rows, self.steps))
        t0 = time.perf_counter()
        for n in ns:
            oracle.weights_g(self.p, self.alpha, self.time, n)
        dt = time.perf_counter() - t0
        cnt = sum(n + 1 for n in ns)
        return {"value": cnt / dt, "sample_seconds": dt,
                "sample": f"the last {rows} rows ({cnt} weights) by the oracle's quadrature, {threads} threads"}


def run_weights(args, wl):
    import torch
    import fpde_hpc_gb300 as fp
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    ctx = fp.Context(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    lib = ctx.lib
    S = wl.steps
    tdev = torch.from_numpy(wl.time).cuda()
    out = torch.zeros((S, S), dtype=torch.float64, device="cuda")
    call = lambda: ctx.weights_g(wl.p, wl.alpha, tdev, 0, S - 1, out=out, sync=False)
    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = lib.fpde_kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = lib.fpde_kernel_launch_count() - launches0
    clk = clocks.stop()
    value = wl.node_steps * world / (ms / 1e3)
    host = np.zeros((S, S))
    ctx.weights_g(wl.p, wl.alpha, wl.time, 0, S - 1, out=host)       # end to end: host time points and rows
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.weights_g(wl.p, wl.alpha, wl.time, 0, S - 1, out=host)
    e2e_s = (time.perf_counter() - t0) / args.steps
    peak, peak_src = measured_peaks()
    gbs = 8.0 * wl.node_steps / (ms / 1e3) / 1e9
    out_j = {"metric": wl.metric, "value": value, "unit": "weights/s", "n_gpus": world, "steps": args.steps,
             "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
             "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded time steps)",
             "config": bench_config(wl, world), "path": "fpde_weights_g",
             "e2e": {"value": wl.node_steps / e2e_s, "unit": "weights/s", "h2d_bytes_per_step": 8 * (S + 1),
                     "d2h_bytes_per_step": 8 * S * S, "ms_per_step": e2e_s * 1e3},
             "gpu_launches": int(launches), "clocks": clk,
             "roofline": {"kernel": "k_weights_g", "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                          "frac": gbs / peak, "peak_source": peak_src, "traffic": None,
                          "limiter": "FP64 transcendentals (pow/expm1/log1p per quadrature node), not HBM",
                          "note": "achieved = 8 B written per weight / kernel time"}}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = wl.cpu_rate(os.cpu_count() or 1)
        out_j["cpu_baseline"] = {"value": cb["value"], "unit": "weights/s", "cores": os.cpu_count() or 1,
                                 "kind": "port", "sample": cb["sample"]}
    ctx.close()
    if rank == 0:
        print(json.dumps(out_j), flush=True)


def bench_config(wl, world):
    """The `config` of both arms (same dict: same workload, same inputs)."""
    if isinstance(wl, WeightsWorkload):
        l2 = "output rows (134 MB) exceed L2; every call recomputes them"
    elif isinstance(wl, SumWorkload):
        l2 = "inputs larger than L2 (snapshots / moments of 2.2 M points, GBs)"
    else:
        l2 = "inputs larger than L2 (the increment history, GBs, is streamed every step)"
    return {"workload": wl.desc, "l2": l2, "parallelism": f"replicas x{world}"}


def make_workload(args):
    if args.workload == "weights":
        return WeightsWorkload(args)
    if args.workload in ("sum1", "sum2"):
        return SumWorkload(args)
    if args.workload in ("config2", "config3"):
        return LineWorkload(args.workload, args)
    if args.workload == "config4":
        return LodWorkload(args)
    if args.workload == "sf3d":
        return SfWorkload(args)
    return BatchWorkload(args)


# ------------------------------------------------------------------ reference arm

def run_reference(args):
    """The reference algorithm on the host cores: the oracle (the CPU restatement of the reference's
    FP64 path) on all host threads. For the time-stepping workloads each bench step is one timed
    sample - the first s steps of the full-size problem, s cycling through three lengths - and the
    value is the full solve's rate from a least-squares fit t(S) = aS + bS^2 of the samples
    (extrapolated; the fit, its residual and the seconds timed are printed). The Sum and weights
    workloads time one bounded call per step directly."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    wl = make_workload(args)
    threads = os.cpu_count() or 1
    unit = "weights/s" if isinstance(wl, WeightsWorkload) else "node-steps/s"
    if hasattr(wl, "run_sample"):
        lens = wl.sample_lengths()
        for _ in range(args.warmup):
            wl.run_sample(lens[0], threads)
        samples = []
        for it in range(args.steps):
            s = lens[it % len(lens)]
            samples.append((s, wl.run_sample(s, threads)))
        extra = [(s, wl.run_sample(s, threads)) for s in lens if not any(x == s for x, _ in samples)]
        cb = cpu_record(wl, samples + extra, threads)
        cb["timed_steps"] = [{"steps": int(x), "seconds": float(t)} for x, t in samples]
        cb["extra_samples_for_fit"] = len(extra)
        value = cb["value"]
        ms_step = 1e3 * float(np.mean([t for _, t in samples])) if samples else None
        note = ("each step is one timed sample (the first s steps at full size); value is the full solve's "
                "rate extrapolated from the samples (cpu_baseline.fit)")
    else:
        for _ in range(args.warmup):
            wl.cpu_rate(threads)
        vals = [wl.cpu_rate(threads) for _ in range(args.steps)]
        value = float(np.median([r["value"] for r in vals]))
        ms_step = 1e3 * float(np.mean([r["sample_seconds"] for r in vals]))
        cb = {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": vals[0]["sample"],
              "extrapolated": False}
        note = "each step is one timed bounded call of the oracle; value is measured directly"
    out = {"impl": "reference", "metric": wl.metric, "value": value, "unit": unit, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "step_note": note,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": bench_config(wl, world), "cpu_baseline": cb,
           "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ our arm

def _timed(obj, u0_dev, steps, reps, stream):
    """reps full solves from reset, CUDA events on the library's stream; ms per solve."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        obj.reset(u0_dev)
        obj.run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _probe(line, u0_dev, steps, every):
    """One probed solve: per-kind event sums (0 FP64 GEMV, 1 tensor-core far contraction over the
    history older than a super-block, 2 solve, 3 contraction over the super-block's own blocks)."""
    import torch
    line.set_probe(every)
    line.reset(u0_dev)
    line.run(steps)           # builds the probed graph
    line.reset(u0_dev)
    line.run(steps)
    torch.cuda.synchronize()
    tot = {k: line.probe_stats(k) for k in (0, 1, 2, 3)}
    line.set_probe(0)
    return tot


# DRAM traffic per launch from ncu captures (profiles/), split into what scales with the
# history length K of a launch and what does not:
#   k_far_tc3 (two weight groups per item, a 256-step super-block): reads per row x history
#     column, writes (the float-pair partials) per launch and row;
#   k_line_block_spec: bytes per node-step (64 steps x 65,537 nodes per launch).
NCU_FAR = {"read_per_row_col": 623.12e6 / (65664 * 1536), "write_per_row": 122.56e6 / 65664,
           "source": "profiles/k_far_tc3_super_N65536_K1536.md"}
NCU_SOLVE = {"per_node_step": (82.01e6 + 27.51e6) / (64 * 65537), "fp64_pipe_active": 0.4844,
             "source": "profiles/k_line_block_spec_N65536_2048steps.md"}


def _kernel_entry(t, name, peak, peak_src, scale=1.0):
    if t["count"] <= 0 or t["ms"] <= 0:
        return None
    gbs = t["bytes"] / (t["ms"] / 1e3) / 1e9
    e = {"kernel": name, "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
         "peak_source": peak_src, "traffic": None, "probed_units": t["count"],
         "ms_per_unit": t["ms"] / t["count"], "est_ms_per_solve": t["ms"] * scale}
    if t["flops"]:
        e["achieved_tflops"] = t["flops"] / (t["ms"] / 1e3) / 1e12
    return e


def split_line_rooflines(tot, steps, nodes, rows, sbk, ms_solve, hbm, hbm_src):
    """Kernel records of the split (bf16x3) line from one probed solve.

    far_tc: k_far_tc3 over the history older than each 256-step super-block (one launch per
    super-block): bound by the tensor cores' operand traffic, reported in TFLOP/s of the six bf16
    products against the sustained dense bf16 peak, with its HBM rate beside it for the bytes it
    reads (6 B per row and history column, three bf16 slices) and for the hi+lo count of the
    benchmark's byte model (4 B); traffic = ncu reads scaled by the mean K plus ncu writes.
    near_far: the same kernel over a super-block's own earlier blocks (every block).
    solve: k_line_block_spec, bound by GB300's FP64 pipe and the per-step chain, not by HBM:
    microseconds per step, with the profile's FP64-pipe activity.
    whole_solve: the benchmark's blocked byte model (history read once per block of B = 64 steps as
    hi+lo bf16 plus the near history and state; and the same at the super-block length) over the
    whole solve time."""
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tflops_peak = peaks.get("bf16_tflops_sustained", 1700.0)
    tsrc = ("of measured (MEASURED_PEAKS.json bf16_tflops_sustained: the kernel runs inside a long solve)"
            if "bf16_tflops_sustained" in peaks else "of fallback 1.7 PFLOP/s sustained")
    out = {}
    t1, t3, t2 = tot[1], tot[3], tot[2]
    if t1["count"] > 0 and t1["ms"] > 0:
        sec = t1["ms"] / 1e3
        n = t1["count"]
        b6 = t1["bytes"]                                      # 6 B x nodes x K, summed over the launches
        b4 = b6 * 4.0 / 6.0
        k_mean = b6 / (6.0 * nodes * n)
        tf = t1["flops"] / sec / 1e12
        out["far_tc"] = {
            "kernel": "k_far_tc3 (tcgen05 far-history contraction, super-block of %d steps)" % (64 * sbk),
            "bound": "tensor", "achieved": tf, "peak": tflops_peak, "unit": "TFLOP/s", "frac": tf / tflops_peak,
            "peak_source": tsrc, "flops_counted": "6 bf16 products x 2 x rows x K x %d steps per launch" % (64 * sbk),
            "launches": n, "ms_per_launch": t1["ms"] / n, "mean_k": k_mean, "est_ms_per_solve": t1["ms"],
            "hbm_6B": {"achieved": b6 / sec / 1e9, "frac": b6 / sec / 1e9 / hbm, "unit": "GB/s",
                       "bytes_per_launch": b6 / n, "note": "three bf16 slices per history element"},
            "hbm_4B": {"achieved": b4 / sec / 1e9, "frac": b4 / sec / 1e9 / hbm, "unit": "GB/s",
                       "bytes_per_launch": b4 / n, "note": "hi+lo bf16 count of the benchmark's byte model"},
            "hbm_peak": hbm, "hbm_peak_source": hbm_src,
            "traffic": NCU_FAR["read_per_row_col"] * rows * k_mean + NCU_FAR["write_per_row"] * rows,
            "traffic_unit": "DRAM bytes per launch at the mean K (ncu reads scaled by K, writes per launch)",
            "traffic_source": NCU_FAR["source"]}
    if t3["count"] > 0 and t3["ms"] > 0:
        out["near_far"] = {"kernel": "k_far_tc3 (contraction over the super-block's own earlier blocks)",
                           "bound": "tensor", "launches": t3["count"], "ms_per_launch": t3["ms"] / t3["count"],
                           "est_ms_per_solve": t3["ms"],
                           "achieved": t3["flops"] / (t3["ms"] / 1e3) / 1e12, "unit": "TFLOP/s",
                           "peak": tflops_peak, "frac": t3["flops"] / (t3["ms"] / 1e3) / 1e12 / tflops_peak,
                           "peak_source": tsrc}
    if t2["count"] > 0 and t2["ms"] > 0:
        us = 1e3 * t2["ms"] / t2["count"]
        out["solve"] = {"kernel": "k_line_block_spec (far fold, float-float near history, speculative FP64 "
                                  "Thomas; one launch per 64-step block)",
                        "bound": "fp64-latency", "achieved": us, "unit": "us/step", "frac": None,
                        "limiter": "GB300's FP64 pipe (about one FP64 warp instruction per 19 cycles per SM) "
                                   "along the per-step chain of dependent operations, plus the per-step exchange",
                        "fp64_pipe_active": NCU_SOLVE["fp64_pipe_active"],
                        "fp64_pipe_source": NCU_SOLVE["source"] + " (ncu sm__pipe_fp64_cycles_active)",
                        "steps": t2["count"], "est_ms_per_solve": t2["ms"] * steps / t2["count"],
                        "traffic": NCU_SOLVE["per_node_step"] * nodes,
                        "traffic_unit": "DRAM bytes per step (ncu, scaled by nodes)",
                        "traffic_source": NCU_SOLVE["source"]}
    # the benchmark's blocked byte model, whole solve
    def model(B):
        tot_b = 0.0
        for n0 in range(0, steps, B):
            tot_b += 4.0 * n0 * nodes
            for t in range(n0, min(n0 + B, steps)):
                tot_b += (8.0 * (t - n0) + 60.0) * nodes
        return tot_b
    m64 = model(64)
    m_sb = 0.0
    for n0 in range(0, steps, 64):
        s0 = n0 - n0 % (64 * sbk)
        m_sb += (4.0 * s0 * nodes if n0 == s0 else 0.0) + 4.0 * (n0 - s0) * nodes
        for t in range(n0, min(n0 + 64, steps)):
            m_sb += (8.0 * (t - n0) + 60.0) * nodes
    sec = ms_solve / 1e3
    out["whole_solve"] = {"bound": "hbm", "unit": "GB/s", "peak": hbm, "peak_source": hbm_src,
                          "model_B64": {"bytes": m64, "achieved": m64 / sec / 1e9, "frac": m64 / sec / 1e9 / hbm,
                                        "note": "history as hi+lo bf16 read once per 64-step block + 8 B per near "
                                                "lag + 60 B per node-step"},
                          "model_superblock": {"bytes": m_sb, "achieved": m_sb / sec / 1e9,
                                               "frac": m_sb / sec / 1e9 / hbm,
                                               "note": "the same with the far history read once per %d-step "
                                                       "super-block (the library's schedule)" % (64 * sbk)}}
    return out


def checkpoint_errors(a, b):
    """Max and RMS relative error of state list a against b (normwise by max |b|)."""
    out = []
    for x, y in zip(a, b):
        x, y = np.concatenate([np.ravel(v) for v in x]), np.concatenate([np.ravel(v) for v in y])
        m = np.max(np.abs(y))
        out.append({"max_rel_err": float(np.max(np.abs(x - y)) / m),
                    "rms_rel_err": float(np.sqrt(np.mean((x - y) ** 2)) / m)})
    return out


def run_pieces(obj, u0_dev, steps, state, k=8):
    """A solve in k pieces; the state after each piece (the checkpoints)."""
    cps = [int(round((i + 1) * steps / k)) for i in range(k)]
    obj.reset(u0_dev)
    out, t = [], 0
    for c in cps:
        obj.run(c - t)
        t = c
        out.append(state())
    return cps, out


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import fpde_hpc_gb300 as fp

    wl = make_workload(args)
    ctx = fp.Context(local)
    # one explicit stream for the library and the timing events (a null handle would select
    # the library's own stream, which torch's events do not order against)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    lib = ctx.lib
    is_line = isinstance(wl, LineWorkload)
    is_sf = isinstance(wl, SfWorkload)
    # default: the exact three-slice split path (every workload has it), with the FP64 arm beside it;
    # the space-fractional workload defaults to FP64, the path that reproduces the reference bit for bit
    prec = {"auto": fp.FPDE_PREC_FP64 if is_sf else fp.FPDE_PREC_SPLIT_BF16X3, "fp64": fp.FPDE_PREC_FP64,
            "bf16": fp.FPDE_PREC_SPLIT_BF16, "f16": fp.FPDE_PREC_SPLIT_F16,
            "bf16x3": fp.FPDE_PREC_SPLIT_BF16X3}[args.precision]
    if not is_line and prec not in (fp.FPDE_PREC_FP64, fp.FPDE_PREC_SPLIT_BF16X3):
        raise SystemExit(f"{wl.name} runs in FP64 or the exact three-slice split")
    pname = {0: "fp64", 1: "split-bf16", 2: "split-fp16", 3: "split-bf16x3"}[prec]

    tuning = None
    lod_tuned = type(wl) is LodWorkload and not args.no_autotune
    if (is_line or lod_tuned) and not args.no_autotune:
        t0 = time.perf_counter()
        tuning = wl.autotune(ctx, prec)
        tune_s = time.perf_counter() - t0
    if is_line:
        obj = wl.build(ctx, prec, tuning)
    elif lod_tuned:
        obj = wl.build(ctx, prec, tuning[0])
    else:
        obj = wl.build(ctx, prec)
    u0_dev = torch.from_numpy(np.ascontiguousarray(wl.u0)).cuda()
    steps = wl.steps
    for _ in range(args.warmup):
        obj.reset(u0_dev)
        obj.run(steps)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    launches0 = lib.fpde_kernel_launch_count()
    it0 = obj.sf_iterations() if is_sf else 0
    ms = _timed(obj, u0_dev, steps, args.steps, stream)
    barrier()
    launches = lib.fpde_kernel_launch_count() - launches0
    sf_iters = (obj.sf_iterations() - it0) / args.steps if is_sf else 0
    clk = clocks.stop()
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    value = wl.node_steps * world / (ms / 1e3)
    u_main = obj.state()

    # end to end through the C ABI with host buffers (pinned)
    u0_h = torch.from_numpy(np.ascontiguousarray(wl.u0).copy()).pin_memory()
    out_h = torch.empty_like(u0_h).pin_memory()
    u0_np, out_np = u0_h.numpy(), out_h.numpy()
    obj.solve_host(u0_np, steps, out_np)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        obj.solve_host(u0_np, steps, out_np)
    e2e_s = (time.perf_counter() - t0) / args.steps
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, "cuda")
    bi, bo = wl.bytes_io()
    e2e = {"value": wl.node_steps * world / e2e_s, "unit": "node-steps/s", "h2d_bytes_per_step": bi,
           "d2h_bytes_per_step": bo, "ms_per_step": e2e_s * 1e3}

    peak, peak_src = measured_peaks()
    out = {"metric": wl.metric, "value": value, "unit": "node-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if prec == 0 else f"{pname}(tensor)+f64",
           "data": "synthetic (seeded; no dataset exists for this operator)",
           "config": bench_config(wl, world), "path": pname,
           "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if tuning is not None and lod_tuned:
        out["tuning"] = {"segments": list(tuning[0]), "tuned_ms_per_step": tuning[1], "autotune_seconds": tune_s,
                         "note": "segments per line of each pass (0 = the built-in rule), fpde_lod3d_autotune"}
    elif tuning is not None:
        out["tuning"] = {"solve_sp": tuning.solve_sp, "chunks": tuning.chunks,
                         "far_splits": tuning.far_splits, "gemv_splits": tuning.gemv_splits,
                         "far_super_blocks": tuning.far_super, "tuned_ms_per_step": tuning.ms_per_step,
                         "autotune_seconds": tune_s, "block_steps": 64}

    if is_line:
        # kernel rooflines from one separate probed solve (events inside the graph)
        every = max(1, steps // 32)
        tot = _probe(obj, u0_dev, steps, every)
        nodes = wl.p.N + 1
        if prec == 0:
            k = _kernel_entry(tot[0], "k_l1_partial (FP64 history GEMV)", peak, peak_src,
                              steps / max(tot[0]["count"], 1))
            kernels = {"hist_gemv": k} if k else {}
        elif prec == fp.FPDE_PREC_SPLIT_BF16X3:
            sbk = tuning.far_super if (tuning is not None and tuning.far_super) else 4
            rows = (nodes + 127) // 128 * 128
            kernels = split_line_rooflines(tot, steps, nodes, rows, sbk, ms, peak, peak_src)
        else:
            k = _kernel_entry(tot[1], "k_far_tc (tcgen05 far-history contraction, two-term split)", peak,
                              peak_src, 1.0)
            kernels = {"far_tc": k} if k else {}
        out["kernels"] = kernels
        if "far_tc" in kernels:
            out["roofline"] = dict(kernels["far_tc"])
            out["roofline_note"] = ("the tensor-core far contraction (the split path's HBM/tensor kernel); the "
                                    "block solve (kernels.solve) takes a comparable share but is bound by the "
                                    "FP64 pipe and its per-step chain, not by HBM or the tensor cores")
        elif "hist_gemv" in kernels:
            out["roofline"] = dict(kernels["hist_gemv"])
    elif is_sf:
        # FP64-pipe work. The fast form fuses every product into its sum (an FMA counted as 2 flops)
        # and sums dot products in trees; the exact form issues every multiply and add on its own (it
        # can reach at most half the nominal rate) and, on lines, adds each dot product on one lane.
        peak = 1250.0
        form = ("exact: the reference's order, separate multiplies and adds, at most 0.5 of the peak"
                if wl.exact else "fast: fused multiply-adds, tree dot products")
        if wl.impl3d:
            ops = sf_iters * wl.grid_iteration_ops()
            kern = "k_sf3d_solve (vmul_T_3d + solve_mln<1>, persistent cooperative)"
            note = (f"{sf_iters:.0f} solver iterations per run ({sf_iters / steps:.1f} per step) x "
                    f"{wl.grid_iteration_ops():.3g} FP64 flops per iteration; {form}; ncu on 64^3 "
                    "(profiles/k_sf3d_solve_64cube.md)")
        else:
            ops = sf_iters * wl.line_iteration_ops()
            lines = 3 * (wl.p.dims[0] - 1) ** 2 * steps
            kern = "k_lod_pass_sf (vmul_T + solve_mln<1>, one CTA per line)"
            note = (f"{sf_iters:.0f} solver iterations per solve ({sf_iters / lines:.1f} per line solve) x "
                    f"{wl.line_iteration_ops()} FP64 flops per line-iteration; {form}")
        gf = ops / (ms / 1e3) / 1e9
        out["roofline"] = {"kernel": kern, "bound": "fp64", "achieved": gf, "peak": peak, "unit": "GFLOP/s (FP64)",
                           "frac": gf / peak,
                           "peak_source": "nominal GB300 FP64 1.25 TFLOP/s (an FMA counted as 2 flops)",
                           "traffic": None, "note": note}
    else:
        # whole-step HBM roofline from the algorithmic history bytes of the run:
        #   FP64: 8 B x nodes x lags, summed over steps;
        #   split: 6 B (three bf16 slices) x nodes x far lags per 64-step block + 8 B x nodes x
        #          near lags per step (the FP64 ring)
        nodes = wl.node_steps / steps
        if prec == 0:
            alg = 8.0 * nodes * steps * (steps - 1) / 2
            name = "whole step (FP64 history GEMV dominant)"
        else:
            nb = steps // 64
            # far: every block b reads 64 b lags of 6 B per node; near: n % 64 ring rows of 8 B per step
            alg = 6.0 * nodes * 64 * nb * (nb - 1) / 2 + 8.0 * nodes * sum(n % 64 for n in range(steps))
            name = "whole step (tensor-core far history + FP64 near history + passes)"
        gbs = alg / (ms / 1e3) / 1e9
        out["roofline"] = {"kernel": name, "bound": "hbm", "achieved": gbs,
                           "peak": peak, "unit": "GB/s", "frac": gbs / peak, "peak_source": peak_src,
                           "traffic": None, "note": "algorithmic history bytes / whole solve time"}

    if prec != 0 and not args.no_fp64_arm:
        # the plain FP64 kernel on the same workload: speed-up and accuracy of the split path
        t64 = wl.autotune(ctx, fp.FPDE_PREC_FP64) if (is_line and not args.no_autotune) else None
        l64 = wl.build(ctx, fp.FPDE_PREC_FP64, t64) if is_line else wl.build(ctx, fp.FPDE_PREC_FP64)
        # both paths in eight pieces (untimed; the FP64 one is also its warm-up): max and RMS
        # relative error of the split path against FP64 at the 8 checkpoints and the final step
        cps, s64 = run_pieces(l64, u0_dev, steps, l64.state)
        _, ssp = run_pieces(obj, u0_dev, steps, obj.state)
        ms64 = _timed(l64, u0_dev, steps, 1, stream)
        u64 = l64.state()
        err = float(np.max(np.abs(u_main - u64)) / np.max(np.abs(u64)))
        rms = float(np.sqrt(np.mean((u_main - u64) ** 2)) / np.max(np.abs(u64)))
        cp_err = checkpoint_errors(ssp, s64)
        for c, e in zip(cps, cp_err):
            e["step"] = c
        out["fp64_kernel"] = {"value": wl.node_steps / (ms64 / 1e3), "ms_per_step": ms64}
        if is_line:
            tot64 = _probe(l64, u0_dev, steps, max(1, steps // 32))
            r64 = _kernel_entry(tot64[0], "k_l1_partial (FP64 history GEMV)", peak, peak_src,
                                steps / max(tot64[0]["count"], 1))
            if r64:
                r64["fp64_fma_ceiling_gbs"] = 4800.0
            out["fp64_kernel"]["roofline"] = r64
        l64.close()
        out["split_vs_fp64"] = {"speedup": ms64 / ms, "max_rel_err": max([err] + [e["max_rel_err"] for e in cp_err]),
                                "final_max_rel_err": err, "final_rms_rel_err": rms, "checkpoints": cp_err,
                                "bound": 1e-7, "norm": "relative to max |u_fp64| at the same step"}
    obj.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not getattr(args, "max_lag", 0):
        threads = os.cpu_count() or 1
        out["cpu_baseline"] = cpu_record(wl, [(s, wl.run_sample(s, threads)) for s in wl.sample_lengths()],
                                         threads)
    ctx.close()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("sum1", "sum2"):
        run_sum(args, SumWorkload(args))
    elif args.workload == "weights":
        run_weights(args, WeightsWorkload(args))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
