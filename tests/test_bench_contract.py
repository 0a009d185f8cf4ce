"""bench.py's reference arm on small cases (CPU only): one JSON line with the keys the
benchmark contract asks for, for every workload family, and the restricted-summing option of
the line workload."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

CASES = [
    ["--workload", "config2", "--nodes", "1024", "--time-steps", "96"],
    ["--workload", "config3", "--nodes", "1024", "--time-steps", "96"],
    ["--workload", "config4", "--nodes", "12", "--time-steps", "24"],
    ["--workload", "config5", "--nodes", "6", "--time-steps", "64"],
    ["--workload", "sum2", "--nodes", "24"],
    ["--workload", "weights", "--time-steps", "256"],
    ["--workload", "sf3d", "--nodes", "12", "--time-steps", "8"],
    ["--workload", "sf3d", "--nodes", "12", "--time-steps", "8", "--implicit3d", "1"],
]


@pytest.mark.parametrize("args", CASES, ids=[" ".join(c[1::2]) for c in CASES])
def test_reference_arm_json(args):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                         env=env, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert "workload" in d["config"]
    if args[1].startswith("config"):
        # time-stepping workloads: an extrapolation from at least three timed sample lengths, with
        # the fit, its residual and the seconds timed in the record; one timed sample per step
        assert cb["extrapolated"] is True
        fit = cb["fit"]
        assert len({x["steps"] for x in fit["samples"]}) >= 3 and fit["relative_rms_residual"] >= 0
        assert fit["a"] >= 0 and fit["b"] >= 0 and cb["seconds_timed"] > 0
        assert len(cb["timed_steps"]) == d["steps"]
        assert d["ms_per_step"] > 0


def test_line_workload_restricted_threshold():
    """--max-lag turns into the threshold that keeps exactly that many lags."""
    sys.path.insert(0, ROOT)
    import bench
    import fpde_hpc_gb300 as fp
    old = sys.argv
    try:
        sys.argv = ["bench.py", "--max-lag", "300", "--nodes", "1024", "--time-steps", "1000"]
        a = bench.parse()
    finally:
        sys.argv = old
    w = bench.LineWorkload("config2", a)
    b = fp.weights_l1_lags(w.p.alpha, 1001)
    kkk0 = w.p.tau ** (1 - w.p.alpha) / (1 - w.p.alpha)
    assert fp.restricted_lags(kkk0 * b[1:], w.restrict_eps) == 300
    assert "newest 300 lags" in w.metric


def test_reference_arm_under_two_ranks():
    """Launched as the multi-GPU runs are (torch.distributed.run, two ranks, 127.0.0.1): rank 0
    alone measures and prints one JSON line; the other rank exits 0 without work."""
    import socket
    with socket.socket() as sk:                      # a free port for the rendezvous
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "config2", "--nodes", "512",
           "--time-steps", "48"]
    out = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def _rank_main(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, "cpu")     # rank 1 is the slower replica
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    """The N > 1 timing rule (each rank's time reduced to the maximum) on two gloo ranks."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=300)
        assert all(p.exitcode == 0 for p in procs)
        assert dict(out) == {0: 2.5, 1: 2.5}
