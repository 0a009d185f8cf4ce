"""C++ host programs calling the library through include/fpde_gb300.h, as the reference would.

tests/cpp/dropin_sum.cpp is the reference's caller (calc_step -> fr_ocl_call_sum ->
time_summing, fpde_hpc_1d.cpp:5155-5158, :1819-1883, :4100-4104) with the
library's gb300_call_sum adapter in place of fr_ocl_call_sum, replayed on the reference's own recorded column run
(tests/golden/fpde_column_a2: its snapshots, kb_3_cache and tau of every step); its Sums must
equal the reference's to 1e-12. tests/cpp/dropin_line.cpp advances a column on the device in one
call, block by block (fpde_step_block) and step by step, each compared with the oracle.
tests/cpp/dropin_sf3d.cpp is calc_step's implicit3d solve_mln<1>(..., vmul_T_3d) call
(fpde_hpc_1d.cpp:5705) with the library in its place, fed the reference's recorded system
(tests/golden/fpde_sf3d_*): its product and solution must equal the reference's bit for bit.

Without a GPU the programs are compiled and linked only (the -m "not gpu" run); on the GPU they
run.
"""
import os
import subprocess

import numpy as np
import pytest

import fgv
import oracle
from conftest import ROOT, golden_path

CPP = os.path.join(ROOT, "tests", "cpp")


@pytest.fixture(scope="module")
def programs(tmp_path_factory):
    from fpde_hpc_gb300 import build
    lib = build.build()
    d = tmp_path_factory.mktemp("dropin")
    exe = {}
    for name in ("dropin_sum", "dropin_line", "dropin_sf3d"):
        out = str(d / name)
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"),
               os.path.join(CPP, name + ".cpp"), "-L", os.path.dirname(lib), "-lfpde_gb300",
               "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert p.returncode == 0, " ".join(cmd) + "\n" + p.stdout
        exe[name] = out
    return exe, d


def test_dropin_programs_compile_and_link(programs):
    exe, _ = programs
    for path in exe.values():
        assert os.access(path, os.X_OK)


def _run(exe, inp, out):
    p = subprocess.run([exe, inp, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert p.returncode == 0, p.stdout
    return p.stdout


@pytest.mark.gpu
def test_reference_call_sequence_reproduces_reference_sums(programs):
    exe, d = programs
    g = fgv.load(golden_path("fpde_column_a2"))
    U0, U = g["U0"].reshape(-1), g["U"].reshape(g["U"].shape[0], -1)
    steps, nodes = U.shape
    off = g["kb_off"].astype(np.int64)
    inp, out = str(d / "sum.in"), str(d / "sum.out")
    with open(inp, "wb") as f:
        np.array([nodes, steps], dtype="<i8").tofile(f)
        U0.astype("<f8").tofile(f)
        U.astype("<f8").tofile(f)
        g["tau"][:steps].astype("<f8").tofile(f)
        off[:steps + 1].astype("<i8").tofile(f)
        g["kb_flat"][:off[steps]].astype("<f8").tofile(f)
    _run(exe["dropin_sum"], inp, out)
    S = np.fromfile(out, dtype="<f8").reshape(steps - 1, nodes)
    # the reference writes its sums on the K-pass nodes only (others keep stale memory)
    sN, M, K = int(g["sN"]), int(g["M"]), int(g["K"])
    mask = np.zeros(g["U0"].shape, dtype=bool)
    mask[1:K + 1, 1:M, 1:sN] = True
    mask = mask.reshape(-1)
    worst = 0.0
    for n in range(1, steps):
        ref = g["S"][n].reshape(-1)[mask]
        worst = float(np.maximum(worst, float(np.max(np.abs(S[n - 1][mask] - ref)) / np.max(np.abs(ref)))))
    print(f"C++ drop-in Sums over {steps - 1} steps vs the reference's: max rel err {worst:.2e}")
    assert worst <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (3, 1e-7)])
def test_cpp_column_whole_blockwise_stepwise(programs, precision, tol):
    from fpde_hpc_gb300 import problems
    exe, d = programs
    p = problems.config2(N=4000, steps=200)
    inp, out = str(d / f"line{precision}.in"), str(d / f"line{precision}.out")
    with open(inp, "wb") as f:
        np.array([p.N, p.steps, precision], dtype="<i8").tofile(f)
        np.array([p.alpha, p.tau, p.Da], dtype="<f8").tofile(f)
        p.k.astype("<f8").tofile(f)
        p.u0.astype("<f8").tofile(f)
    log = _run(exe["dropin_line"], inp, out)
    ways = np.fromfile(out, dtype="<f8").reshape(3, p.N + 1)
    A, B, R = p.coefs()
    uref, _ = oracle.line_run(p.u0, p.steps, p.tau, p.alpha, p.Da, A, B, R)
    for name, u in zip(("whole", "blocks", "steps"), ways):
        err = float(np.max(np.abs(u - uref)) / np.max(np.abs(uref)))
        print(f"C++ column ({name}, precision {precision}) vs oracle: {err:.2e}")
        assert err <= tol, name
    # a block-by-block or step-by-step caller instantiates no CUDA graph
    assert "way 1: 200 steps, graphs cached 0, instantiated 0" in log
    assert "way 2: 200 steps, graphs cached 0, instantiated 0" in log


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["fpde_sf3d_sd1", "fpde_sf3d_tight"])
def test_cpp_sf3d_solve_reproduces_reference(programs, name):
    import sf3d_cases
    exe, d = programs
    c = sf3d_cases.load(name)
    g = c["g"]
    sN, M, K = c["dims"]
    inp, out = str(d / f"{name}.in"), str(d / f"{name}.out")
    with open(inp, "wb") as f:
        np.array([sN, M, K, c["space_der"], c["maxiter"]], dtype="<i8").tofile(f)
        np.array([c["thr"]], dtype="<f8").tofile(f)
        for a in (g["sys_last_mat"], c["mc3d"], *c["Tm3"], c["iw3"], g["sys_last_om"], g["solve_x0"], g["mv_x"]):
            np.ascontiguousarray(a, dtype="<f8").tofile(f)
    _run(exe["dropin_sf3d"], inp, out)
    V = c["V"]
    res = np.fromfile(out, dtype="<f8", count=2 * V)
    iters = int(np.fromfile(out, dtype="<i8", offset=16 * V)[0])
    assert np.array_equal(res[:V], g["mv_r"])
    assert np.array_equal(res[V:], g["solve_sol"]) and iters == c["solve_iters"]
