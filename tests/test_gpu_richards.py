"""The reference's Richards problem on the GPU: solution-dependent line coefficients.

The reference's analytic_test 0 (van Genuchten-Mualem water content, k_form 1 VGM and 2 Averianov
conductivity, no irrigation, zero-flux bottom and sides; fpde_hpc_1d.cpp:2493-2657, :3095-3142)
changes every line's A_/B/R with the solution, so the 3D LOD forms them on the device before
each line solve (fpde_richards). Checks:
  * replay of the reference's own 40-step run on 6^3 cells (fixtures fpde_richards_k1/k2, the
    K-pass source and the evaporation rate of every step recorded by the pin harness): every grid
    within 1e-12 of the reference's (the device's pow and the host's differ by an ulp or two);
  * the split path (far history on the tensor cores) within 1e-7 of FP64 on the same run.
"""
import numpy as np
import pytest

import fgv
from conftest import golden_path
from conftest import relmax

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _lod(ctx, g, kform, precision=0, steps=None):
    import fpde_hpc_gb300 as fp
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    steps = steps or len(g["tau"])
    rich = dict(k_form=kform, k_sat=g["k_sat"], sZ=g["sZ"], dL=(g["sdL"], g["dLx"], g["dLy"]), evaporation=g["E"])
    return fp.Lod3D(ctx, dims, g["alpha"], g["tau"][0], g["Da"], None, None, None, g["U0"], steps,
                    source=g["Rp"], richards=rich, precision=precision)


@pytest.mark.parametrize("kform", [1, 2])
def test_richards_lod_replays_reference_run(ctx, kform):
    g = fgv.load(golden_path(f"fpde_richards_k{kform}"))
    lod = _lod(ctx, g, kform)
    worst = 0.0
    for n in range(len(g["tau"])):
        lod.run(1)
        worst = max(worst, relmax(lod.state(), g["U"][n]))
    lod.close()
    print(f"Richards k_form {kform}: every level vs the reference's run, max rel {worst:.2e}")
    assert worst <= 1e-12


@pytest.mark.parametrize("kform", [1, 2])
def test_richards_lod_runs_in_one_call(ctx, kform):
    g = fgv.load(golden_path(f"fpde_richards_k{kform}"))
    steps = len(g["tau"])
    lod = _lod(ctx, g, kform)
    lod.run(steps)
    e64 = relmax(lod.state(), g["U"][-1])
    lod.close()
    print(f"Richards k_form {kform}, {steps} steps in one call: FP64 vs reference {e64:.2e}")
    assert e64 <= 1e-12


@pytest.mark.parametrize("kform", [1, 2])
def test_richards_lod_split_history_vs_fp64(ctx, kform):
    """200 steps (the recorded source and evaporation rate of the last step repeat): the far
    history of three 64-step blocks on the tensor cores, the coefficients from the solution."""
    g = fgv.load(golden_path(f"fpde_richards_k{kform}"))
    out = []
    for prec in (0, 3):
        lod = _lod(ctx, g, kform, prec, steps=200)
        states = []
        for _ in range(8):
            lod.run(25)
            states.append(lod.state())
        out.append(states)
        lod.close()
    errs = [relmax(x, y) for x, y in zip(out[1], out[0])]
    print(f"Richards k_form {kform}, 200 steps, split vs FP64 at 8 checkpoints: max {max(errs):.2e}")
    assert max(errs) <= 1e-7


def _rich_line(N, steps, kform):
    """A Richards column in the reference's units: depth 3 m in N intervals, H0 = -0.8 - Z,
    Dirichlet H0 - Z[N] at the bottom (bottom_cond 1), the surface condition from the recorded
    evaporation rates of the pinned 3D run, tau 900 s."""
    import math
    g = fgv.load(golden_path(f"fpde_richards_k{kform}"))
    Z = np.arange(N + 1) * 3.0 / N
    dL = np.full(N + 1, 3.0 / N)
    u0 = -0.8 - Z
    alpha = float(g["alpha"])
    return dict(Z=Z, dL=dL, u0=u0, alpha=alpha, Da=1.0 / math.gamma(1.0 - alpha), tau=900.0, E=g["E"],
                ksat=float(g["k_sat"]), kform=kform, N=N, steps=steps)


def _gpu_line(ctx, c, precision, pieces=1):
    import fpde_hpc_gb300 as fp
    rich = dict(k_form=c["kform"], k_sat=c["ksat"], Z=c["Z"], dL=c["dL"], evaporation=c["E"])
    line = fp.Line(ctx, c["N"], c["alpha"], c["tau"], c["Da"], None, None, None, c["u0"], c["steps"],
                   right=(0, c["u0"][-1]), precision=precision, richards=rich)
    out = []
    for k in range(pieces):
        line.run(c["steps"] // pieces)
        out.append(line.state())
    line.close()
    return out


@pytest.mark.parametrize("kform,N", [(1, 2000), (2, 2000), (2, 50000)])
def test_richards_line_fp64_vs_oracle(ctx, kform, N):
    """The line's coefficients from its state every step (k_rich_coefs) and the scan-based Thomas
    solve (k_rich_thomas) against the oracle's sequential restatement: 1e-12, or 4x the oracle's
    one-ulp envelope (node coordinates and steps moved by one ulp) where that is larger."""
    import oracle
    c = _rich_line(N, 100, kform)
    u = _gpu_line(ctx, c, 0)[0]
    ref, _ = oracle.line_run_richards(c["u0"], c["steps"], c["tau"], c["alpha"], c["Da"], c["Z"], c["dL"], kform,
                                      c["ksat"], c["E"], rtype=0, gN=c["u0"][-1])
    rng = np.random.default_rng(0)
    pert = lambda x: x * (1 + 2.2e-16 * rng.choice([-1, 1], size=x.shape))
    ref2, _ = oracle.line_run_richards(c["u0"], c["steps"], c["tau"], c["alpha"], c["Da"], pert(c["Z"]),
                                       pert(c["dL"]), kform, c["ksat"], c["E"], rtype=0, gN=c["u0"][-1])
    env, err = relmax(ref2, ref), relmax(u, ref)
    print(f"Richards line k_form {kform} N={N}, 100 steps: GPU vs oracle {err:.2e} (one-ulp envelope {env:.2e})")
    assert err <= max(1e-12, 4 * env)


@pytest.mark.parametrize("kform", [1, 2])
def test_richards_line_split_vs_fp64(ctx, kform):
    c = _rich_line(4000, 256, kform)
    a, b = _gpu_line(ctx, c, 0, 8), _gpu_line(ctx, c, 3, 8)
    errs = [relmax(x, y) for x, y in zip(b, a)]
    print(f"Richards line k_form {kform}, 256 steps, split vs FP64 at 8 checkpoints: max {max(errs):.2e}")
    assert max(errs) <= 1e-7


def _salt_lod(ctx, g, steps=None):
    import fpde_hpc_gb300 as fp
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    steps = steps or len(g["tau"])
    rich = dict(k_form=int(g["k_form"]), k_sat=g["k_sat"], sZ=g["sZ"], dL=(g["sdL"], g["dLx"], g["dLy"]),
                evaporation=g["E"], c0=g["C0"], nu=g["nu"], sigma=g["sigma"], D=g["D"])
    return fp.Lod3D(ctx, dims, g["alpha"], g["tau"][0], g["Da"], None, None, None, g["U0"], steps, richards=rich)


def test_richards_salt_lod_replays_reference_run(ctx):
    """The reference's run with the salt concentration (equation 1 beside H on every line: chemical
    osmosis in H, the H-driven transport and osmosis in C, C's own history; 6^3 cells, 24 steps):
    H and C at every level within 1e-12 of the reference's (device and host pow differ by an ulp)."""
    g = fgv.load(golden_path("fpde_richards_ct"))
    lod = _salt_lod(ctx, g)
    wu = wc = 0.0
    for n in range(len(g["tau"])):
        lod.run(1)
        wu = max(wu, relmax(lod.state(), g["U"][n]))
        wc = max(wc, relmax(lod.concentration(), g["C"][n]))
    lod.close()
    print(f"Richards with salt: H {wu:.2e}, C {wc:.2e} vs the reference's run")
    assert wu <= 1e-12 and wc <= 1e-12


def test_richards_salt_one_call_reset_and_errors(ctx):
    """One call equals step by step; a reset restores the salt field; the options the salt field does
    not support are refused."""
    import fpde_hpc_gb300 as fp
    g = fgv.load(golden_path("fpde_richards_ct"))
    steps = len(g["tau"])
    lod = _salt_lod(ctx, g)
    lod.run(steps)
    u1, c1 = lod.state(), lod.concentration()
    lod.reset(g["U0"])
    np.testing.assert_array_equal(lod.concentration(), g["C0"])
    lod.run(steps)
    np.testing.assert_array_equal(lod.state(), u1)
    np.testing.assert_array_equal(lod.concentration(), c1)
    lod.close()
    assert relmax(c1, g["C"][-1]) <= 1e-12
    dims = (int(g["sN"]), int(g["M"]), int(g["K"]))
    rich = dict(k_form=1, k_sat=g["k_sat"], sZ=g["sZ"], dL=(g["sdL"], g["dLx"], g["dLy"]), evaporation=g["E"],
                c0=g["C0"], nu=g["nu"], sigma=g["sigma"], D=g["D"])
    with pytest.raises(fp.FpdeError):           # the salt field runs on the FP64 path only
        fp.Lod3D(ctx, dims, g["alpha"], g["tau"][0], g["Da"], None, None, None, g["U0"], 70, richards=rich,
                 precision=3)
