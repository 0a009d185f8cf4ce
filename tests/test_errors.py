"""Every entry point reports bad arguments as an FPDE_ERR_* status with a message (the
reference's OpenCL layer calls exit(0) instead, opencl_cuda_base.cpp:14-17): host-side
functions here, device objects in the gpu-marked tests below."""
import numpy as np
import pytest

FPDE_ERR_ARG, FPDE_ERR_CAPACITY, FPDE_ERR_UNSUPPORTED = 1, 4, 6


def _raises(code, fn, *args, **kw):
    import fpde_hpc_gb300 as fp
    with pytest.raises(fp.FpdeError) as e:
        fn(*args, **kw)
    assert e.value.code == code, (e.value.code, str(e.value))
    assert "failed with status" in str(e.value) and len(str(e.value)) > 30
    return e.value


def test_host_functions_reject_bad_arguments():
    import fpde_hpc_gb300 as fp
    _raises(FPDE_ERR_ARG, fp.line_coefs, np.ones(1), np.ones(1))            # N < 2
    _raises(FPDE_ERR_ARG, fp.weights_l1, 1.5, np.arange(4.0), 4)           # alpha outside (0, 1)
    _raises(FPDE_ERR_ARG, fp.do_weights, [1.5], [1.0], 0.1, 3)             # order outside [0, 1]


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _line(ctx, N=1000, steps=70, **kw):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=N, steps=steps)
    A, B, R = p.coefs()
    return fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, steps, **kw), p


@pytest.mark.gpu
def test_line_rejects_bad_shapes_and_capacity(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=1000, steps=10)
    A, B, R = p.coefs()
    _raises(FPDE_ERR_ARG, fp.Line, ctx, 1, p.alpha, p.tau, p.Da, A, B, R, p.u0, 10)          # N < 2
    _raises(FPDE_ERR_ARG, fp.Line, ctx, p.N, p.alpha, -1.0, p.Da, A, B, R, p.u0, 10)        # tau <= 0
    _raises(FPDE_ERR_ARG, fp.Line, ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, 10, precision=9)
    for prec in (0, 3):
        line, _ = _line(ctx, precision=prec)
        line.run(60)
        _raises(FPDE_ERR_CAPACITY, line.run, 11)                          # beyond max_steps
        assert line.steps_done == 60                                       # nothing ran
        assert line.step_block() == 4                                      # the rest: 64 .. 70
        assert line.step_block() == 6
        assert line.step_block() == 0                                      # history full
        assert np.isfinite(line.state()).all()
        line.close()


@pytest.mark.gpu
def test_grid_and_ensemble_reject_bad_shapes(ctx):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config4(n=8, steps=4)
    cA, cB, cR = p.coefs()
    # one interval along K: arrays shaped for it, rejected by the library (every axis needs 2)
    sl = lambda a: np.ascontiguousarray(a[..., :3, :, :])
    _raises(FPDE_ERR_ARG, fp.Lod3D, ctx, (8, 8, 1), p.alpha, p.tau, p.Da, sl(cA), sl(cB), sl(cR), sl(p.u0), 4)
    with pytest.raises((fp.FpdeError, ValueError)):
        fp.Batch(ctx, [], 4)
