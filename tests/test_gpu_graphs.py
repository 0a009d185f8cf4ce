"""CUDA-graph policy of the device time loops (fpde_line_run, fpde_step_block).

A caller that advances a line one step or one 64-step block at a time (the reference's own time
loop through the drop-in adapter) must not instantiate a graph per call; long runs replay cached
graphs, of which at most eight are kept. Every calling pattern gives the same result as one long
run: the same kernels with the same arguments, except that a block solve started in the middle
of a block rebuilds its near-history sums in another order (1e-12 normwise covers that).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(u, ref):
    assert float(np.max(np.abs(u - ref)) / np.max(np.abs(ref))) <= 1e-12


@pytest.fixture(scope="module")
def ctx():
    import fpde_hpc_gb300 as fp
    c = fp.Context(0)
    yield c
    c.close()


def _line(ctx, precision, steps, N=3000):
    import fpde_hpc_gb300 as fp
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=N, steps=steps)
    A, B, R = p.coefs()
    return fp.Line(ctx, p.N, p.alpha, p.tau, p.Da, A, B, R, p.u0, steps, precision=precision)


@pytest.mark.parametrize("precision", [0, 3])
def test_stepwise_and_blockwise_callers_instantiate_no_graph(ctx, precision):
    steps = 200
    ref = _line(ctx, precision, steps)
    ref.run(steps)
    u_ref = ref.state()
    assert ref.graph_stats() == (1, 1)
    ref.close()

    one = _line(ctx, precision, steps)
    for _ in range(steps):
        one.run(1)
    assert one.graph_stats() == (0, 0)
    _same(one.state(), u_ref)
    one.close()

    blk = _line(ctx, precision, steps)
    while blk.step_block():
        pass
    assert blk.steps_done == steps
    assert blk.graph_stats() == (0, 0)
    _same(blk.state(), u_ref)
    blk.close()


def test_long_runs_replay_a_bounded_cache(ctx):
    from fpde_hpc_gb300 import problems
    p = problems.config2(N=2000, steps=128 * 12)
    line = _line(ctx, 3, 128 * 12, N=2000)
    for _ in range(3):                                    # three 128-step runs: three graphs
        line.run(128)
    assert line.graph_stats() == (3, 3)
    u3 = line.state()
    line.reset(p.u0)
    for _ in range(3):                                    # the same runs again: replayed
        line.run(128)
    assert line.graph_stats() == (3, 3)
    np.testing.assert_array_equal(line.state(), u3)
    for _ in range(9):                                    # nine more positions: eight kept
        line.run(128)
    cached, made = line.graph_stats()
    assert cached == 8 and made == 12
    ref = _line(ctx, 3, 128 * 12, N=2000)
    ref.run(128 * 12)
    _same(line.state(), ref.state())
    ref.close()
    line.close()
