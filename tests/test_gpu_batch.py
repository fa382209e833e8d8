"""Batched form: many independent grids of uneven sizes in one persistent launch per step.

The persistent schedule, the looped schedule (one launch per grid), CUDA-graph replay and
the single-grid context call the same compiled tile function (not inlined into the kernels),
so they must agree bit for bit, and, to the fast path's tolerance, with the oracle.
Different tile shapes are different instantiations that the compiler may fuse differently:
they agree to rounding.  Autotuning itself must leave the state, dt and time untouched."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems
from gpu_util import gpu_run, max_rel_l1, oracle_run

pytestmark = pytest.mark.gpu


def small_batch(n=12, seed=3):
    return problems.batch_four_quadrant(n, lo=20, hi=90, seed=seed)


def run_batch(grids, nsteps, schedule=g.BATCH_PERSISTENT, use_graph=False, autotune=False):
    b = g.Batch([c for c, *_ in grids])
    for k, (c, s, u, _) in enumerate(grids):
        b.import_grid(k, s, u)
    b.set_time(0.0, 0.0)
    b.init_dt()
    if autotune:
        b.autotune(reps=2)
    b.advance(nsteps, schedule=schedule, use_graph=use_graph)
    out = []
    for k, (c, s, u, _) in enumerate(grids):
        s2, u2 = np.zeros_like(s), np.zeros_like(u)
        b.export_grid(k, s2, u2)
        out.append((s2, u2, b.stats(k)))
    info = b.info()
    b.close()
    return out, info


def same(a, c):
    return all(np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1]) and
               x[2].t == y[2].t and x[2].dt == y[2].dt for x, y in zip(a, c))


def test_persistent_equals_looped_and_graph(cuda):
    grids = small_batch()
    a, info = run_batch(grids, 9)
    assert info.ngrids == len(grids) and info.tiles > 0
    c, _ = run_batch(grids, 9, schedule=g.BATCH_LOOPED)
    d, _ = run_batch(grids, 9, use_graph=True)
    assert same(a, c) and same(a, d)
    for x in a:
        assert x[2].steps == 9 and x[2].nonfinite == 0


def test_autotune_keeps_state_and_any_tile_shape_agrees(cuda):
    grids = small_batch(seed=4)
    # autotuning alone leaves every grid's state, dt and time as imported
    t0, _ = run_batch(grids, 0)
    t1, info = run_batch(grids, 0, autotune=True)
    assert all(t > 0 for t in info.tuned_ms)
    assert same(t0, t1)
    # the tuned shape advances the grids as the default shape does, to rounding
    a, _ = run_batch(grids, 6)
    c, _ = run_batch(grids, 6, autotune=True)
    for (c_, *_), x, y in zip(grids, a, c):
        assert max_rel_l1(c_, (x[0], x[1], None), (y[0], y[1], None)) <= 1e-13
        assert abs(x[2].t - y[2].t) <= 1e-13 * x[2].t and x[2].steps == y[2].steps


def test_batch_grid_equals_single_grid_context(cuda):
    grids = small_batch(n=5, seed=5)
    a, _ = run_batch(grids, 7)
    for (cfg, s, u, b), (s2, u2, st) in zip(grids, a):
        ss, us, _, sst = gpu_run(cfg, s, u, b, 7)
        assert np.array_equal(ss, s2) and np.array_equal(us, u2)
        assert sst.t == st.t and sst.dt == st.dt


def test_batch_against_oracle(cuda, oracle_lib):
    grids = small_batch(n=4, seed=6)
    a, _ = run_batch(grids, 10)
    for (cfg, s, u, b), (s2, u2, st) in zip(grids, a):
        so, uo, bo, T_do, TT = oracle_run(oracle_lib, cfg, s, u, b, 10)
        assert max_rel_l1(cfg, (s2, u2, None), (so, uo, None)) <= 1e-10
        assert abs(st.t - TT) <= 1e-11 * TT


def test_looped_sync_equals_looped(cuda):
    """GD_BATCH_LOOPED_SYNC (the host waiting for each launch, as the reference's main loop)
    steps every grid exactly as GD_BATCH_LOOPED; it cannot be captured in a graph."""
    grids = small_batch(6)
    a, _ = run_batch(grids, 5, schedule=g.BATCH_LOOPED)
    c, _ = run_batch(grids, 5, schedule=g.BATCH_LOOPED_SYNC)
    for (s1, u1, st1), (s2, u2, st2) in zip(a, c):
        assert np.array_equal(s1, s2) and np.array_equal(u1, u2)
        assert st1.t == st2.t and st1.dt == st2.dt
    with pytest.raises(g.GdError):
        run_batch(grids, 1, schedule=g.BATCH_LOOPED_SYNC, use_graph=True)


def test_persistent_16x16_keeps_four_ctas_per_sm(cuda):
    """The persistent kernel of the default 16x16 tile runs four CTAs per SM, as the
    single-grid step does (registers and shared memory both allow four).  Its register count
    is sensitive to the tile function's code: at 74 registers it fell to three CTAs per SM
    and the batched step slowed by 13 %."""
    import torch
    grids = problems.batch_four_quadrant(64, lo=64, hi=512, seed=5)
    b = g.Batch([c for c, *_ in grids])
    for k, (c, s, u, _) in enumerate(grids):
        b.import_grid(k, s, u)
    info = b.info()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    b.close()
    assert (info.tile_x, info.tile_y) == (16, 16)
    assert info.ctas == min(4 * sms, info.tiles), (info.ctas, sms)
