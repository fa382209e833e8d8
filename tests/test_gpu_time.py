"""Time control of the resident loop: the dt policy (gd_set_dt_policy) and advancing to a
given time (gd_advance_to), in parity mode bit for bit against the oracle driven with the
same protocol, and in fast mode with and without graphs."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems
from gpu_util import grid_of

pytestmark = pytest.mark.gpu


def oracle_current(o, cfg, s, u, b, nsteps):
    """Each step with the CFL dt of its own input state."""
    grid = grid_of(cfg)
    t = 0.0
    for _ in range(nsteps):
        T = o.dt_only(grid, s, u, b)
        s, u, b, _ = o.step(grid, s, u, b, T)
        t = t + T
    return s, u, b, t


def oracle_to(o, cfg, s, u, b, t_end):
    """The lagged protocol from a dt-only pre-pass, every dt limited to what is left to
    t_end, until the state's time is within 1e-14 t_end of it.  Returns the state, its
    time, the steps taken and the last CFL dt before the limit."""
    grid = grid_of(cfg)
    T_cfl = o.dt_only(grid, s, u, b)
    t = 0.0
    T_do = min(T_cfl, max(t_end - t, 0.0))
    n = 0
    while t_end - t > 1e-14 * t_end:
        s, u, b, T_cfl = o.step(grid, s, u, b, T_do)
        t = t + T_do
        T_do = min(T_cfl, max(t_end - t, 0.0))
        n += 1
    return s, u, b, t, n, T_cfl


def export(sol, s, u, b):
    s2, u2 = np.zeros_like(s), np.zeros_like(u)
    b2 = None if b is None else np.zeros_like(b)
    sol.export_state(s2, u2, b2)
    return s2, u2, b2


@pytest.mark.parametrize("use_graph", [False, True])
def test_dt_current_matches_oracle(cuda, oracle_lib, use_graph):
    cfg, s, u, b = problems.sod(64, 32, mode=g.MODE_PARITY)
    sol = g.Solver(cfg)
    sol.set_dt_policy(g.DT_CURRENT)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    l0 = sol.launch_count()
    sol.advance(12, use_graph=use_graph)
    assert sol.launch_count() - l0 == 12 * 3  # dt-only pass, commit, step
    so, uo, _, to = oracle_current(oracle_lib, cfg, s, u, None, 12)
    sg, ug, _ = export(sol, s, u, None)
    st = sol.stats()
    sol.close()
    assert np.array_equal(sg, so) and np.array_equal(ug, uo)
    assert st.t_state == to and st.steps == 12


@pytest.mark.parametrize("problem", ["sod", "ot"])
def test_advance_to_matches_oracle(cuda, oracle_lib, problem):
    if problem == "sod":
        cfg, s, u, b = problems.sod(64, 32, mode=g.MODE_PARITY)
        t_end = 0.05
    else:
        cfg, s, u, b = problems.orszag_tang(48, 48, mode=g.MODE_PARITY)
        t_end = 0.02
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    n = sol.advance_to(t_end)
    st = sol.stats()
    sg, ug, bg = export(sol, s, u, b)
    so, uo, bo, to, no, T_cfl = oracle_to(oracle_lib, cfg, s, u, b, t_end)
    assert n == no and st.steps == no
    assert st.t_state == to and abs(to - t_end) <= 1e-14 * t_end
    assert np.array_equal(sg, so) and np.array_equal(ug, uo)
    if b is not None:
        assert np.array_equal(bg, bo)
    # the limit is cleared: the pending dt is the CFL dt again
    assert st.dt == T_cfl
    sol.advance(1)
    assert sol.stats().t_state == to + T_cfl
    sol.close()


def test_advance_to_fast_graph_equals_plain(cuda):
    cfg, s, u, b = problems.orszag_tang(128, 128, mode=g.MODE_FAST)
    out = []
    for use_graph in (False, True):
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        n = sol.advance_to(0.03, use_graph=use_graph)
        st = sol.stats()
        out.append((n, st.t_state) + export(sol, s, u, b))
        sol.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    assert abs(out[0][1] - 0.03) <= 1e-14 * 0.03
    for x, y in zip(out[0][2:], out[1][2:]):
        assert np.array_equal(x, y)


def test_advance_to_respects_max_steps_and_rejects_past_times(cuda):
    cfg, s, u, b = problems.sod(32, 32, mode=g.MODE_FAST)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    assert sol.advance_to(10.0, max_steps=7) == 7
    t = sol.stats().t_state
    assert 0.0 < t < 10.0
    with pytest.raises(g.GdError):
        sol.advance_to(t)  # not ahead of the state
    with pytest.raises(g.GdError):
        sol.set_dt_policy(5)
    sol.close()


# Fast mode against the oracle at t = 0.5 on Orszag-Tang 128^2 (416 steps): measured 4.9e-8
# (relative L1 per conserved field, the largest).  The differences are rounding grown
# through minmod near-ties; at 1024^2, where the reference's p <= 0 clamp is reached, they
# grow to 2.8e-2 by t = 0.5 (test_gpu_fullsize.py).  The bound leaves a factor of ~10.
OT128_T05_BOUND = 5e-7


def test_orszag_tang_128_to_t05(cuda, oracle_lib):
    """Orszag-Tang at reduced size run to t = 0.5 as the configuration states: parity mode
    equals the oracle bit for bit (state, time, step count); fast mode is within the stated
    L1 bound of it."""
    from gpu_util import max_rel_l1
    cfg, s, u, b = problems.orszag_tang(128, 128)
    so, uo, bo, to, no, _ = oracle_to(oracle_lib, cfg, s, u, b, 0.5)
    for mode in (g.MODE_PARITY, g.MODE_FAST):
        cfg.mode = mode
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        n = sol.advance_to(0.5, use_graph=True)
        st = sol.stats()
        s2, u2, b2 = export(sol, s, u, b)
        sol.close()
        assert abs(st.t_state - 0.5) <= 1e-14 * 0.5
        if mode == g.MODE_PARITY:
            assert n == no and st.t_state == to
            assert np.array_equal(s2, so) and np.array_equal(u2, uo) and np.array_equal(b2, bo)
        else:
            err = max_rel_l1(cfg, (s2, u2, b2), (so, uo, bo))
            print(f"OT 128^2 t = 0.5: fast vs oracle {err:.3e} after {n} steps (oracle {no})")
            assert err <= OT128_T05_BOUND, err
