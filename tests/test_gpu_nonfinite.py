"""A non-finite value in the state is reported, not hidden: after a step from a state with
one NaN pressure, gd_stats.nonfinite counts the affected cells and gd_get_stats returns
GD_ERR_NONPHYSICAL, for every kernel family and mode."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu

CASES = {
    "euler_fast": lambda: problems.sod(64, 48),
    "euler_parity": lambda: problems.sod(64, 48, mode=g.MODE_PARITY),
    "mhd_fast": lambda: problems.orszag_tang(64, 64),
    "mhd_parity": lambda: problems.orszag_tang(64, 64, mode=g.MODE_PARITY),
    "hancock_fast": lambda: problems.hancock_wind(96, 64),
    "hancock_parity": lambda: problems.hancock_wind(96, 64, mode=g.MODE_PARITY),
}


def test_floor_limit(cuda):
    """Two streams moving apart at Mach ~1e6 open a vacuum: the pressure floor
    (p <= 0 -> 1e-6) is hit; a limit below the hits turns gd_get_stats into
    GD_ERR_NONPHYSICAL, no limit (0) does not."""
    cfg, s, u, b = problems.sod(64, 16)
    s = s.copy()
    u = u.copy()
    s[:, 0], s[:, 1] = 1.0, 1e-12
    x = np.tile(np.arange(cfg.N), cfg.M)
    u[:, 0] = np.where(x < cfg.N // 2, -1.0, 1.0)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(1e-3, 0.0)
    sol.advance(2)
    st = sol.stats()  # no limit: floors are counted, not an error
    hits = st.rho_floor_hits + st.p_floor_hits
    assert hits > 0 and st.nonfinite == 0
    sol.set_floor_limit(hits)
    sol.stats()  # at the limit
    sol.set_floor_limit(hits - 1 if hits > 1 else 1)
    if hits > 1:
        with pytest.raises(g.GdError) as e:
            sol.stats()
        assert e.value.status == 3
    with pytest.raises(g.GdError):
        sol.set_floor_limit(-1)
    sol.close()


@pytest.mark.parametrize("case", sorted(CASES))
def test_nan_in_the_state_is_reported(cuda, case):
    cfg, s, u, b = CASES[case]()
    s = s.copy()
    n, m = cfg.N - 20, cfg.M // 2  # an updated cell, away from every edge and frozen sphere
    s[m * cfg.N + n, 1] = np.nan
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(1e-4, 0.0)
    sol.advance(1)
    st = sol.stats(allow_nonfinite=True)
    assert st.nonfinite >= 1
    with pytest.raises(g.GdError) as e:
        sol.stats()
    assert e.value.status == 3  # GD_ERR_NONPHYSICAL
    sol.close()


BAD_INPUT = {
    "euler": lambda mode: problems.sod(48, 32, mode=mode),
    "mhd": lambda mode: problems.orszag_tang(48, 32, mode=mode),
}


@pytest.mark.parametrize("case", sorted(BAD_INPUT))
def test_zero_pressure_and_negative_density_inputs(cuda, oracle_lib, case):
    """Faults injected from the host: a cell with p = 0 (for MHD also with B = 0: zero fast
    speed) is a legal state (zero sound speed, the face fallback keeps the cell value) and the
    step stays finite, parity mode equal to the oracle bit for bit and fast mode within its
    1e-12 bound; a cell with rho < 0 has no real sound speed and the step does
    not hide it: its NaNs are counted (gd_get_stats -> GD_ERR_NONPHYSICAL) or, where the
    reference's min / max comparisons drop the NaN speeds (Euler HLLC, kernel.cu:853-1165),
    its density floor is hit; parity mode reproduces the oracle's NaN pattern and every
    finite value."""
    from gpu_util import grid_of, gpu_step_ref, max_rel_l1
    bads = ("p0", "p0_b0", "rho_neg") if case == "mhd" else ("p0", "rho_neg")
    for bad in bads:
        for mode in (g.MODE_PARITY, g.MODE_FAST):
            cfg, s, u, b = BAD_INPUT[case](mode)
            s = s.copy()
            k = (cfg.M // 2) * cfg.N + cfg.N // 3
            if bad == "rho_neg":
                s[k, 0] = -0.5
            else:
                s[k, 1] = 0.0
            if bad == "p0_b0":  # zero fast magnetosonic speed in that cell
                b = b.copy()
                b[k, :] = 0.0
            sol = g.Solver(cfg)
            sol.import_state(s, u, b)
            sol.set_time(1e-4, 0.0)
            sol.advance(1)
            st = sol.stats(allow_nonfinite=True)
            if bad != "rho_neg":
                assert st.nonfinite == 0, (bad, mode)
            elif st.nonfinite >= 1:
                with pytest.raises(g.GdError) as e:
                    sol.stats()
                assert e.value.status == 3
            else:
                assert st.rho_floor_hits >= 1, (bad, mode)
            sol.close()
            so, uo, bo, To = oracle_lib.step(grid_of(cfg), s, u, b, 1e-4)
            sg, ug, bg, Tg = gpu_step_ref(cfg, s, u, b, 1e-4)
            if mode != g.MODE_PARITY:
                if bad != "rho_neg":  # a legal state: the fast step's usual bound
                    assert max_rel_l1(cfg, (sg, ug, bg), (so, uo, bo)) <= 1e-12, bad
                    assert abs(Tg - To) <= 1e-12 * To, bad
                continue
            pairs = [(sg, so), (ug, uo)] + ([] if b is None else [(bg, bo)])
            for x, y in pairs:
                assert np.array_equal(np.isnan(x), np.isnan(y)), bad
                assert np.array_equal(x[~np.isnan(x)], y[~np.isnan(y)]), bad
            assert Tg == To or (np.isnan(Tg) and np.isnan(To)), bad
