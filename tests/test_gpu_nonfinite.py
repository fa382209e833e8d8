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
