"""The benchmark configurations at their full sizes, through properties that do not need an
oracle run of that size: conservation on periodic grids, the exact zero of Bz in the 2-D
Orszag-Tang problem, running to the configured end time, fast against parity for the first
step (1e-12) and after 100 steps (the stated bound), and Sod 256^2 in parity mode bit for bit
against the oracle over its 200 steps."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems
from gpu_util import conserved, gpu_run, gpu_step_ref, max_rel_l1, oracle_run

pytestmark = pytest.mark.gpu

# Fast against parity on Orszag-Tang 1024^2 after 100 steps: measured 8.4e-7.  Rounding
# differences grow through minmod choices at near-ties and the reference's p <= 0 -> 1e-6
# clamp (Kernel_TVD kernel.cu:2656), which this problem reaches at this resolution.
OT1024_100_STEPS_BOUND = 2e-6


def sums(cfg, s, u, b):
    return [x.sum() for x in conserved(cfg, s, u, b)]


def test_kh4096_100_steps_conserve_mass_momentum_energy(cuda):
    """Config 3: KH 4096^2 periodic, 100 steps.  Face-once fluxes telescope."""
    cfg, s, u, b = problems.kelvin_helmholtz(4096, 4096)
    sg, ug, _, st = gpu_run(cfg, s, u, None, 100, use_graph=True)
    assert st.steps == 100 and st.nonfinite == 0
    c0, c1 = sums(cfg, s, u, None), sums(cfg, sg, ug, None)
    assert abs(c1[0] - c0[0]) <= 1e-13 * abs(c0[0])                        # mass
    assert abs(c1[3] - c0[3]) <= 1e-13 * abs(c0[3])                        # energy
    assert abs(c1[1] - c0[1]) <= 1e-13 * np.abs(s[:, 0] * u[:, 0]).sum()  # x momentum
    assert abs(c1[2] - c0[2]) <= 1e-11 * np.abs(s[:, 0] * u[:, 1]).sum()  # y momentum


def test_kh4096_first_step_fast_matches_parity(cuda):
    cfg, s, u, b = problems.kelvin_helmholtz(4096, 4096)
    fast = gpu_step_ref(cfg, s, u, None, 1e-4)
    cfg.mode = g.MODE_PARITY
    par = gpu_step_ref(cfg, s, u, None, 1e-4)
    assert max_rel_l1(cfg, fast[:3], par[:3]) <= 1e-12
    assert abs(fast[3] - par[3]) <= 1e-12 * par[3]


def test_ot1024_to_t05(cuda):
    """Config 2 as specified: Orszag-Tang 1024^2, HLLD, CFL 0.4, to t = 0.5."""
    cfg, s, u, b = problems.orszag_tang(1024, 1024)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    n = sol.advance_to(0.5, use_graph=True)
    st = sol.stats()
    s2, u2, b2 = np.zeros_like(s), np.zeros_like(u), np.zeros_like(b)
    sol.export_state(s2, u2, b2)
    sol.close()
    assert abs(st.t_state - 0.5) <= 1e-14 * 0.5 and st.steps == n and n > 1000
    assert st.nonfinite == 0
    c0, c1 = sums(cfg, s, u, b), sums(cfg, s2, u2, b2)
    assert abs(c1[0] - c0[0]) <= 1e-13 * abs(c0[0])  # mass
    # 2-D with v_z = B_z = 0: every B_z flux and star state is an exact zero
    assert not b2[:, 2].any()


def test_ot1024_fast_vs_parity(cuda):
    cfg, s, u, b = problems.orszag_tang(1024, 1024)
    fast1 = gpu_step_ref(cfg, s, u, b, 1e-4)
    cfg_p, *_ = problems.orszag_tang(1024, 1024, mode=g.MODE_PARITY)
    par1 = gpu_step_ref(cfg_p, s, u, b, 1e-4)
    assert max_rel_l1(cfg, fast1[:3], par1[:3]) <= 1e-12
    fast = gpu_run(cfg, s, u, b, 100, use_graph=True)
    par = gpu_run(cfg_p, s, u, b, 100, use_graph=True)
    assert max_rel_l1(cfg, fast[:3], par[:3]) <= OT1024_100_STEPS_BOUND
    # the CFL dt is a minimum over all faces: it follows the state's difference
    assert abs(fast[3].t - par[3].t) <= OT1024_100_STEPS_BOUND * par[3].t


def test_sod256_parity_200_steps_bit_exact(cuda, oracle_lib):
    """Config 1 at full size: parity mode = the oracle (= the reference) over 200 steps."""
    cfg, s, u, b = problems.sod(256, 256, mode=g.MODE_PARITY)
    so, uo, _, T_do, TT = oracle_run(oracle_lib, cfg, s, u, None, 200)
    sg, ug, _, st = gpu_run(cfg, s, u, None, 200)
    assert np.array_equal(sg, so) and np.array_equal(ug, uo)
    assert st.dt == T_do and st.t == TT
