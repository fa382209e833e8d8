"""gd_adj_switches: two replays of the recorded map side by side and the count of the
non-smooth choices (minmod picks, rho / p fallbacks, HLLD wave-speed picks, region and
guards, update floors) on which they differ.

Checks: both outputs are the recorded map's (gd_adj_replay) bit for bit; two equal inputs
differ nowhere; a planted exact tie (a density ramp whose minmod differences are equal,
one cell moved by +-delta) switches exactly the three slopes that see that cell."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def recorded(cfg, s, u, b, nsteps, every, pre=0):
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    if pre:
        sol.advance(pre)
    s0, u0, b0 = np.zeros_like(s), np.zeros_like(u), np.zeros_like(b)
    sol.export_state(s0, u0, b0)
    sol.adj_forward(nsteps, every)
    return sol, (s0, u0, b0)


def switches(sol, Up, Um):
    import torch
    Up = [dev(x) for x in Up]
    Um = [dev(x) for x in Um]
    Op = [torch.zeros_like(x) for x in Up]
    Om = [torch.zeros_like(x) for x in Um]
    c = sol.adj_switches(Up, Um, Op, Om)
    torch.cuda.synchronize()
    return c, [x.cpu().numpy() for x in Op], [x.cpu().numpy() for x in Om]


def replay(sol, U):
    import torch
    U = [dev(x) for x in U]
    O = [torch.zeros_like(x) for x in U]
    sol.adj_replay(*U, *O)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in O]


def test_outputs_are_the_recorded_map_and_equal_runs_never_switch(cuda):
    cfg, s, u, b = problems.orszag_tang(32, 32)
    sol, U0 = recorded(cfg, s, u, b, 7, 3, pre=20)
    rng = np.random.default_rng(5)
    V = [rng.standard_normal(x.shape) for x in U0]
    eps = 1e-7
    Up = [x + eps * v for x, v in zip(U0, V)]
    Um = [x - eps * v for x, v in zip(U0, V)]
    c, Op, Om = switches(sol, Up, Um)
    for a, r in zip(Op, replay(sol, Up)):
        assert np.array_equal(a, r)
    for a, r in zip(Om, replay(sol, Um)):
        assert np.array_equal(a, r)
    assert c["cells"] <= c["cell_steps"] <= 7 * 32 * 32
    c0, O1, O2 = switches(sol, U0, U0)
    assert all(v == 0 for v in c0.values()), c0
    for a, r in zip(O1, O2):
        assert np.array_equal(a, r)
    sol.close()


def test_planted_minmod_tie_switches_three_slopes(cuda):
    cfg, s, u, b = problems.orszag_tang(16, 16)
    N = cfg.N
    n = np.arange(cfg.N * cfg.M) % N
    s = np.stack([1.0 + n * 2.0 ** -7, np.ones(N * cfg.M)], 1)  # equal differences along x
    u = np.zeros_like(u)
    b = np.zeros_like(b)
    sol, U0 = recorded(cfg, s, u, b, 1, 1)
    k = 5 * N + 7                                                # an interior cell
    Up, Um = [x.copy() for x in U0], [x.copy() for x in U0]
    Up[0][k, 0] += 2.0 ** -20
    Um[0][k, 0] -= 2.0 ** -20
    c, _, _ = switches(sol, Up, Um)
    # the x slopes of cells 6, 7 and 8 of that row break the tie the opposite way
    assert c["minmod"] == 3, c
    assert c["fallback"] == 0 and c["floors"] == 0 and c["guards"] == 0, c
    assert c["cells"] >= 4 and c["cells"] == c["cell_steps"], c
    sol.close()


def test_euler_contexts_are_not_supported(cuda):
    import torch
    cfg, s, u, _ = problems.kelvin_helmholtz(16, 16)
    sol = g.Solver(cfg)
    sol.import_state(s, u, None)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.adj_forward(2, 1)
    z = [torch.zeros(16 * 16, 2, dtype=torch.float64, device="cuda") for _ in range(2)]
    zb = torch.zeros(16 * 16, 3, dtype=torch.float64, device="cuda")
    with pytest.raises(g.GdError) as e:
        sol.adj_switches((z[0], z[1], zb), (z[0], z[1], zb), (z[0], z[1], zb),
                         (z[0], z[1], zb))
    assert e.value.status == 5
    sol.close()
