"""Discrete adjoint of the fast Euler step (HLLC, minmod TVD, periodic): the recording is the
plain run, the replay reproduces it, the gradient is the same for any checkpoint interval and
for repeated sweeps, it satisfies the dot-product identity with the forward-mode tangent
(relative 1e-10, also at exact minmod and wave-speed ties), and it
agrees with FP64 central finite differences (relative difference <= 1e-6) on a smooth
periodic state: the Euler counterpart of tests/test_gpu_adjoint.py.  The
map is only piecewise smooth (minmod choices, wave-speed min / max, star regions): a direction
over the bound at eps = 1e-7 is retaken at 1e-8, keeping the closer quotient, as there."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu


def smooth_euler(N):
    """Periodic unit square, gamma 1.4, HLLC: rho = 1 + 0.3 sin 2pi x sin 2pi y,
    p = 1 + 0.2 cos 2pi (x + y), vx = 0.4 sin 2pi y, vy = 0.3 cos 2pi x."""
    cfg, s, u, _ = problems.kelvin_helmholtz(N, N)
    x = (np.arange(N) + 0.5) / N
    X, Y = np.tile(x, N), np.repeat(x, N)
    s = np.stack([1.0 + 0.3 * np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y),
                  1.0 + 0.2 * np.cos(2 * np.pi * (X + Y))], 1)
    u = np.stack([0.4 * np.sin(2 * np.pi * Y), 0.3 * np.cos(2 * np.pi * X)], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u)


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def setup(N=32, nsteps=12, every=5, pre=5):
    cfg, s, u = smooth_euler(N)
    sol = g.Solver(cfg)
    sol.import_state(s, u, None)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(pre)
    sol.export_state(s, u, None)
    sol.adj_forward(nsteps, every)
    sf, uf = np.zeros_like(s), np.zeros_like(u)
    sol.export_state(sf, uf, None)
    return cfg, sol, (s, u), (sf, uf)


def vjp(sol, gs, gu):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (gs, gu)]
    sol.adj_backward(dev(gs), dev(gu), None, o[0], o[1], None)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in o]


def replay(sol, s, u):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (s, u)]
    sol.adj_replay(dev(s), dev(u), None, o[0], o[1], None)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in o]


def dot(a, b):
    return sum(float((x * y).sum()) for x, y in zip(a, b))


def test_replay_reproduces_the_recorded_run(cuda):
    cfg, sol, U0, Uf = setup()
    for x, y in zip(replay(sol, *U0), Uf):
        assert np.array_equal(x, y)
    sol.close()


def test_recording_is_the_plain_run(cuda):
    cfg, s, u = smooth_euler(40)
    out = []
    for record in (False, True):
        sol = g.Solver(cfg)
        sol.import_state(s, u, None)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        sol.advance(3)
        if record:
            sol.adj_forward(11, 4)
        else:
            sol.advance(11)
        sf, uf = np.zeros_like(s), np.zeros_like(u)
        sol.export_state(sf, uf, None)
        st = sol.stats()
        out.append((sf, uf, st.t, st.dt, st.dt_next, st.steps))
        sol.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2:] == out[1][2:]


def test_gradient_repeatable_and_independent_of_checkpoint_interval(cuda):
    grads = []
    for every in (1, 4, 12):
        cfg, sol, U0, _ = setup(40, 12, every)
        lam = [np.random.default_rng(3).standard_normal(x.shape) for x in U0]
        first = vjp(sol, *lam)
        again = vjp(sol, *lam)
        for a, b in zip(first, again):
            assert np.array_equal(a, b)
        grads.append(first)
        sol.close()
    for gr in grads[1:]:
        for a, b in zip(grads[0], gr):
            assert np.array_equal(a, b)


def test_gradient_matches_central_differences(cuda):
    """Smooth periodic state after 5 steps, 20 steps; L = 1/2 sum (rho_n - rho_target)^2 with
    the target the final density of a run from a seeded 1 % velocity perturbation."""
    N, n = 32, 20
    cfg, sol, U0, Uf = setup(N, n, 10, pre=5)
    s0, u0 = U0
    rng = np.random.default_rng(20261203)
    ut = u0 * (1.0 + 0.01 * rng.uniform(-1.0, 1.0, u0.shape))
    tgt = g.Solver(cfg)
    tgt.import_state(s0, ut, None)
    tgt.set_time(0.0, 0.0)
    tgt.init_dt()
    tgt.advance(n)
    st, ut_ = np.zeros_like(s0), np.zeros_like(u0)
    tgt.export_state(st, ut_, None)
    tgt.close()
    rho_t = st[:, 0]
    gs = np.zeros_like(s0)
    gs[:, 0] = Uf[0][:, 0] - rho_t
    grad = vjp(sol, gs, np.zeros_like(u0))
    for k in range(8):
        d = [rng.standard_normal(x.shape) for x in U0]
        nrm = np.sqrt(sum(float((x * x).sum()) for x in d))
        d = [x / nrm for x in d]
        ad = dot(grad, d)
        best = None
        for eps in (1e-7, 1e-8):
            rp = replay(sol, *[x + eps * y for x, y in zip(U0, d)])[0][:, 0]
            rm = replay(sol, *[x - eps * y for x, y in zip(U0, d)])[0][:, 0]
            fd = float(((rp - rm) * (0.5 * (rp + rm) - rho_t)).sum()) / (2 * eps)
            err = abs(fd - ad) / abs(ad)
            best = err if best is None else min(best, err)
            if best <= 1e-6:
                break
        assert best <= 1e-6, (k, best)
    sol.close()


def jvp(sol, vs, vu):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (vs, vu)]
    sol.tangent(dev(vs), dev(vu), None, o[0], o[1], None)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in o]


def test_tangent_adjoint_dot_product(cuda):
    """<lam, J v> = <J^T lam, v> between the forward-mode tangent (the Euler tile instantiated
    with Dual values) and the reverse sweep, both hand-written: relative 1e-10."""
    cfg, sol, U0, _ = setup(48, 12, 5)
    rng = np.random.default_rng(1)
    lam = [rng.standard_normal(x.shape) for x in U0]
    v = [rng.standard_normal(x.shape) for x in U0]
    a, b = dot(lam, jvp(sol, *v)), dot(vjp(sol, *lam), v)
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (a, b)
    sol.close()


def test_tangent_adjoint_dot_product_at_ties(cuda):
    """The Kelvin-Helmholtz shear layer without its perturbation (v_y = 0): a contact at
    rest, which the HLLC step keeps exactly, so every minmod choice (minmod(0, 0)) and every
    wave-speed min / max (equal left and right states) stays an exact tie; the tangent and
    the adjoint break them the same way, so the identity holds there too.  (Near ties are
    another matter: the tangent computes its values in the Dual instantiation of the tile,
    which may round an intermediate value differently from the forward step's, and a choice
    within that rounding can then go the other way: on the perturbed layer after 4 steps,
    40 of its 16384 input columns, in 3 x 3 patches at the interfaces.)"""
    cfg, s, u, _ = problems.kelvin_helmholtz(64, 64)
    u = u.copy()
    u[:, 1] = 0.0
    sol = g.Solver(cfg)
    sol.import_state(s, u, None)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.adj_forward(4, 2)
    rng = np.random.default_rng(2)
    lam = [rng.standard_normal(x.shape) for x in (s, u)]
    v = [rng.standard_normal(x.shape) for x in (s, u)]
    a, b = dot(lam, jvp(sol, *v)), dot(vjp(sol, *lam), v)
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (a, b)
    sol.close()
