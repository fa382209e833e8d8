"""Discrete adjoint and tangent of the fast MHD step (Orszag-Tang, HLLD, periodic).

The differentiated map is n steps with the recorded dt sequence held fixed.  The
Orszag-Tang initial condition itself is not a point where the map is differentiable: rho
and p are uniform and vx, Bx (vy, By) are constant along x (y), so those minmod slopes are
minmod(0, 0), a kink.  The differentiated window therefore starts from the Orszag-Tang
state after `pre` steps, where the fields vary smoothly.  Checks:
  * dot-product identity <lam, J v> = <J^T lam, v> between the forward-mode tangent kernel
    and the reverse sweep (both hand-written), relative difference <= 1e-10;
  * the gradient of L = 1/2 sum (rho_n - rho_target)^2 against FP64 central finite
    differences of the same map on random directions, relative difference <= 1e-6.  The
    TVD map is only piecewise smooth: where a minmod choice switches inside +-eps the
    central difference straddles a kink and is not the derivative the adjoint computes
    (measured: errors ~1e-3 at eps >= 1e-6, ~1e-8 at 1e-7, rounding-dominated below 1e-8).
    The check runs where the quotient resolves (32x32, smooth window) at eps = 1e-7, and a
    direction over the bound is retaken at eps/10, keeping the closer quotient -- the
    switch leaves the stencil as eps shrinks, a wrong derivative would not;
  * the gradient does not depend on the checkpoint interval (bit-identical).
"""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def setup(N=64, nsteps=12, every=5, pre=20):
    cfg, s, u, b = problems.orszag_tang(N, N)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(pre)
    sol.export_state(s, u, b)
    sol.adj_forward(nsteps, every)
    sf, uf, bf = np.zeros_like(s), np.zeros_like(u), np.zeros_like(b)
    sol.export_state(sf, uf, bf)
    return cfg, sol, (s, u, b), (sf, uf, bf)


def vjp(sol, gs, gu, gb):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (gs, gu, gb)]
    sol.adj_backward(dev(gs), dev(gu), dev(gb), *o)
    torch.cuda.synchronize()
    return [host(x) for x in o]


def jvp(sol, vs, vu, vb):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (vs, vu, vb)]
    sol.tangent(dev(vs), dev(vu), dev(vb), *o)
    torch.cuda.synchronize()
    return [host(x) for x in o]


def replay(sol, s, u, b):
    import torch
    o = [torch.zeros_like(dev(x)) for x in (s, u, b)]
    sol.adj_replay(dev(s), dev(u), dev(b), *o)
    torch.cuda.synchronize()
    return [host(x) for x in o]


def dot(a, b):
    return sum(float((x * y).sum()) for x, y in zip(a, b))


def test_replay_reproduces_the_recorded_run(cuda):
    cfg, sol, U0, Uf = setup()
    R = replay(sol, *U0)
    for x, y in zip(R, Uf):
        assert np.array_equal(x, y)
    sol.close()


def test_recording_is_the_plain_run(cuda):
    """The recorded forward run (last segment stepped with its update terms stored) leaves
    the same state, time and next dt as plain steps."""
    cfg, s, u, b = problems.orszag_tang(40, 40)
    out = []
    for record in (False, True):
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        sol.advance(5)
        if record:
            sol.adj_forward(13, 4)
        else:
            sol.advance(13)
        sf, uf, bf = np.zeros_like(s), np.zeros_like(u), np.zeros_like(b)
        sol.export_state(sf, uf, bf)
        st = sol.stats()
        out.append((sf, uf, bf, st.t, st.dt, st.dt_next, st.steps))
        sol.close()
    for x, y in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(x, y)
    assert out[0][3:] == out[1][3:]


def test_backward_repeatable(cuda):
    """The first sweep reverses the recorded last segment directly, later ones recompute it
    (also after a tangent sweep has used the segment buffers): identical gradients."""
    cfg, sol, U0, _ = setup(40, 11, 4)
    lam = [np.random.default_rng(5).standard_normal(x.shape) for x in U0]
    g1 = vjp(sol, *lam)
    g2 = vjp(sol, *lam)
    jvp(sol, *lam)
    g3 = vjp(sol, *lam)
    for a, b_, c in zip(g1, g2, g3):
        assert np.array_equal(a, b_) and np.array_equal(a, c)
    sol.close()


def test_tangent_adjoint_dot_product(cuda):
    cfg, sol, U0, _ = setup()
    rng = np.random.default_rng(1)
    lam = [rng.standard_normal(x.shape) for x in U0]
    v = [rng.standard_normal(x.shape) for x in U0]
    Jv = jvp(sol, *v)
    JTl = vjp(sol, *lam)
    a, b = dot(lam, Jv), dot(JTl, v)
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (a, b)
    sol.close()


def test_tangent_adjoint_dot_product_at_ties(cuda):
    """At the Orszag-Tang initial state many minmod and wave-speed choices are exact ties
    (uniform rho and p; vx, Bx constant along x; symmetric extrema of By and Bx).  The
    tangent and the adjoint must break them the same way, so the identity holds there too."""
    cfg, sol, U0, _ = setup(64, 3, 2, pre=0)
    rng = np.random.default_rng(2)
    lam = [rng.standard_normal(x.shape) for x in U0]
    v = [rng.standard_normal(x.shape) for x in U0]
    a, b = dot(lam, jvp(sol, *v)), dot(vjp(sol, *lam), v)
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (a, b)
    sol.close()


def test_gradient_matches_central_differences(cuda):
    """Orszag-Tang 32x32 from the state after 40 steps (smooth), 30 steps; the target is the
    final density of a run (its own dt) from a seeded 1 % perturbation of the velocity.  The
    quotient is formed per cell: (L+ - L-) = sum (r+ - r-) ((r+ + r-) / 2 - t)."""
    N, n = 32, 30
    cfg, sol, U0, Uf = setup(N, n, 10, pre=40)
    s0, u0, b0 = U0
    rng = np.random.default_rng(20261203)
    ut = u0 * (1.0 + 0.01 * rng.uniform(-1.0, 1.0, u0.shape))
    tgt = g.Solver(cfg)
    tgt.import_state(s0, ut, b0)
    tgt.set_time(0.0, 0.0)
    tgt.init_dt()
    tgt.advance(n)
    st, ut_, bt = np.zeros_like(s0), np.zeros_like(u0), np.zeros_like(b0)
    tgt.export_state(st, ut_, bt)
    tgt.close()
    rho_t = st[:, 0]

    gs = np.zeros_like(s0)
    gs[:, 0] = Uf[0][:, 0] - rho_t
    grad = vjp(sol, gs, np.zeros_like(u0), np.zeros_like(b0))
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


def test_gradient_independent_of_checkpoint_interval(cuda):
    rng = np.random.default_rng(3)
    grads = []
    for every in (1, 4, 12):
        cfg, sol, U0, _ = setup(40, 12, every)
        lam = [np.random.default_rng(3).standard_normal(x.shape) for x in U0]
        grads.append(vjp(sol, *lam))
        sol.close()
    for gr in grads[1:]:
        for x, y in zip(gr, grads[0]):
            assert np.array_equal(x, y)


def test_unsupported_configurations(cuda):
    cfg, s, u, b = problems.sod(32, 32)
    sol = g.Solver(cfg)
    with pytest.raises(g.GdError) as e:
        sol.adj_forward(3, 1)
    assert e.value.status == 5
    sol.close()


@pytest.mark.parametrize("physics", ["mhd", "euler"])
def test_current_dt_policy_is_rejected(cuda, physics):
    """Under GD_DT_CURRENT each step's dt comes from a pass over its own input, which the
    recording and the recomputed segments do not run: gd_adj_forward refuses it, and
    accepts the same context again once the policy is back to the lagged one."""
    if physics == "mhd":
        cfg, s, u, b = problems.orszag_tang(32, 32)
    else:
        cfg, s, u, b = problems.kelvin_helmholtz(32, 32)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.set_dt_policy(g.DT_CURRENT)
    with pytest.raises(g.GdError) as e:
        sol.adj_forward(3, 1)
    assert e.value.status == 5
    sol.set_dt_policy(g.DT_LAGGED)
    sol.adj_forward(3, 1)
    sol.close()
