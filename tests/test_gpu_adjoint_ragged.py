"""Both discrete adjoints (MHD HLLD, Euler HLLC) and their tangents on ragged and tiny periodic
grids: sides that are not multiples of the tiles (the forward's 16 x 16 and 32 x 8 tiles, the
reverse passes' 32 x 4 blocks), down to the smallest grid the context accepts (3 x 3), where
the stencil's periodic wrap reaches across the whole grid.  On each: the replay reproduces the
recorded run bit for bit, and the dot-product identity <lam, J v> = <J^T lam, v> between the
forward-mode tangent and the reverse sweep holds to 1e-10 relative."""
import math

import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu

SIZES = [(37, 23), (33, 17), (5, 3), (3, 3)]


def dev(a):
    import torch
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return None if t is None else t.cpu().numpy()


def smooth_state(physics, N, M):
    """A smooth periodic state on the unit square (N x M cells)."""
    if physics == "mhd":
        cfg, s, u, b = problems.orszag_tang(N, M)
    else:
        cfg, s, u, b = problems.kelvin_helmholtz(N, M)
    x, y = (np.arange(N) + 0.5) / N, (np.arange(M) + 0.5) / M
    X, Y = np.tile(x, M), np.repeat(y, N)
    tp = 2 * math.pi
    s = np.stack([1.0 + 0.3 * np.sin(tp * X) * np.sin(tp * Y), 1.0 + 0.2 * np.cos(tp * (X + Y))], 1)
    u = np.stack([0.4 * np.sin(tp * Y), 0.3 * np.cos(tp * X)], 1)
    if b is not None:
        b = np.stack([0.5 * np.sin(tp * Y), 0.4 * np.cos(tp * X), 0.2 * np.sin(tp * (X - Y))], 1)
    return cfg, s, u, b


def record(physics, N, M, nsteps=6, every=4, pre=2):
    cfg, s, u, b = smooth_state(physics, N, M)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(pre)
    U0 = [np.zeros_like(s), np.zeros_like(u), None if b is None else np.zeros_like(b)]
    sol.export_state(*U0)
    sol.adj_forward(nsteps, every)
    Uf = [np.zeros_like(s), np.zeros_like(u), None if b is None else np.zeros_like(b)]
    sol.export_state(*Uf)
    return sol, U0, Uf


def call(fn, xs):
    import torch
    o = [None if x is None else torch.zeros_like(dev(x)) for x in xs]
    fn(*[dev(x) for x in xs], *o)
    torch.cuda.synchronize()
    return [host(x) for x in o]


def dot(a, b):
    return sum(float((x * y).sum()) for x, y in zip(a, b) if x is not None)


@pytest.mark.parametrize("physics", ["mhd", "euler"])
@pytest.mark.parametrize("N,M", SIZES)
def test_replay_is_the_recorded_run(cuda, physics, N, M):
    sol, U0, Uf = record(physics, N, M)
    for x, y in zip(call(sol.adj_replay, U0), Uf):
        if y is not None:
            assert np.array_equal(x, y), (physics, N, M)
    sol.close()


@pytest.mark.parametrize("physics", ["mhd", "euler"])
@pytest.mark.parametrize("N,M", SIZES)
def test_tangent_adjoint_dot_product(cuda, physics, N, M):
    sol, U0, _ = record(physics, N, M)
    rng = np.random.default_rng(N * 100 + M)
    lam = [None if x is None else rng.standard_normal(x.shape) for x in U0]
    v = [None if x is None else rng.standard_normal(x.shape) for x in U0]
    a, b = dot(lam, call(sol.tangent, v)), dot(call(sol.adj_backward, lam), v)
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (physics, N, M, a, b)
    sol.close()
