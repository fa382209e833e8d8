"""Fresh randomized comparisons of the oracle against the reference's own compiled code.

Needs oracle/_ref/libgdref.so (built from the reference sources; skipped where they are
absent).  Complements the fixed golden vectors with new seeds on every grid shape below."""
import numpy as np
import pytest

import oracle


def rand_state(rng, K, bscale=2.0):
    s = np.stack([rng.uniform(0.2, 2.0, K), rng.uniform(0.05, 2.0, K)], 1)
    u = rng.uniform(-1.5, 1.5, (K, 2))
    b = rng.uniform(-bscale, bscale, (K, 3))
    return s, u, b


@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("N,M", [(33, 17), (64, 8)])
@pytest.mark.parametrize("method", [2, 3])
def test_kernel_tvd_random(oracle_lib, reference, seed, N, M, method):
    rng = np.random.default_rng(seed)
    xmax, ymax = 3.0, 1.7
    reference.set_params(5.0 / 3.0, 0.25, N, M, xmax, ymax)
    s, u, b = rand_state(rng, N * M)
    s2r, u2r, b2r, Tr = reference.kernel_tvd(s, u, b, 1.5e-3, 0, method)
    g = oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), 5.0 / 3.0, 0.25,
                    physics=oracle.MHD, geometry=oracle.AXISYM, order=2, method=method,
                    bc=(oracle.BC_MIRROR_X, oracle.BC_OUTFLOW, oracle.BC_AXIS, oracle.BC_AMBIENT),
                    frozen_radius=0.3)
    s2, u2, b2, T = oracle_lib.step(g, s, u, b, 1.5e-3)
    assert T == Tr
    assert np.array_equal(s2, s2r) and np.array_equal(u2, u2r) and np.array_equal(b2, b2r)


@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_hllc_random_faces(oracle_lib, reference, gamma):
    rng = np.random.default_rng(21)
    reference.set_params(gamma, 0.4, 64, 64, 1.0, 1.0)
    for _ in range(3000):
        L = np.array([rng.uniform(0.01, 5), rng.uniform(0.01, 5), rng.uniform(-4, 4), rng.uniform(-4, 4)])
        R = np.array([rng.uniform(0.01, 5), rng.uniform(0.01, 5), rng.uniform(-4, 4), rng.uniform(-4, 4)])
        n1, n2 = [(1, 0), (0, -1), (-1, 0), (0, 1)][rng.integers(0, 4)]
        t1, F1 = oracle_lib.hllc(L, R, n1, n2, 0.003, gamma, 0.4)
        t2, F2 = reference.hllc(L, R, n1, n2, 0.003)
        assert t1 == t2 and np.array_equal(F1, F2)


def test_hlld_random_faces(oracle_lib, reference):
    rng = np.random.default_rng(22)
    reference.set_params(5.0 / 3.0, 0.4, 64, 64, 1.0, 1.0)
    for it in range(3000):
        def side():
            return np.array([rng.uniform(0.01, 5), rng.uniform(0.01, 5), rng.uniform(-4, 4),
                             rng.uniform(-4, 4), 0.0, rng.uniform(-5, 5), rng.uniform(-5, 5),
                             rng.uniform(-5, 5)])
        L, R = side(), side()
        n1, n2 = [(1, 0), (0, -1), (-1, 0), (0, 1)][rng.integers(0, 4)]
        meth = 2 + (it & 1)
        t1, F1 = oracle_lib.hlld(L, R, n1, n2, 0.0, 0.003, meth, 5.0 / 3.0, 0.4)
        t2, F2 = reference.hlld(L, R, n1, n2, 0.0, 0.003, meth)
        assert t1 == t2 and np.array_equal(F1, F2, equal_nan=True)


@pytest.mark.parametrize("seed,N,M", [(31, 40, 23), (32, 7, 5), (33, 16, 16)])
def test_state_file_writers_random(oracle_lib, reference, tmp_path, seed, N, M):
    """Writers on fresh states and grid shapes (the reference's Tecplot writers take
    Nmin = 3 from its header)."""
    from golden.make_golden import io_state
    rng = np.random.default_rng(seed)
    s, u, b = io_state(rng, N * M)
    xmax, ymax, gamma = 9.0, 5.0, 1.4
    reference.set_params(gamma, 0.25, N, M, xmax, ymax)
    grid = oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), gamma, 0.25)
    pr, po = str(tmp_path / "r"), str(tmp_path / "o")
    reference.write_restart(s, u, b, pr)
    oracle_lib.write_restart(grid, s, u, b, po)
    assert open(pr, "rb").read() == open(po, "rb").read()
    for wb, bb, t in ((0, None, None), (1, b, None), (2, b, 2.5e-3)):
        reference.print_tecplot(s, u, bb, wb, 0.0 if t is None else t, pr)
        oracle_lib.write_tecplot(grid, s, u, bb, 3, xmax / (2.0 * N), xmax, ymax / (2.0 * M),
                                 ymax, po, t)
        assert open(pr, "rb").read() == open(po, "rb").read(), wb


@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_hll_random_faces(oracle_lib, reference, gamma):
    rng = np.random.default_rng(44)
    reference.set_params(gamma, 0.4, 64, 64, 1.0, 1.0)
    for _ in range(400):
        L = np.array([rng.uniform(-0.1, 3), rng.uniform(0.01, 3), rng.uniform(-8, 8),
                      rng.uniform(-8, 8)])
        R = np.array([rng.uniform(-0.1, 3), rng.uniform(0.01, 3), rng.uniform(-8, 8),
                      rng.uniform(-8, 8)])
        n1, n2 = [(1.0, 0.0), (0.0, -1.0), (-1.0, 0.0), (0.0, 1.0)][rng.integers(0, 4)]
        t0, F0 = reference.hll(L, R, n1, n2, 0.01)
        t1, F1 = oracle_lib.hll(L, R, n1, n2, 0.01, gamma, 0.4)
        assert t0 == t1 and np.array_equal(F0, F1, equal_nan=True)


@pytest.mark.parametrize("seed,N,M,xmax,ymax", [(41, 40, 24, 9.0, 5.0), (42, 19, 11, 9.0, 5.0),
                                                (43, 5, 4, 9.0, 5.0), (44, 30, 18, 25.0, 14.0)])
def test_kernel_gkr_random(oracle_lib, reference, seed, N, M, xmax, ymax):
    """Kernel_GKR (kernel.cu:2663-3284) against the oracle's MUSCL-Hancock restatement."""
    rng = np.random.default_rng(seed)
    reference.set_params(5.0 / 3.0, 0.25, N, M, xmax, ymax)
    s, u, b = rand_state(rng, N * M)
    s2r, u2r, b2r, Tr = reference.kernel_gkr(s, u, b, 1.5e-3, 0, 3)
    g = oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), 5.0 / 3.0, 0.25,
                    physics=oracle.MHD, geometry=oracle.AXISYM, order=2, method=3,
                    bc=(oracle.BC_MIRROR_X, oracle.BC_OUTFLOW, oracle.BC_AXIS,
                        oracle.BC_AMBIENT_KEEPB),
                    frozen_radius=2.0, scheme=1, x_max=xmax, y_max=ymax)
    s2, u2, b2, T = oracle_lib.step(g, s, u, b, 1.5e-3)
    assert T == Tr
    assert np.array_equal(s2, s2r) and np.array_equal(u2, u2r) and np.array_equal(b2, b2r)

