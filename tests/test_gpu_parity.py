"""GPU parity mode (GD_MODE_PARITY) reproduces the reference bit for bit.

Compared against the golden vectors written from the reference's own code and against the
oracle on the benchmark problems at reduced sizes.  All calls go through the C ABI."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
import oracle
from conftest import golden
from golikov_2d_gb300 import problems
from gpu_util import gpu_run, gpu_step_ref, grid_of, oracle_run

pytestmark = pytest.mark.gpu


def native_cfg(gz, order, method, physics=g.MHD):
    N, M = int(gz["N"]), int(gz["M"])
    xmax, ymax = float(gz["xmax"]), float(gz["ymax"])
    if physics == g.EULER:
        return g.Config(N=N, M=M, dx=xmax / N, dy=ymax / M, x0=xmax / (2.0 * N),
                        y0=ymax / (2.0 * M), gamma=1.4, krit=0.4, physics=g.EULER, order=1,
                        method=1, bc=(g.BC_TRANSMISSIVE,) * 4, mode=g.MODE_PARITY)
    top = g.BC_AMBIENT if order == 2 else g.BC_AMBIENT_KEEPB
    return g.Config(N=N, M=M, dx=xmax / N, dy=ymax / M, x0=xmax / (2.0 * N), y0=ymax / (2.0 * M),
                    gamma=5.0 / 3.0, krit=0.25, physics=g.MHD, geometry=g.AXISYM, order=order,
                    method=method, bc=(g.BC_MIRROR_X, g.BC_OUTFLOW, g.BC_AXIS, top),
                    frozen_radius=0.3, mode=g.MODE_PARITY)


@pytest.mark.parametrize("kind,order,method", [("tvd", 2, 3), ("tvd", 2, 2), ("add", 1, 2),
                                               ("add", 1, 3)])
def test_native_mhd_step_matches_reference(cuda, kind, order, method):
    gz = golden("step_native.npz")
    cfg = native_cfg(gz, order, method)
    s2, u2, b2, T = gpu_step_ref(cfg, gz["s"], gz["u"], gz["b"], float(gz["T_do"]))
    assert T == gz[f"{kind}{method}_T"]
    assert np.array_equal(s2, gz[f"{kind}{method}_s"])
    assert np.array_equal(u2, gz[f"{kind}{method}_u"])
    assert np.array_equal(b2, gz[f"{kind}{method}_b"])


def test_native_euler_first_order_matches_reference(cuda):
    gz = golden("step_native.npz")
    cfg = native_cfg(gz, 1, 1, physics=g.EULER)
    s2, u2, _, T = gpu_step_ref(cfg, gz["s"], gz["u"], None, float(gz["T_do"]))
    N, M = cfg.N, cfg.M
    mask = np.zeros((M, N), bool)
    mask[: M - 1, : N - 1] = True
    mask = mask.ravel()
    assert np.array_equal(s2[mask], gz["dek_s"][mask])
    assert np.array_equal(u2[mask], gz["dek_u"][mask])


@pytest.mark.parametrize("use_graph", [False, True])
def test_native_run_matches_reference(cuda, use_graph):
    gz = golden("run_native.npz")
    N, M = int(gz["N"]), int(gz["M"])
    cfg, *_ = problems.stellar_wind(N, M, float(gz["xmax"]), float(gz["ymax"]),
                                    mode=g.MODE_PARITY)
    s, u, b, st = gpu_run(cfg, gz["s0"], gz["u0"], gz["b0"], int(gz["nsteps"]), T_do=1e-8,
                          use_graph=use_graph)
    assert st.dt == gz["T_do"] and st.t == gz["TT"] and st.steps == int(gz["nsteps"])
    assert np.array_equal(s, gz["s"]) and np.array_equal(u, gz["u"]) and np.array_equal(b, gz["b"])


def test_native_euler_first_order_hll_matches_reference(cuda):
    """Ker_Dekard with method 0 (HLL everywhere, kernel.cu:1796-1802), golden from the
    reference; the method passed per call as the reference passes it."""
    gz = golden("faces_hll.npz")
    cfg = native_cfg(gz, 1, 1, physics=g.EULER)
    s2, u2, _, T = gpu_step_ref(cfg, gz["s"], gz["u"], None, float(gz["T_do"]),
                                method=g.METHOD_HLL)
    N, M = cfg.N, cfg.M
    mask = np.zeros((M, N), bool)
    mask[: M - 1, : N - 1] = True
    mask = mask.ravel()
    assert np.array_equal(s2[mask], gz["dek_s"][mask])
    assert np.array_equal(u2[mask], gz["dek_u"][mask])


def hll(case):
    cfg, s, u, b = case
    cfg.method = g.METHOD_HLL
    return cfg, s, u, b


CASES = {
    "sod64_hll": lambda: hll(problems.sod(64, 48, mode=g.MODE_PARITY)),
    "kh64_hll": lambda: hll(problems.kelvin_helmholtz(64, 64, mode=g.MODE_PARITY)),
    "quad50_hll": lambda: hll(problems.four_quadrant(50, np.random.default_rng(5),
                                                     mode=g.MODE_PARITY)),
    "sod_o1_hll": lambda: (lambda c: (setattr(c[0], "order", 1), c)[1])(
        hll(problems.sod(48, 32, mode=g.MODE_PARITY))),
    "sod64": lambda: problems.sod(64, 48, mode=g.MODE_PARITY),
    "kh64": lambda: problems.kelvin_helmholtz(64, 64, mode=g.MODE_PARITY),
    "ot48_hlld": lambda: problems.orszag_tang(48, 48, method=g.METHOD_HLLD, mode=g.MODE_PARITY),
    "ot40_hllcmhd": lambda: problems.orszag_tang(40, 40, method=g.METHOD_HLLC_MHD,
                                                 mode=g.MODE_PARITY),
    "quad50": lambda: problems.four_quadrant(50, np.random.default_rng(5), mode=g.MODE_PARITY),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_parity_matches_oracle(cuda, oracle_lib, case):
    cfg, s, u, b = CASES[case]()
    n = 6
    so, uo, bo, T_do, TT = oracle_run(oracle_lib, cfg, s, u, b, n)
    sg, ug, bg, st = gpu_run(cfg, s, u, b, n)
    assert st.dt == T_do and st.t == TT
    assert np.array_equal(sg, so) and np.array_equal(ug, uo)
    if b is not None:
        assert np.array_equal(bg, bo)


@pytest.mark.parametrize("N,M", [(3, 3), (4, 6), (7, 5)])
@pytest.mark.parametrize("physics", [g.EULER, g.MHD])
def test_parity_tiny_grids(cuda, oracle_lib, N, M, physics):
    """The smallest accepted grids, where every stencil reaches a ghost or wrapped cell:
    parity mode equals the oracle bit for bit over 5 steps, periodic and transmissive."""
    rng = np.random.default_rng(N * 10 + M)
    K = N * M
    for bc in (g.BC_PERIODIC, g.BC_TRANSMISSIVE):
        if physics == g.EULER:
            cfg, *_ = problems.kelvin_helmholtz(N, M, mode=g.MODE_PARITY)
            b = None
        else:
            cfg, *_ = problems.orszag_tang(N, M, mode=g.MODE_PARITY)
            b = rng.uniform(-1.0, 1.0, (K, 3))
        cfg.bc = (bc,) * 4
        s = np.stack([rng.uniform(0.5, 2.0, K), rng.uniform(0.5, 2.0, K)], 1)
        u = rng.uniform(-0.5, 0.5, (K, 2))
        so, uo, bo, T_do, TT = oracle_run(oracle_lib, cfg, s, u, b, 5)
        sg, ug, bg, st = gpu_run(cfg, s, u, b, 5)
        assert st.dt == T_do and st.t == TT, bc
        assert np.array_equal(sg, so) and np.array_equal(ug, uo), bc
        if b is not None:
            assert np.array_equal(bg, bo), bc


@pytest.mark.parametrize("case", ["sod256", "ot128", "kh256"])
def test_run_checksums(cuda, case):
    """Whole runs against the committed checksums (tests/golden/checksums.npz, from the
    oracle): parity mode reproduces the state hash, dt and time after 1, 10 and N steps bit
    for bit; fast mode reproduces every field's sum and L1 norm, and dt and time, to 1e-9
    relative (the bound on N steps of the full protocol)."""
    from golden.make_checksums import case_state, digest, field_sums
    gz = golden("checksums.npz")
    steps = [int(k) for k in gz[f"{case}_steps"]]
    for mode in (g.MODE_PARITY, g.MODE_FAST):
        cfg, s, u, b, n = case_state(case, gz)
        cfg.mode = mode
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        done = 0
        for i, k in enumerate(steps):
            sol.advance(k - done)
            done = k
            s2, u2 = np.zeros_like(s), np.zeros_like(u)
            b2 = None if b is None else np.zeros_like(b)
            sol.export_state(s2, u2, b2)
            st = sol.stats()
            T_do, TT = gz[f"{case}_Tdo"][i], gz[f"{case}_TT"][i]
            if mode == g.MODE_PARITY:
                assert digest(s2, u2, b2) == str(gz[f"{case}_sha"][i]), k
                assert st.dt == T_do and st.t == TT, k
            else:
                sm, l1 = field_sums(s2, u2, b2)
                ref_l1 = gz[f"{case}_l1"][i]
                assert np.all(np.abs(sm - gz[f"{case}_sum"][i]) <= 1e-9 * ref_l1), k
                assert np.all(np.abs(l1 - ref_l1) <= 1e-9 * ref_l1), k
                assert abs(st.dt - T_do) <= 1e-9 * T_do and abs(st.t - TT) <= 1e-9 * TT, k
        sol.close()
