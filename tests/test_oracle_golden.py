"""The oracle (oracle/gd_oracle.c) reproduces the reference's own outputs bit for bit.

The golden vectors were written by tests/golden/make_golden.py from the reference's
Gas_Dinamic.cu / kernel.cu compiled for the host; see that script for what each holds.
Comparisons use == on float64 (a zero may differ in sign only)."""
import numpy as np
import pytest

import oracle
from conftest import golden


def test_minmod_linear_linear2(oracle_lib):
    g = golden("recon.npz")
    L = oracle_lib.lib
    mm = np.array([L.gdo_minmod(a, b) for a, b in g["mm_in"]])
    assert np.array_equal(mm, g["mm"])
    x, h, t = g["x"], g["h"], g["t"]
    lin = np.array([L.gdo_linear(x[i], t[i, 0], x[i] + h[i], t[i, 1], x[i] + 2.0 * h[i], t[i, 2],
                                 x[i] + h[i] / 2.0) for i in range(len(x))])
    assert np.array_equal(lin, g["lin"])
    import ctypes
    for i in range(len(x)):
        a, b = ctypes.c_double(), ctypes.c_double()
        L.gdo_linear2(x[i] - h[i], t[i, 0], x[i], t[i, 1], x[i] + h[i], t[i, 2],
                      x[i] - h[i] / 2.0, x[i] + h[i] / 2.0, ctypes.byref(a), ctypes.byref(b))
        assert a.value == g["A"][i] and b.value == g["B"][i]


def test_hllc_faces(oracle_lib):
    g = golden("faces_hllc.npz")
    for i in range(len(g["t"])):
        t, F = oracle_lib.hllc(g["L"][i], g["R"][i], g["normal"][i, 0], g["normal"][i, 1],
                               float(g["rad"]), float(g["gamma"][i]), float(g["krit"]))
        assert t == g["t"][i]
        assert np.array_equal(F, g["flux"][i]), (i, F, g["flux"][i])


def test_hlld_faces(oracle_lib):
    g = golden("faces_hlld.npz")
    for i in range(len(g["t"])):
        t, F = oracle_lib.hlld(g["L"][i], g["R"][i], g["normal"][i, 0], g["normal"][i, 1], 0.0,
                               float(g["rad"]), int(g["method"][i]), float(g["gamma"]),
                               float(g["krit"]))
        assert t == g["t"][i]
        assert np.array_equal(F, g["flux"][i], equal_nan=True), (i, F, g["flux"][i])


def native_grid(g, order, method, physics=oracle.MHD, gamma=5.0 / 3.0, krit=0.25):
    N, M = int(g["N"]), int(g["M"])
    xmax, ymax = float(g["xmax"]), float(g["ymax"])
    if physics == oracle.EULER:
        return oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), 1.4, 0.4,
                           physics=oracle.EULER, order=1, method=1,
                           bc=(oracle.BC_TRANSMISSIVE,) * 4)
    top = oracle.BC_AMBIENT if order == 2 else oracle.BC_AMBIENT_KEEPB
    return oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), gamma, krit,
                       physics=physics, geometry=oracle.AXISYM, order=order, method=method,
                       bc=(oracle.BC_MIRROR_X, oracle.BC_OUTFLOW, oracle.BC_AXIS, top),
                       frozen_radius=0.3)


@pytest.mark.parametrize("kind,order,method", [("tvd", 2, 3), ("tvd", 2, 2), ("add", 1, 2),
                                               ("add", 1, 3)])
def test_native_mhd_step(oracle_lib, kind, order, method):
    """Kernel_TVD / add2 (kernel.cu:2198, 1877) on a random state, reference BCs."""
    g = golden("step_native.npz")
    grid = native_grid(g, order, method)
    s2, u2, b2, T = oracle_lib.step(grid, g["s"], g["u"], g["b"], float(g["T_do"]))
    assert T == g[f"{kind}{method}_T"]
    assert np.array_equal(s2, g[f"{kind}{method}_s"])
    assert np.array_equal(u2, g[f"{kind}{method}_u"])
    assert np.array_equal(b2, g[f"{kind}{method}_b"])


def test_native_euler_first_order(oracle_lib):
    """Ker_Dekard (kernel.cu:1736) leaves the last column and row unwritten; compare the rest."""
    g = golden("step_native.npz")
    grid = native_grid(g, 1, 1, physics=oracle.EULER)
    s2, u2, _, T = oracle_lib.step(grid, g["s"], g["u"], None, float(g["T_do"]))
    N, M = grid.N, grid.M
    mask = np.zeros((M, N), bool)
    mask[: M - 1, : N - 1] = True
    mask = mask.ravel()
    assert np.array_equal(s2[mask], g["dek_s"][mask])
    assert np.array_equal(u2[mask], g["dek_u"][mask])


def test_native_run_20_steps(oracle_lib):
    """The reference protocol (Kernel_TVD + funk_time, kernel.cu:4110-4127) from the wind
    initial condition, 20 steps, bit for bit including the dt sequence."""
    g = golden("run_native.npz")
    N, M = int(g["N"]), int(g["M"])
    xmax, ymax = float(g["xmax"]), float(g["ymax"])
    grid = oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), 5.0 / 3.0,
                       0.25, physics=oracle.MHD, geometry=oracle.AXISYM, order=2, method=3,
                       bc=(oracle.BC_MIRROR_X, oracle.BC_OUTFLOW, oracle.BC_AXIS,
                           oracle.BC_AMBIENT), frozen_radius=0.3)
    s, u, b, T_do, TT = oracle_lib.run(grid, g["s0"], g["u0"], g["b0"], int(g["nsteps"]), 1e-8)
    assert T_do == g["T_do"] and TT == g["TT"]
    assert np.array_equal(s, g["s"]) and np.array_equal(u, g["u"]) and np.array_equal(b, g["b"])


def io_grid(g):
    N, M = int(g["N"]), int(g["M"])
    xmax, ymax = float(g["xmax"]), float(g["ymax"])
    return oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M),
                       float(g["gamma"]), 0.25, physics=oracle.MHD)


def test_state_file_writers(oracle_lib, tmp_path):
    """The oracle's stdio writers produce the reference's files byte for byte: the restart
    dump of its main loop and the three Tecplot writers (golden bytes from the reference)."""
    g = golden("io_files.npz")
    grid = io_grid(g)
    s, u, b = g["s"], g["u"], g["b"]
    xmax, ymax = float(g["xmax"]), float(g["ymax"])
    xmin, ymin = xmax / (2.0 * grid.N), ymax / (2.0 * grid.M)
    p = str(tmp_path / "f")
    oracle_lib.write_restart(grid, s, u, b, p)
    assert open(p, "rb").read() == g["restart"].tobytes()
    for key, bb, t in (("tec_euler", None, None), ("tec_mhd", b, None),
                       ("tec_mhd_t", b, float(g["ttt"]))):
        oracle_lib.write_tecplot(grid, s, u, bb, int(g["nmin"]), xmin, xmax, ymin, ymax, p, t)
        assert open(p, "rb").read() == g[key].tobytes(), key


def test_hll_faces_and_first_order_step(oracle_lib):
    """HLL (kernel.cu:1485) on golden faces, and Ker_Dekard with method 0 (kernel.cu:1796)."""
    g = golden("faces_hll.npz")
    for i in range(len(g["t"])):
        t, F = oracle_lib.hll(g["L"][i], g["R"][i], g["normal"][i, 0], g["normal"][i, 1],
                              float(g["rad"]), float(g["gamma"][i]), float(g["krit"]))
        assert t == g["t"][i]
        assert np.array_equal(F, g["flux"][i], equal_nan=True), (i, F, g["flux"][i])
    grid = native_grid(g, 1, 0, physics=oracle.EULER)
    grid.method = 0
    s2, u2, _, T = oracle_lib.step(grid, g["s"], g["u"], None, float(g["T_do"]))
    N, M = grid.N, grid.M
    mask = np.zeros((M, N), bool)
    mask[: M - 1, : N - 1] = True  # Ker_Dekard leaves the last column and row unwritten
    mask = mask.ravel()
    assert np.array_equal(s2[mask], g["dek_s"][mask])
    assert np.array_equal(u2[mask], g["dek_u"][mask])


def gkr_grid(N, M, xmax, ymax, scheme=1, gamma=5.0 / 3.0, krit=0.25):
    """Kernel_GKR's setting (kernel.cu:2663-3284): its edge cells, metod 3, frozen sphere 2.0."""
    return oracle.Grid(N, M, xmax / N, ymax / M, xmax / (2.0 * N), ymax / (2.0 * M), gamma, krit,
                       physics=oracle.MHD, geometry=oracle.AXISYM, order=2, method=3,
                       bc=(oracle.BC_MIRROR_X, oracle.BC_OUTFLOW, oracle.BC_AXIS,
                           oracle.BC_AMBIENT_KEEPB),
                       frozen_radius=2.0, scheme=scheme, x_max=xmax, y_max=ymax)


@pytest.mark.parametrize("case", range(6))
def test_hancock_step(oracle_lib, case):
    """One Kernel_GKR step on the golden grids (down to 3 x 3, where every stencil point
    of every cell is a substitute), bit for bit including the dt."""
    g = golden("gkr.npz")
    N, M = (int(v) for v in g[f"c{case}_NM"])
    xmax, ymax = (float(v) for v in g[f"c{case}_ext"])
    grid = gkr_grid(N, M, xmax, ymax)
    s2, u2, b2, T = oracle_lib.step(grid, g[f"c{case}_s"], g[f"c{case}_u"], g[f"c{case}_b"],
                                    float(g["T_do"]))
    assert T == g[f"c{case}_T"]
    assert np.array_equal(s2, g[f"c{case}_s2"])
    assert np.array_equal(u2, g[f"c{case}_u2"])
    assert np.array_equal(b2, g[f"c{case}_b2"])


def test_hancock_run_20_steps(oracle_lib):
    """20 steps of Kernel_GKR + funk_time from the wind of problems.hancock_wind, bit for bit
    including the dt sequence."""
    g = golden("gkr.npz")
    N, M = int(g["run_N"]), int(g["run_M"])
    xmax, ymax = (float(v) for v in g["run_ext"])
    grid = gkr_grid(N, M, xmax, ymax)
    s, u, b, T_do, TT = oracle_lib.run(grid, g["run_s0"], g["run_u0"], g["run_b0"],
                                       int(g["run_nsteps"]), 1e-8)
    assert T_do == g["run_T_do"] and TT == g["run_TT"]
    assert np.array_equal(s, g["run_s"]) and np.array_equal(u, g["run_u"])
    assert np.array_equal(b, g["run_b"])


def test_hancock_schemes_differ_only_in_vy_slopes(oracle_lib):
    """Scheme 1 takes the v_y slopes from the pressures (kernel.cu:2966 ...), scheme 2 from
    v_y.  With v_y == p in every cell the two agree exactly on the rows whose stencils meet
    no axis mirror (v_y odd) or ambient substitute (v_y = 0, p = 1/gamma): 2 <= m < M-2.
    On a general state they differ."""
    rng = np.random.default_rng(5)
    N, M, xmax, ymax = 30, 20, 9.0, 5.0
    K = N * M
    s = np.stack([rng.uniform(0.3, 2.0, K), rng.uniform(0.1, 2.0, K)], 1)
    u = np.stack([rng.uniform(-1, 1, K), s[:, 1]], 1)
    b = rng.uniform(-2.0, 2.0, (K, 3))
    r1 = oracle_lib.step(gkr_grid(N, M, xmax, ymax, scheme=1), s, u, b, 2e-3)
    r2 = oracle_lib.step(gkr_grid(N, M, xmax, ymax, scheme=2), s, u, b, 2e-3)
    rows = slice(2 * N, (M - 2) * N)
    for a, c in zip(r1[:3], r2[:3]):
        assert np.array_equal(a[rows], c[rows])
    u[:, 1] = rng.uniform(-1, 1, K)
    r1 = oracle_lib.step(gkr_grid(N, M, xmax, ymax, scheme=1), s, u, b, 2e-3)
    r2 = oracle_lib.step(gkr_grid(N, M, xmax, ymax, scheme=2), s, u, b, 2e-3)
    assert not np.array_equal(r1[1], r2[1])



@pytest.mark.parametrize("case", ["sod256", "ot128", "kh256"])
def test_benchmark_run_checksums(oracle_lib, case):
    """Whole runs of the benchmark problems at reduced size (Sod 256^2 200 steps,
    Orszag-Tang 128^2 and KH 256^2 100 steps): the oracle reproduces the committed state
    hashes, field sums, L1 norms, dt and time after 1, 10 and N steps (checksums.npz,
    written by tests/golden/make_checksums.py)."""
    from golden.make_checksums import case_state, run_case
    gz = golden("checksums.npz")
    cfg, s, u, b, n = case_state(case, gz)
    recs = run_case(oracle_lib, cfg, s, u, b, n)
    assert [r[0] for r in recs] == list(gz[f"{case}_steps"])
    for i, (k, sha, sm, l1, T_do, TT) in enumerate(recs):
        assert sha == str(gz[f"{case}_sha"][i]), k
        assert np.array_equal(sm, gz[f"{case}_sum"][i]) and np.array_equal(l1, gz[f"{case}_l1"][i])
        assert T_do == gz[f"{case}_Tdo"][i] and TT == gz[f"{case}_TT"][i], k
