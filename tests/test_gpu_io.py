"""State files made and read on the GPU (include/gd2d.h: gd_format_text, gd_parse_text,
gd_write/read_text, gd_write/read_binary, gd_format/write_tecplot).

Writers are compared byte for byte with the reference's own writers (golden bytes from
print_file_mini / print_file_mini2 and the restart dump of its main loop, written by the
reference code compiled for the host) and with the oracle's stdio restatement on evolved
states; readers are compared bit for bit with Python's correctly rounded float() of every
token (the reference reads with `istream >> double`, also correctly rounded)."""
import os

import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems
from conftest import golden
from gpu_util import grid_of

pytestmark = pytest.mark.gpu


def golden_config(d, physics):
    N, M = int(d["N"]), int(d["M"])
    xmax, ymax = float(d["xmax"]), float(d["ymax"])
    return g.Config(N=N, M=M, dx=xmax / N, dy=ymax / M, x0=xmax / (2.0 * N), y0=ymax / (2.0 * M),
                    gamma=float(d["gamma"]), krit=0.25, physics=physics,
                    method=g.METHOD_HLLD if physics == g.MHD else g.METHOD_HLLC,
                    bc=(g.BC_PERIODIC,) * 4)


def solver_with(cfg, s, u, b):
    sol = g.Solver(cfg)
    sol.import_state(np.ascontiguousarray(s), np.ascontiguousarray(u),
                     None if b is None else np.ascontiguousarray(b))
    return sol


def exported(sol, cfg):
    K = cfg.N * cfg.M
    s, u = np.zeros((K, 2)), np.zeros((K, 2))
    b = np.zeros((K, 3)) if cfg.physics == g.MHD else None
    sol.export_state(s, u, b)
    return s, u, b


def tokens_as_state(text, K, physics):
    v = np.array([float(t) for t in text.split()[:9 * K]]).reshape(K, 9)
    return v[:, 2:4].copy(), v[:, 4:6].copy(), (v[:, 6:9].copy() if physics == g.MHD else None)


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def tec_args(d, cfg):
    xmax, ymax = float(d["xmax"]), float(d["ymax"])
    return dict(nmin=int(d["nmin"]), x_min=xmax / (2.0 * cfg.N), x_max=xmax,
                y_min=ymax / (2.0 * cfg.M), y_max=ymax)


def test_tecplot_is_the_reference_writer(cuda):
    d = golden("io_files.npz")
    for key, physics, t in (("tec_euler", g.EULER, None), ("tec_mhd", g.MHD, None),
                            ("tec_mhd_t", g.MHD, float(d["ttt"]))):
        cfg = golden_config(d, physics)
        sol = solver_with(cfg, d["s"], d["u"], d["b"] if physics == g.MHD else None)
        out = sol.format_tecplot(time=t, **tec_args(d, cfg))
        assert out == d[key].tobytes(), key
        sol.close()


def test_restart_text_is_the_reference_writer(cuda, tmp_path):
    d = golden("io_files.npz")
    cfg = golden_config(d, g.MHD)
    sol = solver_with(cfg, d["s"], d["u"], d["b"])
    text = sol.format_text()
    assert text == d["restart"].tobytes()
    p = str(tmp_path / "restart.txt")
    sol.write_text(p)
    assert open(p, "rb").read() == text
    p2 = str(tmp_path / "tec.dat")
    sol.write_tecplot(p2, **tec_args(d, cfg))
    assert open(p2, "rb").read() == d["tec_mhd"].tobytes()
    sol.close()


def test_parse_is_correctly_rounded(cuda, tmp_path):
    """The golden restart text and a text of 17-digit numbers with mixed separators parse to
    float() of every token; x, y are skipped, extra tokens after 9K are ignored."""
    d = golden("io_files.npz")
    cfg = golden_config(d, g.MHD)
    K = cfg.N * cfg.M
    text = d["restart"].tobytes()
    sol = g.Solver(cfg)
    sol.parse_text(text)
    for x, y in zip(exported(sol, cfg), tokens_as_state(text.decode(), K, g.MHD)):
        assert same_bits(x, y)
    rng = np.random.default_rng(9)
    vals = rng.standard_normal(9 * K + 5) * 10.0 ** rng.integers(-300, 300, 9 * K + 5)
    seps = [" ", "\t", "\n", "  ", "\r\n", " \n "]
    parts = [repr(float(v)) if i % 3 else f"{v:.17e}" for i, v in enumerate(vals)]
    body = "".join(p + seps[i % len(seps)] for i, p in enumerate(parts))
    p = str(tmp_path / "mixed.txt")
    with open(p, "w") as f:
        f.write("\n" + body)
    sol.read_text(p)
    for x, y in zip(exported(sol, cfg), tokens_as_state(body, K, g.MHD)):
        assert same_bits(x, y)
    sol.close()


def test_parse_errors(cuda):
    cfg, s, u, b = problems.orszag_tang(8, 8)
    sol = solver_with(cfg, s, u, b)
    good = sol.format_text()
    with pytest.raises(g.GdError) as e:
        sol.parse_text(good[: len(good) // 2])       # too few numbers
    assert e.value.status == 1
    # a malformed number and an overflowing one near the end of the text, after most
    # tokens parsed: a failed parse leaves the state as it was
    tail = good.rindex(b" ", 0, len(good) - 2)
    for junk in (b" 1.2.3 ", b" 1e999 "):
        with pytest.raises(g.GdError):
            sol.parse_text(good[:tail] + junk + good[tail + 1:])
        assert sol.format_text() == good
    with pytest.raises(g.GdError):
        sol.parse_text(b"")
    # the state after a good parse is the parsed one
    s2, u2, b2 = s * 1.5, u * 0.5, b * 2.0
    other = solver_with(cfg, s2, u2, b2)
    text2 = other.format_text()
    other.close()
    sol.parse_text(text2)
    assert sol.format_text() == text2
    sol.close()


@pytest.mark.parametrize("case", ["ot", "kh", "sod"])
def test_writers_match_oracle_on_evolved_states(cuda, oracle_lib, tmp_path, case):
    if case == "ot":
        cfg, s, u, b = problems.orszag_tang(96, 64)
    elif case == "kh":
        cfg, s, u, b = problems.kelvin_helmholtz(128, 80)
    else:
        cfg, s, u, b = problems.sod(64, 48)
    sol = solver_with(cfg, s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(12)
    s, u, b = exported(sol, cfg)
    grid = grid_of(cfg)
    p = str(tmp_path / "o")
    oracle_lib.write_restart(grid, s, u, b, p)
    assert sol.format_text() == open(p, "rb").read()
    for nmin, t in ((3, None), (1, 0.75), (5, None)):
        args = dict(nmin=nmin, x_min=cfg.x0, x_max=cfg.x0 + cfg.N * cfg.dx, y_min=cfg.y0,
                    y_max=cfg.y0 + cfg.M * cfg.dy)
        oracle_lib.write_tecplot(grid, s, u, b, nmin, args["x_min"], args["x_max"], args["y_min"],
                                 args["y_max"], p, t)
        assert sol.format_tecplot(time=t, **args) == open(p, "rb").read(), (nmin, t)
    pb = str(tmp_path / "b")
    sol.write_binary(pb)
    oracle_lib.write_binary(grid, s, u, b, p)
    assert open(pb, "rb").read() == open(p, "rb").read()
    # the binary file restores rho, p, vx, vy and Bz (Bx = By = 0: not in the file)
    sol2 = g.Solver(cfg)
    sol2.read_binary(pb)
    s2, u2, b2 = exported(sol2, cfg)
    assert same_bits(s2, s) and same_bits(u2, u)
    if b is not None:
        assert same_bits(b2[:, 2], b[:, 2]) and not b2[:, :2].any()
    sol.close()
    sol2.close()


def test_large_text_round_trip(cuda):
    """Orszag-Tang 1024x1024 after 5 steps: format -> parse into a second context -> format
    again gives the same bytes (the printed values are fixed points of parse + print), and
    the parsed state equals float() of the text on every cell."""
    cfg, s, u, b = problems.orszag_tang(1024, 1024)
    sol = solver_with(cfg, s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(5)
    text = sol.format_text()
    sol2 = g.Solver(cfg)
    sol2.parse_text(text)
    assert sol2.format_text() == text
    K = cfg.N * cfg.M
    tok = np.array([float(t) for t in text.split()[:9 * K]]).reshape(K, 9)
    s2, u2, b2 = exported(sol2, cfg)
    assert same_bits(s2, tok[:, 2:4]) and same_bits(u2, tok[:, 4:6]) and same_bits(b2, tok[:, 6:9])
    sol.close()
    sol2.close()
