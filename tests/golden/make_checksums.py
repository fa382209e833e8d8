"""Writes checksums.npz: per-step field checksums of the benchmark problems at reduced sizes.

Source: the oracle (oracle/gd_oracle.c), not the reference.  The reference has no Cartesian
periodic or transmissive step to run these problems (its kernels carry the axisymmetric
wind problem's boundaries); its pieces are pinned by make_golden.py's fixtures, which the
oracle matches bit for bit.  These checksums pin whole runs of the benchmark problems so
that the GPU tests can check them without running the oracle.

Cases (the configurations' shapes at reduced size, the reference protocol: a dt-only
pre-pass, then each step with the dt of the previous one and funk_time after it):
  sod256  Sod 256 x 256, transmissive, HLLC + minmod, 200 steps
  ot128   Orszag-Tang 128 x 128, periodic, HLLD + minmod, 100 steps
  kh256   Kelvin-Helmholtz 256 x 256, periodic, HLLC + minmod, 100 steps
Stored after 1, 10 and N steps: the SHA-256 of the state bytes (s, u[, b] in the reference's
AoS layout, little-endian doubles), per primitive field the sum and the L1 norm, T_do (the
dt of the next step) and TT.  The Orszag-Tang velocity and field are sines, whose last bit
may depend on the platform's libm: the fixture stores the three 1-D tables (sin 2 pi y_m,
sin 2 pi x_n, sin 4 pi x_n) and every user builds the state from them (case_state), so the
hashes hold on any host.

    python tests/golden/make_checksums.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from golikov_2d_gb300 import problems  # noqa: E402

CASES = {
    "sod256": (lambda: problems.sod(256, 256), 200),
    "ot128": (lambda: problems.orszag_tang(128, 128), 100),
    "kh256": (lambda: problems.kelvin_helmholtz(256, 256), 100),
}
CHECKPOINTS = (1, 10)  # and the case's N


def grid(cfg) -> oracle.Grid:
    return oracle.Grid(cfg.N, cfg.M, cfg.dx, cfg.dy, cfg.x0, cfg.y0, cfg.gamma, cfg.krit,
                       physics=cfg.physics, geometry=cfg.geometry, order=cfg.order,
                       method=cfg.method, bc=tuple(cfg.bc), frozen_radius=cfg.frozen_radius,
                       scheme=cfg.scheme, x_max=cfg.x_max, y_max=cfg.y_max)


def digest(s, u, b) -> str:
    h = hashlib.sha256()
    for a in (s, u, b):
        if a is not None:
            h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def field_sums(s, u, b):
    """Per primitive field (rho, p, vx, vy[, Bx, By, Bz]): sum and L1 norm."""
    X = np.concatenate([s, u] + ([] if b is None else [b]), axis=1)
    return X.sum(axis=0), np.abs(X).sum(axis=0)


def checkpoints(n):
    return [k for k in CHECKPOINTS if k < n] + [n]


def ot_tables(cfg):
    """sin 2 pi y_m (M values), sin 2 pi x_n and sin 4 pi x_n (N values) at cell centres."""
    x = cfg.x0 + np.arange(cfg.N) * cfg.dx
    y = cfg.y0 + np.arange(cfg.M) * cfg.dy
    return np.sin(2 * np.pi * y), np.sin(2 * np.pi * x), np.sin(4 * np.pi * x)


def case_state(name, gz=None):
    """(cfg, s, u, b, N) of a case; the Orszag-Tang sines from the fixture when given."""
    make, n = CASES[name]
    cfg, s, u, b = make()
    if name == "ot128":
        if gz is None:
            sy, sx, s2x = ot_tables(cfg)
        else:
            sy, sx, s2x = gz["ot128_sin2y"], gz["ot128_sin2x"], gz["ot128_sin4x"]
        SY = np.repeat(sy, cfg.N)   # row-major: cell k = m N + n
        SX = np.tile(sx, cfg.M)
        S2X = np.tile(s2x, cfg.M)
        u = np.ascontiguousarray(np.stack([-SY, SX], 1))
        b = np.ascontiguousarray(np.stack([-SY, S2X, np.zeros_like(SY)], 1))
    return cfg, s, u, b, n


def run_case(o, cfg, s, u, b, n):
    """The checkpoint records of one case: list of (steps, sha, sum, l1, T_do, TT)."""
    g = grid(cfg)
    T_do, TT = o.dt_only(g, s, u, b), 0.0
    done, out = 0, []
    for k in checkpoints(n):
        s, u, b, T_do, TT = o.run(g, s, u, b, k - done, T_do, TT)
        done = k
        sm, l1 = field_sums(s, u, b)
        out.append((k, digest(s, u, b), sm, l1, T_do, TT))
    return out


def main():
    oracle.build(ref=False)
    o = oracle.Oracle()
    arrays = {}
    for name in CASES:
        cfg, s, u, b, n = case_state(name)
        if name == "ot128":
            arrays["ot128_sin2y"], arrays["ot128_sin2x"], arrays["ot128_sin4x"] = ot_tables(cfg)
        recs = run_case(o, cfg, s, u, b, n)
        arrays[f"{name}_steps"] = np.array([r[0] for r in recs])
        arrays[f"{name}_sha"] = np.array([r[1] for r in recs])
        arrays[f"{name}_sum"] = np.stack([r[2] for r in recs])
        arrays[f"{name}_l1"] = np.stack([r[3] for r in recs])
        arrays[f"{name}_Tdo"] = np.array([r[4] for r in recs])
        arrays[f"{name}_TT"] = np.array([r[5] for r in recs])
        print(name, [(r[0], r[1][:12], r[4]) for r in recs], flush=True)
    np.savez_compressed(os.path.join(HERE, "checksums.npz"), **arrays)


if __name__ == "__main__":
    main()
