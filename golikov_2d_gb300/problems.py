"""Initial conditions and grid setups of the benchmark and test problems.

Each function returns ``(Config, s, u, b)`` with numpy arrays in the reference's AoS layout
(kernel.cu:3814-3825): ``s`` (K, 2) {rho, p}, ``u`` (K, 2) {vx, vy}, ``b`` (K, 3) Gaussian
{Bx, By, Bz} or None for Euler; cell k = m*N + n, centres x = x0 + n*dx, y = y0 + m*dy.
"""
from __future__ import annotations

import math

import numpy as np

from . import (AXISYM, BC_AMBIENT, BC_AXIS, BC_MIRROR_X, BC_OUTFLOW, BC_PERIODIC,
               BC_TRANSMISSIVE, CARTESIAN, EULER, HANCOCK_BC, MHD, METHOD_HLLC, METHOD_HLLD,
               MODE_FAST, SCHEME_HANCOCK_REF, Config)

KH_SEED = 20261203


def _centres(N, M, dx, dy, x0, y0):
    n = np.arange(N, dtype=np.float64)
    m = np.arange(M, dtype=np.float64)
    x = x0 + n * dx
    y = y0 + m * dy
    X, Y = np.meshgrid(x, y)  # (M, N), row-major like the cell index
    return X.ravel(), Y.ravel()


def unit_square(N, M, gamma, krit, **kw) -> Config:
    dx, dy = 1.0 / N, 1.0 / M
    return Config(N=N, M=M, dx=dx, dy=dy, x0=1.0 / (2.0 * N), y0=1.0 / (2.0 * M), gamma=gamma,
                  krit=krit, **kw)


def sod(N=256, M=256, krit=0.4, mode=MODE_FAST):
    """Sod shock tube along x on the unit square: x < 0.5: (rho, p) = (1, 1), else
    (0.125, 0.1); u = v = 0; gamma 1.4; transmissive boundaries; HLLC + minmod."""
    cfg = unit_square(N, M, 1.4, krit, physics=EULER, order=2, method=METHOD_HLLC,
                      bc=(BC_TRANSMISSIVE,) * 4, mode=mode)
    X, _ = _centres(N, M, cfg.dx, cfg.dy, cfg.x0, cfg.y0)
    left = X < 0.5
    s = np.stack([np.where(left, 1.0, 0.125), np.where(left, 1.0, 0.1)], 1)
    u = np.zeros((N * M, 2))
    return cfg, np.ascontiguousarray(s), u, None


def kelvin_helmholtz(N=4096, M=4096, krit=0.4, seed=KH_SEED, mode=MODE_FAST):
    """Periodic shear layer: rho = 2, vx = 0.5 for |y - 0.5| < 0.25, else rho = 1,
    vx = -0.5; p = 2.5; vy = 0.01 * U(-1, 1) per cell (numpy PCG64 seeded, row-major)."""
    cfg = unit_square(N, M, 1.4, krit, physics=EULER, order=2, method=METHOD_HLLC,
                      bc=(BC_PERIODIC,) * 4, mode=mode)
    _, Y = _centres(N, M, cfg.dx, cfg.dy, cfg.x0, cfg.y0)
    inner = np.abs(Y - 0.5) < 0.25
    rng = np.random.default_rng(seed)
    s = np.stack([np.where(inner, 2.0, 1.0), np.full(N * M, 2.5)], 1)
    u = np.stack([np.where(inner, 0.5, -0.5), 0.01 * rng.uniform(-1.0, 1.0, N * M)], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u), None


def orszag_tang(N=1024, M=1024, krit=0.4, method=METHOD_HLLD, mode=MODE_FAST):
    """Orszag-Tang vortex, periodic unit square, gamma 5/3: rho = 25/(36 pi),
    p = 5/(12 pi), v = (-sin 2 pi y, sin 2 pi x), B = B0 (-sin 2 pi y, sin 4 pi x) with
    B0 = 1/sqrt(4 pi) in Heaviside-Lorentz units, i.e. Gaussian B = (-sin 2 pi y, sin 4 pi x)
    as the reference stores it (its fluxes divide by sqrt(4 pi), Gas_Dinamic.cu:970-976)."""
    cfg = unit_square(N, M, 5.0 / 3.0, krit, physics=MHD, order=2, method=method,
                      bc=(BC_PERIODIC,) * 4, mode=mode)
    X, Y = _centres(N, M, cfg.dx, cfg.dy, cfg.x0, cfg.y0)
    K = N * M
    s = np.stack([np.full(K, 25.0 / (36.0 * math.pi)), np.full(K, 5.0 / (12.0 * math.pi))], 1)
    u = np.stack([-np.sin(2 * math.pi * Y), np.sin(2 * math.pi * X)], 1)
    b = np.stack([-np.sin(2 * math.pi * Y), np.sin(4 * math.pi * X), np.zeros(K)], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u), np.ascontiguousarray(b)


def four_quadrant(side, rng, krit=0.4, mode=MODE_FAST):
    """Four-quadrant Riemann problem on the unit square (transmissive): per quadrant
    rho, p ~ U[0.1, 2] and vx, vy ~ U[-1, 1] drawn from `rng`."""
    cfg = unit_square(side, side, 1.4, krit, physics=EULER, order=2, method=METHOD_HLLC,
                      bc=(BC_TRANSMISSIVE,) * 4, mode=mode)
    X, Y = _centres(side, side, cfg.dx, cfg.dy, cfg.x0, cfg.y0)
    q = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
    rho = rng.uniform(0.1, 2.0, 4)
    p = rng.uniform(0.1, 2.0, 4)
    vx = rng.uniform(-1.0, 1.0, 4)
    vy = rng.uniform(-1.0, 1.0, 4)
    s = np.stack([rho[q], p[q]], 1)
    u = np.stack([vx[q], vy[q]], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u), None


# Problem constants of the reference's production run (Header.h:24-38).
PHI_0, RR_0, M_ALF, M_0, DDIST = 4.0, 0.07, 8.0, 10.0, 0.3


def stellar_wind(N=3226, M=1792, xmax=9.0, ymax=5.0, krit=0.25, method=METHOD_HLLD, order=2,
                 mode=MODE_FAST, gamma=5.0 / 3.0):
    """The reference's production problem (kernel.cu:3901-3941): a magnetised wind sphere
    of radius ddist*1.01 in a uniform ambient medium, axisymmetric about y = 0, with the
    reference's boundary conditions (mirror at x = 0, outflow at x = xmax, axis at y = 0,
    ambient at y = ymax) and the frozen inner sphere dist < ddist."""
    dx, dy = xmax / N, ymax / M
    cfg = Config(N=N, M=M, dx=dx, dy=dy, x0=xmax / (2.0 * N), y0=ymax / (2.0 * M), gamma=gamma,
                 krit=krit, physics=MHD, geometry=AXISYM, order=order, method=method,
                 bc=(BC_MIRROR_X, BC_OUTFLOW, BC_AXIS, BC_AMBIENT), frozen_radius=DDIST,
                 mode=mode)
    X, Y = _centres(N, M, dx, dy, cfg.x0, cfg.y0)
    K = N * M
    dist = np.sqrt(X * X + Y * Y)
    V_E = PHI_0
    ro_E = 1.0 / (PHI_0 * PHI_0 * RR_0 * RR_0)
    P_E = ro_E * V_E * V_E / (gamma * M_0 * M_0)
    B_E = math.sqrt(4.0 * math.pi) / (M_ALF * RR_0)
    inside = dist < DDIST * 1.01
    dsafe = np.where(inside, dist, 1.0)
    s = np.stack([np.where(inside, ro_E / (dsafe / RR_0) ** 2, 1.0),
                  np.where(inside, P_E * (RR_0 / dsafe) ** (2.0 * gamma), 1.0 / gamma)], 1)
    u = np.stack([np.where(inside, V_E * X / dsafe, 0.0), np.where(inside, V_E * Y / dsafe, 0.0)], 1)
    BE = B_E / (dsafe / RR_0)
    bz = np.where(inside, BE * np.sin(np.arccos(np.clip(X / dsafe, -1.0, 1.0))), 0.0)
    b = np.stack([np.zeros(K), np.zeros(K), bz], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u), np.ascontiguousarray(b)


# Kernel_GKR freezes every cell with sqrt(x^2 + y^2) < 2.0 (kernel.cu:2692).
GKR_FROZEN = 2.0


def hancock_config(N, M, xmax=9.0, ymax=5.0, krit=0.25, gamma=5.0 / 3.0,
                   scheme=SCHEME_HANCOCK_REF, mode=MODE_FAST) -> Config:
    """The setting Kernel_GKR (kernel.cu:2663-3284) is written for: axisymmetric MHD, HLLD
    faces, its own edge cells (mirror at x = 0, outflow at x = xmax, axis at y = 0, ambient
    keeping B at y = ymax), the domain constants of kernel.cu:12-20 and its frozen sphere."""
    return Config(N=N, M=M, dx=xmax / N, dy=ymax / M, x0=xmax / (2.0 * N), y0=ymax / (2.0 * M),
                  gamma=gamma, krit=krit, physics=MHD, geometry=AXISYM, order=2,
                  method=METHOD_HLLD, bc=HANCOCK_BC, frozen_radius=GKR_FROZEN, mode=mode,
                  scheme=scheme, x_max=xmax, y_max=ymax)


def hancock_wind(N=3226, M=1792, xmax=9.0, ymax=5.0, scheme=SCHEME_HANCOCK_REF,
                 mode=MODE_FAST, gamma=5.0 / 3.0):
    """A wind for the MUSCL-Hancock step: the production wind profile of stellar_wind
    (kernel.cu:3901-3941) filling the sphere dist < 1.01 * 2.0, which Kernel_GKR keeps
    frozen, in the uniform ambient medium.  Cells are placed where Kernel_GKR places them
    (kernel.cu:2669-2670): x = x0 + n (xmax - x0)/(N - 1), y = y0 + m ymax / M."""
    cfg = hancock_config(N, M, xmax, ymax, gamma=gamma, scheme=scheme, mode=mode)
    n = np.arange(N, dtype=np.float64)
    m = np.arange(M, dtype=np.float64)
    X, Y = np.meshgrid(cfg.x0 + n * (xmax - cfg.x0) / (N - 1), cfg.y0 + m * ymax / M)
    X, Y = X.ravel(), Y.ravel()
    K = N * M
    dist = np.sqrt(X * X + Y * Y)
    V_E = PHI_0
    ro_E = 1.0 / (PHI_0 * PHI_0 * RR_0 * RR_0)
    P_E = ro_E * V_E * V_E / (gamma * M_0 * M_0)
    B_E = math.sqrt(4.0 * math.pi) / (M_ALF * RR_0)
    inside = dist < GKR_FROZEN * 1.01
    dsafe = np.where(inside, dist, 1.0)
    s = np.stack([np.where(inside, ro_E / (dsafe / RR_0) ** 2, 1.0),
                  np.where(inside, P_E * (RR_0 / dsafe) ** (2.0 * gamma), 1.0 / gamma)], 1)
    u = np.stack([np.where(inside, V_E * X / dsafe, 0.0), np.where(inside, V_E * Y / dsafe, 0.0)], 1)
    BE = B_E / (dsafe / RR_0)
    bz = np.where(inside, BE * np.sin(np.arccos(np.clip(X / dsafe, -1.0, 1.0))), 0.0)
    b = np.stack([np.zeros(K), np.zeros(K), bz], 1)
    return cfg, np.ascontiguousarray(s), np.ascontiguousarray(u), np.ascontiguousarray(b)


BATCH_SEED = 20261203


def batch_sides(n=512, lo=64, hi=512, seed=BATCH_SEED):
    """Grid sides log-uniform in [lo, hi]: round(exp(U(ln lo, ln hi))) from the seed."""
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(n)]


def batch_four_quadrant(n=512, lo=64, hi=512, seed=BATCH_SEED, krit=0.4):
    """The batched workload: n independent four-quadrant Riemann problems on square grids
    whose sides are log-uniform in [lo, hi]; per-quadrant rho, p ~ U[0.1, 2] and
    vx, vy ~ U[-1, 1]; HLLC + minmod, transmissive boundaries.  Returns a list of
    (Config, s, u, None)."""
    sides = batch_sides(n, lo, hi, seed)
    rng = np.random.default_rng(seed + 1)
    return [four_quadrant(side, rng, krit=krit) for side in sides]
