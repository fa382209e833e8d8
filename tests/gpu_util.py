"""Helpers for the GPU tests: run the CUDA library and the oracle on the same problem."""
from __future__ import annotations

import numpy as np

import golikov_2d_gb300 as g
import oracle


def grid_of(cfg: g.Config) -> oracle.Grid:
    return oracle.Grid(cfg.N, cfg.M, cfg.dx, cfg.dy, cfg.x0, cfg.y0, cfg.gamma, cfg.krit,
                       physics=cfg.physics, geometry=cfg.geometry, order=cfg.order,
                       method=cfg.method, bc=tuple(cfg.bc), frozen_radius=cfg.frozen_radius,
                       scheme=cfg.scheme, x_max=cfg.x_max, y_max=cfg.y_max)


def to_dev(a):
    import torch
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_step_ref(cfg, s, u, b, T_do, method=g.METHOD_CONFIG):
    """One step through gd_step_ref (device pointers, reference layout)."""
    import torch
    sol = g.Solver(cfg)
    ds, du, db = to_dev(s), to_dev(u), to_dev(b)
    s2, u2 = torch.zeros_like(ds), torch.zeros_like(du)
    b2 = None if db is None else torch.zeros_like(db)
    T = torch.tensor([1e7], dtype=torch.float64, device="cuda")
    Tdo = torch.tensor([T_do], dtype=torch.float64, device="cuda")
    sol.kernel_step(ds, du, db, s2, u2, b2, T, Tdo, 0, method)
    torch.cuda.synchronize()
    res = (s2.cpu().numpy(), u2.cpu().numpy(), None if b2 is None else b2.cpu().numpy(),
           float(T.cpu()[0]))
    sol.close()
    return res


def gpu_run(cfg, s, u, b, nsteps, T_do=None, use_graph=False):
    """nsteps of the resident loop; T_do None -> dt-only pre-pass.  Returns state, stats."""
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    if T_do is None:
        sol.set_time(0.0, 0.0)
        sol.init_dt()
    else:
        sol.set_time(T_do, 0.0)
    sol.advance(nsteps, use_graph=use_graph)
    s2, u2 = np.zeros_like(s), np.zeros_like(u)
    b2 = None if b is None else np.zeros_like(b)
    sol.export_state(s2, u2, b2)
    st = sol.stats(allow_nonfinite=True)
    sol.close()
    return s2, u2, b2, st


def oracle_run(o, cfg, s, u, b, nsteps, T_do=None):
    grid = grid_of(cfg)
    if T_do is None:
        T_do = o.dt_only(grid, s, u, b)
    return o.run(grid, s, u, b, nsteps, T_do)


def conserved(cfg, s, u, b):
    """Conserved fields (rho, rho vx, rho vy, E) [+ Bx, By, Bz] from the AoS primitives."""
    r, p = s[:, 0], s[:, 1]
    vx, vy = u[:, 0], u[:, 1]
    kin = 0.5 * r * (vx * vx + vy * vy)
    if b is None:
        return [r, r * vx, r * vy, p / (cfg.gamma - 1.0) + kin]
    mag = (b * b).sum(1) / (8.0 * np.pi)
    return [r, r * vx, r * vy, p / (cfg.gamma - 1.0) + kin + mag, b[:, 0], b[:, 1], b[:, 2]]


def rel_l1(a, ref):
    den = np.abs(ref).sum()
    num = np.abs(a - ref).sum()
    return num / den if den > 0 else num


def max_rel_l1(cfg, A, B):
    """Largest per-conserved-field relative L1 difference between states A and B."""
    ca, cb = conserved(cfg, *A), conserved(cfg, *B)
    return max(rel_l1(x, y) for x, y in zip(ca, cb))
