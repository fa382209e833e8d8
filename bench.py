"""Benchmark of the fused FP64 finite-volume step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload kh4096|ot1024|sod256] [--no-cpu-baseline]

One step = one pass of the fused step (reconstruction + fluxes + update + CFL dt + the
funk_time rotation) over the whole grid.  Metric: FP64 cell-updates/s, whole job.

* value     K steps timed with CUDA events on the launching stream, state resident in HBM.
* e2e       the same metric through the C ABI with HOST buffers: every step takes the state
            from pinned host memory and returns the result to it (gd_step_host: uploads, the
            step and downloads overlapped in bands of tile rows); copies inside the timed
            region.
* roofline  HBM roofline of the step kernel: algorithmic bytes per launch (each state field
            read once and written once, 8 B each) / average launch time, against the
            measured HBM bandwidth.  The step is FP64-issue bound on GB300; the "fp64"
            object reports that fraction against the FP64 FMA rate measured in this run.
* cpu_baseline  the oracle (the project's C restatement of the reference step, OpenMP over
            all host cores) timed on a bounded sample of the same workload.

--impl reference times the reference path on the host cores (the oracle port: the
reference's own CUDA sources are compiled for the host only where they are present, and
they are not on the GPU host) for the same workload, metric and unit.

Multi-GPU (torchrun): replicas only -- every rank advances its own copy of the workload
(the grid is not decomposed); value = all ranks' cell-updates / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (description, problem factory, bytes per cell-update)
    "kh4096": "Kelvin-Helmholtz 4096x4096 periodic, Euler, HLLC + minmod, CFL 0.4, FP64",
    "ot1024": "Orszag-Tang 1024x1024 periodic, ideal MHD, HLLD + minmod, CFL 0.4, FP64",
    "sod256": "Sod 256x256 transmissive, Euler, HLLC + minmod, CFL 0.4, FP64",
    # reduced cases for ncu captures (state still larger than L2)
    "kh2048": "Kelvin-Helmholtz 2048x2048 periodic, Euler, HLLC + minmod, CFL 0.4, FP64",
    "ot2048": "Orszag-Tang 2048x2048 periodic, ideal MHD, HLLD + minmod, CFL 0.4, FP64",
}
L2_BYTES = 129 * 2 ** 20


def make_problem(name, mode=0):
    from golikov_2d_gb300 import problems
    if name == "kh4096":
        return problems.kelvin_helmholtz(4096, 4096, mode=mode)
    if name == "ot1024":
        return problems.orszag_tang(1024, 1024, mode=mode)
    if name == "sod256":
        return problems.sod(256, 256, mode=mode)
    if name == "kh2048":
        return problems.kelvin_helmholtz(2048, 2048, mode=mode)
    if name == "ot2048":
        return problems.orszag_tang(2048, 2048, mode=mode)
    raise ValueError(name)


def bytes_per_cell(cfg) -> int:
    return 8 * 2 * cfg.nfields


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# FP64 operations per cell-update from one ncu capture of one launch of the kernel at the
# workload's own size: FP64-pipe thread instructions / cells
OPS_SOURCE = ("ncu sm__thread_inst_executed_pipe_fp64_pred_on.sum of one launch / cells, "
              "profiles/ncu_traffic.txt")


def ncu_traffic(workload):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == workload:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def ncu_fp64_per_cell(workload):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == workload:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


def int_products_per_cell(workload):
    """Binary64 products per cell the step kernel forms on the integer pipes (gd_swfp.cuh),
    from the `int_products=<n>` token of the workload's line in profiles/ncu_traffic.txt."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if parts and parts[0] == workload:
            for tok in parts[3:]:
                if tok.startswith("int_products="):
                    try:
                        return float(tok.split("=", 1)[1])
                    except ValueError:
                        return None
    return None


def ncu_l2_hit_pct(workload):
    """L2 sector hit rate of the step kernel (lts__t_sector_hit_rate) where the committed ncu
    summary records one, as an `l2hit=<percent>` token of the workload's line."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if parts and parts[0] == workload:
            for tok in parts[3:]:
                if tok.startswith("l2hit="):
                    try:
                        return float(tok[len("l2hit="):])
                    except ValueError:
                        return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id=None):
        self.bus_id = bus_id
        self.proc = None
        self.lines = []

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "100"]
        if self.bus_id:
            cmd[1:1] = ["-i", self.bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def job_aggregate(t_local, cells_local, device):
    """Whole-job numbers of a replicated run: the slowest rank's time (MAX over ranks) and
    the cell-updates of all ranks (SUM).  Identity when torch.distributed is not running."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return t_local, cells_local
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=device)
    c = torch.tensor([float(cells_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), float(c.item())


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def fp64_pipe_peak(torch, sm_mhz):
    """FP64 pipe peak (ops/s, FMA = 1) at the SM clock sampled during the timed region: 2 FP64
    operations per clock per SM; the maximum clock (2070 MHz) where no sample was taken."""
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = float(sm_mhz) if sm_mhz else 2070.0
    src = "median SM clock sampled in the timed region" if sm_mhz else "maximum SM clock"
    return 2.0 * sms * mhz * 1e6, f"2 ops/clk/SM x {sms} SMs x {mhz:.0f} MHz ({src})"


def fp64_roofline(g, workload, cells_per_s, torch, sm_mhz=None):
    """FP64 roofline of the step kernel.  The pipe peak is 2 FP64 operations per clock per
    SM (FMA counted once), i.e. 2 x SMs x the SM clock sampled while the step was timed;
    `gd_probe_fp64_peak` gives what a register-resident DFMA loop reaches on the same GPU.
    FP64 operations per cell come from the committed ncu capture (profiles/ncu_traffic.txt)."""
    probe = g.probe_fp64_peak()                       # FLOP/s, FMA = 2
    pipe_peak_ops, src = fp64_pipe_peak(torch, sm_mhz)
    out = {"unit": "FP64 ops/s (FMA = 1 op)", "pipe_peak": pipe_peak_ops,
           "dfma_loop_peak": probe / 2.0,
           "pipe_peak_source": src,
           "dfma_loop_source": "gd_probe_fp64_peak in this run"}
    per_cell = ncu_fp64_per_cell(workload)
    if per_cell is not None:
        ach = per_cell * cells_per_s
        out.update({"ops_per_cell": per_cell, "achieved": ach, "frac": ach / pipe_peak_ops,
                    "frac_of_dfma_loop": ach / (probe / 2.0),
                    "ops_source": OPS_SOURCE})
        ip = int_products_per_cell(workload)
        if ip is not None:
            # the binary64 arithmetic of a cell is the FP64-pipe operations plus the products
            # formed on the integer pipes (bit-identical to FP64 multiplies)
            b64 = (per_cell + ip) * cells_per_s
            out.update({"int_pipe_products_per_cell": ip,
                        "binary64_ops_per_cell": per_cell + ip,
                        "binary64_achieved": b64,
                        "binary64_vs_fp64_pipe_peak": b64 / pipe_peak_ops,
                        "int_products_source": "count of integer-pipe products in the kernel "
                                               "source per cell, profiles/ncu_traffic.txt"})
    return out


def measure_ot_to_end(g, torch, N=1024, t_end=0.5):
    """Orszag-Tang 1024^2 as the config states it, to t = 0.5: a dt-only pre-pass, then
    gd_advance_to (graphs, every dt limited to what is left to t_end).  Time to solution on
    the launching stream's events; the chunk read-backs are inside the timed region."""
    from golikov_2d_gb300 import problems
    cfg, s, u, b = problems.orszag_tang(N, N)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    n = sol.advance_to(t_end, use_graph=True)
    z.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(z)
    st = sol.stats(allow_nonfinite=True)
    s2, u2, b2 = np.zeros_like(s), np.zeros_like(u), np.zeros_like(b)
    sol.export_state(s2, u2, b2)
    sol.close()
    m0, m1 = float(s[:, 0].sum()), float(s2[:, 0].sum())
    return {"workload": WORKLOADS["ot1024"] + ", to t = 0.5", "steps": n, "t": st.t_state,
            "seconds": ms * 1e-3, "value": N * N * n / (ms * 1e-3), "unit": "cell-updates/s",
            "mass_rel_change": abs(m1 - m0) / abs(m0), "bz_max_abs": float(np.abs(b2[:, 2]).max()),
            "p_floor_hits": st.p_floor_hits, "nonfinite": st.nonfinite}


def measure_batched(g, torch, steps, ngrids=512):
    """The batched workload: 512 independent four-quadrant Riemann problems, sides log-uniform
    in [64, 512] (seeded), HLLC + minmod.  Persistent launch per step under a captured CUDA
    graph (tile shape from the autotuner) vs a loop of plain launches (one per grid)."""
    from golikov_2d_gb300 import problems
    grids = problems.batch_four_quadrant(ngrids)
    b = g.Batch([c for c, *_ in grids])
    for k, (c, s, u, _) in enumerate(grids):
        b.import_grid(k, s, u)
    b.set_time(0.0, 0.0)
    b.init_dt()
    b.autotune(reps=3)
    info = b.info()
    cells = info.total_cells
    stream = torch.cuda.current_stream()
    res = {"workload": f"{ngrids} four-quadrant Riemann grids, sides log-uniform in [64, 512] "
                       f"(seed {problems.BATCH_SEED}), Euler HLLC + minmod, FP64",
           "total_cells": cells, "steps": steps,
           "tile": f"{info.tile_x}x{info.tile_y}", "ctas": info.ctas, "tiles": info.tiles,
           "autotune_ms_per_step": {f"{tx}x{ty}": round(info.tuned_ms[v], 4) for v, (tx, ty) in
                                    enumerate(((16, 16), (32, 8), (32, 16), (64, 8)))},
           # cells of the tiles that lie outside their grids: tiles are the persistent
           # launch's work items, and a partly filled tile keeps its warps' FP64 issue
           "tile_fill": cells / (info.tiles * info.tile_x * info.tile_y)}
    for name, sched, graph in (("persistent_graph", g.BATCH_PERSISTENT, True),
                               ("looped_plain", g.BATCH_LOOPED, False),
                               ("looped_sync", g.BATCH_LOOPED_SYNC, False)):
        b.advance(steps, schedule=sched, use_graph=graph)  # warm-up (captures the graph)
        torch.cuda.synchronize()
        l0 = b.launch_count()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        b.advance(steps, schedule=sched, use_graph=graph)
        z.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(z)
        res[name] = {"value": cells * steps / (ms * 1e-3), "unit": "cell-updates/s",
                     "ms_per_step": ms / steps, "gpu_launches": b.launch_count() - l0}
    # speedup: against this library's own fused one-launch step looped over the grids, no
    # host synchronisation (the strict baseline); speedup_vs_looped_sync: against the same
    # loop with the host waiting for each launch, as the reference's main loop does after
    # each of its launches (kernel.cu:4113-4137; it issues two per step, the fused step one)
    ops = ncu_fp64_per_cell("batch512")
    if ops is not None:
        pipe, src = fp64_pipe_peak(torch, None)
        v = res["persistent_graph"]["value"]
        res["persistent_graph"]["fp64"] = {"ops_per_cell": ops, "achieved": ops * v,
                                           "pipe_peak": pipe, "frac": ops * v / pipe,
                                           "pipe_peak_source": src, "ops_source": OPS_SOURCE}
        res["persistent_graph"]["traffic_per_step"] = ncu_traffic("batch512")
    res["speedup"] = res["persistent_graph"]["value"] / res["looped_plain"]["value"]
    res["speedup_vs_looped_sync"] = (res["persistent_graph"]["value"] /
                                     res["looped_sync"]["value"])
    bad = sum(b.stats(k, allow_nonfinite=True).nonfinite for k in range(ngrids))
    res["nonfinite_cells"] = bad
    b.close()
    return res


def measure_io(g, torch, N=1024, reps=5, cpu_N=256):
    """State files of Orszag-Tang N x N after 5 steps, made and read on the GPU through the C
    ABI: the restart text (9 numbers per cell, the reference's dump format), the Tecplot
    snapshot at every point and at the reference's Nmin = 3, the binary dump.  Device time =
    formatting, scan and compaction with the image left on the device (gd_format_text with no
    buffer); e2e = the same into host memory (pageable, copy included); parse = host text ->
    device -> state.  CPU baseline: the oracle's stdio writer and reader (one thread, the
    reference writes and reads with one thread) on an N = cpu_N grid of the same problem."""
    import ctypes
    import tempfile
    from golikov_2d_gb300 import problems

    def state_after(n, steps=5):
        cfg, s, u, b = problems.orszag_tang(n, n)
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        sol.advance(steps)
        return cfg, sol

    def best(fn):
        fn()  # warm-up (scratch allocation)
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts), statistics.median(ts)

    cfg, sol = state_after(N)
    K = cfg.N * cfg.M
    lib, h = sol.lib, sol.handle
    n = ctypes.c_size_t(0)

    def fmt_device():
        if lib.gd_format_text(h, None, 0, ctypes.byref(n), None):
            raise RuntimeError("gd_format_text")

    fmt_device()
    nbytes = n.value
    buf = ctypes.create_string_buffer(nbytes)

    def fmt_host():
        if lib.gd_format_text(h, buf, nbytes, ctypes.byref(n), None):
            raise RuntimeError("gd_format_text")

    l0 = sol.launch_count()
    t_dev, t_dev_med = best(fmt_device)
    launches = (sol.launch_count() - l0) // (reps + 1)
    t_e2e, _ = best(fmt_host)
    text = buf.raw[:nbytes]
    sol2 = g.Solver(cfg)
    t_parse, _ = best(lambda: sol2.parse_text(text))
    ok = sol2.format_text() == text
    peak, _ = measured_peaks()
    state_bytes = K * 7 * 8
    res = {"workload": f"Orszag-Tang {N}x{N} MHD state after 5 steps", "cells": K,
           "restart_text": {
               "bytes": nbytes, "bytes_per_cell": nbytes / K,
               "format_device_s": t_dev, "format_device_median_s": t_dev_med,
               "format_cells_per_s": K / t_dev, "format_text_GBps": nbytes / t_dev / 1e9,
               "format_e2e_s": t_e2e, "format_e2e_cells_per_s": K / t_e2e,
               "parse_e2e_s": t_parse, "parse_cells_per_s": K / t_parse,
               "parse_text_GBps": nbytes / t_parse / 1e9, "round_trip_identical": ok,
               "launches_per_format": launches,
               "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak,
                            "algorithmic_bytes": state_bytes + nbytes,
                            "achieved": (state_bytes + nbytes) / t_dev / 1e9,
                            "frac": (state_bytes + nbytes) / t_dev / 1e9 / peak,
                            "note": "state read once + text written once; the formatter is "
                                    "integer-issue bound (digit generation)"}}}
    for nmin in (1, 3):
        o = sol.tecplot_opts(nmin, cfg.x0, cfg.x0 + cfg.N * cfg.dx, cfg.y0,
                             cfg.y0 + cfg.M * cfg.dy)

        def tec():
            if lib.gd_format_tecplot(h, ctypes.byref(o), None, 0, ctypes.byref(n), None):
                raise RuntimeError("gd_format_tecplot")

        t_tec, _ = best(tec)
        res[f"tecplot_nmin{nmin}"] = {"bytes": n.value, "format_device_s": t_tec,
                                      "points_per_s": ((cfg.N + nmin - 1) // nmin) ** 2 / t_tec}
    with tempfile.TemporaryDirectory() as d:
        pb = os.path.join(d, "save_b3.dat")
        t_bin, _ = best(lambda: sol.write_binary(pb))
        res["binary"] = {"bytes": os.path.getsize(pb), "write_file_s": t_bin}
        pt = os.path.join(d, "restart.txt")
        t_wf, _ = best(lambda: sol.write_text(pt))
        res["restart_text"]["write_file_s"] = t_wf
        t_rf, _ = best(lambda: sol2.read_text(pt))
        res["restart_text"]["read_file_s"] = t_rf
        # CPU baseline: the oracle's writer and reader, one thread
        import oracle
        oracle.build(ref=False)
        o = oracle.Oracle()
        cfg_c, sol_c = state_after(cpu_N)
        Kc = cfg_c.N * cfg_c.M
        sc, uc, bc = np.zeros((Kc, 2)), np.zeros((Kc, 2)), np.zeros((Kc, 3))
        sol_c.export_state(sc, uc, bc)
        grid = oracle.Grid(cfg_c.N, cfg_c.M, cfg_c.dx, cfg_c.dy, cfg_c.x0, cfg_c.y0, cfg_c.gamma,
                           cfg_c.krit, physics=oracle.MHD)
        pc = os.path.join(d, "cpu.txt")
        t0 = time.perf_counter()
        o.write_restart(grid, sc, uc, bc, pc)
        t_cw = time.perf_counter() - t0
        t0 = time.perf_counter()
        o.read_restart(grid, pc)
        t_cr = time.perf_counter() - t0
        same = open(pc, "rb").read() == sol_c.format_text()
        sol_c.close()
    res["cpu_baseline"] = {"kind": "port", "cores": 1,
                           "sample": f"Orszag-Tang {cpu_N}x{cpu_N} restart text, oracle "
                                     f"gdo_write_restart / gdo_read_restart (C stdio)",
                           "write_cells_per_s": Kc / t_cw, "read_cells_per_s": Kc / t_cr,
                           "gpu_text_identical": same}
    sol.close()
    sol2.close()
    return res


def adjoint_step_case(g, torch, N=512):
    """A short differentiation run for kernel profiles: Orszag-Tang N x N, 20 plain steps,
    a 10-step recording, one backward sweep and one tangent sweep."""
    H = AdjointHarness(g, torch, N)
    H.start(H.U_ic, 20)
    U0 = H.state()
    H.sol.adj_forward(10, 10)
    rng = np.random.default_rng(1)
    lam = [H.dev(rng.standard_normal(tuple(x.shape))) for x in U0]
    out = H.zeros(U0)
    H.sol.adj_backward(*lam, *out)
    tan = H.jvp(lam)
    torch.cuda.synchronize()
    ok = all(bool(torch.isfinite(x).all()) for x in out + tan)
    H.close()
    print(json.dumps({"case": "adjoint-step", "grid": f"{N}x{N}", "finite": ok}), flush=True)
    return 0 if ok else 1


def batch_step_case(g, torch, ngrids=512):
    """The batched workload for kernel profiles: the 512 grids imported, a dt pass, then four
    persistent steps (16 x 16 tiles, no autotuning), so the fifth euler_batch_kernel launch
    is a plain step."""
    from golikov_2d_gb300 import problems
    grids = problems.batch_four_quadrant(ngrids)
    b = g.Batch([c for c, *_ in grids])
    for k, (c, s, u, _) in enumerate(grids):
        b.import_grid(k, s, u)
    b.set_time(0.0, 0.0)
    b.init_dt()
    b.advance(4, schedule=g.BATCH_PERSISTENT, use_graph=False)
    torch.cuda.synchronize()
    info = b.info()
    bad = sum(b.stats(k, allow_nonfinite=True).nonfinite for k in range(ngrids))
    b.close()
    print(json.dumps({"case": "batch-step", "tiles": info.tiles, "nonfinite_cells": bad}),
          flush=True)
    return 0 if bad == 0 else 1


def adjoint_step_euler_case(g, torch, N=512):
    """The Euler counterpart for kernel profiles: Kelvin-Helmholtz N x N, 20 plain steps, a
    10-step recording, one backward sweep and one tangent sweep."""
    from golikov_2d_gb300 import problems
    cfg, s, u, _ = problems.kelvin_helmholtz(N, N)
    sol = g.Solver(cfg)
    sol.import_state(s, u, None)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(20)
    sol.adj_forward(10, 10)
    rng = np.random.default_rng(1)
    lam = [torch.from_numpy(rng.standard_normal(x.shape)).cuda() for x in (s, u)]
    out = [torch.zeros_like(x) for x in lam]
    sol.adj_backward(lam[0], lam[1], None, out[0], out[1], None)
    tan = [torch.zeros_like(x) for x in lam]
    sol.tangent(lam[0], lam[1], None, tan[0], tan[1], None)
    torch.cuda.synchronize()
    ok = all(bool(torch.isfinite(x).all()) for x in out + tan)
    sol.close()
    print(json.dumps({"case": "adjoint-step-euler", "grid": f"{N}x{N}", "finite": ok}),
          flush=True)
    return 0 if ok else 1


class AdjointHarness:
    """One Orszag-Tang grid with its solver and the device-side helpers of the gradient
    checks (device tensors in the reference AoS layout)."""

    def __init__(self, g, torch, N):
        from golikov_2d_gb300 import problems
        self.torch = torch
        self.cfg, s, u, b = problems.orszag_tang(N, N)
        self.sol = g.Solver(self.cfg)
        self.U_ic = [self.dev(x) for x in (s, u, b)]

    def dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def zeros(self, U):
        return [self.torch.zeros_like(x) for x in U]

    def start(self, U, steps=0):
        self.sol.import_state(*U)
        self.sol.set_time(0.0, 0.0)
        self.sol.init_dt()
        if steps:
            self.sol.advance(steps)

    def state(self):
        out = self.zeros(self.U_ic)
        self.sol.export_state(*out)
        return out

    def replay(self, U):
        o = self.zeros(U)
        self.sol.adj_replay(*U, *o)
        return o

    def jvp(self, V):
        o = self.zeros(V)
        self.sol.tangent(*V, *o)
        return o

    def target_density(self, U, n):
        """Final density of the target run: its own run (own CFL dt sequence) of n steps from
        U with the velocity perturbed by a seeded 1 % per-cell factor."""
        rng = np.random.default_rng(20261203)
        pert = self.dev(1.0 + 0.01 * rng.uniform(-1.0, 1.0, tuple(U[1].shape)))
        self.start([U[0], U[1] * pert, U[2]])
        self.sol.advance(n)
        return self.state()[0][:, 0].clone()

    def gradient(self, U0, n, every):
        """Records n steps from U0 and returns (grad, G, rho_t) of
        L = 1/2 |rho_n - rho_target|^2."""
        rho_t = self.target_density(U0, n)
        self.start(U0)
        self.sol.adj_forward(n, every)
        Uf = self.state()
        G = self.zeros(U0)
        G[0][:, 0] = Uf[0][:, 0] - rho_t
        grad = self.zeros(U0)
        self.sol.adj_backward(*G, *grad)
        return grad, G, rho_t

    def fd_window(self, U0, n, every, ndir, label, bound=None):
        """Gradient of the n-step loss from U0 against central differences and the tangent
        on `ndir` seeded random unit directions.  The difference quotient is formed per cell,
        (L+ - L-) = sum (r+ - r-) ((r+ + r-) / 2 - t), exact algebra that keeps the
        cancellation in the per-cell differences.  A step that straddles a minmod switch or
        a clamp is not the derivative of the active branch; such a direction is retaken at
        eps / 10 and eps / 100 and the closest quotient kept (a wrong derivative stays wrong
        at every eps)."""
        grad, G, rho_t = self.gradient(U0, n, every)
        f0 = self.sol.stats(allow_nonfinite=True).p_floor_hits
        fd_rel, tan_rel, eps_used, first = [], [], [], []
        rng = np.random.default_rng(11)
        for _ in range(ndir):
            d = [self.dev(rng.standard_normal(tuple(x.shape))) for x in U0]
            nrm = math.sqrt(sum(float((x * x).sum()) for x in d))
            d = [x / nrm for x in d]
            ad = sum(float((x * y).sum()) for x, y in zip(grad, d))
            tn = float((G[0][:, 0] * self.jvp(d)[0][:, 0]).sum())
            tan_rel.append(abs(ad - tn) / abs(ad))
            best, beps = None, None
            for eps in (1e-7, 1e-8, 1e-9):
                rp = self.replay([x + eps * y for x, y in zip(U0, d)])[0][:, 0]
                rm = self.replay([x - eps * y for x, y in zip(U0, d)])[0][:, 0]
                fd = float(((rp - rm) * (0.5 * (rp + rm) - rho_t)).sum()) / (2 * eps)
                err = abs(fd - ad) / abs(ad)
                if best is None:
                    first.append(err)
                if best is None or err < best:
                    best, beps = err, eps
                if best <= 1e-6:
                    break
            fd_rel.append(best)
            eps_used.append(beps)
        self.start(U0)            # pressure clamps inside the window: a plain run
        self.sol.advance(n)
        floors = self.sol.stats(allow_nonfinite=True).p_floor_hits - f0
        out = {"grid": f"{self.cfg.N}x{self.cfg.M}", "start": label, "steps": n,
               "ckpt_every": every, "directions": ndir,
               "p_floor_clamps_in_window": int(floors),
               "max_rel": max(fd_rel), "median_rel": float(np.median(fd_rel)),
               "max_rel_at_eps_1e-7": max(first),
               "eps_counts": {f"{e:g}": eps_used.count(e) for e in sorted(set(eps_used))},
               "tangent_max_rel": max(tan_rel)}
        if bound is not None:
            out.update({"bound": bound, "pass": max(fd_rel) <= bound})
        return out

    def fd_switches(self, U0, n, every, ndir, eps_list=(1e-6, 1e-7, 1e-8, 1e-9)):
        """The central-difference check as the configuration states it: n steps from U0
        with checkpoints every `every`, `ndir` seeded random unit directions, each at every
        eps of `eps_list`.  Each pair of runs (U0 + eps v, U0 - eps v) goes through
        gd_adj_switches, which counts the steps and cells where the two runs take different
        branches of a non-smooth choice; the quotient is the derivative of the branch the
        adjoint differentiates only where that count is 0."""
        torch = self.torch
        grad, G, rho_t = self.gradient(U0, n, every)
        rng = np.random.default_rng(11)
        rows = []
        for i in range(ndir):
            d = [self.dev(rng.standard_normal(tuple(x.shape))) for x in U0]
            nrm = math.sqrt(sum(float((x * x).sum()) for x in d))
            d = [x / nrm for x in d]
            ad = sum(float((x * y).sum()) for x, y in zip(grad, d))
            tn = float((G[0][:, 0] * self.jvp(d)[0][:, 0]).sum())
            per_eps = []
            for eps in eps_list:
                Up = [x + eps * y for x, y in zip(U0, d)]
                Um = [x - eps * y for x, y in zip(U0, d)]
                Op, Om = self.zeros(U0), self.zeros(U0)
                c = self.sol.adj_switches(Up, Um, Op, Om)
                rp, rm = Op[0][:, 0], Om[0][:, 0]
                # with the recorded dt sequence held fixed, a run whose own wave speeds
                # exceed the recorded ones can break its CFL limit and turn non-finite
                finite = all(bool(torch.isfinite(x).all()) for x in Op + Om)
                fd = float(((rp - rm) * (0.5 * (rp + rm) - rho_t)).sum()) / (2 * eps)
                per_eps.append({"eps": eps,
                                "rel_err": abs(fd - ad) / abs(ad) if finite else None,
                                "replays_finite": finite,
                                "switched_cells": c["cells"], "switches": c})
            rows.append({"direction": i, "adjoint": ad,
                         "tangent_rel": abs(ad - tn) / abs(ad), "by_eps": per_eps})
        clean = [(r["direction"], e["eps"], e["rel_err"]) for r in rows for e in r["by_eps"]
                 if e["switched_cells"] == 0 and e["replays_finite"]]
        clean_dirs = sorted({c[0] for c in clean})
        errs = lambda r: [e["rel_err"] for e in r["by_eps"] if e["rel_err"] is not None]
        best = [min(errs(r)) for r in rows if errs(r)]
        summary = {
            "grid": f"{self.cfg.N}x{self.cfg.M}", "steps": n, "ckpt_every": every,
            "directions": ndir, "eps": list(eps_list),
            "directions_crossing_a_switch_at_every_eps": ndir - len(clean_dirs),
            "directions_with_a_switch_free_eps": len(clean_dirs),
            "max_rel_err_switch_free": max((c[2] for c in clean), default=None),
            "switch_free_meets_1e-6": all(c[2] <= 1e-6 for c in clean) if clean else None,
            "switch_free_pairs_by_eps": {f"{e:g}": sum(1 for c in clean if c[1] == e)
                                         for e in eps_list},
            "min_switched_cells_by_eps": {
                f"{e:g}": min(r["by_eps"][j]["switched_cells"] for r in rows)
                for j, e in enumerate(eps_list)},
            "nonfinite_replays_by_eps": {
                f"{e:g}": sum(1 for r in rows if not r["by_eps"][j]["replays_finite"])
                for j, e in enumerate(eps_list)},
            "median_rel_err_by_eps": {
                f"{e:g}": (float(np.median(v)) if v else None) for e, v in
                ((e, [r["by_eps"][j]["rel_err"] for r in rows
                      if r["by_eps"][j]["rel_err"] is not None])
                 for j, e in enumerate(eps_list))},
            "best_eps_rel_err_max": max(best) if best else None,
            "best_eps_rel_err_median": float(np.median(best)) if best else None,
            "tangent_max_rel": max(r["tangent_rel"] for r in rows),
        }
        torch.cuda.synchronize()
        return {"summary": summary, "per_direction": rows}

    def close(self):
        self.sol.close()


def measure_adjoint(g, torch, N=512, nsteps=100, every=10, ndir=32, ntan=8,
                    fd_N=32, fd_pre=40, fd_steps=30):
    """Orszag-Tang MHD N x N, HLLD + minmod, `nsteps` steps with checkpoints every `every`;
    loss = 1/2 |rho_n - rho_target|^2, the target being the final density of its own run
    from a seeded 1 % per-cell perturbation of the initial velocity.  Reports

    * the cost of one gradient (checkpointed forward + backward) against the plain forward
      run of the same steps;
    * the gradient against the hand-written tangent kernel (forward mode) on the measured
      problem itself, on `ntan` seeded random directions: both differentiate the branch the
      values take, so they agree to rounding even on the kinks below;
    * the gradient against FP64 central differences on `ndir` seeded random unit
      directions.  The map is piecewise smooth: minmod switches (|l| against |r|, signs),
      the Orszag-Tang initial state itself (rho and p uniform: minmod(0, 0)) and, from step
      59 on the 512 grid, the clamp p <= 0 -> 1e-6.  A difference quotient whose +-eps
      straddles a switch is not the derivative.  The check as configured (N x N from the
      initial state, `nsteps` steps, `ndir` directions) runs every direction at four eps
      through gd_adj_switches, which counts the cells and steps where the +eps and -eps runs
      take different branches (minmod picks, fallbacks, HLLD speeds, region, guards,
      floors); the bound applies where that count is 0.  A bounded check (1e-6) also runs
      on the same problem at `fd_N` (state after `fd_pre` steps, `fd_steps` steps)."""
    stream = torch.cuda.current_stream()

    def timed(fn):
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z)

    H = AdjointHarness(g, torch, N)
    sol, U_ic = H.sol, H.U_ic
    res = {"workload": f"Orszag-Tang MHD {N}x{N}, HLLD + minmod, FP64, {nsteps} steps, "
                       f"checkpoints every {every}", "nsteps": nsteps, "ckpt_every": every}

    # --- cost: plain forward run vs gradient (checkpointed forward + backward) ---------------
    H.start(U_ic)
    sol.advance(3)
    H.start(U_ic)
    ms_fwd = timed(lambda: sol.advance(nsteps))
    grad, G, _ = H.gradient(U_ic, nsteps, every)      # also warms the backward kernels
    l0 = sol.launch_count()
    H.start(U_ic)
    ms_rec = timed(lambda: sol.adj_forward(nsteps, every))
    ms_bwd = timed(lambda: sol.adj_backward(*G, *grad))
    res.update({"forward_ms": ms_fwd, "forward_ms_per_step": ms_fwd / nsteps,
                "record_ms": ms_rec, "backward_ms": ms_bwd,
                "gradient_ms": ms_rec + ms_bwd,
                "gradient_cost_vs_forward": (ms_rec + ms_bwd) / ms_fwd,
                "backward_cost_vs_forward": ms_bwd / ms_fwd,
                "gpu_launches": sol.launch_count() - l0})

    # --- tangent vs adjoint on the measured problem ------------------------------------------
    rng = np.random.default_rng(7)
    rel = []
    for _ in range(ntan):
        d = [H.dev(rng.standard_normal(tuple(x.shape))) for x in U_ic]
        ad = sum(float((x * y).sum()) for x, y in zip(grad, d))
        tn = float((G[0][:, 0] * H.jvp(d)[0][:, 0]).sum())
        rel.append(abs(ad - tn) / max(abs(ad), abs(tn)))
    res["tangent_vs_adjoint"] = {"directions": ntan, "max_rel": max(rel)}

    # --- central differences -------------------------------------------------------------------
    Hs = AdjointHarness(g, torch, fd_N)
    Hs.start(Hs.U_ic, fd_pre)
    res["central_differences"] = Hs.fd_window(Hs.state(), fd_steps, every, ndir,
                                              f"Orszag-Tang state after {fd_pre} steps",
                                              bound=1e-6)
    Hs.close()
    # the configuration's own check: from the initial state, nsteps, checkpoints every
    # `every`, ndir directions, with the branch switches of every difference quotient
    H.start(U_ic)
    U0 = H.state()
    res["central_differences_config"] = H.fd_switches(U0, nsteps, every, ndir)
    H.close()
    return res


def measure_adjoint_euler(g, torch, N=512, nsteps=100, every=10):
    """The Euler (HLLC) adjoint's cost: Kelvin-Helmholtz N x N, `nsteps` steps with
    checkpoints every `every`, one gradient (checkpointed forward + backward) against the
    plain forward run of the same steps."""
    from golikov_2d_gb300 import problems
    stream = torch.cuda.current_stream()
    cfg, s, u, _ = problems.kelvin_helmholtz(N, N)
    sol = g.Solver(cfg)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def start():
        sol.import_state(s, u, None)
        sol.set_time(0.0, 0.0)
        sol.init_dt()

    def timed(fn):
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z)

    rng = np.random.default_rng(11)
    lam = [dev(rng.standard_normal(x.shape)) for x in (s, u)]
    out = [torch.zeros_like(x) for x in lam]
    start()
    sol.advance(3)
    start()
    ms_fwd = timed(lambda: sol.advance(nsteps))
    start()
    sol.adj_forward(nsteps, every)
    sol.adj_backward(lam[0], lam[1], None, out[0], out[1], None)  # warm-up
    start()
    ms_rec = timed(lambda: sol.adj_forward(nsteps, every))
    ms_bwd = timed(lambda: sol.adj_backward(lam[0], lam[1], None, out[0], out[1], None))
    sol.close()
    return {"workload": f"Kelvin-Helmholtz Euler {N}x{N}, HLLC + minmod, FP64, {nsteps} steps, "
                        f"checkpoints every {every}",
            "forward_ms": ms_fwd, "record_ms": ms_rec, "backward_ms": ms_bwd,
            "gradient_cost_vs_forward": (ms_rec + ms_bwd) / ms_fwd}


HANCOCK_WORKLOAD = ("MUSCL-Hancock step of Kernel_GKR (scheme as written), axisymmetric MHD, "
                    "HLLD, wind in ambient medium, 3226x1792 (the reference's production grid), "
                    "CFL 0.25, FP64")


def measure_hancock(g, torch, steps=20, parity_steps=3, warmup=3, N=3226, M=1792,
                    cpu_steps=1, cpu=True):
    """The MUSCL-Hancock step (Kernel_GKR) on the reference's production grid: fast and
    parity modes timed with CUDA events on the launching stream (state 324 MB, larger than
    L2), e2e through host buffers, and the oracle's restatement on the host cores."""
    from golikov_2d_gb300 import problems
    out = {"workload": HANCOCK_WORKLOAD, "cells": N * M, "unit": "cell-updates/s"}
    stream = torch.cuda.current_stream()
    for name, mode, k in (("fast", g.MODE_FAST, steps), ("parity", g.MODE_PARITY, parity_steps)):
        cfg, s, u, b = problems.hancock_wind(N, M, mode=mode)
        sol = g.Solver(cfg)
        sol.import_state(s, u, b)
        sol.set_time(0.0, 0.0)
        sol.init_dt()
        sol.advance(warmup)
        torch.cuda.synchronize()
        l0 = sol.launch_count()
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler() as clk:
            a.record(stream)
            sol.advance(k)
            z.record(stream)
            torch.cuda.synchronize()
        ms = a.elapsed_time(z) / k
        st = sol.stats(allow_nonfinite=True)
        entry = {"value": N * M / (ms * 1e-3), "ms_per_step": ms, "steps": k,
                 "gpu_launches": sol.launch_count() - l0, "nonfinite": st.nonfinite,
                 "rho_floor_hits": st.rho_floor_hits, "p_floor_hits": st.p_floor_hits,
                 "clocks": clk.summary()}
        if mode == g.MODE_FAST:
            hs, hu, hb = (torch.from_numpy(x).pin_memory() for x in (s, u, b))
            hs2, hu2, hb2 = (torch.empty_like(x).pin_memory() for x in (hs, hu, hb))
            for _ in range(2):  # warm-up: the step graphs of both plane sets are captured
                sol.step_host(hs, hu, hb, hs2, hu2, hb2)
            torch.cuda.synchronize()
            n_e2e = 5
            t0 = time.perf_counter()
            for _ in range(n_e2e):
                sol.step_host(hs, hu, hb, hs2, hu2, hb2)
            torch.cuda.synchronize()
            io_bytes = N * M * 7 * 8
            entry["e2e"] = {"value": N * M * n_e2e / (time.perf_counter() - t0),
                            "unit": "cell-updates/s", "h2d_bytes_per_step": io_bytes,
                            "d2h_bytes_per_step": io_bytes}
            ops = ncu_fp64_per_cell("hancock3226")
            if ops is not None:
                pipe, src = fp64_pipe_peak(torch, entry["clocks"]["sm_mhz"])
                entry["fp64"] = {"ops_per_cell": ops, "achieved": ops * entry["value"],
                                 "pipe_peak": pipe, "frac": ops * entry["value"] / pipe,
                                 "pipe_peak_source": src, "ops_source": OPS_SOURCE}
            peak_gbs, kind = measured_peaks()
            ach = N * M * 7 * 16 / (ms * 1e-3) / 1e9
            entry["hbm"] = {"achieved": ach, "peak": peak_gbs, "unit": "GB/s",
                            "frac": ach / peak_gbs, "traffic": ncu_traffic("hancock3226"),
                            "algorithmic_bytes_per_step": N * M * 7 * 16,
                            "peak_source": kind}
        out[name] = entry
        sol.close()
    out["fast_over_parity"] = out["fast"]["value"] / out["parity"]["value"]
    if cpu:
        import oracle
        oracle.build(ref=False)
        o = oracle.Oracle()
        threads = os.cpu_count() or 1
        o.set_threads(threads)
        cfg, s, u, b = problems.hancock_wind(N, M)
        grid = oracle.Grid(cfg.N, cfg.M, cfg.dx, cfg.dy, cfg.x0, cfg.y0, cfg.gamma, cfg.krit,
                           physics=cfg.physics, geometry=cfg.geometry, order=cfg.order,
                           method=cfg.method, bc=tuple(cfg.bc),
                           frozen_radius=cfg.frozen_radius, scheme=cfg.scheme,
                           x_max=cfg.x_max, y_max=cfg.y_max)
        T_do = o.dt_only(grid, s, u, b)
        t0 = time.perf_counter()
        o.run(grid, s, u, b, cpu_steps, T_do)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": N * M * cpu_steps / dt, "unit": "cell-updates/s",
                               "cores": threads, "kind": "port",
                               "sample": f"{cpu_steps} full step(s) of the workload on "
                                         f"{threads} host threads, oracle/gd_oracle.c "
                                         f"(restatement of Kernel_GKR), {dt:.2f} s"}
    return out


def cpu_baseline(workload, cfg, s, u, b, nsteps=24, threads=None):
    """The oracle on all host cores, `nsteps` full steps of the workload (about 10 s of CPU
    work for Kelvin-Helmholtz 4096^2 on 16 cores)."""
    import oracle
    oracle.build(ref=False)
    o = oracle.Oracle()
    threads = threads or os.cpu_count() or 1
    o.set_threads(threads)
    grid = oracle.Grid(cfg.N, cfg.M, cfg.dx, cfg.dy, cfg.x0, cfg.y0, cfg.gamma, cfg.krit,
                       physics=cfg.physics, geometry=cfg.geometry, order=cfg.order,
                       method=cfg.method, bc=tuple(cfg.bc), frozen_radius=cfg.frozen_radius)
    T_do = o.dt_only(grid, s, u, b)
    t0 = time.perf_counter()
    o.run(grid, s, u, b, nsteps, T_do)
    dt = time.perf_counter() - t0
    return {"value": cfg.N * cfg.M * nsteps / dt, "unit": "cell-updates/s", "cores": threads,
            "kind": "port",
            "sample": f"{nsteps} full steps of {workload} ({cfg.N}x{cfg.M}) on {threads} host "
                      f"threads, oracle/gd_oracle.c -O3 OpenMP, {dt:.2f} s"}


def workload_config(workload, cfg, ws):
    """The `config` object of both arms' lines: the same workload, the same dict."""
    K = cfg.N * cfg.M
    state_bytes = K * cfg.nfields * 8
    flush_l2 = 2 * state_bytes <= 2 * L2_BYTES
    return {"workload": WORKLOADS[workload], "cells": K, "fields": cfg.nfields,
            "parallelism": "replicas" if ws > 1 else "single",
            "l2": "flushed before every timed step" if flush_l2 else
                  f"state {2 * state_bytes / 2**20:.0f} MiB > L2 (129 MiB), no flush",
            "steps_per_launch": 1, "dt": "lagged reference protocol, dt-only pre-pass"}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    cfg, s, u, b = make_problem(args.workload)
    import oracle
    oracle.build(ref=False)
    o = oracle.Oracle()
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    grid = oracle.Grid(cfg.N, cfg.M, cfg.dx, cfg.dy, cfg.x0, cfg.y0, cfg.gamma, cfg.krit,
                       physics=cfg.physics, geometry=cfg.geometry, order=cfg.order,
                       method=cfg.method, bc=tuple(cfg.bc), frozen_radius=cfg.frozen_radius)
    T_do = o.dt_only(grid, s, u, b)
    # Each step is one full step of the workload; bounded so the run ends in minutes.
    s, u, b, T_do, _ = o.run(grid, s, u, b, args.warmup, T_do)
    t0 = time.perf_counter()
    o.run(grid, s, u, b, args.steps, T_do)
    dt = time.perf_counter() - t0
    K = cfg.N * cfg.M
    value = K * args.steps / dt
    line = {
        "impl": "reference", "metric": "FP64 cell-updates/s", "value": value,
        "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, cfg, ws),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{args.steps} full steps of {args.workload} after "
                                   f"{args.warmup} warm-up steps, oracle/gd_oracle.c -O3 "
                                   f"(restatement of the reference step, bit-identical to "
                                   f"it) on {threads} threads"},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_e2e(g, torch, cfg, s, u, b, steps=10):
    """gd_step_host per step from and to pinned host buffers, host clock, after one call."""
    sol = g.Solver(cfg)
    hs, hu = torch.from_numpy(s).pin_memory(), torch.from_numpy(u).pin_memory()
    hb = torch.from_numpy(b).pin_memory() if b is not None else None
    hs2, hu2 = torch.empty_like(hs).pin_memory(), torch.empty_like(hu).pin_memory()
    hb2 = torch.empty_like(hb).pin_memory() if hb is not None else None
    sol.import_state(hs, hu, hb)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    for _ in range(2):  # warm-up: the step graphs of both plane sets are captured
        sol.step_host(hs, hu, hb, hs2, hu2, hb2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sol.step_host(hs, hu, hb, hs2, hu2, hb2)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sol.close()
    K = cfg.N * cfg.M
    io = K * (4 + (3 if b is not None else 0)) * 8
    return {"value": K * steps / dt, "unit": "cell-updates/s", "h2d_bytes_per_step": io,
            "d2h_bytes_per_step": io, "path": "gd_step_host"}


def time_workload(name, steps, warmup, torch, g, flush_l2):
    """Device-resident timing of `steps` steps; returns (ms per step, launches)."""
    cfg, s, u, b = make_problem(name)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(warmup)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda") if flush_l2 else None
    l0 = sol.launch_count()
    if flush_l2:
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, z in evs:
            flush.fill_(1.0)
            a.record(stream)
            sol.advance(1)
            z.record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(z) for a, z in evs) / steps
    else:
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        sol.advance(steps)
        z.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(z) / steps
    launches = sol.launch_count() - l0
    st = sol.stats(allow_nonfinite=True)
    sol.close()
    return cfg, ms, launches, st


def run_gb300(args):
    import torch
    import golikov_2d_gb300 as g
    from golikov_2d_gb300 import _build

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    _build.build()
    g.load()

    cfg, s, u, b = make_problem(args.workload)
    K = cfg.N * cfg.M
    state_bytes = K * cfg.nfields * 8
    flush_l2 = 2 * state_bytes <= 2 * L2_BYTES  # both ping-pong buffers could sit in L2

    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(0.0, 0.0)
    sol.init_dt()
    sol.advance(args.warmup)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    bus = None
    try:
        props = torch.cuda.get_device_properties(local)
        bus = f"{props.pci_domain_id:08X}:{props.pci_bus_id:02X}:{props.pci_device_id:02X}.0"
    except Exception:
        bus = None

    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = sol.launch_count()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda") if flush_l2 else None
    with ClockSampler(bus) as clk:
        if flush_l2:
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
            for a, z in evs:
                flush.fill_(1.0)
                a.record(stream)
                sol.advance(1)
                z.record(stream)
            torch.cuda.synchronize()
            ms_total = sum(a.elapsed_time(z) for a, z in evs)
        else:
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sol.advance(args.steps)
            z.record(stream)
            torch.cuda.synchronize()
            ms_total = a.elapsed_time(z)
    launches = sol.launch_count() - l0
    ms_total, job_cells = job_aggregate(ms_total, K * args.steps, "cuda")
    stats = sol.stats(allow_nonfinite=True)
    ms_step = ms_total / args.steps
    value = job_cells / (ms_total * 1e-3)

    # ---- e2e: host buffers through the C ABI, copies inside the timed region ---------------
    hs = torch.from_numpy(s).pin_memory()
    hu = torch.from_numpy(u).pin_memory()
    hb = torch.from_numpy(b).pin_memory() if b is not None else None
    hs2, hu2 = torch.empty_like(hs).pin_memory(), torch.empty_like(hu).pin_memory()
    hb2 = torch.empty_like(hb).pin_memory() if hb is not None else None
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(2):  # warm-up: the step graphs of both plane sets are captured
        sol.step_host(hs, hu, hb, hs2, hu2, hb2)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # state up from pinned host memory, one step, result down: gd_step_host overlaps
        # the two copy directions with the step band by band; returns with the result on
        # the host
        sol.step_host(hs, hu, hb, hs2, hu2, hb2)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s, e2e_cells = job_aggregate(e2e_s, K * e2e_steps, "cuda")
    io_bytes = K * (4 + (3 if b is not None else 0)) * 8
    e2e = {"value": e2e_cells / e2e_s, "unit": "cell-updates/s",
           "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
           "path": "gd_step_host per step: host (pinned) -> device -> step -> host, bands of "
                   "tile rows overlapping the uploads, the step and the downloads"}
    sol.close()

    if rank != 0:
        return 0

    peak_gbs, peak_kind = measured_peaks()
    alg_bytes = K * bytes_per_cell(cfg)
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload)
    clocks = clk.summary()
    fp64 = fp64_roofline(g, args.workload, K / (ms_step * 1e-3), torch, clocks["sm_mhz"])
    line = {
        "metric": "FP64 cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(args.workload, cfg, ws),
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": achieved / peak_gbs,
                     "traffic": traffic, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "note": "FP64-issue bound on GB300; see fp64"},
        "fp64": fp64,
        "clocks": clocks,
        "e2e": e2e,
        "sim": {"t": stats.t, "dt": stats.dt, "steps": stats.steps,
                "rho_floor_hits": stats.rho_floor_hits, "p_floor_hits": stats.p_floor_hits,
                "nonfinite": stats.nonfinite},
    }
    if args.secondary and args.workload != "ot1024":
        try:
            with ClockSampler(bus) as clk2:
                c2, ms2, l2, st2 = time_workload("ot1024", args.steps, args.warmup, torch, g,
                                                 True)
            clocks2 = clk2.summary()
            K2 = c2.N * c2.M
            ach2 = K2 * bytes_per_cell(c2) / (ms2 * 1e-3) / 1e9
            line["secondary"] = {"workload": WORKLOADS["ot1024"], "value": K2 / (ms2 * 1e-3),
                                 "unit": "cell-updates/s", "ms_per_step": ms2,
                                 "roofline": {"bound": "hbm", "achieved": ach2, "peak": peak_gbs,
                                              "unit": "GB/s", "frac": ach2 / peak_gbs,
                                              "traffic": ncu_traffic("ot1024"),
                                              "l2_hit_pct": ncu_l2_hit_pct("ot1024")},
                                 "fp64": fp64_roofline(g, "ot1024", K2 / (ms2 * 1e-3), torch,
                                                       clocks2["sm_mhz"]),
                                 "clocks": clocks2,
                                 "l2": "flushed before every timed step",
                                 "gpu_launches": l2,
                                 "e2e": measure_e2e(g, torch, *make_problem("ot1024"))}
        except Exception as e:  # reported in the line instead of failing the whole run
            line["secondary"] = {"workload": WORKLOADS["ot1024"], "unavailable": str(e)}
    if args.secondary:
        try:
            line["ot_to_t05"] = measure_ot_to_end(g, torch)
        except Exception as e:
            line["ot_to_t05"] = {"unavailable": str(e)}
    if args.batched:
        try:
            line["batched"] = measure_batched(g, torch, 100)  # the workload's 100 steps
        except Exception as e:
            line["batched"] = {"unavailable": str(e)}
    if args.adjoint:
        try:
            line["adjoint"] = measure_adjoint(g, torch)
            line["adjoint"]["euler"] = measure_adjoint_euler(g, torch)
        except Exception as e:
            line["adjoint"] = {"unavailable": str(e)}
    if args.io:
        try:
            line["io"] = measure_io(g, torch)
        except Exception as e:
            line["io"] = {"unavailable": str(e)}
    if args.hancock:
        try:
            line["hancock"] = measure_hancock(g, torch, cpu=not args.no_cpu_baseline)
        except Exception as e:
            line["hancock"] = {"unavailable": str(e)}
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"] = cpu_baseline(args.workload, cfg, s, u, b)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="kh4096", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--secondary", type=int, default=1)
    ap.add_argument("--batched", type=int, default=1)
    ap.add_argument("--adjoint", type=int, default=1)
    ap.add_argument("--io", type=int, default=1)
    ap.add_argument("--hancock", type=int, default=1)
    ap.add_argument("--case", default="bench",
                    choices=["bench", "adjoint-step", "adjoint-step-euler", "io", "hancock",
                             "batch-step"],
                    help="adjoint-step (-euler): a short differentiation run of the MHD (Euler) "
                         "step for kernel profiles; batch-step: the batched workload's "
                         "persistent steps for kernel profiles; "
                         "io: the state-file measurement alone; hancock: the MUSCL-Hancock "
                         "measurement alone")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.case == "adjoint-step":
        import torch
        import golikov_2d_gb300 as g
        return adjoint_step_case(g, torch)
    if args.case == "batch-step":
        import torch
        import golikov_2d_gb300 as g
        from golikov_2d_gb300 import _build
        _build.build()
        return batch_step_case(g, torch)
    if args.case == "adjoint-step-euler":
        import torch
        import golikov_2d_gb300 as g
        return adjoint_step_euler_case(g, torch)
    if args.case == "io":
        import torch
        import golikov_2d_gb300 as g
        print(json.dumps({"case": "io", "io": measure_io(g, torch)}), flush=True)
        return 0
    if args.case == "hancock":
        import torch
        import golikov_2d_gb300 as g
        from golikov_2d_gb300 import _build
        _build.build()
        print(json.dumps({"case": "hancock",
                          "hancock": measure_hancock(g, torch, steps=args.steps,
                                                     warmup=args.warmup,
                                                     cpu=not args.no_cpu_baseline)}),
              flush=True)
        return 0
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
