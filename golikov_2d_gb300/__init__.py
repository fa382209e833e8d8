"""golikov_2d_gb300 -- GB300-native finite-volume step for 2-D Euler and ideal MHD.

Python mirror of the C ABI in ``include/gd2d.h`` (ctypes over ``libgd2d.so``).  The
reference's interface for this path is its kernel launch protocol (kernel.cu main()):

    Kernel_TVD<<<K/256, 256>>>(s, u, b, s2, u2, b2, T, T_do, i, method)   # one step
    funk_time<<<1, 1>>>(T, T_do, TT, i)                                   # dt rotation

``kernel_step`` and ``funk_time`` below keep those names' argument roles and take CUDA
tensors (device pointers) in the reference's AoS layout.  ``Solver`` wraps the resident
state (import / advance / export) used by the benchmark.

The CUDA library is required: importing works without a GPU, but every compute call
raises if ``libgd2d.so`` is missing or no CUDA device is present.  There is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgd2d.so")

EULER, MHD = 0, 1
CARTESIAN, AXISYM = 0, 1
METHOD_HLL, METHOD_HLLC, METHOD_HLLC_MHD, METHOD_HLLD = 0, 1, 2, 3
METHOD_CONFIG = -1  # per-call method argument: the context's configured method
(BC_PERIODIC, BC_TRANSMISSIVE, BC_MIRROR_X, BC_AXIS, BC_AMBIENT, BC_OUTFLOW,
 BC_AMBIENT_KEEPB) = range(7)
# spatial scheme: minmod TVD / first order (Kernel_TVD, add2, Ker_Dekard), or the
# MUSCL-Hancock predictor-corrector of Kernel_GKR as written (v_y slopes from the
# pressures) or with v_y slopes from v_y
SCHEME_TVD, SCHEME_HANCOCK_REF, SCHEME_HANCOCK = 0, 1, 2
# the only setting Kernel_GKR is written for: left, right, bottom, top
HANCOCK_BC = (BC_MIRROR_X, BC_OUTFLOW, BC_AXIS, BC_AMBIENT_KEEPB)
MODE_FAST, MODE_PARITY = 0, 1
DT_LAGGED, DT_CURRENT = 0, 1  # gd_set_dt_policy

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "non-finite state",
          4: "device wait timed out", 5: "unsupported combination"}

# Every symbol include/gd2d.h declares (checked by the tests against the built library).
EXPORTS = (
    "gd_create", "gd_destroy", "gd_get_config", "gd_status_string", "gd_last_cuda_error",
    "gd_abi_version", "gd_step_ref", "gd_funk_time", "gd_import", "gd_export", "gd_set_time",
    "gd_init_dt", "gd_advance", "gd_get_stats", "gd_field_ptr", "gd_launch_count",
    "gd_set_dt_policy", "gd_advance_to", "gd_step_host", "gd_set_floor_limit",
    "gd_probe_fp64_peak", "gd_probe_faces", "gd_step_ref_static", "gd_alloc_counts",
    "gd_check_int_mul", "gd_check_fast_roots",
    "gd_batch_create", "gd_batch_destroy", "gd_batch_import", "gd_batch_export",
    "gd_batch_set_time", "gd_batch_init_dt", "gd_batch_advance", "gd_batch_autotune",
    "gd_batch_get_stats", "gd_batch_get_info", "gd_batch_launch_count",
    "gd_adj_forward", "gd_adj_backward", "gd_tangent", "gd_adj_replay", "gd_adj_switches",
    "gd_format_text", "gd_write_text", "gd_parse_text", "gd_read_text", "gd_write_binary",
    "gd_read_binary", "gd_format_tecplot", "gd_write_tecplot",
)
BATCH_PERSISTENT, BATCH_LOOPED, BATCH_LOOPED_SYNC = 0, 1, 2


class GdError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {STATUS.get(status, status)} (status {status})")
        self.status = status


class gd_config(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("M", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("x0", ctypes.c_double), ("y0", ctypes.c_double),
        ("gamma", ctypes.c_double), ("krit", ctypes.c_double),
        ("physics", ctypes.c_int), ("geometry", ctypes.c_int),
        ("order", ctypes.c_int), ("method", ctypes.c_int),
        ("bc", ctypes.c_int * 4),
        ("frozen_radius", ctypes.c_double),
        ("mode", ctypes.c_int),
        ("scheme", ctypes.c_int),
        ("x_max", ctypes.c_double), ("y_max", ctypes.c_double),
    ]


class gd_batch_info(ctypes.Structure):
    _fields_ = [
        ("ngrids", ctypes.c_int), ("total_cells", ctypes.c_longlong),
        ("tile_x", ctypes.c_int), ("tile_y", ctypes.c_int), ("ctas", ctypes.c_int),
        ("tiles", ctypes.c_longlong), ("tuned_ms", ctypes.c_double * 4),
    ]


class gd_stats(ctypes.Structure):
    _fields_ = [
        ("t", ctypes.c_double), ("dt", ctypes.c_double), ("dt_next", ctypes.c_double),
        ("steps", ctypes.c_longlong), ("rho_floor_hits", ctypes.c_longlong),
        ("p_floor_hits", ctypes.c_longlong), ("nonfinite", ctypes.c_longlong),
        ("t_state", ctypes.c_double),
    ]


class gd_tecplot_opts(ctypes.Structure):
    _fields_ = [("nmin", ctypes.c_int), ("x_min", ctypes.c_double), ("x_max", ctypes.c_double),
                ("y_min", ctypes.c_double), ("y_max", ctypes.c_double),
                ("with_time", ctypes.c_int), ("time", ctypes.c_double)]


_lib = None


def lib_path() -> str:
    return LIB_PATH


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libgd2d.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with golikov_2d_gb300._build.build() "
                           "(there is no CPU fallback)")
    L = ctypes.CDLL(path)
    vp, i, d, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    cfgp = ctypes.POINTER(gd_config)
    L.gd_create.argtypes = [cfgp, ctypes.POINTER(vp)]
    L.gd_destroy.argtypes = [vp]
    L.gd_get_config.argtypes = [vp, cfgp]
    L.gd_status_string.restype = ctypes.c_char_p
    L.gd_status_string.argtypes = [i]
    L.gd_step_ref.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, i, i, vp]
    L.gd_funk_time.argtypes = [vp, vp, vp, vp, vp, vp]
    L.gd_import.argtypes = [vp, vp, vp, vp, i, vp]
    L.gd_export.argtypes = [vp, vp, vp, vp, i, vp]
    L.gd_set_time.argtypes = [vp, d, d, vp]
    L.gd_init_dt.argtypes = [vp, vp]
    L.gd_advance.argtypes = [vp, i, i, vp]
    L.gd_set_dt_policy.argtypes = [vp, i]
    L.gd_set_floor_limit.argtypes = [vp, ll]
    L.gd_step_host.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.gd_advance_to.argtypes = [vp, d, ll, i, ctypes.POINTER(ll), vp]
    L.gd_get_stats.argtypes = [vp, ctypes.POINTER(gd_stats), vp]
    L.gd_field_ptr.argtypes = [vp, i, ctypes.POINTER(vp)]
    L.gd_launch_count.restype = ll
    L.gd_launch_count.argtypes = [vp]
    L.gd_probe_fp64_peak.argtypes = [ctypes.POINTER(d)]
    L.gd_probe_faces.argtypes = [i, i, d, i, ll, vp, vp, vp, vp, vp]
    L.gd_step_ref_static.argtypes = [cfgp, vp, vp, vp, vp, vp, vp, vp, vp, i, vp]
    L.gd_alloc_counts.argtypes = [ctypes.POINTER(ll), ctypes.POINTER(ll)]
    L.gd_check_int_mul.argtypes = [ll, ctypes.c_ulonglong, ctypes.POINTER(ll)]
    L.gd_check_fast_roots.argtypes = [ll, ctypes.c_ulonglong, ctypes.POINTER(ll)]
    L.gd_adj_forward.argtypes = [vp, i, i, vp]
    for name in ("gd_adj_backward", "gd_tangent", "gd_adj_replay"):
        getattr(L, name).argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.gd_adj_switches.argtypes = [vp] + [vp] * 12 + [ctypes.POINTER(ll), vp]
    sz = ctypes.c_size_t
    tecp = ctypes.POINTER(gd_tecplot_opts)
    L.gd_format_text.argtypes = [vp, vp, sz, ctypes.POINTER(sz), vp]
    L.gd_write_text.argtypes = [vp, ctypes.c_char_p, vp]
    L.gd_parse_text.argtypes = [vp, ctypes.c_char_p, sz, vp]
    L.gd_read_text.argtypes = [vp, ctypes.c_char_p, vp]
    L.gd_write_binary.argtypes = [vp, ctypes.c_char_p, vp]
    L.gd_read_binary.argtypes = [vp, ctypes.c_char_p, vp]
    L.gd_format_tecplot.argtypes = [vp, tecp, vp, sz, ctypes.POINTER(sz), vp]
    L.gd_write_tecplot.argtypes = [vp, ctypes.c_char_p, tecp, vp]
    L.gd_batch_create.argtypes = [cfgp, i, ctypes.POINTER(vp)]
    L.gd_batch_destroy.argtypes = [vp]
    L.gd_batch_import.argtypes = [vp, i, vp, vp, vp, i, vp]
    L.gd_batch_export.argtypes = [vp, i, vp, vp, vp, i, vp]
    L.gd_batch_set_time.argtypes = [vp, d, d, vp]
    L.gd_batch_init_dt.argtypes = [vp, vp]
    L.gd_batch_advance.argtypes = [vp, i, i, i, vp]
    L.gd_batch_autotune.argtypes = [vp, i, vp]
    L.gd_batch_get_stats.argtypes = [vp, i, ctypes.POINTER(gd_stats), vp]
    L.gd_batch_get_info.argtypes = [vp, ctypes.POINTER(gd_batch_info)]
    L.gd_batch_launch_count.restype = ll
    L.gd_batch_launch_count.argtypes = [vp]
    for name in ("gd_create", "gd_destroy", "gd_get_config", "gd_step_ref", "gd_funk_time",
                 "gd_import", "gd_export", "gd_set_time", "gd_init_dt", "gd_advance",
                 "gd_set_dt_policy", "gd_advance_to", "gd_step_host", "gd_set_floor_limit",
                 "gd_get_stats", "gd_field_ptr", "gd_probe_fp64_peak", "gd_probe_faces",
                 "gd_step_ref_static", "gd_alloc_counts", "gd_check_int_mul",
                 "gd_check_fast_roots",
                 "gd_batch_create", "gd_batch_destroy", "gd_batch_import", "gd_batch_export",
                 "gd_batch_set_time", "gd_batch_init_dt", "gd_batch_advance",
                 "gd_batch_autotune", "gd_batch_get_stats", "gd_batch_get_info",
                 "gd_adj_forward", "gd_adj_backward", "gd_tangent", "gd_adj_replay",
                 "gd_adj_switches", "gd_format_text", "gd_write_text", "gd_parse_text",
                 "gd_read_text",
                 "gd_write_binary", "gd_read_binary", "gd_format_tecplot", "gd_write_tecplot"):
        getattr(L, name).restype = i
    _lib = L
    return L


def _check(status: int, what: str) -> None:
    if status != 0:
        raise GdError(status, what)


def _stream_handle(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream or None
    return getattr(stream, "cuda_stream", stream) or None


@dataclass
class Config:
    """Grid, physics and boundaries (gd_config)."""
    N: int
    M: int
    dx: float
    dy: float
    x0: float
    y0: float
    gamma: float
    krit: float
    physics: int = EULER
    geometry: int = CARTESIAN
    order: int = 2
    method: int = METHOD_HLLC
    bc: tuple = (BC_TRANSMISSIVE,) * 4
    frozen_radius: float = 0.0
    mode: int = MODE_FAST
    scheme: int = SCHEME_TVD
    x_max: float = 0.0  # domain extents used by the Hancock schemes' cell coordinates
    y_max: float = 0.0

    def cstruct(self) -> gd_config:
        c = gd_config()
        for name, _ in gd_config._fields_:
            if name == "bc":
                for k in range(4):
                    c.bc[k] = int(self.bc[k])
            else:
                setattr(c, name, getattr(self, name))
        return c

    @property
    def nfields(self) -> int:
        return 7 if self.physics == MHD else 4


class Solver:
    """A context: resident state, dt scalars and the step kernels for one grid."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        self.lib = load()
        self._c = cfg.cstruct()
        h = ctypes.c_void_p()
        _check(self.lib.gd_create(ctypes.byref(self._c), ctypes.byref(h)), "gd_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.gd_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the reference's launch protocol (device pointers, AoS layout) ------------------------
    def kernel_step(self, s, u, b, s2, u2, b2, T, T_do, i=0, method=METHOD_CONFIG,
                    stream=None) -> None:
        """gd_step_ref: Kernel_TVD / add2 / Ker_Dekard on CUDA tensors; `method` is the
        reference's code (METHOD_*) or METHOD_CONFIG."""
        p = lambda t: None if t is None else t.data_ptr()
        _check(self.lib.gd_step_ref(self.handle, p(s), p(u), p(b), p(s2), p(u2), p(b2), p(T),
                                    p(T_do), int(i), int(method), _stream_handle(stream)),
               "gd_step_ref")

    def funk_time(self, T, T_do, TT, i, stream=None) -> None:
        _check(self.lib.gd_funk_time(self.handle, T.data_ptr(), T_do.data_ptr(), TT.data_ptr(),
                                     i.data_ptr(), _stream_handle(stream)), "gd_funk_time")

    # -- resident state ------------------------------------------------------------------------
    def import_state(self, s, u, b=None, stream=None) -> None:
        """Load AoS state from torch tensors (CPU or CUDA) or numpy arrays (host)."""
        host, ptrs = self._ptrs(s, u, b)
        _check(self.lib.gd_import(self.handle, *ptrs, 1 if host else 0, _stream_handle(stream)),
               "gd_import")

    def export_state(self, s, u, b=None, stream=None) -> None:
        host, ptrs = self._ptrs(s, u, b)
        _check(self.lib.gd_export(self.handle, *ptrs, 1 if host else 0, _stream_handle(stream)),
               "gd_export")

    @staticmethod
    def _ptrs(s, u, b):
        import numpy as np
        if isinstance(s, np.ndarray):
            arrs = [s, u, b]
            for a in arrs:
                if a is not None:
                    assert a.dtype == np.float64 and a.flags.c_contiguous
            return True, [None if a is None else a.ctypes.data for a in arrs]
        host = not s.is_cuda
        return host, [None if t is None else t.data_ptr() for t in (s, u, b)]

    def set_time(self, T_do: float, TT: float = 0.0, stream=None) -> None:
        _check(self.lib.gd_set_time(self.handle, float(T_do), float(TT), _stream_handle(stream)),
               "gd_set_time")

    def init_dt(self, stream=None) -> None:
        _check(self.lib.gd_init_dt(self.handle, _stream_handle(stream)), "gd_init_dt")

    def advance(self, nsteps: int, use_graph: bool = False, stream=None) -> None:
        _check(self.lib.gd_advance(self.handle, int(nsteps), 1 if use_graph else 0,
                                   _stream_handle(stream)), "gd_advance")

    def step_host(self, s, u, b, s2, u2, b2, stream=None) -> None:
        """gd_step_host: one step from host arrays (s, u, b) into host arrays (s2, u2, b2);
        torch CPU tensors in pinned memory take the overlapped path."""
        host, pin = self._ptrs(s, u, b)
        host2, pout = self._ptrs(s2, u2, b2)
        if not (host and host2):
            raise ValueError("step_host takes host arrays")
        _check(self.lib.gd_step_host(self.handle, *pin, *pout, _stream_handle(stream)),
               "gd_step_host")

    def set_floor_limit(self, max_floor_hits: int) -> None:
        """stats() reports GD_ERR_NONPHYSICAL once floor hits exceed this (0: no limit)."""
        _check(self.lib.gd_set_floor_limit(self.handle, int(max_floor_hits)),
               "gd_set_floor_limit")

    def set_dt_policy(self, policy: int) -> None:
        """DT_LAGGED (the reference's protocol) or DT_CURRENT (each step's own CFL dt)."""
        _check(self.lib.gd_set_dt_policy(self.handle, int(policy)), "gd_set_dt_policy")

    def advance_to(self, t_end: float, max_steps: int = 1 << 40, use_graph: bool = False,
                   stream=None) -> int:
        """Advance until the state's time reaches t_end (the last dt limited to land on it);
        returns the number of steps taken."""
        n = ctypes.c_longlong(0)
        _check(self.lib.gd_advance_to(self.handle, float(t_end), int(max_steps),
                                      1 if use_graph else 0, ctypes.byref(n),
                                      _stream_handle(stream)), "gd_advance_to")
        return int(n.value)

    def stats(self, stream=None, allow_nonfinite: bool = False) -> gd_stats:
        st = gd_stats()
        r = self.lib.gd_get_stats(self.handle, ctypes.byref(st), _stream_handle(stream))
        if not (r == 3 and allow_nonfinite):
            _check(r, "gd_get_stats")
        return st

    # -- differentiation (device tensors, reference AoS layout) --------------------------------
    def adj_forward(self, nsteps: int, ckpt_every: int, stream=None) -> None:
        _check(self.lib.gd_adj_forward(self.handle, int(nsteps), int(ckpt_every),
                                       _stream_handle(stream)), "gd_adj_forward")

    def _vec_call(self, fn, what, ins, outs, stream):
        ptr = lambda t: None if t is None else t.data_ptr()  # Euler: no field tensors
        p = [ptr(t) for t in ins] + [ptr(t) for t in outs]
        _check(fn(self.handle, *p, _stream_handle(stream)), what)

    def adj_backward(self, gs, gu, gb, os_, ou, ob, stream=None) -> None:
        self._vec_call(self.lib.gd_adj_backward, "gd_adj_backward", (gs, gu, gb), (os_, ou, ob),
                       stream)

    def tangent(self, vs, vu, vb, os_, ou, ob, stream=None) -> None:
        self._vec_call(self.lib.gd_tangent, "gd_tangent", (vs, vu, vb), (os_, ou, ob), stream)

    def adj_replay(self, s, u, b, os_, ou, ob, stream=None) -> None:
        self._vec_call(self.lib.gd_adj_replay, "gd_adj_replay", (s, u, b), (os_, ou, ob), stream)

    SWITCH_KINDS = ("minmod", "fallback", "speeds", "region", "guards", "floors",
                    "cell_steps", "cells")

    def adj_switches(self, Up, Um, Op, Om, stream=None) -> dict:
        """Replays the recorded map from Up and Um side by side into Op and Om (each a tuple
        (s, u, b) of device tensors) and returns the branch-switch counts between the two
        runs (gd_adj_switches), keyed by SWITCH_KINDS."""
        counts = (ctypes.c_longlong * 8)()
        p = [t.data_ptr() for t in (*Up, *Um, *Op, *Om)]
        _check(self.lib.gd_adj_switches(self.handle, *p, counts, _stream_handle(stream)),
               "gd_adj_switches")
        return dict(zip(self.SWITCH_KINDS, (int(c) for c in counts)))

    def field_ptr(self, f: int) -> int:
        p = ctypes.c_void_p()
        _check(self.lib.gd_field_ptr(self.handle, int(f), ctypes.byref(p)), "gd_field_ptr")
        return p.value

    def launch_count(self) -> int:
        return int(self.lib.gd_launch_count(self.handle))

    # -- state files (the reference's formats, made on the GPU) --------------------------------
    def _fetch(self, fn, what, *args, stream=None) -> bytes:
        n = ctypes.c_size_t(0)
        _check(fn(self.handle, *args, None, 0, ctypes.byref(n), _stream_handle(stream)), what)
        buf = ctypes.create_string_buffer(n.value)
        _check(fn(self.handle, *args, buf, n.value, ctypes.byref(n), _stream_handle(stream)),
               what)
        return buf.raw[:n.value]

    def format_text(self, stream=None) -> bytes:
        """The restart text of the resident state ("x y rho p vx vy Bx By Bz" per cell)."""
        return self._fetch(self.lib.gd_format_text, "gd_format_text", stream=stream)

    def write_text(self, path: str, stream=None) -> None:
        _check(self.lib.gd_write_text(self.handle, os.fsencode(path), _stream_handle(stream)),
               "gd_write_text")

    def parse_text(self, text: bytes, stream=None) -> None:
        _check(self.lib.gd_parse_text(self.handle, text, len(text), _stream_handle(stream)),
               "gd_parse_text")

    def read_text(self, path: str, stream=None) -> None:
        _check(self.lib.gd_read_text(self.handle, os.fsencode(path), _stream_handle(stream)),
               "gd_read_text")

    def write_binary(self, path: str, stream=None) -> None:
        _check(self.lib.gd_write_binary(self.handle, os.fsencode(path), _stream_handle(stream)),
               "gd_write_binary")

    def read_binary(self, path: str, stream=None) -> None:
        _check(self.lib.gd_read_binary(self.handle, os.fsencode(path), _stream_handle(stream)),
               "gd_read_binary")

    @staticmethod
    def tecplot_opts(nmin, x_min, x_max, y_min, y_max, time=None) -> gd_tecplot_opts:
        return gd_tecplot_opts(int(nmin), float(x_min), float(x_max), float(y_min),
                               float(y_max), 0 if time is None else 1,
                               0.0 if time is None else float(time))

    def format_tecplot(self, nmin, x_min, x_max, y_min, y_max, time=None, stream=None) -> bytes:
        o = self.tecplot_opts(nmin, x_min, x_max, y_min, y_max, time)
        return self._fetch(self.lib.gd_format_tecplot, "gd_format_tecplot", ctypes.byref(o),
                           stream=stream)

    def write_tecplot(self, path, nmin, x_min, x_max, y_min, y_max, time=None,
                      stream=None) -> None:
        o = self.tecplot_opts(nmin, x_min, x_max, y_min, y_max, time)
        _check(self.lib.gd_write_tecplot(self.handle, os.fsencode(path), ctypes.byref(o),
                                         _stream_handle(stream)), "gd_write_tecplot")


class Batch:
    """Many independent Euler grids advanced together (gd_batch_*)."""

    def __init__(self, cfgs):
        self.cfgs = list(cfgs)
        self.lib = load()
        arr = (gd_config * len(self.cfgs))(*[c.cstruct() for c in self.cfgs])
        self._arr = arr
        h = ctypes.c_void_p()
        _check(self.lib.gd_batch_create(arr, len(self.cfgs), ctypes.byref(h)), "gd_batch_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.gd_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def import_grid(self, g, s, u, stream=None) -> None:
        host, ptrs = Solver._ptrs(s, u, None)
        _check(self.lib.gd_batch_import(self.handle, int(g), ptrs[0], ptrs[1], None,
                                        1 if host else 0, _stream_handle(stream)),
               "gd_batch_import")

    def export_grid(self, g, s, u, stream=None) -> None:
        host, ptrs = Solver._ptrs(s, u, None)
        _check(self.lib.gd_batch_export(self.handle, int(g), ptrs[0], ptrs[1], None,
                                        1 if host else 0, _stream_handle(stream)),
               "gd_batch_export")

    def set_time(self, T_do, TT=0.0, stream=None) -> None:
        _check(self.lib.gd_batch_set_time(self.handle, float(T_do), float(TT),
                                          _stream_handle(stream)), "gd_batch_set_time")

    def init_dt(self, stream=None) -> None:
        _check(self.lib.gd_batch_init_dt(self.handle, _stream_handle(stream)), "gd_batch_init_dt")

    def advance(self, nsteps, schedule=BATCH_PERSISTENT, use_graph=False, stream=None) -> None:
        _check(self.lib.gd_batch_advance(self.handle, int(nsteps), int(schedule),
                                         1 if use_graph else 0, _stream_handle(stream)),
               "gd_batch_advance")

    def autotune(self, reps=3, stream=None) -> None:
        _check(self.lib.gd_batch_autotune(self.handle, int(reps), _stream_handle(stream)),
               "gd_batch_autotune")

    def stats(self, g, stream=None, allow_nonfinite=False) -> gd_stats:
        st = gd_stats()
        r = self.lib.gd_batch_get_stats(self.handle, int(g), ctypes.byref(st),
                                        _stream_handle(stream))
        if not (r == 3 and allow_nonfinite):
            _check(r, "gd_batch_get_stats")
        return st

    def info(self) -> gd_batch_info:
        inf = gd_batch_info()
        _check(self.lib.gd_batch_get_info(self.handle, ctypes.byref(inf)), "gd_batch_get_info")
        return inf

    def launch_count(self) -> int:
        return int(self.lib.gd_batch_launch_count(self.handle))


def probe_faces(physics: int, method: int, gamma: float, axis: int, L, R, stream=None):
    """gd_probe_faces: the fast step's face solver on n faces.  L, R: contiguous float64 CUDA
    tensors of shape (n, 4) for EULER or (n, 8) for MHD in the reference's face layouts;
    returns (flux, speed) CUDA tensors of shape (n, 4 | 8) and (n,)."""
    import torch
    n = int(L.shape[0])
    flux = torch.empty((n, L.shape[1]), dtype=torch.float64, device=L.device)
    speed = torch.empty(n, dtype=torch.float64, device=L.device)
    _check(load().gd_probe_faces(int(physics), int(method), float(gamma), int(axis), n,
                                 L.data_ptr(), R.data_ptr(), flux.data_ptr(), speed.data_ptr(),
                                 _stream_handle(stream)), "gd_probe_faces")
    return flux, speed


def probe_fp64_peak() -> float:
    """Measured FP64 FMA throughput of the current device in FLOP/s."""
    L = load()
    v = ctypes.c_double()
    _check(L.gd_probe_fp64_peak(ctypes.byref(v)), "gd_probe_fp64_peak")
    return v.value


def check_int_mul(pairs: int = 1 << 24, seed: int = 1) -> dict:
    """Device check of the step kernels' integer-pipe binary64 multiplication against the
    FP64 unit's multiply (gd_check_int_mul): mismatched results (NaN results excepted), NaN
    payload differences, pairs outside the integer fast path, pairs checked."""
    L = load()
    c = (ctypes.c_longlong * 4)()
    _check(L.gd_check_int_mul(int(pairs), int(seed), c), "gd_check_int_mul")
    return {"mismatches": c[0], "nan_payload": c[1], "slow_path": c[2], "checked": c[3]}


def check_fast_roots(count: int = 1 << 24, seed: int = 1) -> dict:
    """Largest errors, in units of the last place, of the step's two-operation reciprocal and
    root against IEEE division and square root (gd_check_fast_roots)."""
    L = load()
    c = (ctypes.c_longlong * 4)()
    _check(L.gd_check_fast_roots(int(count), int(seed), c), "gd_check_fast_roots")
    return {"rcp_2op_ulp": c[0], "sqrt_over_2op_ulp": c[1], "sqrt_over_ulp": c[2],
            "checked": c[3]}


def alloc_counts() -> tuple[int, int]:
    """(allocations, releases) of device and pinned-host memory the library has made in
    this process (gd_alloc_counts)."""
    L = load()
    a, f = ctypes.c_longlong(), ctypes.c_longlong()
    _check(L.gd_alloc_counts(ctypes.byref(a), ctypes.byref(f)), "gd_alloc_counts")
    return a.value, f.value
