"""ctypes bindings for the oracle (TEST INFRASTRUCTURE ONLY).

Two libraries live here:

* ``_build/libgd_oracle.so`` -- the project's C restatement of the reference step
  (``gd_oracle.c``).  Built everywhere by ``make -C oracle``; it is the oracle the tests
  compare against and the timed CPU baseline in ``bench.py``.
* ``_ref/libgdref.so`` -- the reference's own ``Gas_Dinamic.cu`` / ``kernel.cu`` compiled
  for the host (``ref_build/Makefile``).  It exists only where the reference sources are
  present; tests that need it skip elsewhere.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import
this package.  The product package never does.

State arrays use the reference's AoS layout (kernel.cu:3814-3825): ``s`` = (K, 2) {rho, p},
``u`` = (K, 2) {vx, vy}, ``b`` = (K, 3) {Bx, By, Bz}; cell k = m*N + n.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libgd_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libgdref.so")
# The reference checkout is located by this environment variable; without it the reference
# library is not built, and the tests that need it skip.
REF_SRC_ENV = "GD_REFERENCE_SRC"


def ref_src() -> str | None:
    """The reference sources' directory, if GD_REFERENCE_SRC names one that exists."""
    p = os.environ.get(REF_SRC_ENV)
    return p if p and os.path.isdir(p) else None

EULER, MHD = 0, 1
CARTESIAN, AXISYM = 0, 1
BC_PERIODIC, BC_TRANSMISSIVE, BC_MIRROR_X, BC_AXIS, BC_AMBIENT, BC_OUTFLOW, BC_AMBIENT_KEEPB = range(7)

_d = ctypes.c_double
_i = ctypes.c_int
_pd = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_pd)


class OracleConfig(ctypes.Structure):
    _fields_ = [
        ("N", _i), ("M", _i),
        ("dx", _d), ("dy", _d), ("x0", _d), ("y0", _d),
        ("gamma", _d), ("krit", _d),
        ("physics", _i), ("geometry", _i), ("order", _i), ("method", _i),
        ("bc", _i * 4),
        ("frozen_radius", _d),
        ("scheme", _i), ("x_max", _d), ("y_max", _d),
    ]


def build(ref: bool | None = None, src: str | None = None) -> None:
    """Compile the oracle; also the reference library when its sources are given.

    `src` is the reference checkout (default: GD_REFERENCE_SRC).  ref=None builds the
    reference library when that directory exists, ref=True requires it."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if src is None:
        src = ref_src()
    if ref is None:
        ref = src is not None and os.path.isdir(src)
    if ref:
        if src is None or not os.path.isdir(src):
            raise FileNotFoundError(f"reference sources not found: set {REF_SRC_ENV}")
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_build"), f"REF={src}"],
                       check=True)


@dataclass
class Grid:
    """A problem description shared by the oracle and the tests."""
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
    method: int = 1
    bc: tuple = (BC_TRANSMISSIVE,) * 4
    frozen_radius: float = 0.0
    scheme: int = 0
    x_max: float = 0.0
    y_max: float = 0.0

    def cstruct(self) -> OracleConfig:
        c = OracleConfig()
        c.N, c.M = self.N, self.M
        c.dx, c.dy, c.x0, c.y0 = self.dx, self.dy, self.x0, self.y0
        c.gamma, c.krit = self.gamma, self.krit
        c.physics, c.geometry, c.order, c.method = self.physics, self.geometry, self.order, self.method
        for k in range(4):
            c.bc[k] = self.bc[k]
        c.frozen_radius = self.frozen_radius
        c.scheme, c.x_max, c.y_max = self.scheme, self.x_max, self.y_max
        return c


class Oracle:
    """The C restatement (gd_oracle.c)."""

    def __init__(self, path: str = ORACLE_LIB):
        if not os.path.exists(path):
            build(ref=False)
        L = ctypes.CDLL(path)
        L.gdo_minmod.restype = _d
        L.gdo_minmod.argtypes = [_d, _d]
        L.gdo_linear.restype = _d
        L.gdo_linear.argtypes = [_d] * 7
        L.gdo_linear2.restype = None
        L.gdo_linear2.argtypes = [_d] * 8 + [_pd, _pd]
        for name in ("gdo_hllc", "gdo_hll"):
            getattr(L, name).restype = _d
            getattr(L, name).argtypes = [_pd, _pd, _d, _d, _d, _d, _d, _pd]
        L.gdo_hlld.restype = _d
        L.gdo_hlld.argtypes = [_pd, _pd, _d, _d, _d, _d, _i, _d, _d, _pd]
        L.gdo_step.restype = _d
        L.gdo_step.argtypes = [ctypes.POINTER(OracleConfig), _pd, _pd, _pd, _pd, _pd, _pd, _d, _d, _i]
        L.gdo_set_threads.restype = _i
        L.gdo_set_threads.argtypes = [_i]
        cp = ctypes.POINTER(OracleConfig)
        for name in ("gdo_write_restart", "gdo_write_binary"):
            getattr(L, name).restype = _i
            getattr(L, name).argtypes = [cp, _pd, _pd, _pd, ctypes.c_char_p]
        L.gdo_read_restart.restype = _i
        L.gdo_read_restart.argtypes = [cp, ctypes.c_char_p, _pd, _pd, _pd]
        L.gdo_write_tecplot.restype = _i
        L.gdo_write_tecplot.argtypes = [cp, _pd, _pd, _pd, _i, _d, _d, _d, _d, _i, _d,
                                        ctypes.c_char_p]
        self.lib = L

    def set_threads(self, n: int) -> int:
        return self.lib.gdo_set_threads(n)

    # state files (the reference's writers restated with C stdio)
    def write_restart(self, g: Grid, s, u, b, path) -> None:
        c = g.cstruct()
        args = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (s, u, b)]
        if self.lib.gdo_write_restart(ctypes.byref(c), *[_ptr(a) for a in args],
                                      os.fsencode(path)):
            raise OSError(path)

    def read_restart(self, g: Grid, path, mhd=True):
        """Returns (s, u, b) read from a restart text (b None unless mhd)."""
        c = g.cstruct()
        K = g.N * g.M
        s, u = np.zeros((K, 2)), np.zeros((K, 2))
        b = np.zeros((K, 3)) if mhd else None
        if self.lib.gdo_read_restart(ctypes.byref(c), os.fsencode(path), _ptr(s), _ptr(u),
                                     _ptr(b)):
            raise OSError(path)
        return s, u, b

    def write_binary(self, g: Grid, s, u, b, path) -> None:
        c = g.cstruct()
        args = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (s, u, b)]
        if self.lib.gdo_write_binary(ctypes.byref(c), *[_ptr(a) for a in args],
                                     os.fsencode(path)):
            raise OSError(path)

    def write_tecplot(self, g: Grid, s, u, b, nmin, x_min, x_max, y_min, y_max, path,
                      time=None) -> None:
        c = g.cstruct()
        args = [np.ascontiguousarray(a, np.float64) if a is not None else None for a in (s, u, b)]
        if self.lib.gdo_write_tecplot(ctypes.byref(c), *[_ptr(a) for a in args], int(nmin),
                                      x_min, x_max, y_min, y_max, 0 if time is None else 1,
                                      0.0 if time is None else float(time), os.fsencode(path)):
            raise OSError(path)

    def minmod(self, a, b):
        return self.lib.gdo_minmod(a, b)

    def hllc(self, L, R, n1, n2, rad, gamma, krit):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(4)
        t = self.lib.gdo_hllc(_ptr(L), _ptr(R), n1, n2, rad, gamma, krit, _ptr(out))
        return t, out

    def hll(self, L, R, n1, n2, rad, gamma, krit):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(4)
        t = self.lib.gdo_hll(_ptr(L), _ptr(R), n1, n2, rad, gamma, krit, _ptr(out))
        return t, out

    def hlld(self, L, R, n1, n2, n3, rad, method, gamma, krit):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(8)
        t = self.lib.gdo_hlld(_ptr(L), _ptr(R), n1, n2, n3, rad, method, gamma, krit, _ptr(out))
        return t, out

    def step(self, g: Grid, s, u, b, T_do: float, T_in: float = 1e7, dt_only: bool = False,
             out=None):
        """One step.  Returns (s2, u2, b2, T)."""
        K = g.N * g.M
        s = np.ascontiguousarray(s, np.float64).reshape(K, 2)
        u = np.ascontiguousarray(u, np.float64).reshape(K, 2)
        b = None if b is None else np.ascontiguousarray(b, np.float64).reshape(K, 3)
        if out is None:
            s2, u2 = s.copy(), u.copy()
            b2 = None if b is None else b.copy()
        else:
            s2, u2, b2 = out
        c = g.cstruct()
        T = self.lib.gdo_step(ctypes.byref(c), _ptr(s), _ptr(u), _ptr(b), _ptr(s2), _ptr(u2),
                              _ptr(b2), T_do, T_in, 1 if dt_only else 0)
        return s2, u2, b2, T

    def dt_only(self, g: Grid, s, u, b) -> float:
        return self.step(g, s, u, b, 0.0, 1e7, dt_only=True)[3]

    def run(self, g: Grid, s, u, b, nsteps: int, T_do: float, TT: float = 0.0):
        """nsteps steps of the reference protocol (kernel.cu:4110-4127): step with T_do,
        then funk_time (T_do <- T, TT += T_do, T <- 1e7).  Returns (s, u, b, T_do, TT)."""
        s = np.ascontiguousarray(s, np.float64).copy()
        u = np.ascontiguousarray(u, np.float64).copy()
        b = None if b is None else np.ascontiguousarray(b, np.float64).copy()
        s2, u2 = s.copy(), u.copy()
        b2 = None if b is None else b.copy()
        for _ in range(nsteps):
            _, _, _, T = self.step(g, s, u, b, T_do, 1e7, out=(s2, u2, b2))
            s, s2 = s2, s
            u, u2 = u2, u
            if b is not None:
                b, b2 = b2, b
            T_do = T
            TT += T_do
        return s, u, b, T_do, TT


class Reference:
    """The reference's own functions compiled for the host (oracle/_ref/libgdref.so)."""

    def __init__(self, path: str = REF_LIB):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        L.gdref_set_params.argtypes = [_d, _d, _i, _i, _d, _d]
        L.gdref_set_threads.restype = _i
        L.gdref_set_threads.argtypes = [_i]
        L.gdref_minmod.restype = _d
        L.gdref_minmod.argtypes = [_d, _d]
        L.gdref_linear.restype = _d
        L.gdref_linear.argtypes = [_d] * 7
        L.gdref_linear2.argtypes = [_d] * 8 + [_pd, _pd]
        for name in ("gdref_hllc", "gdref_hll"):
            getattr(L, name).restype = _d
            getattr(L, name).argtypes = [_pd, _pd, _d, _d, _d, _pd]
        L.gdref_hlld.restype = _d
        L.gdref_hlld.argtypes = [_pd, _pd, _d, _d, _d, _d, _i, _pd]
        for name in ("gdref_kernel_tvd", "gdref_add2", "gdref_kernel_gkr"):
            getattr(L, name).argtypes = [_pd, _pd, _pd, _pd, _pd, _pd, _pd, _d, _i, _i]
        for name in ("gdref_ker_dekard", "gdref_kernel_tvd_old"):
            getattr(L, name).argtypes = [_pd, _pd, _pd, _pd, _pd, _d, _i]
        L.gdref_print_tecplot.argtypes = [_pd, _pd, _pd, _i, _d, ctypes.c_char_p]
        L.gdref_write_restart.argtypes = [_pd, _pd, _pd, ctypes.c_char_p]
        self.lib = L

    @staticmethod
    def available(path: str = REF_LIB) -> bool:
        return os.path.exists(path)

    def set_params(self, gamma, krit, N=3226, M=1792, xmax=9.0, ymax=5.0):
        self.lib.gdref_set_params(gamma, krit, N, M, xmax, ymax)

    def hllc(self, L, R, n1, n2, rad):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(4)
        t = self.lib.gdref_hllc(_ptr(L), _ptr(R), n1, n2, rad, _ptr(out))
        return t, out

    def hll(self, L, R, n1, n2, rad):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(4)
        t = self.lib.gdref_hll(_ptr(L), _ptr(R), n1, n2, rad, _ptr(out))
        return t, out

    def hlld(self, L, R, n1, n2, n3, rad, method):
        L = np.ascontiguousarray(L, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        out = np.zeros(8)
        t = self.lib.gdref_hlld(_ptr(L), _ptr(R), n1, n2, n3, rad, method, _ptr(out))
        return t, out

    def _mhd_kernel(self, fn, s, u, b, T_do, i, method, out=None):
        s = np.ascontiguousarray(s, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        s2, u2, b2 = (s.copy(), u.copy(), b.copy()) if out is None else out
        T = np.array([1e7])
        fn(_ptr(s), _ptr(u), _ptr(b), _ptr(s2), _ptr(u2), _ptr(b2), _ptr(T), T_do, i, method)
        return s2, u2, b2, float(T[0])

    def kernel_tvd(self, s, u, b, T_do, i=0, method=3, out=None):
        return self._mhd_kernel(self.lib.gdref_kernel_tvd, s, u, b, T_do, i, method, out)

    def kernel_gkr(self, s, u, b, T_do, i=0, method=3, out=None):
        return self._mhd_kernel(self.lib.gdref_kernel_gkr, s, u, b, T_do, i, method, out)

    def add2(self, s, u, b, T_do, i=0, method=2, out=None):
        return self._mhd_kernel(self.lib.gdref_add2, s, u, b, T_do, i, method, out)

    def print_tecplot(self, s, u, b, with_b, ttt, path):
        """The reference's print_file_mini (with_b 0) / print_file_mini2 (1; 2 = with
        SOLUTIONTIME ttt) for the grid set by set_params."""
        s = np.ascontiguousarray(s, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        b = None if b is None else np.ascontiguousarray(b, np.float64)
        self.lib.gdref_print_tecplot(_ptr(s), _ptr(u), _ptr(b), int(with_b), float(ttt),
                                     os.fsencode(path))

    def write_restart(self, s, u, b, path):
        """The restart dump of the reference's main loop (kernel.cu:4245-4254)."""
        s = np.ascontiguousarray(s, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        self.lib.gdref_write_restart(_ptr(s), _ptr(u), _ptr(b), os.fsencode(path))

    def ker_dekard(self, s, u, T_do, method=1, out=None):
        s = np.ascontiguousarray(s, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        s2, u2 = (s.copy(), u.copy()) if out is None else out
        T = np.array([1e7])
        self.lib.gdref_ker_dekard(_ptr(s), _ptr(u), _ptr(s2), _ptr(u2), _ptr(T), T_do, method)
        return s2, u2, float(T[0])
