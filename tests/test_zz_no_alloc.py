"""gd_step_ref_static: one step that allocates no device memory.

Some callers cannot let a library allocate: a host program that owns all device memory
through its own pool (a coupled multi-physics driver, an in-situ analysis framework) must
not see cudaMalloc calls outside its budget, and cudaFree would synchronise its whole
device.  gd_step_ref_static keeps its scratch in a static device array instead.  These
tests call it through the C ABI, twice in a row (the second call consumes the first call's
output and dt), and compare each result with gd_step_ref on the same inputs, within the
per-step tolerance of the fast-path tests.  This file sorts last so that a run stopping at
the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems
from gpu_util import gpu_step_ref, max_rel_l1, to_dev

pytestmark = pytest.mark.gpu

PER_STEP_TOL = 1e-12


def static_step(cfg, s, u, b, T_do, method=g.METHOD_CONFIG):
    """One call of gd_step_ref_static on device copies of (s, u, b)."""
    import torch
    L = g.load()
    ds, du, db = to_dev(s), to_dev(u), to_dev(b)
    s2, u2 = torch.zeros_like(ds), torch.zeros_like(du)
    b2 = None if db is None else torch.zeros_like(db)
    T = torch.tensor([1e7], dtype=torch.float64, device="cuda")
    Tdo = torch.tensor([T_do], dtype=torch.float64, device="cuda")
    c = cfg.cstruct()
    p = lambda t: None if t is None else t.data_ptr()
    st = L.gd_step_ref_static(ctypes.byref(c), p(ds), p(du), p(db), p(s2), p(u2), p(b2), p(T),
                              p(Tdo), int(method), torch.cuda.current_stream().cuda_stream or None)
    assert st == 0, g.STATUS.get(st, st)
    torch.cuda.synchronize()
    return (s2.cpu().numpy(), u2.cpu().numpy(), None if b2 is None else b2.cpu().numpy(),
            float(T.cpu()[0]))


CASES = {
    "sod256_fast": lambda: problems.sod(256, 256),  # exactly GD_STATIC_MAX_CELLS cells
    "kh128x64_fast": lambda: problems.kelvin_helmholtz(128, 64),
    "kh64_parity": lambda: problems.kelvin_helmholtz(64, 64, mode=g.MODE_PARITY),
    "ot96_hlld_fast": lambda: problems.orszag_tang(96, 96),
    "ot96_hlld_parity": lambda: problems.orszag_tang(96, 96, mode=g.MODE_PARITY),
    "wind_hlld_fast": lambda: problems.stellar_wind(96, 54, 2.25, 1.25),
    # the MUSCL-Hancock step (its edge-band and tile launches in fast mode, the per-cell
    # kernel in parity mode), on a grid whose frozen sphere and edges both lie inside
    "hancock_wind_fast": lambda: problems.hancock_wind(96, 54, 4.5, 2.5),
    "hancock_wind_parity": lambda: problems.hancock_wind(96, 54, 4.5, 2.5,
                                                         mode=g.MODE_PARITY),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_static_step_matches_context_step_twice(cuda, case):
    cfg, s, u, b = CASES[case]()
    T_do = 1e-5
    for _ in range(2):
        a = static_step(cfg, s, u, b, T_do)
        r = gpu_step_ref(cfg, s, u, b, T_do)
        err = max_rel_l1(cfg, a[:3], r[:3])
        assert err <= PER_STEP_TOL, err
        assert abs(a[3] - r[3]) <= PER_STEP_TOL * r[3]
        s, u, b, T_do = a[0], a[1], a[2], a[3]


def test_static_step_rejects_grids_beyond_its_scratch(cuda):
    import torch
    cfg, s, u, b = problems.sod(257, 256)  # 65792 cells > GD_STATIC_MAX_CELLS = 65536
    L = g.load()
    ds, du = to_dev(s), to_dev(u)
    s2, u2 = torch.full_like(ds, 7.0), torch.full_like(du, 7.0)
    T = torch.tensor([1e7], dtype=torch.float64, device="cuda")
    Tdo = torch.tensor([1e-5], dtype=torch.float64, device="cuda")
    st = L.gd_step_ref_static(ctypes.byref(cfg.cstruct()), ds.data_ptr(), du.data_ptr(), None,
                              s2.data_ptr(), u2.data_ptr(), None, T.data_ptr(), Tdo.data_ptr(),
                              g.METHOD_CONFIG, None)
    torch.cuda.synchronize()
    assert st == 1
    assert bool((s2 == 7.0).all()) and float(T.cpu()[0]) == 1e7


def test_static_steps_allocate_nothing(cuda):
    """The property the entry point exists for: once a device is set up, calls make no
    device allocation and no release.  Checked two ways around repeated calls in both
    modes, both physics and both Hancock forms: the library's own allocation counter
    (gd_alloc_counts: every allocation of the library goes through it) and the device's
    free memory (cudaMemGetInfo), which sees any allocation, the CUDA runtime's included."""
    import torch
    L = g.load()
    calls = []
    for name in sorted(CASES):
        cfg, s, u, b = CASES[name]()
        ds, du, db = to_dev(s), to_dev(u), to_dev(b)
        out = (torch.zeros_like(ds), torch.zeros_like(du),
               None if db is None else torch.zeros_like(db))
        T = torch.tensor([1e7], dtype=torch.float64, device="cuda")
        Tdo = torch.tensor([1e-5], dtype=torch.float64, device="cuda")
        calls.append((cfg.cstruct(), (ds, du, db), out, T, Tdo))
    p = lambda t: None if t is None else t.data_ptr()

    def run_all():
        for c, (ds, du, db), (s2, u2, b2), T, Tdo in calls:
            st = L.gd_step_ref_static(ctypes.byref(c), p(ds), p(du), p(db), p(s2), p(u2),
                                      p(b2), p(T), p(Tdo), g.METHOD_CONFIG, None)
            assert st == 0, g.STATUS.get(st, st)
        torch.cuda.synchronize()

    run_all()  # set-up of this device, first launch of every kernel used
    counts0 = g.alloc_counts()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        run_all()
    free1 = torch.cuda.mem_get_info()[0]
    assert g.alloc_counts() == counts0
    assert free1 == free0
    for _, _, (s2, u2, b2), T, _ in calls:
        assert bool(torch.isfinite(s2).all()) and bool(torch.isfinite(u2).all())
        assert 0.0 < float(T.cpu()[0]) < 1e7
