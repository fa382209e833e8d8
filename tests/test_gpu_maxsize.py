"""A grid of more than 2^31 cells (65536 x 32800 Euler, 138 GB of state in HBM): every index
of the step, the layout kernels and the dt reduction is 64-bit.  The state is built in the
context's own planes on the device (gd_field_ptr), so nothing of that size touches the host.
Two identical density bumps, 31776 rows apart (a multiple of the tile height, so both sit at
the same place in their tiles), the second past cell index 2^31: the periodic Cartesian fast
step is translation-invariant, so after three steps the two neighbourhoods are bit for bit
the same, and the dt is that of the bump."""
import ctypes

import pytest

import golikov_2d_gb300 as g

pytestmark = pytest.mark.gpu

N, M = 65536, 32800
ROW_A, ROW_B, COL = 1000, 32776, 1000  # ROW_B * N + COL > 2^31
R = 12  # half-width of the compared neighbourhood (3 steps spread the bump 6 cells)


class _Plane:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 3}


def plane(sol, f):
    import torch
    p = ctypes.c_void_p()
    assert sol.lib.gd_field_ptr(sol.handle, f, ctypes.byref(p)) == 0
    return torch.as_tensor(_Plane(p.value, N * M), device="cuda").view(M, N)


def test_more_than_2_31_cells(cuda):
    import torch
    free, _ = torch.cuda.mem_get_info()
    if free < 150 * 2 ** 30:
        pytest.skip(f"needs ~140 GB of free device memory, {free / 2**30:.0f} GB free")
    assert ROW_B * N + COL > 2 ** 31
    cfg = g.Config(N=N, M=M, dx=1.0 / N, dy=1.0 / M, x0=0.5 / N, y0=0.5 / M, gamma=1.4,
                   krit=0.4, physics=g.EULER, order=2, method=g.METHOD_HLLC,
                   bc=(g.BC_PERIODIC,) * 4, mode=g.MODE_FAST)
    sol = g.Solver(cfg)
    rho, p, vx, vy = (plane(sol, f) for f in range(4))
    rho.fill_(1.0)
    p.fill_(1.0)
    vx.fill_(0.25)
    vy.fill_(0.0)
    for r0 in (ROW_A, ROW_B):
        rho[r0 - 2:r0 + 3, COL - 2:COL + 3] = 1.5
        p[r0 - 1:r0 + 2, COL - 1:COL + 2] = 2.0
    del rho, p, vx, vy
    sol.set_time(1e-5, 0.0)
    sol.advance(3)
    torch.cuda.synchronize()
    st = sol.stats()
    assert st.steps == 3 and st.nonfinite == 0
    for f in range(4):
        q = plane(sol, f)
        a = q[ROW_A - R:ROW_A + R + 1, COL - R:COL + R + 1]
        b = q[ROW_B - R:ROW_B + R + 1, COL - R:COL + R + 1]
        assert torch.equal(a, b), f
        assert not torch.equal(a, torch.full_like(a, a[0, 0].item()))  # the bump is there
    sol.close()
