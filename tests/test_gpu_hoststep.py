"""gd_step_host: a step from host memory to host memory with the transfers overlapped (bands
of block rows on two copy streams) equals gd_import + gd_advance(1) + gd_export bit for bit,
on periodic, transmissive and the reference's native boundaries, in fast and parity modes
(the Hancock scheme's too), over several steps, and through the sequential path for pageable
buffers and small grids."""
import numpy as np
import pytest

import golikov_2d_gb300 as g
from golikov_2d_gb300 import problems

pytestmark = pytest.mark.gpu

CASES = {
    "kh512_periodic": lambda: problems.kelvin_helmholtz(512, 384),
    "sod256_transmissive": lambda: problems.sod(256, 256),
    "ot256_mhd_periodic": lambda: problems.orszag_tang(256, 256),
    "wind_native": lambda: problems.stellar_wind(200, 136, 2.25, 1.25),
    "small_grid": lambda: problems.sod(40, 24),
    "sod256_parity": lambda: problems.sod(256, 256, mode=g.MODE_PARITY),
    "wind_native_parity": lambda: problems.stellar_wind(200, 136, 2.25, 1.25,
                                                        mode=g.MODE_PARITY),
    "hancock_parity": lambda: problems.hancock_wind(160, 96, mode=g.MODE_PARITY),
    "hancock_fast": lambda: problems.hancock_wind(160, 96),
    "hancock_fast_ragged": lambda: problems.hancock_wind(131, 77, scheme=g.SCHEME_HANCOCK),
}


def pinned(a):
    import torch
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).pin_memory()


def reference_steps(cfg, s, u, b, n):
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(1e-4, 0.0)
    out = []
    for _ in range(n):
        sol.advance(1)
        s2, u2 = np.zeros_like(s), np.zeros_like(u)
        b2 = None if b is None else np.zeros_like(b)
        sol.export_state(s2, u2, b2)
        st = sol.stats()
        out.append((s2, u2, b2, st.dt, st.t_state))
    sol.close()
    return out


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("pin", [True, False])
def test_step_host_equals_import_advance_export(cuda, case, pin):
    cfg, s, u, b = CASES[case]()
    ref = reference_steps(cfg, s, u, b, 3)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)  # the context's state is only the starting buffer here
    sol.set_time(1e-4, 0.0)
    conv = pinned if pin else (lambda a: None if a is None else np.ascontiguousarray(a).copy())
    hs, hu, hb = conv(s), conv(u), conv(b)
    os_, ou = conv(np.zeros_like(s)), conv(np.zeros_like(u))
    ob = None if b is None else conv(np.zeros_like(b))
    for k in range(3):
        sol.step_host(hs, hu, hb, os_, ou, ob)
        st = sol.stats()
        r = ref[k]
        got = [np.asarray(x) for x in (os_, ou)] + ([] if b is None else [np.asarray(ob)])
        want = [r[0], r[1]] + ([] if b is None else [r[2]])
        for x, y in zip(got, want):
            assert np.array_equal(x, y), (case, pin, k)
        assert st.dt == r[3] and st.t_state == r[4]
        # the next step starts from this result, as the reference loop does
        hs, hu, hb = (conv(np.asarray(x)) if x is not None else None for x in (os_, ou, ob))
    sol.close()
