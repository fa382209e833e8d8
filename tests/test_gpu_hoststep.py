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
    # grids of many bands (16 to 32, the most a step takes)
    "kh2048x1024_many_bands": lambda: problems.kelvin_helmholtz(2048, 1024),
    "ot1024_many_bands": lambda: problems.orszag_tang(1024, 1024),
    "hancock_fast_many_bands": lambda: problems.hancock_wind(1024, 640),
    "sod1024_parity_many_bands": lambda: problems.sod(1024, 1024, mode=g.MODE_PARITY),
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


def run_reference(case, n):
    cfg, s, u, b = CASES[case]()
    return cfg, s, u, b, reference_steps(cfg, s, u, b, n)


def check_step(sol, out, r, mhd, tag):
    got = [np.asarray(x) for x in out[:2]] + ([np.asarray(out[2])] if mhd else [])
    want = [r[0], r[1]] + ([r[2]] if mhd else [])
    for x, y in zip(got, want):
        assert np.array_equal(x, y), tag
    st = sol.stats()
    assert st.dt == r[3] and st.t_state == r[4], tag


@pytest.mark.parametrize("case", ["kh512_periodic", "ot256_mhd_periodic", "wind_native",
                                  "hancock_fast", "sod256_parity", "ot1024_many_bands"])
def test_step_host_graph_replays(cuda, case):
    """The step graphs are replayed when the same host buffers come back: ping-pong between
    two buffer sets (the reference loop's s -> s2 -> s) for 7 steps, then the same input
    and output buffers every step (the input refilled on the host) for 6 more; every step
    equals gd_advance(1), and each step counts the launches of a directly enqueued one."""
    cfg, s, u, b, ref = run_reference(case, 13)
    mhd = b is not None
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(1e-4, 0.0)
    A = [pinned(x) for x in (s, u, b)]
    B = [pinned(np.zeros_like(x)) if x is not None else None for x in (s, u, b)]
    per_step = None
    for k in range(7):
        src, dst = (A, B) if k % 2 == 0 else (B, A)
        l0 = sol.launch_count()
        sol.step_host(*src, *dst)
        n = sol.launch_count() - l0
        assert per_step is None or n == per_step, (case, k, n, per_step)
        per_step = n
        check_step(sol, dst, ref[k], mhd, (case, k))
    # B holds the result of the last step (k = 6): step from B into A, then copy A into B
    for k in range(7, 13):
        sol.step_host(*B, *A)
        check_step(sol, A, ref[k], mhd, (case, k))
        for x, y in zip(A, B):
            if x is not None:
                y.copy_(x)
    sol.close()


def test_step_host_graph_cache_eviction(cuda):
    """Five buffer sets in rotation (more than the cached graphs): captures replace the
    oldest graphs and every step still equals gd_advance(1)."""
    cfg, s, u, b, ref = run_reference("kh512_periodic", 11)
    sol = g.Solver(cfg)
    sol.import_state(s, u, b)
    sol.set_time(1e-4, 0.0)
    sets = [[pinned(s), pinned(u)]] + [[pinned(np.zeros_like(s)), pinned(np.zeros_like(u))]
                                      for _ in range(4)]
    for k in range(11):
        src, dst = sets[k % 5], sets[(k + 1) % 5]
        sol.step_host(src[0], src[1], None, dst[0], dst[1], None)
        check_step(sol, dst, ref[k], False, k)
    sol.close()
