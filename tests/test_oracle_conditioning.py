"""How far the reference's own arithmetic (the oracle) carries a rounding-level change.

The Orszag-Tang run makes minmod choices at near-ties and, in places, clamps the pressure,
both discontinuous, so two correct evaluations that differ by rounding drift apart.  This
measures that drift for the reference itself: the state moved by one ulp per value, 100
steps at 128^2.  It is the floor under any bound that compares a different rounding (the
fast GPU step) with the reference after N steps (tests/test_gpu_fast.py)."""
import numpy as np

from golikov_2d_gb300 import problems
from gpu_util import max_rel_l1, oracle_run


def test_orszag_tang_128_amplifies_one_ulp_to_about_1e_9(oracle_lib):
    cfg, s, u, b = problems.orszag_tang(128, 128)
    ref = oracle_run(oracle_lib, cfg, s, u, b, 100)
    rng = np.random.default_rng(3)
    drift = []
    for _ in range(3):
        moved = [x + np.spacing(x) * rng.choice([-1.0, 1.0], x.shape) for x in (s, u, b)]
        run = oracle_run(oracle_lib, cfg, *moved, 100)
        drift.append(max_rel_l1(cfg, run[:3], ref[:3]))
    # measured: 5e-10 to 4e-9 (seed 3: 3.8e-9, 5.2e-10, 9.0e-10)
    assert 1e-10 < max(drift) < 1e-8, drift
