"""The snapshot checker (oracle/snapshots.py) against the reference's own
Python: orbital elements from Particles.calculate_aei (golden_aei.npz, made
by tests/golden/make_golden.py from abie/particles.py and abie/tools.py)
and the chunk schedule of Integrator.integrate."""
import os

import numpy as np
import pytest

from abie_gb300 import ics
from oracle import snapshots as S

GOLDEN_AEI = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_aei.npz")


@pytest.mark.parametrize("key,primary", [("com", S.PRIMARY_COM), ("mmax", S.PRIMARY_M_MAX),
                                         ("body3", 3)])
def test_aei_restatement_matches_reference(key, primary):
    g = np.load(GOLDEN_AEI)
    out = S.calculate_aei(g["aei_pos"], g["aei_vel"], g["aei_m"], ics.G_SOLAR, primary)
    assert np.array_equal(out, g["aei_" + key], equal_nan=True)


def test_py_mod_is_python_modulo():
    rng = np.random.default_rng(5)
    for _ in range(2000):
        x, y = rng.uniform(-50, 50), rng.choice([-1, 1]) * rng.uniform(1e-3, 10)
        assert S.py_mod(x, y) == x % y
    assert S.py_mod(0.5, 0.25) == 0.5 % 0.25


def test_chunk_schedule():
    """Exact advances land on the store_dt grid; an overshoot (as Radau15's
    last step gives) snaps the next chunk back onto it."""
    ends = S.chunk_ends(0.0, 1.0, 0.25, lambda t0, t1: t1)
    assert ends == [0.25, 0.5, 0.75, 1.0]
    ends = S.chunk_ends(0.0, 1.0, 0.25, lambda t0, t1: t1 + 0.01)
    assert ends == [0.25, 0.5, 0.75, 1.0]
    # dt = t_end - t = 0.5, and the ends snap to multiples of it, past t_end
    ends = S.chunk_ends(0.1, 0.6, 1.0, lambda t0, t1: t1)
    assert len(ends) == 2 and abs(ends[0] - 0.5) < 1e-15 and ends[1] == 1.0
