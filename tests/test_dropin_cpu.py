"""The drop-in harness itself, on the CPU: the reference's unchanged Python
package runs on its own C library (the CPU build of its pip install) and
equals the oracle bit for bit.  This pins the harness that
tests/test_dropin_gpu.py uses with this library in the reference library's
place.  Skipped where the reference's pip install is absent."""
import glob
import os

import numpy as np
import pytest

import dropin
from abie_gb300 import ics

G = ics.G_SOLAR
pytestmark = pytest.mark.skipif(not dropin.available(), reason="reference package not installed "
                                "in baseline/_ref")


def _ref_lib():
    libs = glob.glob(os.path.join(dropin.ROOT, "baseline", "_ref", "libabie*.so"))
    if not libs:
        pytest.skip("the reference's own C library is not built for this machine")
    return libs[0]


def test_reference_package_on_its_own_library(tmp_path, oracle):
    root = dropin.stage(tmp_path, _ref_lib())
    p, v, m, r = ics.planetary_system(seed=41, n_planets=5, n_tp=20)
    out, log = dropin.run(tmp_path, root, "GaussRadau15", -1, 0.5, 0.01, p, v, m, G)
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.5)
    assert np.array_equal(out["pos"], ref["pos"]) and np.array_equal(out["vel"], ref["vel"])
    assert out["t"][0] == ref["t"]
