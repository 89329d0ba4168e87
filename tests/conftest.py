import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The ensemble's autotuner times candidate launch shapes on each new
# workload; the tests switch it off (their workloads are all different and
# small) except the test of the tuner itself, which turns it on again.
os.environ["ABIE_ENSEMBLE_TUNE"] = "0"

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")
    config.addinivalue_line("markers", "slow: longer CPU cases")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle, build_oracle
    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference, build_reference, reference_available
    if not reference_available():
        try:
            build_reference()
        except Exception:
            pass
    if not reference_available():
        pytest.skip("reference library not built here (no reference sources)")
    return Reference()


@pytest.fixture(scope="session")
def built_lib():
    from abie_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def clib(built_lib):
    from abie_gb300.clibabie import CLibABIE
    return CLibABIE()


def rel_err_per_body(a, b):
    """max over bodies of |a_i - b_i| / |b_i| (3-vectors)."""
    a = np.asarray(a).reshape(-1, 3)
    b = np.asarray(b).reshape(-1, 3)
    num = np.linalg.norm(a - b, axis=1)
    den = np.linalg.norm(b, axis=1)
    ok = den > 0
    out = np.zeros(len(a))
    out[ok] = num[ok] / den[ok]
    out[~ok] = num[~ok]
    return out.max() if out.size else 0.0


@pytest.fixture(scope="session")
def sim(clib):
    """The stateful library, initialized once per process as the reference
    requires: capacity 2^21 bodies, 3 close-encounter and 2 collision slots."""
    clib.initialize_code(4 * np.pi ** 2, 0.0, 1 << 21, MAX_CE_EVENTS=3, MAX_COLLISION_EVENTS=2,
                         close_encounter_distance=0.0, deviceID=0)
    return clib
