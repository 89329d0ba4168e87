"""The drop-in path: the reference's own Python package, unchanged, loads
this library where it expects its libabie and runs on the GPU.

abie.ABIE(deviceID=...), add(), sim.integrator = "GaussRadau15" /
"WisdomHolman", sim.h, sim.integrate() -- the reference's calls through its
abie/clibabie.py into libabie_gb300 (tests/dropin.py stages the package from
its pip install in baseline/_ref next to a symlink to this library; each run
is a fresh process, since the library keeps one simulation per process).
Results are compared with the oracle: Radau15 at a common time within
1e-10 (the library's default fast form: stop times within 1e-5), WH to
1e-10 with the same model time.  The stock default deviceID=-1 (the
reference's CPU setting) runs on GPU 0.  Skipped where the reference's pip
install is absent."""
import numpy as np
import pytest

import dropin
from abie_gb300 import build, ics
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL_FAST, TOL, at_time

G = ics.G_SOLAR
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not dropin.available(),
                                 reason="reference package not installed in baseline/_ref")]


@pytest.fixture(scope="module")
def staged(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("dropin")
    return tmp, dropin.stage(tmp, build.build())


@pytest.mark.parametrize("device", [0, -1])
def test_gauss_radau15_through_the_reference_package(staged, oracle, device):
    tmp, root = staged
    p, v, m, r = ics.planetary_system(seed=1001, n_planets=8, n_tp=200)
    out, log = dropin.run(tmp, root, "GaussRadau15", device, 0.5, 0.01, p, v, m, G)
    assert "libabie" in str(out["lib"])
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.5)
    t = out["t"][0]
    assert abs(t - ref["t"]) <= TIME_TOL_FAST * ref["t"]
    pp, vv = at_time(out["pos"], out["vel"], m, t, ref["t"], oracle)
    assert rel_err_per_body(pp, ref["pos"]) <= TOL
    assert rel_err_per_body(vv, ref["vel"]) <= TOL
    e0 = oracle.energy(p, v, m, G)
    assert abs((out["energy"][0] - e0) / e0) < 1e-12
    if device < 0:
        assert "runs on GPU 0" in log


def test_wisdom_holman_through_the_reference_package(staged, oracle):
    tmp, root = staged
    p, v, m, r = ics.test_particle_swarm(seed=1003, n_tp=500)
    out, log = dropin.run(tmp, root, "WisdomHolman", 0, 1.0, 0.01, p, v, m, G)
    hp, hv = ics.to_heliocentric(p, v)  # the reference's warm-up moves to heliocentric
    ref = oracle.wh(hp, hv, m, G, 0.0, 1.0, 0.01)
    assert out["t"][0] == ref["t"]
    assert rel_err_per_body(out["pos"], ref["pos"]) <= TOL
    assert rel_err_per_body(out["vel"], ref["vel"]) <= TOL
