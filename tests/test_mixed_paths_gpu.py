"""The mixed-precision form on the integrators' paths, each with its error
against the oracle stated and bounded.

* Radau15 (integrator_gr): the fast sweep with the mixed all-pairs force
  (sources below 1e-6 of the heaviest in FP32 pair terms on anchored
  coordinates, tile sums folded into FP64) on every substep, through the
  stepped engine.  On the 2,049-body planetesimal disk (every planetesimal
  light, the star heavy) over 0.05 yr against the oracle.
* The post-Newtonian terms and the naive comparator form have no mixed or
  integrator form: those calls fail loudly with ABIE_ERR_UNSUPPORTED
  instead of running another form.
(The ensemble's mixed form is in test_ensemble_gpu.py, the WH kick's in
test_wh_gpu.py.)"""
import numpy as np
import pytest

from abie_gb300 import ics
from abie_gb300.events import AbieError
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL_FAST, at_time

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
ERR_UNSUPPORTED = -4


def _gr(sim, p, v, m, r, t1, mode, C=0.0):
    old = sim.set_force_mode(mode)
    try:
        sim.set_state(p, v, m, r, m.size, G, C)
        sim.integrator_gr(0.0, t1, 1.0)
        P, V = np.zeros(p.size), np.zeros(v.size)
        sim.get_state(P, V, np.zeros(m.size), np.zeros(m.size))
        return P, V, sim.get_model_time()
    finally:
        sim.set_force_mode(old)


def test_radau_mixed_disk_against_oracle(sim, oracle):
    p, v, m, r = ics.planetesimal_disk(seed=71, n=2048)
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.05)
    P, V, t = _gr(sim, p, v, m, r, 0.05, "mixed")
    assert abs(t - ref["t"]) <= TIME_TOL_FAST * ref["t"]
    P, V = at_time(P, V, m, t, ref["t"], oracle)
    # planetesimals relative to their own position; the star, which sits
    # within about 1e-6 au of the origin, in absolute terms
    ep = rel_err_per_body(P[3:], ref["pos"][3:])
    ev = rel_err_per_body(V[3:], ref["vel"][3:])
    star_p = float(np.abs(P[:3] - ref["pos"][:3]).max())
    e0 = oracle.energy(p, v, m, G)
    de = abs((oracle.energy(P, V, m, G) - e0) / e0)
    print("Radau15 mixed, 2,049-body disk, 0.05 yr: planetesimals max rel %.2e (pos) %.2e "
          "(vel); star %.2e au; |dE/E| %.2e" % (ep, ev, star_p, de))
    assert ep <= 1e-9 and ev <= 1e-9
    assert star_p <= 1e-12
    assert de <= 1e-12


def test_forms_without_a_mixed_or_integrator_form_refuse(sim):
    p, v, m, r = ics.planetary_system(seed=72, n_planets=4, n_tp=0)
    with pytest.raises(AbieError) as exc:
        _gr(sim, p, v, m, r, 0.1, "mixed", C=63239.7263)
    assert exc.value.code == ERR_UNSUPPORTED
    with pytest.raises(AbieError) as exc:
        _gr(sim, p, v, m, r, 0.1, "naive")
    assert exc.value.code == ERR_UNSUPPORTED
    old = sim.set_force_mode("naive")
    try:
        sim.set_state(p, v, m, r, m.size, G, 0.0)
        with pytest.raises(AbieError) as exc:
            sim.integrator_wh(0.0, 0.1, 0.01)
        assert exc.value.code == ERR_UNSUPPORTED
    finally:
        sim.set_force_mode(old)
