"""Runge-Kutta 4 on the device (src/integrator_runge_kutta.c:6-50).

The exact force form with the reference's stage arithmetic reproduces the
reference's doubles: bit for bit against the golden run and the oracle.
The fast form agrees to 1e-12 relative per body.  Both the stateful
integrator_rk and the caller-array integrator_runge_kutta are covered."""
import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR


def _rk(sim, p, v, m, t0, t1, dt):
    sim.set_state(p, v, m, np.zeros(m.size), m.size, G, 0.0)
    t_before = sim.get_model_time()
    sim.integrator_rk(t0, t1, dt)
    pos, vel = np.zeros(p.size), np.zeros(p.size)
    sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
    assert sim.get_model_time() == t_before  # the reference leaves it alone
    return pos, vel


def test_rk_exact_matches_golden(sim, golden):
    old = sim.set_force_mode("exact")
    try:
        t0, t1, dt = golden["rk_span"]
        pos, vel = _rk(sim, golden["rk_in_pos"], golden["rk_in_vel"], golden["rk_m"], t0, t1, dt)
    finally:
        sim.set_force_mode(old)
    assert np.array_equal(pos, golden["rk_pos"]) and np.array_equal(vel, golden["rk_vel"])


@pytest.mark.parametrize("mode,tol", [("exact", 0.0), ("fp64", 1e-12)])
def test_rk_vs_oracle(sim, oracle, mode, tol):
    p, v, m, r = ics.planetary_system(seed=83, n_planets=8, n_tp=200)
    ref = oracle.rk(p, v, m, G, 0.0, 0.3, 0.002)
    old = sim.set_force_mode(mode)
    try:
        pos, vel = _rk(sim, p, v, m, 0.0, 0.3, 0.002)
    finally:
        sim.set_force_mode(old)
    if tol == 0.0:
        assert np.array_equal(pos, ref["pos"]) and np.array_equal(vel, ref["vel"])
    else:
        assert rel_err_per_body(pos, ref["pos"]) <= tol
        assert rel_err_per_body(vel, ref["vel"]) <= tol


def test_rk_caller_arrays(sim, oracle):
    p, v, m, r = ics.planetary_system(seed=84, n_planets=5, n_tp=30)
    ref = oracle.rk(p, v, m, G, 0.0, 0.1, 0.001)
    pos, vel = p.copy(), v.copy()
    old = sim.set_force_mode("exact")
    try:
        sim.integrator_runge_kutta(pos, vel, m, m.size, G, 0.0, 0.1, 0.001)
    finally:
        sim.set_force_mode(old)
    assert np.array_equal(pos, ref["pos"]) and np.array_equal(vel, ref["vel"])
