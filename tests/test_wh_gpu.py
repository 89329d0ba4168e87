"""Wisdom-Holman on the device against the reference's golden run and the
oracle, in three forms: exact (the reference's expressions, the device's
transcendental functions, which differ from the host libm in the last bits),
fast (series Stumpff functions, a third-order starting value for the
Kepler iteration, reciprocals and r^-3 without divisions) and mixed (the
fast form with the planets' pull on each test particle in FP32 two-float
arithmetic on heliocentric coordinates, about 2^-44 relative to those
terms).  States are compared to 1e-10 relative (max over bodies); the step
count and final time are exact."""
import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
TOL = 1e-10


@pytest.fixture(params=["fp64", "exact", "mixed"])
def wh_mode(sim, request):
    old = sim.set_force_mode(request.param)
    yield request.param
    sim.set_force_mode(old)


def _wh(sim, p, v, m, t0, t1, dt):
    sim.set_state(p, v, m, np.zeros(m.size), m.size, G, 0.0)
    sim.integrator_wh(t0, t1, dt)
    pos, vel = np.zeros(p.size), np.zeros(p.size)
    sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
    return pos, vel, sim.get_model_time()


def test_golden_wh(sim, golden, wh_mode):
    t0, t1, dt = golden["wh_span"]
    pos, vel, t = _wh(sim, golden["wh_in_pos"], golden["wh_in_vel"], golden["wh_m"], t0, t1, dt)
    assert t == golden["wh_t"][0]
    assert rel_err_per_body(pos, golden["wh_pos"]) <= TOL
    assert rel_err_per_body(vel, golden["wh_vel"]) <= TOL


def test_wh_massive_bodies_only(sim, oracle, wh_mode):
    """No tail: every body goes through the head kernel."""
    p, v, m, r = ics.planetary_system(seed=61, n_planets=7, n_tp=0)
    p, v = ics.to_heliocentric(p, v)
    ref = oracle.wh(p, v, m, G, 0.0, 2.0, 0.01, sparse=False)
    pos, vel, t = _wh(sim, p, v, m, 0.0, 2.0, 0.01)
    assert t == ref["t"]
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL


def test_wh_interleaved_massless(sim, oracle, wh_mode):
    """A massless body between massive ones stays in the head."""
    p, v, m, r = ics.test_particle_swarm(seed=62, n_tp=50, n_planets=4)
    m = m.copy()
    m[2], m[6] = 0.0, 2e-5
    p, v = ics.to_heliocentric(p, v)
    ref = oracle.wh(p, v, m, G, 0.0, 1.0, 0.01, sparse=True)
    pos, vel, t = _wh(sim, p, v, m, 0.0, 1.0, 0.01)
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL


def test_wh_swarm_64k_vs_oracle(sim, oracle, wh_mode):
    p, v, m, r = ics.test_particle_swarm(seed=63, n_tp=65536)
    p, v = ics.to_heliocentric(p, v)
    ref = oracle.wh(p, v, m, G, 0.0, 0.1, 0.01, sparse=True)
    pos, vel, t = _wh(sim, p, v, m, 0.0, 0.1, 0.01)
    assert t == ref["t"]
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL


def test_wh_full_swarm_steps(sim, oracle, wh_mode):
    """The 1,048,581-body workload, three steps, against the oracle's O(N N_m)
    restatement (bit-identical to the reference's O(N^2) loop)."""
    p, v, m, r = ics.test_particle_swarm()
    p, v = ics.to_heliocentric(p, v)
    ref = oracle.wh(p, v, m, G, 0.0, 0.03, 0.01, sparse=True)
    pos, vel, t = _wh(sim, p, v, m, 0.0, 0.03, 0.01)
    assert t == ref["t"]
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL
    c = sim.counters()
    assert c["kepler_failures"] == 0


def test_wh_mixed_error_stated(sim, oracle):
    """The mixed kick's error against the fast FP64 form on the whole
    1,048,581-body workload after 20 steps: printed, and bounded at 1e-10
    relative like the other WH comparisons (the planets' terms are
    perturbations of the star's, carried to about 2^-44 of themselves)."""
    p, v, m, r = ics.test_particle_swarm()
    p, v = ics.to_heliocentric(p, v)
    old = sim.set_force_mode("fp64")
    try:
        pf, vf, tf = _wh(sim, p, v, m, 0.0, 0.2, 0.01)
        sim.set_force_mode("mixed")
        pm, vm, tm = _wh(sim, p, v, m, 0.0, 0.2, 0.01)
    finally:
        sim.set_force_mode(old)
    assert tf == tm
    err_p, err_v = rel_err_per_body(pm, pf), rel_err_per_body(vm, vf)
    print("WH mixed vs fp64 after 20 steps at 1,048,581 bodies: max rel %.2e (pos) %.2e (vel)"
          % (err_p, err_v))
    assert err_p <= TOL and err_v <= TOL


def _hyperbolic_swarm(seed, n_tp):
    """A star, one Jupiter-mass planet at 5 au and n_tp test particles on
    hyperbolic orbits about the star: distances 2 .. 1e4 au, specific
    energies 1e-3 .. 1e2 (au/yr)^2, directions at random, half of them
    moving inward.  Heliocentric."""
    rng = np.random.default_rng(seed)
    p = [np.zeros(3), np.array([5.0, 0.0, 0.0])]
    v = [np.zeros(3), np.array([0.0, np.sqrt(G * (1.0 + 1e-3) / 5.0), 0.0])]
    for _ in range(n_tp):
        r0 = 10 ** rng.uniform(np.log10(2.0), 4.0)
        e = 10 ** rng.uniform(-3.0, 2.0)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        w = rng.normal(size=3)
        w -= w.dot(u) * u
        w /= np.linalg.norm(w)
        c = rng.uniform(-1.0, 1.0)
        speed = np.sqrt(2.0 * (e + G / r0))
        p.append(r0 * u)
        v.append(speed * (c * u + np.sqrt(1.0 - c * c) * w))
    m = np.zeros(len(p))
    m[0], m[1] = 1.0, 1e-3
    return np.concatenate(p), np.concatenate(v), m


def test_wh_hyperbolic_escapers(sim, oracle, wh_mode):
    """Test particles on hyperbolic orbits, near and far, inbound and
    outbound.  The fast Kepler start is the Taylor series of chi(t) on
    short arcs of any conic, where the reference's logarithmic start needs
    tens of Newton steps; the radius function may turn negative far from
    the root, which the fast reciprocal handles.  Every solve converges
    (no Kepler failure counted), the states stay finite and agree with the
    oracle."""
    p, v, m = _hyperbolic_swarm(63, 96)
    ref = oracle.wh(p, v, m, G, 0.0, 2.0, 0.01, sparse=True)
    sim.reset_counters()
    pos, vel, t = _wh(sim, p, v, m, 0.0, 2.0, 0.01)
    c = sim.counters()
    assert c["kepler_failures"] == 0
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    assert t == ref["t"]
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL
