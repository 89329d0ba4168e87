"""The close-encounter / collision check fused into the force evaluation.

The reference checks every pair after each accepted step
(src/common.c:116-158, called at src/integrator_gauss_radau15.c:342) on
the accepted positions, which are the positions of the step's advance
force evaluation.  The split and persistent Radau15 engines run the check
inside that evaluation: each (sink, massive source) pair the force visits
takes the reference's test there (a pair of two massive bodies once), the
records of a rejected attempt are dropped, and only pairs of two bodies
without positive mass -- which the force never visits -- are scanned after
the accepted step.  Here a test particle rides 0.9 close-encounter
distances from one planet, an extra low-mass planet 0.9 distances from
another (a pair of two massive bodies) and a test particle 1.1 distances
from a third (not an event), beside a hundred far test particles; the
flag, ring buffer, body indices and stop time equal the oracle's, on the
split engine (few planets) and the persistent engine (12 planets), and a
collision between a particle and a planet with radii set does too.

The event times are those of the first accepted steps, whose corrector
sweeps reach the iteration cap (the pair 0.9 distances apart sets a time
scale far below the initial step), so the step control runs on
unconverged coefficients and the reference's own event times move by up
to 7e-6 relative when one input coordinate moves by one unit in the last
place.  The device's pow differs from the host libm's in the last bit on
some inputs, so times and distances are compared within 20 times that
spread of the oracle (measured on the same system with twelve such
perturbations), and never more tightly than the usual trajectory bars."""
import ctypes as C

import numpy as np
import pytest

from abie_gb300 import ics
from abie_gb300.events import CloseEncounterException, CollisionException
from test_radau_gpu import TIME_TOL

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR


def _system(n_planets, ce):
    p, v, m, r = ics.planetary_system(seed=17, n_planets=n_planets, n_tp=100)
    P, V = p.reshape(-1, 3), v.reshape(-1, 3)
    extra_p, extra_v, extra_m = [], [], []
    for body, scale, mass in ((1, 0.9, 0.0), (2, 0.9, 1e-7), (3, 1.1, 0.0)):
        off = np.array([0.0, 0.0, ce * scale])
        extra_p.append(P[body] + off)
        extra_v.append(V[body])
        extra_m.append(mass)
    p = np.concatenate([p, np.concatenate(extra_p)])
    v = np.concatenate([v, np.concatenate(extra_v)])
    m = np.concatenate([m, extra_m])
    r = np.zeros(m.size)
    return p, v, m, r


def _run(sim, p, v, m, r, ce, t1, max_ce, exc_type):
    sim.set_close_encounter_distance(ce)
    sim.reset_close_encounter_buffer()
    sim.reset_collision_buffer()
    old = sim.set_force_mode("exact")
    try:
        sim.set_state(p, v, m, r, m.size, G, 0.0)
        with pytest.raises(exc_type):
            sim.integrator_gr(0.0, t1, 1.0)
        buf = sim.get_close_encounter_data() if exc_type is CloseEncounterException \
            else sim.get_collision_data()
        return buf, sim.get_model_time()
    finally:
        sim.set_force_mode(old)
        sim.set_close_encounter_distance(0.0)
        sim.reset_close_encounter_buffer()
        sim.reset_collision_buffer()


def _spread(oracle, p, v, m, r, gold, key, **kw):
    """Largest relative change of the oracle's event times and distances
    when one input coordinate moves by one unit in the last place (twelve
    such runs), and of its final time."""
    dt = dd = dtf = 0.0
    ref = oracle.radau15(p, v, m, r, G, 0.0, 5.0, **kw)
    for k in range(12):
        q = p.copy()
        i = (7 * k) % q.size
        q[i] = np.nextafter(q[i], np.inf if k % 2 else -np.inf)
        run = oracle.radau15(q, v, m, r, G, 0.0, 5.0, **kw)
        b = run[key].reshape(-1, 4)
        if not np.array_equal(b[:, 1:3], gold[:, 1:3]):
            continue
        dt = max(dt, np.max(np.abs(b[:, 0] - gold[:, 0]) / gold[:, 0]))
        dd = max(dd, np.max(np.abs(b[:, 3] - gold[:, 3]) / gold[:, 3]))
        dtf = max(dtf, abs(run["t"] - ref["t"]) / ref["t"])
    return dt, dd, dtf


def _check(buf, t, gold, t_ref, spread):
    dt, dd, dtf = spread
    tol_t, tol_d, tol_f = max(TIME_TOL, 20 * dt), max(1e-12, 20 * dd), max(TIME_TOL, 20 * dtf)
    et = np.max(np.abs(buf[:, 0] - gold[:, 0]) / gold[:, 0])
    ed = np.max(np.abs(buf[:, 3] - gold[:, 3]) / gold[:, 3])
    print("event times %.2e (bar %.2e), distances %.2e (bar %.2e), final time %.2e (bar %.2e); "
          "the oracle's one-ulp spread %.2e %.2e %.2e"
          % (et, tol_t, ed, tol_d, abs(t - t_ref) / t_ref, tol_f, dt, dd, dtf))
    assert np.array_equal(buf[:, 1:3], gold[:, 1:3])
    assert et <= tol_t
    assert ed <= tol_d
    assert abs(t - t_ref) <= tol_f * t_ref


@pytest.mark.parametrize("n_planets", [3, 12])
def test_fused_close_encounters(sim, oracle, n_planets):
    ce = 0.01
    p, v, m, r = _system(n_planets, ce)
    n0 = m.size - 3
    ref = oracle.radau15(p, v, m, r, G, 0.0, 5.0, ce_dist=ce, max_ce=3, max_coll=2)
    assert ref["flag"] == 1
    gold = ref["buf_ce"].reshape(-1, 4)
    pairs = {(int(a), int(b)) for a, b in gold[:, 1:3]}
    assert pairs == {(1, n0), (2, n0 + 1)}  # particle-planet and planet-planet, not the 1.1 one
    spread = _spread(oracle, p, v, m, r, gold, "buf_ce", ce_dist=ce, max_ce=3, max_coll=2)
    buf, t = _run(sim, p, v, m, r, ce, 5.0, 3, CloseEncounterException)
    _check(buf, t, gold, ref["t"], spread)


@pytest.mark.parametrize("n_planets", [3, 12])
def test_fused_collision(sim, oracle, n_planets):
    """Radii make the particle beside planet 1 a collision (radii sum 0.95
    close-encounter distances against a separation of 0.9)."""
    ce = 0.01
    p, v, m, r = _system(n_planets, ce)
    n0 = m.size - 3
    r = r.copy()
    r[1] = 0.5 * ce
    r[n0] = 0.45 * ce
    ref = oracle.radau15(p, v, m, r, G, 0.0, 5.0, ce_dist=0.0, max_ce=3, max_coll=2)
    assert ref["flag"] == 2
    gold = ref["buf_coll"].reshape(-1, 4)
    assert {(int(a), int(b)) for a, b in gold[:, 1:3]} == {(1, n0)}
    sim.lib.set_close_encounter_distance(C.c_double(0.0))
    spread = _spread(oracle, p, v, m, r, gold, "buf_coll", ce_dist=0.0, max_ce=3, max_coll=2)
    buf, t = _run(sim, p, v, m, r, 0.0, 5.0, 3, CollisionException)
    _check(buf, t, gold, ref["t"], spread)
