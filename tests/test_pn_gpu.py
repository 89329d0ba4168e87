"""Post-Newtonian terms (src/additional_forces.c:14-121) on the device.

calculate_accelerations adds them when the stored speed of light C is
positive (src/common.c:101-107), and Radau15 then integrates with them:
bit-identical accelerations in the exact form, trajectories at a common
time to 1e-10, against the reference's golden vectors and the oracle.
Both Radau15 engines carry them: the split engine (at most 10 massive
bodies) and the general one."""
import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL, TIME_TOL_FAST, TOL, at_time

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR


def _accelerations(sim, p, v, m):
    import ctypes as C
    acc = np.zeros(p.size)
    p, v, m = np.ascontiguousarray(p), np.ascontiguousarray(v), np.ascontiguousarray(m)
    r = np.zeros(m.size)
    rc = sim.lib.calculate_accelerations(C.c_void_p(p.ctypes.data), C.c_void_p(v.ctypes.data),
                                         C.c_size_t(m.size), C.c_double(G), C.c_void_p(m.ctypes.data),
                                         C.c_void_p(r.ctypes.data), C.c_void_p(acc.ctypes.data))
    assert rc == 0
    return acc


@pytest.mark.parametrize("mode,tol", [("exact", 0.0), ("fp64", 1e-13)])
def test_pn_accelerations_golden(sim, golden, mode, tol):
    p, v, m, Cl = golden["pn_in_pos"], golden["pn_in_vel"], golden["pn_m"], golden["pn_C"][0]
    sim.set_state(p, v, m, np.zeros(m.size), m.size, G, Cl)
    old = sim.set_force_mode(mode)
    try:
        acc = _accelerations(sim, p, v, m)
    finally:
        sim.set_force_mode(old)
        sim.set_state(p, v, m, np.zeros(m.size), m.size, G, 0.0)
    if tol == 0.0:
        assert np.array_equal(acc, golden["pn_acc"])
    else:
        assert rel_err_per_body(acc, golden["pn_acc"]) <= tol


@pytest.mark.parametrize("mode,tol_t", [("exact", TIME_TOL), ("fp64", TIME_TOL_FAST)])
def test_pn_radau_golden(sim, oracle, golden, mode, tol_t):
    p, v, m, Cl = golden["pn_in_pos"], golden["pn_in_vel"], golden["pn_m"], golden["pn_C"][0]
    old = sim.set_force_mode(mode)
    try:
        sim.set_state(p, v, m, np.zeros(m.size), m.size, G, Cl)
        sim.integrator_gr(0.0, 2.0, 1.0)
        pos, vel = np.zeros(p.size), np.zeros(p.size)
        sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
        t = sim.get_model_time()
    finally:
        sim.set_force_mode(old)
        sim.set_state(p, v, m, np.zeros(m.size), m.size, G, 0.0)
    t_ref = golden["pn_gr_t"][0]
    assert abs(t - t_ref) <= tol_t * t_ref
    # the Newtonian Taylor shift is enough over the tiny time offset
    pos, vel = at_time(pos, vel, m, t, t_ref, oracle)
    assert rel_err_per_body(pos, golden["pn_gr_pos"]) <= TOL
    assert rel_err_per_body(vel, golden["pn_gr_vel"]) <= TOL


def test_pn_radau_with_test_particle_vs_oracle(sim, oracle):
    """A star, four planets and one massless body (the reference's pair loop
    turns a second massless body into 0/0)."""
    p, v, m, r = ics.planetary_system(seed=85, n_planets=4, n_tp=1)
    Cl = 63239.7263
    ref = oracle.radau15(p, v, m, r, G, 0.0, 1.0, C=Cl)
    old = sim.set_force_mode("exact")
    try:
        sim.set_state(p, v, m, r, m.size, G, Cl)
        sim.integrator_gr(0.0, 1.0, 1.0)
        pos, vel = np.zeros(p.size), np.zeros(p.size)
        sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
        t = sim.get_model_time()
    finally:
        sim.set_force_mode(old)
        sim.set_state(p, v, m, r, m.size, G, 0.0)
    assert abs(t - ref["t"]) <= TIME_TOL * ref["t"]
    pos, vel = at_time(pos, vel, m, t, ref["t"], oracle)
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL


@pytest.mark.parametrize("mode,tol_t", [("exact", TIME_TOL), ("fp64", TIME_TOL_FAST)])
def test_pn_general_engine_vs_oracle(sim, oracle, mode, tol_t):
    """Twelve planets (13 massive bodies: beyond the split engine) and
    one test particle (the reference turns a second massless body into
    0/0), post-Newtonian terms on the general engine."""
    p, v, m, r = ics.planetary_system(seed=86, n_planets=12, n_tp=1)
    Cl = 63239.7263
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.3, C=Cl)
    newton = oracle.radau15(p, v, m, r, G, 0.0, 0.3)
    old = sim.set_force_mode(mode)
    try:
        sim.set_state(p, v, m, r, m.size, G, Cl)
        sim.integrator_gr(0.0, 0.3, 1.0)
        pos, vel = np.zeros(p.size), np.zeros(p.size)
        sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
        t = sim.get_model_time()
    finally:
        sim.set_force_mode(old)
        sim.set_state(p, v, m, r, m.size, G, 0.0)
    assert abs(t - ref["t"]) <= tol_t * ref["t"]
    pos, vel = at_time(pos, vel, m, t, ref["t"], oracle)
    assert rel_err_per_body(pos, ref["pos"]) <= TOL and rel_err_per_body(vel, ref["vel"]) <= TOL
    # the terms matter at this tolerance (about 3e-7 here)
    npos, nvel = at_time(newton["pos"], newton["vel"], m, newton["t"], ref["t"], oracle)
    assert rel_err_per_body(nvel, ref["vel"]) > 100 * TOL


@pytest.mark.parametrize("n", [3, 9, 37])
def test_pn_accelerations_fast_form_sizes(sim, oracle, n):
    """calculate_accelerations with C > 0 at sizes that leave the fast
    kernel's blocks of 8 sinks part-filled, one massless body among them:
    the fast form (one warp per sink, the regrouped pair term) agrees with
    the exact form to 1e-13 per body, and the exact form with the oracle's
    Newton + post-Newtonian sum bit for bit."""
    p, v, m, r = ics.planetary_system(seed=800 + n, n_planets=n - 2, n_tp=1)
    Cl = 63239.7263
    sim.set_state(p, v, m, np.zeros(m.size), m.size, G, Cl)
    try:
        out = {}
        for mode in ("exact", "fp64"):
            old = sim.set_force_mode(mode)
            try:
                out[mode] = _accelerations(sim, p, v, m)
            finally:
                sim.set_force_mode(old)
    finally:
        sim.set_state(p, v, m, np.zeros(m.size), m.size, G, 0.0)
    ref = oracle.post_newtonian(p, v, m, G, Cl, acc=oracle.force(p, m, G))
    assert np.array_equal(out["exact"], ref)
    assert rel_err_per_body(out["fp64"], out["exact"]) <= 1e-13
