"""Gauss-Radau 15 on the device against the reference's golden trajectories
and the oracle.

The device sweep repeats the reference's arithmetic per component; the
exact force form reproduces its accelerations bit for bit, but the step-size
exponentiation uses the device pow(), whose last bit can differ from the
host libm's.  The step size is h / err, so a last-bit change moves every
later step and the time at which the integrator stops past t_end (by up to
~1e-9 relative here).  Trajectories are therefore compared at a common
time: the device's final state is carried to the reference's final time by
a second-order Taylor step (|dt| ~ 1e-9, so the neglected term is ~1e-27),
and then positions and velocities must agree to 1e-10 relative, max over
bodies (measured: 1e-15 .. 6e-12 for the same 1-ulp perturbation injected
into the oracle's pow).  Final times agree to 1e-8 relative; event flags,
counts and body indices exactly."""
import numpy as np
import pytest

from abie_gb300 import ics
from abie_gb300.clibabie import CLibABIE
from abie_gb300.events import CloseEncounterException, CollisionException
from conftest import rel_err_per_body

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
TOL = 1e-10
TIME_TOL = 1e-8       # exact force form: the stop times differ only through pow's last bit
TIME_TOL_FAST = 1e-5  # fast form: b6 sits near round-off, so step sizes carry that noise
GR_CASES = ["gr_sys", "gr_tp", "gr_ens0", "gr_ens1", "gr_ens2"]


def _jerk(pos, vel, m):
    p, v = pos.reshape(-1, 3), vel.reshape(-1, 3)
    src = m > 0
    d = p[:, None, :] - p[None, src, :]
    w = v[:, None, :] - v[None, src, :]
    r2 = (d * d).sum(-1)
    ok = r2 > 0
    r2s = np.where(ok, r2, 1.0)
    inv3 = np.where(ok, r2s ** -1.5, 0.0)
    rv = (d * w).sum(-1)
    term = w * inv3[..., None] - 3.0 * rv[..., None] * d * (inv3 / r2s)[..., None]
    return (-G * (m[src][None, :, None] * term).sum(1)).reshape(-1)


def at_time(pos, vel, m, t_from, t_to, oracle):
    """Carry a state from t_from to t_to with a third-order Taylor step
    (acceleration from the oracle, analytic jerk)."""
    dt = t_to - t_from
    acc = oracle.force(pos, m, G)
    jrk = _jerk(pos, vel, m)
    return (pos + vel * dt + 0.5 * acc * dt * dt + jrk * dt ** 3 / 6.0,
            vel + acc * dt + 0.5 * jrk * dt * dt)


def _direct(clib, pos, vel, m, r, t0, t1, mode):
    """integrator_gauss_radau15 on caller arrays (src/integrator_gauss_radau15.c:221)."""
    import ctypes as C
    lib = clib.lib
    old = clib.set_force_mode(mode)
    p, v = np.array(pos, dtype=np.float64), np.array(vel, dtype=np.float64)
    mm, rr = np.array(m, dtype=np.float64), np.array(r, dtype=np.float64)
    lib.integrator_gauss_radau15.restype = C.c_ssize_t
    rc = lib.integrator_gauss_radau15(C.c_void_p(p.ctypes.data), C.c_void_p(v.ctypes.data),
                                      C.c_void_p(mm.ctypes.data), C.c_void_p(rr.ctypes.data),
                                      C.c_size_t(mm.size), C.c_double(G), C.c_double(t0),
                                      C.c_double(t1), C.c_double(1.0))
    clib.set_force_mode(old)
    return rc, p, v, lib.get_model_time()


@pytest.mark.parametrize("mode", ["exact", "fp64"])
@pytest.mark.parametrize("case", GR_CASES)
def test_golden_trajectories(clib, oracle, golden, case, mode):
    span = golden[case + "_span"]
    m = golden[case + "_m"]
    rc, p, v, t = _direct(clib, golden[case + "_in_pos"], golden[case + "_in_vel"],
                          m, golden[case + "_r"], span[0], span[1], mode)
    assert rc == 0
    t_ref = golden[case + "_t"][0]
    assert abs(t - t_ref) <= (TIME_TOL if mode == "exact" else TIME_TOL_FAST) * abs(t_ref)
    p, v = at_time(p, v, m, t, t_ref, oracle)
    assert rel_err_per_body(p, golden[case + "_pos"]) <= TOL
    assert rel_err_per_body(v, golden[case + "_vel"]) <= TOL


def test_energy_conservation_cfg1(clib, oracle):
    """1,009-body workload over 5 yr: energy drift at the reference's level."""
    p, v, m, r = ics.planetary_system()
    rc, p1, v1, t = _direct(clib, p, v, m, r, 0.0, 5.0, "fp64")
    assert rc == 0 and t > 5.0
    e0 = oracle.energy(p, v, m, G)
    e1 = oracle.energy(p1, v1, m, G)
    assert abs((e1 - e0) / e0) < 1e-13


def test_cfg1_against_oracle_short(clib, oracle):
    p, v, m, r = ics.planetary_system()
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.5)
    rc, p1, v1, t = _direct(clib, p, v, m, r, 0.0, 0.5, "exact")
    assert rc == 0
    assert abs(t - ref["t"]) <= TIME_TOL * ref["t"]
    p1, v1 = at_time(p1, v1, m, t, ref["t"], oracle)
    assert rel_err_per_body(p1, ref["pos"]) <= TOL
    assert rel_err_per_body(v1, ref["vel"]) <= TOL


@pytest.mark.parametrize("case,exc_type", [("gr_ce", CloseEncounterException),
                                           ("gr_coll", CollisionException)])
def test_events_through_integrator_gr(sim, oracle, golden, case, exc_type):
    """Close-encounter / collision flag, counts and ring buffers via the
    stateful reference entry points (initialize_code, set_state, integrator_gr)."""
    span = golden[case + "_span"]
    old = sim.set_force_mode("exact")
    sim.set_close_encounter_distance(span[2])
    sim.reset_close_encounter_buffer()
    sim.reset_collision_buffer()
    m = golden[case + "_m"]
    sim.set_state(golden[case + "_in_pos"], golden[case + "_in_vel"], m, golden[case + "_r"],
                  m.size, G, 0.0)
    with pytest.raises(exc_type) as exc:
        sim.integrator_gr(span[0], span[1], 1.0)
    if case == "gr_ce":
        buf, gold = sim.get_close_encounter_data().reshape(-1), golden[case + "_buf_ce"]
    else:
        buf, gold = sim.get_collision_data().reshape(-1), golden[case + "_buf_coll"]
    assert np.array_equal(buf[1::4], gold[1::4]) and np.array_equal(buf[2::4], gold[2::4])
    assert np.allclose(buf, gold, rtol=TIME_TOL, atol=0)
    assert exc.value.obj1 == int(gold[-3]) and exc.value.obj2 == int(gold[-2])
    pos, vel = np.zeros(3 * m.size), np.zeros(3 * m.size)
    assert sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size)) == m.size
    t, t_ref = sim.get_model_time(), golden[case + "_t"][0]
    assert abs(t - t_ref) <= TIME_TOL * t_ref
    pos, vel = at_time(pos, vel, m, t, t_ref, oracle)
    assert rel_err_per_body(pos, golden[case + "_pos"]) <= TOL
    sim.set_force_mode(old)
    sim.set_close_encounter_distance(0.0)
    sim.reset_close_encounter_buffer()
    sim.reset_collision_buffer()


def test_stateful_chunked_run_matches_oracle(sim, oracle):
    """The Python driver's store_dt chunking (abie/integrator.py:181-188):
    every chunk restarts Radau15 from the stored state."""
    p, v, m, r = ics.planetary_system(seed=9, n_planets=5, n_tp=20)
    sim.set_force_mode("exact")
    sim.set_state(p, v, m, r, m.size, G, 0.0)
    ref_p, ref_v, t_ref = p.copy(), v.copy(), 0.0
    t, t_end, dt = 0.0, 3.0, 1.0
    while t < t_end:
        next_t = t + dt - ((t + dt) % dt)
        sim.integrator_gr(t, next_t, 1.0)
        t = sim.get_model_time()
        out = oracle.radau15(ref_p, ref_v, m, r, G, t_ref, next_t)
        ref_p, ref_v, t_ref = out["pos"], out["vel"], out["t"]
    sim.set_force_mode("fp64")
    pos, vel = np.zeros(p.size), np.zeros(p.size)
    sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
    assert abs(t - t_ref) <= TIME_TOL_FAST * t_ref
    pos, vel = at_time(pos, vel, m, t, t_ref, oracle)
    assert rel_err_per_body(pos, ref_p) <= TOL and rel_err_per_body(vel, ref_v) <= TOL


def test_counters_reported(clib):
    clib.reset_counters()
    p, v, m, r = ics.planetary_system(seed=3, n_planets=3, n_tp=0)
    _direct(clib, p, v, m, r, 0.0, 1.0, "fp64")
    c = clib.counters()
    assert c["accepts"] > 0 and c["attempts"] == c["accepts"] + c["rejects"]
    assert c["force_calls"] >= 7 * c["iterations"] + c["attempts"]


@pytest.mark.parametrize("n_planets,n_tp", [(9, 40), (10, 40), (3, 0), (0, 30)])
def test_split_and_general_engines_vs_oracle(clib, oracle, n_planets, n_tp):
    """Systems at and beyond the split engine's limit (10 massive bodies),
    without test particles, and without massive bodies but the star (a
    lone star plus massless bodies), in both forms, against the oracle."""
    p, v, m, r = ics.planetary_system(seed=77 + n_planets, n_planets=n_planets, n_tp=n_tp)
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.4)
    for mode, tol_t in (("exact", TIME_TOL), ("fp64", TIME_TOL_FAST)):
        rc, p1, v1, t = _direct(clib, p, v, m, r, 0.0, 0.4, mode)
        assert rc == 0
        assert abs(t - ref["t"]) <= tol_t * ref["t"]
        p1, v1 = at_time(p1, v1, m, t, ref["t"], oracle)
        assert rel_err_per_body(p1, ref["pos"]) <= TOL
        assert rel_err_per_body(v1, ref["vel"]) <= TOL


def test_split_engine_matches_general_engine(clib, oracle):
    """The same 1,009-body run on the split engine and, with a forced launch
    shape, on the general engine: equal at a common time."""
    import ctypes as C
    p, v, m, r = ics.planetary_system()
    rc, p1, v1, t1 = _direct(clib, p, v, m, r, 0.0, 0.3, "fp64")
    clib.lib.abie_debug_engine_shape(C.c_int(16), C.c_int(128))
    try:
        rc2, p2, v2, t2 = _direct(clib, p, v, m, r, 0.0, 0.3, "fp64")
    finally:
        clib.lib.abie_debug_engine_shape(C.c_int(0), C.c_int(0))
    assert rc == 0 and rc2 == 0
    assert abs(t1 - t2) <= TIME_TOL_FAST * t2
    p1, v1 = at_time(p1, v1, m, t1, t2, oracle)
    assert rel_err_per_body(p1, p2) <= TOL and rel_err_per_body(v1, v2) <= TOL


def _threshold_pairs(ce, n_planets=3):
    """planetary_system(seed=5, n_planets, 300 test particles) plus four
    test-particle pairs at 30 au, each pair the same orbit offset out of the
    plane: two pairs 1e-4 inside the close-encounter distance ce and two
    1e-4 outside it (over a step the offsets change by ~1e-6)."""
    p, v, m, r = ics.planetary_system(seed=5, n_planets=n_planets, n_tp=300)
    extra_p, extra_v = [], []
    vc = np.sqrt(G * m[0] / 30.0)
    for q, scale in enumerate((1 - 1e-4, 1 + 1e-4, 1 - 1e-4, 1 + 1e-4)):
        ang = 0.5 * np.pi * q + 0.3
        x = np.array([30.0 * np.cos(ang), 30.0 * np.sin(ang), 0.0])
        u = np.array([-vc * np.sin(ang), vc * np.cos(ang), 0.0])
        extra_p += [x, x + np.array([0.0, 0.0, ce * scale])]
        extra_v += [u, u]
    p = np.concatenate([p, np.concatenate(extra_p)])
    v = np.concatenate([v, np.concatenate(extra_v)])
    m = np.concatenate([m, np.zeros(8)])
    r = np.concatenate([r, np.zeros(8)])
    return p, v, m, r


@pytest.mark.parametrize("engine", ["split", "general", "stepped"])
def test_event_prefilter_at_threshold(sim, oracle, engine):
    """Pairs 1e-4 inside and outside the close-encounter distance, among
    hundreds of far-apart bodies that the single-precision prefilter skips:
    the inside pairs are recorded, the outside ones are not, on every
    engine (the stepped one with 12 planets, beyond the split engine); the
    flag, ring buffer and stop time equal the oracle's."""
    import ctypes as C
    ce = 0.01
    p, v, m, r = _threshold_pairs(ce, n_planets=12 if engine == "stepped" else 3)
    ref = oracle.radau15(p, v, m, r, G, 0.0, 10.0, ce_dist=ce, max_ce=3, max_coll=2)
    assert ref["flag"] == 1 and ref["n_ce"] == 4  # two pairs in each of two steps
    n0 = m.size - 8
    gold = ref["buf_ce"].reshape(-1, 4)
    assert sorted(set(map(int, gold[:, 1]))) == [n0, n0 + 4]
    # the stepped engine runs the fast form; the others the exact one
    old = sim.set_force_mode("fp64" if engine == "stepped" else "exact")
    sim.set_close_encounter_distance(ce)
    sim.reset_close_encounter_buffer()
    sim.reset_collision_buffer()
    if engine == "general":
        sim.lib.abie_debug_engine_shape(C.c_int(16), C.c_int(128))
    if engine == "stepped":
        sim.lib.abie_debug_radau_path(C.c_int(2))
    try:
        sim.set_state(p, v, m, r, m.size, G, 0.0)
        with pytest.raises(CloseEncounterException):
            sim.integrator_gr(0.0, 10.0, 1.0)
        buf = sim.get_close_encounter_data()
        t = sim.get_model_time()
    finally:
        sim.lib.abie_debug_engine_shape(C.c_int(0), C.c_int(0))
        sim.lib.abie_debug_radau_path(C.c_int(0))
        sim.set_force_mode(old)
        sim.set_close_encounter_distance(0.0)
        sim.reset_close_encounter_buffer()
        sim.reset_collision_buffer()
    t_tol, sep_tol = (TIME_TOL_FAST, 1e-8) if engine == "stepped" else (TIME_TOL, 1e-12)
    assert np.array_equal(buf[:, 1:3], gold[:, 1:3])
    assert np.allclose(buf[:, 0], gold[:, 0], rtol=t_tol, atol=0)
    assert np.allclose(buf[:, 3], gold[:, 3], rtol=sep_tol, atol=0)
    assert abs(t - ref["t"]) <= t_tol * ref["t"]


def test_stepped_engine_matches_persistent_engine(clib):
    """The stepped engine (one kernel per phase, the standalone force kernel
    for every substep; chosen automatically from 2^20 interactions per
    force evaluation) and the persistent engine with 32 lanes per body run
    the same arithmetic in the same order: a 2,049-body all-massive disk
    over 0.05 yr in the fast form gives the same doubles."""
    import ctypes as C
    p, v, m, r = ics.planetesimal_disk(seed=33, n=2048)
    clib.lib.abie_debug_radau_path(C.c_int(2))
    try:
        rc1, p1, v1, t1 = _direct(clib, p, v, m, r, 0.0, 0.05, "fp64")
        c1 = clib.counters()
    finally:
        clib.lib.abie_debug_radau_path(C.c_int(0))
    clib.lib.abie_debug_radau_path(C.c_int(1))
    clib.lib.abie_debug_engine_shape(C.c_int(32), C.c_int(256))
    try:
        rc2, p2, v2, t2 = _direct(clib, p, v, m, r, 0.0, 0.05, "fp64")
    finally:
        clib.lib.abie_debug_radau_path(C.c_int(0))
        clib.lib.abie_debug_engine_shape(C.c_int(0), C.c_int(0))
    assert rc1 == 0 and rc2 == 0
    assert t1 == t2 and t1 >= 0.05
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2)
