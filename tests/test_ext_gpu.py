"""External accelerations (set_additional_forces, src/common.c:364-380) on
the GPU path against the reference's golden vectors.

The reference adds the stored 3N vector to every force evaluation of
calculate_accelerations (src/common.c:107-112), so it reaches the
accelerations of that entry point and every force call of Radau15.  The
golden run (tests/golden/golden_ext.npz, from the unmodified reference
library) is a 26-body planetary system with a random vector of 1e-3
au/yr^2 per component over 2 yr.  Exact form: the accelerations bit for
bit; trajectories at a common time within 1e-10 (the step-size pow's last
bit moves the stop time, as in the other Radau15 tests)."""
import ctypes as C
import os

import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL, TIME_TOL_FAST, TOL, _direct, at_time

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_ext.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _accelerations(clib, p, v, m, mode):
    lib = clib.lib
    old = clib.set_force_mode(mode)
    acc = np.zeros(p.size)
    try:
        rc = lib.calculate_accelerations(C.c_void_p(p.ctypes.data), C.c_void_p(v.ctypes.data),
                                         C.c_size_t(m.size), C.c_double(G),
                                         C.c_void_p(m.ctypes.data),
                                         C.c_void_p(np.zeros(m.size).ctypes.data),
                                         C.c_void_p(acc.ctypes.data))
    finally:
        clib.set_force_mode(old)
    assert rc == 0
    return acc


@pytest.mark.parametrize("mode", ["exact", "fp64"])
def test_external_accelerations(sim, oracle, gold, mode):
    p, v, m, r, ext = (np.array(gold[k]) for k in ("ext_in_pos", "ext_in_vel", "ext_m", "ext_r",
                                                   "ext_acc_in"))
    t0, t1 = gold["ext_span"]
    sim.set_additional_forces(ext)
    try:
        acc = _accelerations(sim, p, v, m, mode)
        if mode == "exact":
            assert np.array_equal(acc, gold["ext_accel"])
        else:
            assert rel_err_per_body(acc, gold["ext_accel"]) <= 1e-13
        # stateful integrator_gr on the stored state
        old = sim.set_force_mode(mode)
        try:
            sim.set_state(p, v, m, r, m.size, G, 0.0)
            sim.integrator_gr(t0, t1, 1.0)
            P, V = np.zeros(p.size), np.zeros(v.size)
            sim.get_state(P, V, np.zeros(m.size), np.zeros(m.size))
            t = sim.get_model_time()
        finally:
            sim.set_force_mode(old)
        # integrator_gauss_radau15 on caller arrays adds them too
        rc, P2, V2, t2 = _direct(sim, p, v, m, r, t0, t1, mode)
        assert rc == 0
    finally:
        sim.set_additional_forces(None)
    t_ref = gold["ext_gr_t"][0]
    ttol = TIME_TOL if mode == "exact" else TIME_TOL_FAST
    for PP, VV, tt in ((P, V, t), (P2, V2, t2)):
        assert abs(tt - t_ref) <= ttol * t_ref
        pp, vv = at_time(PP, VV, m, tt, t_ref, oracle)
        # the shift to the common time carries the external term too
        dt = t_ref - tt
        pp, vv = pp + 0.5 * ext * dt * dt, vv + ext * dt
        assert rel_err_per_body(pp, gold["ext_gr_pos"]) <= TOL
        assert rel_err_per_body(vv, gold["ext_gr_vel"]) <= TOL
    # switched off, the library integrates without the vector again
    rc, P3, V3, t3 = _direct(sim, p, v, m, r, t0, t1, mode)
    ref = oracle.radau15(p, v, m, r, G, t0, t1)
    p3, v3 = at_time(P3, V3, m, t3, ref["t"], oracle)
    assert rel_err_per_body(p3, ref["pos"]) <= TOL
