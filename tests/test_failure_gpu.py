"""Failure detection on the GPU path, without faulting the GPU.

* Every grid-barrier wait of the persistent Radau15 engines has a time
  limit.  With the limit set to zero (abie_debug_engine_timeout), the first
  block that has to wait for the others gives up, the run stops with
  ABIE_ERR_TIMEOUT and every block leaves at its next barrier; the context
  stays usable, and the next run with the automatic limit matches the
  oracle.
* A non-finite state stops Radau15 with ABIE_ERR_NUMERICS (the host reads
  the status); the library keeps working afterwards.
The failure is made on the host (a zero limit, a NaN in the input): no test
here traps, faults or hangs the GPU."""
import ctypes as C

import numpy as np
import pytest

from abie_gb300 import ics
from abie_gb300.events import AbieError
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL, TOL, at_time

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
ERR_TIMEOUT = -7
ERR_NUMERICS = -8


def _run(sim, p, v, m, r, t1, mode="exact"):
    old = sim.set_force_mode(mode)
    try:
        sim.set_state(p, v, m, r, m.size, G, 0.0)
        sim.integrator_gr(0.0, t1, 1.0)
        P, V = np.zeros(p.size), np.zeros(v.size)
        sim.get_state(P, V, np.zeros(m.size), np.zeros(m.size))
        return P, V, sim.get_model_time()
    finally:
        sim.set_force_mode(old)


@pytest.mark.parametrize("workload", ["split-1009", "engine-2049"])
def test_barrier_wait_limit_stops_the_run(sim, oracle, workload):
    if workload == "split-1009":   # 9 massive bodies: the split engine
        p, v, m, r = ics.planetary_system(seed=31, n_planets=8, n_tp=1000)
        path = 0
    else:                          # every body massive: the persistent engine
        p, v, m, r = ics.planetesimal_disk(seed=32, n=2048)
        path = 1
    lib = sim.lib
    lib.abie_debug_radau_path(C.c_int(path))
    lib.abie_debug_engine_timeout(C.c_longlong(0))
    try:
        with pytest.raises(AbieError) as exc:
            _run(sim, p, v, m, r, 0.05)
        assert exc.value.code == ERR_TIMEOUT
    finally:
        lib.abie_debug_engine_timeout(C.c_longlong(-1))
    try:
        P, V, t = _run(sim, p, v, m, r, 0.05)
    finally:
        lib.abie_debug_radau_path(C.c_int(0))
    ref = oracle.radau15(p, v, m, r, G, 0.0, 0.05)
    assert abs(t - ref["t"]) <= TIME_TOL * ref["t"]
    P, V = at_time(P, V, m, t, ref["t"], oracle)
    assert rel_err_per_body(P, ref["pos"]) <= TOL


@pytest.mark.parametrize("mode", ["exact", "fp64"])
def test_nonfinite_state_stops_radau(sim, oracle, mode):
    p, v, m, r = ics.planetary_system(seed=33, n_planets=6, n_tp=40)
    bad = p.copy()
    bad[3 * 7 + 1] = np.nan
    with pytest.raises(AbieError) as exc:
        _run(sim, bad, v, m, r, 0.2, mode)
    assert exc.value.code == ERR_NUMERICS
    # the library keeps working
    P, V, t = _run(sim, p, v, m, r, 0.2, mode)
    assert np.isfinite(P).all() and t > 0.2
