"""Device snapshots (abie_integrate_snapshots) against the same chunks run
through the library's stateful entry points one at a time, as the
reference's Integrator.integrate drives them (integrator_gr / integrator_wh,
get_state, get_model_time, get_total_energy), with the elements from the
oracle's restatement of Particles.calculate_aei."""
import numpy as np
import pytest

from abie_gb300 import ics
from oracle import snapshots as S

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR


def _host_loop(sim, p, v, m, r, t, t_end, store_dt, integrator, h, primary):
    sim.set_state(p, v, m, r, m.size, G, 0.0)
    snaps = []

    def advance(t0, t1):
        if integrator == "gr":
            sim.integrator_gr(t0, t1, 1.0)
        else:
            sim.integrator_wh(t0, t1, h)
        pos, vel = np.zeros(p.size), np.zeros(p.size)
        sim.get_state(pos, vel, np.zeros(m.size), np.zeros(m.size))
        tt = sim.get_model_time()
        snaps.append((tt, pos, vel, sim.get_total_energy()))
        return tt

    ends = S.chunk_ends(t, t_end, store_dt, advance)
    return ends, snaps


def _elements_close(aei, ref):
    a, e, i = aei[..., 0], aei[..., 1], aei[..., 2]
    ra, re, ri = ref[..., 0], ref[..., 1], ref[..., 2]
    assert np.array_equal(np.isnan(aei), np.isnan(ref))
    ok = ~np.isnan(ra)
    assert np.allclose(a[ok], ra[ok], rtol=1e-12, atol=0)
    assert np.allclose(e[ok], re[ok], rtol=1e-9, atol=1e-14)
    assert np.allclose(i[ok], ri[ok], rtol=0, atol=1e-10)


@pytest.mark.parametrize("integrator,primary", [("gr", "#COM#"), ("gr", "#M_MAX#"), ("wh", 2)])
def test_snapshots_match_host_loop(sim, integrator, primary):
    if integrator == "gr":
        p, v, m, r = ics.planetary_system(seed=93, n_planets=5, n_tp=30)
        h = 0.0
    else:
        p, v, m, r = ics.test_particle_swarm(seed=94, n_tp=500)
        p, v = ics.to_heliocentric(p, v)
        h = 0.01
    t, t_end, store_dt = 0.0, 1.0, 0.25
    ends, host = _host_loop(sim, p, v, m, r, t, t_end, store_dt, integrator, h, primary)
    sim.set_state(p, v, m, r, m.size, G, 0.0)
    out = sim.integrate_snapshots(t, t_end, store_dt, integrator=integrator, h=h, primary=primary)
    assert out["flag"] == 0 and len(out["t"]) == len(host) == len(ends)
    prim = {"#COM#": S.PRIMARY_COM, "#M_MAX#": S.PRIMARY_M_MAX}.get(primary, primary)
    for q, (tt, pos, vel, en) in enumerate(host):
        # the same device computation in the same order: identical
        assert out["t"][q] == tt and out["energy"][q] == en
        assert np.array_equal(out["pos"][q], pos) and np.array_equal(out["vel"][q], vel)
        _elements_close(out["aei"][q], S.calculate_aei(pos, vel, m, G, prim))
    if primary == "#M_MAX#":
        assert np.isnan(out["aei"][:, 0, :]).all()  # the star about itself


def test_snapshot_capacity_and_arguments(sim):
    from abie_gb300.events import AbieError
    p, v, m, r = ics.planetary_system(seed=95, n_planets=3, n_tp=5)
    sim.set_state(p, v, m, r, m.size, G, 0.0)
    with pytest.raises(AbieError):
        sim.integrate_snapshots(0.0, 1.0, 0.1, max_snaps=3)  # ten chunks needed
    with pytest.raises(AbieError):
        sim.integrate_snapshots(0.0, 1.0, 0.1, primary=m.size)
    with pytest.raises(AbieError):
        sim.integrate_snapshots(0.0, 1.0, 0.1, integrator="wh", h=0.0)


def test_snapshots_stop_at_an_event(sim):
    """A close encounter ends the run after its chunk's snapshot, with the
    integrator's flag (the caller handles the event, then continues)."""
    from test_radau_gpu import _threshold_pairs
    ce = 0.01
    p, v, m, r = _threshold_pairs(ce)
    sim.set_close_encounter_distance(ce)
    sim.reset_close_encounter_buffer()
    sim.reset_collision_buffer()
    try:
        sim.set_state(p, v, m, r, m.size, G, 0.0)
        out = sim.integrate_snapshots(0.0, 1.0, 0.25)
    finally:
        sim.set_close_encounter_distance(0.0)
        sim.reset_close_encounter_buffer()
        sim.reset_collision_buffer()
    assert out["flag"] == 1
    assert len(out["t"]) == 1 and 0.0 < out["t"][0] < 0.25  # inside the first chunk
    assert out["t"][0] == sim.get_model_time()
