"""The CPU oracle is pinned bit for bit: against the golden vectors produced
by the unmodified reference library (always), and against that library live
where it can be built (skipped elsewhere)."""
import numpy as np
import pytest

from abie_gb300 import ics
from abie_gb300.radau_constants import double_tables

G = ics.G_SOLAR


def test_radau_tables_match_reference_build(golden):
    h, rs, cs = double_tables()
    assert np.array_equal(np.array(h), golden["radau_hs"])
    assert np.array_equal(np.array(rs).reshape(-1), golden["radau_rs"])
    assert np.array_equal(np.array(cs).reshape(-1), golden["radau_cs"])


@pytest.mark.parametrize("case", ["force_sys", "force_edge", "force_disk", "force_n1",
                                  "force_n2", "force_n3"])
def test_force_golden(oracle, golden, case):
    p, m = golden[case + "_pos"], golden[case + "_m"]
    acc = oracle.force(p, m, G, acc=np.zeros(p.size))
    assert np.array_equal(acc, golden[case + "_acc"])


def test_energy_golden(oracle, golden):
    e = oracle.energy(golden["force_disk_pos"], golden["energy_disk_vel"], golden["force_disk_m"], G)
    assert e == golden["energy_disk"][0]


def test_force_threads_identical(oracle, golden):
    p, m = golden["force_disk_pos"], golden["force_disk_m"]
    assert np.array_equal(oracle.force(p, m, G, threads=4), golden["force_disk_acc"])


@pytest.mark.parametrize("case", ["gr_sys", "gr_tp", "gr_ens0", "gr_ens1", "gr_ens2", "gr_ce",
                                  "gr_coll"])
def test_radau_golden(oracle, golden, case):
    span = golden[case + "_span"]
    out = oracle.radau15(golden[case + "_in_pos"], golden[case + "_in_vel"], golden[case + "_m"],
                         golden[case + "_r"], G, span[0], span[1], ce_dist=span[2],
                         max_ce=int(span[3]), max_coll=int(span[4]))
    assert np.array_equal(out["pos"], golden[case + "_pos"])
    assert np.array_equal(out["vel"], golden[case + "_vel"])
    assert out["t"] == golden[case + "_t"][0]
    flag, n_ce, n_coll = golden[case + "_flag"]
    assert (out["flag"], out["n_ce"], out["n_coll"]) == (flag, n_ce, n_coll)
    assert np.array_equal(out["buf_ce"], golden[case + "_buf_ce"])
    assert np.array_equal(out["buf_coll"], golden[case + "_buf_coll"])


@pytest.mark.parametrize("sparse", [False, True])
def test_wh_golden(oracle, golden, sparse):
    t0, t1, dt = golden["wh_span"]
    out = oracle.wh(golden["wh_in_pos"], golden["wh_in_vel"], golden["wh_m"], G, t0, t1, dt,
                    sparse=sparse)
    assert np.array_equal(out["pos"], golden["wh_pos"])
    assert np.array_equal(out["vel"], golden["wh_vel"])
    assert out["t"] == golden["wh_t"][0]


def test_post_newtonian_golden(oracle, golden):
    p, v, m, C = golden["pn_in_pos"], golden["pn_in_vel"], golden["pn_m"], golden["pn_C"][0]
    acc = oracle.post_newtonian(p, v, m, G, C, acc=oracle.force(p, m, G))
    assert np.array_equal(acc, golden["pn_acc"])
    out = oracle.radau15(p, v, m, np.zeros(m.size), G, 0.0, 2.0, C=C)
    assert np.array_equal(out["pos"], golden["pn_gr_pos"])
    assert np.array_equal(out["vel"], golden["pn_gr_vel"])
    assert out["t"] == golden["pn_gr_t"][0]


def test_live_post_newtonian(oracle, reference):
    p, v, m, r = ics.planetary_system(seed=411, n_planets=6, n_tp=0)
    C = 63239.7263
    a = oracle.post_newtonian(p, v, m, G, C, acc=oracle.force(p, m, G))
    assert np.array_equal(a, reference.accelerations(p, v, m, G, C))


def test_rk_golden(oracle, golden):
    t0, t1, dt = golden["rk_span"]
    out = oracle.rk(golden["rk_in_pos"], golden["rk_in_vel"], golden["rk_m"], G, t0, t1, dt)
    assert np.array_equal(out["pos"], golden["rk_pos"])
    assert np.array_equal(out["vel"], golden["rk_vel"])


def test_live_rk(oracle, reference):
    p, v, m, r = ics.planetary_system(seed=401, n_planets=5, n_tp=20)
    a = oracle.rk(p, v, m, G, 0.0, 0.2, 0.003)
    b = reference.rk(p, v, m, G, 0.0, 0.2, 0.003)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_live_force_energy(oracle, reference, seed):
    p, v, m, r = ics.planetary_system(seed=seed, n_planets=6, n_tp=50)
    assert np.array_equal(oracle.force(p, m, G), reference.force(p, m, G))
    assert oracle.energy(p, v, m, G) == reference.energy(p, v, m, G)


@pytest.mark.parametrize("seed", [201, 202])
def test_live_radau(oracle, reference, seed):
    p, v, m, r = ics.planetary_system(seed=seed, n_planets=4, n_tp=6)
    a = oracle.radau15(p, v, m, r, G, 0.0, 2.0)
    b = reference.radau15(p, v, m, r, G, 0.0, 2.0)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    assert a["t"] == b["t"]


def test_live_wh_sparse(oracle, reference):
    p, v, m, r = ics.test_particle_swarm(seed=301, n_tp=300)
    p, v = ics.to_heliocentric(p, v)
    a = oracle.wh(p, v, m, G, 0.0, 0.5, 0.01, sparse=True)
    b = reference.wh(p, v, m, G, 0.0, 0.5, 0.01)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_oracle_planted_mistake_is_caught(oracle, golden):
    """The golden comparison is sensitive to a last-bit change in the oracle's output."""
    p, m = golden["force_sys_pos"], golden["force_sys_m"]
    acc = oracle.force(p, m, G)
    acc[7] = np.nextafter(acc[7], np.inf)
    assert not np.array_equal(acc, golden["force_sys_acc"])


def test_external_accelerations_golden(oracle):
    """set_additional_forces: the oracle's Radau15 with a constant external
    acceleration added to every force call equals the reference's run, and
    its force plus the vector equals the reference's calculate_accelerations."""
    import os
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_ext.npz"))
    p, v, m, r, ext = (gold["ext_in_pos"], gold["ext_in_vel"], gold["ext_m"], gold["ext_r"],
                       gold["ext_acc_in"])
    acc = oracle.force(p, m, G, acc=np.zeros(p.size)) + ext
    assert np.array_equal(acc, gold["ext_accel"])
    t0, t1 = gold["ext_span"]
    out = oracle.radau15(p, v, m, r, G, t0, t1, ext=ext)
    assert np.array_equal(out["pos"], gold["ext_gr_pos"])
    assert np.array_equal(out["vel"], gold["ext_gr_vel"])
    assert out["t"] == gold["ext_gr_t"][0]
    # without the vector the run differs (the term is live)
    plain = oracle.radau15(p, v, m, r, G, t0, t1)
    assert not np.array_equal(plain["pos"], gold["ext_gr_pos"])


def test_fastform_emulation_is_the_same_integrator(oracle):
    """The oracle's emulation of the GPU fast form's arithmetic (used for the
    long-horizon energy study) integrates a planetary system to the same
    trajectory as the reference's operations: states carried to a common
    time agree to 1e-10, energy to the reference's level."""
    from abie_gb300 import ics
    G = ics.G_SOLAR
    P, V, M, offs = ics.ensemble(n_systems=1, seed0=10003)
    r = np.zeros(M.size)
    ref = oracle.radau15(P, V, M, r, G, 0.0, 1.0)
    fast = oracle.radau15(P, V, M, r, G, 0.0, 1.0, fastform=True)
    assert abs(fast["t"] - ref["t"]) <= 1e-6 * ref["t"]
    # carry the emulation's state to the reference's final time (RK4 substeps)
    x, v = fast["pos"].copy(), fast["vel"].copy()
    sub = 64
    hs = (ref["t"] - fast["t"]) / sub
    for _ in range(sub):
        a1 = oracle.force(x, M, G)
        a2 = oracle.force(x + 0.5 * hs * v, M, G)
        a3 = oracle.force(x + 0.5 * hs * v + 0.25 * hs * hs * a1, M, G)
        a4 = oracle.force(x + hs * v + 0.5 * hs * hs * a2, M, G)
        x, v = (x + hs * v + hs * hs / 6.0 * (a1 + a2 + a3),
                v + hs / 6.0 * (a1 + 2.0 * a2 + 2.0 * a3 + a4))
    d = np.linalg.norm((x - ref["pos"]).reshape(-1, 3), axis=1)
    n = np.linalg.norm(ref["pos"].reshape(-1, 3), axis=1)
    ok = n > 0
    assert np.max(d[ok] / n[ok]) <= 1e-10
    e0 = oracle.energy(P, V, M, G)
    assert abs((oracle.energy(fast["pos"], fast["vel"], M, G) - e0) / e0) <= 1e-13


def test_energy_bar_reading_on_the_committed_runs():
    """The 1e-12 energy bar at 10^4 yr on the committed runs
    (tests/golden/make_horizons.py): over the same 64 ensemble systems, one
    run each and four more moved by one unit in the last place, the fast
    form's arithmetic (the oracle's emulation) against the reference
    method.  Measured: 66.9 % of runs within 1e-12 against 69.4 %, a
    difference within one standard error of the two shares; median 5.0e-13
    against 3.4e-13, 90th percentile 4.3e-12 against 3.1e-12, 99th 8.6e-11
    against 8.2e-11.  The maxima are single runs that a close encounter
    ruins (5.1e-6 against 1.6e-8) and are not compared.  Checked: the
    shares differ by less than two standard errors, and the median, 90th
    and 99th percentiles lie within 10x of the reference method's."""
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    g = np.load(os.path.join(here, "horizon_ensemble.npz"))
    h = list(g["horizons"]).index(10000.0)
    ref = np.concatenate([g["de"][:, h],
                          np.load(os.path.join(here, "horizon_ensemble_spread.npz"))["de"].ravel()])
    f = np.load(os.path.join(here, "horizon_ensemble_fastform.npz"))
    fast = np.concatenate([f["de"], f["de_pert"].ravel()])
    assert ref.size == fast.size and ref.size >= 192
    p_ref, p_fast = (ref <= 1e-12).mean(), (fast <= 1e-12).mean()
    se = np.sqrt(p_ref * (1 - p_ref) / ref.size + p_fast * (1 - p_fast) / fast.size)
    assert p_fast >= p_ref - 2 * se
    for q in (50, 90, 99):
        assert np.percentile(fast, q) <= 10 * np.percentile(ref, q), q
