"""Batched Radau15 ensemble: each system is integrated as integrator_gr would
integrate it alone.  Compared at a common time (see test_radau_gpu.py) to
the reference's golden runs and to the oracle; energy conservation over the
batch; a system with a non-finite state is reported without disturbing the
others."""
import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body
from test_radau_gpu import TIME_TOL, TIME_TOL_FAST, TOL, at_time

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR


def _pack(systems):
    P = np.concatenate([s[0] for s in systems])
    V = np.concatenate([s[1] for s in systems])
    M = np.concatenate([s[2] for s in systems])
    offs = np.concatenate([[0], np.cumsum([s[2].size for s in systems])]).astype(np.int64)
    return P, V, M, offs


def _sl(offs, s):
    return slice(3 * offs[s], 3 * offs[s + 1]), slice(offs[s], offs[s + 1])


TIME_TOLS = {"exact": TIME_TOL, "fp64": TIME_TOL_FAST, "naive": TIME_TOL_FAST,
             "mixed": TIME_TOL_FAST}


@pytest.mark.parametrize("mode", ["exact", "fp64", "naive", "mixed"])
def test_golden_systems(clib, oracle, golden, mode):
    cases = ["gr_ens0", "gr_ens1", "gr_ens2"]
    systems = [(golden[c + "_in_pos"], golden[c + "_in_vel"], golden[c + "_m"]) for c in cases]
    P, V, M, offs = _pack(systems)
    old = clib.set_force_mode(mode)
    try:
        out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 20.0)
    finally:
        clib.set_force_mode(old)
    assert (out["status"] == 0).all()
    for s, c in enumerate(cases):
        sv, sm = _sl(offs, s)
        t_ref = golden[c + "_t"][0]
        assert abs(out["t"][s] - t_ref) <= TIME_TOLS[mode] * t_ref
        p, v = at_time(out["pos"][sv], out["vel"][sv], M[sm], out["t"][s], t_ref, oracle)
        assert rel_err_per_body(p, golden[c + "_pos"]) <= TOL
        assert rel_err_per_body(v, golden[c + "_vel"]) <= TOL


def test_random_batch_vs_oracle(clib, oracle):
    P, V, M, offs = ics.ensemble(n_systems=48, seed0=500)
    out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.5)
    assert (out["status"] == 0).all()
    for s in range(48):
        sv, sm = _sl(offs, s)
        ref = oracle.radau15(P[sv], V[sv], M[sm], np.zeros(M[sm].size), G, 0.0, 0.5)
        assert abs(out["t"][s] - ref["t"]) <= TIME_TOL_FAST * ref["t"]
        assert out["steps"][s] > 0
        p, v = at_time(out["pos"][sv], out["vel"][sv], M[sm], out["t"][s], ref["t"], oracle)
        assert rel_err_per_body(p, ref["pos"]) <= TOL
        assert rel_err_per_body(v, ref["vel"]) <= TOL


def test_energy_conservation_batch(clib, oracle):
    P, V, M, offs = ics.ensemble(n_systems=256, seed0=900)
    out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 2.0)
    assert (out["status"] == 0).all()
    worst = 0.0
    for s in range(256):
        sv, sm = _sl(offs, s)
        e0 = oracle.energy(P[sv], V[sv], M[sm], G)
        e1 = oracle.energy(out["pos"][sv], out["vel"][sv], M[sm], G)
        worst = max(worst, abs((e1 - e0) / e0))
    assert worst <= 1e-12, worst


def test_nonfinite_system_is_isolated(clib):
    P, V, M, offs = ics.ensemble(n_systems=6, seed0=77)
    P = P.copy()
    sv, _ = _sl(offs, 2)
    P[sv.start + 3] = np.nan  # planet 1 of system 2
    out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.2)
    assert out["status"][2] < 0
    others = [s for s in range(6) if s != 2]
    assert (out["status"][others] == 0).all()
    assert all(out["t"][s] > 0.2 for s in others)


def test_rejects_oversized_system(clib):
    from abie_gb300.events import AbieError
    P, V, M, offs = ics.ensemble(n_systems=1, seed0=1, n_planets=(25, 25))
    with pytest.raises(AbieError):
        clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.1)


@pytest.mark.parametrize("mode", ["exact", "fp64", "naive", "mixed"])
def test_edge_sizes_vs_oracle(clib, oracle, mode):
    """Systems of 2, 3, 10, 11 (the first two-warp size) and 21 bodies (the
    largest), each against the oracle.  (A lone body is no case: with zero
    force the reference's step control divides 0 by 0 and never ends.)"""
    systems = []
    for k, n in enumerate([2, 3, 10, 11, 21]):
        p, v, m, r = ics.planetary_system(seed=900 + k, n_planets=n - 1, n_tp=0)
        systems.append((p, v, m))
    P, V, M, offs = _pack(systems)
    old = clib.set_force_mode(mode)
    try:
        out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.3)
    finally:
        clib.set_force_mode(old)
    assert (out["status"] == 0).all()
    for s in range(len(systems)):
        sv, sm = _sl(offs, s)
        ref = oracle.radau15(P[sv], V[sv], M[sm], np.zeros(M[sm].size), G, 0.0, 0.3)
        assert abs(out["t"][s] - ref["t"]) <= TIME_TOLS[mode] * ref["t"]
        p, v = at_time(out["pos"][sv], out["vel"][sv], M[sm], out["t"][s], ref["t"], oracle)
        assert rel_err_per_body(p, ref["pos"]) <= TOL
        assert rel_err_per_body(v, ref["vel"]) <= TOL


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_every_group_class_with_test_particles(clib, oracle, mode):
    """Three 21-body and two 10-body systems, each with massless test
    particles, in the fast and mixed forms: the slowest system runs on four
    warps and at least two 21-body systems on two, so each group size
    evaluates its pairs with massless bodies on one side or both."""
    systems = []
    for k, (npl, ntp) in enumerate([(14, 6), (12, 8), (16, 4), (6, 3), (5, 4)]):
        p, v, m, r = ics.planetary_system(seed=950 + k, n_planets=npl, n_tp=ntp, tp_a=(2.0, 20.0))
        systems.append((p, v, m))
    P, V, M, offs = _pack(systems)
    old = clib.set_force_mode(mode)
    try:
        out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.3)
    finally:
        clib.set_force_mode(old)
    assert (out["status"] == 0).all()
    for s in range(len(systems)):
        sv, sm = _sl(offs, s)
        ref = oracle.radau15(P[sv], V[sv], M[sm], np.zeros(M[sm].size), G, 0.0, 0.3)
        assert abs(out["t"][s] - ref["t"]) <= TIME_TOL_FAST * ref["t"]
        p, v = at_time(out["pos"][sv], out["vel"][sv], M[sm], out["t"][s], ref["t"], oracle)
        assert rel_err_per_body(p, ref["pos"]) <= TOL
        assert rel_err_per_body(v, ref["vel"]) <= TOL


def test_forms_error_against_the_oracle(clib, oracle):
    """Each ensemble form's error against the oracle (the reference's
    algorithm on the CPU), stated and bounded: 64 systems of the benchmark
    workload over 1 yr; the state at a common time (relative, max over
    bodies and systems) and |dE/E| from the oracle's energy.

    * exact: the reference's operations (no FMA);
    * naive: the plain FP64 port (the reference's operations with FMA,
      gpuforce_v2's rsqrt pair term);
    * fp64: the fast form (Newton-form corrector, integer r^-3, pair-once);
    * mixed: the fast form with light partners' terms in FP32 two-float
      arithmetic (about 2^-46 relative to those terms)."""
    P, V, M, offs = ics.ensemble(n_systems=64, seed0=10000)
    ns = offs.size - 1
    refs = []
    for s in range(ns):
        sv, sm = _sl(offs, s)
        refs.append(oracle.radau15(P[sv], V[sv], M[sm], np.zeros(M[sm].size), G, 0.0, 1.0))
    e0 = [oracle.energy(P[_sl(offs, s)[0]], V[_sl(offs, s)[0]], M[_sl(offs, s)[1]], G)
          for s in range(ns)]
    ref_de = max(abs((oracle.energy(r["pos"], r["vel"], M[_sl(offs, s)[1]], G) - e0[s]) / e0[s])
                 for s, r in enumerate(refs))
    table = {}
    for mode in ("exact", "naive", "fp64", "mixed"):
        old = clib.set_force_mode(mode)
        try:
            out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 1.0)
        finally:
            clib.set_force_mode(old)
        assert (out["status"] == 0).all(), mode
        err, de = 0.0, 0.0
        for s in range(ns):
            sv, sm = _sl(offs, s)
            r = refs[s]
            assert abs(out["t"][s] - r["t"]) <= TIME_TOLS[mode] * r["t"], (mode, s)
            p, v = at_time(out["pos"][sv], out["vel"][sv], M[sm], out["t"][s], r["t"], oracle)
            err = max(err, rel_err_per_body(p, r["pos"]), rel_err_per_body(v, r["vel"]))
            e1 = oracle.energy(out["pos"][sv], out["vel"][sv], M[sm], G)
            de = max(de, abs((e1 - e0[s]) / e0[s]))
        table[mode] = (err, de)
    print("ensemble forms vs the oracle, 64 systems, 1 yr (max rel state error at a common time, "
          "max |dE/E|; the oracle's own max |dE/E| %.2e):" % ref_de)
    for mode, (err, de) in table.items():
        print("  %-6s %.2e  %.2e" % (mode, err, de))
    for mode, (err, de) in table.items():
        assert err <= TOL, (mode, err)
        assert de <= 1e-12, (mode, de)


def test_autotuner_times_shapes_and_caches_them(clib, tmp_path, monkeypatch):
    """The ensemble's autotuner: the first call on a workload times the
    candidate shares of four-warp groups on slices of the batch and picks
    one; the second call reads it from the cache file.  In the fast form
    a system's doubles do not depend on its group size, so every call gives
    the same result as a run with the tuner off and the chosen share."""
    import ctypes as C
    monkeypatch.setenv("ABIE_ENSEMBLE_TUNE", "1")
    monkeypatch.setenv("ABIE_TUNE_CACHE", str(tmp_path / "tune.tsv"))
    lib = clib.lib

    def tuning():
        h, src, secs = C.c_int(0), C.c_int(0), C.c_double(0)
        n = lib.abie_ensemble_last_tuning(C.byref(h), C.byref(src), C.byref(secs))
        return n, h.value, src.value, secs.value

    P, V, M, offs = ics.ensemble(n_systems=512, seed0=4000)
    old = clib.set_force_mode("fp64")
    try:
        first = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.5)
        n1, h1, src1, s1 = tuning()
        second = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.5)
        n2, h2, src2, s2 = tuning()
        monkeypatch.setenv("ABIE_ENSEMBLE_TUNE", "0")
        lib.abie_debug_ensemble_heavy(C.c_int(h1))
        try:
            plain = clib.gr_ensemble(P, V, M, offs, G, 0.0, 0.5)
        finally:
            lib.abie_debug_ensemble_heavy(C.c_int(0))
    finally:
        clib.set_force_mode(old)
    print("autotuner: %d candidates, share 1/%d, %.3f s of trials; then from the cache: 1/%d"
          % (n1, h1, s1, h2))
    assert n1 >= 4 and src1 == 0 and s1 > 0 and h1 > 0
    assert src2 == 1 and h2 == h1 and n2 == 0
    assert (tmp_path / "tune.tsv").read_text().count("\t") >= 3
    for out in (first, second):
        assert np.array_equal(out["pos"], plain["pos"]) and np.array_equal(out["t"], plain["t"])
