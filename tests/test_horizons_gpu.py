"""Long horizons against the reference's own runs (tests/golden/make_horizons.py).

* cfg1 over its full 100 yr: the 1,009-body planetary system (8 planets,
  1,000 test particles) through integrator_gr in the exact and fast forms,
  against the unmodified reference library's 100-yr run.  Over 100 yr the
  system amplifies rounding: the reference itself, rerun with one
  coordinate moved by one unit in the last place, ends with its planets
  1.1e-8 (relative) and its test particles up to 8.7e-9 away.  The device
  state, carried to the reference's final time, must agree per group of
  bodies within 50 times that spread (max over planets; median and 99th
  percentile over test particles), with |dE/E| at the reference's level.
* The ensemble's first 64 systems over 100 yr in the fast and mixed forms
  (the forms with the reference's operations take minutes there; they are
  checked over 1 yr in test_ensemble_gpu.py): the per-system |dE/E|
  distribution against the reference method's on the same systems (median,
  90th, 99th percentile and max within 10x of the reference's, and every
  system finished).
"""
import os

import numpy as np
import pytest

from abie_gb300 import ics
from test_radau_gpu import _direct

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture(name):
    return np.load(os.path.join(HERE, "golden", name))


def shift_to(pos, vel, m, t_from, t_to, oracle, max_sub=2e-4):
    """Carry a state from t_from to t_to by classical RK4 in substeps of at
    most max_sub yr with the oracle's accelerations: |t_to - t_from| is at
    most a fraction of an integrator step, and substeps of 2e-4 yr keep
    RK4's error below 1e-13 on orbits of 0.25 yr."""
    sub = max(8, int(np.ceil(abs(t_to - t_from) / max_sub)))
    h = (t_to - t_from) / sub
    x, v = np.array(pos, dtype=float), np.array(vel, dtype=float)
    for _ in range(sub):
        a1 = oracle.force(x, m, G)
        a2 = oracle.force(x + 0.5 * h * v, m, G)
        a3 = oracle.force(x + 0.5 * h * v + 0.25 * h * h * a1, m, G)
        a4 = oracle.force(x + h * v + 0.5 * h * h * a2, m, G)
        x, v = (x + h * v + h * h / 6.0 * (a1 + a2 + a3),
                v + h / 6.0 * (a1 + 2.0 * a2 + 2.0 * a3 + a4))
    return x, v


def _rel(a, b):
    a, b = a.reshape(-1, 3), b.reshape(-1, 3)
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


@pytest.mark.parametrize("mode", ["exact", "fp64"])
def test_cfg1_100yr_against_the_reference(clib, oracle, mode):
    gold = _fixture("horizon_cfg1.npz")
    p, v, m, r = ics.planetary_system(seed=int(gold["seed"][0]))
    t0, t1 = gold["span"]
    rc, P, V, t = _direct(clib, p, v, m, r, t0, t1, mode)
    assert rc == 0
    t_ref = gold["t"][0]
    assert abs(t - t_ref) <= 1e-3 * t_ref
    P, V = shift_to(P, V, m, t, t_ref, oracle)
    spread = _rel(gold["pert_pos"], gold["pos"])
    err = _rel(P, gold["pos"])
    massive = m > 0
    print("cfg1 100 yr, %s form: t %.9f (reference %.9f); planets max %.2e (spread %.2e); "
          "test particles median %.2e p99 %.2e (spread %.2e, %.2e)"
          % (mode, t, t_ref, err[massive].max(), spread[massive].max(),
             np.median(err[~massive]), np.percentile(err[~massive], 99),
             np.median(spread[~massive]), np.percentile(spread[~massive], 99)))
    assert err[massive].max() <= 50 * spread[massive].max()
    assert np.median(err[~massive]) <= 50 * np.median(spread[~massive])
    assert np.percentile(err[~massive], 99) <= 50 * np.percentile(spread[~massive], 99)
    e0 = oracle.energy(p, v, m, G)
    assert abs((oracle.energy(P, V, m, G) - e0) / e0) <= 1e-13


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_ensemble_100yr_energy_distribution(clib, oracle, mode):
    gold = _fixture("horizon_ensemble.npz")
    h = list(gold["horizons"]).index(100.0)
    ref_de = gold["de"][:, h]
    ns = ref_de.size
    P, V, M, offs = ics.ensemble(n_systems=ns, seed0=int(gold["seed0"][0]))
    old = clib.set_force_mode(mode)
    try:
        out = clib.gr_ensemble(P, V, M, offs, G, 0.0, 100.0)
    finally:
        clib.set_force_mode(old)
    assert (out["status"] == 0).all() and (out["t"] >= 100.0).all()
    de = np.zeros(ns)
    for s in range(ns):
        a, b = offs[s], offs[s + 1]
        e0 = oracle.energy(P[3 * a:3 * b], V[3 * a:3 * b], M[a:b], G)
        e1 = oracle.energy(out["pos"][3 * a:3 * b], out["vel"][3 * a:3 * b], M[a:b], G)
        de[s] = abs((e1 - e0) / e0)
    qs = (50, 90, 99, 100)
    ours = np.percentile(de, qs)
    theirs = np.percentile(ref_de, qs)
    print("ensemble 100 yr, %s form: |dE/E| p50 p90 p99 max %s (reference %s), %.1f s"
          % (mode, " ".join("%.2e" % x for x in ours), " ".join("%.2e" % x for x in theirs),
             out["seconds"]))
    assert (ours <= 10 * np.maximum(theirs, 1e-15)).all()
