"""Long-horizon reference runs, committed as small fixtures.

Run in a container where the reference sources exist:

    oracle/build_ref.sh && python tests/golden/make_horizons.py \
        [cfg1|ensemble|ensemble_spread|ensemble_fastform|cfg3|all]

* ``horizon_cfg1.npz``: the 1,009-body planetary system (1 MSun star, 8
  planets, 1,000 test particles; ``ics.planetary_system(seed=1001)``)
  integrated by the unmodified reference library's ``integrator_gr`` from
  0 to 100 yr in one call, with its final state, model time and the energy
  of ``calculate_energy`` before and after.  A second run from the same
  state with body 1's x coordinate moved by one unit in the last place
  gives the spread that rounding alone produces over the same span; the
  GPU tests compare against the first run with tolerances scaled by it.
* ``horizon_ensemble.npz``: the first 64 systems of the batched-ensemble
  workload (``ics.ensemble(seed0=10000)``: 0.5..1.5 MSun stars with 3..12
  planets) integrated by the reference library from 0 to 1, 100 and 10,000
  yr (three runs from t = 0 each), one process per host core.  Per system:
  |dE/E| at each horizon, the model time, and the final state of the
  10,000-yr run.  This is the distribution the reference method itself
  reaches on these systems, which the GPU forms' distributions are
  compared with.

* ``horizon_ensemble_spread.npz``: the same 64 systems over 10,000 yr,
  rerun four times by the reference library with one coordinate moved by
  one unit in the last place (coordinate 5k mod 3n, up for odd k, down for
  even k, k = 1 .. 4).  Over 10^4 yr several of these systems are chaotic, so |dE/E|
  of one system depends on the path: the perturbed runs show how far the
  reference method's own result moves (system 10 of the set: 1.4e-11 to
  1.1e-9 over such runs), and together with the unperturbed run they give
  a 320-sample distribution of the reference method's |dE/E| at 10^4 yr.

* ``horizon_ensemble_fastform.npz``: the same 64 systems over 10,000 yr
  by the oracle with the GPU fast form's arithmetic (``Oracle.radau15(...,
  fastform=True)``: FMA pair sums, the expanded g recurrence, positions
  predicted from g with one rounding at the position's scale, the
  single-precision step-size root, g consistent with each step's guess),
  so that the fast form's energy error over 10^4 yr can be set beside the
  reference method's on the host; with four more runs each moved by one
  unit in the last place, as the reference method's spread runs are.

* ``horizon_cfg3.npz``: the Wisdom-Holman workload (``ics.test_particle_swarm
  (seed=1003)``, heliocentric: 1 MSun star, 5 planets, 1,048,576 test
  particles) at dt = 0.01 yr over 10^4 yr (10^6 steps), for the star, the
  planets and 1,024 test particles drawn with ``default_rng(5)``.  Test
  particles never act on other bodies, so the run of this subset gives
  those particles exactly the trajectories they have in the full run.  The
  reference's O(N^2) loop would take hours here, so the oracle's O(N N_m)
  restatement runs it (pinned to the reference bit for bit at a few hundred
  test particles by tests/test_oracle.py); a second run with planet 1's x
  moved by one unit in the last place gives the rounding spread.

Without the reference library the C restatement in ``oracle/`` (bit for
bit the same doubles, pinned by tests/test_oracle.py) stands in, and the
file records which one ran.
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from abie_gb300 import ics  # noqa: E402

G = ics.G_SOLAR
HERE = os.path.dirname(os.path.abspath(__file__))
ENS_SYSTEMS = 64
ENS_HORIZONS = (1.0, 100.0, 10000.0)


def _build_checkers():
    """Build the reference library (where its sources are) and the oracle,
    once, in the parent process: the workers only load them."""
    import oracle
    try:
        oracle.build_reference()
    except RuntimeError:
        pass
    oracle.build_oracle()


def _checker():
    """(name, object with radau15 and energy) -- the reference when built."""
    import oracle
    if oracle.reference_available():
        return "reference", oracle.Reference()
    return "oracle", oracle.Oracle()


def cfg1_run(perturb):
    kind, R = _checker()
    p, v, m, r = ics.planetary_system(seed=1001)
    if perturb:
        p = p.copy()
        p[3] = np.nextafter(p[3], np.inf)
    e0 = R.energy(p, v, m, G)
    t0 = time.time()
    out = R.radau15(p, v, m, r, G, 0.0, 100.0)
    wall = time.time() - t0
    e1 = R.energy(out["pos"], out["vel"], m, G)
    return {"kind": kind, "pos": out["pos"], "vel": out["vel"], "t": out["t"], "e0": e0,
            "e1": e1, "wall": wall}


def main_cfg1(out=os.path.join(HERE, "horizon_cfg1.npz")):
    _build_checkers()
    with mp.get_context("spawn").Pool(2) as pool:
        base, pert = pool.map(cfg1_run, [False, True])
    np.savez_compressed(
        out, kind=np.array(base["kind"]), seed=np.array([1001]), span=np.array([0.0, 100.0]),
        pos=base["pos"], vel=base["vel"], t=np.array([base["t"]]),
        energy=np.array([base["e0"], base["e1"]]),
        pert_pos=pert["pos"], pert_vel=pert["vel"], pert_t=np.array([pert["t"]]),
        pert_energy=np.array([pert["e0"], pert["e1"]]), wall=np.array([base["wall"]]))
    de = abs((base["e1"] - base["e0"]) / base["e0"])
    print("cfg1: %s, t=%.6f, |dE/E|=%.3g, %.0f s; wrote %s" % (base["kind"], base["t"], de,
                                                              base["wall"], out))


def ens_run(job):
    s, t_end = job[0], job[1]
    k = job[2] if len(job) > 2 else 0
    kind, R = _checker()
    P, V, M, offs = ics.ensemble(n_systems=1, seed0=10000 + s)
    if k:
        P = P.copy()
        i = (5 * k) % P.size
        P[i] = np.nextafter(P[i], np.inf if k % 2 else -np.inf)
    r = np.zeros(M.size)
    e0 = R.energy(P, V, M, G)
    t0 = time.time()
    out = R.radau15(P, V, M, r, G, 0.0, t_end)
    wall = time.time() - t0
    e1 = R.energy(out["pos"], out["vel"], M, G)
    return {"s": s, "t_end": t_end, "k": k, "kind": kind, "t": out["t"],
            "de": abs((e1 - e0) / e0), "pos": out["pos"], "vel": out["vel"], "wall": wall}


def main_ensemble(out=os.path.join(HERE, "horizon_ensemble.npz"), cores=None):
    _build_checkers()
    cores = cores or max(1, (os.cpu_count() or 2) - 1)
    # longest runs first so the pool's tail is short
    jobs = [(s, T) for T in sorted(ENS_HORIZONS, reverse=True) for s in range(ENS_SYSTEMS)]
    t0 = time.time()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(ens_run, jobs, chunksize=1)
    H = len(ENS_HORIZONS)
    de = np.zeros((ENS_SYSTEMS, H))
    tt = np.zeros((ENS_SYSTEMS, H))
    wall = np.zeros((ENS_SYSTEMS, H))
    P, V, M, offs = ics.ensemble(n_systems=ENS_SYSTEMS)
    fpos, fvel = np.zeros_like(P), np.zeros_like(V)
    for r in res:
        h = ENS_HORIZONS.index(r["t_end"])
        de[r["s"], h], tt[r["s"], h], wall[r["s"], h] = r["de"], r["t"], r["wall"]
        if r["t_end"] == ENS_HORIZONS[-1]:
            a, b = offs[r["s"]], offs[r["s"] + 1]
            fpos[3 * a:3 * b], fvel[3 * a:3 * b] = r["pos"], r["vel"]
    np.savez_compressed(out, kind=np.array(res[0]["kind"]), seed0=np.array([10000]),
                        horizons=np.array(ENS_HORIZONS), de=de, t=tt, wall=wall,
                        offsets=offs, pos=fpos, vel=fvel)
    for h, T in enumerate(ENS_HORIZONS):
        q = np.percentile(de[:, h], [50, 90, 99, 100])
        print("ensemble %g yr: |dE/E| median %.2g p90 %.2g p99 %.2g max %.2g; <=1e-12: %d/%d"
              % (T, q[0], q[1], q[2], q[3], int((de[:, h] <= 1e-12).sum()), ENS_SYSTEMS))
    print("%s, %.0f s on %d cores; wrote %s" % (res[0]["kind"], time.time() - t0, cores, out))


def main_ensemble_spread(out=os.path.join(HERE, "horizon_ensemble_spread.npz"), cores=None,
                         perturbations=(1, 2, 3, 4)):
    _build_checkers()
    cores = cores or max(1, (os.cpu_count() or 2) - 1)
    T = ENS_HORIZONS[-1]
    jobs = [(s, T, k) for k in perturbations for s in range(ENS_SYSTEMS)]
    t0 = time.time()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(ens_run, jobs, chunksize=1)
    de = np.zeros((ENS_SYSTEMS, len(perturbations)))
    wall = np.zeros_like(de)
    for r in res:
        j = perturbations.index(r["k"])
        de[r["s"], j], wall[r["s"], j] = r["de"], r["wall"]
    np.savez_compressed(out, kind=np.array(res[0]["kind"]), seed0=np.array([10000]),
                        horizon=np.array([T]), perturbations=np.array(perturbations), de=de,
                        wall=wall)
    q = np.percentile(de, [50, 90, 99, 100])
    print("ensemble %g yr, one-ulp perturbed runs: |dE/E| median %.2g p90 %.2g p99 %.2g max %.2g"
          "; %s, %.0f s on %d cores; wrote %s"
          % (T, q[0], q[1], q[2], q[3], res[0]["kind"], time.time() - t0, cores, out))


def ens_fastform_run(job):
    s, k = job if isinstance(job, tuple) else (job, 0)
    import oracle
    O = oracle.Oracle()
    P, V, M, offs = ics.ensemble(n_systems=1, seed0=10000 + s)
    if k:  # the same one-ulp moves as the reference method's perturbed runs
        P = P.copy()
        i = (5 * k) % P.size
        P[i] = np.nextafter(P[i], np.inf if k % 2 else -np.inf)
    T = ENS_HORIZONS[-1]
    e0 = O.energy(P, V, M, G)
    t0 = time.time()
    out = O.radau15(P, V, M, np.zeros(M.size), G, 0.0, T, fastform=True)
    wall = time.time() - t0
    e1 = O.energy(out["pos"], out["vel"], M, G)
    return {"s": s, "k": k, "de": abs((e1 - e0) / e0), "wall": wall, "t": out["t"]}


def main_ensemble_fastform(out=os.path.join(HERE, "horizon_ensemble_fastform.npz"), cores=None,
                           perturbations=(0, 1, 2, 3, 4)):
    """Run k = 0 is the unperturbed one (``de``); k = 1 .. 4 move one
    coordinate by one unit in the last place as in
    horizon_ensemble_spread.npz (``de_pert``)."""
    _build_checkers()
    cores = cores or max(1, (os.cpu_count() or 2) - 1)
    t0 = time.time()
    jobs = [(s, k) for k in perturbations for s in range(ENS_SYSTEMS)]
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(ens_fastform_run, jobs, chunksize=1)
    all_de = np.zeros((ENS_SYSTEMS, len(perturbations)))
    wall = np.zeros_like(all_de)
    tt = np.zeros_like(all_de)
    for r in res:
        j = perturbations.index(r["k"])
        all_de[r["s"], j], wall[r["s"], j], tt[r["s"], j] = r["de"], r["wall"], r["t"]
    de = all_de[:, 0]
    np.savez_compressed(out, kind=np.array("oracle-fastform"), seed0=np.array([10000]),
                        horizon=np.array([ENS_HORIZONS[-1]]), de=de, de_pert=all_de[:, 1:],
                        perturbations=np.array(perturbations), t=tt, wall=wall)
    q = np.percentile(all_de, [50, 90, 99, 100])
    print("ensemble %g yr, fast-form arithmetic, %d runs: |dE/E| median %.2g p90 %.2g p99 %.2g "
          "max %.2g; <=1e-12: %.0f %%; %.0f s on %d cores; wrote %s"
          % (ENS_HORIZONS[-1], all_de.size, q[0], q[1], q[2], q[3],
             100.0 * (all_de <= 1e-12).mean(), time.time() - t0, cores, out))


CFG3_SAMPLE = 1024
CFG3_SEED = 5


def cfg3_sample_indices(n_bodies, n_massive=6):
    """The bodies of the cfg3 fixture: the massive ones and CFG3_SAMPLE test
    particles, in body order."""
    rng = np.random.default_rng(CFG3_SEED)
    tp = n_massive + rng.choice(n_bodies - n_massive, CFG3_SAMPLE, replace=False)
    return np.concatenate([np.arange(n_massive), np.sort(tp)])


def cfg3_run(perturb):
    import oracle
    O = oracle.Oracle()
    p, v, m, r = ics.test_particle_swarm(seed=1003)
    p, v = ics.to_heliocentric(p, v)
    idx = cfg3_sample_indices(m.size)
    P = p.reshape(-1, 3)[idx].ravel().copy()
    V = v.reshape(-1, 3)[idx].ravel().copy()
    M = m[idx]
    if perturb:
        P[3] = np.nextafter(P[3], np.inf)
    e0 = O.energy(P, V, M, G)
    t0 = time.time()
    out = O.wh(P, V, M, G, 0.0, 10000.0, 0.01)
    wall = time.time() - t0
    return {"pos": out["pos"], "vel": out["vel"], "t": out["t"], "e0": e0,
            "e1": O.energy(out["pos"], out["vel"], M, G), "fails": out["kepler_failures"],
            "wall": wall, "idx": idx}


def main_cfg3(out=os.path.join(HERE, "horizon_cfg3.npz")):
    _build_checkers()
    with mp.get_context("spawn").Pool(2) as pool:
        base, pert = pool.map(cfg3_run, [False, True])
    np.savez_compressed(out, kind=np.array("oracle"), seed=np.array([1003]),
                        span=np.array([0.0, 10000.0, 0.01]), idx=base["idx"],
                        pos=base["pos"], vel=base["vel"], t=np.array([base["t"]]),
                        energy=np.array([base["e0"], base["e1"]]),
                        kepler_failures=np.array([base["fails"]]),
                        pert_pos=pert["pos"], pert_vel=pert["vel"], wall=np.array([base["wall"]]))
    print("cfg3: t=%.6f, |dE/E| (massive bodies) %.3g, %.0f s; wrote %s"
          % (base["t"], abs((base["e1"] - base["e0"]) / base["e0"]), base["wall"], out))


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("cfg1", "all"):
        main_cfg1()
    if what in ("ensemble", "all"):
        main_ensemble()
    if what in ("ensemble_spread", "all"):
        main_ensemble_spread()
    if what in ("ensemble_fastform", "all"):
        main_ensemble_fastform()
    if what in ("cfg3", "all"):
        main_cfg3()
