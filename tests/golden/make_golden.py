"""Generate golden input/output vectors from the unmodified reference library.

Run in a container where the reference sources exist:

    oracle/build_ref.sh && python tests/golden/make_golden.py

Every output array below comes from the reference's own entry points
(ode_n_body_second_order, calculate_accelerations, calculate_energy, integrator_gr,
integrator_wh, integrator_rk,
the event buffers) driven through ctypes by ``oracle.Reference``.  The
inputs are the package's seeded generators.  The resulting ``golden.npz``
is small, committed, and travels with the tests; nothing at test time reads
the reference sources.  ``golden_ext.npz`` (``make_golden.py ext``) holds
the external-acceleration cases.  ``golden_aei.npz`` (``make_golden.py aei``) holds
orbital elements from the reference's own Python (abie/particles.py,
abie/tools.py), imported from its source tree.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from abie_gb300 import ics  # noqa: E402
from oracle import Reference, build_reference  # noqa: E402

G = ics.G_SOLAR


def main(out=os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")):
    build_reference()
    R = Reference()
    gold = {}
    # the Radau15 tables exactly as the reference library was compiled
    import ctypes
    for name, n in (("hs", 8), ("rs", 64), ("cs", 64)):
        gold["radau_" + name] = np.array((ctypes.c_double * n).in_dll(R.lib, name))

    # -- force: planets + test particles, with edge-case masses ---------------
    p, v, m, r = ics.planetary_system(seed=11, n_planets=8, n_tp=100)
    m_edge = m.copy()
    m_edge[5] = -1.0      # deleted particle: not a source, acc untouched
    m_edge[6] = 0.0       # massless planet slot
    for name, mm in (("force_sys", m), ("force_edge", m_edge)):
        gold[name + "_pos"] = p
        gold[name + "_m"] = mm
        gold[name + "_acc"] = R.force(p, mm, G, acc=np.zeros(3 * mm.size))
    # -- force: all-massive planetesimal disk (2,049 bodies) ------------------
    p, v, m, r = ics.planetesimal_disk(seed=12, n=2048)
    gold["force_disk_pos"], gold["force_disk_m"] = p, m
    gold["force_disk_acc"] = R.force(p, m, G)
    gold["energy_disk_vel"] = v
    gold["energy_disk"] = np.array([R.energy(p, v, m, G)])
    # -- tiny N ----------------------------------------------------------------
    for n in (1, 2, 3):
        p, v, m, r = ics.planetary_system(seed=20 + n, n_planets=n - 1, n_tp=0)
        gold["force_n%d_pos" % n], gold["force_n%d_m" % n] = p, m
        gold["force_n%d_acc" % n] = R.force(p, m, G)

    # -- Radau15 trajectories ----------------------------------------------------
    cases = {
        "gr_sys": (ics.planetary_system(seed=31, n_planets=8, n_tp=10), 0.0, 10.0, {}),
        "gr_tp": (ics.planetary_system(seed=32, n_planets=3, n_tp=40), 0.0, 3.0, {}),
    }
    P, V, M, offs = ics.ensemble(n_systems=3, seed0=40)
    for s in range(3):
        sl = slice(offs[s], offs[s + 1])
        cases["gr_ens%d" % s] = ((P[3 * offs[s]:3 * offs[s + 1]], V[3 * offs[s]:3 * offs[s + 1]],
                                  M[sl], np.zeros(offs[s + 1] - offs[s])), 0.0, 20.0, {})
    # close encounters: two planets placed 1e-3 au apart, CE distance 0.05 au
    p, v, m, r = ics.planetary_system(seed=33, n_planets=6, n_tp=4)
    p = p.copy()
    p[15:18] = p[18:21] + 1e-3
    cases["gr_ce"] = ((p, v, m, r), 0.0, 1.0, {"ce_dist": 0.05, "max_ce": 3})
    # collisions: radii large enough that bodies 2 and 3 touch
    p, v, m, r = ics.planetary_system(seed=34, n_planets=5, n_tp=0)
    p = p.copy()
    p[9:12] = p[6:9] + 2e-3
    r = np.full(m.size, 2e-3)
    cases["gr_coll"] = ((p, v, m, r), 0.0, 1.0, {"max_coll": 2})
    for name, ((p, v, m, r), t0, t1, kw) in cases.items():
        out_ = R.radau15(p, v, m, r, G, t0, t1, **kw)
        gold[name + "_in_pos"], gold[name + "_in_vel"] = p, v
        gold[name + "_m"], gold[name + "_r"] = m, r
        gold[name + "_span"] = np.array([t0, t1, kw.get("ce_dist", 0.0),
                                         kw.get("max_ce", 1), kw.get("max_coll", 1)])
        gold[name + "_pos"], gold[name + "_vel"] = out_["pos"], out_["vel"]
        gold[name + "_t"] = np.array([out_["t"]])
        gold[name + "_flag"] = np.array([out_["flag"], out_["n_ce"], out_["n_coll"]])
        gold[name + "_buf_ce"], gold[name + "_buf_coll"] = out_["buf_ce"], out_["buf_coll"]

    # -- Wisdom-Holman ------------------------------------------------------------
    p, v, m, r = ics.test_particle_swarm(seed=51, n_tp=200)
    p, v = ics.to_heliocentric(p, v)
    out_ = R.wh(p, v, m, G, 0.0, 1.0, 0.01)
    gold["wh_in_pos"], gold["wh_in_vel"], gold["wh_m"] = p, v, m
    gold["wh_span"] = np.array([0.0, 1.0, 0.01])
    gold["wh_pos"], gold["wh_vel"], gold["wh_t"] = out_["pos"], out_["vel"], np.array([out_["t"]])
    gold["wh_energy0"] = np.array([R.energy(p, v, m, G)])

    # -- Runge-Kutta 4 (src/integrator_runge_kutta.c) ---------------------------------
    p, v, m, r = ics.planetary_system(seed=71, n_planets=6, n_tp=10)
    out_ = R.rk(p, v, m, G, 0.0, 0.5, 0.005)
    gold["rk_in_pos"], gold["rk_in_vel"], gold["rk_m"] = p, v, m
    gold["rk_span"] = np.array([0.0, 0.5, 0.005])
    gold["rk_pos"], gold["rk_vel"] = out_["pos"], out_["vel"]

    # -- post-Newtonian terms (src/additional_forces.c), C = speed of light in au/yr --
    C = 63239.7263
    p, v, m, r = ics.planetary_system(seed=81, n_planets=5, n_tp=0)
    gold["pn_in_pos"], gold["pn_in_vel"], gold["pn_m"], gold["pn_C"] = p, v, m, np.array([C])
    gold["pn_acc"] = R.accelerations(p, v, m, G, C)
    out_ = R.radau15(p, v, m, r, G, 0.0, 2.0, C=C)
    gold["pn_gr_pos"], gold["pn_gr_vel"], gold["pn_gr_t"] = out_["pos"], out_["vel"], np.array([out_["t"]])

    np.savez_compressed(out, **gold)
    print("wrote", out, os.path.getsize(out), "bytes,", len(gold), "arrays")


def _reference_python(ref_root=None):
    """The reference's abie.particles and abie.tools, imported from its
    source tree (``ref_root`` or the environment variable
    ABIE_REFERENCE_ROOT) without running abie/__init__.py (which needs
    h5py/toml)."""
    import types
    ref_root = ref_root or os.environ.get("ABIE_REFERENCE_ROOT")
    if not ref_root:
        raise SystemExit("set ABIE_REFERENCE_ROOT to the reference project's root")
    if "abie" not in sys.modules:
        pkg = types.ModuleType("abie")
        pkg.__path__ = [os.path.join(ref_root, "abie")]
        sys.modules["abie"] = pkg
    import abie.particles  # noqa: E402
    return abie.particles.Particles


def main_aei(out=os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_aei.npz")):
    """a, e, i of every body about the primary, from the reference's own
    Particles.calculate_aei (abie/particles.py:352-376), for the global
    primary modes the device snapshots support.  The reference's "#M_MAX#"
    and "#M_MIN#" modes fail there (np.argmax's integer is not an ``int`` to
    Particles.__getitem__, which returns None), so the most massive body is
    pinned through its index, the mode's evident meaning."""
    Particles = _reference_python()
    gold = {}
    p, v, m, r = ics.planetary_system(seed=91, n_planets=8, n_tp=40)
    gold["aei_pos"], gold["aei_vel"], gold["aei_m"] = p, v, m
    for key, prim in (("com", "#COM#"), ("mmax", int(np.argmax(m))), ("body3", 3)):
        P = Particles(G)
        for k in range(m.size):
            P.add(pos=p[3 * k:3 * k + 3].copy(), vel=v[3 * k:3 * k + 3].copy(), mass=float(m[k]))
        P.primary = prim
        with np.errstate(divide="ignore", invalid="ignore"):
            gold["aei_" + key] = np.asarray(P.calculate_aei())
    np.savez_compressed(out, **gold)
    print("wrote", out, os.path.getsize(out), "bytes,", len(gold), "arrays")


def main_ext(out=os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_ext.npz")):
    """External accelerations (set_additional_forces, src/common.c:364-380)
    through the reference's calculate_accelerations (:107-112) and its
    Radau15 run, which adds them to every force call."""
    build_reference()
    R = Reference()
    p, v, m, r = ics.planetary_system(seed=91, n_planets=5, n_tp=20)
    ext = np.random.default_rng(92).normal(scale=1e-3, size=p.size)
    gold = {"ext_in_pos": p, "ext_in_vel": v, "ext_m": m, "ext_r": r, "ext_acc_in": ext,
            "ext_span": np.array([0.0, 2.0])}
    gold["ext_accel"] = R.accelerations(p, v, m, G, 0.0, ext=ext)
    out_ = R.radau15(p, v, m, r, G, 0.0, 2.0, ext=ext)
    gold["ext_gr_pos"], gold["ext_gr_vel"] = out_["pos"], out_["vel"]
    gold["ext_gr_t"] = np.array([out_["t"]])
    np.savez_compressed(out, **gold)
    print("wrote", out, os.path.getsize(out), "bytes,", len(gold), "arrays")


if __name__ == "__main__":
    if sys.argv[1:] == ["aei"]:
        main_aei()
    elif sys.argv[1:] == ["ext"]:
        main_ext()
    else:
        main()
        main_aei()
        main_ext()
