"""Seeded synthetic initial conditions for the benchmark workloads.

Units are MSun, au, yr with G = 4 pi^2.  The star sits at the origin at rest;
bodies are placed from orbital elements around it with mu = G (m_p + M_star).
The elements-to-Cartesian map is the standard one the reference uses in
abie/tools.py:36-111 (periapsis unit vector e_vec and its in-plane normal
q_vec; r = a (1 - e^2) / (1 + e cos f)), written here vectorised in numpy.

Every generator takes a seed and draws from ``numpy.random.default_rng``, so
the same call gives the same bodies on every machine.
"""
import numpy as np

G_SOLAR = 4.0 * np.pi ** 2


def elements_to_cartesian(m_p, m_s, a, e, f, inc, omega, Omega, G=G_SOLAR):
    """Position and velocity (n, 3) of bodies relative to their primary."""
    a, e, f, inc, omega, Omega = (np.asarray(v, dtype=np.float64)
                                  for v in (a, e, f, inc, omega, Omega))
    cO, sO = np.cos(Omega), np.sin(Omega)
    co, so = np.cos(omega), np.sin(omega)
    ci, si = np.cos(inc), np.sin(inc)
    ev = np.stack([cO * co - sO * so * ci, sO * co + cO * so * ci, so * si], axis=-1)
    qv = np.stack([-cO * so - sO * co * ci, -sO * so + cO * co * ci, co * si], axis=-1)
    cf, sf = np.cos(f), np.sin(f)
    p = a * (1.0 - e ** 2)
    sep = p / (1.0 + e * cf)
    pos = (sep * cf)[..., None] * ev + (sep * sf)[..., None] * qv
    vt = np.sqrt(G * (np.asarray(m_p) + np.asarray(m_s)) / p)
    vel = (-vt * sf)[..., None] * ev + (vt * (e + cf))[..., None] * qv
    return pos, vel


def _log_uniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def _angles(rng, n):
    return rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n)


def _assemble(m_star, m, pos, vel):
    n = m.size + 1
    P = np.zeros((n, 3))
    V = np.zeros((n, 3))
    P[1:], V[1:] = pos, vel
    M = np.concatenate([[m_star], m])
    return P.reshape(-1).copy(), V.reshape(-1).copy(), M, np.zeros(n)


def planetary_system(seed=1001, n_planets=8, n_tp=1000, m_star=1.0,
                     m_range=(1e-7, 1e-3), a_range=(0.4, 30.0), e_sigma=0.02, i_sigma=0.01,
                     tp_a=(1.0, 50.0), tp_e=(0.0, 0.3), tp_i=(0.0, 0.1), G=G_SOLAR):
    """Star + planets + massless test particles (the 1,009-body GR workload)."""
    rng = np.random.default_rng(seed)
    mp = _log_uniform(rng, *m_range, n_planets)
    ap = _log_uniform(rng, *a_range, n_planets)
    ep = np.minimum(rng.rayleigh(e_sigma, n_planets), 0.9)
    ip = rng.rayleigh(i_sigma, n_planets)
    O, w, f = _angles(rng, n_planets)
    pp, vp = elements_to_cartesian(mp, m_star, ap, ep, f, ip, w, O, G)
    at = rng.uniform(*tp_a, n_tp)
    et = rng.uniform(*tp_e, n_tp)
    it = rng.uniform(*tp_i, n_tp)
    O, w, f = _angles(rng, n_tp)
    pt, vt = elements_to_cartesian(np.zeros(n_tp), m_star, at, et, f, it, w, O, G)
    return _assemble(m_star, np.concatenate([mp, np.zeros(n_tp)]),
                     np.concatenate([pp, pt]), np.concatenate([vp, vt]))


def planetesimal_disk(seed=1002, n=16384, m_body=1e-9, m_star=1.0, a_range=(5.0, 40.0),
                      e_sigma=0.01, i_sigma=0.005, G=G_SOLAR):
    """Star + n equal-mass planetesimals (the 16,385-body all-pairs workload)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(*a_range, n)
    e = np.minimum(rng.rayleigh(e_sigma, n), 0.9)
    inc = rng.rayleigh(i_sigma, n)
    O, w, f = _angles(rng, n)
    m = np.full(n, m_body)
    p, v = elements_to_cartesian(m, m_star, a, e, f, inc, w, O, G)
    return _assemble(m_star, m, p, v)


def test_particle_swarm(seed=1003, n_tp=1 << 20, n_planets=5, m_star=1.0,
                        m_range=(3e-6, 1e-3), a_range=(1.0, 30.0), e_max=0.1, i_sigma=0.01,
                        tp_a=(2.0, 60.0), tp_e=(0.0, 0.4), tp_i=(0.0, 0.2), G=G_SOLAR):
    """Star + planets + a large swarm of test particles (the WH workload)."""
    rng = np.random.default_rng(seed)
    mp = _log_uniform(rng, *m_range, n_planets)
    ap = np.sort(rng.uniform(*a_range, n_planets))
    ep = rng.uniform(0.0, e_max, n_planets)
    ip = rng.rayleigh(i_sigma, n_planets)
    O, w, f = _angles(rng, n_planets)
    pp, vp = elements_to_cartesian(mp, m_star, ap, ep, f, ip, w, O, G)
    at = rng.uniform(*tp_a, n_tp)
    et = rng.uniform(*tp_e, n_tp)
    it = rng.uniform(*tp_i, n_tp)
    O, w, f = _angles(rng, n_tp)
    pt, vt = elements_to_cartesian(np.zeros(n_tp), m_star, at, et, f, it, w, O, G)
    return _assemble(m_star, np.concatenate([mp, np.zeros(n_tp)]),
                     np.concatenate([pp, pt]), np.concatenate([vp, vt]))


def ensemble(n_systems=4096, seed0=10000, n_planets=(3, 12), m_star=(0.5, 1.5),
             m_range=(1e-7, 1e-3), a_range=(0.3, 50.0), e_sigma=0.05, i_sigma=0.02, G=G_SOLAR):
    """Independent planetary systems of uneven size, packed ragged.

    Returns (pos[3*total], vel[3*total], m[total], offsets[n_systems+1]);
    system s owns bodies offsets[s]:offsets[s+1], star first.  System s is
    drawn from its own generator seeded seed0 + s, so any subset of the
    ensemble can be regenerated alone.
    """
    P, V, M, offs = [], [], [], [0]
    for s in range(n_systems):
        rng = np.random.default_rng(seed0 + s)
        k = int(rng.integers(n_planets[0], n_planets[1] + 1))
        ms = rng.uniform(*m_star)
        mp = _log_uniform(rng, *m_range, k)
        ap = _log_uniform(rng, *a_range, k)
        ep = np.minimum(rng.rayleigh(e_sigma, k), 0.9)
        ip = rng.rayleigh(i_sigma, k)
        O, w, f = _angles(rng, k)
        pp, vp = elements_to_cartesian(mp, ms, ap, ep, f, ip, w, O, G)
        p, v, m, _ = _assemble(ms, mp, pp, vp)
        P.append(p)
        V.append(v)
        M.append(m)
        offs.append(offs[-1] + m.size)
    return (np.concatenate(P), np.concatenate(V), np.concatenate(M),
            np.asarray(offs, dtype=np.int64))


def to_heliocentric(pos, vel):
    """Shift a state so body 0 sits at the origin at rest, like the
    reference's WisdomHolman.move_to_helio (abie/integrator_wisdom_holman.py:579-589)."""
    p = pos.reshape(-1, 3).copy()
    v = vel.reshape(-1, 3).copy()
    p[1:] -= p[0]
    v[1:] -= v[0]
    p[0] = 0.0
    v[0] = 0.0
    return p.reshape(-1), v.reshape(-1)
