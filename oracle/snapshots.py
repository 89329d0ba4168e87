"""CPU checker for the device snapshots -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of what the reference's Python layer computes for each
stored snapshot (abie/integrator.py:158-204 and :233-252):

* the chunk schedule of ``Integrator.integrate``: dt = min(store_dt,
  t_end - t) once, then ``next_t = t + dt - ((t + dt) % dt)`` per chunk with
  Python's float modulo, while t < t_end (integrator.py:176-188);
* the primary body of ``Particles.determine_primary_body`` for the global
  modes "#COM#", "#M_MAX#", "#M_MIN#" and a body index
  (abie/particles.py:378-397; centre of mass: particles.py:301-315);
* semi-major axis, eccentricity and inclination of every body about that
  primary, ``Particles.calculate_aei`` (particles.py:352-376) over
  ``Tools.from_cartesian_to_aei``'s single-body branch (abie/tools.py:236-285).

Pinned against the reference's own Python (``tests/golden/make_golden.py aei``
imports abie/particles.py and abie/tools.py and writes golden_aei.npz).
"""
import math

import numpy as np

PRIMARY_COM, PRIMARY_M_MAX, PRIMARY_M_MIN = -1, -2, -3


def py_mod(x, y):
    """Python's float x % y (the result takes the sign of y)."""
    r = math.fmod(x, y)
    if r:
        if (y < 0) != (r < 0):
            r += y
    else:
        r = math.copysign(0.0, y)
    return r


def chunk_ends(t, t_end, store_dt, advance):
    """The chunk end times the reference's integrate() asks for; advance(t0, t1)
    runs one chunk and returns the model time reached."""
    dt = min(store_dt, t_end - t)
    ends = []
    while t < t_end:
        next_t = t + dt - py_mod(t + dt, dt)
        ends.append(next_t)
        t = advance(t, next_t)
    return ends


def primary_body(pos, vel, m, primary):
    """(mass, position[3], velocity[3]) of the primary."""
    p, v = np.asarray(pos).reshape(-1, 3), np.asarray(vel).reshape(-1, 3)
    if primary == PRIMARY_COM:
        cp, cv = np.zeros(3), np.zeros(3)
        for k in range(m.size):       # particles.py:310-312, one body at a time
            cp += p[k] * m[k]
            cv += v[k] * m[k]
        mt = np.sum(m)
        return mt, cp / mt, cv / mt
    if primary == PRIMARY_M_MAX:
        k = int(np.argmax(m))
    elif primary == PRIMARY_M_MIN:
        k = int(np.argmin(m))
    else:
        k = int(primary)
    return m[k], p[k].copy(), v[k].copy()


def aei_one(mp, ms, position, velocity, G):
    """tools.py:256-285 for one body (a, e, i)."""
    mu = G * (mp + ms)
    v_sq = np.dot(velocity, velocity)
    r_sq = np.dot(position, position)
    r = np.sqrt(r_sq)
    if r == 0:
        return np.nan, np.nan, np.nan
    specific_energy = (1.0 / 2.0) * v_sq - G * (mp + ms) / r
    a = -G * (mp + ms) / (2.0 * specific_energy)
    h = np.cross(position, velocity)
    hn = np.sqrt(np.dot(h, h))
    with np.errstate(divide="ignore", invalid="ignore"):
        hu = h / hn
        ecc = ((v_sq - mu / r) * position - np.dot(position, velocity) * velocity) / mu
        inc = np.arccos(np.dot(np.array([0.0, 0.0, 1.0]), hu))
    return a, np.linalg.norm(ecc), inc


def calculate_aei(pos, vel, m, G, primary=PRIMARY_COM):
    """particles.py:352-376: an (N, 3) array of a, e, i about the primary."""
    p, v = np.asarray(pos).reshape(-1, 3), np.asarray(vel).reshape(-1, 3)
    m = np.asarray(m, dtype=np.float64)
    out = np.zeros((m.size, 3))
    if m.size < 2:
        return np.full((m.size, 3), np.nan)
    ms, pp, pv = primary_body(p, v, m, primary)
    for k in range(m.size):
        out[k] = aei_one(m[k], ms, p[k] - pp, v[k] - pv, G)
    return out
