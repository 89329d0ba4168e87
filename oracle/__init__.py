"""CPU oracle for ABIE's gravity hot path -- TEST INFRASTRUCTURE ONLY.

Two checkers live here:

* ``Oracle``: ctypes binding of ``oracle/abie_oracle.c``, a plain C99
  restatement of the reference algorithms (src/common.c,
  src/integrator_gauss_radau15.c, src/integrator_wisdom_holman.c), built by
  ``oracle/Makefile`` into ``oracle/_build/``.
* ``Reference``: ctypes binding of the unmodified reference library built
  from its own sources by ``oracle/build_ref.sh`` into ``oracle/_ref/``.  It
  only exists where the reference sources do; tests that need it skip
  otherwise.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only as the checker.  The product library never calls it.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libabie_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libabie_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def build_oracle(quiet=True):
    """Compile the C restatement (make -C oracle)."""
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return ORACLE_SO


def build_reference(ref_root=None):
    """Compile the reference C library from its sources, when they exist.

    ``ref_root`` (or the environment variable ABIE_REFERENCE_ROOT) names the
    reference project's root; without either, oracle/build_ref.sh looks in
    its own default location and skips the build when no sources are there."""
    ref_root = ref_root or os.environ.get("ABIE_REFERENCE_ROOT")
    if ref_root and not os.path.isfile(os.path.join(ref_root, "src", "common.c")):
        return None
    cmd = ["bash", os.path.join(HERE, "build_ref.sh")] + ([ref_root] if ref_root else [])
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return REF_SO if os.path.isfile(REF_SO) else None


class _Events(ctypes.Structure):
    _fields_ = [("ce_dist", ctypes.c_double),
                ("max_ce", ctypes.c_size_t), ("max_coll", ctypes.c_size_t),
                ("n_ce", ctypes.c_size_t), ("n_coll", ctypes.c_size_t),
                ("buf_ce", _dp), ("buf_coll", _dp)]


class RadauStats(ctypes.Structure):
    _fields_ = [("force_calls", ctypes.c_long), ("iterations", ctypes.c_long),
                ("attempts", ctypes.c_long), ("accepts", ctypes.c_long),
                ("rejects", ctypes.c_long), ("iter_hist", ctypes.c_long * 13),
                ("h_last", ctypes.c_double)]

    def as_dict(self):
        return {"force_calls": self.force_calls, "iterations": self.iterations,
                "attempts": self.attempts, "accepts": self.accepts,
                "rejects": self.rejects, "iter_hist": list(self.iter_hist),
                "h_last": self.h_last}


class Oracle:
    """Binding of the C restatement."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.isfile(path):
            build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.orc_energy.restype = ctypes.c_double
        L.orc_radau15.restype = ctypes.c_int
        L.orc_wh.restype = ctypes.c_long
        L.orc_force_threads.restype = ctypes.c_int

    def force(self, pos, m, G, j0=0, j1=None, threads=1, acc=None):
        pos, m = _f64(pos), _f64(m)
        n = m.size
        j1 = n if j1 is None else j1
        if acc is None:
            acc = np.zeros(3 * n)
        if threads > 1:
            self.lib.orc_force_threads(_ptr(pos), ctypes.c_size_t(n), ctypes.c_double(G),
                                       _ptr(m), _ptr(acc), ctypes.c_size_t(j0),
                                       ctypes.c_size_t(j1), ctypes.c_int(threads))
        else:
            self.lib.orc_force(_ptr(pos), ctypes.c_size_t(n), ctypes.c_double(G), _ptr(m),
                               _ptr(acc), ctypes.c_size_t(j0), ctypes.c_size_t(j1))
        return acc

    def energy(self, pos, vel, m, G):
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        return self.lib.orc_energy(_ptr(pos), _ptr(vel), _ptr(m), ctypes.c_size_t(m.size),
                                   ctypes.c_double(G))

    def post_newtonian(self, pos, vel, m, G, C, acc=None):
        """src/additional_forces.c:14-121 added to acc (zeros by default)."""
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        acc = np.zeros(pos.size) if acc is None else _f64(acc).copy()
        self.lib.orc_post_newtonian(_ptr(pos), _ptr(vel), ctypes.c_size_t(m.size),
                                    ctypes.c_double(G), ctypes.c_double(C), _ptr(m), _ptr(acc))
        return acc

    def radau15(self, pos, vel, m, r, G, t, t_end, ce_dist=0.0, max_ce=1, max_coll=1,
                events=True, C=0.0, ext=None, fastform=False):
        """src/integrator_gauss_radau15.c:221-380; ``ext`` (3N) is added to
        every force call, as set_additional_forces does.  ``fastform``: the
        GPU fast form's arithmetic instead of the reference's operations
        (orc_set_fastform; for the long-horizon accuracy study, Newtonian
        forces only)."""
        pos, vel, m, r = (_f64(pos).copy(), _f64(vel).copy(), _f64(m), _f64(r))
        ext = None if ext is None else _f64(ext).copy()
        ev = _Events()
        buf_ce = np.zeros(4 * max(max_ce, 1))
        buf_coll = np.zeros(4 * max(max_coll, 1))
        ev.ce_dist = ce_dist
        ev.max_ce, ev.max_coll = max_ce, max_coll
        ev.buf_ce = _ptr(buf_ce) if max_ce > 0 else None
        ev.buf_coll = _ptr(buf_coll) if max_coll > 0 else None
        st = RadauStats()
        t_out = ctypes.c_double(t)
        self.lib.orc_set_pn(ctypes.c_double(C))
        self.lib.orc_set_ext(_ptr(ext) if ext is not None else None)
        self.lib.orc_set_fastform(ctypes.c_int(1 if fastform else 0))
        try:
            flag = self.lib.orc_radau15(_ptr(pos), _ptr(vel), _ptr(m), _ptr(r),
                                        ctypes.c_size_t(m.size), ctypes.c_double(G),
                                        ctypes.c_double(t), ctypes.c_double(t_end),
                                        ctypes.byref(ev) if events else None,
                                        ctypes.byref(t_out), ctypes.byref(st))
        finally:
            self.lib.orc_set_pn(ctypes.c_double(0.0))
            self.lib.orc_set_ext(None)
            self.lib.orc_set_fastform(ctypes.c_int(0))
        return {"pos": pos, "vel": vel, "t": t_out.value, "flag": flag,
                "stats": st.as_dict(), "n_ce": ev.n_ce, "n_coll": ev.n_coll,
                "buf_ce": buf_ce, "buf_coll": buf_coll}

    def wh(self, pos, vel, m, G, t, t_end, dt, sparse=True):
        pos, vel, m = _f64(pos).copy(), _f64(vel).copy(), _f64(m)
        t_out = ctypes.c_double(t)
        failed = self.lib.orc_wh(_ptr(pos), _ptr(vel), _ptr(m), ctypes.c_size_t(m.size),
                                 ctypes.c_double(G), ctypes.c_double(t), ctypes.c_double(t_end),
                                 ctypes.c_double(dt), ctypes.byref(t_out), ctypes.c_int(int(sparse)))
        return {"pos": pos, "vel": vel, "t": t_out.value, "kepler_failures": failed}

    def rk(self, pos, vel, m, G, t, t_end, dt):
        """src/integrator_runge_kutta.c:6-50 (orc_rk)."""
        pos, vel, m = _f64(pos).copy(), _f64(vel).copy(), _f64(m)
        t_out = ctypes.c_double(t)
        self.lib.orc_rk(_ptr(pos), _ptr(vel), _ptr(m), ctypes.c_size_t(m.size), ctypes.c_double(G),
                        ctypes.c_double(t), ctypes.c_double(t_end), ctypes.c_double(dt),
                        ctypes.byref(t_out))
        return {"pos": pos, "vel": vel, "t": t_out.value}

    def wh_accel(self, pos, jpos, m, G, sparse=True):
        pos, jpos, m = _f64(pos), _f64(jpos), _f64(m)
        acc = np.zeros(3 * m.size)
        self.lib.orc_wh_accel(_ptr(pos), _ptr(jpos), _ptr(m), ctypes.c_size_t(m.size),
                              ctypes.c_double(G), _ptr(acc), ctypes.c_int(int(sparse)))
        return acc

    def helio2jacobi(self, pos, vel, m):
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        jp, jv = np.zeros_like(pos), np.zeros_like(vel)
        self.lib.orc_helio2jacobi(_ptr(pos), _ptr(vel), _ptr(m), ctypes.c_size_t(m.size),
                                  _ptr(jp), _ptr(jv))
        return jp, jv


class _Simulation(ctypes.Structure):
    """Layout of the reference's global ``struct Simulation`` (src/common.h:26-65)."""
    _fields_ = [("pos", _dp), ("vel", _dp), ("m", _dp), ("r", _dp), ("ext_acc", _dp),
                ("N", ctypes.c_size_t), ("G", ctypes.c_double), ("C", ctypes.c_double),
                ("t", ctypes.c_double), ("dt", ctypes.c_double), ("ce_dist", ctypes.c_double),
                ("n_ce", ctypes.c_size_t), ("n_coll", ctypes.c_size_t),
                ("max_ce", ctypes.c_size_t), ("max_coll", ctypes.c_size_t),
                ("enable_ext", ctypes.c_size_t), ("devID", ctypes.c_int),
                ("buf_ce", _dp), ("buf_coll", _dp)]


def _run_big_stack(fn, stack_bytes=1 << 30):
    """Run fn in a thread with a large stack (the reference keeps 29*3N
    doubles of VLAs on the stack in integrator_gauss_radau15)."""
    box = {}

    def body():
        try:
            box["v"] = fn()
        except BaseException as exc:  # re-raised in the caller
            box["e"] = exc

    old = threading.stack_size()
    threading.stack_size(stack_bytes)
    try:
        th = threading.Thread(target=body)
        th.start()
        th.join()
    finally:
        threading.stack_size(old)
    if "e" in box:
        raise box["e"]
    return box["v"]


class Reference:
    """Binding of the unmodified reference library (oracle/_ref).

    The reference keeps one global simulation and refuses a second
    initialize_code; between runs this binding calls finalize_code and then
    clears the global struct and the once-only flag so the next run starts
    from a clean slate.
    """

    def __init__(self, path=REF_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.get_model_time.restype = ctypes.c_double
        L.calculate_energy.restype = ctypes.c_double
        L.integrator_gr.restype = ctypes.c_int
        self.sim = _Simulation.in_dll(L, "sim")
        self.code_inited = ctypes.c_int.in_dll(L, "code_inited")
        self._live = False

    def _reset(self):
        if self._live:
            self.lib.finalize_code()
        ctypes.memset(ctypes.addressof(self.sim), 0, ctypes.sizeof(self.sim))
        self.code_inited.value = 0
        self._live = False

    def _load(self, pos, vel, m, r, G, C=0.0, max_ce=1, max_coll=1, ce_dist=0.0):
        self._reset()
        n = m.size
        self.lib.initialize_code(ctypes.c_double(G), ctypes.c_double(C), ctypes.c_size_t(n),
                                 ctypes.c_size_t(max_ce), ctypes.c_size_t(max_coll),
                                 ctypes.c_int(-1))
        self._live = True
        self.lib.set_close_encounter_distance(ctypes.c_double(ce_dist))
        self.lib.set_state(_ptr(pos), _ptr(vel), _ptr(m), _ptr(r), ctypes.c_size_t(n),
                           ctypes.c_double(G), ctypes.c_double(C))

    def _state(self, n):
        pos, vel = np.zeros(3 * n), np.zeros(3 * n)
        m, r = np.zeros(n), np.zeros(n)
        self.lib.get_state(_ptr(pos), _ptr(vel), _ptr(m), _ptr(r))
        return pos, vel

    def force(self, pos, m, G, acc=None):
        pos, m = _f64(pos), _f64(m)
        n = m.size
        if acc is None:
            acc = np.zeros(3 * n)
        r = np.zeros(n)
        self.lib.ode_n_body_second_order(_ptr(pos), ctypes.c_size_t(n), ctypes.c_double(G),
                                         _ptr(m), _ptr(r), _ptr(acc))
        return acc

    def energy(self, pos, vel, m, G):
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        self._load(pos, vel, m, np.zeros(m.size), G)
        return self.lib.calculate_energy()

    def accelerations(self, pos, vel, m, G, C, ext=None):
        """calculate_accelerations (Newton, then post-Newtonian terms for C > 0,
        then the external accelerations ``ext`` when given)."""
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        self._load(pos, vel, m, np.zeros(m.size), G, C=C)
        if ext is not None:
            ext = _f64(ext)
            self.lib.set_additional_forces(ctypes.c_size_t(m.size), _ptr(ext))
        acc = np.zeros(pos.size)
        self.lib.calculate_accelerations(_ptr(pos), _ptr(vel), ctypes.c_size_t(m.size),
                                         ctypes.c_double(G), _ptr(m), _ptr(np.zeros(m.size)),
                                         _ptr(acc))
        return acc

    def radau15(self, pos, vel, m, r, G, t, t_end, ce_dist=0.0, max_ce=1, max_coll=1, C=0.0,
                ext=None):
        pos, vel, m, r = _f64(pos), _f64(vel), _f64(m), _f64(r)
        self._load(pos, vel, m, r, G, C=C, max_ce=max_ce, max_coll=max_coll, ce_dist=ce_dist)
        if ext is not None:
            ext = _f64(ext)
            self.lib.set_additional_forces(ctypes.c_size_t(m.size), _ptr(ext))
        flag = _run_big_stack(lambda: self.lib.integrator_gr(
            ctypes.c_double(t), ctypes.c_double(t_end), ctypes.c_double(1.0)))
        p, v = self._state(m.size)
        buf_ce = np.zeros(4 * max(max_ce, 1))
        buf_coll = np.zeros(4 * max(max_coll, 1))
        if max_ce > 0:
            self.lib.get_close_encounter_buffer(_ptr(buf_ce))
        if max_coll > 0:
            self.lib.get_collision_buffer(_ptr(buf_coll))
        return {"pos": p, "vel": v, "t": self.lib.get_model_time(), "flag": flag,
                "n_ce": self.sim.n_ce, "n_coll": self.sim.n_coll,
                "buf_ce": buf_ce, "buf_coll": buf_coll}

    def wh(self, pos, vel, m, G, t, t_end, dt):
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        self._load(pos, vel, m, np.zeros(m.size), G)
        _run_big_stack(lambda: self.lib.integrator_wh(
            ctypes.c_double(t), ctypes.c_double(t_end), ctypes.c_double(dt)))
        p, v = self._state(m.size)
        return {"pos": p, "vel": v, "t": self.lib.get_model_time()}


    def rk(self, pos, vel, m, G, t, t_end, dt):
        """integrator_rk on the stored state (it leaves the model time alone)."""
        pos, vel, m = _f64(pos), _f64(vel), _f64(m)
        self._load(pos, vel, m, np.zeros(m.size), G)
        _run_big_stack(lambda: self.lib.integrator_rk(
            ctypes.c_double(t), ctypes.c_double(t_end), ctypes.c_double(dt)))
        p, v = self._state(m.size)
        return {"pos": p, "vel": v}


def reference_available():
    return os.path.isfile(REF_SO)
