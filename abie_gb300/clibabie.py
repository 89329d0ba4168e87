"""ctypes binding of libabie_gb300 with the reference binding's interface.

``CLibABIE`` has the methods, argument meanings and error behaviour of the
reference's abie/clibabie.py:8-194 (initialize_code, set_state, get_state,
integrator_gr raising CloseEncounterException / CollisionException on
return codes 1 / 2, integrator_wh, get_total_energy, ...).  It differs only
where the reference binding is broken: the wrappers of the direct
integrator entry points pass the full argument list (the reference omits
r_vec), and set_additional_forces passes an integer count.  Negative return
codes of this library raise ``AbieError``.

Extra methods expose the additive entry points: explicit force forms,
counters and the batched ensemble.
"""
import ctypes

import numpy as np

from . import FORCE_MODES, last_error, load
from .events import AbieError, CloseEncounterException, CollisionException

_c = ctypes


def _vp(a):
    return _c.c_void_p(a.ctypes.data)


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


class Counters(_c.Structure):
    _fields_ = [("force_calls", _c.c_longlong), ("iterations", _c.c_longlong),
                ("attempts", _c.c_longlong), ("accepts", _c.c_longlong),
                ("rejects", _c.c_longlong), ("kepler_failures", _c.c_longlong),
                ("wh_steps", _c.c_longlong), ("last_h", _c.c_double),
                ("learned_fallbacks", _c.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CLibABIE(object):
    def __init__(self, path=None):
        self.lib = load(path)
        self.max_close_encounter_events = 1
        self.max_collision_events = 1
        self.N = 0  # bodies of the last set_state

    # -- helpers ------------------------------------------------------------
    def _check(self, rc, what):
        if isinstance(rc, int) and rc < 0:
            raise AbieError(rc, "%s: %s" % (what, last_error()))
        return rc

    # -- reference interface (abie/clibabie.py) -----------------------------
    def initialize_code(self, G, C, N_MAX, MAX_CE_EVENTS=1, MAX_COLLISION_EVENTS=1,
                        close_encounter_distance=0, deviceID=-1):
        rc = self.lib.initialize_code(_c.c_double(G), _c.c_double(C), _c.c_int(N_MAX),
                                      _c.c_int(MAX_CE_EVENTS), _c.c_int(MAX_COLLISION_EVENTS),
                                      _c.c_int(deviceID))
        self._check(rc, "initialize_code")
        self.lib.set_close_encounter_distance(_c.c_double(close_encounter_distance))
        self.max_close_encounter_events = MAX_CE_EVENTS
        self.max_collision_events = MAX_COLLISION_EVENTS

    def finalize_code(self):
        self.lib.finalize_code()

    def set_state(self, pos, vel, masses, radii, N, G, C):
        pos, vel, masses, radii = _f64(pos), _f64(vel), _f64(masses), _f64(radii)
        self.N = int(N)
        self.lib.set_state(_vp(pos), _vp(vel), _vp(masses), _vp(radii), _c.c_int(N),
                           _c.c_double(G), _c.c_double(C))

    def get_state(self, pos, vel, masses, radii):
        rc = self.lib.get_state(_vp(pos), _vp(vel), _vp(masses), _vp(radii))
        return self._check(rc, "get_state")

    def get_model_time(self):
        return self.lib.get_model_time()

    def get_close_encounter_data(self):
        buf = np.zeros(4 * self.max_close_encounter_events)
        self.lib.get_close_encounter_buffer(_vp(buf))
        return buf.reshape(self.max_close_encounter_events, 4)

    def get_collision_data(self):
        buf = np.zeros(4 * self.max_collision_events)
        self.lib.get_collision_buffer(_vp(buf))
        return buf.reshape(self.max_collision_events, 4)

    def reset_close_encounter_buffer(self):
        self.lib.reset_close_encounter_buffer()

    def reset_collision_buffer(self):
        self.lib.reset_collision_buffer()

    def set_close_encounter_distance(self, value):
        self.lib.set_close_encounter_distance(_c.c_double(value))

    def get_total_energy(self):
        return self.lib.calculate_energy()

    def set_additional_forces(self, ext_acc):
        """A constant 3N acceleration added to every force call; None
        switches it off (an addition of this library)."""
        if ext_acc is None:
            self.lib.set_additional_forces(_c.c_int(0), None)
            return
        ext_acc = _f64(ext_acc)
        self._ext = ext_acc  # the library copies it; kept only for inspection
        self.lib.set_additional_forces(_c.c_int(len(ext_acc) // 3), _vp(ext_acc))

    # The reference's wrappers of the direct entry points (abie/clibabie.py:112-146)
    # omit r_vec; these pass the full argument list (radii are unused by all
    # three) and update pos / vel in place.
    def _direct(self, fn, pos, vel, masses, N, G, t, t_end, dt):
        radii = np.zeros(N)
        fn(_vp(pos), _vp(vel), _vp(masses), _vp(radii), _c.c_size_t(N), _c.c_double(G),
           _c.c_double(t), _c.c_double(t_end), _c.c_double(dt))

    def integrator_runge_kutta(self, pos, vel, masses, N, G, t, t_end, dt):
        self._direct(self.lib.integrator_runge_kutta, pos, vel, masses, N, G, t, t_end, dt)

    def integrator_gauss_radau15(self, pos, vel, masses, N, G, t, t_end, dt):
        self._direct(self.lib.integrator_gauss_radau15, pos, vel, masses, N, G, t, t_end, dt)

    def integrator_wisdom_holman(self, pos, vel, masses, N, G, t, t_end, dt):
        self._direct(self.lib.integrator_wisdom_holman, pos, vel, masses, N, G, t, t_end, dt)

    def integrator_gr(self, t, t_end, dt):
        ret = self.lib.integrator_gr(_c.c_double(t), _c.c_double(t_end), _c.c_double(dt))
        if ret == 1:
            buf = self.get_close_encounter_data()
            raise CloseEncounterException(buf[-1, 0], int(buf[-1, 1]), int(buf[-1, 2]), buf[-1, 3])
        elif ret == 2:
            buf = self.get_collision_data()
            raise CollisionException(buf[-1, 0], int(buf[-1, 1]), int(buf[-1, 2]), buf[-1, 3])
        return self._check(ret, "integrator_gr")

    def integrator_rk(self, t, t_end, dt):
        return self._check(self.lib.integrator_rk(_c.c_double(t), _c.c_double(t_end),
                                                  _c.c_double(dt)), "integrator_rk")

    def integrator_wh(self, t, t_end, dt):
        return self._check(self.lib.integrator_wh(_c.c_double(t), _c.c_double(t_end),
                                                  _c.c_double(dt)), "integrator_wh")

    def ode_n_body_second_order(self, x, N, G, masses):
        x, masses = _f64(x), _f64(masses)
        acc = np.zeros(x.size, dtype=np.double)
        radii = np.zeros(N)
        rc = self.lib.ode_n_body_second_order(_vp(x), _c.c_size_t(N), _c.c_double(G), _vp(masses),
                                              _vp(radii), _vp(acc))
        if rc:
            raise AbieError(-1, "ode_n_body_second_order: " + last_error())
        return acc

    # -- additions -----------------------------------------------------------
    def set_force_mode(self, mode):
        mode = FORCE_MODES.get(mode, mode)
        return self._check(self.lib.abie_set_force_mode(_c.c_int(mode)), "set_force_mode")

    def get_force_mode(self):
        return self.lib.abie_get_force_mode()

    def force(self, pos, masses, G, mode="fp64"):
        """All-pairs accelerations of host arrays in an explicit force form."""
        pos, masses = _f64(pos), _f64(masses)
        acc = np.zeros(pos.size)
        rc = self.lib.abie_force_host(_vp(pos), _vp(masses), _c.c_size_t(masses.size),
                                      _c.c_double(G), _vp(acc), _c.c_int(FORCE_MODES.get(mode, mode)))
        self._check(rc, "abie_force_host")
        return acc

    def energy(self, pos, vel, masses, G):
        pos, vel, masses = _f64(pos), _f64(vel), _f64(masses)
        return self.lib.abie_energy_host(_vp(pos), _vp(vel), _vp(masses),
                                         _c.c_size_t(masses.size), _c.c_double(G))

    def counters(self):
        c = Counters()
        self.lib.abie_get_counters(_c.byref(c))
        return c.as_dict()

    def reset_counters(self):
        self.lib.abie_reset_counters()

    def gr_ensemble(self, pos, vel, masses, offsets, G, t0, t_end, learned=False, collect=False,
                    consistent=False):
        """Radau15 over a ragged batch of independent systems.  learned: start
        each step from the learned predictor's guess (with consistent g);
        consistent: the plain guess with g made consistent with it; collect:
        append training samples to the predictor's store."""
        pos, vel, masses = _f64(pos).copy(), _f64(vel).copy(), _f64(masses)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        ns = offsets.size - 1
        t_out = np.zeros(ns)
        status = np.zeros(ns, dtype=np.int32)
        steps = np.zeros(ns, dtype=np.int64)
        rc = self.lib.abie_gr_ensemble(_vp(pos), _vp(vel), _vp(masses), _vp(offsets), _c.c_int(ns),
                                       _c.c_double(G), _c.c_double(t0), _c.c_double(t_end),
                                       _vp(t_out), _vp(status), _vp(steps),
                                       _c.c_int(int(bool(learned)) | (2 if collect else 0) |
                                                (4 if consistent else 0)))
        self._check(rc, "abie_gr_ensemble")
        return {"pos": pos, "vel": vel, "t": t_out, "status": status, "steps": steps,
                "seconds": self.lib.abie_last_ensemble_seconds()}

    def ensemble_tuning(self):
        """Launch shape of the last gr_ensemble call: the share of systems on
        four-warp groups (1 in heavy_div), where it came from ("tuned" in that
        call, "cache", "override", or "default") and the tuner's GPU
        seconds and number of candidates."""
        h, src, secs = _c.c_int(0), _c.c_int(0), _c.c_double(0)
        n = self.lib.abie_ensemble_last_tuning(_c.byref(h), _c.byref(src), _c.byref(secs))
        source = {0: "tuned" if n > 0 else "default", 1: "cache", 2: "override"}[src.value]
        return {"heavy_div": h.value, "source": source, "tune_seconds": secs.value,
                "candidates": int(n)}

    def integrate_snapshots(self, t, t_end, store_dt, integrator="gr", h=0.0, primary="#COM#",
                            max_snaps=None):
        """Integrate the stored state from t to t_end, keeping a snapshot after
        every chunk of store_dt on the GPU (abie/integrator.py:158-204 with
        store_state): times, positions, velocities, a/e/i about the primary
        ("#COM#", "#M_MAX#", "#M_MIN#" or a body index) and energies.
        Returns a dict of arrays and the return code ("flag": 0, or the event
        flag 1 / 2 at which the run stopped)."""
        modes = {"#COM#": -1, "#M_MAX#": -2, "#M_MIN#": -3}
        prim = modes[primary] if isinstance(primary, str) else int(primary)
        n = self.N
        if max_snaps is None:
            max_snaps = int(np.ceil((t_end - t) / min(store_dt, max(t_end - t, 1e-300)))) + 2
        max_snaps = max(int(max_snaps), 0)
        st = np.zeros(max_snaps)
        sp, sv, sa = (np.zeros((max_snaps, 3 * n)) for _ in range(3))
        se = np.zeros(max_snaps)
        k = _c.c_int(0)
        rc = self.lib.abie_integrate_snapshots(
            _c.c_int({"gr": 0, "wh": 1}[integrator]), _c.c_double(t), _c.c_double(t_end),
            _c.c_double(store_dt), _c.c_double(h), _c.c_int(prim), _c.c_int(max_snaps),
            _vp(st), _vp(sp), _vp(sv), _vp(sa), _vp(se), _c.byref(k))
        if rc < 0:
            self._check(rc, "abie_integrate_snapshots")
        k = k.value
        return {"t": st[:k], "pos": sp[:k], "vel": sv[:k], "aei": sa[:k].reshape(k, n, 3),
                "energy": se[:k], "flag": rc}

    def measure_fp64_issue(self, active_lanes):
        """FP64 FMA rate counted over whole warps with only active_lanes lanes working."""
        v = _c.c_double(0)
        self._check(self.lib.abie_measure_fp64_issue(_c.c_int(active_lanes), _c.byref(v)),
                    "fp64 issue probe")
        return v.value

    def measure_peaks(self):
        f64, f32 = _c.c_double(0), _c.c_double(0)
        self._check(self.lib.abie_measure_fp64_peak(_c.c_int(0), _c.byref(f64)), "fp64 probe")
        self._check(self.lib.abie_measure_fp32_peak(_c.c_int(0), _c.byref(f32)), "fp32 probe")
        return {"fp64_tflops": f64.value, "fp32_tflops": f32.value}

    # -- learned Radau15 predictor -----------------------------------------------
    def _mlp_sig(self):
        L = self.lib
        L.abie_mlp_init.argtypes = [_c.c_int, _c.c_void_p]
        L.abie_mlp_train.argtypes = [_c.c_int, _c.c_int, _c.c_double, _c.c_int, _c.c_void_p]
        L.abie_mlp_load_samples.argtypes = [_c.c_void_p, _c.c_longlong]
        L.abie_mlp_get_samples.argtypes = [_c.c_void_p, _c.c_longlong]
        L.abie_mlp_sample_count.restype = _c.c_longlong
        L.abie_mlp_set_params.argtypes = [_c.c_void_p, _c.c_int, _c.c_void_p]
        L.abie_mlp_get_params.argtypes = [_c.c_void_p, _c.c_int]
        L.abie_mlp_set_capacity.argtypes = [_c.c_longlong]
        return L

    @staticmethod
    def _tau7(tau):
        t = np.ones(7) if tau is None else np.broadcast_to(np.asarray(tau, dtype=np.float64), (7,))
        return np.ascontiguousarray(t, dtype=np.float64)

    def mlp_init(self, seed=0, tau=None):
        """Fresh weights (zero output layer); tau: 7 output scales (or one)."""
        t = self._tau7(tau)
        self._check(self._mlp_sig().abie_mlp_init(int(seed), t.ctypes.data), "abie_mlp_init")

    def mlp_enable(self, on=True):
        self.lib.abie_mlp_enable(_c.c_int(int(bool(on))))

    def mlp_clear_samples(self):
        self.lib.abie_mlp_clear_samples()

    def mlp_set_capacity(self, samples):
        self._mlp_sig().abie_mlp_set_capacity(int(samples))

    def mlp_samples(self):
        L = self._mlp_sig()
        n = L.abie_mlp_sample_count()
        out = np.zeros((max(n, 0), 64), dtype=np.float32)
        if n > 0:
            L.abie_mlp_get_samples(out.ctypes.data, n)
        return out

    def mlp_load_samples(self, samples):
        samples = np.ascontiguousarray(samples, dtype=np.float32)
        self._check(self._mlp_sig().abie_mlp_load_samples(samples.ctypes.data, samples.shape[0]),
                    "abie_mlp_load_samples")

    def mlp_train(self, steps, batch, lr, seed=0):
        loss = _c.c_double(0)
        self._check(self._mlp_sig().abie_mlp_train(int(steps), int(batch), float(lr), int(seed),
                                                   _c.byref(loss)), "abie_mlp_train")
        return loss.value

    def mlp_params(self):
        L = self._mlp_sig()
        n = L.abie_mlp_n_params()
        out = np.zeros(n, dtype=np.float32)
        self._check(L.abie_mlp_get_params(out.ctypes.data, n), "abie_mlp_get_params")
        return out

    def mlp_set_params(self, params, tau=None):
        params = np.ascontiguousarray(params, dtype=np.float32)
        t = self._tau7(tau)
        self._check(self._mlp_sig().abie_mlp_set_params(params.ctypes.data, params.size,
                                                        t.ctypes.data), "abie_mlp_set_params")
