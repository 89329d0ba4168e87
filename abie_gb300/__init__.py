"""GB300 (sm_103a) implementation of ABIE's gravity hot path.

``libabie_gb300.so`` exports the reference library's C entry points
(initialize_code, set_state, integrator_gr, integrator_wh, ...; see
include/abie_gb300.h) over a GPU-resident state, plus additive entry points
for explicit force forms, device pointers, counters and batched ensembles.
``abie_gb300.clibabie.CLibABIE`` is the ctypes binding with the reference
binding's method names (abie/clibabie.py).

The library is built in-tree by ``abie_gb300.build.build()``; importing the
binding without a built library raises, there is no fallback.
"""
import ctypes
import os

from . import build as _build

FORCE_EXACT = 0
FORCE_FP64 = 1
FORCE_MIXED = 2
FORCE_NAIVE = 3
FORCE_MODES = {"exact": FORCE_EXACT, "fp64": FORCE_FP64, "mixed": FORCE_MIXED,
               "naive": FORCE_NAIVE}

LIB_PATH = _build.LIB
_lib = None


def library_path():
    return LIB_PATH


def load(path=None):
    """Load (once) and return the ctypes handle of libabie_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.isfile(path):
        raise ImportError("libabie_gb300.so is not built (%s); run "
                          "abie_gb300.build.build() or __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    d, i, sz, vp = ctypes.c_double, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p
    lib.get_model_time.restype = d
    lib.calculate_energy.restype = d
    lib.get_close_encounter_distance.restype = d
    lib.abie_energy_host.restype = d
    lib.abie_last_ensemble_seconds.restype = d
    lib.integrator_gr.restype = i
    lib.integrator_wh.restype = i
    lib.integrator_rk.restype = i
    lib.initialize_code.restype = i
    lib.finalize_code.restype = i
    lib.get_state.restype = i
    lib.set_additional_forces.restype = sz
    lib.ode_n_body_second_order.restype = sz
    lib.calculate_accelerations.restype = sz
    lib.abie_force_host.restype = i
    lib.abie_force_device.restype = i
    lib.abie_force_device.argtypes = [vp, vp, sz, d, vp, i, vp]
    lib.abie_gr_ensemble.restype = i
    lib.abie_set_force_mode.restype = i
    lib.abie_get_force_mode.restype = i
    lib.abie_measure_fp64_peak.restype = i
    lib.abie_measure_fp32_peak.restype = i
    lib.abie_last_error.restype = i
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(1024)
    lib.abie_last_error(buf, ctypes.c_size_t(len(buf)))
    return buf.value.decode(errors="replace")
