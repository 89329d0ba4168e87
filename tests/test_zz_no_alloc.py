"""The allocation-free force entry point (for callers that cannot allocate
GPU memory: inside a capture that must hold no allocation, or with only
their own buffers to spend) against the allocating one, through the C ABI.

Collected last on purpose: it runs after every other test, and must also
pass alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from abie_gb300 import FORCE_FP64, ics
from conftest import rel_err_per_body

pytestmark = pytest.mark.gpu
G = ics.G_SOLAR
C = ctypes
ERR_CAPACITY = -6


def _bind(lib):
    lib.abie_force_device_noalloc.restype = C.c_int
    lib.abie_force_device_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_double,
                                              C.c_void_p, C.c_void_p]
    return lib


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(clib):
    import torch
    lib = _bind(clib.lib)
    dev = torch.device("cuda", 0)
    cases = []
    p, v, m, r = ics.planetesimal_disk(seed=21, n=3000)
    cases.append((p, m))
    p, v, m, r = ics.planetary_system(seed=22, n_planets=9, n_tp=700)  # fewer sources, some massless
    cases.append((p, m))
    for p, m in cases:
        pos = torch.from_numpy(p).to(dev)
        mass = torch.from_numpy(m).to(dev)
        a_ref = torch.zeros_like(pos)
        a_new = torch.full_like(pos, np.nan)
        torch.cuda.synchronize()
        rc = lib.abie_force_device(C.c_void_p(pos.data_ptr()), C.c_void_p(mass.data_ptr()),
                                   C.c_size_t(m.size), C.c_double(G), C.c_void_p(a_ref.data_ptr()),
                                   C.c_int(FORCE_FP64), None)
        assert rc == 0
        rc = lib.abie_force_device_noalloc(pos.data_ptr(), mass.data_ptr(), m.size, G,
                                           a_new.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        ref, new = a_ref.cpu().numpy(), a_new.cpu().numpy()
        assert np.isfinite(new).all()
        assert rel_err_per_body(new, ref) <= 1e-13


def test_noalloc_rejects_sizes_beyond_its_scratch(clib):
    lib = _bind(clib.lib)
    rc = lib.abie_force_device_noalloc(None, None, 65537, G, None, None)
    assert rc == ERR_CAPACITY
