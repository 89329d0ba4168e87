"""The allocation-free force entry point against the allocating one, through
the C ABI.  It serves callers that may not call cudaMalloc (a real-time
loop that must not block on the allocator, or a budget limited to their own
buffers).

Sizes: 3,000 and 709 bodies take the same one-chunk kernel in both entry
points; 8,192 and 65,536 all-massive bodies (the scratch's limit) meet the
symmetric form of abie_force_device, and 10,000 bodies with massless and
deleted ones meet its two-chunk form, so those agree to rounding (1e-13 per
body).  Deleted sinks (m < 0) keep their acc entries in both.  Every case
runs two calls in a row.

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
MAX_BODIES = 65536
SENTINEL = 12345.0


def _bind(lib):
    lib.abie_force_device_noalloc.restype = C.c_int
    lib.abie_force_device_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_double,
                                              C.c_void_p, C.c_void_p]
    return lib


def _cases():
    p, v, m, r = ics.planetesimal_disk(seed=21, n=3000)
    yield "disk-3001", p, m
    p, v, m, r = ics.planetary_system(seed=22, n_planets=9, n_tp=700)  # fewer sources, some massless
    yield "system-710", p, m
    p, v, m, r = ics.planetesimal_disk(seed=23, n=8191)                 # 8,192 bodies, all massive
    yield "disk-8192", p, m
    p, v, m, r = ics.planetesimal_disk(seed=24, n=9999)                 # 10,000 bodies
    rng = np.random.default_rng(25)
    idx = rng.permutation(m.size)
    m = m.copy()
    m[idx[:2000]] = 0.0      # massless
    m[idx[2000:2100]] = -1.0  # deleted
    yield "mixed-10000", p, m
    p, v, m, r = ics.planetesimal_disk(seed=26, n=MAX_BODIES - 1)       # the scratch's limit
    yield "disk-65536", p, m


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(clib):
    import torch
    lib = _bind(clib.lib)
    dev = torch.device("cuda", 0)
    for name, p, m in _cases():
        pos = torch.from_numpy(p).to(dev)
        mass = torch.from_numpy(m).to(dev)
        a_ref = torch.full_like(pos, SENTINEL)
        torch.cuda.synchronize()
        rc = lib.abie_force_device(C.c_void_p(pos.data_ptr()), C.c_void_p(mass.data_ptr()),
                                   C.c_size_t(m.size), C.c_double(G), C.c_void_p(a_ref.data_ptr()),
                                   C.c_int(FORCE_FP64), None)
        assert rc == 0, name
        torch.cuda.synchronize()
        ref = a_ref.cpu().numpy()
        live = np.repeat(m >= 0.0, 3)
        for call in range(2):  # two calls in a row share the scratch
            a_new = torch.full_like(pos, SENTINEL)
            rc = lib.abie_force_device_noalloc(pos.data_ptr(), mass.data_ptr(), m.size, G,
                                               a_new.data_ptr(), None)
            assert rc == 0, (name, call)
            torch.cuda.synchronize()
            new = a_new.cpu().numpy()
            assert np.isfinite(new).all(), (name, call)
            assert (new[~live] == SENTINEL).all() and (ref[~live] == SENTINEL).all(), (name, call)
            err = rel_err_per_body(new[live], ref[live])
            assert err <= 1e-13, (name, call, err)


def test_noalloc_rejects_sizes_beyond_its_scratch(clib):
    lib = _bind(clib.lib)
    assert lib.abie_force_device_noalloc(None, None, MAX_BODIES + 1, G, None, None) == ERR_CAPACITY
    # the full size_t is checked: 2^32 + 10 is not run as 10 bodies
    assert lib.abie_force_device_noalloc(None, None, (1 << 32) + 10, G, None, None) == ERR_CAPACITY
