"""Runs the reference's own Python package, unchanged, on a given libabie.

Test helper, run in a fresh process by tests/test_dropin_*.py:

    python dropin_driver.py PKG_ROOT OUT.npz INTEGRATOR DEVICE T_END H STATE.npz

PKG_ROOT holds the reference's ``abie/`` package (copied unmodified from
the pip install in baseline/_ref) and, beside it, the ``libabie<EXT_SUFFIX>``
that its abie/clibabie.py:9-28 loads: this library or the reference's own.
h5py and toml are not installed here (nor six on every machine), so
minimal stand-ins (an in-memory HDF5 file object with groups, datasets and
attrs; toml functions that are never reached; six.string_types) are put on
the path first: they stand in only for the
reference's output layer, which is not on the path under test.

The script builds the system with ``abie.ABIE(deviceID=...)``, ``add()``,
``sim.integrator = ...``, ``sim.h``, then ``sim.integrate(T_END)`` and
saves the final positions, velocities, model time and energies.
"""
import os
import sys
import types

import numpy as np


def _install_stubs():
    h5 = types.ModuleType("h5py")

    class _Group(dict):
        def __init__(self):
            super().__init__()
            self.attrs = {}

        def create_group(self, name):
            g = _Group()
            self[name] = g
            return g

        def create_dataset(self, name, data=None):
            self[name] = np.array(data)
            return self[name]

    class File(_Group):
        def __init__(self, name, mode="r"):
            super().__init__()
            self.name = name

        def flush(self):
            pass

        def close(self):
            pass

    h5.File = File
    sys.modules["h5py"] = h5
    tm = types.ModuleType("toml")

    def _unused(*a, **k):
        raise RuntimeError("toml is not available in this harness")

    tm.loads = tm.load = tm.dump = tm.dumps = _unused
    sys.modules["toml"] = tm
    try:
        import six  # noqa: F401  (the reference's particles.py imports six.string_types)
    except ImportError:
        sx = types.ModuleType("six")
        sx.string_types = (str,)
        sys.modules["six"] = sx


def main():
    pkg_root, out, integrator, device, t_end, h = sys.argv[1:7]
    state = np.load(sys.argv[7])
    _install_stubs()
    sys.path.insert(0, pkg_root)
    os.chdir(os.path.dirname(os.path.abspath(out)))
    import abie

    assert os.path.dirname(abie.__file__) == os.path.join(pkg_root, "abie"), abie.__file__
    pos, vel, m = state["pos"].reshape(-1, 3), state["vel"].reshape(-1, 3), state["m"]
    sim = abie.ABIE(CONST_G=float(state["G"]), name="dropin", deviceID=int(device))
    for k in range(m.size):
        sim.add(mass=float(m[k]), x=pos[k, 0], y=pos[k, 1], z=pos[k, 2], vx=vel[k, 0],
                vy=vel[k, 1], vz=vel[k, 2], name="b%d" % k)
    sim.integrator = integrator
    sim.h = float(h)
    sim.store_dt = 1e6  # one chunk: integrate() calls the library once
    sim.integrate(float(t_end))
    lib = sim.integrator.libabie
    np.savez(out, pos=sim.particles.positions, vel=sim.particles.velocities,
             t=np.array([sim.t]), energy=np.array([lib.get_total_energy()]),
             lib=np.array(lib.lib._name))
    sim.stop()


if __name__ == "__main__":
    main()
