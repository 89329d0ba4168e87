"""Set-up for running the reference's unchanged Python package on a chosen
libabie (tests/dropin_driver.py does the run).

The package comes from the reference's own pip install into baseline/_ref
(``pip install --no-index --no-build-isolation --target baseline/_ref
<reference>``), which travels with the repository to the GPU machine; its
files are copied unmodified into a scratch directory, next to a symlink
``libabie<EXT_SUFFIX>`` to the library under test, where the reference's
abie/clibabie.py:9-28 looks for it."""
import os
import shutil
import subprocess
import sys
import sysconfig

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_PKG = os.path.join(ROOT, "baseline", "_ref", "abie")
DRIVER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin_driver.py")


def available():
    return os.path.isfile(os.path.join(REF_PKG, "clibabie.py"))


def stage(tmp, lib_path):
    """The reference package beside a libabie that is lib_path; returns the root."""
    root = os.path.join(str(tmp), "pkg")
    os.makedirs(root, exist_ok=True)
    shutil.copytree(REF_PKG, os.path.join(root, "abie"),
                    ignore=shutil.ignore_patterns("__pycache__"))
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    os.symlink(os.path.abspath(lib_path), os.path.join(root, "libabie" + suffix))
    return root


def run(tmp, root, integrator, device, t_end, h, pos, vel, m, G):
    state = os.path.join(str(tmp), "state_%s.npz" % integrator)
    out = os.path.join(str(tmp), "out_%s.npz" % integrator)
    np.savez(state, pos=pos, vel=vel, m=m, G=np.array(G))
    res = subprocess.run([sys.executable, DRIVER, root, out, integrator, str(device), repr(t_end),
                          repr(h), state], capture_output=True, text=True, timeout=600)
    if res.returncode != 0:
        raise RuntimeError("drop-in run failed:\n" + res.stdout[-3000:] + res.stderr[-3000:])
    return dict(np.load(out)), res.stdout + res.stderr
