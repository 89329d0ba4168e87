"""Build libabie_gb300.so in-tree with nvcc for sm_103a.

Each .cu under csrc/ compiles to its own object in parallel; the objects link
into one shared library with the CUDA runtime linked statically, so the
library loads on machines without a GPU driver (its calls then report that
no device is present).  Device code is sm_103a only; every unit is built
with --fmad=false (see csrc/common.cuh), except the plain FP64 ensemble
form (ensemble_plain.cu), built with FMA contraction.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libabie_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=default", "--expt-relaxed-constexpr",
              "-I" + CSRC, "-I" + INCLUDE]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


# Units whose flags differ: the plain FP64 ensemble form is the reference's
# expressions compiled with FMA contraction, as a straightforward port.
FMAD_TRUE = {"ensemble_plain.cu"}


def _flags(src):
    if os.path.basename(src) in FMAD_TRUE:
        return [f if f != "--fmad=false" else "--fmad=true" for f in NVCC_FLAGS]
    return NVCC_FLAGS


def _fingerprint():
    h = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))):
        with open(p, "rb") as fh:
            h.update(p.encode() + fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + sorted(FMAD_TRUE)).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile and link; returns the library path.  Skips work when nothing changed."""
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp")
    fp = _fingerprint()
    if not force and os.path.isfile(LIB) and os.path.isfile(stamp):
        with open(stamp) as fh:
            if fh.read() == fp:
                return LIB
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + ARCH + _flags(src) + extra + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        return src, obj, res

    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for src, obj, res in ex.map(compile_one, _sources()):
            if res.returncode != 0:
                raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, res.stdout, res.stderr))
            if verbose or ptxas_verbose:
                sys.stderr.write(res.stdout + res.stderr)
            objs.append(obj)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-ldl", "-lrt"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                ptxas_verbose="--ptxas" in sys.argv))
