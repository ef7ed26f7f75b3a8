"""Build the CUDA library ``libsqrtsmooth.so`` in-tree for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled by ``nvcc`` in parallel into
``_build/`` and linked into ``sqrt_parallel_smoothers_gb300/_lib/``.  Units
whose object is newer than every source and header are not recompiled.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsqrtsmooth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sqrtsmooth")
    return path


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src, newest_header):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return t < os.path.getmtime(src) or t < newest_header


def _compile(src, obj, verbose):
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr[-4000:]}")
    return r.stderr


def _weight(src):
    """Rough compile cost of an instantiation unit: dual-number units, FP64 and larger state
    sizes take longest."""
    name = os.path.basename(src)
    nums = [int(t) for t in name[:-3].split("_") if t.isdigit()]
    nx = nums[0] if nums else 0
    return 4 * ("grad" in name) + 2 * ("f64" in name) + ("adj" in name) + nx / 4


def build(verbose=False, jobs=None):
    """Compile and link the library; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    newest = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, s, newest):
            todo.append((s, o))
    jobs = jobs or max(1, min(len(todo), os.cpu_count() or 1))
    if todo:
        # the largest units first so the tail of the parallel build is short
        todo.sort(key=lambda so: -_weight(so[0]))
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for log in ex.map(lambda so: _compile(so[0], so[1], verbose), todo):
                if verbose and log:
                    print(log)
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=False))
