"""Build libmsk.so in-tree with nvcc for sm_103a (GB300).

    python -m utr_public_gb300._build          # or __graft_entry__.build()

Every .cu and .cpp file under csrc/ compiles in parallel to an object in _build/,
then the objects link into utr_public_gb300/libmsk.so with the CUDA runtime
linked statically.  Host code is compiled with -ffp-contract=off so that the
reference-exact host arithmetic rounds the same on x86-64 and aarch64.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmsk.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                     "-I" + CSRC]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmsk.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(target, inputs):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in inputs)


def build(verbose=False, jobs=None):
    """Compile (incrementally) and return the path of libmsk.so."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    deps = _deps()
    todo = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [cc] + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        os.replace(obj + ".tmp", obj)
        return src

    if todo:
        jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(jobs) as ex:
            for src in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.relpath(src, ROOT))
    if todo or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-cudart", "static", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
        if verbose:
            print("linked", os.path.relpath(LIB, ROOT))
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
