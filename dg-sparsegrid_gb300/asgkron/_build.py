"""Compile the asgkron CUDA library (libasgkron.so) for sm_103a, in-tree.

Each translation unit is compiled by nvcc in parallel, then linked into one shared
library with the CUDA runtime linked statically (the library is loaded by ctypes; device
pointers and streams from the caller's CUDA context are valid in it).
"""
import os
import subprocess
import sys
import time

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # dg-sparsegrid_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libasgkron.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
          "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(INCLUDE, "asgkron.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Build libasgkron.so if missing or stale; returns its path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    t0 = time.time()
    procs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        cmd = [nvcc] + lang + ARCH + COMMON + ["-c", src, "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        procs.append((src, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, cmd, pr in procs:
        out, _ = pr.communicate()
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
        if pr.returncode != 0:
            failed.append((src, " ".join(cmd), out.decode(errors="replace")))
    if failed:
        msg = "\n".join("%s\n%s\n%s" % f for f in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    link = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(link), r.stdout.decode(errors="replace")))
    os.replace(tmp, LIB_PATH)
    if verbose:
        print("built %s in %.1fs" % (LIB_PATH, time.time() - t0))
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
