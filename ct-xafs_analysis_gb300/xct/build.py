"""Build libxct.so (CUDA, sm_103a) and the C++ drop-in host tools, in-tree.

Each .cu translation unit is compiled by its own nvcc process in parallel, then linked
into ``xct/libxct.so`` (the CUDA runtime is linked statically, so the library needs only
the driver).  Flags: ``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo
--fmad=false`` -- FMAs are written explicitly in the kernels, and nothing else may be
contracted (the backprojector's nearest-bin arithmetic must round exactly as the
reference's expression does).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # ct-xafs_analysis_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
HOST = os.path.join(ROOT, "host")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libxct.so")
LIB_CHECKED = os.path.join(PKG, "libxct_checked.so")
HOST_BIN = os.path.join(PKG, "xct_ct_reconstruction")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                  "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdr = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdr.append(os.path.join(INCLUDE, "xct.h"))
    return cu, hdr


def build_lib(force=False, verbose=False, extra=(), checked=False):
    """libxct.so; with checked, libxct_checked.so: the same sources with -DXCT_CHECKED (every
    shared-memory access whose address follows from geometry is tested against its buffer,
    see csrc/xct_check.cuh), in a build folder of its own."""
    cu, hdr = _sources()
    build_dir = BUILD + ("_checked" if checked else "")
    lib = LIB_CHECKED if checked else LIB
    extra = list(extra) + (["-DXCT_CHECKED"] if checked else [])
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    jobs = []
    for src in cu:
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdr):
            jobs.append([nvcc] + NVFLAGS + list(extra) + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, res):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _newer(lib, objs):
        tmp = lib + ".tmp%d" % os.getpid()
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed: " + " ".join(cmd))
        os.replace(tmp, lib)
    return lib


def build_host(force=False):
    """The C++ drop-in executable (CT_reconstruction equivalent) linked against libxct."""
    if not os.path.isdir(HOST):
        return None
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    if not srcs:
        return None
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".hpp", ".h"))]
    if not (force or _newer(HOST_BIN, srcs + hdrs + [LIB])):
        return HOST_BIN
    tmp = HOST_BIN + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I" + INCLUDE, "-I" + HOST, "-o", tmp] + srcs + [
        "-L" + PKG, "-lxct", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("host build failed")
    os.replace(tmp, HOST_BIN)
    return HOST_BIN


def build(force=False, verbose=False):
    lib = build_lib(force=force, verbose=verbose)
    build_host(force=force)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
