"""Build the CUDA library libtoed_gb300.so in-tree for sm_103a.

Every csrc/*.cu is compiled in parallel with nvcc (one -gencode, no cmake)
and linked into ``libtoed_gb300.so`` next to this file.  Objects go to
``_build/`` (git-ignored).  Rebuilds are incremental on source mtimes.

``build(debug=True)`` builds the bounds-checked variant instead
(-DTOED_DEBUG_BOUNDS: every guarded shared- and global-memory index of the
detection kernel is checked, a failure skips the access and raises
TOED_FLAG_BOUNDS): ``libtoed_gb300_debug.so``, objects in ``_build_debug/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtoed_gb300.so")
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(HERE, "libtoed_gb300_debug.so")
INCLUDE = os.path.abspath(os.path.join(HERE, "..", "include"))
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ["-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
            "-Wno-deprecated-gpu-targets"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(src: str, obj: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return m < os.path.getmtime(src) or m < hdr_mtime


def build(verbose: bool = False, jobs: int | None = None, debug: bool = False) -> str:
    bdir, lib = (BUILD_DEBUG, LIB_DEBUG) if debug else (BUILD, LIB)
    extra = ["-DTOED_DEBUG_BOUNDS"] if debug else []
    os.makedirs(bdir, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_mtime = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(bdir, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(s, o, hdr_mtime):
            todo.append((s, o))
    cc = nvcc()

    def compile_one(so):
        s, o = so
        cmd = [cc] + _flags() + extra + ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return s

    if todo:
        jobs = jobs or max(1, min(len(todo), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(jobs) as ex:
            for s in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(s))
    if todo or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        tmp = lib + ".tmp"
        cmd = [cc, ARCH, "-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
        os.replace(tmp, lib)
    if debug:
        return lib
    build_driver(verbose)
    build_probe(verbose)
    return LIB


PROBE_SRC = os.path.join(HERE, "probe", "toed_probe.cu")
PROBE_LIB = os.path.join(HERE, "libtoed_probe.so")


def build_probe(verbose: bool = False) -> str:
    """bench.py's FP32 / FP64 FMA-rate probe, a library of its own (not part
    of the detector's C ABI)."""
    if os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= os.path.getmtime(PROBE_SRC):
        return PROBE_LIB
    tmp = PROBE_LIB + ".tmp"
    cmd = [nvcc()] + _flags() + ["-shared", PROBE_SRC, "-o", tmp, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("probe build failed:\n" + r.stderr)
    os.replace(tmp, PROBE_LIB)
    if verbose:
        print("built", PROBE_LIB)
    return PROBE_LIB


DRIVER_SRC = os.path.join(HERE, "driver", "toed_batch.cpp")
DRIVER = os.path.join(HERE, "toed_batch")


def build_driver(verbose: bool = False) -> str:
    """The batch command-line driver (host C++ over the C ABI): g++, linked
    against the library with an rpath to it."""
    import platform
    stamp = DRIVER + ".arch"  # the machine the binary was built for (the tree may move between hosts)
    if (os.path.exists(DRIVER) and os.path.exists(stamp) and open(stamp).read() == platform.machine()
            and os.path.getmtime(DRIVER) >= max(os.path.getmtime(DRIVER_SRC), os.path.getmtime(LIB))):
        return DRIVER
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"),
           DRIVER_SRC, "-o", DRIVER, LIB, "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lpthread",
           "-Wl,-rpath," + HERE, "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n" + r.stderr)
    with open(stamp, "w") as f:
        f.write(platform.machine())
    if verbose:
        print("built", DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose=True))
