"""Builds libgvs.so (CUDA sm_103a) in-tree with nvcc.

Every translation unit under gravis_gb300/csrc is compiled in parallel with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then linked into
gravis_gb300/libgvs.so (CUDA runtime linked statically).  Objects go to
gravis_gb300/_build/ (git-ignored).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgvs.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code must not fuse a*b+c (GCC does by default on aarch64): the initial
# conditions and host reductions follow the reference's unfused f64 arithmetic.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills", "-diag-suppress", "1444,177"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgvs.so")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


# Per-file flags: the SPH kernels restate the reference's f64 arithmetic
# statement by statement, so a*b+c must round twice there.
FILE_FLAGS = {"sph.cu": ["--fmad=false"]}


def _compile(nvcc: str, src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _stale(obj, src):
        cmd = [nvcc] + ARCH + NVCC_FLAGS + FILE_FLAGS.get(os.path.basename(src), []) + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose():
            sys.stderr.write(r.stderr)
    return obj


def verbose() -> bool:
    return os.environ.get("GVS_BUILD_VERBOSE", "") not in ("", "0")


def build(force: bool = False, extra: list[str] | None = None) -> str:
    """Compile all sources and link libgvs.so; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = list(extra or [])
    if verbose():
        extra += ["-Xptxas", "-v"]
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(ARCH + NVCC_FLAGS + extra) + repr(sorted(FILE_FLAGS.items()))
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        force = True
        with open(stamp, "w") as fh:
            fh.write(flags)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    if force:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    build_host()
    return LIB


HOST = os.path.join(HERE, "host")
HEADLESS = os.path.join(HERE, "gvs_headless")
HOST_CHECK = os.path.join(HERE, "gvs_host_check")


def _host_binary(out: str, main_src: str) -> str:
    srcs = [os.path.join(HOST, "gravis.cpp"), os.path.join(HOST, main_src)]
    deps = srcs + [os.path.join(HOST, "gravis.hpp"), os.path.join(ROOT, "include", "gvs.h"), LIB]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = out + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wextra", "-o", tmp] + srcs + \
          ["-L" + HERE, "-lgvs", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host build failed ({main_src}):\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build_host() -> str:
    """The C++ host layer (host/gravis.cpp): the headless runner and the check
    program of the drop-in classes, linked against libgvs.so (found next to the
    binaries at run time)."""
    _host_binary(HOST_CHECK, "host_check.cpp")
    return _host_binary(HEADLESS, "headless.cpp")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
