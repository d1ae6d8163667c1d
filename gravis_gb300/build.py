"""Builds libgvs.so (CUDA sm_103a) in-tree with nvcc.

Every translation unit under gravis_gb300/csrc is compiled in parallel with
`-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then linked into
gravis_gb300/libgvs.so (CUDA runtime linked statically), and again with
-DGVS_CHECKED into gravis_gb300/libgvs_checked.so (the bounds-checked build).
Objects go to gravis_gb300/_build/ and _build_checked/ (git-ignored).
Rebuilds only what changed.
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
FILE_FLAGS = {"sph.cu": ["--fmad=false"], "ics_dev.cu": ["--fmad=false"]}


def _compile(nvcc: str, src: str, extra: list[str], build_dir: str) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
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


# The checked build: the same sources with -DGVS_CHECKED (kernels test the indices
# they compute and the tree build its invariants; see csrc/gvs_internal.cuh),
# linked as libgvs_checked.so from objects in _build_checked/.
CHECKED_LIB = os.path.join(HERE, "libgvs_checked.so")
VARIANTS = {"normal": (BUILD, LIB, []), "checked": (os.path.join(HERE, "_build_checked"), CHECKED_LIB,
                                                    ["-DGVS_CHECKED"])}


def build(force: bool = False, extra: list[str] | None = None, checked: bool = True) -> str:
    """Compile all sources and link libgvs.so (and, with checked, libgvs_checked.so:
    both variants' translation units compile in one parallel pool); returns the path
    of libgvs.so."""
    nvcc = _nvcc()
    extra = list(extra or [])
    if verbose():
        extra += ["-Xptxas", "-v"]
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    variants = ["normal", "checked"] if checked else ["normal"]
    jobs = []
    for v in variants:
        bdir, _, vflags = VARIANTS[v]
        os.makedirs(bdir, exist_ok=True)
        stamp = os.path.join(bdir, "flags.txt")
        flags = " ".join(ARCH + NVCC_FLAGS + extra + vflags) + repr(sorted(FILE_FLAGS.items()))
        vforce = force
        if not os.path.exists(stamp) or open(stamp).read() != flags:
            vforce = True
            with open(stamp, "w") as fh:
                fh.write(flags)
        if vforce:
            for o in glob.glob(os.path.join(bdir, "*.o")):
                os.remove(o)
        jobs += [(v, src, extra + vflags, bdir) for src in srcs]
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda j: (j[0], _compile(nvcc, j[1], j[2], j[3])), jobs))
    for v in variants:
        _, lib, _ = VARIANTS[v]
        vobjs = [o for vv, o in objs if vv == v]
        if not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in vobjs):
            tmp = lib + ".tmp"
            cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + vobjs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed ({v}):\n{r.stdout}\n{r.stderr}")
            os.replace(tmp, lib)
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
