"""Build libsphgb.so (the CUDA kernels and the C ABI) for sm_103a, in tree.

Each translation unit under ``csrc/`` is compiled by its own nvcc process, in
parallel, then linked into ``sphgb/libsphgb.so``.  The CUDA runtime is linked
statically, so the library only needs the NVIDIA kernel driver (libcuda) at
run time.  No fast-math:
the kernels rely on IEEE division, square root and denormals for the exact
voxel and neighbour decisions.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libsphgb.so")
# what the library was built on and with: a library built elsewhere (another
# machine type, other flags) is never taken as up to date
STAMP_PATH = os.path.join(BUILD_DIR, "libsphgb.stamp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libsphgb.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stamp(flags) -> str:
    h = hashlib.sha256()
    for src in sorted(_deps()):
        with open(src, "rb") as f:
            h.update(os.path.basename(src).encode() + b"\0" + f.read())
    return f"{platform.machine()} {' '.join(flags)} {h.hexdigest()}"


def up_to_date(extra_flags=None) -> bool:
    """The library exists and was built here, from these sources, with
    these flags (not merely newer than the sources)."""
    if not os.path.exists(LIB_PATH) or not os.path.exists(STAMP_PATH):
        return False
    with open(STAMP_PATH) as f:
        return f.read() == _stamp(NVCC_FLAGS + list(extra_flags or []))


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and up_to_date(extra_flags):
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    flags = NVCC_FLAGS + list(extra_flags or [])
    objs = []
    cmds = []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmds.append([nvcc] + flags + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        outs = list(ex.map(run, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB_PATH + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    with open(STAMP_PATH, "w") as f:
        f.write(_stamp(flags))
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
