"""Builds the in-tree CUDA library hfgpu/libhfgpu.so for sm_103a with nvcc (no cmake, no torch).

The 21 shell-quartet classes are separate translation units (csrc/classes.cu with -DHFG_QCLASS=c) and
compile in parallel; objects are cached in _build/ keyed by source contents and flags.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)  # hartree-fock_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libhfgpu.so")
NUM_CLASSES = 21

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
              "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-std=c++20", "-O2", "-fPIC", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _headers() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))) + [
        os.path.join(INCLUDE, "hfgpu.h")]


def _digest(paths, extra) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()[:16]


def _units():
    hdrs = _headers()
    units = []
    for c in range(NUM_CLASSES):
        src = os.path.join(CSRC, "classes.cu")
        for part in range(3):  # FP64 Fock kernels, FP32 Fock kernels, gradient kernels
            flags = NVCC_FLAGS + [f"-DHFG_QCLASS={c}", f"-DHFG_PART={part}"]
            units.append(("nvcc", src, flags, f"class{c:02d}p{part}", hdrs))
    for name in ("engine.cu", "dispatch.cu", "peak.cu", "boys_check.cu", "scf_device.cu", "onee.cu", "persistent.cu"):
        units.append(("nvcc", os.path.join(CSRC, name), NVCC_FLAGS, name[:-3], hdrs))
    for name in sorted(os.listdir(CSRC)):
        if name.endswith(".cpp"):
            units.append(("cxx", os.path.join(CSRC, name), CXX_FLAGS + ["-I" + os.path.join(cuda_home(), "include")],
                          name[:-4], hdrs))
    return units


def _compile(unit):
    kind, src, flags, stem, hdrs = unit
    key = _digest([src] + hdrs, flags + [kind])
    obj = os.path.join(BUILD_DIR, f"{stem}-{key}.o")
    if os.path.exists(obj):
        return obj, False
    cmd = ([nvcc()] + flags + ["-c", src, "-o", obj + ".tmp"]) if kind == "nvcc" else (
        [os.environ.get("CXX", "g++")] + flags + ["-c", src, "-o", obj + ".tmp"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, True


def build(verbose: bool = True, jobs: int | None = None) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    units = _units()
    jobs = jobs or max(1, min(len(units), os.cpu_count() or 4))
    # Longest first: the d-class units dominate the wall time.
    order = sorted(units, key=lambda u: (u[3].startswith("class") and int(u[3][5:7]) or 0), reverse=True)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(_compile, order))
    objs = [o for o, _ in results]
    # Drop cached objects of earlier source versions.
    keep = {os.path.basename(o) for o in objs}
    for name in os.listdir(BUILD_DIR):
        if name.endswith(".o") and name not in keep:
            os.remove(os.path.join(BUILD_DIR, name))
    rebuilt = any(b for _, b in results) or not os.path.exists(LIB_PATH)
    if rebuilt:
        cuda_lib = os.path.join(cuda_home(), "lib64")
        if not os.path.isdir(cuda_lib):
            cuda_lib = os.path.join(cuda_home(), "lib")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB_PATH + ".tmp"] + objs + [
            "-L" + cuda_lib, "-lcudart", "-lcublas", "-lcusolver", "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    if verbose:
        print(f"hfgpu: {LIB_PATH} ({'rebuilt' if rebuilt else 'up to date'})", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build()
