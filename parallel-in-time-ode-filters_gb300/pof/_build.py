"""Build libpof.so in-tree: nvcc for sm_103a, one job per translation unit.

    python -m pof._build          (from parallel-in-time-ode-filters_gb300/)

Objects go to ``parallel-in-time-ode-filters_gb300/_build/``; the shared
library is written next to this file (``pof/libpof.so``), which is where
``pof._lib`` loads it from.  A rebuild happens only when a source or header
is newer than the library.
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
BUILD_CHECKED = os.path.join(ROOT, "_build_checked")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
LIB = os.path.join(PKG_DIR, "libpof.so")
# the same sources with the runtime bounds checks (POF_CHECKS; relocatable
# device code, so every unit shares the check word)
LIB_CHECKED = os.path.join(PKG_DIR, "libpof_checked.so")
CHECK_FLAGS = ["-DPOF_CHECKS", "-rdc=true", "-DPOF_SHAPE_SUBSET"]
# shapes of the checked build (the registries' POF_SHAPE_SUBSET lists)
CHECK_SHAPES = ("pof_inst_D3_d1.cu", "pof_inst_D8_d2.cu", "pof_inst_D12_d3.cu", "pof_inst_D3_d4.cu",
                "pof_binst_D8_d2.cu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE] + ARCH


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libpof.so needs the CUDA toolkit to build")


def sources(checks=False):
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    if checks:
        srcs = [p for p in srcs if not os.path.basename(p).startswith(("pof_inst_", "pof_binst_"))
                or os.path.basename(p) in CHECK_SHAPES]
    return srcs


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(src, build_dir=BUILD, extra=()):
    obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-4000:]))
    return obj


def build(force=False, jobs=None, verbose=True, checks=False):
    """Compile every CUDA source and link libpof.so (checks=True:
    libpof_checked.so, with the runtime bounds checks); returns its path."""
    lib = LIB_CHECKED if checks else LIB
    build_dir = BUILD_CHECKED if checks else BUILD
    extra = CHECK_FLAGS if checks else []
    if not force and up_to_date(lib):
        return lib
    os.makedirs(build_dir, exist_ok=True)
    srcs = sources(checks)
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 1))
    if verbose:
        print("[pof build] nvcc %d units, %d jobs%s" % (len(srcs), jobs, " (bounds checks)" if checks else ""),
              file=sys.stderr)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda src: _compile(src, build_dir, extra), srcs))
    tmp = lib + ".tmp"
    # relocatable device code is device-linked here
    cmd = [nvcc(), "-shared"] + ARCH + (["-rdc=true"] if checks else []) + ["-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, checks="--checks" in sys.argv))
