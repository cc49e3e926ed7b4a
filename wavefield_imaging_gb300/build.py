"""Build libawe.so (the engine's C-ABI shared library) for sm_103a, in-tree.

    python -m wavefield_imaging_gb300.build

Translation units are compiled in parallel with nvcc (device + host code)
and g++ (pure host code); objects and the library go to
wavefield_imaging_gb300/_build/.  Host code is built with -ffp-contract=off
so set-up tables are bit-identical on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libawe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    deps += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return os.path.getmtime(obj) < max(os.path.getmtime(x) for x in deps)


def _compile(src: str) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not _stale(obj, src):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I" + _cuda_include(), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    build_programs()
    if verbose:
        print("built", LIB)
    return LIB


PROGS = os.path.join(PKG, "programs")
BIN = os.path.join(OUT, "bin")
PROGRAM_NAMES = ["sfAWEFDcart2Dgpu", "sfAWEFDcart3Dgpu", "sfAWEFDspher2Dgpu", "sfAWEFDspher3Dgpu",
                 "sfAWEFDcart2Dcpu", "sfAWEFDcart3Dcpu", "sfDYNAWEFDcart2Dgpu"]


CLOUD_PROGRAM_NAMES = ["sfbycloudwin3d", "sfbycloudmerge3d"]


def build_programs() -> str:
    """Link the drop-in RSF programs (one binary per family, one name per
    program) against libawe.so."""
    os.makedirs(BIN, exist_ok=True)
    for exe_name, main_src, names in (("awe_prog", "awe_prog.c", PROGRAM_NAMES),
                                      ("cloud_prog", "cloud_prog.c", CLOUD_PROGRAM_NAMES)):
        exe = os.path.join(BIN, exe_name)
        srcs = [os.path.join(PROGS, main_src), os.path.join(PROGS, "rsfio.c")]
        deps = srcs + [os.path.join(PROGS, "rsfio.h"), os.path.join(ROOT, "include", "awe.h"), LIB]
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(x) for x in deps):
            cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-Wall", "-ffp-contract=off",
                   "-I" + os.path.join(ROOT, "include"), "-I" + PROGS, *srcs, "-o", exe, "-L" + OUT, "-lawe",
                   "-lm", "-Wl,-rpath,$ORIGIN/.."]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("program link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        for name in names:
            link = os.path.join(BIN, name)
            if not os.path.islink(link):
                if os.path.exists(link):
                    os.remove(link)
                os.symlink(exe_name, link)
    return BIN


if __name__ == "__main__":
    build(verbose=True)
