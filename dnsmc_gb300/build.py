"""Build recipe for libdnsmc.so (the C-ABI library) -- in-tree, sm_103a only.

    python -m dnsmc_gb300.build        # or dnsmc_gb300.build.build()

Compiles the CUDA translation units with nvcc for sm_103a (the marches with
-fmad=false: it is written with explicit fmaf so the host replay can
reproduce it bit for bit; the allocation-free solve; the control-variate
network) and the host runtime with the same nvcc driver, in parallel, then
links one shared library with the static CUDA runtime.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libdnsmc.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = [os.environ.get("NVCC", ""), shutil.which("nvcc") or "", "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or put CUDA on PATH)")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo"] + inc
    # resident 256-thread blocks per SM the march kernels must fit (register cap)
    minb = int(os.environ.get("DNSMC_MINB", "0"))
    regs = [f"-DDNSMC_MINB={minb}"] if minb else []
    jobs = [
        [nvcc, *ARCH, *common, *regs, "-fmad=false", "-c", os.path.join(CSRC, "mc_kernels.cu"),
         "-o", os.path.join(bdir, "mc_kernels.o")],
        # no FMA contraction in host arithmetic: identical results on x86 and Arm hosts
        [nvcc, *common, "-Xcompiler", "-ffp-contract=off", "-x", "c++", "-c", os.path.join(CSRC, "mc_host.cpp"),
         "-o", os.path.join(bdir, "mc_host.o")],
        [nvcc, *ARCH, *common, *regs, "-fmad=false", "-c", os.path.join(CSRC, "mc_march_gen.cu"),
         "-o", os.path.join(bdir, "mc_march_gen.o")],
        [nvcc, *ARCH, *common, *regs, "-fmad=false", "-c", os.path.join(CSRC, "mc_march_pair.cu"),
         "-o", os.path.join(bdir, "mc_march_pair.o")],
        [nvcc, *ARCH, *common, "-c", os.path.join(CSRC, "mc_noalloc.cu"),
         "-o", os.path.join(bdir, "mc_noalloc.o")],
        [nvcc, *ARCH, *common, "-c", os.path.join(CSRC, "mc_cvnet.cu"),
         "-o", os.path.join(bdir, "mc_cvnet.o")],
        [nvcc, *ARCH, *common, "-fmad=false", "-c", os.path.join(CSRC, "mc_ckgen.cu"),
         "-o", os.path.join(bdir, "mc_ckgen.o")],
    ]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    out = lib_path()
    tmp = out + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-fPIC",
          os.path.join(bdir, "mc_kernels.o"), os.path.join(bdir, "mc_host.o"),
          os.path.join(bdir, "mc_noalloc.o"), os.path.join(bdir, "mc_cvnet.o"), os.path.join(bdir, "mc_march_gen.o"),
          os.path.join(bdir, "mc_march_pair.o"), os.path.join(bdir, "mc_ckgen.o"),
          "-o", tmp])
    os.replace(tmp, out)
    if verbose:
        print("built", out)
    return out


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
