"""Build recipe of the oracle (TEST INFRASTRUCTURE ONLY).

    python -m oracle.build

* oracle/liboracle.so  <- oracle/mc_oracle.cpp (the CPU restatement), built
  with -ffp-contract=off so the FP32 packet replay rounds exactly like the
  device code;
* oracle/_ref/libref_{ck,particle}.so  <- the reference's own
  code/read_tables.cpp and code/spline.cpp compiled from where they lie under
  the reference tree with oracle/ref_shim/param.h standing in for the
  reference's compile-time code/param.h (-I- keeps the reference's own param.h
  out of the search path);
* oracle/_ref/libref_ckgen.so  <- the reference's distr/correlatedK.cpp (its
  k-distribution routine correlatedKT) around oracle/ref_ckgen.cpp.
  The reference builds are only made when the reference tree is present
  (at $DNSMC_REFERENCE, default /root/reference).
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: DNSMC_REFERENCE, else the location in this build container
REF_ROOT = os.environ.get("DNSMC_REFERENCE", "/root/reference")
REF_CODE = os.path.join(REF_ROOT, "code")
REF_DIR = os.path.join(HERE, "_ref")


def lib_path() -> str:
    return os.path.join(HERE, "liboracle.so")


def ref_lib_path(kind: str) -> str:
    return os.path.join(REF_DIR, f"libref_{kind}.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _oracle_cmd() -> list[str]:
    return ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
            os.path.join(HERE, "mc_oracle.cpp"), "-o", lib_path()]


def _ref_cmd(kind: str) -> list[str]:
    grey = {"ck": 0, "particle": 2}[kind]
    return ["g++", "-O2", "-fPIC", "-shared", "-w", f"-DREF_GREY={grey}",
            "-I", os.path.join(HERE, "ref_shim"), "-I-", "-I", REF_CODE,
            os.path.join(HERE, "ref_wrap.cpp"),
            os.path.join(REF_CODE, "read_tables.cpp"), os.path.join(REF_CODE, "spline.cpp"),
            "-o", ref_lib_path(kind)]


def _ref_ckgen_cmd() -> list[str]:
    # the reference's k-distribution generator (distr/correlatedK.cpp) with
    # its compile-time sizes (distr/classes.h), around a C entry point
    distr = os.path.join(REF_ROOT, "distr")
    return ["g++", "-O2", "-fPIC", "-shared", "-w", "-include", "cstdio", "-include", "cstdlib", "-I", distr,
            os.path.join(HERE, "ref_ckgen.cpp"), os.path.join(distr, "correlatedK.cpp"),
            "-o", ref_lib_path("ckgen")]


def build(with_ref: bool | None = None) -> None:
    jobs = [_oracle_cmd()]
    if with_ref is None:
        with_ref = os.path.isdir(REF_CODE)
    if with_ref:
        os.makedirs(REF_DIR, exist_ok=True)
        jobs += [_ref_cmd("ck"), _ref_cmd("particle"), _ref_ckgen_cmd()]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))


if __name__ == "__main__":
    build()
    print("built", lib_path())
