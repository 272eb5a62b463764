"""In-tree build of the native parts: the CUDA/C++ library behind include/mclicks.h,
the mclicks command-line tool, and (for tests) the CPU oracle.

Everything is compiled with nvcc / g++ directly, in parallel, one sm_103a target:

    python -m massiveclicks_gb300.build            # library + CLI + oracle
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"

LIB = BUILD / "libmclicks.so"
CLI = BUILD / "mclicks"
ORACLE_LIB = ORACLE_BUILD / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = sorted(CSRC.glob("*.cu"))
HOST_SOURCES = sorted((CSRC / "host").glob("*.cpp"))
CLI_SOURCES = sorted((CSRC / "cli").glob("*.cpp"))


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and Path(cand, "bin", "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)


def _digest(paths: list[Path], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        h.update(str(p).encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def _sources_for_lib() -> list[Path]:
    hdrs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((CSRC / "host").glob("*.h")) + sorted(INCLUDE.glob("*.h*"))
    return CU_SOURCES + HOST_SOURCES + hdrs


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    """Compiles libmclicks.so (CUDA kernels + host code) and the mclicks CLI."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    stamp = BUILD / "lib.stamp"
    key = _digest(_sources_for_lib() + CLI_SOURCES + list((CSRC / "cli").glob("*.h")), " ".join(ARCH))
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == key and (not CLI_SOURCES or CLI.exists()):
        return LIB
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CSRC / 'host'}"]
    nv_flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                "--expt-relaxed-constexpr", *ARCH, *inc]
    cxx_flags = ["-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                 f"-I{cuda / 'include'}", *inc]
    jobs_list = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src.stem + ".cu.o")
        jobs_list.append([nvcc, *nv_flags, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    for src in HOST_SOURCES:
        obj = BUILD / (src.stem + ".o")
        jobs_list.append(["g++", *cxx_flags, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs_list))
    tmp = BUILD / "libmclicks.so.tmp"
    _run([nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lpthread"])
    os.replace(tmp, LIB)
    if CLI_SOURCES:
        cli_objs = []
        cli_jobs = []
        for src in CLI_SOURCES:
            obj = BUILD / ("cli_" + src.stem + ".o")
            cli_jobs.append(["g++", *cxx_flags, f"-I{CSRC / 'cli'}", "-c", str(src), "-o", str(obj)])
            cli_objs.append(obj)
        with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
            list(ex.map(_run, cli_jobs))
        _run(["g++", "-o", str(CLI), *map(str, cli_objs), f"-L{BUILD}", "-lmclicks",
              f"-Wl,-rpath,{BUILD}", f"-L{cuda / 'lib64'}", "-lcudart", "-lpthread"])
    stamp.write_text(key)
    return LIB


def build_oracle(force: bool = False) -> Path:
    """Compiles the CPU oracle (test infrastructure) into oracle/_build/liboracle.so."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    srcs = [ORACLE / "oracle.hpp", ORACLE / "oracle_capi.cpp"]
    stamp = ORACLE_BUILD / "oracle.stamp"
    key = _digest(srcs, "oracle")
    if not force and ORACLE_LIB.exists() and stamp.exists() and stamp.read_text() == key:
        return ORACLE_LIB
    tmp = ORACLE_BUILD / "liboracle.so.tmp"
    _run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(tmp),
          str(ORACLE / "oracle_capi.cpp"), "-lpthread"])
    os.replace(tmp, ORACLE_LIB)
    stamp.write_text(key)
    return ORACLE_LIB


# Where build() looks for the reference's sources when MC_REFERENCE_DIR is not
# set: the read-only checkout of the development container.  Absent elsewhere
# (the GPU machine, a user's machine), in which case nothing is built.
REFERENCE_CHECKOUT = "/root/reference"


def build_reference(ref: str | None = None) -> Path | None:
    """Compiles the reference's CPU path into oracle/_ref/ when its sources are
    present: `ref`, else $MC_REFERENCE_DIR, else REFERENCE_CHECKOUT.  Returns
    the driver path, or None when no checkout is found."""
    ref = ref or os.environ.get("MC_REFERENCE_DIR") or REFERENCE_CHECKOUT
    if not Path(ref, "main.cpp").exists():
        return None
    _run(["make", "-s", "-C", str(ORACLE / "ref"), f"REF={ref}", f"-j{os.cpu_count() or 4}"])
    return ORACLE / "_ref" / "ref_driver"


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_library, force), ex.submit(build_oracle, force)]
        for f in futs:
            f.result()
    build_reference()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB, ORACLE_LIB)
