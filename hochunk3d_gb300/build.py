"""Build recipe of the GB300 library (sm_103a) and of the CPU oracle.

``build_host_library()`` compiles the host-only model set-up (the .par
reader, gridset, the dust tables; no CUDA) into
``hochunk3d_gb300/libhc3d_host.so`` with g++; ``build_library()`` compiles
the CUDA kernels, the C-ABI, the server and the host driver into
``hochunk3d_gb300/libhc3d.so`` with nvcc, linked against the host library;
``build_oracle()`` compiles the CPU restatement used by the tests into
``oracle/_build/libhc3d_oracle.so``.  A process that only sets models up
(the CPU legs of the benchmark) loads the host library alone.
Translation units are compiled in parallel; a unit is rebuilt when its source
or any header is newer than its object file.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhc3d.so"
HOST_LIB = PKG / "libhc3d_host.so"
# host units and their extra flags; the fractal factor rounds every product
# and sum on its own, as the device build of it does
HOST_UNITS = [("hc3d_model.cpp", []), ("hc3d_fractal.cpp", ["-ffp-contract=off"])]
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libhc3d_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]

# (source, extra flags); the all-FP64 kernel and the emissivity tables keep
# multiplies and adds separately rounded so that they reproduce the CPU
# restatement and the host build.  The mixed
# kernel keeps IEEE FP32 division, square root and transcendentals: built
# with --use_fast_math it failed the mixed-vs-FP64 temperature and packet
# bookkeeping tests.
UNITS = [
    ("hc3d_kernel_mixed.cu", []),
    ("hc3d_kernel_fp64.cu", ["--fmad=false"]),
    ("hc3d_capi.cu", []),
    ("hc3d_noalloc.cu", []),
    ("hc3d_gridbuild.cu", []),
    ("hc3d_tablebuild.cu", ["--fmad=false"]),
    ("hc3d_driver.cpp", []),
    ("hc3d_serve.cpp", []),
]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or Path(c).exists()):
            return c
    return "nvcc"


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_headers(), Path(__file__)])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_host_library(verbose: bool = False, force: bool = False) -> Path:
    """Compile the host-only model set-up into libhc3d_host.so (g++, no CUDA)."""
    BUILD.mkdir(exist_ok=True)
    srcs = [CSRC / u for u, _ in HOST_UNITS]
    if force or not HOST_LIB.exists() or any(_stale(HOST_LIB, src) for src in srcs):
        objs = []
        for u, extra in HOST_UNITS:
            obj = BUILD / (Path(u).stem + ".host.o")
            _run(["g++", "-O2", "-std=c++17", *extra, "-fPIC", "-c", str(CSRC / u), "-o", str(obj)])
            objs.append(obj)
        tmp = HOST_LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-Wl,-soname,libhc3d_host.so", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, HOST_LIB)
    if verbose:
        print(f"built {HOST_LIB}")
    return HOST_LIB


def build_library(verbose: bool = False, force: bool = False) -> Path:
    """Compile every translation unit for sm_103a and link libhc3d.so
    against libhc3d_host.so (found beside it at run time)."""
    build_host_library(verbose=verbose, force=force)
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src_name, extra in UNITS:
        src = CSRC / src_name
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            lang = ["-x", "cu"] if src.suffix == ".cu" else []
            cmd = [nvcc, *ARCH, *NVCC_COMMON, *extra, *lang, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for _ in ex.map(_run, jobs):
                pass
    if (force or jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs)
            or HOST_LIB.stat().st_mtime > LIB.stat().st_mtime):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-L" + str(PKG), "-lhc3d_host",
              "-Xlinker", "-rpath=$ORIGIN", "-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    """Compile the CPU restatement (test infrastructure) with gcc."""
    src = ORACLE_DIR / "hc3d_oracle.c"
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    deps = [src, ORACLE_DIR / "philox.h", ROOT / "include" / "hc3d.h"]
    if force or not ORACLE_LIB.exists() or any(p.stat().st_mtime > ORACLE_LIB.stat().st_mtime for p in deps):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11", "-o", str(tmp), str(src),
              "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    build_library(verbose=True, force=force)
    build_oracle(verbose=True, force=force)
