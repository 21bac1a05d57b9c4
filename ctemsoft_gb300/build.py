"""Build recipe for libebsdgpu.so, the ctemebsd executable and (for tests)
the CPU oracle.

Compiles each CUDA translation unit for sm_103a only, in parallel, and links
in-tree into ``ctemsoft_gb300/lib``.  Sources are recompiled only when they
(or a header) are newer than their object file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = LIB / "obj"
ORACLE = ROOT / "oracle"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction of a*b+c, so float expressions round exactly
# like the reference's (explicit fmaf() is still fused); IEEE div/sqrt are
# nvcc's defaults without --use_fast_math.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"] + ARCH
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             f"-I{CUDA_HOME / 'include'}"]

CU_SOURCES = ["ebsd_setup.cu", "ebsd_forward.cu", "ebsd_vjp.cu", "ebsd_so3.cu", "ebsd_mc.cu",
              "ebsd_membw.cu", "ebsd_capi.cu"]
CXX_SOURCES = ["ebsd_host.cpp", "ebsd_program.cpp"]
HEADERS = ["ebsd_internal.h", "ebsd_device.cuh", "ebsd_host.h", "ebsd_noise.cuh"]

LIBNAME = "libebsdgpu.so"
EXES = [("ctemebsd", "ctemebsd_main.cpp"), ("ctemmc", "ctemmc_main.cpp")]


def _newer(src: Path, deps: list[Path], out: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps] if p.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _compile(src: Path) -> Path:
    out = OBJ / (src.name + ".o")
    deps = [CSRC / h for h in HEADERS] + [ROOT / "include" / "ebsd_gpu.h"]
    if _newer(src, deps, out):
        if src.suffix == ".cu":
            _run([NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(out)])
        else:
            _run([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(out)])
    return out


def build_library(verbose: bool = False) -> Path:
    """Compile and link ``lib/libebsdgpu.so``, ``lib/ctemebsd`` and ``lib/ctemmc``."""
    if not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}")
    OBJ.mkdir(parents=True, exist_ok=True)
    srcs = [CSRC / s for s in CU_SOURCES + CXX_SOURCES]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    lib = LIB / LIBNAME
    if not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        _run([NVCC, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lpthread"])
    for name, main in EXES:
        exe = LIB / name
        main_src = CSRC / main
        if _newer(main_src, [lib, ROOT / "include" / "ebsd_gpu.h"], exe):
            _run([CXX, "-O2", "-std=c++17", str(main_src), "-o", str(exe), f"-L{LIB}",
                  "-lebsdgpu", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}")
    return lib


def build_oracle() -> Path:
    """Compile the CPU oracle (test infrastructure) ``oracle/liboracle.so``."""
    out = ORACLE / "liboracle.so"
    srcs = [ORACLE / "ebsd_oracle.c", ORACLE / "ebsd_oracle_grad.c", ORACLE / "ebsd_oracle_so3.c",
            ORACLE / "ebsd_oracle_mc.c"]
    if _newer(srcs[0], [*srcs[1:], ORACLE / "ebsd_oracle.h"], out):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-std=c11",
              "-shared", "-o", str(out), *map(str, srcs), "-lm"])
    return out


def ptxas_report() -> str:
    """Register/spill report of the forward kernels (-Xptxas -v)."""
    r = subprocess.run([NVCC, *NVCC_FLAGS, "-Xptxas", "-v", "-c", str(CSRC / "ebsd_forward.cu"),
                        "-o", os.devnull], capture_output=True, text=True)
    return r.stderr


def clean() -> None:
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    build_library(verbose=True)
    build_oracle()
    if "--ptxas" in sys.argv:
        print(ptxas_report())
