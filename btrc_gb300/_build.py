"""Build the native library in-tree: btrc_gb300/_build/libbtrc_gb300.so.

Host C++ is compiled with g++ and the CUDA sources with nvcc for sm_103a only, each
translation unit in parallel, then linked by nvcc. FP contraction is disabled for host
code so that host-side transforms round identically on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libbtrc_gb300.so"
INCLUDE = PKG.parent / "include"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall", "-Wno-unused-function"]
NVCCFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                    "-Xptxas", "-warn-spills"]
# The wavefront stage kernels use approximate FP32 division and square root (max 2 ulp),
# as the reference's own kernels do (they are built with fast math); denormals and the
# transcendental functions stay accurate. Without the IEEE slow paths at every division
# the shade kernel's code shrinks by a third and it runs ~30 % faster. The traversal and
# the samplers, which match the oracle bit for bit, use explicitly rounded operations.
SHADING_SOURCES = {"integrator.cu"}
SHADING_FLAGS = ["-prec-div=false", "-prec-sqrt=false"]


def _run(cmd: list[str]) -> str:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _sources() -> tuple[list[Path], list[Path]]:
    cpp = sorted(CSRC.glob("*.cpp"))
    cu = sorted(CSRC.glob("*.cu"))
    return cpp, cu


def _needs_rebuild() -> bool:
    if not LIB.exists():
        return True
    lib_time = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [INCLUDE / "btrc.h", Path(__file__)]
    return any(p.stat().st_mtime > lib_time for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    if not force and not _needs_rebuild():
        return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    OUT.mkdir(parents=True, exist_ok=True)
    cpp, cu = _sources()
    inc = [f"-I{CSRC}", f"-I{INCLUDE}", f"-I{os.path.join(CUDA_HOME, 'include')}"]
    jobs = []
    objs = []
    for src in cpp:
        obj = OUT / (src.stem + ".cpp.o")
        objs.append(obj)
        jobs.append(["g++"] + CXXFLAGS + inc + ["-c", str(src), "-o", str(obj)])
    for src in cu:
        obj = OUT / (src.stem + ".cu.o")
        objs.append(obj)
        extra = SHADING_FLAGS if src.name in SHADING_SOURCES else []
        jobs.append([NVCC] + NVCCFLAGS + extra + inc + ["-c", str(src), "-o", str(obj)])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o, file=sys.stderr)
    tmp = OUT / (LIB.name + ".tmp")
    _run([NVCC] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart", "-lpthread"])
    shutil.move(str(tmp), str(LIB))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
