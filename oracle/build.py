"""Build recipe for the oracle (test infrastructure only).

  oracle/_build/liboracle.so : the CPU restatement (oracle/oracle.cpp)
  oracle/_ref/libref_bvh.so  : the reference tree's vendored lib/bvh behind a small C
                               driver (oracle/ref_bvh.cpp), compiled from the headers where
                               they lie; only when the reference tree is present.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use these libraries.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_bvh.so"
# The reference tree: $BTRC_REFERENCE_ROOT, else a checkout named "reference" beside this
# repository. Absent (as on a machine without the reference), lib/bvh is simply not built.
REFERENCE_ROOT = Path(os.environ["BTRC_REFERENCE_ROOT"]) if os.environ.get("BTRC_REFERENCE_ROOT") \
    else HERE.parent.parent / "reference"
REFERENCE_BVH_INCLUDE = REFERENCE_ROOT / "lib" / "bvh" / "include"

FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off"]


def _stale(lib: Path, srcs: list[Path]) -> bool:
    return not lib.exists() or any(s.stat().st_mtime > lib.stat().st_mtime for s in srcs)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "oracle.cpp"
    if force or _stale(ORACLE_LIB, [src, Path(__file__)]):
        ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = ORACLE_LIB.with_suffix(".tmp.so")
        subprocess.run(["g++"] + FLAGS + [str(src), "-o", str(tmp)], check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_ref(force: bool = False) -> Path | None:
    if not REFERENCE_BVH_INCLUDE.is_dir():
        return REF_LIB if REF_LIB.exists() else None
    src = HERE / "ref_bvh.cpp"
    if force or _stale(REF_LIB, [src, Path(__file__)]):
        REF_LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = REF_LIB.with_suffix(".tmp.so")
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
                        f"-I{REFERENCE_BVH_INCLUDE}", str(src), "-o", str(tmp)], check=True)
        os.replace(tmp, REF_LIB)
    return REF_LIB


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_ref(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(ORACLE_LIB, REF_LIB if REF_LIB.exists() else "(no reference tree)")
