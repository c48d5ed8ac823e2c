"""Build libcuflye_gb300.so (sm_103a) and its logf exception table, in tree.

Outputs go to ``cuflye_gb300/_build/``:
  * ``libcuflye_gb300.so`` — the CUDA library behind ``include/cuflye.h``;
  * ``logf_exceptions.bin`` — generated on this machine by ``logf_table``
    from this machine's C library logf (see ``csrc/logf_table.cu``).

Translation units compile in parallel with one ``-gencode`` for sm_103a.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libcuflye_gb300.so"
TABLE = OUT / "logf_exceptions.bin"

SOURCES = ["api.cu", "sort.cu", "radix.cu", "util.cu", "index.cu", "hits.cu", "chain.cu", "r2g.cu",
           "abi.cu", "noalloc.cu", "fastsort.cu", "match_emit.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-ffp-contract=off", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cuflye_gb300")
    return cand


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [
        HERE.parent / "include" / "cuflye.h"]
    procs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nv, *ARCH, *FLAGS, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                                stderr=subprocess.STDOUT, text=True)))
    gen = OUT / "logf_table"
    gsrc = CSRC / "logf_table.cu"
    if force or _stale(gen, [gsrc] + headers):
        cmd = [nv, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-Xcompiler",
               "-pthread", str(gsrc), "-o", str(gen)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(f"$ {' '.join(c)}\n{o}" for c, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or _stale(LIB, objs):
        cmd = [nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        subprocess.run(cmd, check=True)
    if force or _stale(TABLE, [gen]):
        subprocess.run([str(gen), str(TABLE)], check=True, stdout=subprocess.DEVNULL)
    build_abi_caller(force)
    return LIB


CALLER_SRC = HERE.parent / "tests" / "c" / "abi_caller.cpp"
CALLER = OUT / "abi_caller"


def build_abi_caller(force: bool = False) -> Path | None:
    """The compiled C++ caller of the C ABI (tests/c/abi_caller.cpp, through
    the Flye-side adapter cuflye_gb300/flye/cuflye_flye.hpp), linked against
    the library with an rpath to this directory.  None when the source is
    not in the tree."""
    if not CALLER_SRC.exists():
        return None
    adapter = HERE / "flye" / "cuflye_flye.hpp"
    header = HERE.parent / "include" / "cuflye.h"
    if force or _stale(CALLER, [CALLER_SRC, adapter, header, LIB]):
        cxx = shutil.which("g++") or "g++"
        subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", str(HERE.parent / "include"),
                        "-I", str(HERE / "flye"), str(CALLER_SRC), "-o", str(CALLER),
                        "-L", str(OUT), "-lcuflye_gb300", "-Wl,-rpath,$ORIGIN"], check=True)
    return CALLER


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="--force" in sys.argv)
    print(LIB)
