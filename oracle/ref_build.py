"""Test infrastructure: builds the reference's own CPU backends, the checker
beside the oracle.

The reference's CUDA prototypes each carry a host CPU path selected with
``--backend cpu``, one source file each (plus the reference's RAII header):

* ``cuda/cuflye_cuda_overlap_chain_replay.cu``: Flye's chaining DP,
  score-ordered backtrack, overlapTest, k-mer divergence and primary
  selection on overlap-replay fixtures (``computeCpuGroupOverlap`` and
  ``finalizeOverlaps``);
* ``cuda/cuflye_cuda_read_alignment_chain_replay.cu``: ReadAligner's
  ``chainReadAlignments`` on read-alignment replay fixtures.

They are compiled where they lie, with nvcc (the files hold device code that
the CPU path never launches), into ``oracle/_ref/``, which is not committed.
Only the CPU tests run them, to check the oracle; the library never does.
A machine without the reference checkout skips the build and those tests.

The checkout is taken from ``--reference``, else from the
``CUFLYE_REFERENCE`` environment variable, else from the one place this
build environment mounts it (``DEFAULT_REFERENCE``).

Usage: python oracle/ref_build.py [--reference DIR]
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
DEFAULT_REFERENCE = Path(os.environ.get("CUFLYE_REFERENCE") or "/root/reference")

# output name -> source file under the reference's cuda/ directory
PROGRAMS = {
    "overlap_chain_replay": "cuflye_cuda_overlap_chain_replay.cu",
    "read_alignment_chain_replay": "cuflye_cuda_read_alignment_chain_replay.cu",
}


def build(reference: Path = DEFAULT_REFERENCE) -> dict[str, Path]:
    """Compiles every program whose source is present and newer than its
    binary; returns the binaries built or found (empty without the
    reference or nvcc)."""
    src_dir = reference / "cuda"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not src_dir.is_dir() or not Path(nvcc).exists():
        return {}
    OUT.mkdir(exist_ok=True)
    built = {}
    for name, src in PROGRAMS.items():
        source = src_dir / src
        if not source.exists():
            continue
        binary = OUT / name
        if not binary.exists() or binary.stat().st_mtime < source.stat().st_mtime:
            subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode",
                            "arch=compute_103a,code=sm_103a", "-I", str(src_dir), str(source),
                            "-o", str(binary)], check=True)
        built[name] = binary
    return built


def binary(name: str) -> Path | None:
    """The built program, or None when it is absent or cannot run here."""
    path = OUT / name
    if not path.exists():
        return None
    try:
        subprocess.run([str(path), "--help"], capture_output=True, timeout=30, check=True)
    except (OSError, subprocess.SubprocessError):
        return None
    return path


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, default=DEFAULT_REFERENCE)
    for n, p in build(ap.parse_args().reference).items():
        print(n, p)
