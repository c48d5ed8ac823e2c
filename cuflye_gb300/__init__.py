"""cuflye_gb300 — GB300 (sm_103a) implementation of Flye's overlap hot path.

Candidate generation against a device-resident k-mer index, the chaining DP
with backtrack, read-to-graph chains and prefix-scan output compaction,
behind the C ABI in ``include/cuflye.h`` (``_build/libcuflye_gb300.so``).
``backend`` mirrors the reference's candidate-backend seam over that ABI;
``abi`` holds the record layouts and text formats; ``synth`` generates the
seeded synthetic workloads.
"""

from . import abi  # noqa: F401

__all__ = ["abi", "backend", "synth", "build"]
