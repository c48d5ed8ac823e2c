import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))
GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def built_lib():
    from cuflye_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def gpu(built_lib):
    from cuflye_gb300.backend import CudaBackend
    b = CudaBackend(device=0, memory_budget_bytes=0)
    yield b
    b.close()


def read_tsv_reads(path: Path):
    from cuflye_gb300 import synth
    ids, seqs = [], []
    for line in path.read_text().splitlines():
        if not line:
            continue
        a, b = line.split("\t")
        ids.append(int(a))
        seqs.append(b)
    return synth.ReadSet.from_strings(ids, seqs)


@pytest.fixture(scope="session")
def golden_cases():
    import json
    out = {}
    for d in sorted((GOLDEN / "synthetic").iterdir()):
        meta = json.loads((d / "meta.json").read_text())
        out[d.name] = (read_tsv_reads(d / "reads.tsv"), meta, d)
    return out
