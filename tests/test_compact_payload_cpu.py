"""CPU: the compact binary payload of candidate chains
(docs/abi/read-alignment-compact-binary-v0.md), written by the library's host
code (cuflye_compact_binary; no device).  Chains from the CPU oracle's
chainReadAlignments on synthetic replay fixtures become chain records; the
payload must pass the reference's own validator
(tools/validate_read_alignment_binary_payload.py, where the reference
checkout is present) and read back field for field."""

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import REPO
from test_oracle_vs_reference_cpu import _edge_alignments


def _fixtures(seed=41, count=12):
    rng = np.random.default_rng(seed)
    out = []
    for f in range(count):
        rows = _edge_alignments(rng, int(rng.integers(4, 30)))
        read_len = max(r[1] for r in rows) + int(rng.integers(0, 500))
        out.append((1000 + f, read_len, rows))
    return out


def _oracle_records(oracle_mod, fixtures):
    from cuflye_gb300 import abi, synth
    p = synth.R2G_PARAMS
    r2g = oracle_mod.default_r2g(max_jump=p["max_jump"], max_read_overlap=p["max_read_overlap"],
                                 min_overlap=p["min_overlap"],
                                 max_separation=p["max_separation"])
    recs, inputs = [], []
    for qid, read_len, rows in fixtures:
        arr = np.array([[r[0], r[1], r[2], r[3], r[4], r[7]] for r in rows])
        chains = oracle_mod.chain_read_alignments(arr, [r[5] for r in rows],
                                                  [r[6] for r in rows], r2g)
        inputs.append(len(rows))
        for c, chain in enumerate(chains):
            for s, i in enumerate(chain):
                r = rows[i]
                recs.append((qid, c, s, i, 0, 70_000 + i, qid, r[9], r[9] + 5000, r[0], r[1],
                             read_len, r[5], r[6], r[2], r[3], r[4], r[7], r[8]))
    return np.array(recs, dtype=abi.CHAIN_RECORD_DTYPE), np.array(inputs, dtype=np.uint64)


def test_compact_payload_layout_and_roundtrip(built_lib, oracle_mod):
    from cuflye_gb300 import abi
    from cuflye_gb300.backend import compact_binary
    fx = _fixtures()
    recs, inputs = _oracle_records(oracle_mod, fx)
    assert len(recs) > 20
    data = compact_binary(recs, inputs)
    assert len(data) == 64 + 92 * len(recs)
    head, back = abi.read_compact_binary(data)
    assert head["magic"] == b"CUFRALB0" and head["header_bytes"] == 64
    assert head["record_bytes"] == 92 and head["version"] == (0, 0)
    assert head["fixtures"] == len(fx) and head["records"] == len(recs)
    assert head["total_inputs"] == int(inputs.sum())
    assert (head["min_inputs"], head["max_inputs"]) == (int(inputs.min()), int(inputs.max()))
    assert head["output_mode"] == 1 and head["reserved"] == 0
    for name in abi.COMPACT_RECORD_DTYPE.names:
        assert np.array_equal(back[name], recs[name]), name


def test_compact_payload_passes_the_reference_validator(built_lib, oracle_mod, tmp_path):
    ref = Path(os.environ.get("CUFLYE_REFERENCE") or "/root/reference")
    tool = ref / "tools" / "validate_read_alignment_binary_payload.py"
    if not tool.exists():
        pytest.skip("the reference checkout is not here")
    from cuflye_gb300.backend import compact_binary
    fx = _fixtures(seed=43, count=9)
    recs, inputs = _oracle_records(oracle_mod, fx)
    path = tmp_path / "chains.cufralb0"
    path.write_bytes(compact_binary(recs, inputs))
    out = subprocess.run([sys.executable, str(tool), str(path), "--expected-fixture-count",
                          str(len(fx)), "--expected-output-records", str(len(recs)),
                          "--expected-total-input-records", str(int(inputs.sum()))],
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr + out.stdout
    assert '"status": "ok"' in out.stdout
    # and it refuses a truncated copy
    bad = tmp_path / "short.cufralb0"
    bad.write_bytes(path.read_bytes()[:-5])
    out = subprocess.run([sys.executable, str(tool), str(bad)], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode != 0


def test_compact_payload_capacity_and_arguments(built_lib):
    import ctypes
    from cuflye_gb300 import abi
    from cuflye_gb300.backend import load_library
    L = load_library()
    recs = np.zeros(3, dtype=abi.CHAIN_RECORD_DTYPE)
    inp = np.array([5, 7], dtype=np.uint64)
    n = ctypes.c_size_t()
    buf = np.zeros(64, dtype=np.uint8)
    st = L.cuflye_compact_binary(recs.ctypes.data, 3, 2,
                                 inp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                 buf.ctypes.data, len(buf), ctypes.byref(n))
    assert st == 5 and n.value == 64 + 3 * 92  # CUFLYE_ERR_CAPACITY, size written
    st = L.cuflye_compact_binary(None, 3, 2, inp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                 buf.ctypes.data, len(buf), ctypes.byref(n))
    assert st == 1  # CUFLYE_ERR_INVALID
