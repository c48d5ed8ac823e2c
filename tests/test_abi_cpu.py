"""CPU: the C-ABI library builds, loads and exports every symbol that
include/cuflye.h declares; the backend seam parses its environment like the
reference; host-side record formatting follows the ABI text rules.  No call
here touches a GPU."""

import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import REPO


def declared_symbols():
    text = (REPO / "include" / "cuflye.h").read_text()
    return sorted(set(re.findall(r"\b(cuflye_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (cuflye_[a-z_0-9]+)$", out, re.M))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    import ctypes
    lib = ctypes.CDLL(str(built_lib))
    for s in declared_symbols():
        assert hasattr(lib, s)


def _backend_in_subprocess(value):
    env = dict(os.environ)
    if value is None:
        env.pop("CUFLYE_CANDIDATE_BACKEND", None)
    else:
        env["CUFLYE_CANDIDATE_BACKEND"] = value
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from cuflye_gb300 import backend\n"
            "try:\n print('OK', backend.candidate_backend())\n"
            "except RuntimeError as e:\n print('ERR', e)\n") % str(REPO)
    return subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                          text=True, check=True).stdout.strip()


@pytest.mark.parametrize("value,expect", [(None, "OK cpu"), ("", "OK cpu"), ("cpu", "OK cpu"),
                                          ("cuda", "OK cuda"),
                                          ("opencl", "ERR Unsupported CUFLYE_CANDIDATE_BACKEND: opencl")])
def test_backend_selection_matches_reference_seam(built_lib, value, expect):
    """patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:29-43."""
    assert _backend_in_subprocess(value) == expect


def test_record_layouts_match_header():
    from cuflye_gb300 import abi
    assert abi.CANDIDATE_DTYPE.itemsize == 32
    assert abi.OVERLAP_DTYPE.itemsize == 48
    assert abi.READ_ALIGNMENT_DTYPE.itemsize == 72


_C_TYPES = {"int64_t": "<i8", "uint64_t": "<u8", "int32_t": "<i4", "float": "<f4"}


def header_struct(name: str) -> list[tuple[str, str]]:
    """(field, numpy type code) of `typedef struct name {...} name;` in cuflye.h."""
    text = (REPO / "include" / "cuflye.h").read_text()
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), _C_TYPES[ctype]) for n in names.split(",")]
    return fields


def _ctypes_fields(cls) -> list[tuple[str, str]]:
    import ctypes
    code = {ctypes.c_int32: "<i4", ctypes.c_float: "<f4", ctypes.c_int64: "<i8",
            ctypes.c_uint64: "<u8"}
    return [(n, code[t]) for n, t in cls._fields_]


def test_host_mirrors_match_header_structs():
    """Every struct the C ABI passes by pointer has the same fields, order and
    types in the Python mirror (ctypes parameters, numpy records)."""
    import ctypes
    from cuflye_gb300 import abi
    from cuflye_gb300.backend import LaunchShape, OverlapParams, R2GParams
    for cls, name in ((OverlapParams, "cuflye_overlap_params"),
                      (R2GParams, "cuflye_r2g_params"),
                      (LaunchShape, "cuflye_launch_shape")):
        fields = header_struct(name)
        assert _ctypes_fields(cls) == fields, name
        assert ctypes.sizeof(cls) == 4 * len(fields), name
    for dt, name in ((abi.CANDIDATE_DTYPE, "cuflye_candidate"),
                     (abi.FILTERED_DTYPE, "cuflye_filtered_pos"),
                     (abi.OVERLAP_DTYPE, "cuflye_overlap_range"),
                     (abi.READ_ALIGNMENT_DTYPE, "cuflye_read_alignment"),
                     (abi.CHAIN_RECORD_DTYPE, "cuflye_chain_record"),
                     (abi.EDGE_OVERLAP_DTYPE, "cuflye_edge_overlap")):
        assert [(n, dt.fields[n][0].str) for n in dt.names] == header_struct(name), name


def test_float_text_follows_setprecision9():
    """C++ setprecision(9) of a float: 0.01f prints 0.00999999978
    (the reference's own TSV, tests/fixtures/read-alignment-replay-fixture-v0)."""
    from cuflye_gb300.abi import format_float
    assert format_float(0.01) == "0.00999999978"
    assert format_float(0.0) == "0"
    assert format_float(0.02) == "0.0199999996"


def test_canonical_sha_is_order_free():
    from cuflye_gb300.abi import canonical_sha256
    a = ["1\t2\t3\n", "-1\t5\t6\n", "1\t10\t3\n"]
    assert canonical_sha256(a) == canonical_sha256(list(reversed(a)))


def test_logf_table_matches_c_library(built_lib, oracle_mod):
    """The exception table makes logf_wide + table == this machine's logf on a
    sample of floats in [1, 2^24) (the device applies the same table)."""
    import struct
    from pathlib import Path
    tbl = Path(built_lib).parent / "logf_exceptions.bin"
    data = tbl.read_bytes()
    n = struct.unpack("<I", data[:4])[0]
    pairs = np.frombuffer(data[4:], dtype=np.uint32).reshape(n, 2)
    assert np.all(np.diff(pairs[:, 0].astype(np.int64)) > 0)
    rng = np.random.default_rng(0)
    xs = pairs[rng.integers(0, n, size=200), 0].view(np.float32)
    for x, y in zip(xs, pairs[np.searchsorted(pairs[:, 0], xs.view(np.uint32)), 1].view(np.float32)):
        assert oracle_mod.logf(float(x)) == float(y)


def _is_subsequence(small: bytes, big: bytes) -> bool:
    it = iter(big)
    return all(c in it for c in small)


def test_sparse_errors_follow_the_error_model():
    """mutate_sparse (used for the full-size scale configuration) gives each
    error kind at its rate, within five standard deviations."""
    from cuflye_gb300 import synth
    rng = np.random.default_rng(11)
    n = 400_000
    seq = synth.random_genome(rng, n)
    sub = synth.mutate_sparse(np.random.default_rng(1), seq, 0.02)
    assert len(sub) == n
    rate = float(np.mean(sub != seq))
    assert abs(rate - 0.02) < 5 * np.sqrt(0.02 * 0.98 / n)
    dele = synth.mutate_sparse(np.random.default_rng(2), seq, 0.0, 0.0, 0.02)
    assert abs((n - len(dele)) - 0.02 * n) < 5 * np.sqrt(0.02 * n)
    short = seq[:20_000]
    assert _is_subsequence(synth.mutate_sparse(np.random.default_rng(3), short, 0.0, 0.0, 0.05)
                           .tobytes(), short.tobytes())
    ins = synth.mutate_sparse(np.random.default_rng(4), short, 0.0, 0.05, 0.0)
    assert abs((len(ins) - len(short)) - 0.05 * len(short)) < 5 * np.sqrt(0.05 * len(short))
    assert _is_subsequence(short.tobytes(), ins.tobytes())
    both = synth.mutate_sparse(np.random.default_rng(5), seq, 0.02, 0.02, 0.02)
    assert abs(len(both) - n) < 5 * np.sqrt(0.04 * n)
    again = synth.mutate_sparse(np.random.default_rng(5), seq, 0.02, 0.02, 0.02)
    assert np.array_equal(both, again)


def test_synthetic_generator_is_seeded():
    from cuflye_gb300 import synth
    a = synth.small_overlap_case(3, 20_000, 3.0, 3_000)
    b = synth.small_overlap_case(3, 20_000, 3.0, 3_000)
    assert np.array_equal(a.reads.bases, b.reads.bases)
    assert np.array_equal(a.reads.offsets, b.reads.offsets)


def _open_from_env_in_subprocess(device, budget):
    env = dict(os.environ)
    env["CUFLYE_CUDA_DEVICE"] = device
    env["CUFLYE_CUDA_MEMORY_BUDGET_BYTES"] = budget
    code = ("import sys, ctypes; sys.path.insert(0, %r)\n"
            "from cuflye_gb300 import backend\n"
            "L = backend.load_library()\n"
            "h = ctypes.c_void_p()\n"
            "st = L.cuflye_open_from_env(ctypes.byref(h))\n"
            "print(st, h.value is None)\n"
            "print(L.cuflye_last_error(None).decode())\n") % str(REPO)
    return subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                          text=True, check=True).stdout.splitlines()


@pytest.mark.parametrize("device,budget,reason", [
    ("gpu0", "unbounded", "CUFLYE_CUDA_DEVICE is not a device ordinal"),
    ("0", "40GB", "CUFLYE_CUDA_MEMORY_BUDGET_BYTES is neither"),
    ("-1", "1000", "CUFLYE_CUDA_DEVICE is not a device ordinal"),
])
def test_open_from_env_failure_keeps_the_stub_fields(built_lib, device, budget, reason):
    """An unparsable device or budget fails before any CUDA call, with a
    message kept for the thread (cuflye_last_error(NULL)) that starts with
    the reference stub's fields
    (patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46)."""
    status, msg = _open_from_env_in_subprocess(device, budget)
    assert status == "1 True"  # CUFLYE_ERR_INVALID, no context
    assert msg.startswith("cuFlye CUDA candidate backend selected; adapter=cuflye_gb300; "
                          f"CUFLYE_CUDA_DEVICE={device}; "
                          f"CUFLYE_CUDA_MEMORY_BUDGET_BYTES={budget}; ")
    assert reason in msg


def test_cpp_caller_fails_fast_with_the_stub_fields(built_lib):
    """The compiled C++ caller (tests/c/abi_caller.cpp) opens the device
    through the Flye-side adapter; an unparsable CUFLYE_CUDA_DEVICE throws
    before any CUDA call, with the reference stub's fields."""
    from cuflye_gb300 import build
    path = build.build_abi_caller()
    assert path is not None
    env = dict(os.environ, CUFLYE_CUDA_DEVICE="cuda:zero")
    r = subprocess.run([str(path), "open"], env=env, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert r.stdout.startswith("ERROR\tcuFlye CUDA candidate backend selected; "
                               "adapter=cuflye_gb300; CUFLYE_CUDA_DEVICE=cuda:zero; ")
