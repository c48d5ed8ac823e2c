"""GPU: the C ABI called from compiled C++ through the Flye-side adapter
(cuflye_gb300/flye/cuflye_flye.hpp; the program is tests/c/abi_caller.cpp,
built by build()).  Worker threads each take queries on a context of their
own that shares one index (cuflye_open_shared), with output buffers that
start small so every call goes through the CUFLYE_ERR_CAPACITY retry.  The
KmerMatches, filtered positions and overlap rows must equal the Python
binding's for the same queries, and those are checked against the oracle
elsewhere."""

import subprocess

import numpy as np
import pytest

from test_gpu_parity import overlap_tuples_gpu

pytestmark = pytest.mark.gpu


def _caller():
    from cuflye_gb300 import build
    path = build.build_abi_caller()
    assert path is not None and path.exists()
    return path


def _write_reads(path, reads):
    with open(path, "w") as fh:
        for i in range(reads.n):
            fh.write(f"{int(reads.ids[i])}\t{reads.seq(i).decode()}\n")


@pytest.mark.parametrize("threads", [1, 3])
def test_cpp_caller_candidates_match_the_binding(gpu, golden_cases, tmp_path, threads):
    reads, meta, _ = golden_cases["ovl-b"]
    src = tmp_path / "reads.tsv"
    out = tmp_path / "out.tsv"
    _write_reads(src, reads)
    r = subprocess.run([str(_caller()), "candidates", str(src), str(meta["k"]),
                        str(meta["min_freq"]), str(meta["max_freq"]), str(threads), str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = out.read_text().splitlines()
    got_c = [tuple(int(v) for v in l.split("\t")[1:]) for l in lines if l[0] == "C"]
    got_f = [tuple(int(v) for v in l.split("\t")[1:]) for l in lines if l[0] == "F"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    cand, filt = gpu.candidates(reads)
    want_c = list(zip(cand["query_id"].tolist(), cand["query_pos"].tolist(),
                      cand["kmer"].tolist(), cand["target_id"].tolist(),
                      cand["target_pos"].tolist()))
    want_f = list(zip(filt["query_id"].tolist(), filt["pos"].tolist()))
    assert len(got_c) > 10_000
    assert got_c == want_c
    assert got_f == want_f


def test_cpp_caller_overlaps_match_the_binding(gpu, golden_cases, tmp_path):
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    src = tmp_path / "reads.tsv"
    out = tmp_path / "out.tsv"
    _write_reads(src, reads)
    r = subprocess.run([str(_caller()), "overlaps", str(src), str(meta["k"]),
                        str(meta["min_freq"]), str(meta["max_freq"]), "4", str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [tuple(int(v) for v in l.split("\t")) for l in out.read_text().splitlines()]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    # the caller runs the adapter's fixed parameters: overlap-range defaults at this k
    want = overlap_tuples_gpu(gpu.overlaps(reads, OverlapParams.make(kmer_size=meta["k"])))
    assert len(got) > 100
    assert got == want


def test_shared_context_refuses_an_index_build(gpu, golden_cases):
    """A context sharing another's index cannot build one, and the owner
    cannot rebuild while it is open."""
    import ctypes
    from cuflye_gb300.backend import load_library
    L = load_library()
    reads, meta, _ = golden_cases["ovl-a"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    h = ctypes.c_void_p()
    assert L.cuflye_open_shared(gpu._h, 0, ctypes.byref(h)) == 0
    try:
        ids = np.ascontiguousarray(reads.ids, dtype=np.int64)
        offs = np.ascontiguousarray(reads.offsets, dtype=np.int64)
        st = L.cuflye_index_build(h, meta["k"], len(ids),
                                  ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                  offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                  reads.bases.tobytes(), meta["min_freq"], meta["max_freq"])
        assert st == 1 and b"shares another" in L.cuflye_last_error(h)
        with pytest.raises(Exception, match="borrows"):
            gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    finally:
        L.cuflye_close(h)
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])  # closed: fine
