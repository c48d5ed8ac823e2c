"""ctypes front end for the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  It wraps ``oracle/_build/libcuflye_oracle.so`` (built from
``oracle/cuflye_oracle.cpp`` by ``oracle/Makefile``), which restates the
reference's candidate loop, chaining and read-to-graph algorithms on the CPU;
see that file's header for the reference file:line each step follows.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libcuflye_oracle.so"

i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
u64p = ctypes.POINTER(ctypes.c_uint64)
u32p = ctypes.POINTER(ctypes.c_uint32)
f32p = ctypes.POINTER(ctypes.c_float)


class Params(ctypes.Structure):
    """Overlap-detector parameters (field order shared with the C struct)."""

    _fields_ = [
        ("kmer_size", ctypes.c_int32),
        ("min_overlap", ctypes.c_int32),
        ("max_jump", ctypes.c_int32),
        ("max_gap", ctypes.c_int32),
        ("gap_jump_threshold", ctypes.c_int32),
        ("max_overhang", ctypes.c_int32),
        ("check_overhang", ctypes.c_int32),
        ("force_local", ctypes.c_int32),
        ("only_max_ext", ctypes.c_int32),
        ("max_overlaps", ctypes.c_int32),
        ("large_gap_penalty", ctypes.c_float),
        ("small_gap_penalty", ctypes.c_float),
        ("min_kmer_survival_rate", ctypes.c_float),
        ("max_divergence", ctypes.c_float),
        ("sample_rate", ctypes.c_float),
    ]


class R2GParams(ctypes.Structure):
    _fields_ = [
        ("max_jump", ctypes.c_int32),
        ("max_read_overlap", ctypes.c_int32),
        ("min_overlap", ctypes.c_int32),
        ("max_separation", ctypes.c_int32),
        ("long_edge", ctypes.c_int32),
        ("big_aln", ctypes.c_int32),
        ("max_chain_divergence", ctypes.c_float),
    ]


def build() -> Path:
    """Compile the oracle library with its Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp = ctypes.c_void_p
        L.orc_index_build.restype = vp
        L.orc_index_build.argtypes = [ctypes.c_int, ctypes.c_int, i64p, i64p, ctypes.c_char_p,
                                      ctypes.c_uint32, ctypes.c_uint32]
        L.orc_index_from_entries.restype = vp
        L.orc_index_from_entries.argtypes = [ctypes.c_int, ctypes.c_size_t, i64p, i64p, u64p,
                                             ctypes.c_size_t, u64p]
        L.orc_index_free.argtypes = [vp]
        L.orc_index_positions.restype = ctypes.c_uint64
        L.orc_index_positions.argtypes = [vp]
        L.orc_index_keys.restype = ctypes.c_uint64
        L.orc_index_keys.argtypes = [vp]
        L.orc_candidates.restype = vp
        L.orc_candidates.argtypes = [vp, ctypes.c_int, i64p, i64p, ctypes.c_char_p, ctypes.c_int]
        L.orc_candidates_windows.restype = vp
        L.orc_candidates_windows.argtypes = [vp, ctypes.c_size_t, i64p, i64p, u64p, u64p]
        L.orc_overlaps.restype = vp
        L.orc_overlaps.argtypes = [vp, ctypes.c_int, i64p, i64p, ctypes.c_char_p,
                                   ctypes.POINTER(Params), ctypes.c_int]
        L.orc_chain_sorted.restype = vp
        L.orc_chain_sorted.argtypes = [ctypes.c_size_t, i32p, i32p, i64p, ctypes.c_int64,
                                       ctypes.c_int32, ctypes.c_size_t, i64p, i32p,
                                       ctypes.c_size_t, i32p, ctypes.POINTER(Params)]
        L.orc_read_to_graph.restype = vp
        L.orc_read_to_graph.argtypes = [vp, ctypes.c_int, i64p, i64p, i32p, i32p, ctypes.c_int,
                                        i64p, i64p, ctypes.c_char_p, ctypes.POINTER(Params),
                                        ctypes.POINTER(R2GParams), ctypes.c_int]
        L.orc_chain_read_alignments.restype = ctypes.c_size_t
        L.orc_chain_read_alignments.argtypes = [ctypes.c_size_t] + [i32p] * 8 + [
            ctypes.POINTER(R2GParams), i32p, i32p, ctypes.c_size_t]
        L.orc_std_sort_u64.argtypes = [ctypes.c_size_t, u64p, u32p]
        L.orc_logf.restype = ctypes.c_float
        L.orc_logf.argtypes = [ctypes.c_float]
        L.orc_set_stable.argtypes = [ctypes.c_int]
        L.orc_set_sort_mode.argtypes = [ctypes.c_uint]
        for name in ("orc_n_matches", "orc_n_filtered", "orc_n_overlaps", "orc_n_rows"):
            getattr(L, name).restype = ctypes.c_size_t
            getattr(L, name).argtypes = [vp]
        L.orc_get_matches.argtypes = [vp, i64p, i32p, u64p, i64p, i32p]
        L.orc_get_filtered.argtypes = [vp, i64p, i32p]
        L.orc_get_overlaps.argtypes = [vp, i64p, i32p, f32p]
        L.orc_get_rows.argtypes = [vp, i64p, f32p]
        L.orc_result_free.argtypes = [vp]
        _LIB = L
    return _LIB


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class SeqBatch:
    """Sequences as Flye signed ids plus concatenated ASCII bases."""

    ids: np.ndarray  # int64 signed ids
    offsets: np.ndarray  # int64, len(ids)+1
    bases: bytes

    @classmethod
    def from_strings(cls, ids, seqs) -> "SeqBatch":
        offs = np.zeros(len(seqs) + 1, dtype=np.int64)
        offs[1:] = np.cumsum([len(s) for s in seqs])
        blob = "".join(seqs).encode("ascii") if seqs and isinstance(seqs[0], str) else b"".join(seqs)
        return cls(np.asarray(ids, dtype=np.int64), offs, blob)


class Index:
    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_index_free(self.h)
            self.h = None

    @classmethod
    def build(cls, k: int, targets: SeqBatch, min_freq: int, max_freq: int) -> "Index":
        ids = np.ascontiguousarray(targets.ids, dtype=np.int64)
        offs = np.ascontiguousarray(targets.offsets, dtype=np.int64)
        h = lib().orc_index_build(k, len(ids), _p(ids, i64p), _p(offs, i64p), targets.bases,
                                  min_freq, max_freq)
        idx = cls(h)
        idx._keep = (ids, offs, targets.bases)
        return idx

    @classmethod
    def from_entries(cls, k, target_ids, positions, keys, repetitive_keys) -> "Index":
        t = np.ascontiguousarray(target_ids, dtype=np.int64)
        p = np.ascontiguousarray(positions, dtype=np.int64)
        kk = np.ascontiguousarray(keys, dtype=np.uint64)
        r = np.ascontiguousarray(repetitive_keys, dtype=np.uint64)
        return cls(lib().orc_index_from_entries(k, len(t), _p(t, i64p), _p(p, i64p), _p(kk, u64p),
                                                len(r), _p(r, u64p)))

    @property
    def n_positions(self) -> int:
        return int(lib().orc_index_positions(self.h))


def _take_matches(r) -> dict:
    L = lib()
    n = L.orc_n_matches(r)
    out = {k: np.empty(n, dtype=d) for k, d in
           (("query_id", np.int64), ("query_pos", np.int32), ("kmer", np.uint64),
            ("target_id", np.int64), ("target_pos", np.int32))}
    L.orc_get_matches(r, _p(out["query_id"], i64p), _p(out["query_pos"], i32p),
                      _p(out["kmer"], u64p), _p(out["target_id"], i64p),
                      _p(out["target_pos"], i32p))
    nf = L.orc_n_filtered(r)
    fq = np.empty(nf, dtype=np.int64)
    fp = np.empty(nf, dtype=np.int32)
    L.orc_get_filtered(r, _p(fq, i64p), _p(fp, i32p))
    out["filtered_query"] = fq
    out["filtered_pos"] = fp
    return out


def candidates(index: Index, queries: SeqBatch, sorted_like_flye: bool = False) -> dict:
    """Candidate records per query in generation order (or after Flye's sort)."""
    ids = np.ascontiguousarray(queries.ids, dtype=np.int64)
    offs = np.ascontiguousarray(queries.offsets, dtype=np.int64)
    r = lib().orc_candidates(index.h, len(ids), _p(ids, i64p), _p(offs, i64p), queries.bases,
                             int(sorted_like_flye))
    try:
        return _take_matches(r)
    finally:
        lib().orc_result_free(r)


def candidates_windows(index: Index, qids, qpos, kmers, keys) -> dict:
    a = np.ascontiguousarray(qids, dtype=np.int64)
    b = np.ascontiguousarray(qpos, dtype=np.int64)
    c = np.ascontiguousarray(kmers, dtype=np.uint64)
    d = np.ascontiguousarray(keys, dtype=np.uint64)
    r = lib().orc_candidates_windows(index.h, len(a), _p(a, i64p), _p(b, i64p), _p(c, u64p),
                                     _p(d, u64p))
    try:
        return _take_matches(r)
    finally:
        lib().orc_result_free(r)


def _take_overlaps(r) -> dict:
    L = lib()
    n = L.orc_n_overlaps(r)
    cols = np.empty((n, 9), dtype=np.int64)
    cl = np.empty(n, dtype=np.int32)
    dv = np.empty(n, dtype=np.float32)
    L.orc_get_overlaps(r, _p(cols, i64p), _p(cl, i32p), _p(dv, f32p))
    return {"cols": cols, "chain_length": cl, "divergence": dv}


def overlaps(index: Index, queries: SeqBatch, params: Params, threads: int = 1) -> dict:
    ids = np.ascontiguousarray(queries.ids, dtype=np.int64)
    offs = np.ascontiguousarray(queries.offsets, dtype=np.int64)
    r = lib().orc_overlaps(index.h, len(ids), _p(ids, i64p), _p(offs, i64p), queries.bases,
                           ctypes.byref(params), threads)
    try:
        return _take_overlaps(r)
    finally:
        lib().orc_result_free(r)


def chain_sorted(cur_pos, ext_pos, ext_ids, query_id, query_len, target_ids, target_lens,
                 filtered, params: Params) -> dict:
    a = np.ascontiguousarray(cur_pos, dtype=np.int32)
    b = np.ascontiguousarray(ext_pos, dtype=np.int32)
    c = np.ascontiguousarray(ext_ids, dtype=np.int64)
    t = np.ascontiguousarray(target_ids, dtype=np.int64)
    tl = np.ascontiguousarray(target_lens, dtype=np.int32)
    f = np.ascontiguousarray(filtered, dtype=np.int32)
    r = lib().orc_chain_sorted(len(a), _p(a, i32p), _p(b, i32p), _p(c, i64p), query_id,
                               query_len, len(t), _p(t, i64p), _p(tl, i32p), len(f),
                               _p(f, i32p), ctypes.byref(params))
    try:
        return _take_overlaps(r)
    finally:
        lib().orc_result_free(r)


def read_to_graph(index: Index, edge_ids, seq_ids, left, right, reads: SeqBatch,
                  params: Params, r2g: R2GParams, threads: int = 1) -> dict:
    e = np.ascontiguousarray(edge_ids, dtype=np.int64)
    s = np.ascontiguousarray(seq_ids, dtype=np.int64)
    lft = np.ascontiguousarray(left, dtype=np.int32)
    rgt = np.ascontiguousarray(right, dtype=np.int32)
    ids = np.ascontiguousarray(reads.ids, dtype=np.int64)
    offs = np.ascontiguousarray(reads.offsets, dtype=np.int64)
    L = lib()
    r = L.orc_read_to_graph(index.h, len(e), _p(e, i64p), _p(s, i64p), _p(lft, i32p),
                            _p(rgt, i32p), len(ids), _p(ids, i64p), _p(offs, i64p),
                            reads.bases, ctypes.byref(params), ctypes.byref(r2g), threads)
    try:
        n = L.orc_n_rows(r)
        cols = np.empty((n, 12), dtype=np.int64)
        dv = np.empty(n, dtype=np.float32)
        L.orc_get_rows(r, _p(cols, i64p), _p(dv, f32p))
        return {"cols": cols, "divergence": dv}
    finally:
        L.orc_result_free(r)


def chain_read_alignments(rows: np.ndarray, left, right, r2g: R2GParams) -> list[list[int]]:
    """rows: int32 array (n, 6) = read_begin, read_end, edge_begin, edge_end, edge_len, score."""
    rows = np.asarray(rows, dtype=np.int32)
    cols = [np.ascontiguousarray(rows[:, i]) for i in range(6)]
    lft = np.ascontiguousarray(left, dtype=np.int32)
    rgt = np.ascontiguousarray(right, dtype=np.int32)
    cap = 4 * len(rows) * len(rows) + 16
    oc = np.empty(cap, dtype=np.int32)
    oi = np.empty(cap, dtype=np.int32)
    n = lib().orc_chain_read_alignments(len(rows), *[_p(c, i32p) for c in cols], _p(lft, i32p),
                                        _p(rgt, i32p), ctypes.byref(r2g), _p(oc, i32p),
                                        _p(oi, i32p), cap)
    chains: list[list[int]] = []
    for c, i in zip(oc[:n], oi[:n]):
        while len(chains) <= c:
            chains.append([])
        chains[c].append(int(i))
    return chains


def std_sort_u64(keys: np.ndarray, payload: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    k = np.array(keys, dtype=np.uint64)
    p = np.array(payload, dtype=np.uint32)
    lib().orc_std_sort_u64(len(k), _p(k, u64p), _p(p, u32p))
    return k, p


def set_stable(stable: bool) -> None:
    lib().orc_set_stable(int(stable))


# Sort places for set_sort_mode (bits of the stable-sort mask).
SORT_KMERMATCH, SORT_EXT, SORT_SCORE, SORT_PRIMARY, SORT_CHAIN_INPUT = 1, 2, 4, 8, 16


def set_sort_mode(stable_mask: int) -> None:
    """Stable sorts at the places in `stable_mask`, std::sort at the others."""
    lib().orc_set_sort_mode(int(stable_mask))


def logf(x: float) -> float:
    return float(lib().orc_logf(ctypes.c_float(x)))


def default_params(**kw) -> Params:
    """Flye's chaining constants as the reference's fixtures record them."""
    p = Params(kmer_size=15, min_overlap=1000, max_jump=1500, max_gap=500,
               gap_jump_threshold=100, max_overhang=1500, check_overhang=1, force_local=0,
               only_max_ext=1, max_overlaps=0, large_gap_penalty=2.0, small_gap_penalty=0.5,
               min_kmer_survival_rate=0.01, max_divergence=1.0, sample_rate=1.0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def default_r2g(**kw) -> R2GParams:
    r = R2GParams(max_jump=1500, max_read_overlap=50, min_overlap=1000, max_separation=500,
                  long_edge=900, big_aln=500, max_chain_divergence=0.25)
    for k, v in kw.items():
        setattr(r, k, v)
    return r
