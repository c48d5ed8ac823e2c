"""Host-side mirror of the reference's candidate-backend seam over the C ABI.

The reference selects the candidate backend from ``CUFLYE_CANDIDATE_BACKEND``
(``patches/flye/2.9.6/0002-cuflye-candidate-backend-seam.patch:29-43``), opens
the CUDA device named by ``CUFLYE_CUDA_DEVICE`` under
``CUFLYE_CUDA_MEMORY_BUDGET_BYTES`` and fails fast with the stub's message
when the CUDA path cannot serve a request
(``patches/flye/2.9.6/0003-cuflye-cuda-backend-stub.patch:37-46``).  This
module keeps those names, meanings and errors and calls
``libcuflye_gb300.so`` through ``include/cuflye.h``.  There is no CPU path
here: if the library is missing, or a call is unsupported, it raises.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcuflye_gb300.so"

STATUS = {0: "CUFLYE_OK", 1: "CUFLYE_ERR_INVALID", 2: "CUFLYE_ERR_UNSUPPORTED",
          3: "CUFLYE_ERR_BUDGET", 4: "CUFLYE_ERR_CUDA", 5: "CUFLYE_ERR_CAPACITY",
          6: "CUFLYE_ERR_TIMEOUT", 7: "CUFLYE_ERR_NO_INDEX", 8: "CUFLYE_PENDING"}
ERR_CAPACITY = 5
PENDING = 8


class CuflyeError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class OverlapParams(ctypes.Structure):
    """cuflye_overlap_params; defaults are the chaining constants recorded by
    the reference's Flye fixtures (maximum_jump 1500, max_jump_gap 500,
    penalties 2 / 0.5 above / below 100, survival rate 0.01, ...)."""

    _fields_ = [(n, ctypes.c_int32) for n in (
        "kmer_size", "min_overlap", "max_jump", "max_gap", "gap_jump_threshold", "max_overhang",
        "check_overhang", "force_local", "only_max_ext", "max_overlaps")] + [
        (n, ctypes.c_float) for n in ("large_gap_penalty", "small_gap_penalty",
                                      "min_kmer_survival_rate", "max_divergence", "sample_rate")]

    @classmethod
    def make(cls, **kw) -> "OverlapParams":
        p = cls(kmer_size=15, min_overlap=1000, max_jump=1500, max_gap=500,
                gap_jump_threshold=100, max_overhang=1500, check_overhang=1, force_local=0,
                only_max_ext=1, max_overlaps=0, large_gap_penalty=2.0, small_gap_penalty=0.5,
                min_kmer_survival_rate=0.01, max_divergence=1.0, sample_rate=1.0)
        for k, v in kw.items():
            setattr(p, k, v)
        return p


class R2GParams(ctypes.Structure):
    """cuflye_r2g_params (ReadAligner constants: SMALL_ALN/BIG_ALN/LONG_EDGE at
    patches/flye/2.9.6/0025-cuflye-read-alignment-dump.patch:94-96)."""

    _fields_ = [(n, ctypes.c_int32) for n in (
        "max_jump", "max_read_overlap", "min_overlap", "max_separation", "long_edge",
        "big_aln")] + [("max_chain_divergence", ctypes.c_float)]

    @classmethod
    def make(cls, **kw) -> "R2GParams":
        p = cls(max_jump=1500, max_read_overlap=50, min_overlap=1000, max_separation=500,
                long_edge=900, big_aln=500, max_chain_divergence=0.25)
        for k, v in kw.items():
            setattr(p, k, v)
        return p


_LIB = None
class LaunchShape(ctypes.Structure):
    """cuflye_launch_shape: blocks per SM of the chaining DP (1-8), the
    backtrack (1-4), the KmerMatch radix scatter (1-2) and the rounds of the
    libstdc++-order sort (1-2); 0 keeps a kernel's default."""
    _fields_ = [("dp_blocks_per_sm", ctypes.c_int32), ("backtrack_blocks_per_sm", ctypes.c_int32),
                ("scatter_blocks_per_sm", ctypes.c_int32), ("round_blocks_per_sm", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


_vp = ctypes.c_void_p
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_szp = ctypes.POINTER(ctypes.c_size_t)


def load_library(path: Path | None = None) -> ctypes.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = Path(path or os.environ.get("CUFLYE_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"libcuflye_gb300.so not built ({p}); run cuflye_gb300.build.build()")
    L = ctypes.CDLL(str(p))
    S = ctypes.c_int
    L.cuflye_candidate_backend.restype = ctypes.c_int
    L.cuflye_candidate_backend.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.cuflye_open.restype = S
    L.cuflye_open.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.cuflye_open_from_env.restype = S
    L.cuflye_open_from_env.argtypes = [ctypes.POINTER(_vp)]
    L.cuflye_close.argtypes = [_vp]
    L.cuflye_open_shared.restype = S
    L.cuflye_open_shared.argtypes = [_vp, ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.cuflye_last_error.restype = ctypes.c_char_p
    L.cuflye_last_error.argtypes = [_vp]
    L.cuflye_memory_stats.restype = S
    L.cuflye_memory_stats.argtypes = [_vp, _u64p, _u64p]
    L.cuflye_index_build.restype = S
    L.cuflye_index_build.argtypes = [_vp, ctypes.c_int, ctypes.c_size_t, _i64p, _i64p,
                                     ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32]
    L.cuflye_index_from_entries.restype = S
    L.cuflye_index_from_entries.argtypes = [_vp, ctypes.c_int, ctypes.c_size_t, _i64p, _i64p,
                                            _u64p, ctypes.c_size_t, _u64p]
    L.cuflye_index_stats.restype = S
    L.cuflye_index_stats.argtypes = [_vp, _u64p, _u64p, _u64p]
    L.cuflye_candidates.restype = S
    L.cuflye_candidates.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, ctypes.c_char_p, _vp,
                                    ctypes.c_size_t, _szp, _vp, ctypes.c_size_t, _szp]
    L.cuflye_overlaps.restype = S
    L.cuflye_overlaps.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, ctypes.c_char_p,
                                  ctypes.POINTER(OverlapParams), _vp, ctypes.c_size_t, _szp]
    L.cuflye_set_batch_queries.restype = S
    L.cuflye_set_batch_queries.argtypes = [_vp, ctypes.c_size_t]
    L.cuflye_graph_set.restype = S
    L.cuflye_graph_set.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, _i32p, _i32p]
    L.cuflye_read_to_graph.restype = S
    L.cuflye_read_to_graph.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, ctypes.c_char_p,
                                       ctypes.POINTER(OverlapParams), ctypes.POINTER(R2GParams),
                                       _vp, ctypes.c_size_t, _szp]
    L.cuflye_read_to_graph_chains.restype = S
    L.cuflye_read_to_graph_chains.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p,
                                              ctypes.c_char_p, ctypes.POINTER(OverlapParams),
                                              ctypes.POINTER(R2GParams), _vp, ctypes.c_size_t,
                                              _szp, _u64p]
    L.cuflye_chain_read_alignments.restype = S
    L.cuflye_chain_read_alignments.argtypes = [
        _vp, ctypes.c_size_t, _u64p, _i64p, _vp, ctypes.POINTER(R2GParams),
        ctypes.POINTER(ctypes.c_float), ctypes.c_size_t, _vp, ctypes.c_size_t, _szp,
        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t, _szp,
        _vp, ctypes.c_size_t, _szp]
    L.cuflye_compact_binary.restype = S
    L.cuflye_compact_binary.argtypes = [_vp, ctypes.c_size_t, ctypes.c_size_t, _u64p, _vp,
                                        ctypes.c_size_t, _szp]
    L.cuflye_std_sort_segments.restype = S
    L.cuflye_std_sort_segments.argtypes = [_vp, _u64p, _u32p, _u64p, ctypes.c_size_t]
    L.cuflye_kernel_launches.restype = S
    L.cuflye_kernel_launches.argtypes = [_u64p]
    L.cuflye_last_timing.restype = S
    L.cuflye_last_timing.argtypes = [_vp, ctypes.POINTER(ctypes.c_double), _u64p, ctypes.c_size_t]
    L.cuflye_last_sort_stats.restype = S
    L.cuflye_last_sort_stats.argtypes = [_vp, _u64p, ctypes.c_size_t]
    L.cuflye_last_pass_stats.restype = S
    L.cuflye_last_pass_stats.argtypes = [_vp, _u64p, _u64p, ctypes.POINTER(ctypes.c_double)]
    L.cuflye_last_passes.restype = S
    L.cuflye_last_passes.argtypes = [_vp, _u64p]
    L.cuflye_set_sorted_emission.restype = S
    L.cuflye_set_sorted_emission.argtypes = [_vp, ctypes.c_int]
    L.cuflye_set_launch_shape.restype = S
    L.cuflye_set_launch_shape.argtypes = [_vp, ctypes.POINTER(LaunchShape)]
    L.cuflye_get_launch_shape.restype = S
    L.cuflye_get_launch_shape.argtypes = [_vp, ctypes.POINTER(LaunchShape)]
    L.cuflye_autotune.restype = S
    L.cuflye_autotune.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, ctypes.c_char_p,
                                  ctypes.POINTER(OverlapParams), ctypes.POINTER(LaunchShape),
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.cuflye_set_index_build_windows.restype = S
    L.cuflye_set_index_build_windows.argtypes = [_vp, ctypes.c_uint64]
    L.cuflye_last_index_ranges.restype = S
    L.cuflye_last_index_ranges.argtypes = [_vp, _u64p]
    L.cuflye_server_open.restype = S
    L.cuflye_server_open.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(OverlapParams),
                                     ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.cuflye_submit.restype = S
    L.cuflye_submit.argtypes = [_vp, ctypes.c_size_t, _i64p, _i64p, ctypes.c_char_p, _u64p]
    L.cuflye_poll.restype = S
    L.cuflye_poll.argtypes = [_vp, ctypes.c_uint64, ctypes.c_int, _vp, ctypes.c_size_t, _szp]
    L.cuflye_trim.restype = S
    L.cuflye_trim.argtypes = [_vp]
    L.cuflye_poll_any.restype = S
    L.cuflye_poll_any.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64), _vp,
                                  ctypes.c_size_t, _szp]
    L.cuflye_server_stats.restype = S
    L.cuflye_server_stats.argtypes = [_vp, _u64p, _u64p, _u64p]
    L.cuflye_server_last_error.restype = ctypes.c_char_p
    L.cuflye_server_last_error.argtypes = [_vp]
    L.cuflye_server_close.argtypes = [_vp]
    _LIB = L
    return L


def candidate_backend() -> str:
    """'cpu' or 'cuda' from CUFLYE_CANDIDATE_BACKEND; anything else raises
    ``Unsupported CUFLYE_CANDIDATE_BACKEND: <value>`` like the reference."""
    buf = ctypes.create_string_buffer(256)
    r = load_library().cuflye_candidate_backend(buf, 256)
    if r < 0:
        raise RuntimeError(buf.value.decode())
    return "cuda" if r == 1 else "cpu"


def stub_message(device: str | None = None, budget: str | None = None) -> str:
    """The fail-fast text of the reference stub for an unsupported request."""
    device = device if device is not None else (os.environ.get("CUFLYE_CUDA_DEVICE") or "0")
    budget = budget if budget is not None else (
        os.environ.get("CUFLYE_CUDA_MEMORY_BUDGET_BYTES") or "unbounded")
    return ("cuFlye CUDA candidate backend selected; adapter=cuflye_gb300; "
            f"CUFLYE_CUDA_DEVICE={device}; CUFLYE_CUDA_MEMORY_BUDGET_BYTES={budget}; ")


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class Sequences:
    """Flye-style records: signed ids and concatenated ASCII bases."""

    ids: np.ndarray
    offsets: np.ndarray
    bases: np.ndarray  # uint8

    @classmethod
    def of(cls, reads) -> "Sequences":
        if isinstance(reads, Sequences):
            return reads
        return cls(np.ascontiguousarray(reads.ids, dtype=np.int64),
                   np.ascontiguousarray(reads.offsets, dtype=np.int64),
                   np.ascontiguousarray(reads.bases, dtype=np.uint8))

    @property
    def n(self) -> int:
        return len(self.ids)


class CudaBackend:
    """One device context: resident index, optional graph, device arena."""

    def __init__(self, device: int | None = None, memory_budget_bytes: int | None = None):
        L = load_library()
        h = _vp()
        if device is None and memory_budget_bytes is None:
            st = L.cuflye_open_from_env(ctypes.byref(h))
        else:
            st = L.cuflye_open(int(device or 0), int(memory_budget_bytes or 0), ctypes.byref(h))
        if st != 0:
            # the library keeps the failed open's message for this thread
            msg = L.cuflye_last_error(None)
            raise CuflyeError(st, msg.decode() if msg else stub_message() + "cuflye_open failed")
        self._h = h
        self._L = L
        self.k = None

    # -- plumbing
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.cuflye_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        if st != 0:
            raise CuflyeError(st, self._L.cuflye_last_error(self._h).decode())

    def memory_stats(self) -> tuple[int, int]:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.cuflye_memory_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_batch_queries(self, n: int) -> None:
        self._check(self._L.cuflye_set_batch_queries(self._h, int(n)))

    def last_timing(self) -> tuple[list[float], list[int]]:
        ms = (ctypes.c_double * 7)()
        by = (ctypes.c_uint64 * 7)()
        self._check(self._L.cuflye_last_timing(self._h, ms, by, 7))
        return list(ms), list(by)

    SORT_STATS = ("match_plain", "match_libstdcxx", "ext_plain", "ext_libstdcxx", "score_plain",
                  "score_libstdcxx", "backtrack_redo", "emission_fallbacks")

    def last_sort_stats(self) -> dict:
        """How the last overlaps / read-to-graph call's sort points ran (segments per path)."""
        v = (ctypes.c_uint64 * 8)()
        self._check(self._L.cuflye_last_sort_stats(self._h, v, 8))
        return dict(zip(self.SORT_STATS, list(v)))

    def set_sorted_emission(self, mode) -> None:
        """Hits straight into KmerMatch order: 1 / True where windows are
        dense (the default), 2 for every pass, 0 / False never (emit + sort)."""
        self._check(self._L.cuflye_set_sorted_emission(self._h, int(mode)))

    def trim(self) -> None:
        """Returns the context's cached working buffers to the device (the
        index stays)."""
        self._check(self._L.cuflye_trim(self._h))

    def last_pass_stats(self) -> dict:
        """Passes of the last call, budget retries, and host ms in allocation."""
        a, b, t = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_double()
        self._check(self._L.cuflye_last_pass_stats(self._h, ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(t)))
        return {"passes": a.value, "retries": b.value, "alloc_ms": round(t.value, 1)}

    def last_passes(self) -> int:
        """Passes (runs of queries through the device) of the last call."""
        v = ctypes.c_uint64()
        self._check(self._L.cuflye_last_passes(self._h, ctypes.byref(v)))
        return int(v.value)

    def set_launch_shape(self, **blocks_per_sm) -> None:
        """Sets blocks per SM by field name of LaunchShape (others keep their value)."""
        cur = self.launch_shape()
        cur.update(blocks_per_sm)
        self._check(self._L.cuflye_set_launch_shape(self._h, ctypes.byref(LaunchShape(**cur))))

    def launch_shape(self) -> dict:
        v = LaunchShape()
        self._check(self._L.cuflye_get_launch_shape(self._h, ctypes.byref(v)))
        return v.as_dict()

    def autotune(self, queries, params: "OverlapParams") -> dict:
        """Picks the launch shape with the least device time on `queries` (a
        sample of the workload) and keeps it for later calls."""
        q = Sequences.of(queries)
        shape = LaunchShape()
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cuflye_autotune(self._h, q.n, _ptr(q.ids, _i64p),
                                            _ptr(q.offsets, _i64p),
                                            q.bases.ctypes.data_as(ctypes.c_char_p),
                                            ctypes.byref(params), ctypes.byref(shape),
                                            ctypes.byref(a), ctypes.byref(b)))
        return {"shape": shape.as_dict(), "ms_start": a.value, "ms_chosen": b.value}

    def set_index_build_windows(self, max_windows: int) -> None:
        """Caps the windows of one key range of the index build (0: budget decides)."""
        self._check(self._L.cuflye_set_index_build_windows(self._h, int(max_windows)))

    def last_index_ranges(self) -> int:
        """Key ranges the last index build ran in (1: all windows at once)."""
        v = ctypes.c_uint64()
        self._check(self._L.cuflye_last_index_ranges(self._h, ctypes.byref(v)))
        return int(v.value)

    # -- index
    def build_index(self, targets, k: int, min_freq: int, max_freq: int) -> dict:
        t = Sequences.of(targets)
        self._check(self._L.cuflye_index_build(self._h, int(k), t.n, _ptr(t.ids, _i64p),
                                               _ptr(t.offsets, _i64p),
                                               t.bases.ctypes.data_as(ctypes.c_char_p),
                                               int(min_freq), int(max_freq)))
        self.k = k
        return self.index_stats()

    def index_from_entries(self, k, target_ids, positions, keys, repetitive_keys=()) -> dict:
        t = np.ascontiguousarray(target_ids, dtype=np.int64)
        p = np.ascontiguousarray(positions, dtype=np.int64)
        kk = np.ascontiguousarray(keys, dtype=np.uint64)
        r = np.ascontiguousarray(repetitive_keys, dtype=np.uint64)
        self._check(self._L.cuflye_index_from_entries(self._h, int(k), len(t), _ptr(t, _i64p),
                                                      _ptr(p, _i64p), _ptr(kk, _u64p), len(r),
                                                      _ptr(r, _u64p)))
        self.k = k
        return self.index_stats()

    def index_stats(self) -> dict:
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.cuflye_index_stats(self._h, ctypes.byref(a), ctypes.byref(b),
                                               ctypes.byref(c)))
        return {"keys": a.value, "positions": b.value, "repetitive": c.value}

    # -- candidate loop (collectCandidateMatches)
    def candidates(self, queries, capacity: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        q = Sequences.of(queries)
        cap = capacity if capacity is not None else max(1024, int(q.offsets[-1]) * 8)
        fcap = max(1024, int(q.offsets[-1]) + 1)
        while True:
            out = np.empty(cap, dtype=abi.CANDIDATE_DTYPE)
            fout = np.empty(fcap, dtype=abi.FILTERED_DTYPE)
            n, nf = ctypes.c_size_t(), ctypes.c_size_t()
            st = self._L.cuflye_candidates(self._h, q.n, _ptr(q.ids, _i64p),
                                           _ptr(q.offsets, _i64p),
                                           q.bases.ctypes.data_as(ctypes.c_char_p),
                                           out.ctypes.data, cap, ctypes.byref(n),
                                           fout.ctypes.data, fcap, ctypes.byref(nf))
            if st == ERR_CAPACITY:
                cap, fcap = max(cap, n.value), max(fcap, nf.value)
                continue
            self._check(st)
            return out[:n.value].copy(), fout[:nf.value].copy()

    # -- OverlapDetector::getSeqOverlaps
    def overlaps(self, queries, params: OverlapParams, capacity: int | None = None,
                 out: np.ndarray | None = None) -> np.ndarray:
        """Rows of every query; ``out`` may supply a (pinned) output buffer.

        A call whose rows exceed the buffer returns CUFLYE_ERR_CAPACITY after
        all its work and runs again with the exact size, so the default buffer
        is generous: 256 rows per query (untouched pages cost no memory), at
        most 2^27 rows."""
        q = Sequences.of(queries)
        cap = capacity if capacity is not None else max(1024, min(256 * q.n, 1 << 27))
        caller_buffer = out is not None
        if out is not None:
            cap = len(out)
        while True:
            if out is None or len(out) < cap:
                out = np.empty(cap, dtype=abi.OVERLAP_DTYPE)
            n = ctypes.c_size_t()
            st = self._L.cuflye_overlaps(self._h, q.n, _ptr(q.ids, _i64p), _ptr(q.offsets, _i64p),
                                         q.bases.ctypes.data_as(ctypes.c_char_p),
                                         ctypes.byref(params), out.ctypes.data, cap,
                                         ctypes.byref(n))
            if st == ERR_CAPACITY:
                cap = n.value
                caller_buffer = False
                continue
            self._check(st)
            # a view of the caller's buffer; a copy of an internal one, so the
            # generous default allocation is not kept alive by the result
            return out[:n.value] if caller_buffer else out[:n.value].copy()

    # -- ReadAligner::alignReads per-read body
    def set_graph(self, edge_ids, seq_ids, left, right) -> None:
        e = np.ascontiguousarray(edge_ids, dtype=np.int64)
        s = np.ascontiguousarray(seq_ids, dtype=np.int64)
        lft = np.ascontiguousarray(left, dtype=np.int32)
        rgt = np.ascontiguousarray(right, dtype=np.int32)
        self._check(self._L.cuflye_graph_set(self._h, len(e), _ptr(e, _i64p), _ptr(s, _i64p),
                                             _ptr(lft, _i32p), _ptr(rgt, _i32p)))

    def read_to_graph(self, reads, params: OverlapParams, r2g: R2GParams,
                      capacity: int | None = None) -> np.ndarray:
        q = Sequences.of(reads)
        cap = capacity if capacity is not None else max(1024, 64 * q.n)
        while True:
            out = np.empty(cap, dtype=abi.READ_ALIGNMENT_DTYPE)
            n = ctypes.c_size_t()
            st = self._L.cuflye_read_to_graph(self._h, q.n, _ptr(q.ids, _i64p),
                                              _ptr(q.offsets, _i64p),
                                              q.bases.ctypes.data_as(ctypes.c_char_p),
                                              ctypes.byref(params), ctypes.byref(r2g),
                                              out.ctypes.data, cap, ctypes.byref(n))
            if st == ERR_CAPACITY:
                cap = n.value
                continue
            self._check(st)
            return out[:n.value].copy()

    def read_to_graph_chains(self, reads, params: OverlapParams, r2g: R2GParams,
                             capacity: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Candidate chains (before the divergence filter) as chain records,
        and each read's chain-input overlap count."""
        q = Sequences.of(reads)
        cap = capacity if capacity is not None else max(1024, 64 * q.n)
        inputs = np.zeros(max(q.n, 1), dtype=np.uint64)
        while True:
            out = np.empty(cap, dtype=abi.CHAIN_RECORD_DTYPE)
            n = ctypes.c_size_t()
            st = self._L.cuflye_read_to_graph_chains(
                self._h, q.n, _ptr(q.ids, _i64p), _ptr(q.offsets, _i64p),
                q.bases.ctypes.data_as(ctypes.c_char_p), ctypes.byref(params), ctypes.byref(r2g),
                out.ctypes.data, cap, ctypes.byref(n), _ptr(inputs, _u64p))
            if st == ERR_CAPACITY:
                cap = n.value
                continue
            self._check(st)
            return out[:n.value].copy(), inputs[:q.n].copy()

    def chain_read_alignments(self, fixtures: list[np.ndarray], query_ids, r2g: R2GParams,
                              chain_divergences=None) -> dict:
        """Read-alignment replay fixtures (arrays of EDGE_OVERLAP_DTYPE):
        candidate chains as chain records, per chain its divergence and
        whether it is kept, and the kept chains' rows with complements."""
        offs = np.zeros(len(fixtures) + 1, dtype=np.uint64)
        offs[1:] = np.cumsum([len(f) for f in fixtures])
        ov = (np.concatenate(fixtures) if fixtures else
              np.zeros(0, dtype=abi.EDGE_OVERLAP_DTYPE)).astype(abi.EDGE_OVERLAP_DTYPE)
        ov = np.ascontiguousarray(ov)
        qids = np.ascontiguousarray(query_ids, dtype=np.int64)
        din = None if chain_divergences is None else np.ascontiguousarray(chain_divergences,
                                                                           dtype=np.float32)
        cap = max(64, 4 * len(ov))
        while True:
            out = np.empty(cap, dtype=abi.CHAIN_RECORD_DTYPE)
            div = np.empty(cap, dtype=np.float32)
            kept = np.empty(cap, dtype=np.uint8)
            rows = np.empty(2 * cap, dtype=abi.READ_ALIGNMENT_DTYPE)
            n, nc, nr = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
            st = self._L.cuflye_chain_read_alignments(
                self._h, len(fixtures), _ptr(offs, _u64p), _ptr(qids, _i64p), ov.ctypes.data,
                ctypes.byref(r2g),
                None if din is None else din.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                0 if din is None else len(din), out.ctypes.data, cap, ctypes.byref(n),
                div.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                kept.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), cap, ctypes.byref(nc),
                rows.ctypes.data, 2 * cap, ctypes.byref(nr))
            if st == ERR_CAPACITY:
                cap = max(cap * 2, n.value, nc.value, nr.value)
                continue
            self._check(st)
            return {"records": out[:n.value].copy(), "divergence": div[:nc.value].copy(),
                    "kept": kept[:nc.value].astype(bool), "rows": rows[:nr.value].copy()}

    # -- the device sort behind every Flye sort point
    def std_sort_segments(self, keys, values, seg_offsets) -> tuple[np.ndarray, np.ndarray]:
        k = np.array(keys, dtype=np.uint64)
        v = np.array(values, dtype=np.uint32)
        o = np.ascontiguousarray(seg_offsets, dtype=np.uint64)
        self._check(self._L.cuflye_std_sort_segments(self._h, _ptr(k, _u64p), _ptr(v, _u32p),
                                                     _ptr(o, _u64p), len(o) - 1))
        return k, v


class CudaServer:
    """Continuous batching of overlap requests (cuflye_server_*): requests
    are submitted as they arrive, and each worker context takes every request
    waiting when it falls idle, so batches overlap on the device."""

    def __init__(self, backend: CudaBackend, params: OverlapParams, workers: int = 2,
                 max_batch_bases: int = 0):
        self._L = backend._L
        self._backend = backend  # keeps the owner (and its index) alive
        self._params = params
        h = _vp()
        st = self._L.cuflye_server_open(backend._h, int(workers), ctypes.byref(params),
                                        int(max_batch_bases), ctypes.byref(h))
        if st != 0:
            raise CuflyeError(st, self._L.cuflye_last_error(backend._h).decode())
        self._h = h

    def _err(self, st: int):
        raise CuflyeError(st, self._L.cuflye_server_last_error(self._h).decode())

    def submit(self, queries) -> int:
        q = Sequences.of(queries)
        t = ctypes.c_uint64()
        st = self._L.cuflye_submit(self._h, q.n, _ptr(q.ids, _i64p), _ptr(q.offsets, _i64p),
                                   q.bases.ctypes.data_as(ctypes.c_char_p), ctypes.byref(t))
        if st != 0:
            self._err(st)
        return t.value

    def poll(self, ticket: int, wait_ms: int = -1, capacity: int = 4096):
        """Rows of a finished request, or None while it is pending."""
        cap = capacity
        while True:
            out = np.empty(cap, dtype=abi.OVERLAP_DTYPE)
            n = ctypes.c_size_t()
            st = self._L.cuflye_poll(self._h, int(ticket), int(wait_ms), out.ctypes.data, cap,
                                     ctypes.byref(n))
            if st == PENDING:
                return None
            if st == ERR_CAPACITY:
                cap = n.value
                continue
            if st != 0:
                self._err(st)
            return out[:n.value]

    def poll_any(self, wait_ms: int = -1, capacity: int = 4096):
        """The next finished request in completion order: (ticket, rows), or
        None when none finished within wait_ms.  A request that failed raises
        its error."""
        tk = ctypes.c_uint64()
        out = np.empty(capacity, dtype=abi.OVERLAP_DTYPE)
        n = ctypes.c_size_t()
        st = self._L.cuflye_poll_any(self._h, int(wait_ms), ctypes.byref(tk), out.ctypes.data,
                                     capacity, ctypes.byref(n))
        if st == PENDING:
            return None
        if st == ERR_CAPACITY:  # kept for poll on its ticket
            return tk.value, self.poll(tk.value, 0, capacity=n.value)
        if st != 0:
            self._err(st)
        return tk.value, out[:n.value]

    def stats(self) -> dict:
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        self._L.cuflye_server_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {"batches": a.value, "requests": b.value, "pending": c.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.cuflye_server_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def collect_candidate_matches_cuda(backend: CudaBackend, query_id: int, sequence: bytes):
    """collectCandidateMatchesCuda*: candidate records and filtered positions of
    one query, in Flye's generation order (the callee of
    patches/flye/2.9.6/0005-cuflye-real-data-pack-dump.patch:246-250)."""
    seq = np.frombuffer(sequence, dtype=np.uint8)
    q = Sequences(np.array([query_id], dtype=np.int64),
                  np.array([0, len(seq)], dtype=np.int64), seq.copy())
    return backend.candidates(q)


def compact_binary(records: np.ndarray, inputs_per_fixture) -> bytes:
    """The compact binary payload of chain records (host code of the
    library, no device)."""
    L = load_library()
    rec = np.ascontiguousarray(records, dtype=abi.CHAIN_RECORD_DTYPE)
    inp = np.ascontiguousarray(inputs_per_fixture, dtype=np.uint64)
    n = ctypes.c_size_t()
    st = L.cuflye_compact_binary(rec.ctypes.data, len(rec), len(inp), _ptr(inp, _u64p), None, 0,
                                 ctypes.byref(n))
    if st not in (0, ERR_CAPACITY):
        raise CuflyeError(st, "compact binary payload")
    out = np.zeros(n.value, dtype=np.uint8)
    st = L.cuflye_compact_binary(rec.ctypes.data, len(rec), len(inp), _ptr(inp, _u64p),
                                 out.ctypes.data, len(out), ctypes.byref(n))
    if st != 0:
        raise CuflyeError(st, "compact binary payload")
    return out.tobytes()
