"""Record layouts and text formats of the three output contracts.

* candidate-record-v1 (docs/abi/candidate-record-v1.md:31-51):
  ``query_id  query_pos  kmer  target_id  target_pos  target_strand``
* overlap-range-v1 (docs/abi/overlap-range-v1.md:21-41):
  ``cur_id cur_begin cur_end cur_len ext_id ext_begin ext_end ext_len score seq_divergence``
* read-alignment-v1 (docs/abi/read-alignment-v1.md:25-48):
  ``chain_id segment_id read_id read_begin read_end read_len edge_id edge_seq_id
  edge_begin edge_end edge_len score seq_divergence``

Floats print as C++ ``std::setprecision(9)`` of a float does (``%.9g`` of the
float value), with an exact zero as ``0``, matching
``tools/validate_overlap_dump.py:24-27``.  Equality is canonical: rows sorted
on all fields, then SHA-256 of the text (``tools/diff_candidate_dumps.py``).
"""

from __future__ import annotations

import hashlib

import numpy as np

CANDIDATE_DTYPE = np.dtype([("query_id", "<i8"), ("target_id", "<i8"), ("kmer", "<u8"),
                            ("query_pos", "<i4"), ("target_pos", "<i4")], align=True)
FILTERED_DTYPE = np.dtype([("query_id", "<i8"), ("pos", "<i4"), ("reserved", "<i4")],
                          align=True)
OVERLAP_DTYPE = np.dtype([("cur_id", "<i8"), ("ext_id", "<i8"), ("cur_begin", "<i4"),
                          ("cur_end", "<i4"), ("cur_len", "<i4"), ("ext_begin", "<i4"),
                          ("ext_end", "<i4"), ("ext_len", "<i4"), ("score", "<i4"),
                          ("seq_divergence", "<f4")], align=True)
READ_ALIGNMENT_DTYPE = np.dtype([("chain_id", "<i8"), ("segment_id", "<i8"), ("read_id", "<i8"),
                                 ("edge_id", "<i8"), ("edge_seq_id", "<i8"),
                                 ("read_begin", "<i4"), ("read_end", "<i4"),
                                 ("read_len", "<i4"), ("edge_begin", "<i4"),
                                 ("edge_end", "<i4"), ("edge_len", "<i4"), ("score", "<i4"),
                                 ("seq_divergence", "<f4")], align=True)

# cuflye_chain_record: a candidate chain's segment, the fields of one
# compact-binary record (docs/abi/read-alignment-compact-binary-v0.md:37-58)
CHAIN_RECORD_DTYPE = np.dtype([("query_id", "<i8"), ("chain_id", "<i4"), ("segment_id", "<i4"),
                               ("overlap_index", "<i4"), ("reserved", "<i4"),
                               ("candidate_id", "<i8"), ("read_id", "<i8"), ("edge_id", "<i8"),
                               ("edge_seq_id", "<i8"), ("read_begin", "<i4"),
                               ("read_end", "<i4"), ("read_len", "<i4"), ("edge_left", "<i4"),
                               ("edge_right", "<i4"), ("edge_begin", "<i4"),
                               ("edge_end", "<i4"), ("edge_len", "<i4"), ("score", "<i4"),
                               ("seq_divergence", "<f4")], align=True)
# cuflye_edge_overlap: a read-alignment replay fixture's input row
# (edge-overlaps.tsv of docs/abi/read-alignment-replay-fixture-v0.md)
EDGE_OVERLAP_DTYPE = np.dtype([("candidate_id", "<i8"), ("read_id", "<i8"),
                               ("read_begin", "<i4"), ("read_end", "<i4"), ("read_len", "<i4"),
                               ("edge_left", "<i4"), ("edge_right", "<i4"),
                               ("edge_begin", "<i4"), ("edge_end", "<i4"), ("edge_len", "<i4"),
                               ("edge_id", "<i8"), ("edge_seq_id", "<i8"), ("score", "<i4"),
                               ("seq_divergence", "<f4")], align=True)
# the compact binary payload's fixed-width little-endian record (92 bytes,
# no padding), for reading a payload back
COMPACT_RECORD_DTYPE = np.dtype([("query_id", "<i8"), ("chain_id", "<i4"), ("segment_id", "<i4"),
                                 ("overlap_index", "<i4"), ("candidate_id", "<i8"),
                                 ("read_id", "<i8"), ("read_begin", "<i4"), ("read_end", "<i4"),
                                 ("read_len", "<i4"), ("edge_id", "<i8"), ("edge_left", "<i4"),
                                 ("edge_right", "<i4"), ("edge_seq_id", "<i8"),
                                 ("edge_begin", "<i4"), ("edge_end", "<i4"),
                                 ("edge_len", "<i4"), ("score", "<i4"),
                                 ("seq_divergence", "<f4")])

assert CHAIN_RECORD_DTYPE.itemsize == 96
assert EDGE_OVERLAP_DTYPE.itemsize == 72
assert COMPACT_RECORD_DTYPE.itemsize == 92
assert CANDIDATE_DTYPE.itemsize == 32
assert FILTERED_DTYPE.itemsize == 16
assert OVERLAP_DTYPE.itemsize == 48
assert READ_ALIGNMENT_DTYPE.itemsize == 72


def format_float(value: float) -> str:
    v = float(np.float32(value))
    return "0" if v == 0 else format(v, ".9g")


def candidate_lines(rec: np.ndarray) -> list[str]:
    return [f"{r['query_id']}\t{r['query_pos']}\t{r['kmer']}\t{r['target_id']}\t"
            f"{r['target_pos']}\t{'+' if r['target_id'] > 0 else '-'}\n" for r in rec]


def overlap_lines(rec: np.ndarray) -> list[str]:
    return [f"{r['cur_id']}\t{r['cur_begin']}\t{r['cur_end']}\t{r['cur_len']}\t{r['ext_id']}\t"
            f"{r['ext_begin']}\t{r['ext_end']}\t{r['ext_len']}\t{r['score']}\t"
            f"{format_float(r['seq_divergence'])}\n" for r in rec]


def read_alignment_lines(rec: np.ndarray) -> list[str]:
    return [f"{r['chain_id']}\t{r['segment_id']}\t{r['read_id']}\t{r['read_begin']}\t"
            f"{r['read_end']}\t{r['read_len']}\t{r['edge_id']}\t{r['edge_seq_id']}\t"
            f"{r['edge_begin']}\t{r['edge_end']}\t{r['edge_len']}\t{r['score']}\t"
            f"{format_float(r['seq_divergence'])}\n" for r in rec]


def write_tsv(path, lines: list[str]) -> None:
    with open(path, "w", encoding="utf-8", newline="\n") as fh:
        fh.writelines(lines)


def _canonical_key(line: str):
    out = []
    for f in line.rstrip("\n").split("\t"):
        try:
            out.append((0, int(f)))
        except ValueError:
            try:
                out.append((1, float(f)))
            except ValueError:
                out.append((2, f))
    return out


def canonical_sha256(lines: list[str]) -> str:
    """SHA-256 of the rows sorted on all fields (numeric where numeric)."""
    h = hashlib.sha256()
    for line in sorted(lines, key=_canonical_key):
        h.update(line.encode("utf-8"))
    return h.hexdigest()


def read_compact_binary(data: bytes) -> tuple[dict, np.ndarray]:
    """The header fields and records of a compact binary payload."""
    u32 = lambda o: int.from_bytes(data[o:o + 4], "little")
    u64 = lambda o: int.from_bytes(data[o:o + 8], "little")
    head = {"magic": data[:8], "header_bytes": u32(8), "record_bytes": u32(12),
            "version": (u32(16), u32(20)), "fixtures": u64(24), "records": u64(32),
            "total_inputs": u64(40), "min_inputs": u32(48), "max_inputs": u32(52),
            "output_mode": u32(56), "reserved": u32(60)}
    recs = np.frombuffer(data, dtype=COMPACT_RECORD_DTYPE, offset=64,
                         count=(len(data) - 64) // 92)
    return head, recs
