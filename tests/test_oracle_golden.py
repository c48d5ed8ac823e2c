"""CPU: pins the oracle to the reference's own golden vectors and to the
outputs of the reference's replay tools on seeded synthetic cases."""

import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN

REF = GOLDEN / "reference"


def enc(s: str) -> int:
    m = {"A": 0, "C": 1, "G": 2, "T": 3}
    r = 0
    for c in s:
        r = (r << 2) + m.get(c.upper(), 0)
    return r


def rc(x: int, k: int) -> int:
    r = 0
    for _ in range(k):
        r = (r << 2) + ((~x) & 3)
        x >>= 2
    return r


def std(x: int, k: int) -> int:
    return min(x, rc(x, k))


def rows(path):
    return [l.rstrip("\n").split("\t") for l in open(path) if l.strip()]


def as_records(m):
    return sorted((int(m["query_id"][i]), int(m["query_pos"][i]), int(m["kmer"][i]),
                   int(m["target_id"][i]), int(m["target_pos"][i]),
                   "+" if m["target_id"][i] > 0 else "-") for i in range(len(m["query_id"])))


def expected(d):
    return sorted((int(a), int(b), int(c), int(e), int(f), g)
                  for a, b, c, e, f, g in rows(REF / d / "expected.candidates.tsv"))


def test_kmer_join_fixture(oracle_mod):
    O = oracle_mod
    d = "kmer-join-smoke-v0"
    ix = rows(REF / d / "index.tsv")
    q = rows(REF / d / "queries.tsv")
    rep = [int(r[0]) for r in rows(REF / d / "repetitive-kmers.tsv")]
    idx = O.Index.from_entries(4, [int(r[1]) for r in ix], [int(r[2]) for r in ix],
                               [int(r[0]) for r in ix], rep)
    m = O.candidates_windows(idx, [int(r[0]) for r in q], [int(r[1]) for r in q],
                             [int(r[2]) for r in q], [int(r[3]) for r in q])
    assert as_records(m) == expected(d)


def test_kmer_encode_fixture(oracle_mod):
    O = oracle_mod
    d = "kmer-encode-smoke-v0"
    ix = rows(REF / d / "index.tsv")
    q = rows(REF / d / "queries.tsv")
    rep = [std(enc(r[0]), 4) for r in rows(REF / d / "repetitive-kmers.tsv")]
    idx = O.Index.from_entries(4, [int(r[0]) for r in ix], [int(r[1]) for r in ix],
                               [std(enc(r[3]), 4) for r in ix], rep)
    m = O.candidates_windows(idx, [int(r[0]) for r in q], [int(r[1]) for r in q],
                             [enc(r[2]) for r in q], [std(enc(r[2]), 4) for r in q])
    assert as_records(m) == expected(d)


def test_read_window_fixture(oracle_mod):
    O = oracle_mod
    d = "read-window-smoke-v0"
    ix = rows(REF / d / "index.tsv")
    rd = rows(REF / d / "reads.tsv")
    rep = [std(enc(r[0]), 4) for r in rows(REF / d / "repetitive-kmers.tsv")]
    idx = O.Index.from_entries(4, [int(r[0]) for r in ix], [int(r[1]) for r in ix],
                               [std(enc(r[3]), 4) for r in ix], rep)
    m = O.candidates(idx, O.SeqBatch.from_strings([int(r[0]) for r in rd], [r[1] for r in rd]))
    assert as_records(m) == expected(d)
    # TTCA (repetitive) sits at position 15 of read 1
    assert list(zip(m["filtered_query"].tolist(), m["filtered_pos"].tolist())) == [(1, 15)]


def test_read_alignment_fixture(oracle_mod):
    """tests/fixtures/read-alignment-replay-fixture-v0/simple: 2 inputs -> 2
    candidate chains; the accepted one is [0, 1] (the fixture's oracle TSV)."""
    O = oracle_mod
    d = REF / "read-alignment-replay-fixture-v0" / "simple"
    man = json.loads((d / "manifest.json").read_text())
    eo = rows(d / "edge-overlaps.tsv")
    arr = np.array([[int(r[2]), int(r[3]), int(r[9]), int(r[10]), int(r[11]), int(r[12])]
                    for r in eo])
    r2g = O.default_r2g(max_jump=man["maximum_jump"], max_read_overlap=man["max_read_overlap"],
                        min_overlap=man["minimum_overlap"], max_separation=man["max_separation"])
    chains = O.chain_read_alignments(arr, [int(r[6]) for r in eo], [int(r[7]) for r in eo], r2g)
    assert len(chains) == man["candidate_chains"]
    flags = [int(r[2]) for r in rows(d / "chain-divergence.tsv")]
    accepted = [c for c, f in zip(chains, flags) if f]
    assert len(accepted) == man["oracle_chains"]
    oracle_rows = rows(d / "oracle.read-alignment.tsv")
    got = [(ci, si, eo[idx][1]) for ci, c in enumerate(accepted) for si, idx in enumerate(c)]
    assert [(int(r[0]), int(r[1]), r[2]) for r in oracle_rows] == got


@pytest.mark.parametrize("case", ["ovl-a", "ovl-d"])
def test_synthetic_candidates_sha(oracle_mod, golden_cases, case):
    """Candidate multiset of the committed synthetic cases (canonical SHA-256)."""
    O = oracle_mod
    reads, meta, _ = golden_cases[case]
    b = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    idx = O.Index.build(meta["k"], b, meta["min_freq"], meta["max_freq"])
    m = O.candidates(idx, b)
    assert len(m["query_id"]) == meta["candidate_records"]
    text = "".join(f"{a}\t{p}\t{km}\t{t}\t{tp}\t{'+' if t > 0 else '-'}\n"
                   for a, p, km, t, tp in sorted(zip(m["query_id"].tolist(),
                                                     m["query_pos"].tolist(),
                                                     m["kmer"].tolist(),
                                                     m["target_id"].tolist(),
                                                     m["target_pos"].tolist())))
    assert hashlib.sha256(text.encode()).hexdigest() == meta["candidate_canonical_sha256"]


@pytest.mark.parametrize("case", ["ovl-a", "ovl-d"])
def test_synthetic_overlaps_vs_reference_tools(oracle_mod, golden_cases, case):
    """Oracle chaining reproduces tools/replay_overlap_chains.py (stable sorts)
    and tools/replay_read_to_graph_source_pack.py (libstdc++ sort emulation)."""
    O = oracle_mod
    reads, meta, d = golden_cases[case]
    b = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    idx = O.Index.build(meta["k"], b, meta["min_freq"], meta["max_freq"])
    # libstdc++ mode, replay_group parameters (no overhang check, all primaries)
    p = O.default_params(**dict(meta["params"], check_overhang=0, only_max_ext=0,
                                max_overhang=0))
    got = []
    for i in range(reads.n):
        one = O.SeqBatch.from_strings([int(reads.ids[i])], [reads.seq(i)])
        r = O.overlaps(idx, one, p)
        got += ["\t".join(str(int(v)) for v in row) for row in r["cols"]]
    assert got == (d / "ref.overlaps.libstdcxx.tsv").read_text().splitlines()
    # stable mode against replay_overlap_chains.py, including divergence text
    from cuflye_gb300.abi import format_float
    srt = O.candidates(idx, b, sorted_like_flye=True)
    gen = O.candidates(idx, b)
    lens = {int(reads.ids[i]): int(reads.offsets[i + 1] - reads.offsets[i])
            for i in range(reads.n)}
    O.set_stable(True)
    try:
        got = []
        for i in range(reads.n):
            q = int(reads.ids[i])
            sel = srt["query_id"] == q
            f = gen["filtered_pos"][gen["filtered_query"] == q]
            r = O.chain_sorted(srt["query_pos"][sel], srt["target_pos"][sel],
                               srt["target_id"][sel], q, lens[q], list(lens), list(lens.values()),
                               f, O.default_params(**meta["params"]))
            got += ["\t".join(str(int(v)) for v in row) + "\t" + format_float(dv)
                    for row, dv in zip(r["cols"], r["divergence"])]
    finally:
        O.set_stable(False)
    assert got == (d / "ref.overlaps.stable.tsv").read_text().splitlines()


def test_oracle_std_sort_matches_reference_emulation(oracle_mod):
    """libstdc++ std::sort tie order: the oracle calls std::sort itself; the
    reference restates it in Python (cpp_sort_in_place), whose orders for
    seeded key sets with heavy ties are the committed fixture
    (tests/golden/make_sort_ties.py)."""
    import json
    from conftest import GOLDEN
    fx = json.loads((GOLDEN / "sort_ties.json").read_text())
    for case in fx["cases"]:
        keys = np.array(case["keys"], dtype=np.uint64)
        vals = np.arange(len(keys), dtype=np.uint32)
        _, v2 = oracle_mod.std_sort_u64(keys, vals)
        assert v2.tolist() == case["values_after_sort"], len(keys)
