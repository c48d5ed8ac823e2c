"""GPU parity: the CUDA library, called through the C ABI, against the CPU
oracle on the same seeded inputs (bit-exact: integer fields and the float
divergence bits), and against the committed golden vectors."""

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

REF = GOLDEN / "reference"


def _std4(s):
    m = {"A": 0, "C": 1, "G": 2, "T": 3}
    x = 0
    for c in s:
        x = (x << 2) + m[c]
    r, y = 0, x
    for _ in range(4):
        r = (r << 2) + ((~y) & 3)
        y >>= 2
    return min(x, r)


def _rows(path):
    return [l.rstrip("\n").split("\t") for l in open(path) if l.strip()]


def oracle_index(O, reads, k, min_freq, max_freq):
    b = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    return O.Index.build(k, b, min_freq, max_freq), b


def cand_tuples_gpu(rec):
    return list(zip(rec["query_id"].tolist(), rec["query_pos"].tolist(), rec["kmer"].tolist(),
                    rec["target_id"].tolist(), rec["target_pos"].tolist()))


def cand_tuples_oracle(m):
    return list(zip(m["query_id"].tolist(), m["query_pos"].tolist(), m["kmer"].tolist(),
                    m["target_id"].tolist(), m["target_pos"].tolist()))


def overlap_tuples_gpu(rec):
    return [(int(r["cur_id"]), int(r["cur_begin"]), int(r["cur_end"]), int(r["cur_len"]),
             int(r["ext_id"]), int(r["ext_begin"]), int(r["ext_end"]), int(r["ext_len"]),
             int(r["score"]), np.float32(r["seq_divergence"]).view(np.uint32).item())
            for r in rec]


def overlap_tuples_oracle(r):
    return [tuple(int(v) for v in row) + (np.float32(dv).view(np.uint32).item(),)
            for row, dv in zip(r["cols"], r["divergence"])]


def test_read_window_fixture_gpu(gpu):
    """tests/fixtures/read-window-smoke-v0 through the device path."""
    from cuflye_gb300 import synth
    d = REF / "read-window-smoke-v0"
    ix = _rows(d / "index.tsv")
    rd = _rows(d / "reads.tsv")
    rep = [_std4(r[0]) for r in _rows(d / "repetitive-kmers.tsv")]
    gpu.index_from_entries(4, [int(r[0]) for r in ix], [int(r[1]) for r in ix],
                           [_std4(r[3]) for r in ix], rep)
    reads = synth.ReadSet.from_strings([int(r[0]) for r in rd], [r[1] for r in rd])
    cand, filt = gpu.candidates(reads)
    got = sorted((a, b, c, d_, e, "+" if d_ > 0 else "-") for a, b, c, d_, e in
                 cand_tuples_gpu(cand))
    exp = sorted((int(a), int(b), int(c), int(e), int(f), g)
                 for a, b, c, e, f, g in _rows(d / "expected.candidates.tsv"))
    assert got == exp
    assert list(zip(filt["query_id"].tolist(), filt["pos"].tolist())) == [(1, 15)]


@pytest.mark.parametrize("case", ["ovl-a", "ovl-b", "ovl-c", "ovl-d"])
def test_candidates_match_oracle(gpu, oracle_mod, golden_cases, case):
    reads, meta, _ = golden_cases[case]
    idx, b = oracle_index(oracle_mod, reads, meta["k"], meta["min_freq"], meta["max_freq"])
    st = gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    assert st["positions"] == idx.n_positions
    cand, filt = gpu.candidates(reads)
    m = oracle_mod.candidates(idx, b)
    assert len(cand) == meta["candidate_records"]
    assert cand_tuples_gpu(cand) == cand_tuples_oracle(m)  # generation order, exactly
    assert filt["query_id"].tolist() == m["filtered_query"].tolist()
    assert filt["pos"].tolist() == m["filtered_pos"].tolist()


@pytest.mark.parametrize("case", ["ovl-a", "ovl-b", "ovl-c", "ovl-d"])
def test_overlaps_match_oracle(gpu, oracle_mod, golden_cases, case):
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases[case]
    idx, b = oracle_index(oracle_mod, reads, meta["k"], meta["min_freq"], meta["max_freq"])
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    for variant in ({}, {"only_max_ext": 0}, {"only_max_ext": 0, "check_overhang": 0},
                    {"max_overlaps": 3}):
        params = dict(meta["params"], **variant)
        got = gpu.overlaps(reads, OverlapParams.make(**params))
        exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**params))
        assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp), variant


@pytest.mark.parametrize("seed", [11, 12])
def test_equal_keys_take_the_libstdcxx_paths(gpu, oracle_mod, seed):
    """Tandem arrays put equal keys at every sort point: queries whose KmerMatch
    keys repeat, ext-sorted groups with equal ext positions and groups whose
    backtrack depends on Flye's order among equal scores.  Those take the
    libstdc++-order paths, the rest the plain sorts, and the rows still match
    the oracle bit for bit."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    oracle_mod.set_stable(False)
    wl = synth.tandem_case(seed)
    idx, b = oracle_index(oracle_mod, wl.reads, wl.k, wl.min_freq, wl.max_freq)
    gpu.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
    seen = dict.fromkeys(gpu.SORT_STATS, 0)
    for variant in ({}, {"only_max_ext": 0}, {"only_max_ext": 0, "check_overhang": 0}):
        params = dict(wl.params, **variant)
        got = gpu.overlaps(wl.reads, OverlapParams.make(**params))
        for key, v in gpu.last_sort_stats().items():
            seen[key] += v
        exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**params))
        assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp), variant
    for key in ("match_plain", "match_libstdcxx", "ext_plain", "ext_libstdcxx", "score_plain",
                "backtrack_redo"):
        assert seen[key] > 0, seen


def test_long_reads_against_long_targets(gpu, oracle_mod):
    """Reads of up to 100 kb against 1 Mb target pieces with interspersed
    repeats: a read's group on its own piece holds tens of thousands of hits,
    out of ext-pos order (repeat and random hits), which takes the device-scratch
    ext re-sort, or the heap ranges of the emulated introsort where ext
    positions repeat; singletons and short chains tie on score in every group.
    Rows bit-exact with the oracle."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    oracle_mod.set_stable(False)
    sw = synth.serving_workload(seed=5, genome_len=2_000_000, n_queries=60)
    lens = np.diff(sw.queries.offsets)
    q = sw.queries.subset(np.sort(np.argsort(lens)[-8:]))
    assert int(np.diff(q.offsets).min()) > 40_000
    idx, _ = oracle_index(oracle_mod, sw.targets, sw.k, sw.min_freq, sw.max_freq)
    gpu.build_index(sw.targets, sw.k, sw.min_freq, sw.max_freq)
    b = oracle_mod.SeqBatch(q.ids, q.offsets, q.bases.tobytes())
    for variant in ({}, {"only_max_ext": 1}):
        params = dict(sw.params, **variant)
        got = gpu.overlaps(q, OverlapParams.make(**params))
        exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**params))
        assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp), variant
        assert len(got) > 0
        assert gpu.last_sort_stats()["ext_plain"] > 0


@pytest.mark.parametrize("case", ["ovl-a", "ovl-d"])
def test_overlaps_match_reference_tool_output(gpu, golden_cases, case):
    """Against tools/replay_read_to_graph_source_pack.py's rows (committed)."""
    from cuflye_gb300.backend import OverlapParams
    reads, meta, d = golden_cases[case]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    params = dict(meta["params"], check_overhang=0, only_max_ext=0, max_overhang=0)
    got = gpu.overlaps(reads, OverlapParams.make(**params))
    lines = ["\t".join(str(v) for v in t[:9]) for t in overlap_tuples_gpu(got)]
    assert lines == (d / "ref.overlaps.libstdcxx.tsv").read_text().splitlines()


def test_plain_path_equals_batched(gpu, golden_cases):
    """One read per launch gives the same rows as one batch."""
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    p = OverlapParams.make(**meta["params"])
    gpu.set_batch_queries(0)
    batched = gpu.overlaps(reads, p)
    gpu.set_batch_queries(1)
    try:
        plain = gpu.overlaps(reads, p)
    finally:
        gpu.set_batch_queries(0)
    assert overlap_tuples_gpu(plain) == overlap_tuples_gpu(batched)


@pytest.mark.parametrize("n,key_range", [(5, 2), (16, 3), (17, 2), (100, 4), (5000, 7),
                                         (8192, 50), (8193, 3), (60_000, 1000),
                                         (300_000, 20), (300_000, 1 << 40)])
def test_std_sort_segments_match_libstdcxx(gpu, oracle_mod, n, key_range):
    rng = np.random.default_rng(n + key_range)
    keys = rng.integers(0, key_range, size=n, dtype=np.uint64)
    vals = np.arange(n, dtype=np.uint32)
    k2, v2 = gpu.std_sort_segments(keys, vals, [0, n])
    ek, ev = oracle_mod.std_sort_u64(keys, vals)
    assert np.array_equal(k2, ek)
    assert np.array_equal(v2, ev)


def test_std_sort_many_segments(gpu, oracle_mod):
    rng = np.random.default_rng(11)
    sizes = rng.integers(0, 3000, size=300)
    sizes[::37] = rng.integers(9000, 40000, size=len(sizes[::37]))
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(offs[-1])
    keys = rng.integers(0, 64, size=n, dtype=np.uint64)
    vals = rng.integers(0, 1 << 31, size=n, dtype=np.uint32)
    k2, v2 = gpu.std_sort_segments(keys, vals, offs)
    for s in range(len(sizes)):
        a, b = int(offs[s]), int(offs[s + 1])
        ek, ev = oracle_mod.std_sort_u64(keys[a:b], vals[a:b])
        assert np.array_equal(k2[a:b], ek) and np.array_equal(v2[a:b], ev), s


@pytest.mark.parametrize("n,scale", [(20_000, 1), (200_000, 1), (200_000, 1 << 41),
                                     (300_000, 1), (400_000, 1), (400_000, 1 << 41)])
def test_heap_fallback_ranges_match_libstdcxx(gpu, oracle_mod, n, scale):
    """Organ-pipe keys (every value twice) drive libstdc++'s introsort into
    heapsort on ranges of 4k-95k elements: n = 200,000 gives heap ranges of
    47,105, 42,183, 21,505 and 12,089 elements (one block's shared memory),
    n = 300,000 one of 95,233 and n = 400,000 ones of 95,233 and 84,615 (a
    block pair's).  The heap's order among equal keys must match; keys spanning
    more than 47 bits (scale 2**41) take the 12-byte heap in shared memory or
    the one in device memory instead of the rank-packed ones.
    n = 20,000 spends its recursion budget inside a block-wide partition of a
    shared-memory task, leaving leaves of 12 and 16 elements at depth 0 that
    libstdc++ insertion-sorts rather than heap-sorts."""
    i = np.arange(n, dtype=np.uint64)
    keys = np.where(i < n // 2, i, n - i).astype(np.uint64) * np.uint64(scale)
    vals = np.random.default_rng(n).permutation(n).astype(np.uint32)
    k2, v2 = gpu.std_sort_segments(keys, vals, [0, n])
    ek, ev = oracle_mod.std_sort_u64(keys, vals)
    assert np.array_equal(k2, ek)
    assert np.array_equal(v2, ev)


def test_sorted_and_presorted_inputs(gpu, oracle_mod):
    for keys in (np.arange(20000, dtype=np.uint64), np.arange(20000, 0, -1).astype(np.uint64),
                 np.zeros(20000, dtype=np.uint64),
                 np.tile(np.array([1, 0], dtype=np.uint64), 10000)):
        vals = np.arange(len(keys), dtype=np.uint32)
        k2, v2 = gpu.std_sort_segments(keys, vals, [0, len(keys)])
        ek, ev = oracle_mod.std_sort_u64(keys, vals)
        assert np.array_equal(v2, ev)


# ---------------------------------------------------------------- edge cases

def test_empty_and_short_queries(gpu, golden_cases):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    empty = synth.ReadSet.from_strings([], [])
    cand, filt = gpu.candidates(empty)
    assert len(cand) == 0 and len(filt) == 0
    short = synth.ReadSet.from_strings([900001, 900002], ["ACGT", ""])
    cand, filt = gpu.candidates(short)
    assert len(cand) == 0
    assert len(gpu.overlaps(short, OverlapParams.make(**meta["params"]))) == 0


def test_param_and_budget_errors(built_lib, golden_cases):
    from cuflye_gb300.backend import CudaBackend, CuflyeError, OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    with CudaBackend(device=0, memory_budget_bytes=0) as b:
        with pytest.raises(CuflyeError, match="NO_INDEX"):
            b.overlaps(reads, OverlapParams.make(**meta["params"]))
        b.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
        with pytest.raises(CuflyeError, match="kmer_size"):
            b.overlaps(reads, OverlapParams.make(**dict(meta["params"], kmer_size=meta["k"] + 2)))
        with pytest.raises(CuflyeError, match="UNSUPPORTED"):
            b.build_index(reads, 32, 2, 100)
    with pytest.raises(CuflyeError, match="BUDGET"):
        with CudaBackend(device=0, memory_budget_bytes=4 << 20) as b:
            b.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
            b.overlaps(reads, OverlapParams.make(**meta["params"]))


def test_determinism(gpu, golden_cases):
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases["ovl-b"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    p = OverlapParams.make(**meta["params"])
    a = gpu.overlaps(reads, p)
    b = gpu.overlaps(reads, p)
    assert a.tobytes() == b.tobytes()


def test_queries_that_differ_from_their_indexed_read(gpu, oracle_mod, golden_cases):
    """Queries under indexed ids whose sequences differ from the indexed ones
    (mutated copies, and one reverse complement under the negated id): hit
    counting cannot use the index's record of each indexed window's own
    entry for them, and must find the query's own entries (where they exist)
    as for any query.  Candidates and overlaps against the oracle."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    idx, _ = oracle_index(oracle_mod, reads, meta["k"], meta["min_freq"], meta["max_freq"])
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    rng = np.random.default_rng(23)
    ids, seqs = [], []
    for i in range(0, min(reads.n, 60), 3):
        s = np.frombuffer(reads.seq(i), dtype=np.uint8)
        ids.append(int(reads.ids[i]))
        seqs.append(synth.mutate(rng, s, 0.01, 0.002, 0.002).tobytes())
    ids.append(-int(reads.ids[1]))
    seqs.append(synth.revcomp(np.frombuffer(reads.seq(1), dtype=np.uint8)).tobytes())
    q = synth.ReadSet.from_strings(np.array(ids, dtype=np.int64), seqs)
    qb = oracle_mod.SeqBatch(q.ids, q.offsets, q.bases.tobytes())
    rec, filt = gpu.candidates(q)
    exp = oracle_mod.candidates(idx, qb)
    assert cand_tuples_gpu(rec) == cand_tuples_oracle(exp)  # generation order, exactly
    assert filt["pos"].tolist() == exp["filtered_pos"].tolist()
    params = OverlapParams.make(**meta["params"])
    oracle_mod.set_stable(False)
    got = overlap_tuples_gpu(gpu.overlaps(q, params))
    exp = oracle_mod.overlaps(idx, qb, oracle_mod.default_params(**meta["params"]))
    assert got == overlap_tuples_oracle(exp)
