"""GPU: read-alignment chains before and after the divergence filter.

* The reference's read-alignment replay fixture
  (tests/fixtures/read-alignment-replay-fixture-v0/simple, copied under
  tests/golden/reference): chained on the device through
  cuflye_chain_read_alignments, its candidate chains carry the fixture's
  chain divergences (chain-divergence.tsv), the accept test gives the
  fixture's flags, and the kept chain's rows are oracle.read-alignment.tsv.
* Synthetic replay fixtures: the device's candidate chains equal the CPU
  oracle's chainReadAlignments, segment for segment, and the k-mer form of
  the chain divergence equals the oracle's float arithmetic bit for bit.
* In-process reads (cuflye_read_to_graph_chains): each chain record agrees
  with the quickSeqOverlaps row it names (candidate id), and the chains the
  k-mer divergence keeps, with their complements, are cuflye_read_to_graph's
  rows.  The payload written from them reads back intact.
"""

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_vs_reference_cpu import _edge_alignments

pytestmark = pytest.mark.gpu

FIX = GOLDEN / "reference" / "read-alignment-replay-fixture-v0" / "simple"


def _rows(path):
    return [l.rstrip("\n").split("\t") for l in open(path) if l.strip()]


def _fixture_overlaps(path):
    from cuflye_gb300 import abi
    rows = _rows(path)
    out = np.zeros(len(rows), dtype=abi.EDGE_OVERLAP_DTYPE)
    for i, r in enumerate(rows):
        out[i] = (int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[6]), int(r[7]),
                  int(r[9]), int(r[10]), int(r[11]), int(r[5]), int(r[8]), int(r[12]),
                  np.float32(float(r[13])))
    return out


def test_reference_replay_fixture(gpu):
    import json
    from cuflye_gb300 import abi
    from cuflye_gb300.backend import R2GParams
    man = json.loads((FIX / "manifest.json").read_text())
    r2g = R2GParams.make(max_jump=man["maximum_jump"], max_read_overlap=man["max_read_overlap"],
                         min_overlap=man["minimum_overlap"],
                         max_separation=man["max_separation"],
                         max_chain_divergence=man["read_align_ovlp_divergence"])
    ov = _fixture_overlaps(FIX / "edge-overlaps.tsv")
    div = [(float(r[1]), r[2] == "1") for r in _rows(FIX / "chain-divergence.tsv")]
    got = gpu.chain_read_alignments([ov], [man["query_id"]], r2g,
                                    chain_divergences=[d for d, _ in div])
    assert len(got["divergence"]) == man["candidate_chains"] == len(div)
    assert list(got["kept"]) == [k for _, k in div]
    assert int(got["kept"].sum()) == man["oracle_chains"]
    # the kept chain's rows (before its complement) are the fixture's oracle rows
    want = [l.rstrip("\n") for l in open(FIX / "oracle.read-alignment.tsv") if l.strip()]
    lines = [l.rstrip("\n") for l in abi.read_alignment_lines(got["rows"])]
    # the fixture prints the float as 0.01, C++ setprecision(9) as 0.00999999978
    norm = lambda l: l.split("\t")[:12] + [str(np.float32(float(l.split("\t")[12])))]
    assert [norm(l) for l in lines[:len(want)]] == [norm(l) for l in want]
    # its complement follows: reversed segments, negated ids
    comp = got["rows"][len(want):]
    assert len(comp) == len(want)
    assert list(comp["read_id"]) == [-int(r.split("\t")[2]) for r in reversed(want)]
    # candidate chains as records: chain 0 holds both overlaps, chain 1 the first
    rec = got["records"]
    assert [(int(r["chain_id"]), int(r["segment_id"]), int(r["overlap_index"])) for r in rec] == \
        [(0, 0, 0), (0, 1, 1), (1, 0, 0)]
    assert list(rec["candidate_id"]) == [0, 1, 0]
    assert all(int(q) == man["query_id"] for q in rec["query_id"])


def _synthetic_fixtures(seed, count):
    from cuflye_gb300 import abi
    rng = np.random.default_rng(seed)
    fx, raw = [], []
    for f in range(count):
        rows = _edge_alignments(rng, int(rng.integers(4, 60)))
        read_len = max(r[1] for r in rows) + int(rng.integers(0, 500))
        arr = np.zeros(len(rows), dtype=abi.EDGE_OVERLAP_DTYPE)
        for i, r in enumerate(rows):
            arr[i] = (50_000 + i, 7, r[0], r[1], read_len, r[5], r[6], r[2], r[3], r[4], r[9],
                      r[9] + 5000, r[7], np.float32(r[8]))
        fx.append(arr)
        raw.append(rows)
    return fx, raw


def _kmer_divergence(arr, chain):
    s, t = np.float32(0), np.float32(0)
    for i in chain:
        rr = np.float32(int(arr[i]["read_end"]) - int(arr[i]["read_begin"]))
        s = np.float32(s + np.float32(arr[i]["seq_divergence"] * rr))
        t = np.float32(t + rr)
    return np.float32(s / t)


def test_replay_chains_match_oracle(gpu, oracle_mod):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import R2GParams
    p = synth.R2G_PARAMS
    r2g = R2GParams.make(**p)
    ocfg = oracle_mod.default_r2g(max_jump=p["max_jump"], max_read_overlap=p["max_read_overlap"],
                                  min_overlap=p["min_overlap"],
                                  max_separation=p["max_separation"])
    fx, raw = _synthetic_fixtures(51, 60)
    got = gpu.chain_read_alignments(fx, list(range(100, 100 + len(fx))), r2g)
    rec = got["records"]
    k = 0
    chains_seen = 0
    for f, (arr, rows) in enumerate(zip(fx, raw)):
        m = np.array([[r[0], r[1], r[2], r[3], r[4], r[7]] for r in rows])
        want = oracle_mod.chain_read_alignments(m, [r[5] for r in rows], [r[6] for r in rows],
                                                ocfg)
        mine = rec[rec["query_id"] == 100 + f]
        chains: list[list[int]] = []
        for r in mine:
            while len(chains) <= int(r["chain_id"]):
                chains.append([])
            assert int(r["segment_id"]) == len(chains[int(r["chain_id"])])
            chains[int(r["chain_id"])].append(int(r["overlap_index"]))
        assert chains == want, f
        for c in want:
            d = _kmer_divergence(arr, c)
            assert np.float32(got["divergence"][k]).view(np.uint32) == d.view(np.uint32)
            assert bool(got["kept"][k]) == bool(d < np.float32(p["max_chain_divergence"]))
            k += 1
        chains_seen += len(want)
    assert k == len(got["divergence"]) and chains_seen >= 60
    # records carry the overlap they name
    flat = np.concatenate(fx)
    offs = np.concatenate([[0], np.cumsum([len(a) for a in fx])])
    for r in rec[:200]:
        f = int(r["query_id"]) - 100
        o = flat[offs[f] + int(r["overlap_index"])]
        assert int(r["candidate_id"]) == int(o["candidate_id"])
        assert (int(r["read_begin"]), int(r["edge_end"]), int(r["edge_left"])) == \
            (int(o["read_begin"]), int(o["edge_end"]), int(o["edge_left"]))


def test_replay_rejects_a_wrong_divergence_count(gpu):
    from cuflye_gb300.backend import CuflyeError, R2GParams
    fx, _ = _synthetic_fixtures(52, 3)
    with pytest.raises(CuflyeError, match="chain divergences"):
        gpu.chain_read_alignments(fx, [1, 2, 3], R2GParams.make(), chain_divergences=[0.1])


def test_in_process_chains_agree_with_read_to_graph(gpu):
    from cuflye_gb300 import abi, synth
    from cuflye_gb300.backend import OverlapParams, R2GParams, compact_binary
    wl = synth.read_to_graph(seed=3, genome_len=400_000, n_edges=24, coverage=4.0)
    g = wl.graph
    gpu.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
    gpu.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
    p, r2g = OverlapParams.make(**wl.params), R2GParams.make(**synth.R2G_PARAMS)
    rows = gpu.read_to_graph(wl.reads, p, r2g)
    rec, inputs = gpu.read_to_graph_chains(wl.reads, p, r2g)
    assert len(rec) > 0 and len(inputs) == wl.reads.n
    # the k-mer divergence filter over the candidate chains, then complements
    kept, comp = [], []
    chain_base = 0
    for q in range(wl.reads.n):
        mine = rec[rec["query_id"] == wl.reads.ids[q]]
        chains: dict[int, list] = {}
        for r in mine:
            chains.setdefault(int(r["chain_id"]), []).append(r)
        good = []
        for c in sorted(chains):
            segs = chains[c]
            s, t = np.float32(0), np.float32(0)
            for r in segs:
                rr = np.float32(int(r["read_end"]) - int(r["read_begin"]))
                s = np.float32(s + np.float32(r["seq_divergence"] * rr))
                t = np.float32(t + rr)
            if np.float32(s / t) < np.float32(r2g.max_chain_divergence):
                good.append(segs)
        for i, segs in enumerate(good):
            for j, r in enumerate(segs):
                kept.append((chain_base + i, j, int(r["read_id"]), int(r["read_begin"]),
                             int(r["read_end"]), int(r["edge_id"]), int(r["edge_seq_id"])))
        for i, segs in enumerate(good):
            for j, r in enumerate(reversed(segs)):
                kept.append((chain_base + len(good) + i, j, -int(r["read_id"]),
                             int(r["read_len"]) - int(r["read_end"]) - 1,
                             int(r["read_len"]) - int(r["read_begin"]) - 1, -int(r["edge_id"]),
                             -int(r["edge_seq_id"])))
        chain_base += 2 * len(good)
    got = [(int(r["chain_id"]), int(r["segment_id"]), int(r["read_id"]), int(r["read_begin"]),
            int(r["read_end"]), int(r["edge_id"]), int(r["edge_seq_id"])) for r in rows]
    assert got == kept
    # candidate ids index the read's quickSeqOverlaps rows before the filter
    ovl = gpu.overlaps(wl.reads, p)
    for q in range(min(wl.reads.n, 40)):
        qo = ovl[ovl["cur_id"] == wl.reads.ids[q]]
        for r in rec[rec["query_id"] == wl.reads.ids[q]]:
            o = qo[int(r["candidate_id"])]
            assert (int(o["cur_begin"]), int(o["cur_end"]), int(o["ext_begin"]),
                    int(o["ext_end"]), int(o["score"])) == \
                (int(r["read_begin"]), int(r["read_end"]), int(r["edge_begin"]),
                 int(r["edge_end"]), int(r["score"]))
            assert abs(int(o["ext_id"])) == abs(int(r["edge_seq_id"]))
    data = compact_binary(rec, inputs)
    head, back = abi.read_compact_binary(data)
    assert head["records"] == len(rec) and head["fixtures"] == wl.reads.n
    assert head["total_inputs"] == int(inputs.sum())
    assert np.array_equal(back["candidate_id"], rec["candidate_id"])
    assert np.array_equal(back["seq_divergence"].view(np.uint32),
                          rec["seq_divergence"].view(np.uint32))
