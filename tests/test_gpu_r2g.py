"""GPU parity of the read-to-graph chains (read-alignment-v1 rows) against the
CPU oracle: quickSeqOverlaps against the edge index, the LONG_EDGE / BIG_ALN
filter, the curBegin sort, chainReadAlignments, the chain divergence filter
and the complement chains, on a small seeded graph."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_graph_case(seed=3):
    from cuflye_gb300 import synth
    return synth.read_to_graph(seed=seed, genome_len=400_000, n_edges=24, coverage=4.0)


def rows_gpu(rec):
    return [(int(r["chain_id"]), int(r["segment_id"]), int(r["read_id"]), int(r["read_begin"]),
             int(r["read_end"]), int(r["read_len"]), int(r["edge_id"]), int(r["edge_seq_id"]),
             int(r["edge_begin"]), int(r["edge_end"]), int(r["edge_len"]), int(r["score"]),
             np.float32(r["seq_divergence"]).view(np.uint32).item()) for r in rec]


def rows_oracle(res):
    return [tuple(int(v) for v in row) + (np.float32(d).view(np.uint32).item(),)
            for row, d in zip(res["cols"], res["divergence"])]


@pytest.mark.parametrize("r2g_over", [{}, {"min_overlap": 100, "max_chain_divergence": 1.0}])
def test_read_to_graph_matches_oracle(gpu, oracle_mod, r2g_over):
    from cuflye_gb300.backend import OverlapParams, R2GParams
    O = oracle_mod
    wl = small_graph_case()
    g = wl.graph
    es = g.seqs
    gpu.build_index(es, wl.k, wl.min_freq, wl.max_freq)
    gpu.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
    r2g = dict(R2G_DEFAULTS, **r2g_over)
    got = gpu.read_to_graph(wl.reads, OverlapParams.make(**wl.params), R2GParams.make(**r2g))
    eb = O.SeqBatch(es.ids, es.offsets, es.bases.tobytes())
    idx = O.Index.build(wl.k, eb, wl.min_freq, wl.max_freq)
    rb = O.SeqBatch(wl.reads.ids, wl.reads.offsets, wl.reads.bases.tobytes())
    exp = O.read_to_graph(idx, g.edge_ids, g.seq_ids, g.left, g.right, rb,
                          O.default_params(**wl.params), O.default_r2g(**r2g))
    assert len(exp["cols"]) > 0
    assert rows_gpu(got) == rows_oracle(exp)


R2G_DEFAULTS = dict(max_jump=1500, max_read_overlap=50, min_overlap=1000, max_separation=500,
                    long_edge=900, big_aln=500, max_chain_divergence=0.25)


def test_read_to_graph_complement_rows_mirror(gpu):
    """Every good chain is followed (after all good chains of the read) by its
    complement: reversed segments, negated ids, mirrored coordinates."""
    from cuflye_gb300.backend import OverlapParams, R2GParams
    wl = small_graph_case()
    g = wl.graph
    gpu.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
    gpu.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
    rec = gpu.read_to_graph(wl.reads, OverlapParams.make(**wl.params),
                            R2GParams.make(**R2G_DEFAULTS))
    by_read = {}
    for r in rec:
        by_read.setdefault(int(abs(r["read_id"])), []).append(r)
    checked = 0
    for rows in by_read.values():
        chains = {}
        for r in rows:
            chains.setdefault(int(r["chain_id"]), []).append(r)
        ids = sorted(chains)
        half = len(ids) // 2
        for a, b in zip(ids[:half], ids[half:]):
            fwd, rev = chains[a], chains[b]
            assert len(fwd) == len(rev)
            for x, y in zip(fwd, reversed(rev)):
                assert y["read_id"] == -x["read_id"] and y["edge_id"] == -x["edge_id"]
                assert y["read_begin"] == x["read_len"] - x["read_end"] - 1
                assert y["edge_end"] == x["edge_len"] - x["edge_begin"] - 1
            checked += 1
    assert checked > 0
