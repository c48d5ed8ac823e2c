"""The scale configuration's path, scaled down: ONT-like reads with 6 % error
over a repeat-bearing genome, streamed through the device in passes.  Rows
are a property of the reads alone, so they must not depend on how a call is
cut into passes, whether by a query count or by the memory budget; a sample
of the longest reads is checked against the oracle bit for bit."""

import numpy as np
import pytest

from test_gpu_parity import oracle_index, overlap_tuples_gpu, overlap_tuples_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scale_case():
    from cuflye_gb300 import synth
    return synth.scale_ont(seed=6, genome_len=3_000_000, coverage=8.0)


def test_passes_do_not_change_rows(built_lib, scale_case):
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    wl = scale_case
    p = OverlapParams.make(**wl.params)
    nwin = int(np.maximum(np.diff(wl.reads.offsets) - wl.k + 1, 0).sum())
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        # the index laid out as a budget-bound build lays it out (key ranges)
        be.set_index_build_windows(nwin // 4 + 1)
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        index_bytes = be.memory_stats()[0]
        whole = be.overlaps(wl.reads, p)
        assert be.last_passes() == 1
        hits = be.last_timing()[1][1] // 24
        be.set_batch_queries(97)
        by_count = be.overlaps(wl.reads, p)
        assert be.last_passes() == -(-wl.reads.n // 97)
        be.set_batch_queries(0)
    assert len(whole) > 0 and hits > 0
    assert by_count.tobytes() == whole.tobytes()
    # a budget that holds the index and about a sixth of the hits' buffers:
    # the index is built in key ranges and the overlaps run in passes
    budget = int(index_bytes + 64 * hits / 6 + (64 << 20))
    with CudaBackend(device=0, memory_budget_bytes=budget) as be:
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() >= 2
        by_budget = be.overlaps(wl.reads, p)
        assert be.last_passes() >= 3
        peak = be.memory_stats()[1]
    assert peak <= budget
    assert by_budget.tobytes() == whole.tobytes()


def test_long_ont_reads_match_oracle(gpu, oracle_mod, scale_case):
    from cuflye_gb300.backend import OverlapParams
    wl = scale_case
    oracle_mod.set_stable(False)
    idx, _ = oracle_index(oracle_mod, wl.reads, wl.k, wl.min_freq, wl.max_freq)
    gpu.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
    lens = np.diff(wl.reads.offsets)
    q = wl.reads.subset(np.sort(np.argsort(lens)[-12:]))
    b = oracle_mod.SeqBatch(q.ids, q.offsets, q.bases.tobytes())
    for variant in ({}, {"only_max_ext": 0}):
        params = dict(wl.params, **variant)
        got = gpu.overlaps(q, OverlapParams.make(**params))
        exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**params))
        assert len(got) > 0
        assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp), variant


def test_read_to_graph_passes_do_not_change_rows(built_lib):
    """Read-to-graph chains (ids numbered across the whole call) are the same
    in one pass and in passes of 37 reads."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend, OverlapParams, R2GParams
    wl = synth.read_to_graph(seed=7, genome_len=2_000_000, n_edges=60, coverage=6.0)
    g = wl.graph
    p = OverlapParams.make(**wl.params)
    r = R2GParams.make(**synth.R2G_PARAMS)
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        be.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
        be.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
        whole = be.read_to_graph(wl.reads, p, r)
        be.set_batch_queries(37)
        split = be.read_to_graph(wl.reads, p, r)
        assert be.last_passes() == -(-wl.reads.n // 37)
    assert len(whole) > 0
    assert split.tobytes() == whole.tobytes()


def test_candidates_passes_do_not_change_records(built_lib, scale_case):
    from cuflye_gb300.backend import CudaBackend
    wl = scale_case
    q = wl.reads.subset(np.arange(200))
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        cand, filt = be.candidates(q)
        be.set_batch_queries(29)
        cand2, filt2 = be.candidates(q)
    assert len(cand) > 0
    assert cand2.tobytes() == cand.tobytes() and filt2.tobytes() == filt.tobytes()


def test_small_calls_do_not_shrink_later_passes(built_lib, scale_case):
    """Under a budget, one-read calls before a large call leave its passes as
    they are: the pass body's other buffers are learned per hit only from
    passes where they take a real share of the budget."""
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    wl = scale_case
    p = OverlapParams.make(**wl.params)
    with CudaBackend(device=0, memory_budget_bytes=16 << 30) as be:
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        whole = be.overlaps(wl.reads, p)
        assert be.last_passes() == 1
        for i in range(5):
            be.overlaps(wl.reads.subset(np.arange(i, i + 1)), p)
        again = be.overlaps(wl.reads, p)
        assert be.last_passes() == 1
        assert be.last_pass_stats()["retries"] == 0
    assert again.tobytes() == whole.tobytes()
