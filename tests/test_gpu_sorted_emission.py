"""GPU: the sorted emission (hits written straight into KmerMatch order, the
default) against the emit + sort path and the oracle.

The two device paths must give the same rows, float bits included, on every
shape the parity cases hold: flagged queries with equal keys, ext-sorted
groups, long reads against long targets, read-to-graph, passes cut by a
budget.  A query hitting more distinct targets than a query's dictionary
holds (2,048) makes its pass take the emit + sort path by itself; its rows
still match the oracle."""

import numpy as np
import pytest

from test_gpu_parity import oracle_index, overlap_tuples_gpu, overlap_tuples_oracle

pytestmark = pytest.mark.gpu


def _both_paths(gpu, reads, params):
    from cuflye_gb300.backend import OverlapParams
    p = OverlapParams.make(**params)
    gpu.set_sorted_emission(2)  # every pass, sparse ones included
    fused = overlap_tuples_gpu(gpu.overlaps(reads, p))
    stats = gpu.last_sort_stats()
    gpu.set_sorted_emission(0)
    try:
        plain = overlap_tuples_gpu(gpu.overlaps(reads, p))
    finally:
        gpu.set_sorted_emission(1)
    return fused, plain, stats


@pytest.mark.parametrize("case", ["ovl-a", "ovl-b", "ovl-c", "ovl-d"])
def test_sorted_emission_equals_emit_and_sort(gpu, golden_cases, case):
    reads, meta, _ = golden_cases[case]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    for variant in ({}, {"only_max_ext": 0, "check_overhang": 0}):
        fused, plain, stats = _both_paths(gpu, reads, dict(meta["params"], **variant))
        assert fused == plain, variant
        assert stats["emission_fallbacks"] == 0
        assert len(fused) > 0


def test_sorted_emission_on_tandem_ties(gpu, oracle_mod):
    """Flagged queries (equal keys) keep generation order for the
    libstdc++-order sort; their groups are prefiltered after it."""
    from cuflye_gb300 import synth
    wl = synth.tandem_case(11)
    gpu.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
    fused, plain, stats = _both_paths(gpu, wl.reads, dict(wl.params, only_max_ext=0))
    assert fused == plain
    assert stats["match_libstdcxx"] > 0 and stats["match_plain"] > 0


def test_sorted_emission_long_reads_and_passes(gpu, oracle_mod):
    """Long reads against 1 Mb pieces (ext-sorted groups out of ext order)
    and the same queries cut into passes by a tight budget."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    sw = synth.serving_workload(seed=5, genome_len=2_000_000, n_queries=60)
    gpu.build_index(sw.targets, sw.k, sw.min_freq, sw.max_freq)
    fused, plain, _ = _both_paths(gpu, sw.queries, sw.params)
    assert fused == plain and len(fused) > 0
    gpu.set_batch_queries(7)
    gpu.set_sorted_emission(2)
    try:
        cut = overlap_tuples_gpu(gpu.overlaps(sw.queries, OverlapParams.make(**sw.params)))
        assert gpu.last_passes() > 1
    finally:
        gpu.set_batch_queries(0)
        gpu.set_sorted_emission(1)
    assert cut == fused


def test_sorted_emission_read_to_graph(gpu):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams, R2GParams
    wl = synth.read_to_graph(seed=3, genome_len=400_000, n_edges=24, coverage=4.0)
    g = wl.graph
    gpu.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
    gpu.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
    p, r = OverlapParams.make(**wl.params), R2GParams.make(**synth.R2G_PARAMS)
    gpu.set_sorted_emission(2)
    try:
        fused = gpu.read_to_graph(wl.reads, p, r)
    finally:
        gpu.set_sorted_emission(1)
    gpu.set_sorted_emission(0)
    try:
        plain = gpu.read_to_graph(wl.reads, p, r)
    finally:
        gpu.set_sorted_emission(1)
    assert fused.tobytes() == plain.tobytes() and len(fused) > 0


def _crowded_case(seed=21, region=6000, targets=2200, tlen=3000):
    """2,200 reads of one 6 kb region (both strands, 1 % error) as targets,
    and queries that hit more than 2,048 of them."""
    from cuflye_gb300 import synth
    rng = np.random.default_rng(seed)
    genome = synth.random_genome(rng, region)
    seqs = []
    for _ in range(targets):
        s = int(rng.integers(0, region - tlen + 1))
        x = genome[s:s + tlen]
        if rng.random() < 0.5:
            x = synth.revcomp(x)
        seqs.append(synth.mutate(rng, x, 0.005, 0.0025, 0.0025).tobytes())
    tg = synth.ReadSet.from_strings(np.arange(1, targets + 1), seqs)
    q = synth.ReadSet.from_strings([10_001, -10_002],
                                   [genome.tobytes(), synth.revcomp(genome[500:5500]).tobytes()])
    return tg, q


def test_query_beyond_the_dictionary_falls_back(gpu, oracle_mod):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    oracle_mod.set_stable(False)
    tg, q = _crowded_case()
    k, min_freq, max_freq = 15, 1, 100_000
    gpu.build_index(tg, k, min_freq, max_freq)
    params = dict(synth.OVERLAP_PARAMS, kmer_size=k, only_max_ext=0)
    gpu.set_sorted_emission(2)  # two queries: below the default's queries per SM
    try:
        got = gpu.overlaps(q, OverlapParams.make(**params))
        assert gpu.last_sort_stats()["emission_fallbacks"] >= 1
    finally:
        gpu.set_sorted_emission(1)
    idx, _ = oracle_index(oracle_mod, tg, k, min_freq, max_freq)
    b = oracle_mod.SeqBatch(q.ids, q.offsets, q.bases.tobytes())
    exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**params))
    assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp)
    assert len(got) > 2048
