"""CPU: the seeded generators give the shapes the benchmark configurations
name (read length distribution and bounds, coverage, error class, k, index
pieces), checked at reduced genome lengths.  Read lengths are measured after
the errors, which move them by the insertions less the deletions."""

import numpy as np
import pytest


def _lengths(reads) -> np.ndarray:
    return np.diff(reads.offsets)


def _check_reads(reads, genome_len, coverage, mean, sd, lo, hi, mean_tol=0.06):
    lens = _lengths(reads)
    assert abs(lens.mean() - mean) < mean_tol * mean, lens.mean()
    assert abs(lens.std() - sd) < 0.2 * sd, lens.std()
    assert lens.min() >= 0.95 * lo and lens.max() <= 1.05 * hi
    cov = lens.sum() / genome_len
    assert coverage * 0.98 <= cov <= coverage * 1.05, cov
    assert set(np.unique(reads.bases)) <= set(b"ACGT")
    assert len(np.unique(reads.ids)) == reads.n


def test_config1_plain_overlap_shapes():
    from cuflye_gb300 import synth
    wl = synth.plain_overlap(genome_len=300_000)
    assert wl.k == 15 and wl.params["kmer_size"] == 15
    assert wl.params["max_jump"] == 1500 and wl.params["max_gap"] == 500
    assert wl.params["min_overlap"] == 1000
    _check_reads(wl.reads, 300_000, 20.0, 10_000, 5_000, 1_000, 50_000)


def test_config2_batched_repeats_shapes():
    from cuflye_gb300 import synth
    wl = synth.batched_repeats(genome_len=1_000_000)
    assert wl.k == 17 and wl.params["kmer_size"] == 17
    _check_reads(wl.reads, 1_000_000, 40.0, 15_000, 3_000, 1_000, 100_000)


def test_config3_read_to_graph_shapes():
    from cuflye_gb300 import synth
    wl = synth.read_to_graph(genome_len=2_000_000, n_edges=40)
    assert wl.k == 15
    g = wl.graph
    # 40 edges plus 10 % duplicated copies (with the source's nodes)
    assert len(g.edge_ids) == 44
    assert np.array_equal(g.left[40:], g.left[np.searchsorted(g.left[:40], g.left[40:])])
    assert int(np.diff(g.seqs.offsets)[:40].sum()) == 2_000_000
    _check_reads(wl.reads, 2_000_000, 30.0, 20_000, 12_000, 1_000, 150_000)


@pytest.mark.parametrize("sparse", [False, True])
def test_config5_scale_shapes(sparse):
    from cuflye_gb300 import synth
    wl = synth.scale_ont(genome_len=2_000_000, coverage=30.0, sparse_errors=sparse)
    assert wl.k == 17 and wl.min_freq == 3 and wl.max_freq == 150
    _check_reads(wl.reads, 2_000_000, 30.0, 25_000, 15_000, 1_000, 150_000)


def test_config4_serving_shapes():
    from cuflye_gb300 import synth
    sw = synth.serving_workload(genome_len=5_000_000, n_queries=400)
    assert sw.k == 15
    assert sw.targets.n == 5 and int(sw.targets.offsets[-1]) == 5_000_000
    lens = _lengths(sw.queries)
    assert lens.min() >= 0.95 * 1_000 and lens.max() <= 1.05 * 100_000
    # log-uniform 1-100 kb: the median near 10 kb, the log-mean near log(10 kb)
    assert 7_000 < np.median(lens) < 14_000
    assert abs(np.log(lens).mean() - np.log(10_000)) < 0.2
    assert int(sw.queries.ids[0]) == 1_000_001
