"""The k-mer index built one key range at a time is the same index as the
one-range build.  Ranges are forced either by a window cap or by a memory
budget below the one-range build's peak.  Both builds must give the same
counts, the same candidate records and the same overlaps, and the ranged
index must give the oracle's rows."""

import numpy as np
import pytest

from test_gpu_parity import oracle_index, overlap_tuples_gpu, overlap_tuples_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    from cuflye_gb300 import synth
    return synth.scale_ont(seed=11, genome_len=1_000_000, coverage=6.0)


def _windows(reads, k: int) -> int:
    return int(np.maximum(np.diff(reads.offsets) - k + 1, 0).sum())


def _sample(reads, n: int):
    rng = np.random.default_rng(5)
    return reads.subset(np.sort(rng.choice(reads.n, size=min(n, reads.n), replace=False)))


def test_window_cap_gives_the_same_index(built_lib, case):
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    wl = case
    p = OverlapParams.make(**wl.params)
    q = _sample(wl.reads, 150)
    nwin = _windows(wl.reads, wl.k)
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        one = be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() == 1
        cand_one = be.candidates(q)
        ov_one = be.overlaps(wl.reads, p)
        be.set_index_build_windows(nwin // 6 + 1)
        many = be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() >= 6
        cand_many = be.candidates(q)
        ov_many = be.overlaps(wl.reads, p)
        # a cap above the window count leaves the build in one range
        be.set_index_build_windows(nwin + 1)
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() == 1
    assert many == one
    assert len(cand_one[0]) > 0 and len(ov_one) > 0
    assert cand_many[0].tobytes() == cand_one[0].tobytes()
    assert cand_many[1].tobytes() == cand_one[1].tobytes()
    assert ov_many.tobytes() == ov_one.tobytes()


def test_ranged_index_matches_oracle(built_lib, oracle_mod, case):
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    wl = case
    oracle_mod.set_stable(False)
    idx, _ = oracle_index(oracle_mod, wl.reads, wl.k, wl.min_freq, wl.max_freq)
    lens = np.diff(wl.reads.offsets)
    q = wl.reads.subset(np.sort(np.argsort(lens)[-10:]))
    b = oracle_mod.SeqBatch(q.ids, q.offsets, q.bases.tobytes())
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        be.set_index_build_windows(_windows(wl.reads, wl.k) // 4 + 1)
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() >= 4
        got = be.overlaps(q, OverlapParams.make(**wl.params))
    exp = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**wl.params))
    assert len(got) > 0
    assert overlap_tuples_gpu(got) == overlap_tuples_oracle(exp)


def test_budget_below_one_range_peak_builds_in_ranges(built_lib, case):
    from cuflye_gb300.backend import CudaBackend, OverlapParams
    wl = case
    p = OverlapParams.make(**wl.params)
    q = _sample(wl.reads, 200)
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        one = be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        build_peak = be.memory_stats()[1]
        ov_one = be.overlaps(q, p)
    budget = int(build_peak * 0.7)
    with CudaBackend(device=0, memory_budget_bytes=budget) as be:
        got = be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.last_index_ranges() >= 2
        assert be.memory_stats()[1] <= budget
        ov = be.overlaps(q, p)
    assert got == one
    assert ov.tobytes() == ov_one.tobytes()


def test_small_k_ranges(built_lib):
    """k = 6: 4,096 prefix bins of the whole 12-bit key (no shift)."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend
    wl = synth.small_overlap_case(seed=3, genome_len=8_000, coverage=3.0, mean_len=2_000, k=6)
    nwin = _windows(wl.reads, 6)
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        one = be.build_index(wl.reads, 6, 1, 15)
        cand_one = be.candidates(wl.reads)
        be.set_index_build_windows(nwin // 3 + 1)
        many = be.build_index(wl.reads, 6, 1, 15)
        assert be.last_index_ranges() >= 3
        cand_many = be.candidates(wl.reads)
    assert many == one and one["repetitive"] > 0
    assert cand_many[0].tobytes() == cand_one[0].tobytes()
    assert cand_many[1].tobytes() == cand_one[1].tobytes()
