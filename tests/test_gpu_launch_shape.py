"""Launch shapes change no result.  The overlap rows are the same under every
blocks-per-SM choice of the chaining DP, the backtrack, the KmerMatch radix
scatter and the libstdc++-order sort's rounds, and after the autotuner has
picked a shape.  The tandem-repeat workload sends queries down both the radix
path and the libstdc++-order rounds."""

import pytest

pytestmark = pytest.mark.gpu

SHAPES = (
    {"dp_blocks_per_sm": 1, "backtrack_blocks_per_sm": 1, "scatter_blocks_per_sm": 1,
     "round_blocks_per_sm": 1},
    {"dp_blocks_per_sm": 3, "backtrack_blocks_per_sm": 2, "scatter_blocks_per_sm": 2,
     "round_blocks_per_sm": 1},
    {"dp_blocks_per_sm": 8, "backtrack_blocks_per_sm": 4, "scatter_blocks_per_sm": 2,
     "round_blocks_per_sm": 2},
)
LIMITS = {"dp_blocks_per_sm": 8, "backtrack_blocks_per_sm": 4, "scatter_blocks_per_sm": 2,
          "round_blocks_per_sm": 2}


def test_shapes_and_autotune_keep_rows(built_lib):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend, CuflyeError, OverlapParams
    wl = synth.tandem_case(seed=4)
    p = OverlapParams.make(**wl.params)
    with CudaBackend(device=0, memory_budget_bytes=0) as be:
        be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        assert be.launch_shape() == {k: 0 for k in LIMITS}
        base = be.overlaps(wl.reads, p)
        paths = be.last_sort_stats()
        assert len(base) > 0
        assert paths["match_plain"] > 0 and paths["match_libstdcxx"] > 0
        for shape in SHAPES:
            be.set_launch_shape(**shape)
            assert be.launch_shape() == shape
            assert be.overlaps(wl.reads, p).tobytes() == base.tobytes(), shape
        for name, most in LIMITS.items():
            with pytest.raises(CuflyeError):
                be.set_launch_shape(**{name: most + 1})
        be.set_launch_shape(**{k: 0 for k in LIMITS})
        tuned = be.autotune(wl.reads, p)
        for name, most in LIMITS.items():
            assert 1 <= tuned["shape"][name] <= most
        assert 0 < tuned["ms_chosen"] <= tuned["ms_start"]
        assert be.launch_shape() == tuned["shape"]
        assert be.overlaps(wl.reads, p).tobytes() == base.tobytes()
