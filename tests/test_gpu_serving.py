"""Serving (continuous batching) through the C ABI: a request's rows are the
same when it runs alone and when it shares batches with concurrent requests,
and equal the oracle's rows for its queries (bit-exact)."""

import threading

import numpy as np
import pytest

from test_gpu_parity import oracle_index, overlap_tuples_gpu, overlap_tuples_oracle

pytestmark = pytest.mark.gpu


def _split(reads, sizes):
    out, i = [], 0
    for s in sizes:
        out.append(reads.subset(np.arange(i, min(i + s, reads.n))))
        i += s
    return [r for r in out if r.n]


def test_requests_same_alone_and_in_the_mix(gpu, oracle_mod, golden_cases):
    from cuflye_gb300.backend import CudaServer, OverlapParams
    oracle_mod.set_stable(False)
    reads, meta, _ = golden_cases["ovl-d"]
    idx, _ = oracle_index(oracle_mod, reads, meta["k"], meta["min_freq"], meta["max_freq"])
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    params = OverlapParams.make(**meta["params"])
    reqs = _split(reads, [1, 7, 3, 20, 2, 11, 5, 30, 4, 9])
    direct = [overlap_tuples_gpu(gpu.overlaps(r, params)) for r in reqs]
    oracle = []
    for r in reqs:
        b = oracle_mod.SeqBatch(r.ids, r.offsets, r.bases.tobytes())
        oracle.append(overlap_tuples_oracle(
            oracle_mod.overlaps(idx, b, oracle_mod.default_params(**meta["params"]))))
    assert direct == oracle
    with CudaServer(gpu, params, workers=2) as srv:
        alone = [overlap_tuples_gpu(srv.poll(srv.submit(r), -1)) for r in reqs]
        s0 = srv.stats()
        # every request submitted at once from four threads, then polled
        tickets = [None] * len(reqs)

        def submit(ks):
            for k in ks:
                tickets[k] = srv.submit(reqs[k])

        th = [threading.Thread(target=submit, args=(range(t, len(reqs), 4),)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        mixed = [overlap_tuples_gpu(srv.poll(tk, -1, capacity=1)) for tk in tickets]
        s1 = srv.stats()
    assert alone == direct
    assert mixed == direct
    assert s0["batches"] == len(reqs)  # alone: one request per batch
    # in the mix, batches carried several requests each
    assert s1["requests"] - s0["requests"] == len(reqs)
    assert s1["batches"] - s0["batches"] < len(reqs)


def test_server_errors(gpu, golden_cases):
    from cuflye_gb300.backend import CudaServer, CuflyeError, OverlapParams
    reads, meta, _ = golden_cases["ovl-a"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    with CudaServer(gpu, OverlapParams.make(**meta["params"]), workers=1) as srv:
        with pytest.raises(CuflyeError) as e:
            srv.poll(12345, 0)
        assert e.value.status == 1  # unknown ticket
        t = srv.submit(reads.subset(np.arange(3)))
        rows = srv.poll(t, -1)
        assert rows is not None
        with pytest.raises(CuflyeError):
            srv.poll(t, 0)  # consumed
        with pytest.raises(CuflyeError):  # the server borrows the index
            gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])  # closed: fine
    with pytest.raises(CuflyeError):  # k of the params must match the index
        CudaServer(gpu, OverlapParams.make(**dict(meta["params"], kmer_size=meta["k"] + 2)))


def test_poll_any_returns_each_request_once_in_completion_order(gpu, golden_cases):
    """cuflye_poll_any hands back every finished request exactly once, with
    the rows cuflye_overlaps gives it alone; a request whose rows do not fit
    stays for cuflye_poll on its ticket; one that cuflye_poll consumed first
    is skipped; with nothing in flight it reports pending."""
    from cuflye_gb300.backend import CudaServer, OverlapParams
    reads, meta, _ = golden_cases["ovl-d"]
    gpu.build_index(reads, meta["k"], meta["min_freq"], meta["max_freq"])
    params = OverlapParams.make(**meta["params"])
    reqs = _split(reads, [2, 5, 1, 9, 3, 12, 4, 6])
    direct = [overlap_tuples_gpu(gpu.overlaps(r, params)) for r in reqs]
    with CudaServer(gpu, params, workers=2) as srv:
        assert srv.poll_any(0) is None
        tickets = [srv.submit(r) for r in reqs]
        which = {tk: i for i, tk in enumerate(tickets)}
        got = {}
        while len(got) < len(reqs):
            tk, rows = srv.poll_any(-1, capacity=1)  # small: some take the poll route
            assert tk in which and tk not in got
            got[tk] = overlap_tuples_gpu(rows)
        assert [got[tk] for tk in tickets] == direct
        assert srv.poll_any(0) is None
        # consumed by poll first: poll_any skips it
        t1 = srv.submit(reqs[0])
        assert overlap_tuples_gpu(srv.poll(t1, -1)) == direct[0]
        t2 = srv.submit(reqs[1])
        tk, rows = srv.poll_any(-1)
        assert tk == t2 and overlap_tuples_gpu(rows) == direct[1]
        assert srv.poll_any(0) is None
