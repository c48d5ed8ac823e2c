"""GPU parity on the benchmark configurations at their stated sizes.

The other GPU parity tests use small or scaled-down cases; these run the
workloads the bench times, with the full index of each, and compare the CUDA
path (through the C ABI) with the CPU oracle bit for bit, float divergence
bits included:

* the plain 1 Mb / 20x configuration (k = 15): all 2,007 reads;
* the 5 Mb repeat-bearing genome at 40x HiFi (k = 17): 300 reads against the
  index of all 13,338 reads;
* read-to-graph on the 20 Mb genome cut into 400 edges plus 40 duplicated
  repeat edges (k = 15): 200 ONT reads against the whole graph, half of them
  sampled over the duplicated edges;
* serving on the 100 Mb genome with 5 % repeats (k = 15): 200 requests
  through cuflye_submit / cuflye_poll, alone and all in flight at once.

The oracle runs in libstdc++ sort mode, the order Flye's std::sort gives."""

import os
import threading

import numpy as np
import pytest

from test_gpu_parity import overlap_tuples_gpu, overlap_tuples_oracle
from test_gpu_r2g import rows_gpu, rows_oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _oracle_overlaps(O, idx, reads, params):
    b = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    return overlap_tuples_oracle(O.overlaps(idx, b, O.default_params(**params), threads=THREADS))


def _oracle_index(O, seqs, k, min_freq, max_freq):
    b = O.SeqBatch(seqs.ids, seqs.offsets, seqs.bases.tobytes())
    return O.Index.build(k, b, min_freq, max_freq)


def test_config1_plain_overlap_all_reads(gpu, oracle_mod):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    oracle_mod.set_stable(False)
    wl = synth.plain_overlap()
    assert wl.reads.n == 2007
    gpu.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
    got = overlap_tuples_gpu(gpu.overlaps(wl.reads, OverlapParams.make(**wl.params)))
    idx = _oracle_index(oracle_mod, wl.reads, wl.k, wl.min_freq, wl.max_freq)
    exp = _oracle_overlaps(oracle_mod, idx, wl.reads, wl.params)
    assert len(exp) > 50_000
    assert got == exp


def test_config2_batched_repeats_sample_against_full_index(gpu, oracle_mod):
    """300 reads, spread over the read set (every 44th), against the index of
    the whole 200 Mb read set; the same rows whether the 300 reads run alone
    or inside the batch of all reads."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams
    oracle_mod.set_stable(False)
    wl = synth.batched_repeats()
    assert wl.reads.n == 13338
    p = OverlapParams.make(**wl.params)
    gpu.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
    pick = np.arange(0, wl.reads.n, 44)[:300]
    sub = wl.reads.subset(pick)
    got = overlap_tuples_gpu(gpu.overlaps(sub, p))
    idx = _oracle_index(oracle_mod, wl.reads, wl.k, wl.min_freq, wl.max_freq)
    exp = _oracle_overlaps(oracle_mod, idx, sub, wl.params)
    assert len(exp) > 10_000
    assert got == exp
    # the same reads' rows inside the full batched call
    full = gpu.overlaps(wl.reads, p)
    ids = set(int(i) for i in sub.ids)
    in_batch = overlap_tuples_gpu(r for r in full if int(r["cur_id"]) in ids)
    assert in_batch == got
    # the full call's working buffers go back to the device (the session's
    # context otherwise keeps most of the GPU for the tests after this one)
    held = gpu.memory_stats()[0]
    gpu.trim()
    assert gpu.memory_stats()[0] < held
    assert overlap_tuples_gpu(gpu.overlaps(sub, p)) == got


def _reads_over_duplicated_edges(wl, count):
    """Reads whose sampled interval covers at least 2 kb of an edge that the
    graph holds twice (the original and its 0.5 %-diverged copy)."""
    g = wl.graph
    n0 = int(np.sum(g.edge_ids <= len(g.edge_ids) * 10 // 11))
    offs = g.seqs.offsets
    starts = offs[:n0]
    ends = offs[1:n0 + 1]
    dup = sorted({int(g.left[e]) // 2 for e in range(n0, len(g.edge_ids))})
    r = wl.reads
    lens = np.diff(r.offsets)
    picked = []
    for i in range(r.n):
        a, b = int(r.origin[i]), int(r.origin[i] + lens[i])
        for d in dup:
            if min(b, int(ends[d])) - max(a, int(starts[d])) >= 2000:
                picked.append(i)
                break
        if len(picked) == count:
            break
    return picked


def test_config3_read_to_graph_with_repeat_edges(gpu, oracle_mod):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import OverlapParams, R2GParams
    oracle_mod.set_stable(False)
    wl = synth.read_to_graph()
    g = wl.graph
    assert len(g.edge_ids) == 440
    over_dup = _reads_over_duplicated_edges(wl, 100)
    assert len(over_dup) == 100
    rest = [i for i in range(wl.reads.n) if i not in set(over_dup)][:100]
    sub = wl.reads.subset(np.array(sorted(over_dup + rest)))
    gpu.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
    gpu.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
    got = gpu.read_to_graph(sub, OverlapParams.make(**wl.params),
                            R2GParams.make(**synth.R2G_PARAMS))
    idx = _oracle_index(oracle_mod, g.seqs, wl.k, wl.min_freq, wl.max_freq)
    rb = oracle_mod.SeqBatch(sub.ids, sub.offsets, sub.bases.tobytes())
    exp = oracle_mod.read_to_graph(idx, g.edge_ids, g.seq_ids, g.left, g.right, rb,
                                   oracle_mod.default_params(**wl.params),
                                   oracle_mod.default_r2g(**synth.R2G_PARAMS))
    assert rows_gpu(got) == rows_oracle(exp)
    assert len(got) > 300
    # the chaining input of the reads over duplicated edges holds overlaps with
    # both copies (edge-sequence ids above 400 are the copies)
    dup_reads = wl.reads.subset(np.array(over_dup))
    ovl = gpu.overlaps(dup_reads, OverlapParams.make(**wl.params))
    assert any(abs(int(r["ext_id"])) > 400 for r in ovl)
    assert any(abs(int(r["ext_id"])) <= 400 for r in ovl)


def test_config4_serving_requests_alone_and_in_flight(gpu, oracle_mod):
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaServer, OverlapParams, Sequences
    oracle_mod.set_stable(False)
    sw = synth.serving_workload(seed=4)
    q = sw.queries
    reqs = [Sequences(q.ids[i:i + 1].copy(),
                      np.array([0, q.offsets[i + 1] - q.offsets[i]], dtype=np.int64),
                      np.ascontiguousarray(q.bases[q.offsets[i]:q.offsets[i + 1]]))
            for i in range(200)]
    gpu.build_index(sw.targets, sw.k, sw.min_freq, sw.max_freq)
    p = OverlapParams.make(**sw.params)
    idx = _oracle_index(oracle_mod, sw.targets, sw.k, sw.min_freq, sw.max_freq)
    sub = q.subset(np.arange(200))
    b = oracle_mod.SeqBatch(sub.ids, sub.offsets, sub.bases.tobytes())
    res = oracle_mod.overlaps(idx, b, oracle_mod.default_params(**sw.params), threads=THREADS)
    exp_all = overlap_tuples_oracle(res)
    exp = [[r for r in exp_all if r[0] == int(s.ids[0])] for s in reqs]
    assert sum(len(e) for e in exp) == len(exp_all) > 100
    with CudaServer(gpu, p, workers=2, max_batch_bases=32_000_000) as srv:
        alone = [overlap_tuples_gpu(srv.poll(srv.submit(s), -1)) for s in reqs]
        tickets = [None] * len(reqs)

        def submit(ks):
            for k in ks:
                tickets[k] = srv.submit(reqs[k])

        th = [threading.Thread(target=submit, args=(range(t, len(reqs), 4),)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        mixed = [overlap_tuples_gpu(srv.poll(tk, -1)) for tk in tickets]
    assert alone == exp
    assert mixed == exp
