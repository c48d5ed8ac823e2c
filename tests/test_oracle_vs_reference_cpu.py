"""CPU: the oracle agrees with the reference's own compiled CPU backends
(built by oracle/ref_build.py from the reference checkout), beyond the golden
vectors.  Seeded synthetic queries become overlap-replay fixtures
(docs/abi/overlap-replay-fixture-v0.md), and the overlap chain replay's
``--backend cpu`` chains them (cuflye_cuda_overlap_chain_replay.cu:
buildGroups, computeCpuGroupOverlap, finalizeOverlaps).  Its rows must equal
the oracle's, text for text, with the oracle sorting as the prototype does:
std::sort for the ext re-sort, backtrack starts and primary choice in index
order among equal scores.  (Flye itself, and the library, use std::sort at
all of these places; the reference's Python replays pin those orders.)
Skipped where the reference checkout is absent."""

import json
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref_overlap_bin():
    from oracle import ref_build
    ref_build.build()
    path = ref_build.binary("overlap_chain_replay")
    if path is None:
        pytest.skip("the reference's CPU backends are not built here (no reference checkout)")
    return path


def fmt9(x: float) -> str:
    return "0" if x == 0 else format(float(np.float32(x)), ".9g")


def _manifest_params(k: int, p: dict) -> dict:
    return {
        "kmer_size": k, "minimum_overlap": p["min_overlap"], "maximum_jump": p["max_jump"],
        "max_jump_gap": p["max_gap"], "chain_gap_jump_threshold": p["gap_jump_threshold"],
        "chain_large_gap_penalty": p["large_gap_penalty"],
        "chain_small_gap_penalty": p["small_gap_penalty"],
        "min_kmer_survival_rate": p["min_kmer_survival_rate"],
        "maximum_overhang": p["max_overhang"], "check_overhang": bool(p["check_overhang"]),
        "force_local": bool(p["force_local"]), "only_max_ext": True, "max_overlaps": 0,
        "max_divergence": p["max_divergence"], "sample_rate": p["sample_rate"],
        "keep_alignment": False, "nucl_alignment": False, "partition_bad_mappings": False,
        "use_hpc": False,
    }


def _write_fixtures(O, wl, root, limit, **overrides):
    """One fixture directory per query with candidates (at most `limit`
    queries), chaining parameters overridden by `overrides`; returns
    {fixture name: expected overlap-range-v1 lines}."""
    reads = wl.reads
    batch = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    idx = O.Index.build(wl.k, batch, wl.min_freq, wl.max_freq)
    O.set_stable(False)
    gen = O.candidates(idx, batch, sorted_like_flye=False)
    srt = O.candidates(idx, batch, sorted_like_flye=True)
    lens = {int(reads.ids[i]): int(reads.offsets[i + 1] - reads.offsets[i])
            for i in range(reads.n)}
    params = dict(wl.params, **overrides, only_max_ext=1, max_overlaps=0)
    oparams = O.default_params(**params)
    mparams = _manifest_params(wl.k, params)
    expected = {}
    for q in [int(x) for x in reads.ids]:
        sel = srt["query_id"] == q
        if not sel.any():
            continue
        qpos, tpos, tid, km = (srt["query_pos"][sel], srt["target_pos"][sel],
                               srt["target_id"][sel], srt["kmer"][sel])
        filtered = sorted(int(x) for x in gen["filtered_pos"][gen["filtered_query"] == q])
        targets = sorted(set(int(t) for t in tid))
        name = f"query_{q}"
        d = root / name
        d.mkdir()
        (d / "candidates.tsv").write_text("".join(
            f"{q}\t{int(a)}\t{int(c)}\t{int(t)}\t{int(b)}\t{'+' if t > 0 else '-'}\n"
            for a, b, t, c in zip(qpos, tpos, tid, km)))
        (d / "filtered-positions.tsv").write_text("".join(f"{x}\n" for x in filtered))
        (d / "targets.tsv").write_text("".join(f"{t}\t{lens[abs(t)]}\n" for t in targets))
        (d / "oracle.overlaps.tsv").write_text("")
        (d / "manifest.json").write_text(json.dumps({
            "schema": "cuflye-overlap-replay-fixture-v0", "query_id": q,
            "query_length": lens[q], "candidate_records": int(sel.sum()),
            "target_records": len(targets), "oracle_overlap_records": 0,
            "files": {"candidates": "candidates.tsv",
                      "filtered_positions": "filtered-positions.tsv",
                      "targets": "targets.tsv", "oracle_overlaps": "oracle.overlaps.tsv"},
            "parameters": mparams}))
        # the prototype's sort places: std::sort for the ext re-sort, score
        # order and primary choice in index order (stable)
        O.set_sort_mode(O.SORT_SCORE | O.SORT_PRIMARY)
        r = O.chain_sorted(qpos, tpos, tid, q, lens[q], list(lens.keys()),
                           list(lens.values()), filtered, oparams)
        O.set_stable(False)
        expected[name] = ["\t".join(str(int(v)) for v in row) + "\t" + fmt9(dv)
                          for row, dv in zip(r["cols"], r["divergence"])]
        if len(expected) == limit:
            break
    return expected


CASES = [
    # seed, genome, coverage, mean read length, k, (sub, ins, del), repeat
    (21, 40_000, 8.0, 5_000, 15, (0.01, 0.005, 0.005), False),
    (22, 50_000, 10.0, 6_000, 15, (0.01, 0.005, 0.005), True),
    (23, 40_000, 12.0, 4_000, 17, (0.002, 0.001, 0.001), True),
    (24, 30_000, 6.0, 3_000, 11, (0.03, 0.01, 0.01), False),
]


@pytest.mark.parametrize("case", CASES, ids=[f"seed{c[0]}" for c in CASES])
def test_reference_cpu_chaining_matches_oracle(oracle_mod, ref_overlap_bin, tmp_path, case):
    from cuflye_gb300 import synth
    seed, glen, cov, mlen, k, (sub, ins, dele), rep = case
    wl = synth.small_overlap_case(seed, glen, cov, mlen, k, sub, ins, dele, rep)
    fx = tmp_path / "fixtures"
    fx.mkdir()
    expected = _write_fixtures(oracle_mod, wl, fx, limit=60)
    assert expected
    (tmp_path / "list.txt").write_text("".join(f"{fx / n}\n" for n in expected))
    subprocess.run([str(ref_overlap_bin), "--batch-fixtures-file", str(tmp_path / "list.txt"),
                    "--batch-output-dir", str(tmp_path / "out"), "--batch-json-output",
                    str(tmp_path / "out.json"), "--backend", "cpu"],
                   check=True, capture_output=True, text=True, timeout=300)
    rows = 0
    for name, want in expected.items():
        got = (tmp_path / "out" / name / "overlaps.tsv").read_text().splitlines()
        assert got == want, name
        rows += len(got)
    assert rows > 0


def test_reference_cpu_chaining_on_tandem_ties(oracle_mod, ref_overlap_bin, tmp_path):
    """Tandem arrays: equal KmerMatch keys, equal ext positions and equal
    scores, where the order of ties decides the rows."""
    from cuflye_gb300 import synth
    wl = synth.tandem_case(seed=4)
    fx = tmp_path / "fixtures"
    fx.mkdir()
    expected = _write_fixtures(oracle_mod, wl, fx, limit=80)
    (tmp_path / "list.txt").write_text("".join(f"{fx / n}\n" for n in expected))
    subprocess.run([str(ref_overlap_bin), "--batch-fixtures-file", str(tmp_path / "list.txt"),
                    "--batch-output-dir", str(tmp_path / "out"), "--batch-json-output",
                    str(tmp_path / "out.json"), "--backend", "cpu"],
                   check=True, capture_output=True, text=True, timeout=300)
    for name, want in expected.items():
        got = (tmp_path / "out" / name / "overlaps.tsv").read_text().splitlines()
        assert got == want, name


def test_reference_cpu_chaining_other_parameters(oracle_mod, ref_overlap_bin, tmp_path):
    """No overhang check, local overlaps forced, a shorter jump, gap and
    minimum overlap and a higher survival rate: the overlapTest and group
    prefilter branches the default parameters do not reach."""
    from cuflye_gb300 import synth
    wl = synth.small_overlap_case(25, 40_000, 10.0, 4_000, 15, 0.02, 0.01, 0.01, True)
    fx = tmp_path / "fixtures"
    fx.mkdir()
    expected = _write_fixtures(oracle_mod, wl, fx, limit=60, check_overhang=0, force_local=1,
                               max_jump=1000, max_gap=300, min_overlap=800,
                               min_kmer_survival_rate=0.02, max_divergence=0.5)
    (tmp_path / "list.txt").write_text("".join(f"{fx / n}\n" for n in expected))
    subprocess.run([str(ref_overlap_bin), "--batch-fixtures-file", str(tmp_path / "list.txt"),
                    "--batch-output-dir", str(tmp_path / "out"), "--batch-json-output",
                    str(tmp_path / "out.json"), "--backend", "cpu"],
                   check=True, capture_output=True, text=True, timeout=300)
    rows = 0
    for name, want in expected.items():
        got = (tmp_path / "out" / name / "overlaps.tsv").read_text().splitlines()
        assert got == want, name
        rows += len(got)
    assert rows > 0


# ---------------------------------------------------------------- read-to-graph chains


@pytest.fixture(scope="module")
def ref_r2g_bin():
    from oracle import ref_build
    ref_build.build()
    path = ref_build.binary("read_alignment_chain_replay")
    if path is None:
        pytest.skip("the reference's CPU backends are not built here (no reference checkout)")
    return path


def _edge_alignments(rng, n_path: int) -> list[dict]:
    """One read's edge alignments in read_begin order: a walk over graph
    nodes (each edge's right node usually the next one's left node), with
    gaps, small overlaps, broken links and alignments that start or end far
    inside their edge, plus unrelated alignments on other nodes."""
    rows = []
    pos = int(rng.integers(0, 2_000))
    node = int(rng.integers(0, 30))
    for _ in range(n_path):
        elen = int(rng.integers(600, 8_000))
        eb = int(rng.integers(0, 150)) if rng.random() < 0.8 else int(rng.integers(0, 2_500))
        ee = min(elen, eb + int(rng.integers(200, 6_000)))
        if rng.random() < 0.8:
            ee = max(ee, elen - int(rng.integers(0, 200)))
        nxt = int(rng.integers(0, 30))
        span = ee - eb + int(rng.integers(-40, 40))
        rows.append([pos, pos + max(span, 50), eb, ee, elen, node, nxt])
        node = nxt if rng.random() < 0.85 else int(rng.integers(0, 30))
        pos = pos + max(span, 50) + int(rng.integers(-70, 300))
    for _ in range(n_path // 3):
        elen = int(rng.integers(600, 8_000))
        eb = int(rng.integers(0, elen - 300))
        ee = int(rng.integers(eb + 200, elen + 1))
        rb = int(rng.integers(0, max(pos, 1)))
        rows.append([rb, rb + ee - eb, eb, ee, elen, int(rng.integers(0, 30)),
                     int(rng.integers(0, 30))])
    rows.sort(key=lambda r: r[0])  # stable: equal read_begin keep this order
    for i, r in enumerate(rows):
        span = r[3] - r[2]
        r.append(int(span * rng.uniform(0.3, 1.0)))           # score
        r.append(float(np.float32(rng.uniform(0.0, 0.3))))    # seq divergence
        r.append(1_000 + i)                                   # edge id (unique)
    return rows


def test_reference_cpu_read_alignment_chains_match_oracle(oracle_mod, ref_r2g_bin, tmp_path):
    """Synthetic read-alignment replay fixtures
    (docs/abi/read-alignment-replay-fixture-v0.md) chained by the read-
    alignment replay's CPU backend in its pre-divergence mode
    (cuflye_cuda_read_alignment_chain_replay.cu:872-984, every candidate
    chain, no divergence filter) give the oracle's chains, segment for
    segment."""
    from cuflye_gb300 import synth
    O = oracle_mod
    p = synth.R2G_PARAMS
    r2g = O.default_r2g(max_jump=p["max_jump"], max_read_overlap=p["max_read_overlap"],
                        min_overlap=p["min_overlap"], max_separation=p["max_separation"])
    rng = np.random.default_rng(31)
    chains_seen = 0
    for f in range(40):
        rows = _edge_alignments(rng, int(rng.integers(4, 40)))
        read_len = max(r[1] for r in rows) + int(rng.integers(0, 500))
        d = tmp_path / f"read_{f}"
        d.mkdir()
        (d / "edge-overlaps.tsv").write_text("".join(
            f"{i}\t{7}\t{r[0]}\t{r[1]}\t{read_len}\t{r[9]}\t{r[5]}\t{r[6]}\t{r[9] + 5000}\t"
            f"{r[2]}\t{r[3]}\t{r[4]}\t{r[7]}\t{fmt9(r[8])}\n" for i, r in enumerate(rows)))
        (d / "manifest.json").write_text(json.dumps({
            "schema": "cuflye-read-alignment-replay-fixture-v0", "query_id": 7,
            "alignment_input_records": len(rows), "candidate_chains": 0, "oracle_chains": 0,
            "maximum_jump": p["max_jump"], "max_read_overlap": p["max_read_overlap"],
            "minimum_overlap": p["min_overlap"], "max_separation": p["max_separation"],
            "read_align_ovlp_divergence": p["max_chain_divergence"],
            "reads_base_alignment": False}))
        subprocess.run([str(ref_r2g_bin), "--fixture-dir", str(d), "--output-tsv",
                        str(d / "out.tsv"), "--json-output", str(d / "out.json"), "--backend",
                        "cpu", "--emit-pre-divergence-chains"],
                       check=True, capture_output=True, text=True, timeout=120)
        by_edge = {r[9]: i for i, r in enumerate(rows)}
        got: list[list[int]] = []
        for line in (d / "out.tsv").read_text().splitlines():
            c = line.split("\t")
            chain, seg = int(c[0]), int(c[1])
            while len(got) <= chain:
                got.append([])
            assert seg == len(got[chain])
            got[chain].append(by_edge[int(c[6])])
        arr = np.array([[r[0], r[1], r[2], r[3], r[4], r[7]] for r in rows])
        want = O.chain_read_alignments(arr, [r[5] for r in rows], [r[6] for r in rows], r2g)
        assert got == want, f"read_{f}"
        chains_seen += len(want)
    assert chains_seen >= 40
