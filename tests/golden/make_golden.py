#!/usr/bin/env python3
"""Generate the committed golden vectors that pin the CPU oracle.

Run where the reference checkout is present (``--reference DIR`` or the
``CUFLYE_REFERENCE`` environment variable);
the tests never run this script, they only read the fixtures it writes.
For each seeded synthetic case it:

1. builds the oracle's k-mer index and collects every query's candidate
   records in generation order;
2. replays chaining with the reference's own Python tools:
   * ``tools/replay_overlap_chains.py`` (``chain_target``; stable sorts,
     overhang checks, only_max_ext) on the candidates in Flye's sorted order,
   * ``tools/replay_read_to_graph_source_pack.py`` (``cpp_sort_in_place``
     libstdc++ emulation at every sort point, ``replay_group``) on the
     candidates in generation order;
3. writes the inputs and the reference tools' outputs under
   ``tests/golden/synthetic/<case>/``;
4. asserts the oracle reproduces both outputs.

Usage: python tests/golden/make_golden.py [--reference DIR]
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

from cuflye_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = REPO / "tests" / "golden" / "synthetic"

CASES = [
    # name, seed, genome, coverage, mean read length, k, errors (sub, ins, del), repeat
    ("ovl-a", 11, 40_000, 8.0, 5_000, 15, (0.01, 0.005, 0.005), False),
    ("ovl-b", 12, 50_000, 10.0, 6_000, 15, (0.01, 0.005, 0.005), True),
    ("ovl-c", 13, 40_000, 12.0, 4_000, 17, (0.002, 0.001, 0.001), True),
    ("ovl-d", 14, 30_000, 6.0, 3_000, 11, (0.03, 0.01, 0.01), False),
]


def fmt9(x: float) -> str:
    return "0" if x == 0 else format(float(np.float32(x)), ".9g")


def write_reads(path: Path, reads: synth.ReadSet) -> None:
    with path.open("w") as fh:
        for i in range(reads.n):
            fh.write(f"{int(reads.ids[i])}\t{reads.seq(i).decode()}\n")


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("CUFLYE_REFERENCE"),
                    required=not os.environ.get("CUFLYE_REFERENCE"),
                    help="the reference checkout (default: $CUFLYE_REFERENCE)")
    args = ap.parse_args()
    sys.path.insert(0, str(Path(args.reference) / "tools"))
    import replay_overlap_chains as ROC  # type: ignore
    import replay_read_to_graph_source_pack as RSP  # type: ignore

    OUT.mkdir(parents=True, exist_ok=True)
    summary = {}
    for name, seed, glen, cov, mlen, k, (sub, ins, dele), rep in CASES:
        wl = synth.small_overlap_case(seed, glen, cov, mlen, k, sub, ins, dele, rep)
        reads = wl.reads
        batch = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
        idx = O.Index.build(k, batch, wl.min_freq, wl.max_freq)
        lens = {int(reads.ids[i]): int(reads.offsets[i + 1] - reads.offsets[i])
                for i in range(reads.n)}
        gen = O.candidates(idx, batch, sorted_like_flye=False)
        srt = O.candidates(idx, batch, sorted_like_flye=True)
        cdir = OUT / name
        cdir.mkdir(parents=True, exist_ok=True)
        write_reads(cdir / "reads.tsv", reads)

        # --- pin 1: stable-sort replay (tools/replay_overlap_chains.py)
        params = dict(wl.params)
        manifest_params = {
            "kmer_size": k, "minimum_overlap": params["min_overlap"],
            "maximum_jump": params["max_jump"], "max_jump_gap": params["max_gap"],
            "chain_gap_jump_threshold": params["gap_jump_threshold"],
            "chain_large_gap_penalty": params["large_gap_penalty"],
            "chain_small_gap_penalty": params["small_gap_penalty"],
            "min_kmer_survival_rate": params["min_kmer_survival_rate"],
            "maximum_overhang": params["max_overhang"],
            "check_overhang": bool(params["check_overhang"]),
            "force_local": bool(params["force_local"]),
            "only_max_ext": bool(params["only_max_ext"]),
            "max_overlaps": params["max_overlaps"],
            "max_divergence": params["max_divergence"],
            "sample_rate": params["sample_rate"],
        }
        ref_stable: list[str] = []
        ref_cpp: list[str] = []
        O.set_stable(True)
        orc_stable: list[str] = []
        orc_cpp: list[str] = []
        qid_arr = srt["query_id"]
        starts = np.searchsorted(qid_arr, reads.ids, side="left") if len(qid_arr) else []
        for qi in range(reads.n):
            q = int(reads.ids[qi])
            qlen = lens[q]
            sel = srt["query_id"] == q
            fsel = gen["filtered_query"] == q
            filtered = sorted(int(x) for x in gen["filtered_pos"][fsel])
            cands = [ROC.Candidate(q, int(c), int(km), int(t), int(tp), "+" if t > 0 else "-")
                     for c, km, t, tp in zip(srt["query_pos"][sel], srt["kmer"][sel],
                                             srt["target_id"][sel], srt["target_pos"][sel])]
            manifest = {"query_id": q, "query_length": qlen, "parameters": manifest_params}
            s = 0
            det = []
            signed_lens = {**lens, **{-t: v for t, v in lens.items()}}
            while s < len(cands):
                e = s + 1
                while e < len(cands) and cands[e].target_id == cands[s].target_id:
                    e += 1
                det.extend(ROC.chain_target(cands[s:e], manifest, signed_lens, filtered))
                s = e
            ref_stable.extend(o.as_tsv() for o in det)
            r = O.chain_sorted(srt["query_pos"][sel], srt["target_pos"][sel],
                               srt["target_id"][sel], q, qlen, list(lens.keys()),
                               list(lens.values()), filtered, O.default_params(**params))
            for row, dv in zip(r["cols"], r["divergence"]):
                orc_stable.append("\t".join(str(int(v)) for v in row) + "\t" + fmt9(dv))
        O.set_stable(False)

        # --- pin 2: libstdc++ std::sort emulation (tools/replay_read_to_graph_source_pack.py)
        gp = O.default_params(**dict(params, check_overhang=0, only_max_ext=0, max_overhang=0))
        for qi in range(reads.n):
            q = int(reads.ids[qi])
            qlen = lens[q]
            sel = gen["query_id"] == q
            fsel = gen["filtered_query"] == q
            matches = [RSP.Match(int(c), int(tp), int(t), int(km), o)
                       for o, (c, km, t, tp) in enumerate(zip(
                           gen["query_pos"][sel], gen["kmer"][sel], gen["target_id"][sel],
                           gen["target_pos"][sel]))]
            RSP.cpp_sort_in_place(matches, RSP.less_match_by_ext_id_cur_pos)
            i = 0
            while i < len(matches):
                ext = matches[i].ext_id
                e = i + 1
                while e < len(matches) and matches[e].ext_id == ext:
                    e += 1
                det, _ = RSP.replay_group(q, qlen, ext, lens[abs(ext)], matches[i:e],
                                          kmer_size=k, max_jump=params["max_jump"],
                                          min_overlap=params["min_overlap"], force_local=False)
                for o in det:
                    ref_cpp.append("\t".join(str(v) for v in (
                        o.query_id, o.cur_begin, o.cur_end, o.cur_len, o.ext_id, o.ext_begin,
                        o.ext_end, o.ext_len, o.score)))
                i = e
            # oracle: no filtered positions (the replay's divergence has none)
            one = O.SeqBatch.from_strings([q], [reads.seq(qi)])
            # reuse the full index: only the query changes
            r = O.overlaps(idx, one, gp)
            for row in r["cols"]:
                orc_cpp.append("\t".join(str(int(v)) for v in row))

        (cdir / "ref.overlaps.stable.tsv").write_text("".join(x + "\n" for x in ref_stable))
        (cdir / "ref.overlaps.libstdcxx.tsv").write_text("".join(x + "\n" for x in ref_cpp))
        cand_text = "".join(
            f"{a}\t{b}\t{c}\t{d}\t{e}\t{'+' if d > 0 else '-'}\n"
            for a, b, c, d, e in sorted(zip(gen["query_id"].tolist(), gen["query_pos"].tolist(),
                                            gen["kmer"].tolist(), gen["target_id"].tolist(),
                                            gen["target_pos"].tolist())))
        meta = {
            "seed": seed, "genome_len": glen, "coverage": cov, "mean_read_len": mlen, "k": k,
            "errors": [sub, ins, dele], "repeat": rep, "min_freq": wl.min_freq,
            "max_freq": wl.max_freq, "params": params, "reads": reads.n,
            "candidate_records": int(len(gen["query_id"])),
            "candidate_canonical_sha256": hashlib.sha256(cand_text.encode()).hexdigest(),
            "filtered_positions": int(len(gen["filtered_pos"])),
            "ref_overlaps_stable": len(ref_stable), "ref_overlaps_libstdcxx": len(ref_cpp),
            "generator": "tests/golden/make_golden.py",
            "reference_tools": ["tools/replay_overlap_chains.py:chain_target",
                                "tools/replay_read_to_graph_source_pack.py:replay_group"],
        }
        (cdir / "meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
        ok1 = ref_stable == orc_stable
        ok2 = ref_cpp == orc_cpp
        summary[name] = {"stable_match": ok1, "libstdcxx_match": ok2,
                         "overlaps": len(ref_stable), "candidates": meta["candidate_records"]}
        print(name, summary[name], flush=True)
        if not ok1:
            for a, b in zip(ref_stable, orc_stable):
                if a != b:
                    print(" stable ref ", a, "\n stable orc ", b)
                    break
        if not ok2:
            for a, b in zip(ref_cpp, orc_cpp):
                if a != b:
                    print(" cpp ref ", a, "\n cpp orc ", b)
                    break
    return 0 if all(v["stable_match"] and v["libstdcxx_match"] for v in summary.values()) else 1


if __name__ == "__main__":
    raise SystemExit(main())
