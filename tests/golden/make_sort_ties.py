#!/usr/bin/env python3
"""Generate the committed fixture of libstdc++ std::sort tie orders as the
reference restates them in Python (``cpp_sort_in_place`` in
``tools/replay_read_to_graph_source_pack.py``), for seeded key sets with
heavy ties.  Run where the reference checkout is present (``--reference
DIR`` or the ``CUFLYE_REFERENCE`` environment variable); the tests only read
``sort_ties.json``.

Usage: python tests/golden/make_sort_ties.py [--reference DIR]
"""

from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "sort_ties.json"
SIZES = (3, 17, 40, 300, 2000)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("CUFLYE_REFERENCE"),
                    required=not os.environ.get("CUFLYE_REFERENCE"),
                    help="the reference checkout (default: $CUFLYE_REFERENCE)")
    args = ap.parse_args()
    tool = Path(args.reference) / "tools" / "replay_read_to_graph_source_pack.py"
    sys.path.insert(0, str(tool.parent))
    spec = importlib.util.spec_from_file_location("rsp", tool)
    rsp = importlib.util.module_from_spec(spec)
    sys.modules["rsp"] = rsp
    spec.loader.exec_module(rsp)
    rng = np.random.default_rng(5)
    cases = []
    for n in SIZES:
        keys = rng.integers(0, max(2, n // 8), size=n).astype(np.uint64).tolist()
        items = list(zip(keys, range(n)))
        rsp.cpp_sort_in_place(items, lambda a, b: a[0] < b[0])
        cases.append({"keys": keys, "values_after_sort": [v for _, v in items]})
    OUT.write_text(json.dumps({"source": "tools/replay_read_to_graph_source_pack.py "
                                         "cpp_sort_in_place", "cases": cases}) + "\n")
    print(f"wrote {OUT} ({len(cases)} cases)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
