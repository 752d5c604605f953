"""Copy the reference's recorded verification-suite metrics into a small fixture.

The reference recorded the results of its analytical verification suite for its
own float64 solver (artifacts/benchmark_results.json).  The cases whose set-up is
fully analytic (dam breaks, smooth hump, Thacker, bump, tilted plane, coupling
closure) are kept as regression targets for the CUDA engine; the lake-at-rest and
closed-storm cases ran on the reference's own city terrain and are left out.

    python tests/golden/extract_suite_metrics.py /root/reference
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

KEEP = ("2", "2b", "3", "4", "5", "6", "7")


def main(ref_root: str) -> None:
    src = Path(ref_root) / "artifacts" / "benchmark_results.json"
    data = json.loads(src.read_text())
    out = {"source": "reference artifacts/benchmark_results.json",
           "provenance": {k: data["provenance"][k] for k in ("device", "precision", "seed", "timestamp")},
           "results": {r["key"]: {"name": r["name"], "metrics": r["metrics"]} for r in data["results"]
                       if r["key"] in KEEP}}
    dst = Path(__file__).resolve().parent / "suite_recorded.json"
    dst.write_text(json.dumps(out, indent=1, sort_keys=True))
    print(f"wrote {dst} ({len(out['results'])} cases)")


if __name__ == "__main__":
    import os
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HIS_REFERENCE")
    if not root:
        raise SystemExit("usage: extract_suite_metrics.py <reference checkout>  (or set HIS_REFERENCE)")
    main(root)
