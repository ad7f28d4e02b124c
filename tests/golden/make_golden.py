"""Regenerate the golden vectors in this folder from the reference's own test fixtures.

The reference (lega0208/cuscan) pins its exact HDBSCAN path with 19 fixture cases produced by
``fast_hdbscan==0.3.2`` (``crates/hdbscan/tests/fixtures/{case}.npz`` + ``{case}.json``,
listed in ``manifest.json``). This script copies the arrays and parameters of each case, as
they are, into one compressed ``{case}.npz`` here plus ``manifest.json``, so that tests run
without the reference checkout. It also copies ``hdbscan_prediction.json`` (the
``approximate_predict`` fixture generated by the reference from the original ``hdbscan``
package: controlled trees, fitted models with candidate rows and expected predictions) as it is.
Run it where the reference checkout is available, passing its root directory:

    python tests/golden/make_golden.py <reference checkout root>
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def main(reference_root: str) -> None:
    fixtures = Path(reference_root) / "crates" / "hdbscan" / "tests" / "fixtures"
    manifest = json.loads((fixtures / "manifest.json").read_text())
    cases = []
    for case in manifest["cases"]:
        cid = case["id"]
        meta = json.loads((fixtures / f"{cid}.json").read_text())
        arrays = np.load(fixtures / f"{cid}.npz")
        out = {name: arrays[name] for name in arrays.files}
        np.savez_compressed(HERE / f"{cid}.npz", **out)
        cases.append({
            "id": cid,
            "n": case["n"],
            "dimensions": case["dimensions"],
            "params": meta.get("parameters", case["params"]),
            "manifest_params": case["params"],
            "status": case["status"],
            "divergence": case["divergence"],
            "tie_classification": meta.get("tie_classification"),
            "reason": meta.get("reason"),
        })
    (HERE / "hdbscan_prediction.json").write_text(
        (fixtures / "hdbscan_prediction.json").read_text())
    (HERE / "manifest.json").write_text(json.dumps({
        "source": "crates/hdbscan/tests/fixtures (lega0208/cuscan v0.1.3)",
        "generator": manifest["reference"]["package"] + "==" + manifest["reference"]["version"],
        "cases": cases,
    }, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout root>")
    main(sys.argv[1])
