"""Regenerate tests/golden/reference_artifacts.json from the gravis checkout.

The reference publishes three numeric artefacts produced by its own CPU code:
  artifacts/benchmarks/m1_kepler_diag.csv      (TwoBody e=0.5, 1e5 KDK steps)
  artifacts/benchmarks/m1_plummer_1k_diag.csv  (Plummer N=1000 seed 42, 1000 steps)
  artifacts/benchmarks/m3_accuracy.csv         (Barnes-Hut vs BruteForce error)
This script copies their rows verbatim (as strings and parsed floats) into a
JSON fixture so the tests can run where the reference is not mounted.

Usage: python tests/golden/make_golden.py <path-to-gravis-checkout>
"""
import csv
import json
import os
import sys

FILES = ("m1_kepler_diag.csv", "m1_plummer_1k_diag.csv", "m3_accuracy.csv")


def main(root: str) -> None:
    out = {}
    for name in FILES:
        path = os.path.join(root, "artifacts", "benchmarks", name)
        with open(path, newline="") as fh:
            rows = list(csv.reader(fh))
        header, body = rows[0], rows[1:]
        out[name] = {"source": f"artifacts/benchmarks/{name}", "header": header,
                     "rows": [[float(v) if v != "" else None for v in r] for r in body],
                     "raw": [",".join(r) for r in body]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_artifacts.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path-to-gravis-checkout>")
    main(sys.argv[1])
