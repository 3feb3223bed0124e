"""Writes tests/golden/oracle_fixtures.npz from the CPU oracle.

The reference ships no golden vectors; its engine is pinned through libstdc++
(oracle/pin_mt.cpp).  These fixtures freeze the oracle's outputs for the cases
in tests/golden_cases.py so that any later change to the oracle or to the
library shows up as a diff.  manifest.json records the SHA-256 of the oracle
sources that produced them.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")]
import golden_cases  # noqa: E402
import pyoracle  # noqa: E402


def main():
    pyoracle.build()
    out = {name: golden_cases.run_oracle(pyoracle, c) for name, c in golden_cases.CASES.items()}
    np.savez_compressed(os.path.join(HERE, "oracle_fixtures.npz"), **out)
    h = hashlib.sha256()
    for f in ("oracle.c", "ormath.c", "oracle.h", "ormath_tables.h"):
        h.update(open(os.path.join(ROOT, "oracle", f), "rb").read())
    json.dump({"oracle_sha256": h.hexdigest(), "cases": sorted(out)}, open(os.path.join(HERE, "manifest.json"), "w"),
              indent=1)
    print(f"wrote {len(out)} fixtures")


if __name__ == "__main__":
    main()
