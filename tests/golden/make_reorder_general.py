"""Reorders of tensors whose dimensions are not all powers of two, computed
by the unmodified reference (Tensor::reorder, which takes its naive path for
such dimensions, src/tensor.cpp:377-492 and :905), built by oracle/Makefile:

    python tests/golden/make_reorder_general.py

Each case holds the dimensions, the new order (new_order[i] = old position
of the index that goes to position i) and the reordered data of the tensor
whose element p is p. Writes tests/golden/reorder_general.json.
"""
from __future__ import annotations

import json
import math
import random
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref" / "qflex_ref"


def reference_reorder(dims, order):
    out = subprocess.run([str(REF), "reorder_dims", str(len(dims)), *map(str, dims), *map(str, order)],
                         capture_output=True, text=True, check=True)
    return [int(x) for x in out.stdout.split()]


def main():
    rng = random.Random(11)
    cases = [([3, 5, 2], [2, 0, 1]), ([6, 4, 3, 2, 5], [4, 2, 0, 3, 1]), ([7, 3], [1, 0]),
             ([1, 9, 1, 4], [3, 1, 0, 2]), ([5, 3, 6], [0, 1, 2])]
    for _ in range(5):
        r = rng.randint(2, 5)
        dims = [rng.randint(1, 7) for _ in range(r)]
        while r and math.prod(dims) > 1000:
            dims[rng.randrange(r)] = 1
        order = list(range(r))
        rng.shuffle(order)
        cases.append((dims, order))
    out = [{"dims": d, "new_order": o, "reordered": reference_reorder(d, o)} for d, o in cases]
    path = Path(__file__).resolve().parent / "reorder_general.json"
    path.write_text(json.dumps({"source": "oracle/_ref/qflex_ref reorder_dims", "cases": out}))
    print("wrote", path, len(out), "cases")


if __name__ == "__main__":
    main()
