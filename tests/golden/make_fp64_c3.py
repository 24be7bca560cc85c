"""FP64 amplitudes of the benchmark workload (7x7 grid, depth (1+32+1), two
cuts with 4 values each) for its first output strings, computed with the
oracle in complex128 and exact (double) gate constants:

    python tests/golden/make_fp64_c3.py [count (default 16)]

bench.py compares the amplitudes it computes for these strings with this
file and reports the largest relative error.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import qflex_oracle as qo  # noqa: E402
from qflex_gb300 import rqc  # noqa: E402


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 16
    circuit, ordering, grid, initial, finals = rqc.workload("c3")
    path = Path(__file__).resolve().parent / "c3_fp64.json"
    # Strings already in the file are kept; the next ones are appended (the
    # file is rewritten after each string, so an interrupted run resumes).
    out = json.loads(path.read_text())["amplitudes"] if path.exists() else []
    assert [r["final"] for r in out] == finals[:len(out)]
    for f in finals[len(out):count]:
        t = time.time()
        inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), initial, f)
        a = qo.evaluate_circuit(inp, np.complex128, float(1 << 40))[0][1]
        out.append({"final": f, "amplitude": [a.real, a.imag]})
        print(f, a, f"{time.time() - t:.1f} s", flush=True)
        with open(path, "w") as fh:
            json.dump({"workload": "c3", "initial": initial, "amplitudes": out}, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
