"""FP64-oracle amplitudes of the benchmark workload (7x7 grid, depth
(1+32+1), two cuts with 4 values each = 16 slices) for its first output
strings, computed on the GPU by the complex128 contraction:

    python tests/golden/make_fp64_c3_gpu.py [--count 256] [--out PATH]

The float-float mode (QFLEX_GB300_FP64_FF) computes every string; the
native FP64 mode recomputes the first --native strings, and the strings
that tests/golden/c3_fp64.json holds (CPU numpy complex128 oracle) are
compared too. Both agreements are stored in the file, which bench.py and
the tests use to state the per-amplitude error of the complex64 paths.
Needs a GPU; strings are processed in batches and the file is rewritten
after each batch, so an interrupted run resumes where it stopped.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from qflex_gb300 import FP64, FP64_FF, Context, rqc  # noqa: E402


def max_rel(got, want):
    return max(abs(a - b) / abs(b) for a, b in zip(got, want))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--native", type=int, default=2)
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent / "c3_fp64_gpu.json"))
    args = ap.parse_args()
    circuit, ordering, grid, initial, finals = rqc.workload("c3")
    out = Path(args.out)
    doc = json.loads(out.read_text()) if out.exists() else {}
    rows = doc.get("amplitudes", [])
    assert [r["final"] for r in rows] == finals[:len(rows)]
    ff = Context(0, FP64_FF)
    dev_ms = doc.get("ff_device_ms", 0.0)
    while len(rows) < args.count:
        todo = finals[len(rows):min(args.count, len(rows) + args.batch)]
        t = time.time()
        res = ff.evaluate_many(circuit, ordering, grid, initial, todo, 1 << 40)
        dev_ms += ff.stats()["device_ms"]
        rows += [{"final": f, "amplitude": [a.real, a.imag]} for f, (_, a) in zip(todo, res)]
        print(f"{len(rows)} strings, {time.time() - t:.1f} s for {len(todo)}", flush=True)
        doc.update({"workload": "c3", "initial": initial, "precision": "fp64ff", "amplitudes": rows,
                    "ff_device_ms": dev_ms})
        out.write_text(json.dumps(doc, indent=0))
    got = {r["final"]: complex(*r["amplitude"]) for r in rows}
    # Cross-checks: native FP64 on the GPU, numpy complex128 on the CPU.
    native = Context(0, FP64)
    strings = finals[:args.native]
    t = time.time()
    nat = [a for _, a in native.evaluate_many(circuit, ordering, grid, initial, strings, 1 << 40)]
    doc["native_fp64"] = {"strings": len(strings), "max_rel_diff": max_rel([got[f] for f in strings], nat),
                          "device_ms": native.stats()["device_ms"], "seconds": time.time() - t}
    cpu = json.loads((ROOT / "tests" / "golden" / "c3_fp64.json").read_text())
    common = [r for r in cpu["amplitudes"] if r["final"] in got]
    doc["cpu_complex128"] = {"strings": len(common), "max_rel_diff": max_rel(
        [got[r["final"]] for r in common], [complex(*r["amplitude"]) for r in common])}
    out.write_text(json.dumps(doc, indent=0))
    print(json.dumps({k: v for k, v in doc.items() if k != "amplitudes"}))


if __name__ == "__main__":
    main()
