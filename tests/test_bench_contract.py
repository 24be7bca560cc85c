"""The bench's reference arm runs on the CPU alone: its JSON line carries the
keys of the bench contract (metric, unit, config.workload, cpu_baseline with
its kind, cores and sample, and an e2e object without host-device copies),
and the process never loads the product library."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

# Runs bench.py's reference arm in this process, then reports whether the
# product library was mapped into it.
_PROBE = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print(json.dumps({"product_library_loaded": "libqflex_gb300" in maps}))
"""


def test_reference_arm_json_line_without_product_library():
    out = subprocess.run([sys.executable, "-c", "import json\n" + _PROBE], capture_output=True, text=True,
                         check=True, timeout=900, cwd=ROOT)
    lines = out.stdout.strip().splitlines()
    line = json.loads(lines[-2])
    assert json.loads(lines[-1]) == {"product_library_loaded": False}
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["steps"] == 1 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    want_kind = "reference" if (ROOT / "oracle" / "_ref" / "qflex_ref").exists() else "port"
    assert cb["kind"] == want_kind and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert "4 of the 16 cut slices" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_workload_flop_constants(ref_cases):
    """The flop totals the CPU baseline scales its sample with: the planner's
    totals for the three orderings, and for one slice the sum over the
    products the reference itself handed to BLAS (its logged shapes)."""
    from qflex_gb300 import Context, rqc
    circuit, ordering, grid, initial, finals = rqc.workload("c3")
    plan = Context(-1)
    for slices, o in ((16, ordering), (4, rqc.ordering_7x7((0,), (0, 1, 2, 3))), (1, rqc.ordering_7x7((0,), (0,)))):
        plan.evaluate(circuit, o, grid, initial, finals[0], 1 << 40)
        assert plan.stats()["gemm_flop"] == rqc.C3_GEMM_FLOP[slices], slices
    case = ref_cases["c3_7x7_d32_one_slice"]
    assert sum(8 * m * n * k for m, n, k in case["runs"][0]["gemms"]) == rqc.C3_GEMM_FLOP[1]
