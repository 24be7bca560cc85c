"""The fSim workload: 6 x 9 grid with one disabled site (53 qubits),
fSim(pi/2, pi/6 + jitter) couplers on four alternating patterns, three cuts
with partial value lists and a 6-qubit output region kept open, so that one
contraction gives 64 amplitudes.

Parity: the FP32 path against the reference's own outputs on two reduced
cases (tests/golden/fsim_cases.json, made by oracle/_ref/qflex_ref), every
path against the FP64 GPU oracle, and one prefix of the full workload (8
slices, 64 amplitudes) in 3xFP16 against the FP64 GPU oracle."""
import json

import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import FP16X3, FP32, FP64_FF, Context, rqc
from tests.conftest import ROOT, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def fsim_cases():
    return {c["name"]: c for c in json.loads((ROOT / "tests" / "golden" / "fsim_cases.json").read_text())}


@pytest.mark.parametrize("name", ["fsim_6x9_d4_region", "fsim_6x9_d8_one_slice"])
def test_fsim_cases_match_reference_and_fp64(built_lib, fsim_cases, name):
    case = fsim_cases[name]
    limit = qo.parse_memory(case["memory_limit"])
    run = case["runs"][0]
    want = [complex(*a) for a in run["amplitudes"]]
    results = {}
    for precision in (FP32, FP16X3, FP64_FF):
        ctx = Context(0, precision)
        out = ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], run["final"], limit)
        assert [s for s, _ in out] == run["states"]
        assert ctx.final_state() == run["final_out"]
        results[precision] = [a for _, a in out]
    # The reference's complex<float> results, and the FP64 oracle.
    assert rel_err(results[FP32], want) < TOL
    assert rel_err(results[FP64_FF], want) < TOL
    assert rel_err(results[FP16X3], results[FP64_FF]) < TOL


def test_fsim_workload_prefix_against_fp64(built_lib):
    """One string prefix of the full workload: 8 slices, 64 amplitudes from
    one contraction with the region open, in 3xFP16 against the complex128
    contraction of the same network."""
    circuit, ordering, grid, initial, finals = rqc.workload_c4()
    fast = Context(0, FP16X3)
    got = fast.evaluate_many(circuit, ordering, grid, initial, finals[:1], 1 << 40)
    assert len(got) == 64 and fast.stats()["n_leaves"] == 512
    wide = Context(0, FP64_FF)
    want = wide.evaluate_many(circuit, ordering, grid, initial, finals[:1], 1 << 40)
    assert [s for s, _ in got] == [s for s, _ in want]
    a = np.array([x for _, x in got])
    b = np.array([x for _, x in want])
    assert rel_err(a, b) < TOL
    # The region's 64 amplitudes are those of 64 fully specified strings.
    region = [k for k, ch in enumerate(finals[0]) if ch == "x"]
    assert len(region) == 6 and all(s[k] in "01" for s, _ in got for k in region)
