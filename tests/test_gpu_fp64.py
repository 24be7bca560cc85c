"""The complex128 contraction (the FP64 GPU oracle) through the C ABI.

Both arithmetic modes -- FP64 FMAs throughout (QFLEX_GB300_FP64) and
float-float tiled products (QFLEX_GB300_FP64_FF) -- are pinned against the
numpy complex128 oracle on the reference's fixture cases, and against each
other and the CPU complex128 oracle on the full 16-slice 7x7 (1+32+1)
workload. The complex64 paths' per-amplitude errors are measured against
this oracle (tests/golden/c3_fp64_gpu.json, bench.py)."""
import json

import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import FP64, FP64_FF, Context, QflexGb300Error, rqc
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

# Per-amplitude relative error allowed between two complex128 contractions
# (different summation orders; ff products carry ~44 significant bits).
FP64_TOL = 1e-9

CASES = ["simple", "c1_4x5_d16", "rect4x4_cut_terminal", "c2_6x6_d24_partial_cut", "fsim_3x4_off",
         "c3_7x7_d32_one_slice"]


def _oracle128(circuit, ordering, grid, initial, final, limit=float(1 << 40)):
    inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), initial, final)
    return qo.evaluate_circuit(inp, np.complex128, limit)


def _max_rel(got, want):
    g = np.asarray(got, dtype=np.complex128)
    w = np.asarray(want, dtype=np.complex128)
    return float(np.max(np.abs(g - w) / np.abs(w)))


@pytest.mark.parametrize("precision", [FP64, FP64_FF])
@pytest.mark.parametrize("name", CASES)
def test_fp64_paths_match_numpy_complex128(built_lib, ref_cases, name, precision):
    case = ref_cases[name]
    ctx = Context(0, precision)
    for run in case["runs"]:
        out = ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], run["final"],
                           1 << 40)
        want = _oracle128(case["circuit"], case["ordering"], case["grid"], case["initial"], run["final"])
        # Bookkeeping is the same as on every path, bit for bit.
        assert [s for s, _ in out] == [s for s, _ in want] == run["states"]
        assert ctx.initial_state() == run["initial_out"] and ctx.final_state() == run["final_out"]
        err = _max_rel([a for _, a in out], [a for _, a in want])
        assert err < FP64_TOL, (name, precision, err)


def test_fp64_paths_on_the_16_slice_workload(built_lib):
    """Full 7x7 (1+32+1) workload, both cuts with 4 values (16 slices): the
    float-float mode against the CPU complex128 oracle on the first four
    strings of tests/golden/c3_fp64.json, and against the native FP64 mode
    on one."""
    ref = json.loads((ROOT / "tests" / "golden" / "c3_fp64.json").read_text())
    circuit, ordering, grid, initial, finals = rqc.workload("c3")
    assert ref["initial"] == initial
    strings = [r["final"] for r in ref["amplitudes"][:4]]
    want = [complex(*r["amplitude"]) for r in ref["amplitudes"][:4]]
    ff = Context(0, FP64_FF)
    got = [a for _, a in ff.evaluate_many(circuit, ordering, grid, initial, strings, 1 << 40)]
    assert _max_rel(got, want) < FP64_TOL
    native = Context(0, FP64)
    one = native.evaluate(circuit, ordering, grid, initial, strings[0], 1 << 40)[0][1]
    assert _max_rel([one], [want[0]]) < FP64_TOL
    assert _max_rel([one], [got[0]]) < FP64_TOL


def test_complex64_tensor_ops_refused_in_fp64_mode(built_lib):
    import torch
    ctx = Context(0, FP64)
    a, b, c = (torch.zeros((64, 64), dtype=torch.complex64, device="cuda") for _ in range(3))
    with pytest.raises(QflexGb300Error) as e:
        ctx.multiply(a.data_ptr(), b.data_ptr(), c.data_ptr(), 64, 64, 64)
    assert "complex64" in str(e.value)
