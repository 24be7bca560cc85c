"""The oracle (oracle/qflex_oracle.py, numpy) against the reference's own
outputs: golden fixtures produced by the unmodified reference build
(tests/golden/make_golden.py) and the reference's known-answer values."""
import numpy as np
import pytest

from oracle import qflex_oracle as qo
from tests.conftest import rel_err


def _run(case, final, dtype=np.complex64, log=None):
    inp = qo.Input(qo.Circuit.loads(case["circuit"]), qo.load_ordering(case["ordering"]),
                   qo.Grid.loads(case["grid"]), case["initial"], final)
    limit = qo.parse_memory(case["memory_limit"])
    out = qo.evaluate_circuit(inp, dtype, limit, log)
    return inp, out


def test_known_answer_simple_circuit():
    # tests/src/evaluate_circuit_test.cpp:199-206 (tolerance 1e-5 there).
    from tests.golden.make_golden import SIMPLE_CIRCUIT, SIMPLE_ORDERING, SIMPLE_GRID
    inp = qo.Input(qo.Circuit.loads(SIMPLE_CIRCUIT), qo.load_ordering(SIMPLE_ORDERING),
                   qo.Grid.loads(SIMPLE_GRID), "00000", "1100x")
    out = qo.evaluate_circuit(inp)
    assert [s for s, _ in out] == ["11000", "11001"]
    assert abs(out[0][1] - (0.10669 + 0.04419j)) < 1e-5 * 2
    assert abs(out[1][1] - (-0.01831 - 0.25758j)) < 1e-5 * 2


def test_multiply_known_answer():
    # tests/src/tensor_test.cpp:496-530: {20, 14, 100, 78}.
    a = qo.Tensor(["a", "b", "c"], [2, 2, 2], np.arange(8, dtype=np.complex64))
    b = qo.Tensor(["b", "c", "d"], [2, 2, 2], np.arange(8, 0, -1).astype(np.complex64))
    c = qo.multiply(a, b)
    assert c.indices == ["a", "d"] and c.dims == [2, 2]
    assert np.array_equal(c.data.real, np.array([20, 14, 100, 78], dtype=np.float32))


@pytest.mark.parametrize("name", ["simple", "c1_4x5_d16", "rect4x4_cut_terminal",
                                  "c2_6x6_d24_partial_cut", "fsim_3x4_off"])
def test_oracle_matches_reference(ref_cases, name):
    case = ref_cases[name]
    for run in case["runs"]:
        log = []
        inp, out = _run(case, run["final"], log=log)
        assert [s for s, _ in out] == run["states"]
        assert inp.initial_state == run["initial_out"]
        assert inp.final_state == run["final_out"]
        got = [a for _, a in out]
        want = [complex(*a) for a in run["amplitudes"]]
        assert rel_err(got, want) < 1e-5
        if run["gemms"]:
            contraction = log[len(log) - len(run["gemms"]):]
            assert [tuple(x[1:]) for x in contraction] == [tuple(g) for g in run["gemms"]]


def test_oracle_fp64_close_to_reference(ref_cases):
    case = ref_cases["c2_6x6_d24_partial_cut"]
    for run in case["runs"]:
        _, out = _run(case, run["final"], dtype=np.complex128)
        want = [complex(*a) for a in run["amplitudes"]]
        assert rel_err([a for _, a in out], want) < 1e-4


@pytest.mark.parametrize("name,fragment", [
    ("err_memory_limit", "exceeds memory limit"),
    ("err_cut_after_expand", "has to be equal to indices[0]"),
    ("err_bad_gate", "Invalid gate name provided: foo"),
    ("err_bad_op", "Received an invalid operation in config."),
])
def test_oracle_errors_match_reference(ref_cases, name, fragment):
    case = ref_cases[name]
    ref_msg = case["runs"][0]["error"]
    assert fragment in ref_msg
    with pytest.raises(qo.QflexError) as e:
        _run(case, case["runs"][0]["final"])
    assert fragment in str(e.value)


def test_planned_bytes_match_reference_message(ref_cases):
    case = ref_cases["err_memory_limit"]
    with pytest.raises(qo.QflexError) as e:
        _run(case, "")
    # "Required space (1.12 GB) exceeds memory limit (1 GB)"
    assert "Required space (" in case["runs"][0]["error"]
    ref_space = case["runs"][0]["error"].split("Required space (")[1].split(")")[0]
    assert f"Required space ({ref_space})" in str(e.value)
