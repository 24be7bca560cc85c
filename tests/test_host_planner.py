"""Host logic of the engine through the C ABI, without a GPU: a planning-only
context (device -1) parses, validates and plans exactly as a GPU context
does, so its output states, mutated input states, product sequence and
error texts are compared with the reference's golden fixtures."""
import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import FP32, Context, QflexGb300Error, rqc


@pytest.fixture(scope="module")
def plan_ctx(built_lib):
    """Planning-only context that contracts exactly as the reference does
    (terminal cuts projected per value), so its products are the
    reference's CBLAS calls."""
    ctx = Context(-1)
    ctx.set_option("open_terminals", 0)
    return ctx


CASES = ["simple", "c1_4x5_d16", "rect4x4_cut_terminal", "c2_6x6_d24_partial_cut",
         "fsim_3x4_off", "c3_7x7_d32_one_slice"]


@pytest.mark.parametrize("name", CASES)
def test_plan_matches_reference(plan_ctx, ref_cases, name):
    case = ref_cases[name]
    limit = qo.parse_memory(case["memory_limit"])
    for run in case["runs"]:
        out = plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"],
                                run["final"], limit)
        assert [s for s, _ in out] == run["states"]
        assert plan_ctx.initial_state() == run["initial_out"]
        assert plan_ctx.final_state() == run["final_out"]
        if run["gemms"]:
            assert plan_ctx.gemms() == [tuple(g) for g in run["gemms"]]


@pytest.mark.parametrize("name,fragment", [
    ("err_memory_limit", "Required space (1.12 GB) exceeds memory limit (1 GB). Cancelling simulation."),
    ("err_cut_after_expand", "Index: '(0,1),(0,2)' has to be equal to indices[0]: '(0,0),(0,1)'."),
    ("err_bad_gate", "Invalid gate name provided: foo"),
    ("err_bad_op", "Parsing failed on line: '' with error: Received an invalid operation in config."),
])
def test_errors_match_reference(plan_ctx, ref_cases, name, fragment):
    case = ref_cases[name]
    assert fragment in case["runs"][0]["error"]
    with pytest.raises(QflexGb300Error) as e:
        plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"],
                          case["runs"][0]["final"], qo.parse_memory(case["memory_limit"]))
    assert fragment in str(e.value)
    assert e.value.code == 1


def test_reference_plan_bytes_equal_oracle(plan_ctx, ref_cases):
    case = ref_cases["c3_7x7_d32_one_slice"]
    plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], "", "", 1 << 40)
    inp = qo.Input(qo.Circuit.loads(case["circuit"]), qo.load_ordering(case["ordering"]),
                   qo.Grid.loads(case["grid"]))
    ops = qo.parse_ordering(inp.ordering, inp.grid)
    base, fq, _ = qo.output_states(inp.grid, ops, "0" * 49, "")
    g2 = qo.build_grid(inp.circuit, inp.grid, "0" * 49, base, fq, ops, np.complex64)
    assert plan_ctx.stats()["reference_bytes"] == qo.planned_bytes(ops, g2)


def test_validation_errors(plan_ctx):
    c = rqc.random_circuit(2, 2, 4, 0)
    g = rqc.grid_text(2, 2)
    cases = [
        ("expand a 0\nexpand a 0\nexpand a 1\nexpand a 2\nexpand a 3\n", "is contracted multiple times"),
        ("expand a 0\ncut () 0 1\nexpand a 1\n", "is added to non-empty patch a after a cut"),
        ("cut (0,1 0 1\n", "Cut values must be comma-separated ints"),
        ("expand a 7\n", "Index 7 must be within grid boundaries."),
        ("cut () 0 1\ncut () 1 0\nexpand a 0\n", "is cut multiple times"),
    ]
    for ordering, fragment in cases:
        with pytest.raises(QflexGb300Error) as e:
            plan_ctx.evaluate(c, ordering, g, "", "", 1 << 30)
        assert fragment in str(e.value), (ordering, str(e.value))


def test_circuit_format_errors(plan_ctx):
    g = rqc.grid_text(1, 2)
    o = "expand a 0\nexpand a 1\n"
    for circuit, fragment in [
        ("2\n0 h 0\n0 h 0\n", "Qubits can only used once per cycle."),
        ("2\n1 h 0\n0 h 1\n", "Cycle number can only increase."),
        ("2\n0 h(0 0\n", "Not-matching parentheses."),
        ("2\n0 h\n", "Gate must be specified as"),
        ("2\n0 foo 0\n", "Invalid gate name provided: foo"),
        ("3\n0 h 0\n", "does not match the number of active qubits"),
        ("2\n0 cz 0 2\n", "must correspond to an active qubit"),
    ]:
        with pytest.raises(QflexGb300Error) as e:
            plan_ctx.evaluate(circuit, o, g, "", "", 1 << 30)
        assert fragment in str(e.value), (circuit, str(e.value))


def test_state_length_errors(plan_ctx):
    c = rqc.random_circuit(1, 2, 2, 0)
    with pytest.raises(QflexGb300Error) as e:
        plan_ctx.evaluate(c, "expand a 0\nexpand a 1\n", "1 1\n", "000", "", 1 << 30)
    assert "Size of initial_conf: 3, must be equal to the number of qubits: 2." in str(e.value)
    with pytest.raises(QflexGb300Error) as e:
        plan_ctx.evaluate(c, "expand a 0\nexpand a 1\n", "1 1\n", "00", "0", 1 << 30)
    assert "Size of final_conf: 1, must be equal to size of initial_conf: 2." in str(e.value)


def test_workload_plans(plan_ctx):
    """The benchmark workloads plan within the documented memory and work."""
    for name, max_gb in (("c1", 0.01), ("c2", 1.0), ("c3", 1.5)):
        c, o, g, ini, fins = rqc.workload(name)
        plan_ctx.evaluate(c, o, g, ini, fins[0], 1 << 40)
        s = plan_ctx.stats()
        assert s["arena_bytes"] < max_gb * 2 ** 30
        assert s["gemm_flop"] > 0


def _terminal_case(n_terminal=3):
    """4x5 (1+16+1) circuit: a row sweep of the first qubits into patch a,
    terminal cuts on the last `n_terminal` qubits, which patch b takes
    before it merges into a."""
    c, _, g, ini, fins = rqc.workload("c1", seed=9)
    qs = list(range(20))
    term = qs[-n_terminal:]
    lines = [f"expand a {q}" for q in qs[:-n_terminal]]
    lines += [f"cut () {q}" for q in term]
    lines += [f"expand b {q}" for q in term] + ["merge a b"]
    finals = []
    for f in fins[:3]:
        f = list(f)
        for q in term:
            f[q] = "x"
        finals.append("".join(f))
    return c, "\n".join(lines) + "\n", g, ini, finals


def test_open_terminal_plan_matches_projection(built_lib):
    """Terminal cuts as open indices: same output states, far fewer ops,
    the same amplitude for every leaf's value."""
    c, o, g, ini, finals = _terminal_case(3)
    res = {}
    for mode in (0, 1):
        plan = Context(-1, FP32)
        plan.set_option("open_terminals", mode)
        out = plan.evaluate(c, o, g, ini, finals[0], 1 << 40)
        res[mode] = ([s for s, _ in out], plan.stats())
    assert res[0][0] == res[1][0] and len(res[0][0]) == 8
    assert res[1][1]["n_leaves"] == res[0][1]["n_leaves"] == 8
    assert res[1][1]["n_ops"] < res[0][1]["n_ops"]


def test_open_terminals_fall_back_to_projection(built_lib):
    """A partial value list on a terminal cut keeps the reference's
    projection per value (same plan with the option on or off)."""
    c, o, g, ini, finals = _terminal_case(2)
    partial = o.replace("cut () 19", "cut (1) 19")
    p0, p1 = Context(-1, FP32), Context(-1, FP32)
    p0.set_option("open_terminals", 0)
    a = p0.evaluate(c, partial, g, ini, finals[0], 1 << 40)
    b = p1.evaluate(c, partial, g, ini, finals[0], 1 << 40)
    assert [s for s, _ in a] == [s for s, _ in b] and len(a) == 2
    assert p0.stats()["n_ops"] == p1.stats()["n_ops"]


def _sweep(I, J, off, order):
    """A one-patch sweep over the active qubits: row by row, column by
    column, or row by row snaking."""
    cells = []
    if order == "cols":
        cells = [(i, j) for j in range(J) for i in range(I)]
    else:
        for i in range(I):
            row = [(i, j) for j in range(J)]
            cells += row[::-1] if order == "snake" and i % 2 else row
    return [i * J + j for i, j in cells if (i, j) not in off]


@pytest.mark.parametrize("seed", range(16))
def test_random_plans_match_oracle(plan_ctx, seed):
    """Seeded random grids, depths, sweep orders, two-patch sweeps with a
    merge, two-qubit cuts (full or partial value lists) and terminal cuts:
    the planner's output states, mutated input states and product sequence
    equal the oracle's (the products after the oracle's flatten phase,
    which the engine runs as flatten_kernel instead)."""
    import random

    rng = random.Random(seed)
    I, J = rng.choice([(3, 3), (3, 4), (4, 3), (2, 5)])
    off = {(rng.randrange(I), rng.randrange(J))} if seed % 3 == 2 else set()
    depth = rng.choice([8, 12])
    circuit = rqc.random_circuit(I, J, depth, seed, off)
    grid = rqc.grid_text(I, J, off)
    seq = _sweep(I, J, off, rng.choice(["rows", "cols", "snake"]))
    n_term = rng.choice([0, 0, 1, 2])
    term = seq[len(seq) - n_term:] if n_term else []
    lines = []
    if seed % 2:
        # A cut on a bond between horizontal neighbours, placed before any
        # expansion of their tensors (a cut must precede them).
        pairs = [(i * J + j, i * J + j + 1) for i in range(I) for j in range(J - 1)
                 if (i, j) not in off and (i, j + 1) not in off
                 and i * J + j not in term and i * J + j + 1 not in term]
        q1, q2 = rng.choice(pairs)
        lines.append(f"cut ({rng.choice(['0,1', '1'])}) {q1} {q2}")
    main = seq[:len(seq) - n_term]
    if seed % 4 >= 2:
        # Two patches over the sweep's halves, the first merged into the second.
        half = len(main) // 2
        lines += [f"expand a {q}" for q in main[:half]] + [f"expand m {q}" for q in main[half:]]
        lines.append("merge a m")
        last = "m"
    else:
        lines += [f"expand a {q}" for q in main]
        last = "a"
    if term:
        lines += [f"cut () {q}" for q in term] + [f"expand t {q}" for q in term] + [f"merge {last} t"]
    ordering = "\n".join(lines) + "\n"
    active = [i * J + j for i in range(I) for j in range(J) if (i, j) not in off]
    final = list(rqc.random_bitstrings(len(active), 1, seed + 100)[0])
    for q in term:
        final[active.index(q)] = "x"
    final = "".join(final)
    initial = rqc.random_bitstrings(len(active), 1, seed + 200)[0]

    got = plan_ctx.evaluate(circuit, ordering, grid, initial, final, 1 << 40)
    log = []
    inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), initial, final)
    want = qo.evaluate_circuit(inp, np.complex64, float(1 << 40), log=log)
    assert [s for s, _ in got] == [s for s, _ in want]
    assert len(got) == 2 ** n_term
    assert plan_ctx.initial_state() == inp.initial_state
    assert plan_ctx.final_state() == inp.final_state
    gemms = plan_ctx.gemms()
    assert gemms and [tuple(x[1:]) for x in log[len(log) - len(gemms):]] == gemms


def _input_error_cases():
    import json

    from tests.conftest import ROOT
    return json.loads((ROOT / "tests" / "golden" / "input_errors.json").read_text())


def _squash(text):
    return " ".join(text.split())


@pytest.mark.parametrize("case", _input_error_cases()["cases"], ids=lambda c: c["name"])
def test_malformed_inputs_match_reference(plan_ctx, case):
    """Seeded malformed circuits, orderings, grids and states, and a few valid
    ones, against the unmodified reference's outcome
    (tests/golden/input_errors.json, made by make_input_errors.py): the same
    output states, or an error whose text contains the reference's innermost
    message (whitespace compared loosely: the reference's driver prints its
    multi-line messages on one line)."""
    run = lambda: plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"],  # noqa: E731
                                    case["initial"], case["final"], 1 << 30)
    if "error" in case:
        with pytest.raises(QflexGb300Error) as e:
            run()
        assert _squash(case["error"]) in _squash(str(e.value)), str(e.value)
    else:
        assert [s for s, _ in run()] == case["states"]


@pytest.mark.parametrize("case", _input_error_cases()["reference_undefined"], ids=lambda c: c["name"])
def test_inputs_undefined_in_the_reference_are_refused(plan_ctx, case):
    """Where the reference's behaviour is undefined (the fixture says why),
    the engine refuses the input with an error instead of computing."""
    with pytest.raises(QflexGb300Error):
        plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], case["final"],
                          1 << 30)


@pytest.mark.parametrize("case", _input_error_cases()["reference_crashed"], ids=lambda c: c["name"])
def test_inputs_that_crash_the_reference_are_refused(plan_ctx, case):
    """Inputs on which the reference crashes instead of throwing are refused
    with an error by the engine."""
    with pytest.raises(QflexGb300Error):
        plan_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], case["final"],
                          1 << 30)
