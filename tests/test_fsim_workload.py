"""The fSim workload's generator, ordering and plan, on the CPU: circuit
structure, bookkeeping and product sequence against the reference's own
runs (tests/golden/fsim_cases.json), and the full-depth circuit's rejection
by the reference's memory check."""
import json
import re
from collections import Counter

import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import Context, QflexGb300Error, rqc
from tests.conftest import ROOT


@pytest.fixture(scope="module")
def fsim_cases():
    return {c["name"]: c for c in json.loads((ROOT / "tests" / "golden" / "fsim_cases.json").read_text())}


def test_patterns_cover_every_coupler_once():
    off = [(2, 3)]
    seen = Counter()
    for pat in "ABCD":
        for a, b in rqc.fsim_pattern_pairs(6, 9, pat, off):
            seen[(a, b)] += 1
            assert abs(a[0] - b[0]) + abs(a[1] - b[1]) == 1 and (2, 3) not in (a, b)
    # 6 x 8 horizontal + 5 x 9 vertical couplers, minus the 4 at the off site.
    assert len(seen) == 6 * 8 + 5 * 9 - 4 and set(seen.values()) == {1}


def test_fsim_circuit_structure():
    off = rqc.random_off_site(6, 9, 7)
    text = rqc.fsim_circuit(6, 9, 8, seed=0, off=[off])
    lines = text.splitlines()
    assert lines[0] == "53"
    fsims = [ln for ln in lines[1:] if "fsim" in ln]
    singles = [ln.split() for ln in lines[1:] if "fsim" not in ln]
    assert {s[1] for s in singles} == {"x_1_2", "y_1_2", "hz_1_2"}
    assert len(singles) == 53 * 9  # 8 layers before the couplers, one after
    per_pair = Counter(tuple(ln.split()[-2:]) for ln in fsims)
    assert set(per_pair.values()) == {2}  # ABCDCDAB: two fSims per coupler -> bond 16
    thetas, phis = zip(*[map(float, re.search(r"fsim\(([^,]+), ([^)]+)\)", ln).groups()) for ln in fsims])
    assert set(thetas) == {0.5}
    assert all(abs(p - 1 / 6) < 0.1 for p in phis) and len(set(phis)) > 50
    # No qubit's single-qubit gate repeats from one layer to the next.
    by_q = {}
    for t, g, q in singles:
        assert by_q.get(q) != g
        by_q[q] = g


def test_fsim_plan_matches_reference_products(built_lib, fsim_cases):
    case = fsim_cases["fsim_6x9_d8_one_slice"]
    ctx = Context(-1)
    ctx.set_option("open_terminals", 0)
    run = case["runs"][0]
    out = ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], run["final"],
                       qo.parse_memory(case["memory_limit"]))
    assert [s for s, _ in out] == run["states"]
    assert ctx.gemms() == [tuple(g) for g in run["gemms"]]


def test_fsim_workload_plan(built_lib, fsim_cases):
    circuit, ordering, grid, initial, finals = rqc.workload_c4()
    assert len(finals) == 64 and all(f.count("x") == 6 for f in finals)
    ctx = Context(-1)
    out = ctx.evaluate(circuit, ordering, grid, initial, finals[0], 1 << 40)
    st = ctx.stats()
    assert len(out) == 64 and st["n_leaves"] == 8 * 64
    # The region's amplitudes are those of the reference's terminal cuts.
    region = fsim_cases["fsim_6x9_d4_region"]["runs"][0]
    assert [s for s, _ in out] == region["states"]


def test_fsim_full_depth_is_rejected_by_the_memory_check(built_lib):
    """20 cycles put five fSims on every coupler (bond 1024): the reference's
    memory check (src/contraction_utils.cpp:147-155) refuses the plan before
    anything is allocated, as it would on the reference itself."""
    off = rqc.random_off_site(6, 9, 7)
    circuit = rqc.fsim_circuit(6, 9, 20, seed=0, off=[off])
    ctx = Context(-1)
    with pytest.raises(QflexGb300Error) as e:
        ctx.evaluate(circuit, rqc.ordering_6x9(off), rqc.grid_text(6, 9, [off]), "", "", 1 << 40)
    assert "too large" in str(e.value) or "exceeds memory limit" in str(e.value)
