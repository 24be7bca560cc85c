"""Generates tests/golden/input_errors.json: seeded malformed (and a few
valid) circuit / ordering / grid / state inputs, each run through the
unmodified reference, built by oracle/Makefile into oracle/_ref/qflex_ref.

Every case records the reference's outcome: the output states of a valid
input, or the innermost message of the error it throws (the text after the
last "--> " of its nested "Failed to call X()" chain, which names the
reference's own source paths and is not kept). Inputs on which the reference
itself crashes instead of throwing are recorded apart; those on which its
behaviour is undefined (UNDEFINED below) are recorded apart, with the reason,
and are no parity target.

    python tests/golden/make_input_errors.py
"""
from __future__ import annotations

import json
import random
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tests.golden.make_golden import REF, run_ref  # noqa: E402

OUT = ROOT / "tests" / "golden" / "input_errors.json"

# A valid 2x3 instance: six active qubits, depth (1+4+1).
GRID = "1 1 1\n1 1 1\n"
CIRCUIT = """6
0 h 0
0 h 1
0 h 2
0 h 3
0 h 4
0 h 5
1 cz 0 1
1 t 2
1 cz 3 4
2 x_1_2 0
2 cz 1 2
2 y_1_2 5
3 cz 0 3
3 t 4
4 cz 2 5
4 fsim(0.25, 0.1) 1 4
5 h 0
5 h 1
5 h 2
5 h 3
5 h 4
5 h 5
"""
ORDERING = "expand a 0\nexpand a 1\nexpand a 2\nexpand a 3\nexpand a 4\nexpand a 5\n"
TERMINAL_ORDERING = ("expand a 0\nexpand a 1\nexpand a 2\nexpand a 3\n"
                     "cut () 4\ncut () 5\nexpand b 4\nexpand b 5\nmerge a b\n")


# Inputs on which the reference's behaviour is undefined, so that they are
# no parity target (the engine refuses them with its own message instead).
UNDEFINED = {
    "circuit: fsim with one parameter":
        "the reference reads params[1] of a one-element vector (src/read_circuit.cpp:156-158)",
    "ordering: expand without patch":
        "the reference reads the qubit index from an exhausted stream into an uninitialized "
        "variable (src/contraction_utils.cpp:390-396)",
}


def innermost(message: str) -> str:
    text = message.rstrip().rstrip("]").rstrip()
    return text.rsplit("--> ", 1)[-1].strip()


def circuit_mutations(rng: random.Random):
    lines = CIRCUIT.splitlines()
    body = list(range(1, len(lines)))
    out = []
    for _ in range(4):
        i = rng.choice(body)
        parts = lines[i].split()
        bad = rng.choice(["foo", "cz3", "hh", "rz", "x_1_3", "CZ"])
        out.append(("bad gate name", "\n".join(lines[:i] + [" ".join([parts[0], bad] + parts[2:])] + lines[i + 1:])))
    out.append(("too many qubits declared", "7\n" + "\n".join(lines[1:])))
    out.append(("too few qubits declared", "5\n" + "\n".join(lines[1:])))
    out.append(("missing qubit count", "\n".join(lines[1:])))
    out.append(("two-qubit gate missing a qubit", CIRCUIT.replace("1 cz 0 1", "1 cz 0")))
    out.append(("qubit used twice in a cycle", CIRCUIT.replace("1 t 2", "1 t 1")))
    out.append(("cycle decreases", CIRCUIT.replace("3 t 4", "1 t 4")))
    out.append(("unmatched parenthesis", CIRCUIT.replace("fsim(0.25, 0.1)", "fsim(0.25, 0.1")))
    out.append(("qubit outside the grid", CIRCUIT.replace("2 y_1_2 5", "2 y_1_2 9")))
    out.append(("non-numeric cycle", CIRCUIT.replace("3 t 4", "c t 4")))
    out.append(("non-numeric qubit", CIRCUIT.replace("3 t 4", "3 t q")))
    out.append(("gate without qubits", CIRCUIT.replace("3 t 4", "3 t")))
    out.append(("fsim with one parameter", CIRCUIT.replace("fsim(0.25, 0.1)", "fsim(0.25)")))
    out.append(("comments and blank lines (valid)", CIRCUIT.replace("3 t 4", "3 t 4  # a comment\n\n")))
    out.append(("three qubits on a cz", CIRCUIT.replace("1 cz 0 1", "1 cz 0 1 2")))
    out.append(("cx on one qubit", CIRCUIT.replace("1 t 2", "1 cx 2")))
    out.append(("half of a cz on one qubit", CIRCUIT.replace("1 t 2", "1 cz_q1 2")))
    out.append(("one-qubit gate on two qubits", CIRCUIT.replace("3 t 4", "3 t 4 5")))
    return out


def ordering_mutations(rng: random.Random):
    L = ORDERING.splitlines()
    out = []
    out.append(("unknown operation", ORDERING.replace("expand a 3", "contract a 3")))
    out.append(("qubit outside the grid", ORDERING.replace("expand a 3", "expand a 11")))
    out.append(("qubit expanded twice", ORDERING.replace("expand a 3", "expand a 2")))
    out.append(("qubit never expanded", "\n".join(L[:-1]) + "\n"))
    out.append(("cut values not comma-separated", "cut (0 1) 0 1\n" + ORDERING))
    out.append(("cut missing parenthesis", "cut 0,1 0 1\n" + ORDERING))
    out.append(("cut of non-neighbours", "cut () 0 5\n" + ORDERING))
    out.append(("cut after expansion", "expand a 0\ncut () 0 1\n" + "\n".join(L[1:]) + "\n"))
    out.append(("cut value too large", "cut (5) 0 1\n" + ORDERING))
    out.append(("cut twice", "cut () 0 1\ncut () 1 0\n" + ORDERING))
    out.append(("merge of an unknown patch", ORDERING + "merge a z\n"))
    out.append(("expand without patch", ORDERING.replace("expand a 3", "expand 3")))
    out.append(("terminal cut and patch (valid)", TERMINAL_ORDERING))
    out.append(("bond cut with a partial list (valid)", "cut (1) 0 1\n" + ORDERING))
    shuffled = L[:]
    rng.shuffle(shuffled)
    out.append(("shuffled sweep (valid)", "\n".join(shuffled) + "\n"))
    return out


def format_variants():
    """Formatting that real input files carry: (what, circuit, ordering, grid)."""
    crlf = lambda t: t.replace("\n", "\r\n")  # noqa: E731
    return [
        ("CRLF line endings in the circuit", crlf(CIRCUIT), ORDERING, GRID),
        ("CRLF line endings in the ordering", CIRCUIT, crlf(ORDERING), GRID),
        ("CRLF line endings in the grid", CIRCUIT, ORDERING, crlf(GRID)),
        ("tabs between circuit tokens", CIRCUIT.replace("1 cz 0 1", "1\tcz\t0\t1"), ORDERING, GRID),
        ("leading spaces in the circuit", CIRCUIT.replace("3 t 4", "   3 t 4"), ORDERING, GRID),
        ("trailing spaces in the circuit", CIRCUIT.replace("3 t 4", "3 t 4   "), ORDERING, GRID),
        ("spaces inside gate parameters", CIRCUIT.replace("fsim(0.25, 0.1)", "fsim( 0.25 , 0.1 )"), ORDERING, GRID),
        ("comment lines in the ordering", CIRCUIT, "# sweep\n" + ORDERING.replace("expand a 3", "# here\nexpand a 3"),
         GRID),
        ("blank lines in the ordering", CIRCUIT, ORDERING.replace("expand a 3\n", "expand a 3\n\n"), GRID),
        ("trailing blank lines in the grid", CIRCUIT, ORDERING, GRID + "\n\n"),
        ("extra spaces in the grid", CIRCUIT, ORDERING, "1  1 1\n 1 1 1\n"),
        ("tabs in the ordering", CIRCUIT, ORDERING.replace("expand a 3", "expand\ta\t3"), GRID),
    ]


def grid_mutations():
    return [
        ("ragged grid", "1 1 1\n1 1\n"),
        ("invalid character", "1 1 1\n1 2 1\n"),
        ("switched-off qubit the circuit uses", "1 1 1\n1 1 0\n"),
        ("empty grid", ""),
    ]


def state_mutations():
    return [
        ("initial state too short", "00000", ""),
        ("initial state too long", "0000000", ""),
        ("final state too short", "", "00000"),
        ("invalid character in initial state", "0a0000", ""),
        ("invalid character in final state", "", "01201x"),
        ("terminal x on a non-terminal qubit", "", "x00000"),
        ("valid states", "010101", "110011"),
    ]


def main() -> None:
    if not REF.exists():
        sys.exit(f"{REF} missing: run `make -C oracle ref REFERENCE=<qflex project>` first")
    rng = random.Random(20261204)
    inputs = []
    for what, c in circuit_mutations(rng):
        inputs.append(("circuit: " + what, c, ORDERING, GRID, "", ""))
    for what, o in ordering_mutations(rng):
        inputs.append(("ordering: " + what, CIRCUIT, o, GRID, "", ""))
    for what, g in grid_mutations():
        inputs.append(("grid: " + what, CIRCUIT, ORDERING, g, "", ""))
    for what, c, o, g in format_variants():
        inputs.append(("format: " + what, c, o, g, "", ""))
    for what, ini, fin in state_mutations():
        inputs.append(("states: " + what, CIRCUIT, ORDERING, GRID, ini, fin))
    for what, ini, fin in (("terminal states", "", "0101xx"), ("terminal x in a cut-free qubit", "", "x101xx")):
        inputs.append(("states: " + what, CIRCUIT, TERMINAL_ORDERING, GRID, ini, fin))
    cases, undefined, crashed = [], [], []
    for name, c, o, g, ini, fin in inputs:
        rec = {"name": name, "circuit": c, "ordering": o, "grid": g, "initial": ini, "final": fin}
        try:
            r = run_ref(c, o, g, ini, fin, "1GB")
        except RuntimeError:
            crashed.append(rec)
            continue
        if "error" in r:
            rec["error"] = innermost(r["error"])
        else:
            rec["states"] = r["states"]
        if name in UNDEFINED:
            undefined.append(dict(rec, why=UNDEFINED[name]))
        else:
            cases.append(rec)
    OUT.write_text(json.dumps({"cases": cases, "reference_undefined": undefined, "reference_crashed": crashed},
                              indent=1) + "\n")
    print(f"{len(cases)} cases ({sum('error' in c for c in cases)} errors), {len(undefined)} undefined, "
          f"reference crashed on {[c['name'] for c in crashed]}")


if __name__ == "__main__":
    main()
