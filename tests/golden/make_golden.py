"""Generates the golden fixtures in tests/golden/ from the unmodified
reference, built by oracle/Makefile into oracle/_ref/qflex_ref.

    make -C oracle ref REFERENCE=/path/to/qflex && python tests/golden/make_golden.py

Every case stores its inputs (circuit, ordering and grid texts: seeded
circuits from qflex_gb300.rqc, plus the known-answer circuit of the
reference's tests/src/evaluate_circuit_test.cpp:142-207), the reference's
outputs (states, complex amplitudes, mutated initial/final states) or its
error text, and the (m, n, k) of every CBLAS product the reference issued
inside ContractGrid.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import qflex_oracle as qo  # noqa: E402
from qflex_gb300 import rqc  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "qflex_ref"
OUT = Path(__file__).resolve().parent

# Known-answer case of the reference's tests (evaluate_circuit_test.cpp:142-207).
SIMPLE_CIRCUIT = """5
0 h 0
0 h 1
0 h 2
0 h 3
0 h 5
1 t 0
1 t 1
1 t 2
1 t 3
1 t 5
2 cz 0 1
3 cx 0 2
4 cx 1 3
5 cz 2 3
6 cz 3 5
11 cz 0 1
12 cx 0 2
13 cx 1 3
14 cz 2 3
15 cx 3 5
17 h 0
17 h 1
17 h 2
17 h 3
17 h 5
"""
SIMPLE_ORDERING = "#\ncut () 1 3\nexpand a 1\nexpand a 0\nexpand a 2\ncut () 5\nexpand b 5\nexpand b 3\nmerge a b\n"
SIMPLE_GRID = "1 1\n1 1\n0 1\n"


def run_ref(circuit, ordering, grid, initial, final, memory="64GB"):
    with tempfile.TemporaryDirectory() as d:
        paths = []
        for name, text in (("c", circuit), ("o", ordering), ("g", grid)):
            p = os.path.join(d, name)
            with open(p, "w") as f:
                f.write(text)
            paths.append(p)
        log = os.path.join(d, "gemm.log")
        env = dict(os.environ, QFLEX_REF_GEMM_LOG=log, OMP_NUM_THREADS="8")
        r = subprocess.run([str(REF), "eval", *paths, initial or "-", final or "-", memory],
                           capture_output=True, text=True, env=env)
        lines = r.stdout.splitlines()
        gemms = []
        if os.path.exists(log):
            with open(log) as f:
                gemms = [tuple(int(x) for x in ln.split()[1:]) for ln in f if ln.strip()]
    if r.returncode == 2:
        err = [ln for ln in lines if ln.startswith("ERROR ")]
        return {"error": err[0][6:] if err else r.stdout}
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    res = {"initial_out": lines[0].split(" ", 1)[1] if len(lines[0].split(" ", 1)) > 1 else "",
           "final_out": lines[1].split(" ", 1)[1] if len(lines[1].split(" ", 1)) > 1 else "",
           "states": [], "amplitudes": [], "gemms": gemms}
    for ln in lines[2:]:
        s, re, im = ln.split()
        res["states"].append(s)
        res["amplitudes"].append([float(re), float(im)])
    return res


def contraction_gemm_count(circuit, ordering, grid, initial, final):
    """Number of flatten products that precede ContractGrid in the
    reference's BLAS log (read from the oracle's restatement)."""
    inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid),
                   initial, final)
    ops = qo.parse_ordering(inp.ordering, inp.grid)
    n = inp.grid.I * inp.grid.J - len(inp.grid.qubits_off)
    init = initial or "0" * n
    base, fq, states = qo.output_states(inp.grid, ops, init, final)
    flog = []
    import numpy as np
    qo.build_grid(inp.circuit, inp.grid, init, base, fq, ops, np.complex64, flog)
    return len(flog)


def case(name, circuit, ordering, grid, initial, finals, memory="64GB", keep_gemms=True):
    runs = []
    for f in finals:
        r = run_ref(circuit, ordering, grid, initial, f, memory)
        if "gemms" in r:
            nf = contraction_gemm_count(circuit, ordering, grid, initial, f)
            r["gemms"] = r["gemms"][nf:] if keep_gemms else []
        runs.append(dict(final=f, **r))
        keep_gemms = False  # the product sequence does not depend on the final bits
    return {"name": name, "circuit": circuit, "ordering": ordering, "grid": grid,
            "initial": initial, "memory_limit": memory, "runs": runs}


def main():
    if not REF.exists():
        sys.exit(f"{REF} missing: run `make -C oracle ref` first")
    cases = []
    cases.append(case("simple", SIMPLE_CIRCUIT, SIMPLE_ORDERING, SIMPLE_GRID, "00000",
                      ["1100x", "0000x", ""]))
    # c1: 4x5, depth (1+16+1), row sweep, no cut.
    c, o, g, ini, fins = rqc.workload("c1", seed=0)
    cases.append(case("c1_4x5_d16", c, o, g, ini, fins[:16]))
    # 4x4 with one cut, two patches and two terminal cuts.
    c4 = rqc.random_circuit(4, 4, 16, seed=3)
    o4 = ("cut () 5 6\n" + "".join(f"expand a {q}\n" for q in (0, 1, 4, 5, 8, 9, 12, 13)) +
          "cut () 14\ncut (1) 15\n" + "".join(f"expand b {q}\n" for q in (3, 2, 7, 6, 11, 10, 15, 14)) +
          "merge a b\n")
    cases.append(case("rect4x4_cut_terminal", c4, o4, rqc.grid_text(4, 4),
                      rqc.random_bitstrings(16, 1, 9)[0],
                      ["0110" * 3 + "01xx", ""]))
    # 6x6, depth (1+24+1), central cut with a partial value list.
    c6 = rqc.random_circuit(6, 6, 24, seed=5)
    o6 = rqc.ordering_6x6(cut_values=(0, 3))
    cases.append(case("c2_6x6_d24_partial_cut", c6, o6, rqc.grid_text(6, 6), "",
                      rqc.random_bitstrings(36, 2, 11)))
    # fSim + hz_1_2 + rz on a 3x4 grid with one qubit off.
    off = [(1, 3)]
    fs = fsim_circuit(3, 4, off, seed=7)
    ofs = ("cut () 1 2\n" + "".join(f"expand a {q}\n" for q in (0, 4, 8, 1, 5, 9)) +
           "cut () 10\n" + "".join(f"expand b {q}\n" for q in (3, 2, 6, 10, 11)) + "merge a b\n")
    cases.append(case("fsim_3x4_off", fs, ofs, rqc.grid_text(3, 4, off), "",
                      ["0" * 11, "10110100101", ""]))
    # 7x7, depth (1+32+1): the benchmark ordering with one value per cut.
    c7 = rqc.random_circuit(7, 7, 32, seed=0)
    o7 = rqc.ordering_7x7((0,), (1,))
    cases.append(case("c3_7x7_d32_one_slice", c7, o7, rqc.grid_text(7, 7), "",
                      rqc.random_bitstrings(49, 1, 2)))
    # Errors the reference raises at run time.
    cases.append(case("err_memory_limit", c7, o7, rqc.grid_text(7, 7), "", [""], memory="1GB"))
    bad_cut = ("expand a 0\nexpand a 1\ncut () 1 2\nexpand b 2\nexpand b 3\nmerge a b\n")
    cases.append(case("err_cut_after_expand", rqc.random_circuit(1, 4, 8, 2), bad_cut,
                      rqc.grid_text(1, 4), "", [""]))
    cases.append(case("err_bad_gate", "2\n0 h 0\n1 foo 1\n", "expand a 0\nexpand a 1\n", "1 1\n", "", [""]))
    cases.append(case("err_bad_op", rqc.random_circuit(1, 2, 2, 0), "expand a 0\nswap a 1\n", "1 1\n", "",
                      [""]))
    with open(OUT / "reference_cases.json", "w") as f:
        json.dump(cases, f, indent=1)
    print(f"wrote {len(cases)} cases to {OUT / 'reference_cases.json'}")


def fsim_circuit(I, J, off, seed):
    """A small fSim-gate circuit (two-qubit fSim(pi/2, pi/6 + jitter) on the
    four coupler patterns, single-qubit x_1_2 / y_1_2 / hz_1_2 and rz)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    offs = set(map(tuple, off))
    act = [(i, j) for i in range(I) for j in range(J) if (i, j) not in offs]
    lines = [str(len(act))] + [f"0 h {i * J + j}" for i, j in act]
    cyc = 1
    for rnd in range(4):
        for i, j in act[:-1]:
            g = ["x_1_2", "y_1_2", "hz_1_2"][int(rng.integers(3))]
            lines.append(f"{cyc} {g} {i * J + j}")
        lines.append(f"{cyc} rz({rng.uniform(-1, 1):.6f}) {act[-1][0] * J + act[-1][1]}")
        cyc += 1
        pat = rqc.pattern_pairs(I, J, [1, 2, 3, 4][rnd % 4])
        for a, b in pat:
            if a in offs or b in offs:
                continue
            th, ph = 0.5, 1.0 / 6 + rng.normal(0, 0.05) / np.pi
            lines.append(f"{cyc} fsim({th:.6f},{ph:.6f}) {a[0] * J + a[1]} {b[0] * J + b[1]}")
        cyc += 1
    lines += [f"{cyc} h {i * J + j}" for i, j in act]
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    main()
