"""Seeded random quantum circuits, grids and orderings for the benchmark
workloads, written in the reference's text formats (docs/input_formats.md).

Circuit construction (rectangular I x J grid, all qubits active unless
``off`` is given):
  * cycle 0: Hadamard on every qubit;
  * cycles 1..depth: CZ gates on one of the 8 staggered nearest-neighbour
    coupler patterns, pattern (c - 1) mod 8. Horizontal patterns (odd c,
    r = (c - 1) / 2) couple (i, j)-(i, j+1) when (j - r - 2 (i mod 2)) mod 4
    is 0; vertical patterns couple (i, j)-(i+1, j) for c = 2 / 4 / 6 / 8
    when i is odd / even / odd / even and floor(i / 2) + j is even / even /
    odd / odd. These are the patterns of the shipped
    config/circuits/rectangular_*x*_1-*-1_0.txt files;
  * in cycle c a single-qubit gate goes on every qubit that is idle in c and
    was busy in c - 1 (the Hadamard layer counts as busy): T the first time
    on that qubit, afterwards drawn uniformly from {t, x_1_2, y_1_2} minus
    the qubit's previous single-qubit gate;
  * cycle depth + 1: Hadamard on every qubit.
"""
from __future__ import annotations

from typing import Iterable, List, Optional, Sequence, Tuple

import numpy as np

Coord = Tuple[int, int]


def pattern_pairs(I: int, J: int, cycle: int) -> List[Tuple[Coord, Coord]]:
    """CZ couplers of cycle ``cycle`` (>= 1) on an I x J grid."""
    c = (cycle - 1) % 8 + 1
    pairs = []
    if c % 2 == 1:
        r = (c - 1) // 2
        for i in range(I):
            for j in range(J - 1):
                if (j - r - 2 * (i % 2)) % 4 == 0:
                    pairs.append(((i, j), (i, j + 1)))
    else:
        want_odd_i = c in (2, 6)
        parity = 0 if c in (2, 4) else 1
        for i in range(I - 1):
            if (i % 2 == 1) != want_odd_i:
                continue
            for j in range(J):
                if (i // 2 + j) % 2 == parity:
                    pairs.append(((i, j), (i + 1, j)))
    return pairs


def random_circuit(I: int, J: int, depth: int, seed: int,
                   off: Iterable[Coord] = ()) -> str:
    """Circuit text of the construction above; qubits are numbered
    i * J + j (the reference's numbering, src/contraction_utils.cpp:521)."""
    rng = np.random.default_rng(seed)
    off = set(map(tuple, off))
    active = [(i, j) for i in range(I) for j in range(J) if (i, j) not in off]
    q = {p: p[0] * J + p[1] for p in active}
    lines = [str(len(active))]
    lines += [f"0 h {q[p]}" for p in active]
    cz_prev: set = set()       # qubits in a CZ in cycle c - 1
    sq_prev: dict = {}         # qubit -> single-qubit gate in cycle c - 1
    for cycle in range(1, depth + 1):
        pairs = [(a, b) for a, b in pattern_pairs(I, J, cycle) if a not in off and b not in off]
        busy = {p for ab in pairs for p in ab}
        for a, b in pairs:
            lines.append(f"{cycle} cz {q[a]} {q[b]}")
        sq = {}
        for p in active:
            if p in busy:
                continue
            if cycle == 1:
                g = "t"
            elif p in cz_prev:
                g = ("x_1_2", "y_1_2")[int(rng.integers(2))]
            elif sq_prev.get(p) in ("x_1_2", "y_1_2"):
                g = "t"
            else:
                continue
            sq[p] = g
            lines.append(f"{cycle} {g} {q[p]}")
        cz_prev, sq_prev = busy, sq
    lines += [f"{depth + 1} h {q[p]}" for p in active]
    return "\n".join(lines) + "\n"


def grid_text(I: int, J: int, off: Iterable[Coord] = ()) -> str:
    off = set(map(tuple, off))
    return "".join(" ".join("0" if (i, j) in off else "1" for j in range(J)) + "\n" for i in range(I))


def row_sweep_ordering(I: int, J: int, off: Iterable[Coord] = ()) -> str:
    """One patch expanded row by row, no cuts."""
    off = set(map(tuple, off))
    return "".join(f"expand a {i * J + j}\n" for i in range(I) for j in range(J) if (i, j) not in off)


def _vals(values: Optional[Sequence[int]]) -> str:
    return "(" + ",".join(str(v) for v in values) + ")" if values else "()"


def ordering_7x7(cut1_values: Optional[Sequence[int]] = None,
                 cut2_values: Optional[Sequence[int]] = None,
                 terminal_region: bool = False) -> str:
    """The 7x7 "alternative" contraction of arXiv:1811.09599 as spelled out in
    the reference's tests (tests/src/contraction_utils_test.cpp:306-374), with
    the second cut moved before the expansion of patch pC so that every cut
    precedes the expansion of its two tensors. Two cuts; each takes all bond
    values or the listed partial values. With ``terminal_region`` the six
    qubits of patch C become terminal cuts (64 amplitudes per contraction)."""
    def q(i, j):
        return i * 7 + j
    L = []
    for c in [(0, 0), (0, 1), (1, 0), (1, 1), (0, 2), (2, 0), (1, 2), (2, 1), (2, 2)]:
        L.append(f"expand A {q(*c)}")
    for c in [(6, 0), (5, 0), (4, 0), (3, 0), (6, 1), (5, 1), (4, 1), (3, 1)]:
        L.append(f"expand pB {q(*c)}")
    for c in [(6, 6), (6, 5), (5, 6), (5, 5), (6, 4), (4, 6), (5, 4), (4, 5), (4, 4)]:
        L.append(f"expand ppD {q(*c)}")
    L.append(f"cut {_vals(cut1_values)} {q(6, 2)} {q(6, 3)}")
    L.append("merge pB B")
    for c in [(6, 2), (5, 2), (4, 2), (3, 2)]:
        L.append(f"expand B {q(*c)}")
    L.append("merge A B")
    L.append("merge ppD pD")
    for c in [(6, 3), (5, 3), (4, 3)]:
        L.append(f"expand pD {q(*c)}")
    L.append(f"cut {_vals(cut2_values)} {q(2, 6)} {q(3, 6)}")
    for c in [(0, 6), (1, 6), (2, 6), (0, 5), (1, 5), (2, 5)]:
        L.append(f"expand pC {q(*c)}")
    L.append("merge pD D")
    for c in [(3, 6), (3, 5), (3, 4), (3, 3)]:
        L.append(f"expand D {q(*c)}")
    L.append("merge B D")
    region = [(0, 4), (1, 4), (2, 4), (0, 3), (1, 3), (2, 3)]
    if terminal_region:
        for c in region:
            L.append(f"cut () {q(*c)}")
    L.append("merge pC C")
    for c in region:
        L.append(f"expand C {q(*c)}")
    L.append("merge D C")
    return "\n".join(L) + "\n"


def random_bitstrings(n_qubits: int, count: int, seed: int) -> List[str]:
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2, size=(count, n_qubits))
    return ["".join("1" if b else "0" for b in row) for row in bits]


# ---- the benchmark workloads ----------------------------------------------

def workload(name: str, seed: int = 0):
    """(circuit, ordering, grid, initial_state, final_states) of a named
    workload.
      c1: 4x5 grid, depth (1+16+1), row sweep, no cut, 16 random strings.
      c2: 6x6 grid, depth (1+24+1), one cut on a central bond with the
          partial value list (0,1,2,3), 256 random strings.
      c3: 7x7 grid, depth (1+32+1), two cuts with values (0,1,2,3) each
          (16 slices), 1024 random strings.
    """
    if name == "c1":
        I, J, depth, n_out = 4, 5, 16, 16
        ordering = row_sweep_ordering(I, J)
    elif name == "c2":
        I, J, depth, n_out = 6, 6, 24, 256
        ordering = ordering_6x6(cut_values=(0, 1, 2, 3))
    elif name == "c3":
        I, J, depth, n_out = 7, 7, 32, 1024
        ordering = ordering_7x7((0, 1, 2, 3), (0, 1, 2, 3))
    else:
        raise ValueError(f"unknown workload {name!r}")
    circuit = random_circuit(I, J, depth, seed)
    n = I * J
    initial = random_bitstrings(n, 1, seed + 1)[0]
    finals = random_bitstrings(n, n_out, seed + 2)
    return circuit, ordering, grid_text(I, J), initial, finals


# ---- fSim circuits on a rectangular grid ----------------------------------

FSIM_PATTERNS = "ABCDCDAB"  # coupler pattern of cycle c is FSIM_PATTERNS[(c - 1) % 8]


def fsim_pattern_pairs(I: int, J: int, pattern: str, off: Iterable[Coord] = ()) -> List[Tuple[Coord, Coord]]:
    """Couplers of one of the four alternating patterns on an I x J grid:
    A horizontal (i, j)-(i, j+1) with j even, B the same with j odd, C
    vertical (i, j)-(i+1, j) with i even, D the same with i odd. Couplers
    touching an off site are left out. Every coupler of the grid belongs to
    exactly one pattern."""
    off = set(map(tuple, off))
    pairs = []
    if pattern in "AB":
        par = 0 if pattern == "A" else 1
        pairs = [((i, j), (i, j + 1)) for i in range(I) for j in range(J - 1) if j % 2 == par]
    elif pattern in "CD":
        par = 0 if pattern == "C" else 1
        pairs = [((i, j), (i + 1, j)) for i in range(I - 1) if i % 2 == par for j in range(J)]
    else:
        raise ValueError(pattern)
    return [(a, b) for a, b in pairs if a not in off and b not in off]


def random_off_site(I: int, J: int, seed: int) -> Coord:
    """One disabled site drawn from the grid's interior (seeded)."""
    rng = np.random.default_rng(seed)
    return (int(rng.integers(1, I - 1)), int(rng.integers(1, J - 1)))


def fsim_circuit(I: int, J: int, cycles: int, seed: int, off: Iterable[Coord] = (),
                 theta: float = 0.5, phi: float = 1.0 / 6.0, jitter_rad: float = 0.05) -> str:
    """Circuit text of an fSim random circuit: cycle c (1..cycles) is a layer
    of single-qubit gates on every active qubit at time 2c - 1, drawn
    uniformly from {x_1_2, y_1_2, hz_1_2} minus the qubit's previous one, and
    fSim(theta, phi + jitter) on the couplers of pattern
    FSIM_PATTERNS[(c - 1) % 8] at time 2c; a last single-qubit layer follows
    at time 2 cycles + 1. Angles are in units of pi, as the circuit format
    gives them (src/read_circuit.cpp:157-158); every coupler draws its own
    phase jitter once, from N(0, jitter_rad) radians. Each fSim splits into
    two tensors joined by a bond of dimension 4, so a coupler that gets g
    fSims carries a bond of 4^g."""
    rng = np.random.default_rng(seed)
    off = set(map(tuple, off))
    active = [(i, j) for i in range(I) for j in range(J) if (i, j) not in off]
    q = {p: p[0] * J + p[1] for p in active}
    jitter = {}
    for pat in "ABCD":
        for pair in fsim_pattern_pairs(I, J, pat, off):
            jitter[pair] = rng.normal(0.0, jitter_rad) / np.pi
    names = ["x_1_2", "y_1_2", "hz_1_2"]
    last = {p: None for p in active}
    lines = [str(len(active))]

    def single_layer(t):
        for p in active:
            choices = [g for g in names if g != last[p]]
            g = choices[int(rng.integers(len(choices)))]
            last[p] = g
            lines.append(f"{t} {g} {q[p]}")

    for c in range(1, cycles + 1):
        single_layer(2 * c - 1)
        for a, b in fsim_pattern_pairs(I, J, FSIM_PATTERNS[(c - 1) % 8], off):
            lines.append(f"{2 * c} fsim({theta!r}, {phi + jitter[(a, b)]!r}) {q[a]} {q[b]}")
    single_layer(2 * cycles + 1)
    return "\n".join(lines) + "\n"


def ordering_6x9(off: Coord, cut_values: Optional[Sequence[int]] = (0, 1), terminal_region: bool = True) -> str:
    """Column sweep of a 6 x 9 grid (one site off): columns 0-3 are
    contracted first (patch P, shared by every cut value), then three cuts on
    the couplers (0,4)-(0,5), (1,4)-(1,5), (2,4)-(2,5), each taking
    `cut_values` (None: all values), then P continues column by column. The
    six qubits of column 8 form the output region: with ``terminal_region``
    they are terminal cuts, so one contraction yields the region's 64
    amplitudes. Every cut precedes the expansion of its tensors and every
    merge goes into a patch created after the last cut, as the reference
    requires (src/contraction_utils.cpp:534-610)."""
    I, J = 6, 9

    def col(j):
        return [(i, j) for i in range(I) if (i, j) != tuple(off)]

    L = [f"expand P {i * J + j}" for j in range(4) for i, _ in col(j)]
    for i in range(3):
        L.append(f"cut {_vals(cut_values)} {i * J + 4} {i * J + 5}")
    if terminal_region:
        L += [f"cut () {i * J + 8}" for i, _ in col(8)]
    L.append("merge P L")
    L += [f"expand L {i * J + j}" for j in range(4, J) for i, _ in col(j)]
    return "\n".join(L) + "\n"


def workload_c4(seed: int = 0, cycles: int = 8, n_prefixes: int = 64):
    """The fSim workload: 6 x 9 grid with one seeded disabled site (53 active
    qubits), fsim_circuit(cycles) with fSim(pi/2, pi/6 + N(0, 0.05) rad),
    ordering_6x9 (3 cuts x 2 values = 8 slices) and `n_prefixes` random
    output strings whose last-column region is open ('x'): each gives the 64
    amplitudes of the strings that share its 47 other bits (4096 amplitudes
    for 64 prefixes). At 8 cycles every coupler carries 2 fSims (bond 16);
    20 cycles would put 5 on each (bond 1024, grid tensors of up to 2^40
    elements), which no grid contraction can hold."""
    I, J = 6, 9
    off = random_off_site(I, J, seed + 7)
    circuit = fsim_circuit(I, J, cycles, seed, off=[off])
    grid = grid_text(I, J, [off])
    ordering = ordering_6x9(off)
    active = [(i, j) for i in range(I) for j in range(J) if (i, j) != off]
    region = {k for k, p in enumerate(active) if p[1] == 8}
    initial = random_bitstrings(len(active), 1, seed + 1)[0]
    finals = ["".join("x" if k in region else b for k, b in enumerate(f))
              for f in random_bitstrings(len(active), n_prefixes, seed + 2)]
    return circuit, ordering, grid, initial, finals


# Real flop (8 m n k summed over the complex products) of one amplitude of
# the c3 workload, keyed by the number of cut slices summed: 16 for the
# workload's ordering, 4 for ordering_7x7((0,), (0, 1, 2, 3)) and 1 for
# ordering_7x7((0,), (0,)). They depend on the ordering only, not on the
# strings. The CPU baseline scales a timed sample of slices to the 16-slice
# amplitude with them.
C3_GEMM_FLOP = {16: 14910827790336.0, 4: 3964990390272.0, 1: 1772918145024.0}


def ordering_7x7_learned() -> str:
    """The learned cost model's choice for the c3 workload (same cuts and
    values as ordering_7x7((0, 1, 2, 3), (0, 1, 2, 3)), so the same
    amplitudes), kept in orderings/c3_learned.txt."""
    from pathlib import Path
    return (Path(__file__).resolve().parent / "orderings" / "c3_learned.txt").read_text()


def ordering_6x6(cut_values: Optional[Sequence[int]] = None) -> str:
    """6x6: cut the vertical bond (2,3)-(3,3) first, contract the top half
    (rows 0-2) and the bottom half (rows 5..3) as two patches, row by row
    towards the cut, then merge."""
    def q(i, j):
        return i * 6 + j
    L = [f"cut {_vals(cut_values)} {q(2, 3)} {q(3, 3)}"]
    for i in range(3):
        for j in range(6):
            L.append(f"expand T {q(i, j)}")
    for i in (5, 4, 3):
        for j in range(6):
            L.append(f"expand U {q(i, j)}")
    L.append("merge T U")
    return "\n".join(L) + "\n"
