"""CPU oracle for the qFlex grid tensor-network contraction path.

TEST INFRASTRUCTURE ONLY. This module restates, in numpy, the reference's
algorithm for turning a circuit + grid + contraction ordering into output
amplitudes. Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may import it, and only as a checker; the product path
(``qflex_gb300``) never calls it.

Every function names the reference file:line it follows (paths are relative to
the ngnrsaa/qflex project root). Complex GEMMs go through ``numpy.matmul`` /
``numpy.dot``, which call the same OpenBLAS ``cgemm``/``zgemm`` family the
reference calls through CBLAS (src/tensor.cpp:973-1041), so a ``complex64``
run reproduces the reference's FP32 arithmetic closely and a ``complex128``
run is the FP64 oracle. Index permutation is ``numpy.transpose`` (bit-exact).

Parity is pinned: tests/test_oracle_golden.py checks this module against
fixtures produced by the unmodified reference (oracle/_ref, built by
oracle/Makefile) and against the reference's own golden values.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


class QflexError(Exception):
    """Stands in for the reference's ``throw std::string`` errors
    (src/errors.h:7-9). Tests match on message substrings, as the reference's
    own tests do."""


# ---------------------------------------------------------------------------
# Input formats: circuit, grid, ordering.
# ---------------------------------------------------------------------------

_SPECIAL = re.compile(r"[^)(\s\ta-zA-Z0-9_.,-]")


def _strip_common(line: str) -> str:
    line = re.sub(r"#.*", "", line)
    line = _SPECIAL.sub("", line)
    line = line.replace("\t", " ")
    line = re.sub(r"\s{2,}", " ", line)
    line = re.sub(r"\s+$", "", line)
    return line


def _is_number(tok: str) -> bool:
    # std::stol accepts a leading integer prefix (src/circuit.cpp:32-39).
    return re.match(r"^\s*[+-]?\d", tok) is not None


def _stol(tok: str) -> int:
    return int(re.match(r"^\s*([+-]?\d+)", tok).group(1))


def _stod(tok: str) -> float:
    m = re.match(r"^\s*([+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?))", tok)
    return float(m.group(1))


@dataclass
class Gate:
    name: str
    cycle: int
    qubits: List[int]
    params: List[float]
    raw: str


@dataclass
class Circuit:
    """QflexCircuit (src/circuit.h:27-35); ``load`` follows
    src/circuit.cpp:30-206."""
    num_active_qubits: int = 0
    depth: int = 0
    gates: List[Gate] = field(default_factory=list)

    @staticmethod
    def loads(text_or_lines) -> "Circuit":
        lines = text_or_lines.splitlines() if isinstance(text_or_lines, str) else list(text_or_lines)
        c = Circuit()
        last_cycle = 0
        used: set = set()
        for counter, raw_line in enumerate(lines):
            line = _strip_common(raw_line)
            line = re.sub(r"\s+\(", "(", line)
            line = re.sub(r"\s+(?=[^()]*\))", "", line)
            if not line:
                continue

            def err(msg, _c=counter, _l=line):
                return QflexError(f"[{_c + 1}: {_l}] {msg}")

            n_open, n_close = line.count("("), line.count(")")
            if n_open != n_close or n_open > 1:
                raise err("Not-matching parentheses.")
            tokens = line.split()
            if counter == 0:
                if len(tokens) != 1 or not _is_number(tokens[0]) or _stol(tokens[0]) <= 0:
                    raise err("First line in circuit must be the number of active qubits.")
                c.num_active_qubits = _stol(tokens[0])
                continue
            if len(tokens) < 3:
                raise err("Gate must be specified as: cycle gate_name[(p1[,p2,...])] q1 [q2, ...]")
            if not (_is_number(tokens[0]) and _stol(tokens[0]) == _stod(tokens[0])):
                raise err("First token must be a valid cycle number.")
            cycle = _stol(tokens[0])
            if cycle < last_cycle:
                raise err("Cycle number can only increase.")
            if cycle != last_cycle:
                used.clear()
                last_cycle = cycle
            params: List[float] = []
            tok = tokens[1]
            beg = tok.find("(")
            if beg >= 0:
                name = tok[:beg]
                inner = tok[beg + 1: tok.find(")")]
                for p in [x for x in inner.split(",") if x]:
                    if not _is_number(p) and not re.match(r"^\s*[+-]?\.\d", p):
                        raise QflexError("Params must be valid numbers.")
                    params.append(_stod(p))
            else:
                name = tok
            qubits = []
            for t in tokens[2:]:
                if not (_is_number(t) and _stol(t) == _stod(t)):
                    raise err("Qubit must be a valid number.")
                qubits.append(_stol(t))
            for q in qubits:
                if q in used:
                    raise err("Qubits can only used once per cycle.")
                used.add(q)
            c.gates.append(Gate(name, cycle, qubits, params, line))
        layers: Dict[Tuple[int, int], int] = {}
        for g in c.gates:
            if len(g.qubits) > 2:
                raise QflexError("Depth calculation does not handle k-qubit gates with k > 2.")
            if len(g.qubits) == 2:
                q1, q2 = g.qubits
                if q2 > q1:
                    q1, q2 = q2, q1
                layers[(q1, q2)] = layers.get((q1, q2), 0) + (2 if g.name == "fsim" else 1)
                c.depth = max(c.depth, layers[(q1, q2)])
        return c


@dataclass
class Grid:
    """QflexGrid (src/grid.h:13-20); ``loads`` follows src/grid.cpp:11-45."""
    I: int = 0
    J: int = 0
    qubits_off: List[Tuple[int, int]] = field(default_factory=list)

    @staticmethod
    def loads(text_or_lines) -> "Grid":
        lines = text_or_lines.splitlines() if isinstance(text_or_lines, str) else list(text_or_lines)
        g = Grid()
        counter = 0
        for line in lines:
            if not line or line[0] == "#":
                continue
            counter += 1
            bits = "".join(ch for ch in line if ch in "01")
            if not bits:
                continue
            if g.J != 0 and g.J != len(bits):
                raise QflexError(
                    f"Grid size at line {counter} is inconsistent with a width of {len(bits)} instead of {g.J}.")
            g.J = len(bits)
            for q, ch in enumerate(bits):
                if ch == "0":
                    g.qubits_off.append((g.I, q))
            g.I += 1
        return g


def load_ordering(text_or_lines) -> List[str]:
    """QflexOrdering::load (src/ordering.cpp:10-45): stripped, non-empty lines."""
    lines = text_or_lines.splitlines() if isinstance(text_or_lines, str) else list(text_or_lines)
    out = []
    for raw in lines:
        line = _strip_common(raw)
        line = re.sub(r"\s+(?=[^()]*\))", "", line)
        if line:
            out.append(line)
    return out


# ---------------------------------------------------------------------------
# Tensor with named indices (src/tensor.h:34-344).
# ---------------------------------------------------------------------------

class Tensor:
    __slots__ = ("indices", "dims", "data")

    def __init__(self, indices: Sequence[str], dims: Sequence[int], data: np.ndarray):
        if len(indices) != len(dims):
            raise QflexError(
                f"The number of indices: {len(indices)}, and number of dimensions: {len(dims)}, should be equal.")
        self.indices = list(indices)
        self.dims = [int(d) for d in dims]
        self.data = np.ascontiguousarray(data).reshape(-1)

    def size(self) -> int:
        return int(np.prod(self.dims, dtype=np.int64)) if self.dims else 1

    def dim_of(self, name: str) -> int:
        return self.dims[self.indices.index(name)]

    def copy(self) -> "Tensor":
        return Tensor(self.indices, self.dims, self.data.copy())

    def reorder(self, new_order: Sequence[str]) -> None:
        """Tensor::reorder (src/tensor.cpp:866-911). The fast/naive
        variants (src/tensor.cpp:377-864) are all the same index permutation;
        numpy.transpose computes it exactly."""
        new_order = list(new_order)
        if not new_order and not self.indices:
            return
        if set(new_order) != set(self.indices) or len(new_order) != len(self.indices):
            raise QflexError(
                f"new_ordering: {{{', '.join(new_order)}}} must be a reordering of current indices: "
                f"{{{', '.join(self.indices)}}}.")
        if new_order == self.indices:
            return
        axes = [self.indices.index(n) for n in new_order]
        arr = self.data.reshape(self.dims).transpose(axes)
        self.dims = [self.dims[a] for a in axes]
        self.indices = new_order
        self.data = np.ascontiguousarray(arr).reshape(-1)

    def project(self, index: str, value: int) -> "Tensor":
        """Tensor::project (src/tensor.cpp:280-316): slice of the leading
        index."""
        if index != self.indices[0]:
            raise QflexError(f"Index: '{index}' has to be equal to indices[0]: '{self.indices[0]}'.")
        if value >= self.dims[0]:
            raise QflexError(f"index_value: {value} must be contained in [0, {self.dims[0]}).")
        sub = self.size() // self.dims[0]
        return Tensor(self.indices[1:], self.dims[1:], self.data[value * sub:(value + 1) * sub].copy())

    def rename_index(self, old: str, new: str) -> None:
        """Tensor::rename_index (src/tensor.cpp:318-331)."""
        if old not in self.indices:
            raise QflexError(f"old_name: {old}, has to be a valid index.")
        if new in self.indices:
            raise QflexError(f"new_name: {new}, cannot be an existing index.")
        self.indices[self.indices.index(old)] = new

    def bundle(self, to_bundle: Sequence[str], name: str) -> None:
        """Tensor::bundle (src/tensor.cpp:333-375): metadata only; the bundled
        index is row-major over ``to_bundle`` (first listed most significant)."""
        to_bundle = list(to_bundle)
        if not all(i in self.indices for i in to_bundle):
            raise QflexError(f"indices_to_bundle has to be contained in indices.")
        in_order = [i for i in self.indices if i in to_bundle]
        if in_order != to_bundle:
            raise QflexError("indices_to_bundle must be in its original order.")
        # An empty bundle (neighbours without a shared gate) inserts a
        # dimension-1 index at position 0, as the reference does.
        pos = self.indices.index(to_bundle[0]) if to_bundle else 0
        dim = 1
        for i in to_bundle:
            dim *= self.dim_of(i)
        rest_idx = [i for i in self.indices if i not in to_bundle]
        rest_dim = [self.dim_of(i) for i in rest_idx]
        rest_idx.insert(pos, name)
        rest_dim.insert(pos, dim)
        self.indices, self.dims = rest_idx, rest_dim


GemmLog = List[Tuple[str, int, int, int]]


def multiply(A: Tensor, B: Tensor, log: Optional[GemmLog] = None) -> Tensor:
    """multiply (src/tensor.cpp:1045-1194): A and B are permuted IN PLACE to
    (left, common) and (common, right); C = A @ B with indices
    (left, right). The four BLAS cases (src/tensor.cpp:1125-1164) are all a
    matrix product here; ``log`` records the case and (m, n, k) as the
    reference would pass them to CBLAS."""
    left = [i for i in A.indices if i not in B.indices]
    right = [i for i in B.indices if i not in A.indices]
    common = [i for i in A.indices if i in B.indices]
    m = int(np.prod([A.dim_of(i) for i in left], dtype=np.int64)) if left else 1
    n = int(np.prod([B.dim_of(i) for i in right], dtype=np.int64)) if right else 1
    k = 1
    for pos, i in enumerate(common):
        if A.dim_of(i) != B.dim_of(i):
            raise QflexError(
                f"Common indices must have matching dimensions, but at index: {pos}, the dimensions are "
                f"A: {A.dim_of(i)}, B: {B.dim_of(i)}.")
        k *= A.dim_of(i)
    A.reorder(left + common)
    B.reorder(common + right)
    if log is not None:
        kind = "MM" if left and right else ("Mv" if left else ("vM" if right else "vv"))
        log.append((kind, m, n, k))
    out = np.matmul(A.data.reshape(m, k), B.data.reshape(k, n))
    dims = [A.dim_of(i) for i in left] + [B.dim_of(i) for i in right]
    return Tensor(left + right, dims, out.reshape(-1))


def bundle_between(A: Tensor, B: Tensor, name: str) -> None:
    """bundle_between (src/tensor.cpp:1214-1246)."""
    left = [i for i in A.indices if i not in B.indices]
    right = [i for i in B.indices if i not in A.indices]
    common = [i for i in A.indices if i in B.indices]
    A.reorder(left + common)
    B.reorder(common + right)
    A.bundle(common, name)
    B.bundle(common, name)


# ---------------------------------------------------------------------------
# Gate tables (src/read_circuit.cpp:27-165).
# ---------------------------------------------------------------------------

def gate_table(dtype) -> Dict[str, np.ndarray]:
    """Gate matrices in row-major (input, output) or (input, virtual,
    output) order. The constants are those of src/read_circuit.cpp:27-79
    (the balanced SVD split of cz and cx). For complex64 they are rounded
    to float, as the reference stores them (``s_type``)."""
    r = np.sqrt(0.5)
    t = {
        "delta_0": [1, 0],
        "delta_1": [0, 1],
        "h": [r, r, r, -r],
        "hz_1_2": [0.5 + 0.5j, r, -r * 1j, 0.5 + 0.5j],
        "t": [1, 0, 0, r + r * 1j],
        "x_1_2": [0.5 + 0.5j, 0.5 - 0.5j, 0.5 - 0.5j, 0.5 + 0.5j],
        "y_1_2": [0.5 + 0.5j, 0.5 + 0.5j, -0.5 - 0.5j, 0.5 + 0.5j],
        "cz_q1": [-0.3446133714352872, 0, 1.1381806476131544, 0, 0, -1.1381806476131544, 0, -0.3446133714352872],
        "cz_q2": [-1.0484937059720079, 0, 0.5611368023131075, 0, 0, 0.5611368023131075, 0, 1.0484937059720079],
        "cx_q1": [0.8408964152537143, 0, 0.8408964152537143, 0, 0, -0.8408964152537143, 0, 0.8408964152537143],
        "cx_q2": [0.5946035575013604, -0.5946035575013604, 0.5946035575013604, 0.5946035575013604,
                  -0.5946035575013604, 0.5946035575013604, 0.5946035575013604, 0.5946035575013604],
    }
    return {k: np.array(v, dtype=dtype) for k, v in t.items()}


def rz_gate(param: float, dtype) -> np.ndarray:
    """rz (src/read_circuit.cpp:84-88): diag(conj(p), p), p = exp(i*pi*x/2);
    evaluated in the working precision, as the reference does in float."""
    ftype = np.float32 if dtype == np.complex64 else np.float64
    half = ftype(math.pi * param / 2)
    ph = np.exp(np.array(1j, dtype=dtype) * half).astype(dtype)
    return np.array([np.conj(ph), 0, 0, ph], dtype=dtype)


def fsim_halves(theta_pi: float, phi_pi: float, dtype) -> np.ndarray:
    """fSim decomposition (src/read_circuit.cpp:105-139), angles in units of
    pi (src/read_circuit.cpp:157-158). Both halves are the same
    (input, virtual[4], output) array; the arithmetic is done in the working
    precision, as the reference does in float."""
    ftype = np.float32 if dtype == np.complex64 else np.float64
    th = ftype(math.pi * theta_pi)
    ph = ftype(math.pi * phi_pi)
    one_j = np.array(1j, dtype=dtype)
    c1 = dtype(0.5) * (np.exp(-one_j * (ph / ftype(2))) + dtype(np.cos(th)))
    c2 = dtype(0.5) * (np.exp(-one_j * (ph / ftype(2))) - dtype(np.cos(th)))
    c3 = dtype(-0.5j) * dtype(np.sin(th))
    s1, s2, s3 = np.sqrt(dtype(c1)), np.sqrt(dtype(c2)), np.sqrt(dtype(c3))
    s4 = s3
    d = np.exp(one_j * (ph / ftype(4)))
    z = dtype(0)
    arr = [d * s1, z, d * s2, z, z, s3, z, one_j * s4,
           z, np.conj(d) * s1, z, -np.conj(d) * s2, s3, z, -one_j * s4, z]
    return np.array(arr, dtype=dtype)


# ---------------------------------------------------------------------------
# Contraction ordering IR (src/contraction_utils.h:54-99).
# ---------------------------------------------------------------------------

Coord = Tuple[int, int]


@dataclass
class Op:
    kind: str                  # "expand" | "cut" | "merge"
    patch: str = ""            # expand: patch id
    tensor: Coord = (0, 0)     # expand: grid position
    tensors: List[Coord] = field(default_factory=list)  # cut: 1 or 2 positions
    values: List[int] = field(default_factory=list)     # cut: values ([] = all)
    source: str = ""           # merge
    target: str = ""           # merge


def index_name(p1: Sequence[int], p2: Sequence[int]) -> str:
    """index_name (src/contraction_utils.cpp:477-500)."""
    if len(p1) == 2 and len(p2) == 2:
        return f"({p1[0]},{p1[1]}),({p2[0]},{p2[1]})"
    if len(p1) == 3 and len(p2) == 3:
        return f"({p1[0]},{p1[1]},{p1[2]}),({p2[0]},{p2[1]},{p2[2]})"
    if len(p1) == 2 and len(p2) == 0:
        return f"({p1[0]},{p1[1]}),(o)"
    raise QflexError("Failed to construct tensor name with the following vectors.")


def cut_index_name(tensors: Sequence[Coord]) -> str:
    if len(tensors) == 2:
        return index_name(tensors[0], tensors[1])
    if len(tensors) == 1:
        return index_name(tensors[0], ())
    raise QflexError(f"Failed to construct tensor name with input tensors size: {len(tensors)}.")


def qubit_coords(q: int, J: int) -> Coord:
    """get_qubit_coords (src/contraction_utils.cpp:521-524)."""
    return (q // J, q % J)


def parse_ordering(lines: Sequence[str], grid: Grid) -> List[Op]:
    """ordering_data_to_contraction_ordering
    (src/contraction_utils.cpp:358-475)."""
    ops: List[Op] = []
    grid_size = grid.I * grid.J
    off = set(map(tuple, grid.qubits_off))
    for line in lines:
        if not line or line[0] == "#":
            continue

        def err(msg):
            # The reference quotes an outer, never-assigned `line`
            # (src/contraction_utils.cpp:365-370): always ''.
            return QflexError(f"Parsing failed on line: '' with error: {msg}")

        def check(idx):
            if idx < 0 or idx >= grid_size:
                raise err(f"Index {idx} must be within grid boundaries.")

        toks = line.split()
        op = toks[0]
        if op == "expand":
            idx = _stol(toks[2]) if len(toks) > 2 and _is_number(toks[2]) else 0
            check(idx)
            pos = qubit_coords(idx, grid.J)
            if pos in off:
                raise err("Index must specify an active qubit.")
            ops.append(Op("expand", patch=toks[1] if len(toks) > 1 else "", tensor=pos))
        elif op == "cut":
            vs = toks[1] if len(toks) > 1 else ""
            if not re.fullmatch(r"\([0-9,]*\)", vs):
                raise err("Cut values must be comma-separated ints, e.g. (0,1,3).")
            inner = vs[1:-1]
            values = []
            if inner:
                for piece in inner.split(","):
                    mm = re.match(r"^\s*[+-]?\d+", piece)
                    values.append(int(mm.group(0)) if mm else 0)
            idx1 = _stol(toks[2]) if len(toks) > 2 and _is_number(toks[2]) else 0
            check(idx1)
            p1 = qubit_coords(idx1, grid.J)
            if p1 in off:
                raise err("Index 1 must specify an active qubit.")
            if len(toks) <= 3:
                ops.append(Op("cut", tensors=[p1], values=values))
            else:
                idx2 = _stol(toks[3]) if _is_number(toks[3]) else 0
                check(idx2)
                p2 = qubit_coords(idx2, grid.J)
                if p2 in off:
                    raise err("Index 2 must specify an active qubit.")
                pair = [p1, p2] if idx1 < idx2 else [p2, p1]
                ops.append(Op("cut", tensors=pair, values=values))
        elif op == "merge":
            ops.append(Op("merge", source=toks[1], target=toks[2]))
        else:
            raise err("Received an invalid operation in config.")
    validate_ordering(ops)
    return ops


def validate_ordering(ops: Sequence[Op]) -> None:
    """ValidateOrdering (src/contraction_utils.cpp:534-610)."""
    active: Dict[str, bool] = {}
    used: Dict[str, bool] = {}
    merged: Dict[str, bool] = {}
    cut_idx: set = set()
    tensors: set = set()
    msg = ""
    for op in ops:
        if op.kind == "expand":
            p = op.patch
            t = op.tensor
            for flag in (used.get(p), merged.get(p)):
                if flag:
                    msg += f"\nTensor at ({t[0]},{t[1]}) is added to non-empty patch {p} after a cut."
            name = f"({t[0]},{t[1]})"
            if name in tensors:
                msg += f"\nTensor {name} is contracted multiple times."
            tensors.add(name)
            active[p] = True
        elif op.kind == "cut":
            for p, a in active.items():
                if a:
                    used[p] = True
            idx = cut_index_name(op.tensors)
            if idx in cut_idx:
                msg += f"\nIndex {idx} is cut multiple times."
            cut_idx.add(idx)
        else:
            if merged.get(op.source):
                msg += f"\nPatch {op.source} is merged multiple times."
            if used.get(op.target):
                msg += f"\nPatch {op.source} is merged into non-empty patch {op.target} after a cut."
            merged[op.source] = True
            active[op.target] = True
    if msg:
        raise QflexError(msg)


# ---------------------------------------------------------------------------
# Network build: 3D grid of gate tensors, flatten, bundling, index order.
# ---------------------------------------------------------------------------

def _order_key(ops: Sequence[Op], local: Coord):
    """order_func (src/read_circuit.cpp:191-291): the comparator that sorts a
    grid tensor's neighbours so that cut bonds come first, then bonds in the
    order the contraction reaches them."""

    def less(lhs: Coord, rhs: Coord) -> bool:
        lp = [local, lhs] if (local[0] < lhs[0] or local[1] < lhs[1]) else [lhs, local]
        rp = [local, rhs] if (local[0] < rhs[0] or local[1] < rhs[1]) else [rhs, local]
        for op in ops:
            if op.kind != "cut":
                continue
            if lp == list(op.tensors):
                return True
            if rp == list(op.tensors):
                return False

        def find(pos):
            n = 0
            for op in ops:
                if op.kind != "expand":
                    continue
                if op.tensor == pos:
                    return op.patch, n
                n += 1
            return None, None

        lpatch, lpos = find(lhs)
        if lpos is None:
            raise QflexError(f"Left hand side of pair not found: ({local[0]},{local[1]}),({lhs[0]},{lhs[1]}).")
        rpatch, rpos = find(rhs)
        if rpos is None:
            raise QflexError(f"Right hand side of pair not found: ({local[0]},{local[1]}),({rhs[0]},{rhs[1]}).")
        if lpatch == rpatch:
            return lpos < rpos
        local_patch = ""
        for op in ops:
            if op.kind == "expand" and op.tensor == local:
                local_patch = op.patch
                break
        if lpatch == local_patch:
            return True
        if rpatch == local_patch:
            return False
        for op in ops:
            if op.kind != "merge":
                continue
            if local_patch == op.source:
                if lpatch == op.target:
                    return True
                if rpatch == op.target:
                    return False
                local_patch = op.target
            elif local_patch == op.target:
                if lpatch == op.source:
                    return True
                if rpatch == op.source:
                    return False
            elif lpatch == op.source:
                lpatch = op.target
            elif rpatch == op.source:
                rpatch = op.target
        raise QflexError(f"Failed to compare ({lhs[0]},{lhs[1]}) and ({rhs[0]},{rhs[1]}) "
                         f"for local ({local[0]},{local[1]}).")

    return less


def _insertion_sort(items: List[Coord], less) -> List[Coord]:
    # std::sort on fewer than 16 elements is an insertion sort in libstdc++;
    # the same algorithm keeps ties and odd comparators resolved alike.
    out = list(items)
    for i in range(1, len(out)):
        v = out[i]
        if less(v, out[0]):
            out[1:i + 1] = out[0:i]
            out[0] = v
        else:
            j = i
            while less(v, out[j - 1]):
                out[j] = out[j - 1]
                j -= 1
            out[j] = v
    return out


def build_grid(circuit: Circuit, grid: Grid, initial: str, final: str,
               final_region: Sequence[Coord], ops: Sequence[Op], dtype,
               log: Optional[GemmLog] = None) -> List[List[Optional[Tensor]]]:
    """circuit_data_to_tensor_network (src/read_circuit.cpp:296-544) followed
    by flatten_grid_of_tensors (src/read_circuit.cpp:548-689)."""
    I, J = grid.I, grid.J
    off = set(map(tuple, grid.qubits_off))
    final_region = set(map(tuple, final_region))
    n_active = I * J - len(off)
    if circuit.num_active_qubits != n_active:
        raise QflexError(
            f"The number of active qubits read from the file: {circuit.num_active_qubits}, does not match "
            f"the number of active qubits read from the grid: {n_active}.")
    if len(initial) != n_active:
        raise QflexError(f"Size of initial_conf: {len(initial)}, must be equal to the number of qubits: {n_active}.")
    if len(final) != len(initial):
        raise QflexError(f"Size of final_conf: {len(final)}, must be equal to size of initial_conf: {len(initial)}.")
    gates = gate_table(dtype)
    cols: Dict[Coord, List[Tensor]] = {}
    counters: Dict[Coord, int] = {}
    idx = 0
    for q in range(I * J):
        pos = qubit_coords(q, J)
        if pos in off:
            continue
        name = f"({pos[0]},{pos[1]}),(0)"
        cols[pos] = [Tensor([name], [2], gates["delta_0" if initial[idx] == "0" else "delta_1"])]
        counters[pos] = 0
        idx += 1
    for (x, y) in off:
        if x >= I or y >= J:
            raise QflexError(f"Off qubit '({x}, {y})' is outside the grid.")
    links: Dict[str, int] = {}
    used: set = set()
    last_cycle = 0
    for g in circuit.gates:
        if g.cycle != last_cycle:
            last_cycle = g.cycle
            used.clear()
        for q in g.qubits:
            if q in used:
                raise QflexError(f"Qubit {q} has been used twice in the same cycle: {g.cycle}")
            used.add(q)
        if len(g.qubits) == 1:
            p = qubit_coords(g.qubits[0], J)
            if p in off:
                raise QflexError(f"Qubit '{g.qubits[0]}' in gate '{g.raw}' must correspond to an active qubit.")
            a = f"({p[0]},{p[1]}),({counters[p]})"
            counters[p] += 1
            b = f"({p[0]},{p[1]}),({counters[p]})"
            if g.name == "rz":
                data = rz_gate(g.params[0], dtype)
            elif g.name in gates:
                data = gates[g.name]
            else:
                raise QflexError(f"Invalid gate name provided: {g.name}")
            cols[p].append(Tensor([a, b], [2, 2], data))
        elif len(g.qubits) == 2:
            q1, q2 = g.qubits
            p1, p2 = qubit_coords(q1, J), qubit_coords(q2, J)
            if p1 in off:
                raise QflexError(f"Qubit '{q1}' in gate '{g.raw}' must correspond to an active qubit.")
            if p2 in off:
                raise QflexError(f"Qubit '{q2}' in gate '{g.raw}' must correspond to an active qubit.")
            if abs(p1[0] - p2[0]) + abs(p1[1] - p2[1]) != 1:
                raise QflexError(f"Qubits {q1} and {q2} are not nearest neighbors.")
            if g.name == "cz":
                d1, d2, vd = gates["cz_q1"], gates["cz_q2"], 2
            elif g.name == "cx":
                d1, d2, vd = gates["cx_q1"], gates["cx_q2"], 2
            elif g.name == "fsim":
                d1 = fsim_halves(g.params[0], g.params[1], dtype)
                d2, vd = d1, 4
            else:
                raise QflexError(f"Invalid gate name provided: {g.name}")
            link = index_name(p1, p2)
            links[link] = links.get(link, 0) + 1
            c = links[link]
            lo = (min(p1[0], p2[0]), min(p1[1], p2[1]))
            hi = (max(p1[0], p2[0]), max(p1[1], p2[1]))
            virt = f"({lo[0]},{lo[1]},{c}),({hi[0]},{hi[1]},{c})"
            for p, d in ((p1, d1), (p2, d2)):
                a = f"({p[0]},{p[1]}),({counters[p]})"
                counters[p] += 1
                b = f"({p[0]},{p[1]}),({counters[p]})"
                cols[p].append(Tensor([a, virt, b], [2, vd, 2], d))
        else:
            raise QflexError("k-qubit gates with k > 2 not yet implemented.")
    idx = 0
    for q in range(I * J):
        pos = qubit_coords(q, J)
        if pos in off:
            continue
        last = f"({pos[0]},{pos[1]}),({counters[pos]})"
        if pos in final_region:
            cols[pos][-1].rename_index(last, f"({pos[0]},{pos[1]}),(o)")
        else:
            cols[pos].append(Tensor([last], [2], gates["delta_0" if final[idx] == "0" else "delta_1"]))
        idx += 1

    # Flatten each time column (src/read_circuit.cpp:559-587).
    grid2d: List[List[Optional[Tensor]]] = [[None] * J for _ in range(I)]
    for i in range(I):
        for j in range(J):
            if (i, j) in off:
                continue
            col = cols[(i, j)]
            A = col[0].copy()
            for B in col[1:]:
                A = multiply(A, B, log)
            grid2d[i][j] = A
    # Bundle bonds between neighbours (src/read_circuit.cpp:590-621).
    for i in range(I):
        for j in range(J):
            if (i, j) in off:
                continue
            for (a, b) in ((i + 1, j), (i, j + 1)):
                if a < I and b < J and (a, b) not in off:
                    bundle_between(grid2d[i][j], grid2d[a][b], index_name((i, j), (a, b)))
    # Final index order (src/read_circuit.cpp:624-688).
    for i in range(I):
        for j in range(J):
            if (i, j) in off:
                continue
            pairs = [(a, b) for (a, b) in ((i - 1, j), (i, j - 1), (i + 1, j), (i, j + 1))
                     if 0 <= a < I and 0 <= b < J and (a, b) not in off]
            order = []
            if (i, j) in final_region:
                order.append(index_name((i, j), ()))
            pairs = _insertion_sort(pairs, _order_key(ops, (i, j)))
            for p in pairs:
                q1, q2 = (p, (i, j)) if (p[0] < i or p[1] < j) else ((i, j), p)
                order.append(index_name(q1, q2))
            grid2d[i][j].reorder(order)
    return grid2d


# ---------------------------------------------------------------------------
# Contraction (src/contraction_utils.cpp:16-354).
# ---------------------------------------------------------------------------

def planned_bytes(ops: Sequence[Op], grid2d) -> int:
    """The scratch plan of ContractionData::Initialize
    (src/contraction_utils.cpp:30-148), in bytes of complex64."""
    dim: Dict[str, int] = {}
    gidx: Dict[Coord, List[str]] = {}
    for i, row in enumerate(grid2d):
        for j, t in enumerate(row):
            if t is None:
                continue
            gidx[(i, j)] = list(t.indices)
            for n, d in zip(t.indices, t.dims):
                dim[n] = d
    pidx: Dict[str, List[str]] = {}
    pmax: Dict[str, int] = {}
    cut_copy: Dict[str, int] = {}

    def sym(a, b):
        u = a + [x for x in b if x not in a]
        inter = [x for x in a if x in b]
        return [x for x in u if x not in inter]

    for op in ops:
        if op.kind == "expand":
            pidx[op.patch] = sym(pidx.get(op.patch, []), gidx[op.tensor])
            s = 1
            for n in pidx[op.patch]:
                s *= dim[n]
            pmax[op.patch] = max(pmax.get(op.patch, 0), s)
        elif op.kind == "cut":
            name = cut_index_name(op.tensors)
            for side, t in enumerate(op.tensors):
                gidx[t] = [x for x in gidx[t] if x != name]
                cut_copy[f"cut-{name}:size-{side}"] = grid2d[t[0]][t[1]].size()
        else:
            pidx[op.target] = sym(pidx.get(op.target, []), pidx.get(op.source, []))
            s = 1
            for n in pidx[op.target]:
                s *= dim[n]
            pmax[op.target] = max(pmax.get(op.target, 0), s)
    sizes = list(pmax.values())
    total = (max(sizes) if sizes else 0) + sum(set(sizes)) + sum(sizes) + sum(cut_copy.values())
    return total * 8


def readable_memory(b: float) -> str:
    """utils::readable_memory_string (src/utils.cpp:60-68)."""
    suffix = [" B", " kB", " MB", " GB"]
    s = 0
    while b >= 1024:
        s += 1
        b /= 1024
    v = int(b * 100) / 100.0
    txt = f"{v:g}" if v != int(v) else str(int(v))
    return txt + suffix[s]


def contract(ops: Sequence[Op], grid2d, n_amplitudes: int, dtype,
             log: Optional[GemmLog] = None) -> np.ndarray:
    """ContractionData::ContractGrid (src/contraction_utils.cpp:223-354):
    ops before a cut run once; the rest runs once per cut value. Amplitudes
    accumulate in complex128 (src/contraction_utils.cpp:352)."""
    amps = np.zeros(n_amplitudes, dtype=np.complex128)

    def run(todo: List[Op], out_idx: int, patches: Dict[str, Tensor]) -> None:
        patches = dict(patches)
        output = None
        todo = list(todo)
        while todo:
            op = todo.pop(0)
            if op.kind == "expand":
                nxt = grid2d[op.tensor[0]][op.tensor[1]]
                if op.patch not in patches:
                    patches[op.patch] = nxt.copy()
                    continue
                res = multiply(patches[op.patch], nxt, log)
                if not todo:
                    output = res
                    continue
                patches[op.patch] = res
            elif op.kind == "cut":
                name = cut_index_name(op.tensors)
                ta = grid2d[op.tensors[0][0]][op.tensors[0][1]]
                copy_a = ta.copy()
                values = list(op.values) or list(range(copy_a.dim_of(name)))
                if len(op.tensors) > 1:
                    tb = grid2d[op.tensors[1][0]][op.tensors[1][1]]
                    copy_b = tb.copy()
                    for v in values:
                        grid2d[op.tensors[0][0]][op.tensors[0][1]] = copy_a.project(name, v)
                        grid2d[op.tensors[1][0]][op.tensors[1][1]] = copy_b.project(name, v)
                        run(todo, out_idx, patches)
                    grid2d[op.tensors[1][0]][op.tensors[1][1]] = copy_b
                else:
                    out_idx *= len(values)
                    for v in values:
                        grid2d[op.tensors[0][0]][op.tensors[0][1]] = copy_a.project(name, v)
                        run(todo, out_idx, patches)
                        out_idx += 1
                grid2d[op.tensors[0][0]][op.tensors[0][1]] = copy_a
                return
            else:
                src = patches[op.source]
                if op.target not in patches:
                    patches[op.target] = src.copy()
                    continue
                res = multiply(src, patches[op.target], log)
                if not todo:
                    output = res
                    continue
                patches[op.target] = res
        if output is None or output.size() != 1:
            desc = "none" if output is None else f"rank {len(output.indices)}"
            raise QflexError(f"Contraction did not complete; final tensor is: {desc}")
        amps[out_idx] += complex(output.data[0])

    run(list(ops), 0, {})
    return amps


# ---------------------------------------------------------------------------
# EvaluateCircuit (src/evaluate_circuit.cpp:22-253).
# ---------------------------------------------------------------------------

def output_pos(grid: Grid, pos: Coord) -> int:
    """find_output_pos (src/evaluate_circuit.cpp:22-36)."""
    p = pos[0] * grid.J + pos[1]
    for (a, b) in grid.qubits_off:
        if a < pos[0] or (a == pos[0] and b < pos[1]):
            p -= 1
    return p


def output_states(grid: Grid, ops: Sequence[Op], initial: str, final: str):
    """get_output_states (src/evaluate_circuit.cpp:38-104): the first terminal
    cut is the most significant digit of the amplitude index."""
    base = final if final else "0" * len(initial)
    unspecified = not final
    base = list(base)
    positions, value_lists, final_qubits = [], [], []
    for op in ops:
        if op.kind != "cut" or len(op.tensors) != 1:
            continue
        p = output_pos(grid, op.tensors[0])
        if unspecified:
            base[p] = "x"
        positions.append(p)
        value_lists.append(list(op.values) or [0, 1])
        final_qubits.append(op.tensors[0])
    base = "".join(base)
    states = [base]
    for p, vals in zip(positions, value_lists):
        nxt = []
        for s in states:
            for v in vals:
                nxt.append(s[:p] + str(v)[0] + s[p + 1:])
        states = nxt
    for i, ch in enumerate(states[0]):
        if ch not in "01":
            raise QflexError(f"Final state has non-binary character {ch} at index {i}despite having "
                             f"no terminal cut there.")
    return base, final_qubits, states


@dataclass
class Input:
    circuit: Circuit
    ordering: List[str]
    grid: Grid
    initial_state: str = ""
    final_state: str = ""


def evaluate_circuit(inp: Input, dtype=np.complex64, memory_limit: float = float(1 << 30),
                     log: Optional[GemmLog] = None) -> List[Tuple[str, complex]]:
    """EvaluateCircuit (src/evaluate_circuit.cpp:106-253). Mutates
    ``inp.initial_state`` / ``inp.final_state`` as the reference does."""
    if inp is None:
        raise QflexError("Input must be non-null.")
    ops = parse_ordering(inp.ordering, inp.grid)
    n = inp.grid.I * inp.grid.J - len(inp.grid.qubits_off)
    if not inp.initial_state:
        inp.initial_state = "0" * n
    base, final_qubits, states = output_states(inp.grid, ops, inp.initial_state, inp.final_state)
    inp.final_state = base
    grid2d = build_grid(inp.circuit, inp.grid, inp.initial_state, inp.final_state, final_qubits, ops, dtype, log)
    need = planned_bytes(ops, grid2d)
    if need > memory_limit:
        raise QflexError(f"Required space ({readable_memory(need)}) exceeds memory limit "
                         f"({readable_memory(memory_limit)}). Cancelling simulation.")
    amps = contract(ops, grid2d, len(states), dtype, log)
    return [(s, complex(a)) for s, a in zip(states, amps)]


def simulate(options: dict, dtype=np.complex64) -> List[Tuple[str, complex]]:
    """The pybind entry ``qflex.simulate`` (src/pybind_main.cpp:75-138):
    errors print to stderr and return ``[]``."""
    import sys
    try:
        mem = options.get("memory_limit", 1 << 30)
        if isinstance(mem, str):
            mem = parse_memory(mem)
        elif mem <= 0:
            raise QflexError("'memory_limit' must be positive.")

        def load(key, fn):
            if key in options:
                return fn(list(options[key]))
            if key + "_filename" in options:
                with open(options[key + "_filename"]) as f:
                    return fn(f.read())
            return fn([])

        grid = load("grid", Grid.loads)
        circuit = load("circuit", Circuit.loads)
        ordering = load("ordering", load_ordering)
        inp = Input(circuit, ordering, grid, options.get("initial_state", ""), options.get("final_state", ""))
        return evaluate_circuit(inp, dtype, float(mem))
    except QflexError as e:
        print(str(e), file=sys.stderr)
        return []


def parse_memory(s: str) -> int:
    """utils::from_readable_memory_string (src/utils.cpp:19-57)."""
    s = _SPECIAL.sub("", s).replace("\t", " ").replace(" ", "").upper()
    m = re.match(r"^(\d+)(.*)$", s)
    if not m:
        raise QflexError(f"Memory string {s} not recognized.")
    v, suf = int(m.group(1)), m.group(2)
    scale = {"GB": 1 << 30, "MB": 1 << 20, "KB": 1 << 10, "B": 1, "": 1}
    if suf not in scale:
        raise QflexError(f"Suffix {suf} not recognized.")
    return v * scale[suf]
