"""One evaluation sharded over processes (one GPU per process).

The reference runs every cut slice and every output string in one process:
ContractGrid recurses over the values of each cut and adds the slices'
results into complex<double> amplitudes (src/contraction_utils.cpp:260-316,
352), and the Cirq layer loops over output strings
(qflexcirq/interface/qflex_simulator.py:44-53). Both loops are independent
units, so they shard with no exchange on the data path:

  by="strings"  rank r evaluates a contiguous range of the output strings;
                the ranks' results are concatenated in rank order.
  by="slices"   rank r evaluates a contiguous range of the values of one
                two-qubit cut (the ordering's first one by default); the
                ranks' FP64 amplitude partials are summed in rank order on
                the host, so every rank ends with the same amplitudes.

The exchange goes through a key-value store (torch.distributed.TCPStore or
anything with set/get/wait): results are tiny (16 bytes per amplitude).
Before anything is combined, every rank publishes a status; a rank that
raised is reported by every rank, and one that never reports ends the
others' wait with an error after `timeout_s` -- failures surface on the
host between steps, never inside a kernel.
"""
from __future__ import annotations

import datetime
import json
import re
from typing import Callable, List, Optional, Sequence, Tuple

Result = List[Tuple[str, complex]]
Evaluate = Callable[[str, str, str, str, Sequence[str]], Result]

_CUT = re.compile(r"^\s*cut\s+\(([^)]*)\)\s+(\d+)\s+(\d+)\s*$")


class ShardError(RuntimeError):
    """A rank failed or did not report."""


def string_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous range [lo, hi) of `n` units for `rank` of `world`; the
    first n % world ranks take one extra unit."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def bond_dimension(circuit: str, q1: int, q2: int) -> int:
    """Dimension of the bundled bond between qubits q1 and q2: 2 per CZ or
    CX and 4 per fSim acting on the pair (the virtual dimensions of the
    two-qubit gate splits, src/read_circuit.cpp:146-165)."""
    dim = 1
    pair = {q1, q2}
    for line in circuit.splitlines()[1:]:
        line = line.split("#")[0]
        name_m = re.match(r"\s*\d+\s+([A-Za-z_0-9]+)", line)
        if not name_m:
            continue
        toks = re.sub(r"\([^)]*\)", " ", line).split()
        if len(toks) < 4:
            continue
        name = name_m.group(1)
        try:
            qs = {int(toks[2]), int(toks[3])}
        except ValueError:
            continue
        if qs == pair:
            dim *= 4 if name == "fsim" else 2
    return dim


def cut_lines(ordering: str) -> List[Tuple[int, List[int], int, int]]:
    """(line number, values, q1, q2) of every two-qubit cut of an ordering;
    an empty value list means every value of the bond."""
    out = []
    for i, line in enumerate(ordering.splitlines()):
        m = _CUT.match(line.split("#")[0])
        if m:
            vals = [int(v) for v in m.group(1).replace(",", " ").split()]
            out.append((i, vals, int(m.group(2)), int(m.group(3))))
    return out


def shard_ordering(circuit: str, ordering: str, rank: int, world: int, which: int = 0) -> str:
    """The ordering with cut number `which` restricted to this rank's
    contiguous share of its values."""
    cuts = cut_lines(ordering)
    if which >= len(cuts):
        raise ValueError(f"the ordering has {len(cuts)} two-qubit cuts; cannot shard cut {which}")
    line_no, vals, q1, q2 = cuts[which]
    if not vals:
        vals = list(range(bond_dimension(circuit, q1, q2)))
    if len(vals) < world:
        raise ValueError(f"cut {which} has {len(vals)} values for {world} ranks")
    lo, hi = string_range(len(vals), rank, world)
    lines = ordering.splitlines()
    lines[line_no] = f"cut ({','.join(str(v) for v in vals[lo:hi])}) {q1} {q2}"
    return "\n".join(lines) + "\n"


def _wait(store, keys: List[str], timeout_s: float) -> List[str]:
    """Keys of `keys` that did not appear within `timeout_s`."""
    try:
        store.wait(keys, datetime.timedelta(seconds=timeout_s))
        return []
    except Exception:  # the store's timeout error type varies across versions
        missing = []
        for k in keys:
            try:
                store.wait([k], datetime.timedelta(milliseconds=1))
            except Exception:
                missing.append(k)
        return missing


def encode_result(result: Result) -> bytes:
    """A rank's (state, amplitude) list as JSON: [[state, re, im], ...].
    JSON, unlike pickle, runs nothing when read, and Python writes floats
    with repr, so every double round-trips exactly."""
    return json.dumps([[str(st), float(complex(a).real), float(complex(a).imag)] for st, a in result]).encode()


def decode_result(data: bytes) -> Result:
    rows = json.loads(data.decode())
    if not isinstance(rows, list) or not all(
            isinstance(r, list) and len(r) == 3 and isinstance(r[0], str) and all(
                isinstance(x, (int, float)) for x in r[1:]) for r in rows):
        raise ShardError("malformed result payload")
    return [(st, complex(re_, im)) for st, re_, im in rows]


def exchange(store, tag: str, rank: int, world: int, payload: Result, error: Optional[str],
             timeout_s: float) -> List[Result]:
    """Publishes this rank's results (or error), waits for every rank and
    returns the results in rank order. Raises ShardError on every rank if
    any rank failed or did not report in time."""
    if error is None:
        store.set(f"{tag}/data/{rank}", encode_result(payload))
        store.set(f"{tag}/status/{rank}", b"ok")
    else:
        store.set(f"{tag}/status/{rank}", b"error:" + error.encode())
    keys = [f"{tag}/status/{r}" for r in range(world)]
    missing = _wait(store, keys, timeout_s)
    if missing:
        ranks = [int(k.rsplit("/", 1)[1]) for k in missing]
        raise ShardError(f"rank(s) {ranks} did not report within {timeout_s:g} s")
    failed = []
    for r in range(world):
        st = store.get(f"{tag}/status/{r}")
        if st != b"ok":
            failed.append(f"rank {r}: {st[len(b'error:'):].decode(errors='replace')}")
    if failed:
        raise ShardError("; ".join(failed))
    return [decode_result(store.get(f"{tag}/data/{r}")) for r in range(world)]


def evaluate_sharded(evaluate: Evaluate, circuit: str, ordering: str, grid: str, initial: str,
                     finals: Sequence[str], *, rank: int, world: int, store, tag: str = "qflex",
                     by: str = "slices", which_cut: int = 0, timeout_s: float = 60.0) -> Result:
    """Evaluates `finals` over `world` ranks and returns the full result
    (the same list EvaluateCircuit would give per final state, concatenated)
    on every rank. `evaluate(circuit, ordering, grid, initial, finals)` is
    the per-rank evaluation, e.g. a Context's evaluate_many with a memory
    limit bound in."""
    if by not in ("slices", "strings"):
        raise ValueError(f"by must be 'slices' or 'strings', not {by!r}")
    payload, error = None, None
    try:
        if by == "strings":
            lo, hi = string_range(len(finals), rank, world)
            payload = evaluate(circuit, ordering, grid, initial, list(finals[lo:hi])) if hi > lo else []
        else:
            mine = shard_ordering(circuit, ordering, rank, world, which_cut)
            payload = evaluate(circuit, mine, grid, initial, list(finals))
    except Exception as e:  # reported to every rank below
        error = f"{type(e).__name__}: {e}"
    parts = exchange(store, tag, rank, world, payload, error, timeout_s)
    if by == "strings":
        return [x for part in parts for x in part]
    out = []
    for i, (state, _) in enumerate(parts[0]):
        acc = 0j
        for part in parts:  # rank order: the same sum on every rank
            if part[i][0] != state:
                raise ShardError(f"ranks disagree on output state {i}: {state} vs {part[i][0]}")
            acc += complex(part[i][1])
        out.append((state, acc))
    return out
