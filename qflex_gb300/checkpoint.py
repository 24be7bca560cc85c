"""Checkpoint and resume of a long evaluation.

The reference's state during ContractGrid is the cut cursor of its
recursion and the complex<double> amplitude sums
(src/contraction_utils.cpp:260-316, 352); it keeps them in memory only. Here
an evaluation is cut into pieces over the values of one two-qubit cut (the
same partition as qflex_gb300.shards), each piece's FP64 amplitudes are
written to a checkpoint file when the piece finishes, and a rerun with the
same inputs and file skips the finished pieces. The pieces are added in
piece order at the end, so an interrupted and resumed run gives the same
sums as an uninterrupted one.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path
from typing import Callable, List, Sequence, Tuple

from .shards import shard_ordering

Result = List[Tuple[str, complex]]
Evaluate = Callable[[str, str, str, str, Sequence[str]], Result]


def _signature(circuit: str, ordering: str, grid: str, initial: str, finals: Sequence[str], parts: int,
               which_cut: int) -> str:
    h = hashlib.sha256()
    for part in (circuit, ordering, grid, initial, "\x00".join(finals), str(parts), str(which_cut)):
        h.update(part.encode())
        h.update(b"\x01")
    return h.hexdigest()


def _load(path: Path, signature: str) -> dict:
    try:
        state = json.loads(path.read_text())
    except (OSError, ValueError):
        return {"signature": signature, "pieces": {}}
    if state.get("signature") != signature:
        raise ValueError(f"checkpoint {path} belongs to another evaluation")
    return state


def _save(path: Path, state: dict) -> None:
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_text(json.dumps(state))
    os.replace(tmp, path)  # a crash leaves the old file or the new one


def evaluate_resumable(evaluate: Evaluate, circuit: str, ordering: str, grid: str, initial: str,
                       finals: Sequence[str], path, parts: int = 4, which_cut: int = 0) -> Result:
    """Evaluates `finals` in `parts` pieces over the values of cut number
    `which_cut`, checkpointing to `path` after every piece, and returns the
    summed amplitudes. A rerun with the same inputs resumes after the last
    finished piece; a checkpoint of other inputs is refused."""
    path = Path(path)
    sig = _signature(circuit, ordering, grid, initial, list(finals), parts, which_cut)
    state = _load(path, sig)
    for r in range(parts):
        key = str(r)
        if key in state["pieces"]:
            continue
        piece = evaluate(circuit, shard_ordering(circuit, ordering, r, parts, which_cut), grid, initial,
                         list(finals))
        state["pieces"][key] = [[s, complex(a).real, complex(a).imag] for s, a in piece]
        _save(path, state)
    first = state["pieces"]["0"]
    out = []
    for i, (s, _, _) in enumerate(first):
        acc = 0j
        for r in range(parts):
            ps, re, im = state["pieces"][str(r)][i]
            if ps != s:
                raise ValueError(f"pieces disagree on output state {i}: {s} vs {ps}")
            acc += complex(re, im)
        out.append((s, acc))
    return out
