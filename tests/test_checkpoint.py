"""Checkpoint and resume over the values of one cut, with the FP64 oracle as
the per-piece evaluation (no GPU): an evaluation interrupted after one piece
and resumed gives the uninterrupted sums; a checkpoint of other inputs is
refused."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import checkpoint

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_cases.json"


def _case():
    d = json.loads(GOLDEN.read_text())
    c = next(x for x in d if x["name"] == "rect4x4_cut_terminal")
    return c["circuit"], c["ordering"], c["grid"], c["initial"], [r["final"] for r in c["runs"]]


def oracle_evaluate(circuit, ordering, grid, initial, finals):
    out = []
    for f in finals:
        inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), initial, f)
        out.extend(qo.evaluate_circuit(inp, np.complex128, float(1 << 40)))
    return out


class Interrupt(Exception):
    pass


def test_resume_after_interruption_gives_the_uninterrupted_sums(tmp_path):
    circuit, ordering, grid, initial, finals = _case()
    want = oracle_evaluate(circuit, ordering, grid, initial, finals)
    path = tmp_path / "ckpt.json"
    calls = []

    def flaky(*args):
        calls.append(args[1])
        if len(calls) == 2:
            raise Interrupt()
        return oracle_evaluate(*args)

    with pytest.raises(Interrupt):
        checkpoint.evaluate_resumable(flaky, circuit, ordering, grid, initial, finals, path, parts=4)
    saved = json.loads(path.read_text())
    assert list(saved["pieces"]) == ["0"]
    resumed = checkpoint.evaluate_resumable(oracle_evaluate, circuit, ordering, grid, initial, finals, path,
                                            parts=4)
    whole = checkpoint.evaluate_resumable(oracle_evaluate, circuit, ordering, grid, initial, finals,
                                          tmp_path / "other.json", parts=4)
    assert resumed == whole
    assert [s for s, _ in resumed] == [s for s, _ in want]
    got, ref = np.array([a for _, a in resumed]), np.array([a for _, a in want])
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_checkpoint_of_other_inputs_is_refused(tmp_path):
    circuit, ordering, grid, initial, finals = _case()
    path = tmp_path / "ckpt.json"
    checkpoint.evaluate_resumable(oracle_evaluate, circuit, ordering, grid, initial, finals[:1], path, parts=2)
    with pytest.raises(ValueError):
        checkpoint.evaluate_resumable(oracle_evaluate, circuit, ordering, grid, initial, finals, path, parts=2)
