"""Sharding one evaluation over processes: two CPU ranks in a gloo process
group whose TCPStore (127.0.0.1) carries the exchange. The per-rank
evaluation is the FP64 oracle (no GPU here); the product passes a
Context's evaluate_many. Covers slice sharding (FP64 partial sums), string
sharding, a rank that raises, and a rank that never reports."""
import json
import multiprocessing as mp
import os
import socket
from datetime import timedelta
from pathlib import Path

import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import rqc, shards

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


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, mode, q):
    import torch
    import torch.distributed as dist
    try:
        store = dist.TCPStore("127.0.0.1", port, world, rank == 0, timeout=timedelta(seconds=30))
        dist.init_process_group("gloo", store=store, rank=rank, world_size=world, timeout=timedelta(seconds=30))
        circuit, ordering, grid, initial, finals = _case()
        evaluate = oracle_evaluate
        if mode == "raise" and rank == 1:
            def evaluate(*a):
                raise RuntimeError("injected failure")
        if mode == "vanish" and rank == 1:
            q.put((rank, "vanished", None))
            q.close()
            q.join_thread()  # flush the queue before the hard exit
            os._exit(0)  # leaves without reporting to the store
        by = "strings" if mode == "strings" else "slices"
        res = shards.evaluate_sharded(evaluate, circuit, ordering, grid, initial, finals, rank=rank,
                                      world=world, store=store, by=by, timeout_s=5.0 if mode == "vanish" else 30.0)
        # Every rank holds the same result: compare a checksum over gloo.
        t = torch.tensor([sum(a.real for _, a in res), sum(a.imag for _, a in res)], dtype=torch.float64)
        lo, hi = t.clone(), t.clone()
        dist.all_reduce(lo, op=dist.ReduceOp.MIN)
        dist.all_reduce(hi, op=dist.ReduceOp.MAX)
        assert torch.equal(lo, hi)
        dist.destroy_process_group()
        q.put((rank, "ok", res))
    except Exception as e:  # noqa: BLE001 -- reported to the parent
        q.put((rank, "error", f"{type(e).__name__}: {e}"))


def _run(mode, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, mode, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(world):
        r, status, payload = q.get(timeout=120)
        out[r] = (status, payload)
    for p in procs:
        p.join(timeout=60)
    return out


def test_string_range_partitions():
    for n in (0, 1, 5, 16, 1023):
        for world in (1, 2, 3, 8):
            got = [shards.string_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            assert max(h - l for l, h in got) - min(h - l for l, h in got) <= 1


def test_shard_ordering_splits_cut_values():
    circuit, ordering, grid, initial, finals = _case()
    assert shards.bond_dimension(circuit, 5, 6) == 4
    parts = [shards.shard_ordering(circuit, ordering, r, 2) for r in range(2)]
    assert parts[0].splitlines()[0] == "cut (0,1) 5 6"
    assert parts[1].splitlines()[0] == "cut (2,3) 5 6"
    assert parts[0].splitlines()[1:] == ordering.strip().splitlines()[1:]
    c3 = rqc.workload("c3")
    p = shards.shard_ordering(c3[0], c3[1], 1, 2, which=1)
    assert [v for _, v, _, _ in shards.cut_lines(p)] == [[0, 1, 2, 3], [2, 3]]
    with pytest.raises(ValueError):
        shards.shard_ordering(circuit, ordering, 0, 5)


def test_slices_sharded_over_two_ranks_sum_to_full_result():
    circuit, ordering, grid, initial, finals = _case()
    want = oracle_evaluate(circuit, ordering, grid, initial, finals)
    out = _run("slices")
    for r in range(2):
        status, res = out[r]
        assert status == "ok", res
        assert [s for s, _ in res] == [s for s, _ in want]
        got = np.array([a for _, a in res])
        ref = np.array([a for _, a in want])
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert out[0][1] == out[1][1]  # same rank-order sum on both ranks


def test_strings_sharded_over_two_ranks_concatenate():
    circuit, ordering, grid, initial, finals = _case()
    want = oracle_evaluate(circuit, ordering, grid, initial, finals)
    out = _run("strings")
    for r in range(2):
        status, res = out[r]
        assert status == "ok", res
        assert [s for s, _ in res] == [s for s, _ in want]
        assert np.allclose([a for _, a in res], [a for _, a in want], rtol=0, atol=1e-15)


def test_rank_that_raises_is_reported_on_every_rank():
    out = _run("raise")
    for r in range(2):
        status, msg = out[r]
        assert status == "error"
        assert "rank 1" in msg and "injected failure" in msg


def test_rank_that_never_reports_times_out():
    out = _run("vanish")
    assert out[1][0] == "vanished"
    status, msg = out[0]
    assert status == "error" and "did not report" in msg and "[1]" in msg


def test_result_codec_round_trips_doubles_exactly():
    """Ranks exchange results as JSON (nothing runs when a payload is read);
    every double comes back bit for bit, NaN included (planning-only
    contexts return NaN amplitudes), and a malformed payload is refused."""
    import math
    import struct

    vals = [0.1 + 0.2j, complex(-1e-300, 5e-324), complex(1.7976931348623157e308, -0.0),
            complex(float("nan"), 1.0), 0j]
    res = [(f"{i:05b}", v) for i, v in enumerate(vals)]
    back = shards.decode_result(shards.encode_result(res))
    assert [s for s, _ in back] == [s for s, _ in res]
    bits = lambda x: struct.pack("<d", x)  # noqa: E731
    for (_, a), (_, b) in zip(res, back):
        for x, y in ((a.real, b.real), (a.imag, b.imag)):
            assert (math.isnan(x) and math.isnan(y)) or bits(x) == bits(y)
    for bad in (b'{"a": 1}', b'[["00", "x", 1.0]]', b'[["00", 1.0]]'):
        with pytest.raises(shards.ShardError):
            shards.decode_result(bad)
