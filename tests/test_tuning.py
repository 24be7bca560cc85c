"""Tuning options of a context and the autotuner: option validation and
the tensor-core shape list on CPU (planning-only context); on the GPU,
results that do not depend on the kernel variant, graph replay or the
strings-per-pass limit, and an autotuning run."""
import numpy as np
import pytest

from qflex_gb300 import TF32X3, Context, QflexGb300Error, autotune, rqc
from tests.conftest import rel_err


def test_options_round_trip_and_validation(built_lib):
    c = Context(-1, TF32X3)
    assert c.get_option("tc_chunk") >= 1
    for name, value in (("tc_chunk", 4), ("tc_pair", 0), ("graphs", 0), ("max_batch", 3), ("fuse_splits", 0),
                        ("open_terminals", 0)):
        c.set_option(name, value)
        assert c.get_option(name) == value
    for name, value in (("tc_chunk", 0), ("tc_chunk", 65), ("tc_chunk", 1.5), ("tc_pair", 2),
                        ("graphs", -1), ("max_batch", -1), ("fuse_splits", 2), ("no_such_option", 1)):
        with pytest.raises(QflexGb300Error):
            c.set_option(name, value)
    with pytest.raises(QflexGb300Error):
        c.get_option("no_such_option")
    c.set_tc_variant(4096, 4096, 4096, 1)
    c.set_tc_variant(4096, 4096, 4096, 2)
    c.set_tc_variant(4096, 4096, 4096, 3)
    c.set_tc_variant(4096, 4096, 4096, -1)
    c.set_tc_variant(4096, 4096, 4096, 4)
    c.set_tc_variant(4096, 4096, 4096, -1)
    with pytest.raises(QflexGb300Error):
        c.set_tc_variant(64, 64, 64, 5)
    c.set_option("tc_variant", 4)
    assert c.get_option("tc_variant") == 4
    with pytest.raises(QflexGb300Error):
        c.set_option("tc_variant", 5)


def test_tc_shapes_of_7x7_plan(built_lib):
    circuit, ordering, grid, _, _ = rqc.workload("c3")
    shapes = autotune.tc_shapes(circuit, ordering, grid)
    assert shapes[0] == (4096, 4096, 4096, 20)
    assert (65536, 256, 256, 109) in shapes
    assert all(autotune.tc_eligible(m, n, k) for m, n, k, _ in shapes)
    flops = [m * n * k * c for m, n, k, c in shapes]
    assert flops == sorted(flops, reverse=True)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["tf32x3", "fp16x3"])
def test_variants_graphs_and_batches_agree(built_lib, precision):
    from qflex_gb300 import FP16X3
    circuit, ordering, grid, initial, finals = rqc.workload("c2")
    finals = finals[:6]
    ctx = Context(0, TF32X3 if precision == "tf32x3" else FP16X3)
    base = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)]
    shapes = autotune.tc_shapes(circuit, ordering, grid)
    assert shapes
    for variant in autotune.variants(ctx):
        for m, n, k, _ in shapes:
            ctx.set_tc_variant(m, n, k, variant)
        for _ in range(3):  # eager, captured, replayed
            got = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)]
            assert rel_err(got, base) < 1e-5, variant
    ctx.set_option("graphs", 0)
    ctx.set_option("max_batch", 4)  # 6 strings -> passes of 4 and 2
    got = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)]
    assert rel_err(got, base) < 1e-5
    assert ctx.stats()["batch"] == 4


def test_choose_batch_prefers_larger_passes_on_near_ties():
    """The strings-per-pass rule: the largest limit within 1 % of the
    fastest, otherwise the fastest."""
    assert autotune.choose_batch({1: 48.5, 2: 46.3, 4: 44.12, 8: 43.89}) == 8
    assert autotune.choose_batch({1: 48.5, 2: 46.3, 4: 43.89, 8: 44.12}) == 8
    assert autotune.choose_batch({1: 48.5, 2: 46.3, 4: 43.0, 8: 44.12}) == 4
    assert autotune.choose_batch({4: 10.0}) == 4
    assert autotune.choose_batch({1: 10.0, 2: 10.05}, tolerance=0.0) == 1


@pytest.mark.gpu
def test_autotune_sets_choices(built_lib, tmp_path):
    import torch
    circuit, ordering, grid, initial, finals = rqc.workload("c2")
    finals = finals[:4]
    ctx = Context(0, TF32X3)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    cache = tmp_path / "tune.json"
    res = autotune.tune(ctx, circuit, ordering, grid, initial, finals, batches=(1, 2, 4), cache=cache,
                        stream=stream)
    assert not res["cached"] and res["max_batch"] in (1, 2, 4)
    assert res["products"] and all(r["variant"] in (0, 1) for r in res["products"].values())
    assert ctx.get_option("max_batch") == res["max_batch"]
    again = autotune.tune(Context(0, TF32X3), circuit, ordering, grid, initial, finals, batches=(1, 2, 4),
                          cache=cache, stream=stream)
    assert again["cached"] and again["max_batch"] == res["max_batch"]
    out = ctx.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)
    assert np.isfinite([abs(a) for _, a in out]).all()


@pytest.mark.gpu
def test_fused_fp16_planes_match_split(built_lib):
    """3xFP16 with permutations writing the products' A planes directly
    (per-32-value scales) against the separate split (per-row scales) and
    the FP64 oracle, on the 6x6 workload and one 7x7 slice."""
    from oracle import qflex_oracle as qo
    from qflex_gb300 import FP16X3
    cases = [rqc.workload("c2")[:4] + (rqc.workload("c2")[4][:3],)]
    c7 = rqc.random_circuit(7, 7, 32, seed=0)
    cases.append((c7, rqc.ordering_7x7((0,), (1,)), rqc.grid_text(7, 7), "", rqc.random_bitstrings(49, 2, 5)))
    for circuit, ordering, grid, initial, finals in cases:
        fused, split = Context(0, FP16X3), Context(0, FP16X3)
        split.set_option("fuse_splits", 0)
        a = [x for _, x in fused.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)]
        b = [x for _, x in split.evaluate_many(circuit, ordering, grid, initial, finals, 1 << 40)]
        assert fused.stats()["launches"] < split.stats()["launches"]
        want = []
        for f in finals:
            inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), initial, f)
            want.append(qo.evaluate_circuit(inp, np.complex128, float(1 << 40))[0][1])
        assert rel_err(a, want) < 1e-5 and rel_err(b, want) < 1e-5
        assert rel_err(a, b) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [1, 2, 3, 4], ids=["pair", "deep", "wide", "narrow"])
def test_fp16x3_variant_matches_single_and_fp64(built_lib, variant):
    """The CTA-pair, five-stage, 16-epilogue-warp and 64-column 3xFP16 kernels on every product of one
    7x7 slice (fused plane permutations included) against the single-CTA
    kernel and the FP64 oracle."""
    from oracle import qflex_oracle as qo
    from qflex_gb300 import FP16X3
    circuit, grid = rqc.random_circuit(7, 7, 32, seed=0), rqc.grid_text(7, 7)
    ordering, finals = rqc.ordering_7x7((0,), (1,)), rqc.random_bitstrings(49, 2, 9)
    single, pair = Context(0, FP16X3), Context(0, FP16X3)
    for m, n, k, _ in autotune.tc_shapes(circuit, ordering, grid):
        pair.set_tc_variant(m, n, k, variant)
    a = [x for _, x in single.evaluate_many(circuit, ordering, grid, "", finals, 1 << 40)]
    b = [x for _, x in pair.evaluate_many(circuit, ordering, grid, "", finals, 1 << 40)]
    want = []
    for f in finals:
        inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(ordering), qo.Grid.loads(grid), "", f)
        want.append(qo.evaluate_circuit(inp, np.complex128, float(1 << 40))[0][1])
    assert rel_err(b, want) < 1e-5 and rel_err(a, want) < 1e-5
    assert rel_err(a, b) < 1e-5


def test_variant_sets_per_precision(built_lib):
    """The product tuner times the five-stage kernel only for 3xFP16."""
    from qflex_gb300 import FP16X3
    assert autotune.variants(Context(-1, FP16X3)) == (0, 1, 2, 3, 4)
    assert autotune.variants(Context(-1, TF32X3)) == (0, 1)
    c = Context(-1, TF32X3)
    c.set_precision("fp16x3")
    assert autotune.variants(c) == (0, 1, 2, 3, 4)
