"""Parity of the CUDA path with the oracle and the reference's golden
fixtures, through the C ABI. FP32 CUDA-core path: every amplitude within
1e-5 of the reference's complex<float> result (relative to that amplitude);
permutations bit-exact; products within FP32 rounding."""
import random

import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import Context, QflexGb300Error, rqc, simulate
from tests.conftest import rel_err, rel_err_per_amplitude

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5


def _torch():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch


def test_permute_bit_exact(gpu_ctx):
    torch = _torch()
    rng = random.Random(1)
    for trial in range(80):
        r = rng.randint(0, 14)
        dims = [2 ** rng.randint(0, 3) for _ in range(r)]
        while r and np.prod(dims) > 2 ** 22:
            dims[rng.randrange(r)] = 1
        order = list(range(r))
        rng.shuffle(order)
        n = int(np.prod(dims)) if r else 1
        batch = rng.choice([1, 1, 3])
        host = (np.random.default_rng(trial).standard_normal((batch, n)) +
                1j * np.random.default_rng(trial + 99).standard_normal((batch, n))).astype(np.complex64)
        src = torch.from_numpy(host).cuda()
        dst = torch.zeros_like(src)
        torch.cuda.synchronize()
        gpu_ctx.permute(src.data_ptr(), dst.data_ptr(), dims, order, batch, n)
        gpu_ctx.synchronize()
        for b in range(batch):
            want = host[b].reshape(dims).transpose(order).reshape(-1) if r else host[b]
            assert np.array_equal(dst[b].cpu().numpy(), want), (dims, order)


def test_permute_large(gpu_ctx):
    torch = _torch()
    order = list(range(24))
    random.Random(3).shuffle(order)
    host = np.arange(2 ** 24, dtype=np.float32).astype(np.complex64)
    src = torch.from_numpy(host).cuda()
    dst = torch.empty_like(src)
    torch.cuda.synchronize()
    gpu_ctx.permute(src.data_ptr(), dst.data_ptr(), [2] * 24, order)
    gpu_ctx.synchronize()
    assert np.array_equal(dst.cpu().numpy(), host.reshape([2] * 24).transpose(order).reshape(-1))


def test_reorder_in_place(gpu_ctx):
    torch = _torch()
    dims, order = [4, 2, 8, 16], [2, 0, 3, 1]
    host = (np.arange(1024) * (1 + 0.5j)).astype(np.complex64)
    data = torch.from_numpy(host).cuda()
    scratch = torch.empty_like(data)
    torch.cuda.synchronize()
    gpu_ctx.reorder(data.data_ptr(), scratch.data_ptr(), dims, order)
    gpu_ctx.synchronize()
    assert np.array_equal(data.cpu().numpy(), host.reshape(dims).transpose(order).reshape(-1))


def test_permute_general_dims_bit_exact(gpu_ctx):
    """Dimensions that are not powers of two (the reference's naive reorder):
    the reference's own reorders (tests/golden/reorder_general.json), a
    batched large case, and the in-place reorder, bit for bit."""
    import json

    from tests.conftest import ROOT
    torch = _torch()
    cases = json.loads((ROOT / "tests" / "golden" / "reorder_general.json").read_text())["cases"]
    for case in cases:
        dims, order = case["dims"], case["new_order"]
        n = int(np.prod(dims))
        src = torch.from_numpy(np.arange(n, dtype=np.float32).astype(np.complex64)).cuda()
        dst = torch.zeros_like(src)
        torch.cuda.synchronize()
        gpu_ctx.permute(src.data_ptr(), dst.data_ptr(), dims, order)
        gpu_ctx.synchronize()
        assert np.array_equal(dst.cpu().numpy().real.astype(np.int64), np.array(case["reordered"])), dims
    dims, order, batch = [3, 100, 7, 50, 5], [3, 0, 4, 2, 1], 3
    n = int(np.prod(dims))
    host = (np.random.default_rng(2).standard_normal((batch, n)) + 1j).astype(np.complex64)
    src = torch.from_numpy(host).cuda()
    dst = torch.zeros_like(src)
    torch.cuda.synchronize()
    gpu_ctx.permute(src.data_ptr(), dst.data_ptr(), dims, order, batch, n)
    gpu_ctx.synchronize()
    for b in range(batch):
        assert np.array_equal(dst[b].cpu().numpy(), host[b].reshape(dims).transpose(order).reshape(-1))
    data = torch.from_numpy(host[0].copy()).cuda()
    scratch = torch.empty_like(data)
    torch.cuda.synchronize()
    gpu_ctx.reorder(data.data_ptr(), scratch.data_ptr(), dims, order)
    gpu_ctx.synchronize()
    assert np.array_equal(data.cpu().numpy(), host[0].reshape(dims).transpose(order).reshape(-1))


SHAPES = [(1, 1, 1), (2, 4, 2), (16, 1, 2), (1, 4, 4), (3, 5, 7), (64, 64, 64), (130, 70, 33),
          (256, 16, 16), (16, 256, 16), (4096, 1, 64), (1, 4096, 64), (1, 1, 100000),
          (2, 3, 50000), (513, 257, 129), (1024, 16, 16), (8, 300, 9),
          # vector times matrix with long k: the split-k row-reading kernel
          (1, 64, 1 << 16), (1, 2, 8192), (1, 200, 5000), (1, 256, 4096),
          # n = 16 with short rows: the row-per-thread kernel (ragged last block)
          (128, 16, 16), (300, 16, 7), (65536, 16, 16), (1000, 16, 32), (129, 16, 1)]


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_multiply_matches_fp64(gpu_ctx, m, n, k):
    torch = _torch()
    g = np.random.default_rng(m * 1000 + n * 10 + k)
    A = (g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))).astype(np.complex64)
    B = (g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))).astype(np.complex64)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.zeros((m, n), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    gpu_ctx.multiply(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k)
    gpu_ctx.synchronize()
    want = A.astype(np.complex128) @ B.astype(np.complex128)
    # FP32 accumulation over k terms of unit-variance products.
    tol = 1e-6 * np.sqrt(k) * 8
    assert np.max(np.abs(dC.cpu().numpy() - want)) / np.sqrt(k) < tol


@pytest.mark.parametrize("m,n,k", [(64, 48, 40), (300, 16, 16)])
def test_multiply_batched(gpu_ctx, m, n, k):
    torch = _torch()
    batch = 5
    stride = m * k + k * n + m * n
    g = np.random.default_rng(5)
    buf = (g.standard_normal((batch, stride)) + 1j * g.standard_normal((batch, stride))).astype(np.complex64)
    d = torch.from_numpy(buf).cuda()
    base = d.data_ptr()
    torch.cuda.synchronize()
    gpu_ctx.multiply(base, base + 8 * m * k, base + 8 * (m * k + k * n), m, n, k, batch, stride)
    gpu_ctx.synchronize()
    out = d.cpu().numpy()
    for b in range(batch):
        A = buf[b, :m * k].reshape(m, k).astype(np.complex128)
        B = buf[b, m * k:m * k + k * n].reshape(k, n).astype(np.complex128)
        C = out[b, m * k + k * n:].reshape(m, n)
        assert np.max(np.abs(C - A @ B)) < 1e-4


ENGINE_CASES = ["simple", "c1_4x5_d16", "rect4x4_cut_terminal", "c2_6x6_d24_partial_cut",
                "fsim_3x4_off", "c3_7x7_d32_one_slice"]


@pytest.mark.parametrize("name", ENGINE_CASES)
def test_engine_matches_reference(gpu_ctx, ref_cases, name):
    case = ref_cases[name]
    limit = qo.parse_memory(case["memory_limit"])
    for run in case["runs"]:
        out = gpu_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"],
                               run["final"], limit)
        assert [s for s, _ in out] == run["states"]
        assert gpu_ctx.initial_state() == run["initial_out"]
        assert gpu_ctx.final_state() == run["final_out"]
        want = [complex(*a) for a in run["amplitudes"]]
        assert rel_err_per_amplitude([a for _, a in out], want) < FP32_TOL, name


def test_evaluate_many_matches_single(gpu_ctx, ref_cases):
    case = ref_cases["c1_4x5_d16"]
    finals = [r["final"] for r in case["runs"]]
    many = gpu_ctx.evaluate_many(case["circuit"], case["ordering"], case["grid"], case["initial"], finals)
    for f, (s, a) in zip(finals, many):
        single = gpu_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], case["initial"], f)
        assert single[0][0] == s
        assert abs(single[0][1] - a) <= 1e-6 * abs(a) + 1e-12
    want = [complex(*r["amplitudes"][0]) for r in case["runs"]]
    assert rel_err([a for _, a in many], want) < FP32_TOL


def test_engine_matches_fp64_oracle(gpu_ctx):
    c, o, g, ini, fins = rqc.workload("c1", seed=4)
    out = gpu_ctx.evaluate_many(c, o, g, ini, fins[:4])
    want = []
    for f in fins[:4]:
        inp = qo.Input(qo.Circuit.loads(c), qo.load_ordering(o), qo.Grid.loads(g), ini, f)
        want.append(qo.evaluate_circuit(inp, np.complex128)[0][1])
    assert rel_err([a for _, a in out], want) < FP32_TOL


def test_cut_linearity_at_full_size(gpu_ctx):
    """7x7 (1+32+1), the benchmark ordering: the sum over a cut's value list
    equals the sum of the sums over a partition of that list (a property of
    any size, checked here at the benchmark's own size)."""
    c = rqc.random_circuit(7, 7, 32, seed=0)
    g = rqc.grid_text(7, 7)
    f = rqc.random_bitstrings(49, 1, 2)[0]
    whole = gpu_ctx.evaluate(c, rqc.ordering_7x7((0, 1, 2, 3), (1,)), g, "", f, 1 << 40)[0][1]
    parts = [gpu_ctx.evaluate(c, rqc.ordering_7x7(v, (1,)), g, "", f, 1 << 40)[0][1]
             for v in ((0, 1), (2,), (3,))]
    assert abs(whole - sum(parts)) <= FP32_TOL * abs(whole)


def test_ordering_invariance(gpu_ctx):
    """Amplitudes do not depend on the contraction ordering."""
    c, _, g, ini, fins = rqc.workload("c1", seed=6)
    rows = rqc.row_sweep_ordering(4, 5)
    cols = "".join(f"expand a {i * 5 + j}\n" for j in range(5) for i in range(4))
    two = ("".join(f"expand a {i * 5 + j}\n" for i in range(2) for j in range(5)) +
           "".join(f"expand b {i * 5 + j}\n" for i in (3, 2) for j in range(5)) + "merge a b\n")
    res = [gpu_ctx.evaluate_many(c, o, g, ini, fins[:3]) for o in (rows, cols, two)]
    for other in res[1:]:
        assert rel_err([a for _, a in other], [a for _, a in res[0]]) < FP32_TOL


def test_errors_on_gpu(gpu_ctx, ref_cases):
    for name, frag in (("err_memory_limit", "exceeds memory limit"),
                       ("err_cut_after_expand", "has to be equal to indices[0]")):
        case = ref_cases[name]
        with pytest.raises(QflexGb300Error) as e:
            gpu_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], "", "",
                             qo.parse_memory(case["memory_limit"]))
        assert frag in str(e.value)
    # The context stays usable after an error.
    case = ref_cases["simple"]
    out = gpu_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], "00000", "1100x")
    assert abs(out[0][1] - (0.10669 + 0.04419j)) < 2e-5


def test_simulate_drop_in(built_lib, ref_cases, capsys):
    case = ref_cases["simple"]
    out = simulate({"circuit": case["circuit"].splitlines(), "ordering": case["ordering"].splitlines(),
                    "grid": case["grid"].splitlines(), "initial_state": "00000", "final_state": "1100x"})
    assert [s for s, _ in out] == ["11000", "11001"]
    assert abs(out[1][1] - (-0.01831 - 0.25758j)) < 2e-5
    # Errors print and return [] (src/pybind_main.cpp:127-137).
    bad = simulate({"circuit": case["circuit"].splitlines(), "ordering": case["ordering"].splitlines(),
                    "grid": case["grid"].splitlines(), "initial_state": "00000", "final_state": "1100x",
                    "memory_limit": 512})  # the plan needs 832 bytes
    assert bad == []
    assert "exceeds memory limit" in capsys.readouterr().err


def test_simulate_as_the_cirq_adapter_calls_it(built_lib, ref_cases, tmp_path):
    """The call pattern of the reference's Cirq adapter
    (qflexcirq/interface/qflex_simulator.py:44-60): circuit, ordering and
    grid written to files whose paths go in the *_filename keys, no initial
    state, one simulate() per final state, amplitudes taken as complex(amp[1])
    in the order returned. cirq itself is not installed, so the adapter's own
    code does not run here."""
    case = ref_cases["simple"]
    paths = {}
    for name in ("circuit", "ordering", "grid"):
        paths[name] = tmp_path / f"{name}.txt"
        paths[name].write_text(case[name])
    amplitudes = []
    for bitstring in ("1100x", "0000x"):
        options = {"circuit_filename": str(paths["circuit"]), "ordering_filename": str(paths["ordering"]),
                   "grid_filename": str(paths["grid"]), "final_state": bitstring}
        amplitudes.append([complex(amp[1]) for amp in simulate(options)])
    assert len(amplitudes[0]) == len(amplitudes[1]) == 2
    # The reference's known answer for 1100x from the all-zero initial state
    # (tests/src/evaluate_circuit_test.cpp:203-206).
    assert abs(amplitudes[0][0] - (0.10669 + 0.04419j)) < 2e-5
    assert abs(amplitudes[0][1] - (-0.01831 - 0.25758j)) < 2e-5


@pytest.mark.parametrize("precision", ["fp32", "fp16x3"])
def test_open_terminals_match_projection_and_fp64(built_lib, precision):
    """Terminal cuts as open indices give the amplitudes of the reference's
    projection per value (both engine modes) and of the FP64 oracle."""
    from tests.test_host_planner import _terminal_case
    c, o, g, ini, finals = _terminal_case(3)
    opened, projected = Context(0), Context(0)
    opened.set_precision(precision)
    projected.set_precision(precision)
    projected.set_option("open_terminals", 0)
    a = opened.evaluate_many(c, o, g, ini, finals, 1 << 40)
    b = projected.evaluate_many(c, o, g, ini, finals, 1 << 40)
    assert [s for s, _ in a] == [s for s, _ in b] and len(a) == 8 * len(finals)
    assert opened.stats()["n_ops"] < projected.stats()["n_ops"]
    want = []
    for f in finals:
        inp = qo.Input(qo.Circuit.loads(c), qo.load_ordering(o), qo.Grid.loads(g), ini, f)
        want += qo.evaluate_circuit(inp, np.complex128, float(1 << 40))
    assert [s for s, _ in a] == [s for s, _ in want]
    assert rel_err([x for _, x in a], [x for _, x in b]) < FP32_TOL
    assert rel_err([x for _, x in a], [x for _, x in want]) < FP32_TOL
