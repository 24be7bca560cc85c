"""Split-precision tcgen05 products (3xTF32, 3xFP16 with power-of-two row
scaling, BF16x3) and the engine in those modes; every test runs for each.
Tolerance: per-amplitude error within 1e-5 of the RMS amplitude against
the reference's complex<float> results and the FP64 oracle; products within
2e-5 of the FP64 product relative to its mean magnitude (the FP32
CUDA-core kernel's own error at k = 4096)."""
import numpy as np
import pytest

from oracle import qflex_oracle as qo
from qflex_gb300 import BF16X3, FP16X3, TF32X3, Context, rqc
from tests.conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module", params=[TF32X3, FP16X3, BF16X3], ids=["tf32x3", "fp16x3", "bf16x3"])
def tc_ctx(built_lib, request):
    return Context(0, request.param)


# Ragged m and n leave whole tiles partly outside the matrix; an odd n
# (97, 131) takes the epilogue's plain stores instead of the bulk tensor
# stores.
@pytest.mark.parametrize("m,n,k", [(128, 128, 16), (64, 64, 16), (256, 512, 128), (1024, 256, 256),
                                   (300, 128, 64), (128, 1024, 40), (4096, 256, 256), (256, 64, 16),
                                   (512, 96, 24), (768, 200, 100), (2048, 2048, 2048), (256, 97, 64),
                                   (200, 131, 48)])
def test_split_multiply(tc_ctx, m, n, k):
    import torch
    g = np.random.default_rng(m + 7 * n + 13 * k)
    A = (g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))).astype(np.complex64)
    B = (g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))).astype(np.complex64)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.full((m, n), float("nan"), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    tc_ctx.multiply(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k)
    tc_ctx.synchronize()
    got = dC.cpu().numpy()
    want = A.astype(np.complex128) @ B.astype(np.complex128)
    # Relative to the mean magnitude: FP32 CUDA-core products reach 1.7e-5
    # at k = 4096 on this data; the split product must do as well.
    err = np.max(np.abs(got - want)) / np.mean(np.abs(want))
    assert np.isfinite(got).all()
    assert err < 2e-5, err


ENGINE_CASES = ["c1_4x5_d16", "rect4x4_cut_terminal", "c2_6x6_d24_partial_cut", "fsim_3x4_off",
                "c3_7x7_d32_one_slice"]


@pytest.mark.parametrize("name", ENGINE_CASES)
def test_split_engine_close_to_reference(tc_ctx, ref_cases, name):
    """Against the reference's complex<float> results. The split path
    evaluates the gates from double constants; the reference's float gate
    constants alone move a 7x7 amplitude by ~7e-6, so the bound there is
    3e-5 (the FP64 tests below hold the split path to 1e-5)."""
    case = ref_cases[name]
    limit = qo.parse_memory(case["memory_limit"])
    finals = [r["final"] for r in case["runs"]]
    out = tc_ctx.evaluate_many(case["circuit"], case["ordering"], case["grid"], case["initial"], finals,
                               limit)
    want = [complex(*a) for r in case["runs"] for a in r["amplitudes"]]
    assert [s for s, _ in out] == [s for r in case["runs"] for s in r["states"]]
    tol = 3e-5 if name.startswith("c3") else TOL
    assert rel_err([a for _, a in out], want) < tol, name


@pytest.mark.parametrize("name", ["c1_4x5_d16", "rect4x4_cut_terminal", "fsim_3x4_off", "c2_6x6_d24_partial_cut"])
def test_split_engine_matches_fp64(tc_ctx, ref_cases, name):
    case = ref_cases[name]
    runs = case["runs"][:3]
    out = tc_ctx.evaluate_many(case["circuit"], case["ordering"], case["grid"], case["initial"],
                               [r["final"] for r in runs], 1 << 40)
    want = []
    for r in runs:
        inp = qo.Input(qo.Circuit.loads(case["circuit"]), qo.load_ordering(case["ordering"]),
                       qo.Grid.loads(case["grid"]), case["initial"], r["final"])
        want += [a for _, a in qo.evaluate_circuit(inp, np.complex128, float(1 << 40))]
    assert rel_err([a for _, a in out], want) < TOL, name


def test_split_7x7_within_1e5_of_fp64(tc_ctx):
    """7x7 (1+32+1), benchmark ordering with one value per cut: per-amplitude
    relative error against the FP64 oracle below 1e-5."""
    c = rqc.random_circuit(7, 7, 32, seed=0)
    g = rqc.grid_text(7, 7)
    o = rqc.ordering_7x7((0,), (1,))
    finals = rqc.random_bitstrings(49, 2, 21)
    got = [a for _, a in tc_ctx.evaluate_many(c, o, g, "", finals, 1 << 40)]
    for f, a in zip(finals, got):
        inp = qo.Input(qo.Circuit.loads(c), qo.load_ordering(o), qo.Grid.loads(g), "", f)
        want = qo.evaluate_circuit(inp, np.complex128, float(1 << 40))[0][1]
        assert abs(a - want) <= TOL * abs(want), (f, a, want)


def test_split_plan_uses_tensor_cores(tc_ctx, ref_cases):
    case = ref_cases["c3_7x7_d32_one_slice"]
    tc_ctx.evaluate(case["circuit"], case["ordering"], case["grid"], "", "", 1 << 40)
    plan = Context(-1, TF32X3)
    plan.evaluate(case["circuit"], case["ordering"], case["grid"], "", "", 1 << 40)
    assert plan.gemms() == [tuple(g) for g in case["runs"][0]["gemms"]]


def test_split_vs_fp64_oracle_c1(tc_ctx):
    c, o, g, ini, fins = rqc.workload("c1", seed=8)
    out = tc_ctx.evaluate_many(c, o, g, ini, fins[:4])
    want = []
    for f in fins[:4]:
        inp = qo.Input(qo.Circuit.loads(c), qo.load_ordering(o), qo.Grid.loads(g), ini, f)
        want.append(qo.evaluate_circuit(inp, np.complex128)[0][1])
    assert rel_err([a for _, a in out], want) < TOL


def test_fp16x3_rows_of_any_magnitude(built_lib):
    """Rows of A and B spanning 1e-30 .. 1e30: the power-of-two row scales
    keep every output element within 2e-5 of its own row-column scale."""
    import torch
    ctx = Context(0, FP16X3)
    m, n, k = 256, 128, 64
    g = np.random.default_rng(3)
    ra = 10.0 ** g.uniform(-30, 30, size=(m, 1))
    rb = 10.0 ** g.uniform(-8, 8, size=(1, n))
    A = ((g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))) * ra).astype(np.complex64)
    B = ((g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))) * rb).astype(np.complex64)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.empty((m, n), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.multiply(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k)
    ctx.synchronize()
    got = dC.cpu().numpy().astype(np.complex128)
    want = A.astype(np.complex128) @ B.astype(np.complex128)
    scale = ra * rb * np.sqrt(k)  # typical magnitude of each element
    ok = np.isfinite(scale) & (scale > 1e-36) & (scale < 1e36)  # products FP32 can hold
    err = np.abs(got - want) / scale
    assert np.max(err[ok]) < 2e-5, np.max(err[ok])


@pytest.mark.parametrize("precision,variant", [(TF32X3, 1), (FP16X3, 1), (FP16X3, 2)],
                         ids=["tf32x3_pair", "fp16x3_pair", "fp16x3_deep"])
@pytest.mark.parametrize("m,n,k", [(256, 128, 16), (300, 128, 64), (512, 96, 24), (1024, 256, 256),
                                   (128, 128, 32), (1536, 384, 1024)])
def test_kernel_variant(built_lib, precision, variant, m, n, k):
    """The CTA-pair (cta_group::2) kernels and the five-stage 3xFP16 kernel,
    ragged shapes included (m = 128 leaves the odd CTA's rows of a pair
    outside the matrix)."""
    import torch
    ctx = Context(0, precision)
    ctx.set_tc_variant(m, n, k, variant)
    g = np.random.default_rng(m + n + k)
    A = (g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))).astype(np.complex64)
    B = (g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))).astype(np.complex64)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.full((m, n), float("nan"), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.multiply(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), m, n, k)
    ctx.synchronize()
    got = dC.cpu().numpy()
    want = A.astype(np.complex128) @ B.astype(np.complex128)
    assert np.isfinite(got).all()
    assert np.max(np.abs(got - want)) / np.mean(np.abs(want)) < 2e-5


@pytest.mark.parametrize("extra", [0, 1], ids=["even_stride", "odd_stride"])
def test_tensorcore_multiply_batched(tc_ctx, extra):
    """Batched products with the batch entries `stride` complex apart; an odd
    stride takes the plain-store epilogue, an even one the bulk stores."""
    import torch
    m, n, k, batch = 192, 96, 48, 3
    stride = m * k + k * n + m * n + extra
    g = np.random.default_rng(11 + extra)
    buf = (g.standard_normal((batch, stride)) + 1j * g.standard_normal((batch, stride))).astype(np.complex64)
    d = torch.from_numpy(buf).cuda()
    base = d.data_ptr()
    torch.cuda.synchronize()
    tc_ctx.multiply(base, base + 8 * m * k, base + 8 * (m * k + k * n), m, n, k, batch, stride)
    tc_ctx.synchronize()
    out = d.cpu().numpy()
    for b in range(batch):
        A = buf[b, :m * k].reshape(m, k).astype(np.complex128)
        B = buf[b, m * k:m * k + k * n].reshape(k, n).astype(np.complex128)
        C = out[b, m * k + k * n:m * k + k * n + m * n].reshape(m, n)
        want = A @ B
        assert np.max(np.abs(C - want)) / np.mean(np.abs(want)) < 2e-5, b
        assert np.array_equal(out[b, m * k + k * n + m * n:], buf[b, m * k + k * n + m * n:])


@pytest.mark.parametrize("precision", [FP16X3, TF32X3], ids=["fp16x3", "tf32x3"])
def test_expired_pipeline_wait_is_reported_and_context_recovers(built_lib, precision):
    """Every pipeline wait of the tensor-core kernels is bounded. With the
    limit set to 1 ns the first wait that has to spin runs out: its thread
    block drains what it started and returns, the call reports
    QFLEX_GB300_ERR_CUDA, and with the default limit restored the same
    context computes the same amplitudes and products as before."""
    import torch

    from qflex_gb300 import QflexGb300Error
    circuit = rqc.random_circuit(6, 6, 24, seed=0)
    grid = rqc.grid_text(6, 6)
    ordering = rqc.ordering_6x6(cut_values=(1,))
    finals = rqc.random_bitstrings(36, 2, 3)
    ctx = Context(0, precision)
    good = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, "", finals, 1 << 40)]
    g = np.random.default_rng(4)
    m = n = k = 512
    A = torch.from_numpy((g.standard_normal((m, k)) + 1j * g.standard_normal((m, k))).astype(np.complex64)).cuda()
    B = torch.from_numpy((g.standard_normal((k, n)) + 1j * g.standard_normal((k, n))).astype(np.complex64)).cuda()
    C = torch.zeros((m, n), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()

    ctx.set_option("tc_wait_ns", 1)
    assert ctx.get_option("tc_wait_ns") == 1
    with pytest.raises(QflexGb300Error) as e:
        ctx.evaluate_many(circuit, ordering, grid, "", finals, 1 << 40)
    assert e.value.code == 2 and "pipeline wait expired" in str(e.value)
    ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    with pytest.raises(QflexGb300Error) as e:
        ctx.synchronize()
    assert e.value.code == 2 and "pipeline wait expired" in str(e.value)

    ctx.set_option("tc_wait_ns", 0)
    again = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, "", finals, 1 << 40)]
    assert again == good
    ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    ctx.synchronize()
    want = A.cpu().numpy().astype(np.complex128) @ B.cpu().numpy().astype(np.complex128)
    assert np.max(np.abs(C.cpu().numpy() - want)) < 2e-5 * np.mean(np.abs(want))



def test_split_paths_per_amplitude_on_the_16_slice_workload(built_lib):
    """The full 7x7 (1+32+1) workload (two cuts x 4 values, 16 slices).
    Every split precision: each of the 16 amplitudes of
    tests/golden/c3_fp64.json (CPU complex128 oracle) within 1e-5 of it.
    The default 3xFP16 path on the 256 strings of
    tests/golden/c3_fp64_gpu.json (GPU complex128 oracle): every amplitude
    within 5e-6 of the RMS amplitude, the systematic shrink left after the
    compensation of the tensor core's truncating accumulation below 1e-6,
    and at least 95 % of the
    amplitudes within 1e-5 of themselves (the rest are the smallest
    amplitudes, down to 0.05 of the RMS, whose relative error complex64
    arithmetic cannot hold to 1e-5: the FP32 CUDA-core path's largest is
    5.5e-5 on the same strings)."""
    import json

    from tests.conftest import ROOT, rel_err_per_amplitude
    circuit, ordering, grid, initial, finals = rqc.workload("c3")
    cpu = json.loads((ROOT / "tests" / "golden" / "c3_fp64.json").read_text())
    strings = [r["final"] for r in cpu["amplitudes"]]
    want = [complex(*r["amplitude"]) for r in cpu["amplitudes"]]
    assert len(strings) >= 16
    for precision in (TF32X3, FP16X3, BF16X3):
        ctx = Context(0, precision)
        got = [a for _, a in ctx.evaluate_many(circuit, ordering, grid, initial, strings, 1 << 40)]
        assert rel_err_per_amplitude(got, want) < TOL, precision
        ctx.close()
    gpu = json.loads((ROOT / "tests" / "golden" / "c3_fp64_gpu.json").read_text())
    strings = [r["final"] for r in gpu["amplitudes"]]
    want = np.array([complex(*r["amplitude"]) for r in gpu["amplitudes"]])
    ctx = Context(0, FP16X3)
    got = []
    for i in range(0, len(strings), 8):
        got += [a for _, a in ctx.evaluate_many(circuit, ordering, grid, initial, strings[i:i + 8], 1 << 40)]
    got = np.array(got)
    rms = np.sqrt(np.mean(np.abs(want) ** 2))
    per_amp = np.abs(got - want) / np.abs(want)
    assert np.max(np.abs(got - want)) / rms < 5e-6
    assert abs(np.mean((got / want).real) - 1) < 1e-6
    assert np.mean(per_amp <= TOL) >= 0.95 and np.max(per_amp) < 3e-5



@pytest.mark.parametrize("precision", [FP16X3, TF32X3, BF16X3], ids=["fp16x3", "tf32x3", "bf16x3"])
def test_truncation_bias_compensation(built_lib, precision):
    """A split product comes out smaller than the exact product by a stable
    fraction (the tensor core's accumulation rounds toward zero); with
    tc_debias (the default) the mean relative bias over a product's elements,
    Re<C - C64, C64> / <C64, C64>, is a tenth of what it is without, at the
    default chunk of two k-steps."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(1)
    m, n, k = 4096, 256, 1024
    A = torch.randn((m, k), dtype=torch.complex64, device="cuda", generator=g)
    B = torch.randn((k, n), dtype=torch.complex64, device="cuda", generator=g)
    ref = A.to(torch.complex128) @ B.to(torch.complex128)
    beta = {}
    for debias in (0, 1):
        ctx = Context(0, precision)
        assert ctx.get_option("tc_debias") == 1 and ctx.get_option("tc_chunk") == 2
        ctx.set_option("tc_debias", debias)
        C = torch.empty((m, n), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
        ctx.synchronize()
        d = C.to(torch.complex128) - ref
        beta[debias] = float((d * ref.conj()).real.sum() / (ref.abs() ** 2).sum())
    assert beta[0] < -5e-8
    assert abs(beta[1]) < 0.1 * abs(beta[0])
