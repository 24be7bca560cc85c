"""Micro-benchmarks of the engine's kernels through the C ABI.

    python -m qflex_gb300.kernel_bench gemm --m 4096 --n 4096 --k 4096 --precision tf32x3
    python -m qflex_gb300.kernel_bench gemm --m 65536 --n 256 --k 256 --precision fp16x3 --batch 8
    python -m qflex_gb300.kernel_bench permute --bits 24 --seed 1
    python -m qflex_gb300.kernel_bench step --steps 3 --warmup 2 [--ordering supplied] [--chunk 2]
    python -m qflex_gb300.kernel_bench ops --batch 8 --max-batch 4
    python -m qflex_gb300.kernel_bench bias --precision fp16x3 --chunk 2

Times launches with CUDA events on the context's stream (after warm-up) and
prints one JSON line: average milliseconds per launch and the achieved
rate (algorithmic 8*m*n*k flop per complex product; 16 bytes per element
moved by a permutation).
"""
from __future__ import annotations

import argparse
import json
import random


def _setup(precision: str):
    import torch

    from . import Context
    from ._lib import PRECISIONS
    ctx = Context(0, PRECISIONS[precision])
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    return torch, ctx, stream


def _time(torch, stream, fn, reps: int, warmup: int) -> float:
    for _ in range(warmup):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def gemm(m: int, n: int, k: int, precision: str, reps: int, warmup: int, batch: int = 1,
         variant: int = -1, chunk: int = 0) -> dict:
    """`batch` products per launch (operands of entry b at b * (m k + k n +
    m n) complex); `variant` >= 0 sets the tensor-core kernel variant of the
    shape (qflex_gb300_set_tc_variant)."""
    torch, ctx, stream = _setup(precision)
    if variant >= 0:
        ctx.set_tc_variant(m, n, k, variant)
    if chunk > 0:
        ctx.set_option("tc_chunk", chunk)
    stride = m * k + k * n + m * n
    buf = torch.randn((batch, stride), dtype=torch.complex64, device="cuda")
    base = buf.data_ptr()
    a, b, c = base, base + 8 * m * k, base + 8 * (m * k + k * n)
    ms = _time(torch, stream, lambda: ctx.multiply(a, b, c, m, n, k, batch, stride), reps, warmup)
    return {"kernel": "multiply", "precision": precision, "m": m, "n": n, "k": k, "batch": batch,
            "variant": variant, "chunk": chunk, "ms": ms, "tflops": 8.0 * m * n * k * batch / (ms / 1e3) / 1e12}


def permute(bits: int, seed: int, reps: int, warmup: int) -> dict:
    torch, ctx, stream = _setup("fp32")
    order = list(range(bits))
    random.Random(seed).shuffle(order)
    src = torch.randn(1 << bits, dtype=torch.complex64, device="cuda")
    dst = torch.empty_like(src)
    ms = _time(torch, stream,
               lambda: ctx.permute(src.data_ptr(), dst.data_ptr(), [2] * bits, order), reps, warmup)
    return {"kernel": "permute", "bits": bits, "order": order, "ms": ms,
            "gbs": 16.0 * (1 << bits) / (ms / 1e3) / 1e9}


def step(precision: str, steps: int, warmup: int, batch: int, ordering: str, chunk: int, max_batch: int,
         variant: int = -1, debias: int = -1) -> dict:
    """The benchmark step alone: evaluate_many over `batch` new output
    strings of the 7x7 (1+32+1) workload (16 cut slices), `warmup` untimed
    steps then `steps` timed ones (device time), with the learned or the
    supplied ordering."""
    torch, ctx, stream = _setup(precision)
    from . import rqc
    circuit, supplied, grid, initial, finals = rqc.workload("c3")
    text = rqc.ordering_7x7_learned() if ordering == "learned" else supplied
    if chunk > 0:
        ctx.set_option("tc_chunk", chunk)
    if max_batch > 0:
        ctx.set_option("max_batch", max_batch)
    if variant >= 0:
        ctx.set_option("tc_variant", variant)
    if debias >= 0:
        ctx.set_option("tc_debias", debias)
    for w in range(warmup):
        ctx.evaluate_many(circuit, text, grid, initial, finals[batch * w:batch * (w + 1)], 1 << 40)
    ms = 0.0
    for s in range(steps):
        lo = batch * (warmup + s)
        ctx.evaluate_many(circuit, text, grid, initial, finals[lo:lo + batch], 1 << 40)
        ms += ctx.stats()["device_ms"]
    return {"kernel": "step", "precision": precision, "ordering": ordering, "chunk": chunk, "max_batch": max_batch,
            "variant": variant, "debias": debias,
            "strings": steps * batch, "ms_per_step": ms / steps,
            "amplitudes_per_s": steps * batch / (ms / 1e3)}


def bias(precision: str, chunk: int, debias: int, shapes) -> dict:
    """Mean relative bias of split tensor-core products against complex128
    products of the same complex64 operands (Gaussian entries): beta =
    Re<C - C64, C64> / <C64, C64>, the fraction of itself a product loses to
    the tensor core's truncating accumulation, and the relative RMS error.
    The constants of tc_debias come from this measurement."""
    torch, ctx, stream = _setup(precision)
    ctx.set_option("tc_chunk", chunk)
    ctx.set_option("tc_debias", debias)
    g = torch.Generator(device="cuda").manual_seed(0)
    rows = []
    for m, n, k in shapes:
        A = torch.randn((m, k), dtype=torch.complex64, device="cuda", generator=g)
        B = torch.randn((k, n), dtype=torch.complex64, device="cuda", generator=g)
        C = torch.empty((m, n), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
        ctx.synchronize()
        ref = A.to(torch.complex128) @ B.to(torch.complex128)
        d = C.to(torch.complex128) - ref
        norm = float((ref.abs() ** 2).sum())
        rows.append({"m": m, "n": n, "k": k, "beta": float((d * ref.conj()).real.sum()) / norm,
                     "rel_rms": (float((d.abs() ** 2).sum()) / norm) ** 0.5})
    return {"kernel": "bias", "precision": precision, "chunk": chunk, "debias": debias, "shapes": rows}


def ops(precision: str, batch: int, max_batch: int, reps: int, warmup: int) -> dict:
    """Device time of the benchmark step by operation, warm: `warmup` untimed
    calls of evaluate_many over `batch` strings of the 7x7 (1+32+1)
    workload, then `reps` profiled ones, in which every device op of the last
    pass is bracketed by the engine's own CUDA events (captured graphs are
    not used while profiling). Ops are grouped by kind and shape; times are
    per pass (max_batch strings each) averaged over the profiled calls."""
    import collections
    torch, ctx, stream = _setup(precision)
    from . import rqc
    circuit, _, grid, initial, finals = rqc.workload("c3")
    text = rqc.ordering_7x7_learned()
    if max_batch > 0:
        ctx.set_option("max_batch", max_batch)
    strings = finals[:batch]
    for _ in range(warmup):
        ctx.evaluate_many(circuit, text, grid, initial, strings, 1 << 40)
    names = ["permute", "cuda-core", "tensor-core", "skinny"]
    ms, count, flop = collections.Counter(), collections.Counter(), collections.Counter()
    ctx.set_profiling(True)
    try:
        for _ in range(reps):
            ctx.evaluate_many(circuit, text, grid, initial, strings, 1 << 40)
            for r in ctx.ops():
                key = (names[int(r[0])], int(r[1]), int(r[2]), int(r[3]))
                ms[key] += r[7] / reps
                count[key] += 1.0 / reps
                flop[key] += r[4] * r[6] / reps
    finally:
        ctx.set_profiling(False)
    total = sum(ms.values())
    rows = [{"op": k[0], "m": k[1], "n": k[2], "k": k[3], "launches": round(count[k], 1), "ms": v,
             "share": v / total, "tflops": flop[k] / (v / 1e3) / 1e12 if flop[k] else None}
            for k, v in sorted(ms.items(), key=lambda kv: -kv[1])]
    return {"kernel": "ops", "precision": precision, "strings_per_pass": max_batch, "ms_per_pass": total,
            "ops": rows}


def main() -> None:
    p = argparse.ArgumentParser()
    sub = p.add_subparsers(dest="what", required=True)
    g = sub.add_parser("gemm")
    g.add_argument("--m", type=int, default=4096)
    g.add_argument("--n", type=int, default=4096)
    g.add_argument("--k", type=int, default=4096)
    g.add_argument("--precision", default="tf32x3")
    g.add_argument("--batch", type=int, default=1)
    g.add_argument("--variant", type=int, default=-1,
                   help="tensor-core kernel variant: 0 single CTA, 1 CTA pair, 2 five stages")
    q = sub.add_parser("permute")
    q.add_argument("--bits", type=int, default=24)
    q.add_argument("--seed", type=int, default=1)
    bs = sub.add_parser("bias")
    bs.add_argument("--precision", default="fp16x3")
    bs.add_argument("--chunk", type=int, default=1)
    bs.add_argument("--debias", type=int, default=0)
    st = sub.add_parser("step")
    st.add_argument("--precision", default="fp16x3")
    st.add_argument("--steps", type=int, default=3)
    st.add_argument("--batch", type=int, default=8)
    st.add_argument("--ordering", default="learned", choices=["learned", "supplied"])
    st.add_argument("--chunk", type=int, default=0, help="TMEM chunk (0: the default)")
    st.add_argument("--max-batch", type=int, default=4, help="strings per device pass (0: all that fit)")
    st.add_argument("--variant", type=int, default=-1, help="tensor-core kernel of every product (tc_variant)")
    st.add_argument("--debias", type=int, default=-1, help="tc_debias option (-1: the default)")
    op = sub.add_parser("ops")
    op.add_argument("--precision", default="fp16x3")
    op.add_argument("--batch", type=int, default=8)
    op.add_argument("--max-batch", type=int, default=4, help="strings per device pass")
    for s in (g, q):
        s.add_argument("--reps", type=int, default=5)
    op.add_argument("--reps", type=int, default=3)
    for s in (g, q, st, op):
        s.add_argument("--warmup", type=int, default=2)
    g.add_argument("--chunk", type=int, default=0, help="TMEM chunk (0: the default)")
    a = p.parse_args()
    if a.what == "gemm":
        out = gemm(a.m, a.n, a.k, a.precision, a.reps, a.warmup, a.batch, a.variant, a.chunk)
    elif a.what == "step":
        out = step(a.precision, a.steps, a.warmup, a.batch, a.ordering, a.chunk, a.max_batch, a.variant, a.debias)
    elif a.what == "ops":
        out = ops(a.precision, a.batch, a.max_batch, a.reps, a.warmup)
    elif a.what == "bias":
        out = bias(a.precision, a.chunk, a.debias,
                   [(4096, 4096, 4096), (65536, 256, 256), (4096, 256, 4096), (16384, 1024, 64), (1024, 1024, 16)])
    else:
        out = permute(a.bits, a.seed, a.reps, a.warmup)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
