"""Micro-benchmarks of the engine's kernels through the C ABI.

    python -m qflex_gb300.kernel_bench gemm --m 4096 --n 4096 --k 4096 --precision tf32x3
    python -m qflex_gb300.kernel_bench gemm --m 65536 --n 256 --k 256 --precision fp16x3 --batch 8
    python -m qflex_gb300.kernel_bench permute --bits 24 --seed 1

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
         variant: int = -1) -> dict:
    """`batch` products per launch (operands of entry b at b * (m k + k n +
    m n) complex); `variant` >= 0 sets the tensor-core kernel variant of the
    shape (qflex_gb300_set_tc_variant)."""
    torch, ctx, stream = _setup(precision)
    if variant >= 0:
        ctx.set_tc_variant(m, n, k, variant)
    stride = m * k + k * n + m * n
    buf = torch.randn((batch, stride), dtype=torch.complex64, device="cuda")
    base = buf.data_ptr()
    a, b, c = base, base + 8 * m * k, base + 8 * (m * k + k * n)
    ms = _time(torch, stream, lambda: ctx.multiply(a, b, c, m, n, k, batch, stride), reps, warmup)
    return {"kernel": "multiply", "precision": precision, "m": m, "n": n, "k": k, "batch": batch,
            "variant": variant, "ms": ms, "tflops": 8.0 * m * n * k * batch / (ms / 1e3) / 1e12}


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
    for s in (g, q):
        s.add_argument("--reps", type=int, default=5)
        s.add_argument("--warmup", type=int, default=2)
    a = p.parse_args()
    if a.what == "gemm":
        out = gemm(a.m, a.n, a.k, a.precision, a.reps, a.warmup, a.batch, a.variant)
    else:
        out = permute(a.bits, a.seed, a.reps, a.warmup)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
