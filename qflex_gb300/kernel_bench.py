"""Micro-benchmarks of the engine's kernels through the C ABI.

    python -m qflex_gb300.kernel_bench gemm --m 4096 --n 4096 --k 4096 --precision tf32x3
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


def gemm(m: int, n: int, k: int, precision: str, reps: int, warmup: int) -> dict:
    torch, ctx, stream = _setup(precision)
    A = torch.randn((m, k), dtype=torch.complex64, device="cuda")
    B = torch.randn((k, n), dtype=torch.complex64, device="cuda")
    C = torch.empty((m, n), dtype=torch.complex64, device="cuda")
    ms = _time(torch, stream, lambda: ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k),
               reps, warmup)
    return {"kernel": "multiply", "precision": precision, "m": m, "n": n, "k": k, "ms": ms,
            "tflops": 8.0 * m * n * k / (ms / 1e3) / 1e12}


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
    q = sub.add_parser("permute")
    q.add_argument("--bits", type=int, default=24)
    q.add_argument("--seed", type=int, default=1)
    for s in (g, q):
        s.add_argument("--reps", type=int, default=5)
        s.add_argument("--warmup", type=int, default=2)
    a = p.parse_args()
    if a.what == "gemm":
        out = gemm(a.m, a.n, a.k, a.precision, a.reps, a.warmup)
    else:
        out = permute(a.bits, a.seed, a.reps, a.warmup)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
