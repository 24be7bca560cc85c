"""Autotuner of the engine's launch choices for one workload.

Chosen by measurement on the current GPU:
  * for every tensor-core product shape of the plan, the kernel variant --
    the single-CTA 128 x 128 tile or the CTA-pair (cta_group::2) 256 x 128
    tile -- timing both on random operands of that shape through the C
    ABI's multiply (qflex_gb300_multiply);
  * the number of output strings per device pass (the "max_batch" option),
    timing evaluate_many on the workload's own strings.
The TMEM chunk length is not tuned: it trades accuracy for speed, and 2
k-steps is the longest that keeps 7x7 (1+32+1) amplitudes within 1e-5 of
FP64. Results can be cached in a JSON file keyed by the GPU name and the
plan's product shapes.
"""
from __future__ import annotations

import json
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Tuple

from ._lib import FP16X3, TF32X3, Context

VARIANTS = (0, 1)  # single CTA, CTA pair
FP16_VARIANTS = (0, 1, 2, 3, 4)  # + five stages, 16 epilogue warps, 64-column tiles (3xFP16)


def variants(ctx: Context) -> Tuple[int, ...]:
    """Kernel variants the product tuner times for the context's precision."""
    return FP16_VARIANTS if getattr(ctx, "precision", None) == FP16X3 else VARIANTS


def tc_eligible(m: int, n: int, k: int) -> bool:
    """Shapes the engine runs on the tensor cores (tc_eligible in
    qflex_gb300/csrc/tc_gemm.cu)."""
    return m >= 64 and n >= 64 and k >= 16 and k % 4 == 0


def tc_shapes(circuit: str, ordering: str, grid: str, memory_limit: float = float(1 << 40)
              ) -> List[Tuple[int, int, int, int]]:
    """(m, n, k, count) of the plan's tensor-core products, most flop first."""
    plan = Context(-1, TF32X3)
    try:
        plan.evaluate(circuit, ordering, grid, "", "", memory_limit)
        shapes = [s for s in plan.shapes() if tc_eligible(*s[:3])]
    finally:
        plan.close()
    return sorted(shapes, key=lambda s: -s[0] * s[1] * s[2] * s[3])


def _time_multiply(ctx: Context, stream, m: int, n: int, k: int, reps: int, warmup: int) -> float:
    """CUDA-event time of one product on `stream`, the torch stream the
    context runs on."""
    import torch
    with torch.cuda.stream(stream):
        A = torch.randn((m, k), dtype=torch.complex64, device="cuda")
        B = torch.randn((k, n), dtype=torch.complex64, device="cuda")
        C = torch.empty((m, n), dtype=torch.complex64, device="cuda")
    stream.synchronize()
    for _ in range(warmup):
        ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    e1.record(stream)
    stream.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_products(ctx: Context, stream, shapes: Sequence[Tuple[int, int, int, int]], reps: int = 3,
                  warmup: int = 1, max_shapes: int = 8) -> Dict[str, dict]:
    """Times every variant on the `max_shapes` heaviest shapes and sets the
    fastest on `ctx`. Returns {"m,n,k": {"variant": v, "ms": {v: ms}}}."""
    out = {}
    for m, n, k, _ in list(shapes)[:max_shapes]:
        ms = {}
        for v in variants(ctx):
            ctx.set_tc_variant(m, n, k, v)
            ms[v] = _time_multiply(ctx, stream, m, n, k, reps, warmup)
        best = min(ms, key=ms.get)
        ctx.set_tc_variant(m, n, k, best)
        out[f"{m},{n},{k}"] = {"variant": best, "ms": {str(v): t for v, t in ms.items()}}
    return out


def choose_batch(per_amp: dict, tolerance: float = 0.01) -> int:
    """The strings-per-pass limit to use, from device time per amplitude by
    limit: the largest limit within `tolerance` of the fastest. Such near
    ties are inside the spread of one call at the power cap, and a larger
    pass makes fewer launches for the same work."""
    best = min(per_amp.values())
    return max(b for b, t in per_amp.items() if t <= best * (1.0 + tolerance))


def tune_batch(ctx: Context, circuit: str, ordering: str, grid: str, initial: str,
               finals: Sequence[str], memory_limit: float, batches: Sequence[int] = (1, 2, 4, 8, 16),
               reps: int = 3) -> dict:
    """Device time per amplitude of evaluate_many over `finals` for each
    strings-per-pass limit, the best of `reps` calls after one untimed call;
    sets choose_batch's pick as "max_batch". Neighbouring limits often differ
    by 1-2 %, about the spread of a single call at the power cap, hence the
    repeats and the tie rule."""
    per_amp = {}
    for b in batches:
        if b > len(finals):
            continue
        ctx.set_option("max_batch", b)
        ctx.evaluate_many(circuit, ordering, grid, initial, list(finals), memory_limit)  # warm-up / graph
        best = float("inf")
        for _ in range(reps):
            ctx.evaluate_many(circuit, ordering, grid, initial, list(finals), memory_limit)
            best = min(best, ctx.stats()["device_ms"])
        per_amp[b] = best / len(finals)
    if not per_amp:
        return {"max_batch": 0, "ms_per_string": {}}
    choice = choose_batch(per_amp)
    ctx.set_option("max_batch", choice)
    return {"max_batch": choice, "ms_per_string": {str(b): t for b, t in per_amp.items()}}


def tune(ctx: Context, circuit: str, ordering: str, grid: str, initial: str, finals: Sequence[str],
         memory_limit: float = float(1 << 40), batches: Sequence[int] = (1, 2, 4, 8, 16),
         cache: Optional[Path] = None, stream=None, products: bool = True) -> dict:
    """Tunes `ctx` for this workload (products first unless `products` is
    False, then strings per pass) and returns the choices. `stream` is the torch stream the context
    runs on (a new one is set on the context when None). With `cache`, a
    result stored for the same GPU and product shapes is applied instead of
    measured again."""
    import torch
    if stream is None:
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
    shapes = tc_shapes(circuit, ordering, grid, memory_limit)
    key = json.dumps({"gpu": torch.cuda.get_device_name(), "shapes": shapes, "strings": len(finals)})
    store = {}
    if cache is not None and Path(cache).exists():
        try:
            store = json.loads(Path(cache).read_text())
        except ValueError:
            store = {}
        if key in store:
            apply(ctx, store[key])
            return dict(store[key], cached=True)
    result = {"products": tune_products(ctx, stream, shapes) if products else {}}
    result.update(tune_batch(ctx, circuit, ordering, grid, initial, finals, memory_limit, batches))
    if cache is not None:
        store[key] = result
        Path(cache).write_text(json.dumps(store, indent=1))
    return dict(result, cached=False)


def apply(ctx: Context, tuned: dict) -> None:
    """Sets a tuning result on a context."""
    for shape, r in tuned.get("products", {}).items():
        m, n, k = (int(x) for x in shape.split(","))
        ctx.set_tc_variant(m, n, k, int(r["variant"]))
    ctx.set_option("max_batch", int(tuned.get("max_batch", 0)))
