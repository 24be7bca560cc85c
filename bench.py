"""Benchmark: output amplitudes per second of the 7x7 grid random circuit of
depth (1+32+1) (49 qubits, CZ bond dimension 16), contracted with the
two-cut 7x7 ordering (4 values per cut -> 16 slices summed per amplitude).

One step = one call of the engine's public C-ABI entry
qflex_gb300_evaluate_many for B random 49-bit output strings (host texts
and strings in, complex128 amplitudes out). Every step uses new strings.

  value  amplitudes/s from the engine's device time (flatten + program +
         FP64 sums, CUDA events on the launching stream; inputs already in
         HBM once the strings' bits are uploaded)
  e2e    amplitudes/s of the whole C-ABI call (host->device bits, device->
         host amplitudes, host planning cached) timed with CUDA events
         around the K steps.

Launch: python bench.py [--gpus N --steps K --warmup W --batch B]
        python bench.py --impl reference ...   (reference's CPU path)
Under torchrun each rank runs independent replicas on its own strings
(the path shards over output strings; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "amplitudes/s on 7x7 1+32+1 RQC; split-precision vs FP32, rel err≤1e-5 vs FP64"
UNIT = "amplitudes/s"
WORKLOAD = "c3"
FP32_PEAK_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12  # TFLOP/s, FP32 CUDA-core FMA
# DRAM bytes (read + write) per product of the dominant shape, from the ncu
# captures summarised in profiles/ (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch divided by its products): 3xTF32 at 1
# product per launch, 3xFP16 at 4 (the step's pass size), 5.728 GB / 4.
TRAFFIC = {("tf32x3", 4096, 4096, 4096): 2.322e9, ("fp16x3", 4096, 4096, 4096): 1.432e9}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--batch", type=int, default=8, help="output strings per step")
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--precision", default="fp16x3", choices=["fp16x3", "tf32x3", "bf16x3", "fp32"])
    p.add_argument("--ordering", default="learned", choices=["learned", "supplied"],
                   help="the cost model's ordering of the workload (qflex_gb300/orderings/c3_learned.txt) or the "
                        "supplied one; both sum the same cut slices")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true",
                   help="skip the tensor-core kernel / strings-per-pass autotuning before warm-up")
    p.add_argument("--cpu-sample", type=int, default=0, metavar="SLICES",
                   help="only time the CPU oracle on SLICES cut slices and print that as JSON")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


REF_BIN = ROOT / "oracle" / "_ref" / "qflex_ref"


def _rqc():
    """qflex_gb300/rqc.py loaded on its own (it needs numpy only), so that the
    CPU baseline legs build the workload without importing the product
    package or loading its library."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("qflex_rqc_standalone", ROOT / "qflex_gb300" / "rqc.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def reference_binary():
    """The unmodified reference build (oracle/Makefile), if this machine has
    one that runs."""
    return REF_BIN if REF_BIN.exists() and os.access(REF_BIN, os.X_OK) else None


def cpu_sample(slices: int = 4, threads: int = 0, reps: int = 1):
    """The reference's CPU path on `slices` of the benchmark workload's 16 cut
    slices x one output string, `reps` times: the unmodified reference
    (oracle/_ref/qflex_ref, OpenBLAS + OpenMP) when it is built here, else
    the oracle port (numpy over OpenBLAS). `threads` (0: all host cores)
    sets the OpenBLAS / OpenMP thread count. Each run is scaled to the
    16-slice amplitude by the planned flop ratio (constants committed with
    the workload, pinned by a test against the reference's own product log).
    Returns (seconds per run, amplitudes/s per run, description, threads, kind)."""
    rqc = _rqc()
    circuit, _, grid, initial, finals = rqc.workload(WORKLOAD)
    sample = rqc.ordering_7x7((0,), tuple(range(slices)))
    flop_sample, flop_full = rqc.C3_GEMM_FLOP[slices], rqc.C3_GEMM_FLOP[16]
    threads = threads or os.cpu_count()
    ref = reference_binary()
    secs = []
    if ref is not None:
        import tempfile
        with tempfile.TemporaryDirectory() as d:
            paths = []
            for name, text in (("circuit", circuit), ("ordering", sample), ("grid", grid)):
                path = Path(d) / name
                path.write_text(text)
                paths.append(str(path))
            env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS=str(threads))
            out = subprocess.run([str(ref), "threads", str(threads), "time", str(reps), "eval", *paths, initial,
                                  finals[0], "64GB"], env=env, capture_output=True, text=True, check=True,
                                 timeout=3600)
            secs = [float(ln.split()[1]) for ln in out.stdout.splitlines() if ln.startswith("SECONDS ")]
        kind, what = "reference", "the unmodified reference (oracle/_ref/qflex_ref, OpenBLAS + OpenMP)"
    else:
        if threads != os.cpu_count():
            raise RuntimeError("the oracle port takes its thread count from the environment of a new process")
        import numpy as np

        from oracle import qflex_oracle as qo
        inp = qo.Input(qo.Circuit.loads(circuit), qo.load_ordering(sample), qo.Grid.loads(grid), initial,
                       finals[0])
        for _ in range(reps):
            inp.initial_state, inp.final_state = initial, finals[0]
            t0 = time.perf_counter()
            qo.evaluate_circuit(inp, np.complex64, float(1 << 40))
            secs.append(time.perf_counter() - t0)
        kind, what = "port", "the oracle port (the reference's algorithm in numpy over OpenBLAS)"
    values = [(flop_sample / flop_full) / dt for dt in secs]
    desc = (f"{what} on {slices} of the 16 cut slices x 1 string of the 7x7 (1+32+1) workload "
            f"({flop_sample:.4e} flop, {statistics.mean(secs):.2f} s per run, {threads} threads), scaled to the "
            f"16-slice amplitude ({flop_full:.4e} flop) by the flop ratio")
    return secs, values, desc, threads, kind


def run_reference(args, rank):
    """--impl reference: the reference's CPU implementation of the path on
    this machine's host cores, rank 0 only. Warm-up steps run one cut slice,
    timed steps four of the 16 (one process, EvaluateCircuit timed alone)."""
    if rank != 0:
        return
    if args.warmup:
        cpu_sample(slices=1, reps=args.warmup)
    t0 = time.perf_counter()
    secs, vals, desc, cores, kind = cpu_sample(slices=4, reps=args.steps)
    wall = time.perf_counter() - t0
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(secs),
            "wall_s": wall, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic", "config": config(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config(args):
    return {"workload": "7x7 grid RQC depth (1+32+1), 49 qubits, CZ bond 16, two cuts x 4 values "
                        "(16 slices), random 49-bit output strings",
            "strings_per_step": args.batch, "precision": args.precision, "ordering": args.ordering,
            "parallelism": f"replicas{args.gpus}",
            "l2": "inputs larger than L2 (1.1 GB HBM arena per output string)"}


def dominant_product(ctx, circuit, ordering, grid, initial, strings):
    """The product shape with the most device time in one profiled pass of
    the benchmark step (CUDA events around every launch on the context's
    stream): (m, n, k, launches, batch, mean ms per launch incl. the
    B-operand split, share of the pass)."""
    import collections
    ctx.set_profiling(True)
    try:
        ctx.evaluate_many(circuit, ordering, grid, initial, strings, 1 << 40)
        ops = ctx.ops()
    finally:
        ctx.set_profiling(False)
    agg = collections.defaultdict(lambda: [0, 0.0, 1])
    total = 0.0
    for r in ops:
        total += r[7]
        if int(r[0]) in (1, 2):
            a = agg[(int(r[1]), int(r[2]), int(r[3]))]
            a[0] += 1
            a[1] += r[7]
            a[2] = int(r[6])
    (m, n, k), (cnt, ms, batch) = max(agg.items(), key=lambda kv: kv[1][1])
    return m, n, k, cnt, batch, ms / cnt, ms / total


def dominant_kernel_time(ctx, torch, m, n, k, reps=5):
    """CUDA-event time of one product of shape (m, n, k) through the public
    multiply entry (both operands split, B transposed) on the context's
    stream."""
    A = torch.randn((m, k), dtype=torch.complex64, device="cuda")
    B = torch.randn((k, n), dtype=torch.complex64, device="cuda")
    C = torch.empty((m, n), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        ctx.multiply(A.data_ptr(), B.data_ptr(), C.data_ptr(), m, n, k)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def fp64_reference():
    """FP64-oracle amplitudes of the workload's first output strings: the
    GPU complex128 contraction's (tests/golden/c3_fp64_gpu.json, 256
    strings) when committed, else the CPU complex128 oracle's
    (tests/golden/c3_fp64.json)."""
    gpu = ROOT / "tests" / "golden" / "c3_fp64_gpu.json"
    cpu = ROOT / "tests" / "golden" / "c3_fp64.json"
    for path, what in ((gpu, "FP64 GPU oracle (complex128 contraction, float-float products; "
                             "tests/golden/c3_fp64_gpu.json)"),
                       (cpu, "FP64 CPU oracle (numpy complex128, double gate constants; tests/golden/c3_fp64.json)")):
        if path.exists():
            ref = json.loads(path.read_text())
            return ref, what
    return None, None


def accuracy_vs_fp64(ctx, circuit, ordering, grid, batch):
    """Per-amplitude relative error |a - a64| / |a64| of this context's
    amplitudes against the FP64 oracle, over every string of the oracle
    fixture, evaluated `batch` strings per call after one untimed call. The
    calls' device time gives the path's throughput over those steps."""
    import math
    ref, what = fp64_reference()
    if ref is None:
        return None
    finals = [r["final"] for r in ref["amplitudes"]]
    want = [complex(*r["amplitude"]) for r in ref["amplitudes"]]
    ctx.evaluate_many(circuit, ordering, grid, ref["initial"], finals[:batch], 1 << 40)
    got, device_ms = [], 0.0
    for i in range(0, len(finals), batch):
        got += [a for _, a in ctx.evaluate_many(circuit, ordering, grid, ref["initial"], finals[i:i + batch],
                                                1 << 40)]
        device_ms += ctx.stats()["device_ms"]
    errs = sorted(abs(a - b) / abs(b) for a, b in zip(got, want))
    n = len(errs)
    rms = math.sqrt(sum(abs(b) ** 2 for b in want) / n)
    return {"max_rel_err_vs_fp64": errs[-1], "median_rel_err": errs[n // 2],
            "p99_rel_err": errs[min(n - 1, int(math.ceil(0.99 * n)) - 1)],
            "over_1e-5": sum(e > 1e-5 for e in errs),
            "max_err_over_rms": max(abs(a - b) for a, b in zip(got, want)) / rms,
            "mean_ratio_minus_1": sum((a / b).real for a, b in zip(got, want)) / n - 1.0,
            "amplitudes": n, "reference": what,
            "throughput": {"value": n / (device_ms / 1e3), "unit": UNIT, "steps": (n + batch - 1) // batch,
                           "strings_per_step": batch}}


def timed_steps(ctx, torch, stream, circuit, ordering, grid, initial, strings, first, steps):
    """Runs `steps` evaluate_many calls; returns (device ms, event ms)."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    device_ms = 0.0
    torch.cuda.synchronize()
    e0.record(stream)
    for s in range(steps):
        ctx.evaluate_many(circuit, ordering, grid, initial, strings(first + s), 1 << 40)
        device_ms += ctx.stats()["device_ms"]
    e1.record(stream)
    torch.cuda.synchronize()
    return device_ms, e0.elapsed_time(e1)


def shared_region(ctx, torch, stream, circuit, grid, initial, finals, strings=2, steps=2):
    """Amplitudes/s when output strings share all bits but a 6-qubit region
    of patch C: the region's qubits are terminal cuts, so one contraction
    gives its 64 amplitudes (the reference's batching of amplitudes,
    src/contraction_utils.cpp:300-314). Same circuit, cuts and precision
    as the main line; `strings` 43-bit prefixes per step."""
    from qflex_gb300 import rqc
    ordering = rqc.ordering_7x7((0, 1, 2, 3), (0, 1, 2, 3), terminal_region=True)
    region = [i * 7 + j for i, j in [(0, 4), (1, 4), (2, 4), (0, 3), (1, 3), (2, 3)]]

    def prefixes(step):
        out = []
        for i in range(strings):
            f = list(finals[(step * strings + i) % len(finals)])
            for q in region:
                f[q] = "x"
            out.append("".join(f))
        return out

    out = ctx.evaluate_many(circuit, ordering, grid, initial, prefixes(0), 1 << 40)
    per_step = len(out)
    ms, _ = timed_steps(ctx, torch, stream, circuit, ordering, grid, initial, prefixes, 1, steps)
    st = ctx.stats()
    return {"value": per_step * steps / (ms / 1e3), "unit": UNIT, "amplitudes_per_contraction": 64,
            "strings_per_step": strings, "steps": steps, "ops": st["n_ops"],
            "gemm_flop_per_contraction": st["gemm_flop"],
            "note": "not the headline: strings share 43 of 49 bits"}


def fsim_workload(torch, stream, local, precision, batch=8):
    """The fSim workload: 6 x 9 grid with one disabled site (53 qubits),
    8 cycles of fSim(pi/2, pi/6 + jitter) on four alternating coupler
    patterns (bond 16), three cuts x 2 values (8 slices), 64 string prefixes
    whose 6-qubit last column is open: 4096 amplitudes, 64 per contraction.
    Device-timed over all prefixes, `batch` per call, after one untimed call;
    the first prefix's 64 amplitudes against the complex128 contraction."""
    from qflex_gb300 import FP64_FF, Context, rqc
    from qflex_gb300._lib import PRECISIONS
    circuit, ordering, grid, initial, finals = rqc.workload_c4()
    ctx = Context(local, PRECISIONS[precision])
    ctx.set_stream(stream.cuda_stream)
    ctx.evaluate_many(circuit, ordering, grid, initial, finals[:batch], 1 << 40)
    amps, ms, first = 0, 0.0, None
    for i in range(0, len(finals), batch):
        out = ctx.evaluate_many(circuit, ordering, grid, initial, finals[i:i + batch], 1 << 40)
        ms += ctx.stats()["device_ms"]
        amps += len(out)
        if first is None:
            first = [a for _, a in out[:64]]
    st = ctx.stats()
    ctx.close()
    wide = Context(local, FP64_FF)
    wide.set_stream(stream.cuda_stream)
    want = [a for _, a in wide.evaluate_many(circuit, ordering, grid, initial, finals[:1], 1 << 40)]
    wide.close()
    errs = [abs(a - b) / abs(b) for a, b in zip(first, want)]
    rms = (sum(abs(b) ** 2 for b in want) / len(want)) ** 0.5
    return {"value": amps / (ms / 1e3), "unit": UNIT, "amplitudes": amps, "amplitudes_per_contraction": 64,
            "strings_per_step": batch, "precision": precision, "gemm_flop_per_contraction": st["gemm_flop"],
            "slices": st["n_leaves"] // 64,
            "workload": "6x9 grid, one disabled site (53 qubits), 8 fSim cycles (bond 16), 3 cuts x 2 values, "
                        "6-qubit open region, 64 prefixes x 64 amplitudes",
            "accuracy": {"max_rel_err_vs_fp64": max(errs), "max_err_over_rms": max(abs(a - b) for a, b in
                                                                                   zip(first, want)) / rms,
                         "amplitudes": len(errs), "reference": "complex128 contraction of the same network"},
            "note": "not the headline metric"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.cpu_sample:
        secs, vals, desc, cores, kind = cpu_sample(slices=args.cpu_sample)
        print(json.dumps({"seconds": secs[0], "value": vals[0], "sample": desc, "kind": kind}))
        return
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    import torch.distributed as dist
    from qflex_gb300 import Context, rqc
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(local)
    ctx.set_precision(args.precision)
    ctx.set_stream(stream.cuda_stream)
    circuit, ordering, grid, initial, finals = rqc.workload(WORKLOAD)
    if args.ordering == "learned":
        ordering = rqc.ordering_7x7_learned()
    B = args.batch

    def strings(step):
        # rank r takes its own strings; the 1024-string list is reused
        # cyclically beyond 1024 / (world * B) steps.
        base = ((step * world) + rank) * B
        return [finals[(base + i) % len(finals)] for i in range(B)]

    tuned = None
    if args.precision != "fp32" and not args.no_autotune:
        # Untimed: kernel variant per product shape (3xTF32 only), strings
        # per device pass (on strings from the end of the list, not used by
        # the steps).
        from qflex_gb300 import autotune
        tuned = autotune.tune(ctx, circuit, ordering, grid, initial, finals[-B:],
                              batches=[b for b in (1, 2, 4, 8, 16) if b <= B], stream=stream,
                              products=args.precision == "tf32x3")
    for w in range(args.warmup):
        ctx.evaluate_many(circuit, ordering, grid, initial, strings(w), 1 << 40)
    with ClockSampler(local) as clocks:
        barrier()
        device_ms, e2e_ms = timed_steps(ctx, torch, stream, circuit, ordering, grid, initial, strings,
                                        args.warmup, args.steps)
        barrier()
    st = ctx.stats()
    if world > 1:
        t = torch.tensor([device_ms, e2e_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        device_ms, e2e_ms = t.tolist()
    amps = args.steps * B * world
    value = amps / (device_ms / 1000.0)
    e2e = amps / (e2e_ms / 1000.0)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": e2e_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": dict(config(args), autotune=None if tuned is None else {
                "variants": {sh: r["variant"] for sh, r in tuned["products"].items()},
                "max_batch": tuned["max_batch"], "ms_per_string": tuned.get("ms_per_string")}),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * 49 * B,
                    "d2h_bytes_per_step": 16 * B},
            "gpu_launches": int(st["launches"]) * args.steps,
            "algorithmic_tflops": st["gemm_flop"] * amps / (device_ms / 1e3) / 1e12,
            "clocks": clocks.summary(),
            "plan": {"gemm_flop_per_amplitude": st["gemm_flop"],
                     "permute_bytes_per_amplitude": st["permute_bytes"],
                     "arena_bytes_per_string": st["arena_bytes"], "ops": st["n_ops"],
                     "slices": st["n_leaves"]}}

    if rank == 0 and world == 1:
        # Accuracy of this path against the FP64 oracle, then the plain FP32
        # CUDA-core path and the other split precisions on the same workload.
        line["accuracy"] = accuracy_vs_fp64(ctx, circuit, ordering, grid, B)
        m, n, k, launches, pbatch, op_ms, share = dominant_product(ctx, circuit, ordering, grid, initial,
                                                                   strings(0))
        achieved = 8.0 * m * n * k * pbatch / (op_ms / 1e3) / 1e12
        single = 8.0 * m * n * k / (dominant_kernel_time(ctx, torch, m, n, k) / 1e3) / 1e12
        pk = peaks()
        if args.precision == "fp32":
            line["roofline"] = {
                "bound": "fp32", "kernel": f"cgemm_fp32 ({m},{n},{k})", "achieved": achieved,
                "peak": FP32_PEAK_NOMINAL, "unit": "TFLOP/s", "frac": achieved / FP32_PEAK_NOMINAL,
                "peak_source": "nominal FP32 CUDA-core FMA rate (152 SMs x 128 lanes x 2 x 2.07 GHz); "
                               "the measured peaks hold no FP32 CUDA-core figure",
                "traffic": None, "timing": f"CUDA events around each of the {launches} launches of this shape "
                                           f"(batch {pbatch}) in one profiled pass of the step; "
                                           f"{100 * share:.0f}% of the pass"}
        else:
            # Algorithmic rate (8 m n k per complex product, whatever the
            # method) against the measured bf16 dense peak; the kernel is
            # timed inside a seconds-long step, so the sustained figure is
            # the denominator. The split methods issue more MMA work than
            # that: 4 real products x 3 terms (3xTF32, 3xFP16) or x 6 terms
            # (BF16x3) per complex product, at the bf16 rate (FP16, BF16)
            # or half of it (TF32); mma_frac is that issued rate against
            # the same peak, and caps.tensor_method is the algorithmic
            # ceiling the method leaves.
            sustained = "bf16_tflops_sustained" in pk
            peak = pk.get("bf16_tflops_sustained", 1700.0)
            src = ("measured bf16 dense, sustained (MEASURED_PEAKS.json bf16_tflops_sustained)" if sustained
                   else "fallback 1.7 PFLOP/s bf16 sustained")
            fp16 = args.precision in ("fp16x3", "bf16x3")
            mma_peak = peak if fp16 else peak / 2
            terms = 6.0 if args.precision == "bf16x3" else 3.0
            mma_rate = terms * achieved
            ai = 8.0 * m * n * k / (8.0 * (m * k + k * n + m * n))  # flop per byte, operands and result once
            line["roofline"] = {
                "bound": "tensor", "kernel": f"cgemm_{args.precision} ({m},{n},{k}) x{pbatch} incl. its operand splits",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": src,
                "mma_achieved": mma_rate, "mma_peak": mma_peak, "mma_frac": mma_rate / mma_peak,
                "mma_unit": "TFLOP/s (16-bit MMA)" if fp16 else "TFLOP/s (TF32 MMA)",
                "caps": {"tensor_method": mma_peak / terms, "hbm": ai * pk.get("hbm_gbs", 6800.0) / 1e3,
                         "unit": "TFLOP/s algorithmic"},
                "traffic": (TRAFFIC[(args.precision, m, n, k)] * pbatch
                            if (args.precision, m, n, k) in TRAFFIC else None),
                "traffic_source": "ncu dram__bytes_read+write per product of this shape (profiles/tc_*_4096.md), "
                                  "times the products per launch",
                "algorithmic_bytes": 8.0 * (m * k + k * n + m * n) * pbatch,
                "timing": f"CUDA events around each of the {launches} launches of this shape (batch {pbatch}) "
                          f"in one profiled pass of the step on the context stream; {100 * share:.0f}% of the pass",
                "single_product_tflops": single}
            # The other paths on the same workload: each runs every string of
            # the FP64 oracle fixture, B strings per step (after one untimed
            # step); the device time of those steps is its throughput.
            for other in [q for q in ("fp32", "tf32x3", "bf16x3", "fp16x3") if q != args.precision]:
                fp = Context(local)
                fp.set_precision(other)
                fp.set_stream(stream.cuda_stream)
                acc = accuracy_vs_fp64(fp, circuit, ordering, grid, B)
                o_value = acc["throughput"]["value"]
                line[f"{other}_path"] = {"value": o_value, "unit": UNIT, "steps": acc["throughput"]["steps"],
                                         "speedup_of_this_path": value / o_value, "accuracy": acc}
                fp.close()
            line["shared_region"] = shared_region(ctx, torch, stream, circuit, grid, initial, finals)
            line["fsim_workload"] = fsim_workload(torch, stream, local, args.precision)
        if not args.no_cpu_baseline:
            secs, vals, desc, cores, kind = cpu_sample(slices=4)
            line["cpu_baseline"] = {"value": vals[0], "unit": UNIT, "cores": cores, "kind": kind,
                                    "sample": desc}
            if kind == "reference":
                # Threading helps the large products and hurts the small ones.
                secs, vals, desc, _, _ = cpu_sample(slices=1, threads=1)
                line["cpu_baseline"]["single_thread"] = {"value": vals[0], "unit": UNIT, "cores": 1,
                                                         "sample": desc}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
