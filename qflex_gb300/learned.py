"""Learned ordering choice: candidate contraction orderings, per-op features,
and a small perceptron, trained on the engine's own per-op timings, that
ranks candidates by predicted GB300 time.

The reference's auto-orderer ranks contraction steps with an analytic cost
(qflexcirq/ordering/order_circuit_simulation.py:87-106, ``2**op_size``);
here the cost of a plan is the sum of the predicted times of its device ops
(permutes and products), so kernel efficiency by shape is learned rather
than assumed. The supplied ordering stays the fallback, and measured time
decides: ``choose_ordering`` returns the predicted best only if it plans
within the memory budget.

Every candidate contracts the same network with full cuts, so all of them
give the same amplitudes (up to rounding).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from ._lib import OK, QflexGb300Error, load_library

N_FEATURES = 10
KINDS = 4  # permute, CUDA-core product, tensor-core product, split-k skinny product


def op_features(ops: np.ndarray) -> np.ndarray:
    """Features of device ops (rows of Context.ops()): kind one-hot,
    log2 m, n, k, flop, bytes and batch."""
    ops = np.asarray(ops, dtype=np.float64).reshape(-1, 8)
    kind = ops[:, 0].astype(int)
    onehot = np.eye(KINDS)[np.clip(kind, 0, KINDS - 1)]
    lg = lambda x: np.log2(np.maximum(x, 1.0))  # noqa: E731
    feats = np.column_stack([onehot, lg(ops[:, 1]), lg(ops[:, 2]), lg(ops[:, 3]), lg(ops[:, 4] + 1),
                             lg(ops[:, 5] + 1), lg(ops[:, 6])])
    return feats.astype(np.float32)


def analytic_ms(ops: np.ndarray, tc_tflops: float = 190.0, cuda_tflops: float = 50.0,
                hbm_gbs: float = 3000.0) -> float:
    """Roofline estimate of a plan's device time: every op takes the larger
    of its flop time and its byte time at fixed rates."""
    ops = np.asarray(ops, dtype=np.float64).reshape(-1, 8)
    rate = np.where(ops[:, 0] == 2, tc_tflops, cuda_tflops) * 1e12
    t = np.maximum(ops[:, 4] / rate, ops[:, 5] / (hbm_gbs * 1e9))
    return float(t.sum() * 1e3)


# ---------------------------------------------------------------------------
# Candidate orderings.
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class Candidate:
    text: str
    label: str


def _lines(I: int, J: int, transpose: bool):
    """Grid lines (rows, or columns when transposed) as lists of qubit
    numbers i * J + j, in the line's natural order."""
    if not transpose:
        return [[i * J + j for j in range(J)] for i in range(I)]
    return [[i * J + j for i in range(I)] for j in range(J)]


def candidate_orderings(I: int, J: int, count: Optional[int] = None, seed: int = 0) -> List[Candidate]:
    """Two-patch sweeps of an I x J grid (all qubits active): the grid is
    split between two adjacent lines (rows or columns); each patch is swept
    line by line towards the split, left-to-right or right-to-left, plain
    or snaking; optionally one bond across the split is cut with all its
    values, either before everything or just before the two boundary lines
    (so the rest of both patches is reused across the cut values). With
    ``count`` a seeded random subset is returned."""
    out: List[Candidate] = []
    for transpose in (False, True):
        lines = _lines(I, J, transpose)
        L = len(lines)
        for s in range(1, L):
            for rev in (False, True):
                for snake in (False, True):
                    def sweep(ls, rev=rev, snake=snake):
                        seq = []
                        for t, line in enumerate(ls):
                            back = rev ^ (snake and t % 2 == 1)
                            seq += list(reversed(line)) if back else list(line)
                        return seq
                    a_lines, b_lines = lines[:s], lines[s:][::-1]
                    base = f"{'cols' if transpose else 'rows'} split={s} rev={int(rev)} snake={int(snake)}"
                    plain = ("".join(f"expand A {q}\n" for q in sweep(a_lines)) +
                             "".join(f"expand B {q}\n" for q in sweep(b_lines)) + "merge A B\n")
                    out.append(Candidate(plain, base + " cut=none"))
                    for c in range(len(lines[s])):
                        q1, q2 = lines[s - 1][c], lines[s][c]
                        out.append(Candidate(f"cut () {q1} {q2}\n" + plain, base + f" cut=early@{c}"))
                        # late cut: boundary lines after the cut, in renamed patches
                        a_pre, b_pre = sweep(a_lines[:-1]), sweep(b_lines[:-1])
                        txt = "".join(f"expand A {q}\n" for q in a_pre)
                        txt += "".join(f"expand B {q}\n" for q in b_pre)
                        txt += f"cut () {q1} {q2}\n"
                        if a_pre:
                            txt += "merge A A2\n"
                        txt += "".join(f"expand A2 {q}\n" for q in sweep([a_lines[-1]]))
                        if b_pre:
                            txt += "merge B B2\n"
                        txt += "".join(f"expand B2 {q}\n" for q in sweep([b_lines[-1]]))
                        txt += "merge A2 B2\n"
                        out.append(Candidate(txt, base + f" cut=late@{c}"))
    if count is not None and count < len(out):
        rng = np.random.default_rng(seed)
        idx = sorted(rng.choice(len(out), size=count, replace=False))
        out = [out[i] for i in idx]
    return out


def _rect_sweep(rows: Sequence[int], cols: Sequence[int], col_major: bool, rev_outer: bool, rev_inner: bool,
                snake: bool) -> List[Tuple[int, int]]:
    """Cells of a rectangle swept line by line: rows (or columns with
    ``col_major``), each direction optionally reversed, snaking or not.
    Every cell after the first touches an earlier one."""
    outer, inner = (list(cols), list(rows)) if col_major else (list(rows), list(cols))
    if rev_outer:
        outer.reverse()
    seq = []
    for t, o in enumerate(outer):
        line = list(reversed(inner)) if (rev_inner ^ (snake and t % 2 == 1)) else list(inner)
        seq += [(i, o) if col_major else (o, i) for i in line]
    return seq


def sweep_candidates_7x7(cut1_values: Optional[Sequence[int]], cut2_values: Optional[Sequence[int]],
                         count: int = 500, seed: int = 0) -> List[Candidate]:
    """Seeded random row and column sweep variants of the 7x7 grid ordering
    of rqc.ordering_7x7: the same patches (A, pB, ppD, B, pD, pC, D, C), the
    same two cuts with the same values and the same merges, and in every
    patch a sweep drawn at random: each rectangle swept by rows or by
    columns from its corner on the grid's edge, snaking or not (the single
    lines grow from the cuts outwards). 1024 variants exist.
    All candidates sum the same cut slices, so they give the same
    amplitudes; they differ in product shapes (so in flop), in the
    permutations between products and in memory. Duplicates are dropped."""
    rng = np.random.default_rng(seed)

    def q(c):
        return c[0] * 7 + c[1]

    def rect(rows, cols):
        # Starts at the rectangle's first (row, column) corner, as listed:
        # rows and cols are given from the grid's outside inwards.
        return _rect_sweep(rows, cols, bool(rng.integers(2)), False, False, bool(rng.integers(2)))

    out, seen = [], set()
    tries = 0
    while len(out) < count and tries < 50 * count:
        tries += 1
        A = rect(range(0, 3), range(0, 3))
        pB = rect(range(6, 2, -1), range(0, 2))
        ppD = rect(range(6, 3, -1), range(6, 3, -1))
        # Single lines grow from the cut outwards, as in rqc.ordering_7x7:
        # the other direction holds tensors of more than 2^31 elements.
        Bc = [(r, 2) for r in range(6, 2, -1)]
        pDc = [(r, 3) for r in range(6, 3, -1)]
        pC = rect(range(0, 3), range(6, 4, -1))
        Dr = [(3, c) for c in range(6, 2, -1)]
        # Region cells: column 4 before column 3 in each row (connectivity).
        region = rect(range(0, 3), (4, 3))
        L = [f"expand A {q(c)}" for c in A] + [f"expand pB {q(c)}" for c in pB] + \
            [f"expand ppD {q(c)}" for c in ppD]
        L.append(f"cut {_vals(cut1_values)} {q((6, 2))} {q((6, 3))}")
        L.append("merge pB B")
        L += [f"expand B {q(c)}" for c in Bc]
        L.append("merge A B")
        L.append("merge ppD pD")
        L += [f"expand pD {q(c)}" for c in pDc]
        L.append(f"cut {_vals(cut2_values)} {q((2, 6))} {q((3, 6))}")
        L += [f"expand pC {q(c)}" for c in pC]
        L.append("merge pD D")
        L += [f"expand D {q(c)}" for c in Dr]
        L.append("merge B D")
        L.append("merge pC C")
        L += [f"expand C {q(c)}" for c in region]
        L.append("merge D C")
        text = "\n".join(L) + "\n"
        if text in seen:
            continue
        seen.add(text)
        out.append(Candidate(text, f"sweep#{len(out)}"))
    return out


def _vals(values: Optional[Sequence[int]]) -> str:
    return "(" + ",".join(str(v) for v in values) + ")" if values else "()"


def auto_orderer_cost(ops: np.ndarray) -> float:
    """The reference auto-orderer's cost of a plan: the sum over its
    contractions of 2^op_size, op_size = log2 of (m k) + (k n) - k... i.e.
    rank(A) - d + rank(B) - d + d for two tensors sharing a bond of 2^d
    (qflexcirq/ordering/order_circuit_simulation.py:87-106), which is m n k
    of the product. Permutations cost nothing in it."""
    ops = np.asarray(ops, dtype=np.float64).reshape(-1, 8)
    prod = ops[:, 0] != 0
    return float((ops[prod, 1] * ops[prod, 2] * ops[prod, 3]).sum())


# ---------------------------------------------------------------------------
# The perceptron (kernels in libqflex_gb300.so).
# ---------------------------------------------------------------------------

class CostModel:
    """3-layer perceptron (N_FEATURES -> hidden -> hidden -> 1, ReLU) that
    predicts log(op milliseconds). Training and inference run on the GPU
    through the library's own kernels."""

    def __init__(self, hidden: int = 64, seed: int = 0):
        import torch
        self.torch = torch
        self.lib = load_library()
        self.hidden = hidden
        self.d = N_FEATURES
        self.count = self.lib.qflex_gb300_mlp_param_count(self.d, hidden)
        g = np.random.default_rng(seed)
        p = np.zeros(self.count, dtype=np.float32)
        h, d = hidden, self.d
        p[:h * d] = g.normal(0, math.sqrt(2.0 / d), h * d)
        o = h * d + h
        p[o:o + h * h] = g.normal(0, math.sqrt(2.0 / h), h * h)
        o += h * h + h
        p[o:o + h] = g.normal(0, math.sqrt(1.0 / h), h)
        self.params = torch.from_numpy(p).cuda()
        self.mu = np.zeros(self.d, dtype=np.float32)
        self.sd = np.ones(self.d, dtype=np.float32)
        self.t_mu, self.t_sd = 0.0, 1.0

    def _ptr(self, t) -> C.c_void_p:
        return C.c_void_p(t.data_ptr())

    def _stream(self) -> C.c_void_p:
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream or None)

    def _norm(self, X: np.ndarray):
        return self.torch.from_numpy(((X - self.mu) / self.sd).astype(np.float32)).cuda()

    def loss_and_grad(self, X: np.ndarray, target: np.ndarray):
        """MSE on normalized inputs/targets and its parameter gradient
        (device tensors), as the training step computes them."""
        torch = self.torch
        x = self._norm(X)
        t = torch.from_numpy(((target - self.t_mu) / self.t_sd).astype(np.float32)).cuda()
        n = x.shape[0]
        work = torch.empty(self.lib.qflex_gb300_mlp_work_floats(n, self.hidden), dtype=torch.float32,
                           device="cuda")
        grads = torch.empty(self.count, dtype=torch.float32, device="cuda")
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        rc = self.lib.qflex_gb300_mlp_loss_grad(self._stream(), self._ptr(self.params), self._ptr(x),
                                                self._ptr(t), n, self.d, self.hidden, self._ptr(work),
                                                self._ptr(grads), self._ptr(loss))
        if rc != OK:
            raise QflexGb300Error(rc, "mlp_loss_grad failed")
        return loss, grads

    def fit(self, X: np.ndarray, ms: np.ndarray, epochs: int = 1500, lr: float = 3e-3) -> List[float]:
        """Full-batch Adam on log(ms); returns the loss history."""
        torch = self.torch
        X = np.asarray(X, dtype=np.float32)
        y = np.log(np.maximum(np.asarray(ms, dtype=np.float64), 1e-4))
        self.mu = X.mean(axis=0)
        self.sd = np.maximum(X.std(axis=0), 1e-3)
        self.t_mu, self.t_sd = float(y.mean()), float(max(y.std(), 1e-3))
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        hist = []
        for step in range(1, epochs + 1):
            loss, grads = self.loss_and_grad(X, y)
            rc = self.lib.qflex_gb300_mlp_adam(self._stream(), self._ptr(self.params), self._ptr(grads),
                                               self._ptr(m), self._ptr(v), self.count, step, C.c_float(lr))
            if rc != OK:
                raise QflexGb300Error(rc, "mlp_adam failed")
            if step % 50 == 0 or step == 1:
                hist.append(float(loss.item()))
        return hist

    def predict_log_ms(self, X: np.ndarray) -> np.ndarray:
        torch = self.torch
        X = np.asarray(X, dtype=np.float32)
        if len(X) == 0:
            return np.zeros(0)
        x = self._norm(X)
        n = x.shape[0]
        work = torch.empty(self.lib.qflex_gb300_mlp_work_floats(n, self.hidden), dtype=torch.float32,
                           device="cuda")
        y = torch.empty(n, dtype=torch.float32, device="cuda")
        rc = self.lib.qflex_gb300_mlp_forward(self._stream(), self._ptr(self.params), self._ptr(x), n, self.d,
                                              self.hidden, self._ptr(work), self._ptr(y))
        if rc != OK:
            raise QflexGb300Error(rc, "mlp_forward failed")
        return y.cpu().numpy().astype(np.float64) * self.t_sd + self.t_mu

    def predict_plan_ms(self, ops: np.ndarray) -> float:
        return float(np.exp(self.predict_log_ms(op_features(ops))).sum())

    def state(self) -> Dict[str, np.ndarray]:
        return {"params": self.params.cpu().numpy(), "mu": self.mu, "sd": self.sd,
                "t": np.array([self.t_mu, self.t_sd]), "hidden": np.array([self.hidden])}


# ---------------------------------------------------------------------------
# Planning, profiling and choice.
# ---------------------------------------------------------------------------

def plan_ops(circuit: str, ordering: str, grid: str, precision: int, batch: int = 1,
             memory_limit: float = float(1 << 40)) -> Tuple[np.ndarray, float]:
    """Device ops of an ordering's plan (planning only, no GPU) and its HBM
    arena bytes per output string."""
    from ._lib import Context
    ctx = Context(-1, precision)
    ctx.evaluate(circuit, ordering, grid, "", "", memory_limit)
    ops = ctx.ops()
    ops[:, 6] = batch
    return ops, ctx.stats()["arena_bytes"]


def profile(ctx, circuit: str, ordering: str, grid: str, finals: Sequence[str], repeats: int = 2):
    """Runs an ordering with per-op timing; returns (ops with measured ms,
    device ms of the last run, amplitudes)."""
    ctx.set_profiling(True)
    try:
        for _ in range(repeats):
            amps = ctx.evaluate_many(circuit, ordering, grid, "", list(finals), float(1 << 40))
        return ctx.ops(), ctx.stats()["device_ms"], [a for _, a in amps]
    finally:
        ctx.set_profiling(False)


def choose_ordering(model: CostModel, circuit: str, grid: str, candidates: Sequence[Candidate],
                    supplied: str, precision: int, batch: int, arena_budget: float):
    """The candidate with the smallest predicted time that fits the budget,
    or the supplied ordering when nothing beats its predicted time."""
    best = (model.predict_plan_ms(plan_ops(circuit, supplied, grid, precision, batch)[0]), supplied, "supplied")
    for cand in candidates:
        try:
            ops, arena = plan_ops(circuit, cand.text, grid, precision, batch)
        except QflexGb300Error:
            continue
        if arena * batch > arena_budget:
            continue
        t = model.predict_plan_ms(ops)
        if t < best[0]:
            best = (t, cand.text, cand.label)
    return best


# ---------------------------------------------------------------------------
# The search: candidates ranked by the learned model and by the baselines,
# the picks measured.
# ---------------------------------------------------------------------------

def _spearman(a, b) -> float:
    ra = np.argsort(np.argsort(a))
    rb = np.argsort(np.argsort(b))
    return float(np.corrcoef(ra, rb)[0, 1])


def run_search(circuit: str, grid: str, supplied: str, candidates: Sequence[Candidate], finals: Sequence[str],
               precision: int, n_train: int = 12, n_sample: int = 20, memory_limit: float = 180e9,
               seed: int = 0, repeats: int = 2, log=print) -> dict:
    """Plans every candidate (planning only; those beyond the memory limit
    or the 2^31-element tensor limit drop out), profiles `n_train` of them
    op by op on the GPU, fits the cost model on those timings, and ranks the
    rest by three costs: the model's predicted time, the reference
    auto-orderer's sum of m n k (auto_orderer_cost) and the roofline
    estimate (analytic_ms). Each ranking's pick is measured, with the
    supplied ordering and `n_sample` held-out candidates for the rank
    correlations. Amplitudes of every measured ordering are compared with
    the supplied ordering's. Returns a report (dict)."""
    from ._lib import Context
    batch = len(finals)
    rng = np.random.default_rng(seed)
    plans = []
    for cand in candidates:
        try:
            ops, arena = plan_ops(circuit, cand.text, grid, precision, batch)
        except QflexGb300Error:
            continue
        if arena * batch > memory_limit:
            continue
        plans.append((cand, ops))
    log(f"{len(plans)} of {len(candidates)} candidates plan within the limits")
    order = rng.permutation(len(plans))
    train = [plans[i] for i in order[:n_train]]
    held = [plans[i] for i in order[n_train:]]
    ctx = Context(0, precision)
    feats, times = [], []
    ref_amps = None
    for cand, _ in train:
        ops, _, amps = profile(ctx, circuit, cand.text, grid, finals, repeats=repeats)
        feats.append(op_features(ops))
        times.append(ops[:, 7])
    model = CostModel(hidden=64, seed=seed)
    model.fit(np.vstack(feats), np.concatenate(times), epochs=1500)
    pred = np.array([model.predict_plan_ms(ops) for _, ops in held])
    auto = np.array([auto_orderer_cost(ops) for _, ops in held])
    roof = np.array([analytic_ms(ops) for _, ops in held])

    def measure(text):
        ctx.evaluate_many(circuit, text, grid, "", list(finals), memory_limit)
        best, out = float("inf"), None
        for _ in range(repeats):
            out = ctx.evaluate_many(circuit, text, grid, "", list(finals), memory_limit)
            best = min(best, ctx.stats()["device_ms"])
        return best, [a for _, a in out]

    t_sup, ref_amps = measure(supplied)

    def rel(amps):
        g = np.asarray(amps)
        w = np.asarray(ref_amps)
        return float(np.max(np.abs(g - w)) / np.sqrt(np.mean(np.abs(w) ** 2)))

    picks = {}
    for name, score in (("model", pred), ("auto_orderer", auto), ("roofline", roof)):
        i = int(np.argmin(score))  # ties go to the first candidate in list order
        t, amps = measure(held[i][0].text)
        picks[name] = {"label": held[i][0].label, "index": i, "measured_ms": t, "amplitude_err_vs_supplied": rel(amps),
                       "gemm_flop": float(held[i][1][:, 4].sum()),
                       "permute_bytes": float(held[i][1][held[i][1][:, 0] == 0, 5].sum())}
        log(f"{name} pick {held[i][0].label}: {t:.1f} ms")
    sample = rng.choice(len(held), size=min(n_sample, len(held)), replace=False)
    measured = []
    for i in sample:
        t, amps = measure(held[i][0].text)
        measured.append(t)
        assert rel(amps) < 1e-4, held[i][0].label
    measured = np.array(measured)
    # Regret of each ranking on random subsets of the measured sample: the
    # measured time of the subset's pick over the subset's best.
    regret = {}
    subsets = [rng.choice(len(sample), size=min(8, len(sample)), replace=False) for _ in range(2000)]
    for name, score in (("model", pred[sample]), ("auto_orderer", auto[sample]), ("roofline", roof[sample])):
        r = [measured[sub[int(np.argmin(score[sub]))]] / measured[sub].min() - 1.0 for sub in subsets]
        regret[name] = float(np.mean(r))
    disagree = [sub for sub in subsets if int(np.argmin(pred[sample][sub])) != int(np.argmin(auto[sample][sub]))]
    faster = sum(measured[sub[int(np.argmin(pred[sample][sub]))]] < measured[sub[int(np.argmin(auto[sample][sub]))]]
                 for sub in disagree)
    return {
        "candidates": len(candidates), "planned": len(plans), "trained_on": len(train), "held_out": len(held),
        "strings": batch, "supplied_ms": t_sup, "picks": picks,
        "sample": {"size": int(len(sample)), "best_ms": float(measured.min()), "worst_ms": float(measured.max()),
                   "spearman": {"model": _spearman(pred[sample], measured),
                                "auto_orderer": _spearman(auto[sample], measured),
                                "roofline": _spearman(roof[sample], measured)},
                   "mean_regret_8_of_sample": regret,
                   "subsets_where_model_and_auto_orderer_disagree": len(disagree),
                   "of_those_model_pick_faster": int(faster)},
        "model_text": held[picks["model"]["index"]][0].text,
    }


def main(argv=None) -> None:
    """python -m qflex_gb300.learned --depth 40 [--slices 1] [--count 500] --out report.json"""
    import argparse
    import json

    from . import rqc
    from ._lib import PRECISIONS
    ap = argparse.ArgumentParser()
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--values", type=int, default=1, help="values per cut (slices = values^2)")
    ap.add_argument("--count", type=int, default=500)
    ap.add_argument("--strings", type=int, default=1)
    ap.add_argument("--train", type=int, default=12)
    ap.add_argument("--sample", type=int, default=20)
    ap.add_argument("--precision", default="fp16x3")
    ap.add_argument("--memory", type=float, default=180e9)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", required=True)
    args = ap.parse_args(argv)
    circuit = rqc.random_circuit(7, 7, args.depth, seed=0)
    grid = rqc.grid_text(7, 7)
    vals = tuple(range(args.values))
    supplied = rqc.ordering_7x7(vals, vals)
    finals = rqc.random_bitstrings(49, args.strings, 2)
    cands = sweep_candidates_7x7(vals, vals, count=args.count, seed=args.seed)
    rep = run_search(circuit, grid, supplied, cands, finals, PRECISIONS[args.precision], n_train=args.train,
                     n_sample=args.sample, memory_limit=args.memory, seed=args.seed)
    rep.update({"workload": f"7x7 grid, depth (1+{args.depth}+1), 2 cuts x {args.values} values",
                "precision": args.precision})
    with open(args.out, "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({k: v for k, v in rep.items() if k != "model_text"}, indent=1))


if __name__ == "__main__":
    main()
