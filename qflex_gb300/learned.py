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
