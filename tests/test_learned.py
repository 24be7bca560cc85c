"""Learned ordering choice: candidate generation (CPU), the perceptron's
kernels against the CPU oracle (gradient check), and what the trained model
gains over the supplied ordering and the analytic cost on a real circuit."""
import numpy as np
import pytest

from oracle import mlp_oracle
from qflex_gb300 import Context, FP32, TF32X3, rqc
from qflex_gb300.learned import (N_FEATURES, CostModel, analytic_ms, candidate_orderings, choose_ordering,
                                 op_features, plan_ops, profile)
from tests.conftest import rel_err


def test_candidates_are_valid_orderings(built_lib):
    c = rqc.random_circuit(4, 5, 16, seed=1)
    g = rqc.grid_text(4, 5)
    cands = candidate_orderings(4, 5)
    assert len(cands) > 100
    labels = {x.label for x in cands}
    assert len(labels) == len(cands)
    plan = Context(-1, TF32X3)
    for cand in cands:
        out = plan.evaluate(c, cand.text, g, "", "", 1 << 40)
        assert len(out) == 1  # one amplitude, full cuts only
    sub = candidate_orderings(4, 5, count=20, seed=3)
    assert len(sub) == 20 and all(s in cands for s in sub)


def test_op_features_shape(built_lib):
    c, o, g, _, _ = rqc.workload("c1")
    ops, arena = plan_ops(c, o, g, TF32X3)
    X = op_features(ops)
    assert X.shape == (len(ops), N_FEATURES)
    assert np.isfinite(X).all()
    assert analytic_ms(ops) > 0 and arena > 0


@pytest.mark.gpu
def test_mlp_gradient_matches_cpu_oracle(built_lib):
    model = CostModel(hidden=64, seed=1)
    g = np.random.default_rng(2)
    X = g.normal(size=(300, N_FEATURES)).astype(np.float32)
    t = g.normal(size=300)
    model.mu = np.zeros(N_FEATURES, np.float32)
    model.sd = np.ones(N_FEATURES, np.float32)
    model.t_mu, model.t_sd = 0.0, 1.0
    loss, grads = model.loss_and_grad(X, t)
    p = model.params.cpu().numpy()
    want_loss, want_g = mlp_oracle.loss_grad(p, X, t, N_FEATURES, 64)
    got = grads.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - want_loss) <= 1e-4 * abs(want_loss)
    assert np.max(np.abs(got - want_g)) <= 1e-4 * max(np.max(np.abs(want_g)), 1e-6)
    pred = model.predict_log_ms(X)
    want_y, _, _ = mlp_oracle.forward(p, X, N_FEATURES, 64)
    assert np.max(np.abs(pred - want_y)) <= 1e-4 * max(np.max(np.abs(want_y)), 1.0)


@pytest.mark.gpu
def test_mlp_training_reduces_loss(built_lib):
    g = np.random.default_rng(5)
    X = g.normal(size=(500, N_FEATURES)).astype(np.float32)
    ms = np.exp(0.7 * X[:, 4] - 0.3 * X[:, 6] + 0.1 * X[:, 4] * X[:, 5])
    model = CostModel(hidden=64, seed=3)
    hist = model.fit(X, ms, epochs=600, lr=3e-3)
    assert hist[-1] < 0.05 * hist[0]


def _spearman(a, b):
    ra = np.argsort(np.argsort(a))
    rb = np.argsort(np.argsort(b))
    return float(np.corrcoef(ra, rb)[0, 1])


@pytest.mark.gpu
def test_learned_choice_on_6x6(built_lib, capsys):
    """6x6 grid, depth (1+24+1) (CZ bond 8), 8 output strings. The model is
    trained on the per-op timings of 10 profiled candidates, then ranks 40
    others; every candidate is measured. Amplitudes agree across all
    orderings; the model ranks the held-out candidates better than the
    roofline estimate and its choice is not slower than the supplied
    ordering."""
    circuit = rqc.random_circuit(6, 6, 24, seed=11)
    grid = rqc.grid_text(6, 6)
    supplied = rqc.ordering_6x6()  # full cut on the central bond
    finals = rqc.random_bitstrings(36, 8, 12)
    ctx = Context(0, TF32X3)
    cands = candidate_orderings(6, 6, count=50, seed=7)
    train, held = cands[:10], cands[10:]
    feats, times = [], []
    ref_amps = None
    for cand in train:
        ops, _, amps = profile(ctx, circuit, cand.text, grid, finals)
        feats.append(op_features(ops))
        times.append(ops[:, 7])
        if ref_amps is None:
            ref_amps = amps
        assert rel_err(amps, ref_amps) < 1e-5
    model = CostModel(hidden=64, seed=0)
    model.fit(np.vstack(feats), np.concatenate(times), epochs=1500)

    def measure(text):
        ctx.evaluate_many(circuit, text, grid, "", finals, 1 << 40)
        best = float("inf")
        for _ in range(3):
            out = ctx.evaluate_many(circuit, text, grid, "", finals, 1 << 40)
            best = min(best, ctx.stats()["device_ms"])
        return best, [a for _, a in out]

    measured, predicted, analytic = [], [], []
    for cand in held:
        ops, _ = plan_ops(circuit, cand.text, grid, TF32X3, batch=len(finals))
        t, amps = measure(cand.text)
        assert rel_err(amps, ref_amps) < 1e-5, cand.label
        measured.append(t)
        predicted.append(model.predict_plan_ms(ops))
        analytic.append(analytic_ms(ops))
    rho_model = _spearman(predicted, measured)
    rho_analytic = _spearman(analytic, measured)
    t_supplied, amps = measure(supplied)
    assert rel_err(amps, ref_amps) < 1e-5
    pred_best, text, label = choose_ordering(model, circuit, grid, held, supplied, TF32X3, len(finals), 8e9)
    t_chosen, _ = measure(text)
    t_best = min(measured)
    t_analytic_pick = measured[int(np.argmin(analytic))]
    with capsys.disabled():
        print(f"\nlearned ordering (6x6, 8 strings): spearman model {rho_model:.3f} vs roofline "
              f"{rho_analytic:.3f}; supplied {t_supplied:.2f} ms, model pick '{label}' {t_chosen:.2f} ms, "
              f"roofline pick {t_analytic_pick:.2f} ms, best measured {t_best:.2f} ms")
    assert rho_model > 0.7
    assert rho_model >= rho_analytic - 0.05
    assert t_chosen <= 1.1 * t_supplied
