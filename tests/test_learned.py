"""Learned ordering choice: candidate generation (CPU), the perceptron's
kernels against the CPU oracle (gradient check), and what the trained model
gains over the supplied ordering and the analytic cost on a real circuit."""
import numpy as np
import pytest

from oracle import mlp_oracle
from qflex_gb300 import FP16X3, TF32X3, Context, rqc
from qflex_gb300.learned import N_FEATURES, CostModel, analytic_ms, candidate_orderings, op_features, plan_ops


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


def test_sweep_candidates_and_auto_orderer_cost(built_lib):
    """The 7x7 sweep variants keep the supplied ordering's cuts, so they
    plan to the same slices; most fit the 2^31-element tensor limit; the
    reference auto-orderer's cost is the plan's sum of m n k."""
    from qflex_gb300._lib import QflexGb300Error
    from qflex_gb300.learned import auto_orderer_cost, sweep_candidates_7x7
    c = rqc.random_circuit(7, 7, 32, seed=0)
    g = rqc.grid_text(7, 7)
    cands = sweep_candidates_7x7((0,), (1,), count=120, seed=2)
    assert len(cands) == 120 and len({x.text for x in cands}) == 120
    assert all("cut (0) 44 45" in x.text and "cut (1) 20 27" in x.text for x in cands)
    ok = 0
    for cand in cands:
        try:
            ops, _ = plan_ops(c, cand.text, g, FP16X3)
        except QflexGb300Error as e:
            assert "2^31" in str(e)
            continue
        ok += 1
        prod = ops[:, 0] != 0
        assert auto_orderer_cost(ops) == pytest.approx(ops[prod, 4].sum() / 8)
    assert ok > 60


@pytest.mark.gpu
def test_learned_choice_on_7x7(built_lib, capsys):
    """7x7 grid, depth (1+32+1), one value per cut, 4 output strings, 3xFP16:
    about 500 seeded sweep variants, the model trained on the per-op
    timings of 12, the rest ranked by the model, by the reference
    auto-orderer's cost (sum of m n k) and by the roofline estimate; the
    three picks, the supplied ordering and 40 held-out candidates measured.
    Every measured ordering gives the supplied ordering's amplitudes; the
    model ranks the measured candidates at least as well as the
    auto-orderer's cost, with no more regret on random subsets of 8, and its
    pick is not slower than the supplied ordering."""
    from qflex_gb300.learned import run_search, sweep_candidates_7x7
    circuit = rqc.random_circuit(7, 7, 32, seed=0)
    grid = rqc.grid_text(7, 7)
    supplied = rqc.ordering_7x7((0,), (1,))
    finals = rqc.random_bitstrings(49, 4, 12)
    cands = sweep_candidates_7x7((0,), (1,), count=500, seed=1)
    rep = run_search(circuit, grid, supplied, cands, finals, FP16X3, n_train=12, n_sample=40, seed=3,
                     repeats=3, log=lambda *a: None)
    picks, sample = rep["picks"], rep["sample"]
    with capsys.disabled():
        print(f"\nlearned ordering (7x7 d32, {rep['planned']} of {rep['candidates']} candidates planned): "
              f"spearman {sample['spearman']}; regret {sample['mean_regret_8_of_sample']}; "
              f"disagreeing subsets {sample['subsets_where_model_and_auto_orderer_disagree']}, model faster in "
              f"{sample['of_those_model_pick_faster']}; supplied {rep['supplied_ms']:.1f} ms, picks "
              + ", ".join(f"{k} {v['label']} {v['measured_ms']:.1f} ms" for k, v in picks.items()))
    for v in picks.values():
        assert v["amplitude_err_vs_supplied"] < 1e-5
    rho = sample["spearman"]
    assert rho["model"] > 0.8 and rho["model"] >= rho["auto_orderer"] - 0.02
    reg = sample["mean_regret_8_of_sample"]
    assert reg["model"] <= reg["auto_orderer"] + 0.005
    assert picks["model"]["measured_ms"] <= 1.03 * rep["supplied_ms"]


def test_learned_ordering_of_the_benchmark_workload(built_lib):
    """The committed learned ordering of the 7x7 (1+32+1) workload sums the
    same 16 cut slices as the supplied ordering, with no more flop."""
    c, o, g, ini, finals = rqc.workload("c3")
    plan = Context(-1, FP16X3)
    a = plan.evaluate(c, rqc.ordering_7x7_learned(), g, ini, finals[0], 1 << 40)
    learned = plan.stats()
    b = plan.evaluate(c, o, g, ini, finals[0], 1 << 40)
    supplied = plan.stats()
    assert [s for s, _ in a] == [s for s, _ in b]
    assert learned["n_leaves"] == supplied["n_leaves"] == 16
    assert learned["gemm_flop"] <= supplied["gemm_flop"]


@pytest.mark.gpu
def test_learned_ordering_amplitudes_match_fp64(built_lib):
    import json

    from tests.conftest import ROOT, rel_err_per_amplitude
    c, _, g, ini, _ = rqc.workload("c3")
    ref = json.loads((ROOT / "tests" / "golden" / "c3_fp64.json").read_text())
    strings = [r["final"] for r in ref["amplitudes"]]
    want = [complex(*r["amplitude"]) for r in ref["amplitudes"]]
    ctx = Context(0, FP16X3)
    got = [x for _, x in ctx.evaluate_many(c, rqc.ordering_7x7_learned(), g, ini, strings, 1 << 40)]
    assert rel_err_per_amplitude(got, want) < 1e-5
