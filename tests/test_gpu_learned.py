"""Learned Newton predictor: device network against the FP64 oracle, training, and what the trained
predictor gains over the method without it on held-out load paths (FP64 residual judged)."""
import numpy as np
import pytest

from ikarus_gb300 import problems
from oracle import mlp as mlp_oracle

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_oracle(ikr):
    rng = np.random.default_rng(3)
    net = ikr.MLP(n_in=21, width=64, depth=4, n_out=16, seed=7)
    dims = mlp_oracle.layer_dims(21, 64, 4, 16)
    p = net.params
    x = rng.standard_normal((37, 21)).astype(np.float32)
    t = rng.standard_normal((37, 16)).astype(np.float32)
    y = net.forward(x)
    y_ref = mlp_oracle.forward(p, dims, x)
    assert np.abs(y - y_ref).max() <= 1e-4 * np.abs(y_ref).max()
    loss, g = net.loss_grad(x, t)
    loss_ref, g_ref = mlp_oracle.loss_grad(p, dims, x, t)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert np.abs(g - g_ref).max() <= 1e-4 * np.abs(g_ref).max()


def test_mlp_training_fits_a_smooth_map(ikr):
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (512, 3)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], x[:, 2] ** 2 - 0.3], axis=1).astype(np.float32)
    net = ikr.MLP(3, 64, 3, 2, seed=1)
    l0 = float(((net.forward(x) - t) ** 2).mean())
    loss = net.train(x, t, epochs=200, batch=64, lr=2e-3, seed=2)
    l1 = float(((net.forward(x) - t) ** 2).mean())
    assert l1 < 0.05 * l0 and loss < 0.05 * l0


def _run(ikr, p, fes, asm, theta, kind=0, pred=None, record=False):
    fes.clear_neumann()
    fe, fl, tr = problems.learned_loads(p, theta)
    fes.add_neumann(fe, fl, tr)
    req = ikr.FERequirements(fes)
    st = ikr.NRSettings(tol=1e-8, maxIter=30, relative=True, eisenstat_walker=True, linear_rtol=1e-2,
                        linear_rtol_min=1e-6)
    nr = ikr.NewtonRaphson(asm, ikr.NewtonRaphsonConfig(st, ikr.LinearSolver()))
    lc = ikr.LoadControl(nr, p.load_steps)
    lc.set_predictor(kind, pred, theta, record)
    info = lc.run(req)
    hist = None
    if kind:
        # per step: |R| unpredicted, |R| previous increment, |R| learned, kept (0 none, 1 previous, 2 learned)
        hist = lc.predictor_history()[:, 1:5].copy()
        print(np.array2string(hist, precision=3))
    _run.history = hist
    return info, req.globalSolution(), lc.predictor_stats()


def test_learned_predictor_against_its_fallback(ikr):
    """The trained predictor is judged against the previous-increment predictor it falls back to: on held-out paths
    every step keeps the candidate with the smaller FP64 residual (the learned one only where it beats the previous
    increment), every path reaches the FP64 tolerance, and the Newton iterations of the three predictors are
    reported.  At this training size (30 paths, 300 snapshots) the network does not beat its fallback measurably:
    the iteration assertion is that the learned predictor, with its gate, is never worse than the fallback by more
    than one iteration per path, and strictly better than no predictor."""
    p = problems.learned_cantilever(16, 4, 4, load_steps=10)
    fes, asm = problems.build_gpu(p, precision=1)
    rng = np.random.default_rng(11)
    pred = ikr.LearnedPredictor(fes, n_params=9, n_modes=16, width=128, depth=4, capacity=400, seed=3)
    for _ in range(30):
        info, _, _ = _run(ikr, p, fes, asm, problems.sample_load_parameters(rng), kind=0, pred=pred, record=True)
        assert info.success
    assert pred.num_snapshots() == 300
    loss, energy = pred.fit(epochs=400, batch=32, lr=1e-3)
    assert energy > 0.99
    plain_its, prev_its, learned_its = 0, 0, 0
    for _ in range(5):
        theta = problems.sample_load_parameters(rng)
        info0, u0, _ = _run(ikr, p, fes, asm, theta, kind=0)
        info1, u1, _ = _run(ikr, p, fes, asm, theta, kind=1)
        info2, u2, (acc, rej) = _run(ikr, p, fes, asm, theta, kind=2, pred=pred)
        assert info0.success and info1.success and info2.success
        h = _run.history
        for r_prev, r_learned, kept in h[:, 1:4]:
            if kept == 2:
                assert r_learned <= r_prev  # the learned candidate is kept only where its FP64 residual is smaller
            elif kept == 1 and np.isfinite(r_learned) and r_learned > 0:
                assert r_learned >= r_prev
        # all reach the FP64 tolerance; the converged paths agree
        assert np.abs(u2 - u0).max() <= 1e-5 * np.abs(u0).max()
        plain_its += info0.totalIterations
        prev_its += info1.totalIterations
        learned_its += info2.totalIterations
        assert acc + rej == p.load_steps
    print(f"Newton iterations over 5 held-out paths: none {plain_its}, previous increment {prev_its}, "
          f"learned {learned_its}")
    assert learned_its < plain_its
    assert learned_its <= prev_its + 5


def test_second_order_extrapolation_predictor_reaches_the_same_path(ikr):
    """Predictor kind 3 (u + 2 du_{k-1} - du_{k-2}, previous increment as its fallback): every step reaches the
    FP64 tolerance and the converged path agrees with the unpredicted one; from the third step on the candidate is
    evaluated (its residual norm is recorded) and kept or rejected by the residual test."""
    p = problems.learned_cantilever(16, 4, 4, load_steps=10)
    fes, asm = problems.build_gpu(p, precision=1)
    theta = problems.sample_load_parameters(np.random.default_rng(5))
    info0, u0, _ = _run(ikr, p, fes, asm, theta, kind=0)
    info3, u3, (acc, rej) = _run(ikr, p, fes, asm, theta, kind=3)
    assert info0.success and info3.success
    assert np.abs(u3 - u0).max() <= 1e-5 * np.abs(u0).max()
    assert acc + rej == p.load_steps
