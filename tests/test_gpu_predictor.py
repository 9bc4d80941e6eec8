"""Learned secular initial iterate: GPU training gradient vs the FP64 numpy
oracle, training reduces the loss, and the learned start never changes the
roots beyond the solver's tolerance while cutting evaluations."""
import numpy as np
import pytest
import torch

import hsspack_gb300 as hp
from hsspack_gb300 import predictor as pr
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_gradient_matches_numpy_oracle():
    probs = pr.merge_problems(6, sizes=(64, 128), seed=11)
    X, T = pr.collect(probs)
    assert torch.isfinite(X).all() and torch.isfinite(T).all()
    norm = torch.cat([X.mean(0), X.std(0) + 1e-6]).contiguous()
    W = torch.tensor(pr.init_weights(3), device="cuda")
    loss, G = pr.grad(X, T, norm, W)
    lr, gr = mlp_ref.loss_and_grad(X.cpu().numpy(), T.cpu().numpy(), norm.cpu().numpy(),
                                   W.cpu().numpy())
    assert abs(float(loss) - lr) <= 1e-4 * lr
    G = G.cpu().numpy()
    assert np.max(np.abs(G - gr)) <= 2e-4 * np.max(np.abs(gr)), np.max(np.abs(G - gr))


def test_training_and_learned_start():
    train_p = pr.merge_problems(120, seed=21, kinds=("uniform", "toeplitz"))
    test_p = pr.merge_problems(30, seed=22, kinds=("uniform", "toeplitz"))
    X, T = pr.collect(train_p)
    norm0 = torch.cat([X.mean(0), X.std(0) + 1e-6]).contiguous()
    W0 = torch.tensor(pr.init_weights(0), device="cuda")
    l0 = float(pr.grad(X, T, norm0, W0)[0])
    W, norm, loss = pr.train(X, T, epochs=8, batch=2048)
    assert loss < 0.8 * l0
    rc = hp.load().hss_predictor_set(W.ctypes.data, norm.ctypes.data)
    assert rc == 0
    base, _, lam0 = pr.iterations(test_p, False)
    learned, fb, lam1 = pr.iterations(test_p, True)
    for a, b in zip(lam0, lam1):
        assert np.max(np.abs(a - b)) <= 1e-14 * max(1.0, np.max(np.abs(a)))
    # what the trained network gains: fewer FP64 pole-sum evaluations per root
    # than the standard start (measured 4.05 vs 4.21 with the committed weights)
    assert learned < base, (learned, base)


def test_committed_weights_gain():
    assert pr.install(), "committed predictor weights missing"
    test_p = pr.merge_problems(60, seed=31, kinds=("uniform", "uniform", "toeplitz", "graded"))
    base, _, lam0 = pr.iterations(test_p, False)
    learned, fb, lam1 = pr.iterations(test_p, True)
    for a, b in zip(lam0, lam1):
        assert np.max(np.abs(a - b)) <= 1e-14 * max(1.0, np.max(np.abs(a)))
    assert learned < base, (learned, base)
