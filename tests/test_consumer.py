"""The device-side MLP consumer of propagated features (runs on CPU tensors here)."""
import numpy as np
import pytest
import torch

from gde import consumer


def test_weighted_f1_matches_sklearn():
    metrics = pytest.importorskip("sklearn.metrics")
    rng = np.random.default_rng(0)
    t = rng.integers(0, 5, 400)
    p = np.where(rng.random(400) < 0.7, t, rng.integers(0, 5, 400))
    ours = consumer.weighted_f1(torch.from_numpy(p), torch.from_numpy(t), 5)
    assert ours == pytest.approx(metrics.f1_score(t, p, average="weighted"), abs=1e-12)


def test_mlp_learns_a_linear_labelling():
    rng = np.random.default_rng(1)
    n, f, c = 3000, 16, 4
    X = rng.standard_normal((n, f)).astype(np.float32)
    y = (X @ rng.standard_normal((f, c))).argmax(1)
    split = consumer.random_split(n, "cpu", seed=2)
    out = consumer.train_eval(torch.from_numpy(X), torch.from_numpy(y), split, hidden=64, epochs=40, patience=40,
                              batch=512)
    assert out["test_acc"] > 0.85
    assert 0.0 <= out["valid_f1"] <= 1.0
