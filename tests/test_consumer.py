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


@pytest.mark.gpu
def test_mlp_on_device_resident_propagated_features():
    """The hand-off of instantGNN-arxiv-exp.py:34-171: P from the device feature push goes to the MLP without a copy."""
    from gde import _lib as L
    from gde import api, graphs
    g = graphs.chung_lu(4000, 2.3, 8.0, 200.0, seed=5)
    deg = np.diff(g.indptr).astype(np.int64)
    rng = np.random.default_rng(3)
    f, c = 16, 4
    X = rng.standard_normal((g.n, f)).astype(np.float32)
    y = torch.from_numpy((X @ rng.standard_normal((f, c))).argmax(1)).cuda()
    Gd = api.Graph(g.indptr, g.indices, row_len=deg, degree=deg.astype(np.float64))
    P = torch.zeros((g.n, f), dtype=torch.float32, device="cuda")
    R = torch.from_numpy(X).cuda()
    ptr = P.data_ptr()
    api.feature_push(Gd, L.IGN, P, R, 1e-5, alpha=0.5, beta=0.5, prec="fp32")
    assert P.data_ptr() == ptr and P.is_cuda and torch.isfinite(P).all()
    split = consumer.random_split(g.n, "cuda", seed=2)
    out = consumer.train_eval(P, y, split, hidden=64, epochs=40, patience=40, batch=512)
    # labels are a linear map of X; alpha = 0.5 keeps half of each node's own features in P
    assert out["test_acc"] > 0.6
    assert 0.0 <= out["valid_f1"] <= 1.0
