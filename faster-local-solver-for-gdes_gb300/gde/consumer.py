"""Downstream consumer of propagated features, kept on the device.

The reference's InstantGNN experiment trains an MLP classifier on the
propagated feature matrix after every snapshot (instantGNN-arxiv-exp.py:34-171:
Linear + BatchNorm + ReLU + dropout layers, NLL loss, early stopping on the
validation weighted F1, then train / valid / test accuracy), moving batches
through host DataLoaders.  Here the propagated matrix P produced by
``api.feature_push`` / ``api.feature_update`` is already a device tensor: it
is normalised, sliced into mini-batches and scored without leaving the GPU;
only the scalar metrics come back.
"""
from __future__ import annotations

import torch
import torch.nn as nn
import torch.nn.functional as F


class ClassMLP(nn.Module):
    """``num_layers`` linear layers with batch norm, ReLU and dropout between them."""

    def __init__(self, in_dim: int, hidden: int, classes: int, num_layers: int = 3, dropout: float = 0.3):
        super().__init__()
        dims = [in_dim] + [hidden] * (num_layers - 1) + [classes]
        self.lins = nn.ModuleList(nn.Linear(a, b) for a, b in zip(dims[:-1], dims[1:]))
        self.norms = nn.ModuleList(nn.BatchNorm1d(h) for h in dims[1:-1])
        self.dropout = dropout

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        for lin, bn in zip(self.lins[:-1], self.norms):
            x = F.dropout(F.relu(bn(lin(x))), p=self.dropout, training=self.training)
        return torch.log_softmax(self.lins[-1](x), dim=-1)


def weighted_f1(pred: torch.Tensor, target: torch.Tensor, classes: int) -> float:
    """Support-weighted mean of per-class F1 (computed on the device)."""
    tp = torch.bincount(target[pred == target], minlength=classes).double()
    pc = torch.bincount(pred, minlength=classes).double()
    tc = torch.bincount(target, minlength=classes).double()
    f1 = torch.where(pc + tc > 0, 2 * tp / (pc + tc).clamp(min=1), torch.zeros_like(tp))
    return float((f1 * tc).sum() / tc.sum().clamp(min=1))


def _accuracy(model, X, y, idx, batch):
    model.eval()
    correct = 0
    preds = []
    with torch.no_grad():
        for s in range(0, idx.numel(), batch):
            b = idx[s:s + batch]
            p = model(X[b]).argmax(dim=1)
            preds.append(p)
            correct += int((p == y[b]).sum())
    return correct / max(idx.numel(), 1), torch.cat(preds) if preds else y[:0]


def train_eval(P: torch.Tensor, labels: torch.Tensor, split: dict, *, hidden: int = 256, num_layers: int = 3,
               dropout: float = 0.3, lr: float = 1e-3, epochs: int = 50, patience: int = 10, batch: int = 8192,
               seed: int = 0) -> dict:
    """Train a ClassMLP on the rows of device matrix ``P``; returns accuracies and the best valid F1.

    ``split`` maps "train" / "valid" / "test" to device index tensors.
    """
    dev = P.device
    g = torch.Generator(device="cpu").manual_seed(seed)
    torch.manual_seed(seed)
    X = P.float()
    mu = X[split["train"]].mean(0, keepdim=True)
    sd = X[split["train"]].std(0, keepdim=True).clamp(min=1e-12)
    X = (X - mu) / sd
    y = labels.to(dev).long()
    classes = int(y.max()) + 1
    model = ClassMLP(X.shape[1], hidden, classes, num_layers, dropout).to(dev)
    opt = torch.optim.Adam(model.parameters(), lr=lr)
    tr = split["train"]
    best_f1, best_state, bad = -1.0, None, 0
    for _ in range(epochs):
        model.train()
        perm = tr[torch.randperm(tr.numel(), generator=g).to(dev)]
        for s in range(0, perm.numel(), batch):
            b = perm[s:s + batch]
            loss = F.nll_loss(model(X[b]), y[b])
            opt.zero_grad()
            loss.backward()
            opt.step()
        _, pv = _accuracy(model, X, y, split["valid"], batch)
        f1 = weighted_f1(pv, y[split["valid"]], classes)
        if f1 > best_f1:
            best_f1, bad = f1, 0
            best_state = {k: v.detach().clone() for k, v in model.state_dict().items()}
        else:
            bad += 1
            if bad >= patience:
                break
    model.load_state_dict(best_state)
    out = {"valid_f1": best_f1}
    for k in ("train", "valid", "test"):
        out[k + "_acc"] = _accuracy(model, X, y, split[k], batch)[0]
    return out


def random_split(n: int, device, seed: int = 0, frac=(0.6, 0.2)) -> dict:
    """Random train / valid / test node split as device index tensors."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g)
    a, b = int(frac[0] * n), int((frac[0] + frac[1]) * n)
    return {"train": perm[:a].to(device), "valid": perm[a:b].to(device), "test": perm[b:].to(device)}
