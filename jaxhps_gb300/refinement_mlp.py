"""Learned refinement proposal for adaptive octree meshing.

A 513 -> 64 -> 64 -> 1 MLP (ReLU) reads 8^3 uniform samples of f over an
octree node (scaled by the meshing's current global norm of f) plus the
node's depth, and predicts the probability that the plain interpolation
criterion (_adaptive_discretization_3D.py:475-503 in the reference) refines
the node.  Inference, the loss, back-propagation and Adam all run in the
library's own CUDA kernels (hps_mlp_*).

``RefinementProposer`` plugs into ``generate_adaptive_mesh_level_restriction``
(and ``Domain.from_adaptive_discretization(proposer=...)``): queued nodes
whose predicted probability exceeds ``threshold`` are refined without the
full check; all other nodes, and therefore every leaf of the accepted tree,
are decided by the plain criterion.  ``LabelRecorder`` collects (features,
refine/keep) pairs from plain meshing runs for training.  This component has
no counterpart in the reference.
"""

from __future__ import annotations

import ctypes as C
from typing import Callable, List, Sequence

import numpy as np
import torch

from . import _native as nat
from ._adaptive_discretization_3D import evaluate_f

N_IN, N_HIDDEN = 513, 64


def _offsets():
    w1 = 0
    b1 = w1 + N_HIDDEN * N_IN
    w2 = b1 + N_HIDDEN
    b2 = w2 + N_HIDDEN * N_HIDDEN
    w3 = b2 + N_HIDDEN
    b3 = w3 + N_HIDDEN
    return dict(W1=(w1, (N_HIDDEN, N_IN)), b1=(b1, (N_HIDDEN,)), W2=(w2, (N_HIDDEN, N_HIDDEN)), b2=(b2, (N_HIDDEN,)),
                w3=(w3, (N_HIDDEN,)), b3=(b3, (1,)))


def node_features(bounds: np.ndarray, depths: Sequence[int], f_fn: Callable, scale: float, device) -> torch.Tensor:
    """X (n, 513) FP32 on ``device``: f at the 8x8x8 cell centres of every node
    divided by ``scale``, then depth / 16."""
    L = nat.lib()
    dev = torch.device(device)
    b = torch.as_tensor(np.ascontiguousarray(bounds, dtype=np.float64), device=dev)
    n = b.shape[0]
    pts = torch.empty((n, 512, 3), dtype=torch.float64, device=dev)
    sp = nat.stream_ptr()
    nat.check(L.hps_mlp_sample_points(n, b.data_ptr(), pts.data_ptr(), sp), "hps_mlp_sample_points")
    fv = evaluate_f(f_fn, pts).reshape(n, 512).contiguous()
    d = torch.as_tensor(np.asarray(depths, dtype=np.int32), device=dev)
    X = torch.empty((n, N_IN), dtype=torch.float32, device=dev)
    nat.check(L.hps_mlp_features(n, fv.data_ptr(), d.data_ptr(), float(scale), X.data_ptr(), sp), "hps_mlp_features")
    return X


class RefinementMLP:
    """The network's parameters (one FP32 vector on the device) and Adam state."""

    def __init__(self, device=None, seed: int = 0):
        L = nat.lib()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.n_params = int(L.hps_mlp_param_count())
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n_params, dtype=np.float32)
        off = _offsets()
        for name, fan_in in (("W1", N_IN), ("W2", N_HIDDEN), ("w3", N_HIDDEN)):
            o, shape = off[name]
            p[o:o + int(np.prod(shape))] = rng.standard_normal(int(np.prod(shape))) * np.sqrt(2.0 / fan_in)
        self.params = torch.as_tensor(p, device=self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0

    # -- parameters ---------------------------------------------------------
    def state(self) -> dict:
        p = self.params.cpu().numpy()
        return {k: p[o:o + int(np.prod(s))].reshape(s).copy() for k, (o, s) in _offsets().items()}

    def load_state(self, state: dict) -> None:
        p = np.zeros(self.n_params, dtype=np.float32)
        for k, (o, s) in _offsets().items():
            p[o:o + int(np.prod(s))] = np.asarray(state[k], dtype=np.float32).ravel()
        self.params = torch.as_tensor(p, device=self.device)

    def save(self, path: str) -> None:
        np.savez(path, **self.state())

    @classmethod
    def load(cls, path: str, device=None) -> "RefinementMLP":
        net = cls(device=device)
        with np.load(path) as z:
            net.load_state({k: z[k] for k in z.files})
        return net

    # -- compute ------------------------------------------------------------
    def forward(self, X: torch.Tensor, keep_hidden: bool = False):
        L = nat.lib()
        n = X.shape[0]
        X = X.contiguous()
        logit = torch.empty(n, dtype=torch.float32, device=self.device)
        H1 = torch.empty((n, N_HIDDEN), dtype=torch.float32, device=self.device) if keep_hidden else None
        H2 = torch.empty((n, N_HIDDEN), dtype=torch.float32, device=self.device) if keep_hidden else None
        nat.check(L.hps_mlp_forward(n, X.data_ptr(), self.params.data_ptr(), nat.ptr(H1), nat.ptr(H2),
                                    logit.data_ptr(), nat.stream_ptr()), "hps_mlp_forward")
        return (logit, H1, H2) if keep_hidden else logit

    def predict_proba(self, X: torch.Tensor) -> torch.Tensor:
        return torch.sigmoid(self.forward(X))

    def loss_and_grad(self, X: torch.Tensor, y: torch.Tensor, pos_weight: float = 1.0):
        """Mean weighted BCE over the rows and its gradient (FP32 vectors)."""
        L = nat.lib()
        n = X.shape[0]
        logit, H1, H2 = self.forward(X, keep_hidden=True)
        dlogit = torch.empty_like(logit)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        y = y.to(device=self.device, dtype=torch.float32).contiguous()
        sp = nat.stream_ptr()
        nat.check(L.hps_mlp_bce(n, logit.data_ptr(), y.data_ptr(), float(pos_weight), dlogit.data_ptr(),
                                loss.data_ptr(), sp), "hps_mlp_bce")
        grad = torch.zeros_like(self.params)
        nat.check(L.hps_mlp_backward(n, X.contiguous().data_ptr(), self.params.data_ptr(), H1.data_ptr(), H2.data_ptr(),
                                     dlogit.data_ptr(), grad.data_ptr(), sp), "hps_mlp_backward")
        return loss / n, grad

    def adam_step(self, grad: torch.Tensor, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999,
                  eps: float = 1e-8) -> None:
        self.step += 1
        nat.check(nat.lib().hps_mlp_adam(self.params.data_ptr(), grad.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                         lr, beta1, beta2, eps, self.step, nat.stream_ptr()), "hps_mlp_adam")

    def train(self, X: torch.Tensor, y: torch.Tensor, epochs: int = 30, batch: int = 1024, lr: float = 1e-3,
              pos_weight: float | None = None, seed: int = 0) -> List[float]:
        """Adam on mini-batches; returns the mean loss of every epoch."""
        n = X.shape[0]
        y = y.to(device=self.device, dtype=torch.float32)
        if pos_weight is None:
            npos = float(y.sum().item())
            pos_weight = max(1.0, (n - npos) / max(npos, 1.0))
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.device)
            tot = 0.0
            for s in range(0, n, batch):
                idx = perm[s:s + batch]
                loss, grad = self.loss_and_grad(X[idx], y[idx], pos_weight)
                self.adam_step(grad, lr=lr)
                tot += float(loss.item()) * idx.numel()
            hist.append(tot / n)
        return hist


class RefinementProposer:
    """Meshing hook: refine without the full check when the network is sure."""

    def __init__(self, mlp: RefinementMLP, threshold: float = 0.97):
        self.mlp = mlp
        self.threshold = threshold
        self.proposed = 0

    def confident_refine(self, queue, f_fn, global_nrm, device) -> np.ndarray:
        bounds = np.array([n.bounds for n in queue])
        X = node_features(bounds, [n.depth for n in queue], f_fn, max(abs(global_nrm), 1e-300), device)
        sure = (self.mlp.predict_proba(X) > self.threshold).cpu().numpy()
        self.proposed += int(sure.sum())
        return sure

    def record(self, queue, check_idx, fails) -> None:
        pass


class LabelRecorder:
    """Meshing hook that proposes nothing and records, for every fully checked
    node, its features and whether the plain criterion refined it."""

    def __init__(self, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.X: List[torch.Tensor] = []
        self.y: List[np.ndarray] = []
        self._f = None
        self._scale = 1.0

    def confident_refine(self, queue, f_fn, global_nrm, device) -> np.ndarray:
        self._f = f_fn
        self._scale = max(abs(global_nrm), 1e-300)
        return np.zeros(len(queue), dtype=bool)

    def record(self, queue, check_idx, fails) -> None:
        nodes = [queue[i] for i in check_idx]
        bounds = np.array([n.bounds for n in nodes])
        self.X.append(node_features(bounds, [n.depth for n in nodes], self._f, self._scale, self.device))
        self.y.append(np.asarray(fails, dtype=np.float32))

    def dataset(self):
        X = torch.cat(self.X) if self.X else torch.empty((0, N_IN), device=self.device)
        y = torch.as_tensor(np.concatenate(self.y) if self.y else np.zeros(0, np.float32), device=self.device)
        return X, y
