"""GPU tests of the learned refinement proposal: the hand-written forward,
loss, backward and Adam kernels against the NumPy oracle; training on a
separable set; and meshing with the trained proposer against plain meshing
(fewer full checks, every accepted leaf still passes the plain criterion)."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from jaxhps_gb300 import _adaptive_discretization_3D as ad
from jaxhps_gb300 import refinement_mlp as rm
from jaxhps_gb300._discretization_tree import get_all_leaves
from jaxhps_gb300._discretization_tree_operations_3D import add_eight_children
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _net_and_data(cuda, n=70, seed=0):
    net = rm.RefinementMLP(device=cuda, seed=seed)
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 513)).astype(np.float32)
    y = (rng.random(n) > 0.6).astype(np.float32)
    return net, X, y


def test_forward_matches_oracle(cuda):
    net, X, _ = _net_and_data(cuda)
    z = net.forward(torch.as_tensor(X, device=cuda)).cpu().numpy()
    zr, _, _ = O.mlp_forward(net.params.cpu().numpy(), X.astype(np.float64))
    assert np.abs(z - zr).max() <= 1e-4 * max(1.0, np.abs(zr).max())


def test_loss_and_gradient_match_oracle(cuda):
    net, X, y = _net_and_data(cuda, n=100, seed=1)
    loss, grad = net.loss_and_grad(torch.as_tensor(X, device=cuda), torch.as_tensor(y, device=cuda), pos_weight=2.0)
    p = net.params.cpu().numpy().astype(np.float64)
    lr = O.mlp_loss(p, X.astype(np.float64), y, 2.0)
    gr = O.mlp_grad(p, X.astype(np.float64), y, 2.0)
    assert abs(float(loss.item()) - lr) <= 1e-5 * max(1.0, lr)
    g = grad.cpu().numpy()
    assert np.abs(g - gr).max() <= 1e-4 * np.abs(gr).max()


def test_adam_step_matches_oracle(cuda):
    net, X, y = _net_and_data(cuda, n=64, seed=2)
    p0 = net.params.cpu().numpy().astype(np.float64)
    m = np.zeros_like(p0)
    v = np.zeros_like(p0)
    for step in (1, 2):
        _, grad = net.loss_and_grad(torch.as_tensor(X, device=cuda), torch.as_tensor(y, device=cuda))
        g = grad.cpu().numpy().astype(np.float64)
        net.adam_step(grad, lr=1e-2)
        p0, m, v = O.adam_step(p0, g, m, v, step, lr=1e-2)
        assert np.abs(net.params.cpu().numpy() - p0).max() <= 1e-5


def test_features_kernel(cuda):
    b = np.array([[0.0, 1.0, 0.0, 0.5, -1.0, 1.0], [0.25, 0.5, 0.5, 0.75, 0.0, 0.25]])
    X = rm.node_features(b, [2, 5], lambda x: x[..., 0] + 2 * x[..., 1] - x[..., 2], 4.0, cuda).cpu().numpy()
    for i in range(2):
        c = [(np.arange(8) + 0.5) * (b[i, 2 * d + 1] - b[i, 2 * d]) / 8 + b[i, 2 * d] for d in range(3)]
        Xg, Yg, Zg = np.meshgrid(*c, indexing="ij")
        assert np.allclose(X[i, :512], ((Xg + 2 * Yg - Zg) / 4.0).ravel(), atol=1e-6)
    assert np.allclose(X[:, 512], [2 / 16, 5 / 16])


def test_training_learns_a_separable_rule(cuda):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((4000, 513)).astype(np.float32)
    y = (X[:, :64].std(1) * X[:, 7] > 0.3).astype(np.float32)
    net = rm.RefinementMLP(device=cuda, seed=3)
    Xt = torch.as_tensor(X, device=cuda)
    hist = net.train(Xt, torch.as_tensor(y, device=cuda), epochs=25, batch=512, lr=2e-3)
    assert hist[-1] < 0.5 * hist[0]
    acc = ((net.predict_proba(Xt).cpu().numpy() > 0.5) == (y > 0.5)).mean()
    assert acc > 0.9


def _front(c, R, k):
    def f(x):
        xp = torch if isinstance(x, torch.Tensor) else np
        r = xp.sqrt(((x[..., 0] - c[0]) ** 2 + (x[..., 1] - c[1]) ** 2 + (x[..., 2] - c[2]) ** 2))
        return xp.arctan(k * (r - R))
    return f


def _all_leaves_pass(root, f, tol, p, gn, cuda):
    """Every leaf passes the plain L-infinity criterion at norm gn."""
    leaves = get_all_leaves(root)
    consts = ad._CheckConstants(p, cuda)
    diff, ref, _ = ad.refinement_check(np.array([lf.bounds for lf in leaves]), f, consts, cuda)
    return bool(np.all(diff / np.maximum(gn, ref) < tol))


def test_trained_proposer_saves_checks(cuda):
    p, q, tol = 6, 4, 1e-3
    rec = rm.LabelRecorder(device=cuda)
    rng = np.random.default_rng(7)
    for _ in range(6):
        f = _front(rng.uniform(-0.2, 0.3, 3), rng.uniform(0.5, 0.9), rng.uniform(8, 30))
        root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
        add_eight_children(root, root=root, q=q)
        ad.generate_adaptive_mesh_level_restriction(root, f, tol, p, q, proposer=rec)
    X, y = rec.dataset()
    assert X.shape[0] > 500 and 0.05 < float(y.mean()) < 0.95
    net = rm.RefinementMLP(device=cuda, seed=0)
    net.train(X, y, epochs=40, batch=256, lr=2e-3)
    target = _front((-0.05, -0.05, -0.05), 0.7, 20.0)
    runs = {}
    for name, prop in (("plain", None), ("mlp", rm.RefinementProposer(net, threshold=0.9))):
        root = hps.DiscretizationNode3D(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
        add_eight_children(root, root=root, q=q)
        st = {}
        ad.generate_adaptive_mesh_level_restriction(root, target, tol, p, q, proposer=prop, stats=st)
        runs[name] = (root, st)
    plain, mlp = runs["plain"][1], runs["mlp"][1]
    assert mlp["proposed"] > 0
    assert mlp["checked"] < plain["checked"]
    assert mlp["leaves"] <= 1.25 * plain["leaves"]
    # the plain criterion, at the plain run's final global norm, decides every accepted leaf of both trees
    gn = plain["global_norm"]
    for root, _ in runs.values():
        assert _all_leaves_pass(root, target, tol, p, gn, cuda)
