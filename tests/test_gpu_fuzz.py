"""Seeded randomized parity sweep over (p, q, L, nsrc, coefficients, root,
precision) for the uniform 2D DtN build + solve, against the FP64 oracle.
The configurations are drawn once from a fixed seed (the same list on every
run, so a failure names its case); each stays small enough for the oracle to
finish in about a second.

Tolerances (relative max error against the oracle): FP64 path 1e-11, mixed
path 1e-10, as in the fixed-case tests."""

import numpy as np
import pytest
import torch

import jaxhps_gb300 as hps
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


def _cases(n=12, seed=20261204):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        p = int(rng.integers(4, 17))
        q = int(rng.integers(max(2, p - 4), p - 1)) if p > 4 else 2
        L = int(rng.integers(1, 4 if p <= 12 else 3))
        nsrc = [None, 1, 3][int(rng.integers(0, 3))]
        terms = sorted(str(t) for t in rng.choice(["D_x", "D_y", "D_xy", "I"], size=int(rng.integers(0, 3)),
                                                  replace=False))
        x0, y0 = (float(v) for v in rng.uniform(-1.0, 1.0, 2))
        side = float(rng.uniform(0.5, 3.0))
        precision = "mixed" if p >= 6 and rng.random() < 0.5 else "float64"
        root = (x0, x0 + side, y0, y0 + side)
        out.append((p, q, L, nsrc, tuple(terms), root, precision, int(rng.integers(1 << 30))))
    return out


def _coefficient(name, x, rng):
    a, b = rng.uniform(-0.3, 0.3, 2)
    if name == "I":
        return 1.0 + 0.5 * np.exp(-((x[..., 0] - a) ** 2 + (x[..., 1] - b) ** 2))
    return 0.2 * np.sin(a + x[..., 0]) * np.cos(b + x[..., 1])


@pytest.mark.parametrize("p,q,L,nsrc,terms,root,precision,seed", _cases())
def test_random_configuration_matches_oracle(cuda, p, q, L, nsrc, terms, root, precision, seed):
    rng = np.random.default_rng(seed)
    dom = hps.Domain(p=p, q=q, root=hps.DiscretizationNode2D(*root), L=L)
    x = dom.interior_points
    # a diffusion term with a positive varying coefficient keeps the leaf problems well posed
    kxx = 1.0 + 0.3 * np.cos(x[..., 0]) ** 2
    kyy = 1.0 + 0.3 * np.sin(x[..., 1]) ** 2
    coeffs = {"D_xx": kxx, "D_yy": kyy}
    for name in terms:
        coeffs[name] = _coefficient(name, x, rng)
    f = rng.standard_normal(x.shape[:2] + ((nsrc,) if nsrc else ()))
    pde = hps.PDEProblem(dom, source=f, **{f"{k}_coefficients": v for k, v in coeffs.items()})
    hps.build_solver(pde, precision=precision)
    bp = dom.boundary_points
    g = np.cos(bp[:, 0]) * np.exp(0.3 * bp[:, 1])
    if nsrc:
        g = np.stack([g * (k + 1) - k for k in range(nsrc)], -1)
    u = hps.solve(pde, g)
    u = u.numpy() if isinstance(u, torch.Tensor) else np.asarray(u)
    ur = O.Problem2D(root, L, p, q, coeffs, f).build().solve(g)
    assert u.shape == ur.shape
    err = np.abs(u - ur).max() / np.abs(ur).max()
    assert err < (1e-10 if precision == "mixed" else 1e-11), err
