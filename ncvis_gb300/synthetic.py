"""Seeded synthetic inputs with the shapes of the benchmark configurations
(the reference's own datasets are not available):

* gaussian_mixture: isotropic Gaussian mixture, centres ~ N(0, center_std^2 I),
  within-cluster std sigma, equal weights (the 10k x 64 default-parameter
  configuration, the differentiable-loss graph and the batched problems).
* vmf_mixture: unit vectors from a von Mises-Fisher mixture with uniform
  random mean directions, concentration kappa and Dirichlet(1) weights (the
  131,072 x 100 and 1,024,000 x 100 cosine configurations).  The component
  along the mean direction is drawn with Wood's rejection method (A. T. A.
  Wood, "Simulation of the von Mises Fisher distribution", Comm. Statist.
  Simul. Comput. 23(1), 1994); the orthogonal part is a uniform direction.
"""
from __future__ import annotations

import numpy as np


def gaussian_mixture(N: int, D: int, n_comp: int = 10, center_std: float = 5.0,
                     sigma: float = 1.0, seed: int = 42):
    rng = np.random.default_rng(seed)
    centers = rng.normal(0.0, center_std, size=(n_comp, D))
    labels = rng.integers(0, n_comp, size=N)
    X = centers[labels] + rng.normal(0.0, sigma, size=(N, D))
    return X.astype(np.float32), labels


def _wood_w(rng, kappa: float, D: int, n: int) -> np.ndarray:
    """n samples of w = <x, mu> for x ~ vMF(mu, kappa) on S^(D-1)."""
    m = D - 1
    b = m / (2.0 * kappa + np.sqrt(4.0 * kappa ** 2 + m ** 2))
    x0 = (1.0 - b) / (1.0 + b)
    c = kappa * x0 + m * np.log(1.0 - x0 ** 2)
    out = np.empty(n)
    filled = 0
    while filled < n:
        need = n - filled
        batch = int(need * 1.3) + 16
        z = rng.beta(m / 2.0, m / 2.0, size=batch)
        w = (1.0 - (1.0 + b) * z) / (1.0 - (1.0 - b) * z)
        u = rng.random(batch)
        ok = kappa * w + m * np.log(1.0 - x0 * w) - c >= np.log(u)
        acc = w[ok][:need]
        out[filled:filled + acc.size] = acc
        filled += acc.size
    return out


def vmf_mixture(N: int, D: int = 100, n_comp: int = 128, kappa: float = 50.0, seed: int = 42,
                chunk: int = 1 << 17):
    rng = np.random.default_rng(seed)
    mus = rng.normal(size=(n_comp, D))
    mus /= np.linalg.norm(mus, axis=1, keepdims=True)
    weights = rng.dirichlet(np.ones(n_comp))
    labels = rng.choice(n_comp, size=N, p=weights)
    X = np.empty((N, D), np.float32)
    for s in range(0, N, chunk):
        e = min(N, s + chunk)
        mu = mus[labels[s:e]]
        w = _wood_w(rng, kappa, D, e - s)
        v = rng.normal(size=(e - s, D))
        v -= (v * mu).sum(1, keepdims=True) * mu
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        X[s:e] = (w[:, None] * mu + np.sqrt(np.clip(1.0 - w * w, 0.0, None))[:, None] * v)
    return X, labels
