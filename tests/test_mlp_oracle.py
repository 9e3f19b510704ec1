"""The NumPy MLP oracle's gradients against central finite differences (pins
the checker of the library's training kernels)."""
import numpy as np


def test_oracle_gradients_by_finite_differences():
    import mlp_oracle
    dims = [3, 5, 4, 2]
    rng = np.random.default_rng(0)
    p = rng.normal(size=sum(a * b + b for a, b in zip(dims[:-1], dims[1:])))
    X, T = rng.normal(size=(6, 3)), rng.normal(size=(6, 2))
    M = (rng.random((6, 2)) > 0.3).astype(float)
    _, g = mlp_oracle.loss_and_grads(p, dims, X, T, M)
    h = 1e-6
    fd = np.array([(mlp_oracle.loss_and_grads(p + e, dims, X, T, M)[0] -
                    mlp_oracle.loss_and_grads(p - e, dims, X, T, M)[0]) / (2 * h) for e in np.eye(len(p)) * h])
    assert np.abs(fd - g).max() <= 1e-7 * np.abs(g).max()
