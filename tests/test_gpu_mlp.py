"""The library's MLP training kernels against the FP64 NumPy oracle: forward
pass, loss and every gradient; then a short training run that must fit; and
the BF16 tensor-core inference against the oracle with the same BF16
roundings."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(rng, n, dims):
    X = rng.normal(size=(n, dims[0])).astype(np.float32)
    T = rng.normal(size=(n, dims[-1])).astype(np.float32)
    M = (rng.random((n, dims[-1])) > 0.2).astype(np.float32)
    return X, T, M


@pytest.mark.parametrize("dims,n", [([7, 33, 20, 5], 50), ([96, 256, 256, 256, 256, 128], 300)])
def test_gradients_match_oracle(lib, cuda_device, dims, n):
    import torch
    import mlp_oracle
    from pyblastafterglowmag_gb300.mlp import MLP
    rng = np.random.default_rng(1)
    net = MLP(dims, cuda_device)
    p0 = net.init_params(seed=2)
    X, T, M = _data(rng, n, dims)
    dev = torch.device("cuda", cuda_device)
    dX, dT, dM = (torch.from_numpy(a).to(dev) for a in (X, T, M))
    dY = torch.zeros((n, dims[-1]), dtype=torch.float32, device=dev)
    net.forward(n, dX.data_ptr(), dY.data_ptr())
    Y_ref, _, _ = mlp_oracle.forward(p0, dims, X)
    np.testing.assert_allclose(dY.cpu().numpy(), Y_ref, rtol=2e-4, atol=2e-4 * np.abs(Y_ref).max())
    loss = net.train_step(n, dX.data_ptr(), dT.data_ptr(), dM.data_ptr(), update=False)
    loss_ref, g_ref = mlp_oracle.loss_and_grads(p0, dims, X, T, M)
    _, g = net.params(grads=True)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    # per-tensor relative error of the gradients
    o = 0
    for din, dout in zip(dims[:-1], dims[1:]):
        for size in (din * dout, dout):
            a, b = g[o:o + size].astype(np.float64), g_ref[o:o + size]
            assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-12, (din, dout, size)
            o += size


def test_training_fits(lib, cuda_device):
    import torch
    from pyblastafterglowmag_gb300.mlp import MLP
    rng = np.random.default_rng(3)
    dims = [4, 64, 64, 2]
    n = 4096
    X = rng.uniform(-1, 1, size=(n, 4)).astype(np.float32)
    T = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], X[:, 2] ** 2 - X[:, 3]], axis=1).astype(np.float32)
    dev = torch.device("cuda", cuda_device)
    dX, dT = torch.from_numpy(X).to(dev), torch.from_numpy(T).to(dev)
    net = MLP(dims, cuda_device)
    net.init_params(seed=4)
    first = net.train_step(n, dX.data_ptr(), dT.data_ptr(), lr=3e-3, update=False)
    for it in range(600):
        last = net.train_step(n, dX.data_ptr(), dT.data_ptr(), lr=3e-3)
    assert last < 0.02 * first, (first, last)


def _bf16(a):
    """Round FP32 values to BF16 (nearest even), kept as FP32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _forward_bf16(params, dims, X):
    """Forward pass with weights and every layer input rounded to BF16, FP64
    accumulation (the tensor-core kernel accumulates in FP32)."""
    o = 0
    H = _bf16(X).astype(np.float64)
    for l, (din, dout) in enumerate(zip(dims[:-1], dims[1:])):
        W = _bf16(params[o:o + din * dout].reshape(dout, din)).astype(np.float64)
        o += din * dout
        b = params[o:o + dout].astype(np.float64)
        o += dout
        Z = H @ W.T + b
        if l < len(dims) - 2:
            Z = Z / (1.0 + np.exp(-Z))
            H = _bf16(Z.astype(np.float32)).astype(np.float64)
        else:
            H = Z
    return H


@pytest.mark.parametrize("dims,n", [([128, 256, 256, 256, 256, 128], 1000), ([64, 96, 32], 130),
                                    ([128, 256, 256, 256, 256, 256], 4096)])
def test_bf16_inference_on_tensor_cores(lib, cuda_device, dims, n):
    import torch
    import mlp_oracle
    from pyblastafterglowmag_gb300.mlp import MLP
    rng = np.random.default_rng(5)
    net = MLP(dims, cuda_device)
    p0 = net.init_params(seed=6)
    X = rng.normal(size=(n, dims[0])).astype(np.float32)
    dev = torch.device("cuda", cuda_device)
    dX = torch.from_numpy(X).to(dev)
    dY = torch.full((n, dims[-1]), float("nan"), dtype=torch.float32, device=dev)
    net.infer(n, dX.data_ptr(), dY.data_ptr())
    Y = dY.cpu().numpy().astype(np.float64)
    ref = _forward_bf16(p0, dims, X)
    # same roundings: differences only from FP32 accumulation order and the
    # occasional activation that rounds to the neighbouring BF16 value
    assert np.linalg.norm(Y - ref) <= 2e-3 * np.linalg.norm(ref)
    Y32, _, _ = mlp_oracle.forward(p0, dims, X)
    # against FP32 inference: the BF16 rounding itself
    assert np.linalg.norm(Y - Y32) <= 3e-2 * np.linalg.norm(Y32)
    # after a parameter change the weights are laid out again
    p1 = p0 * np.float32(0.5)
    net.set_params(p1)
    net.infer(n, dX.data_ptr(), dY.data_ptr())
    ref1 = _forward_bf16(p1, dims, X)
    assert np.linalg.norm(dY.cpu().numpy() - ref1) <= 2e-3 * np.linalg.norm(ref1)


def test_bf16_inference_rejects_unsupported_shapes(lib, cuda_device):
    from pyblastafterglowmag_gb300 import _lib
    from pyblastafterglowmag_gb300.mlp import MLP
    net = MLP([7, 33, 5], cuda_device)
    net.init_params(seed=1)
    with pytest.raises(_lib.PbagError):
        net.infer(4, 0, 0)
