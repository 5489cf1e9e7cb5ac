"""The surrogate MLP's CPU oracle, pinned by finite differences, and the GPU
kernels' gradients against the oracle."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO

SIZES = [8, 128, 128, 128, 3]


def batch(n, seed=1):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1, 1, (n, SIZES[0]))
    T = np.stack([np.sin(2 * X[:, 0]) * X[:, 1], np.cos(X[:, 2] + X[:, 3]), X[:, 4] * X[:, 5]], 1)
    return X, T


def test_oracle_gradient_matches_finite_differences():
    sizes = [5, 7, 6, 2]
    rng = np.random.default_rng(3)
    p = MO.glorot(sizes, seed=2) + rng.normal(0, 0.05, sum((sizes[i] + 1) * sizes[i + 1] for i in range(3)))
    X = rng.uniform(-1, 1, (11, 5))
    T = rng.normal(0, 1, (11, 2))
    g, _ = MO.gradient(p, sizes, X, T)
    idx = np.arange(g.size)
    fd = MO.finite_difference(p, sizes, X, T, idx)
    assert np.max(np.abs(fd - g)) < 1e-8 * max(1.0, np.max(np.abs(g)))


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_oracle():
    from volcanor_gb300 import lib
    net = lib.Mlp(SIZES, seed=7)
    rng = np.random.default_rng(5)
    p = net.get_params().astype(np.float64)
    p += rng.normal(0, 0.02, p.size)  # nonzero biases too
    net.set_params(p)
    p32 = net.get_params().astype(np.float64)
    X, T = batch(700)
    # the FP32 CUDA-core forward pass (the arithmetic of training); the BF16
    # tensor-core pass has its own bound in test_gpu_mlp_tc.py
    net.set_inference(lib.Mlp.INFER_FP32)
    Y = net.forward(X)
    Yo = MO.forward(p32, SIZES, X.astype(np.float32))
    assert np.max(np.abs(Y - Yo)) < 1e-5 * max(1.0, np.max(np.abs(Yo)))
    g, loss = net.gradient(X, T)
    go, losso = MO.gradient(p32, SIZES, X.astype(np.float32), T.astype(np.float32))
    assert abs(loss - losso) <= 1e-5 * losso
    # FP32 kernels vs FP64 oracle: norm-wise and element-wise
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    assert np.max(np.abs(g - go)) <= 1e-4 * np.max(np.abs(go))
    # reproducible: the same call gives the same bits
    g2, _ = net.gradient(X, T)
    assert np.array_equal(g, g2)


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_function():
    from volcanor_gb300 import lib
    net = lib.Mlp(SIZES, seed=0)
    X, T = batch(8192, seed=2)
    Xv, Tv = batch(2048, seed=3)
    l0 = float(np.mean((net.forward(Xv) - Tv) ** 2))
    net.train(X, T, batch=512, iters=1500, lr=2e-3)
    l1 = float(np.mean((net.forward(Xv) - Tv) ** 2))
    print("validation loss ratio", l1 / l0)
    # the same network, data and schedule in PyTorch reach about 1e-3
    assert l1 < 0.005 * l0


def test_bf16_rounding():
    """Round to nearest, ties to even, at BF16's 8-bit significand."""
    one = 1.0
    assert MO.bf16(one) == 1.0
    assert MO.bf16(1 + 2 ** -8) == 1.0                # halfway, even below
    assert MO.bf16(1 + 3 * 2 ** -8) == 1 + 2 ** -6    # halfway, even above
    assert MO.bf16(1 + 2 ** -8 + 2 ** -12) == 1 + 2 ** -7
    assert MO.bf16(-3.0) == -3.0
    x = np.random.default_rng(0).normal(0, 10, 10000).astype(np.float32)
    r = MO.bf16(x)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)
    torch = pytest.importorskip("torch")
    assert np.array_equal(r, torch.from_numpy(x).to(torch.bfloat16).float().numpy().astype(np.float64))
