"""Tensor-core inference of the surrogate MLP (tcgen05, BF16 operands, FP32
accumulation, all layers in one kernel) against the oracle's BF16 forward
pass and against the FP32 CUDA-core forward pass."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO
from volcanor_gb300 import lib

pytestmark = pytest.mark.gpu

SIZES = [12, 128, 128, 128, 3]  # the surrogate's default network


def _net(sizes, seed):
    net = lib.Mlp(sizes, seed=seed)
    rng = np.random.default_rng(seed)
    p = net.get_params()
    p = p + rng.normal(0, 0.05, p.size).astype(np.float32)  # nonzero biases as after training
    net.set_params(p)
    return net, p


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40000])
def test_tensor_core_forward_matches_bf16_oracle(n):
    net, p = _net(SIZES, 5)
    assert net.inference == lib.Mlp.INFER_TENSOR_CORES
    rng = np.random.default_rng(n)
    X = rng.uniform(-1.5, 1.5, (n, SIZES[0])).astype(np.float32)
    Y = net.forward(X)
    R = MO.forward_bf16(p, SIZES, X)
    scale = np.sqrt(np.mean(R ** 2))
    # same rounding points: the outputs agree to FP32 summation rounding
    # except where a hidden activation falls on the other side of a BF16
    # rounding boundary (one BF16 unit, 2^-8 relative, of one activation)
    d = np.abs(Y - R)
    assert np.max(d) <= 1e-2 * scale
    assert np.median(d) <= 1e-6 * scale
    assert np.mean(d > 1e-5 * scale) <= 0.05
    net.set_inference(lib.Mlp.INFER_FP32)
    Y32 = net.forward(X)
    F = MO.forward(p, SIZES, X)
    assert np.max(np.abs(Y32 - F)) <= 1e-4 * scale
    # BF16 inference against exact FP32-parameter inference
    assert np.sqrt(np.mean((Y - F) ** 2)) <= 2e-2 * scale


@pytest.mark.parametrize("sizes", [[5, 16, 3], [12, 64, 64, 3], [20, 256, 48, 7], [12, 128, 128, 128, 128, 128, 3]])
def test_tensor_core_forward_other_shapes(sizes):
    net, p = _net(sizes, 11)
    X = np.random.default_rng(2).uniform(-1, 1, (777, sizes[0])).astype(np.float32)
    Y = net.forward(X)
    R = MO.forward_bf16(p, sizes, X)
    scale = np.sqrt(np.mean(R ** 2))
    d = np.abs(Y - R)
    assert np.max(d) <= 1e-2 * scale and np.median(d) <= 1e-6 * scale


def test_tensor_core_forward_after_training_step():
    """The packed BF16 image follows the parameters after an update."""
    net, _ = _net(SIZES, 7)
    rng = np.random.default_rng(4)
    X = rng.uniform(-1, 1, (512, 12)).astype(np.float32)
    T = rng.normal(0, 1, (512, 3)).astype(np.float32)
    y0 = net.forward(X)
    net.train(X, T, batch=256, iters=5, lr=1e-2)
    p = net.get_params()
    y1 = net.forward(X)
    assert not np.array_equal(y0, y1)
    R = MO.forward_bf16(p, SIZES, X)
    d = np.abs(y1 - R)
    scale = np.sqrt(np.mean(R ** 2))
    assert np.max(d) <= 1e-2 * scale and np.median(d) <= 1e-6 * scale


def test_wide_network_keeps_fp32_inference():
    net = lib.Mlp([12, 512, 3], seed=1)
    assert net.inference == lib.Mlp.INFER_FP32
    with pytest.raises(lib.VlmError):
        net.set_inference(lib.Mlp.INFER_TENSOR_CORES)
