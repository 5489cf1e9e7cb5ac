"""TEST INFRASTRUCTURE ONLY -- the CPU oracle of the surrogate's MLP.

FP64 numpy restatement of the network the library trains on the GPU
(volcanor_gb300/csrc/mlp.cu): linear layers W_l (out x in, row major) + b_l,
tanh on every layer but the last, loss = mean over all outputs of the batch
of (y - t)^2.  The reference has no learned component; this oracle is pinned
by central finite differences of its own loss (tests/test_mlp_oracle.py).
Only tests may import it.
"""
import numpy as np


def unpack(p, sizes):
    p = np.asarray(p, dtype=np.float64)
    Ws, bs, o = [], [], 0
    for l in range(len(sizes) - 1):
        n_in, n_out = sizes[l], sizes[l + 1]
        Ws.append(p[o:o + n_in * n_out].reshape(n_out, n_in))
        o += n_in * n_out
        bs.append(p[o:o + n_out])
        o += n_out
    assert o == p.size
    return Ws, bs


def forward(p, sizes, X, keep=False):
    Ws, bs = unpack(p, sizes)
    H = [np.asarray(X, dtype=np.float64)]
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = H[-1] @ W.T + b
        H.append(Z if l == len(Ws) - 1 else np.tanh(Z))
    return H if keep else H[-1]


def bf16(x):
    """Rounds to the nearest BF16 value (ties to even), returned as float64:
    the top 16 bits of the float32 after adding the rounding bias."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(p, sizes, X):
    """The tensor-core inference arithmetic: weights, inputs and every hidden
    activation rounded to BF16, products summed exactly (FP64 here, FP32 on
    the GPU), FP32 biases, tanh before the rounding."""
    Ws, bs = unpack(np.asarray(p, dtype=np.float32).astype(np.float64), sizes)
    H = bf16(X)
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = H @ bf16(W).T + b
        H = Z if l == len(Ws) - 1 else bf16(np.tanh(Z))
    return H


def loss(p, sizes, X, T):
    Y = forward(p, sizes, X)
    return float(np.mean((Y - np.asarray(T, dtype=np.float64)) ** 2))


def gradient(p, sizes, X, T):
    """Back-propagation of the batch MSE; returns (gradient in the parameter
    layout, loss)."""
    Ws, _ = unpack(p, sizes)
    H = forward(p, sizes, X, keep=True)
    T = np.asarray(T, dtype=np.float64)
    n = T.size
    dZ = 2.0 * (H[-1] - T) / n
    grads = []
    for l in range(len(Ws) - 1, -1, -1):
        if l < len(Ws) - 1:
            dZ = dZ * (1.0 - H[l + 1] ** 2)
        grads.append((dZ.T @ H[l], dZ.sum(0)))
        dZ = dZ @ Ws[l]
    out = []
    for dW, db in reversed(grads):
        out.append(dW.ravel())
        out.append(db)
    return np.concatenate(out), float(np.mean((H[-1] - T) ** 2))


def finite_difference(p, sizes, X, T, idx, h=1e-6):
    p = np.asarray(p, dtype=np.float64).copy()
    g = []
    for i in idx:
        a = p[i]
        p[i] = a + h
        lp = loss(p, sizes, X, T)
        p[i] = a - h
        lm = loss(p, sizes, X, T)
        p[i] = a
        g.append((lp - lm) / (2 * h))
    return np.array(g)


def glorot(sizes, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for l in range(len(sizes) - 1):
        a = np.sqrt(6.0 / (sizes[l] + sizes[l + 1]))
        out.append(rng.uniform(-a, a, sizes[l + 1] * sizes[l]))
        out.append(np.zeros(sizes[l + 1]))
    return np.concatenate(out)
