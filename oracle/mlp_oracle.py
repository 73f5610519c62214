"""CPU oracle of the join-proposal MLP (TEST INFRASTRUCTURE ONLY): numpy
float32 forward/backward with the same BF16 rounding points as the CUDA
kernels (inputs, weights and hidden activations rounded to bf16, products
accumulated in fp32)."""
import numpy as np

DIMS = (32, 256, 256, 128, 1)


def bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even), kept as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def forward(W, b, X):
    a = bf16(X)
    H = []
    for i in range(3):
        z = a @ bf16(W[i]) + b[i]
        a = bf16(np.maximum(z, 0.0))
        H.append(a)
    y = a @ bf16(W[3]).reshape(-1) + b[3][0]
    return y.astype(np.float32), H


def backward(W, b, X, t):
    y, H = forward(W, b, X)
    B = X.shape[0]
    dy = (2.0 * (y - t) / B).astype(np.float32)
    gW, gb = [None] * 4, [None] * 4
    w4 = bf16(W[3]).reshape(-1)
    gW[3] = (H[2].T @ dy).reshape(-1, 1).astype(np.float32)
    gb[3] = np.array([dy.sum()], np.float32)
    dZ = bf16(np.where(H[2] > 0, dy[:, None] * w4[None, :], 0.0))
    for i in (2, 1, 0):
        a_in = bf16(X) if i == 0 else H[i - 1]
        gW[i] = (a_in.T @ dZ).astype(np.float32)
        gb[i] = dZ.sum(axis=0).astype(np.float32)
        if i > 0:
            dH = bf16(dZ @ bf16(W[i]).T)
            dZ = np.where(H[i - 1] > 0, dH, 0.0).astype(np.float32)
    loss = float(np.mean((y - t) ** 2))
    return y, loss, gW, gb
