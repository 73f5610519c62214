"""The BF16 tensor-core MLP kernels against the CPU oracle: forward
predictions and every parameter gradient agree within a relative
Frobenius error of 2e-2 (bf16 rounding of activations makes bit-exact
agreement impossible; the tolerance is stated here)."""
import numpy as np
import pytest
import torch

from oracle import mlp_oracle as M
from poyd_gb300 import mlp

pytestmark = pytest.mark.gpu
TOL = 2e-2


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)


@pytest.mark.parametrize("batch", [64, 250, 1024])
def test_forward_backward_match_oracle(batch):
    net = mlp.MLP(seed=3)
    rng = np.random.default_rng(batch)
    X = rng.normal(size=(batch, 32)).astype(np.float32)
    t = rng.normal(size=batch).astype(np.float32)
    Xd = torch.from_numpy(X).cuda()
    y = net.forward(Xd.to(torch.bfloat16)).cpu().numpy()
    loss, gW, gb = net.backward(torch.from_numpy(t).cuda())
    st = net.state()
    y_ref, loss_ref, gW_ref, gb_ref = M.backward(st["W"], st["b"], X, t)
    assert rel(y, y_ref) < TOL
    assert abs(float(loss.item()) - loss_ref) <= TOL * max(loss_ref, 1e-6)
    for i in range(4):
        assert rel(gW[i].cpu().numpy().reshape(gW_ref[i].shape), gW_ref[i]) < TOL, i
        assert rel(gb[i].cpu().numpy().reshape(-1), gb_ref[i].reshape(-1)) < TOL, i


def test_training_reduces_loss():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(16384, 32)).astype(np.float32)
    w = rng.normal(size=32).astype(np.float32)
    y = (np.tanh(X @ w / 4) * 3 + 0.5 * X[:, 0] * X[:, 1]).astype(np.float32)
    net = mlp.MLP(seed=1)
    Xd, yd = torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()
    p0 = net.predict(Xd)
    l0 = float(((p0 - yd) ** 2).mean().item())
    net.fit(Xd, yd, epochs=8, batch=1024, lr=2e-3)
    p1 = net.predict(Xd)
    l1 = float(((p1 - yd) ** 2).mean().item())
    assert l1 < 0.25 * l0, (l0, l1)


@pytest.mark.parametrize("rows", [1, 63, 64, 1000, 70001])
def test_fused_inference_equals_layer_by_layer(rows):
    """poyd_mlp_forward (one launch, activations in shared memory) gives
    forward()'s predictions bit for bit, also for partial 64-row tiles, and
    after training steps have moved the weights."""
    net = mlp.MLP(seed=5)
    g = torch.Generator(device="cpu").manual_seed(rows)
    X = torch.randn((rows, 32), generator=g).cuda()
    if rows >= 1000:
        net.fit(X[:4096], torch.randn(min(rows, 4096), generator=g).cuda(), epochs=1, batch=512)
    want = torch.cat([net.forward(X[s:s + 65536].to(torch.bfloat16).contiguous()).clone()
                      for s in range(0, rows, 65536)])
    got = net.predict(X)
    assert torch.equal(want, got)
