"""The closure's tensor-core kernels against the CPU restatement
(oracle/mlp_ref.py): forward pass, loss and gradients, and training."""
import numpy as np
import pytest

from des_gb300 import abi, closure
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _as_dict(net):
    return {k: net.arr(k).astype(np.float64) for k in ("w1", "b1", "w2", "b2", "w3", "b3")}


def _net(seed):
    rng = np.random.default_rng(seed)
    ref = mlp_ref.random_net(rng)
    net = abi.Mlp()
    for k, v in ref.items():
        net.arr(k)[:] = v
    net.arr("in_scale")[:] = 1
    net.arr("out_scale")[:] = 1
    net.tol = 1e-3
    return net


def _data(seed, n):
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 16), np.float32)
    x[:, :14] = rng.normal(0, 1, (n, 14))
    y = np.zeros((n, 8), np.float32)
    y[:, :7] = rng.normal(0, 1, (n, 7))
    return x, y


# 38,989 samples: 305 tiles, the last one ragged, so that the persistent CTAs
# (one per multiprocessor) take several tiles each
@pytest.mark.parametrize("n", [1, 17, 64, 1000, 38989])
def test_forward_matches_cpu(gpu, n):
    net = _net(1)
    x, _ = _data(2, n)
    y = closure.forward(net, x)
    ref, _ = mlp_ref.forward(_as_dict(net), x, bf16=True)
    err = np.linalg.norm(y[:, :7] - ref[:, :7]) / np.linalg.norm(ref[:, :7])
    assert err < 1e-3, err
    assert np.all(y[:, 7] == 0)


@pytest.mark.parametrize("n", [64, 200, 4096, 38989])
def test_gradients_match_cpu(gpu, n):
    net = _net(3)
    x, t = _data(4, n)
    loss, g = closure.loss_grad(net, x, t)
    lref, gref = mlp_ref.loss_grad(_as_dict(net), x, t, bf16=True)
    _, g64 = mlp_ref.loss_grad(_as_dict(net), x, t, bf16=False)
    assert loss == pytest.approx(lref, rel=1e-4)
    for k in ("w1", "b1", "w2", "b2", "w3", "b3"):
        gk = g.arr(k)
        e16 = np.linalg.norm(gk - gref[k]) / np.linalg.norm(gref[k])
        e64 = np.linalg.norm(gk - g64[k]) / np.linalg.norm(g64[k])
        assert e16 < 1e-2, (k, e16)     # same BF16 operands, FP32 vs FP64 sums
        assert e64 < 5e-2, (k, e64)     # the exact gradient, BF16 operands aside
    assert np.all(g.arr("w1")[:, 14:] == 0)
    assert np.all(g.arr("w3")[7] == 0) and g.arr("b3")[7] == 0


def test_training_fits_a_teacher(gpu):
    """Adam on the GPU fits data made by another network to a small loss."""
    teacher = _net(5)
    x, _ = _data(6, 1 << 15)
    t = closure.forward(teacher, x)
    student = _net(7)
    loss0, _ = closure.loss_grad(student, x, t)
    trace = closure.train(student, x, t, epochs=30, batch=1024, lr=2e-3, seed=8)
    loss1, _ = closure.loss_grad(student, x, t)
    assert np.isfinite(trace).all()
    assert loss1 < 0.05 * loss0, (loss0, loss1)
