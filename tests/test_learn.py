"""The learned warm start's network: tcgen05 forward and gradient kernels
against the CPU oracle (oracle/mlp_oracle.py), and the oracle's own backward
pass against finite differences."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(mo.N_PARAMS, np.float32)
    p[mo.OFF_W1:mo.OFF_B1] = rng.uniform(-1, 1, mo.N_FEAT * mo.N_HID) * np.sqrt(6 / mo.N_FEAT)
    p[mo.OFF_B1:mo.OFF_W2] = rng.uniform(-0.1, 0.1, mo.N_HID)
    p[mo.OFF_W2:mo.OFF_B2] = rng.uniform(-1, 1, mo.N_HID * mo.N_HID) * np.sqrt(6 / mo.N_HID)
    p[mo.OFF_B2:mo.OFF_W3] = rng.uniform(-0.1, 0.1, mo.N_HID)
    p[mo.OFF_W3:mo.OFF_B3] = rng.uniform(-1, 1, mo.N_HID * mo.N_OUT) * 0.2
    p[mo.OFF_B3:] = rng.uniform(-0.1, 0.1, mo.N_OUT)
    return p


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = mo.bf16(rng.normal(0, 1.5, (n, mo.N_FEAT)).astype(np.float32))
    x[:, 0] = 1.0
    t = rng.normal(0, 1, (n, mo.N_OUT)).astype(np.float32)
    return x, t


def test_oracle_gradient_matches_finite_differences():
    p = _params(1).astype(np.float64)
    x, t = _data(37, 2)
    g = mo.grad_exact(p, x, t)
    rng = np.random.default_rng(3)
    idx = rng.choice(mo.N_PARAMS, 60, replace=False)
    h = 1e-6
    for k in idx:
        e = np.zeros_like(p)
        e[k] = h
        fd = (mo.loss_exact(p + e, x, t) - mo.loss_exact(p - e, x, t)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), (k, fd, g[k])


def test_oracle_rounded_gradient_tracks_exact_gradient():
    # the bf16 operand roundings of the kernels leave the gradient's
    # direction intact
    p = _params(4).astype(np.float64)
    x, t = _data(300, 5)
    _, g = mo.loss_and_grad(p, x, t)
    ge = mo.grad_exact(p, x, t)
    cos = g @ ge / (np.linalg.norm(g) * np.linalg.norm(ge))
    assert cos > 0.999


def _block_errors(g, ref):
    out = {}
    for name, a, b in (("W1", mo.OFF_W1, mo.OFF_B1), ("b1", mo.OFF_B1, mo.OFF_W2), ("W2", mo.OFF_W2, mo.OFF_B2),
                       ("b2", mo.OFF_B2, mo.OFF_W3), ("W3", mo.OFF_W3, mo.OFF_B3), ("b3", mo.OFF_B3, mo.N_PARAMS)):
        d = np.linalg.norm(g[a:b] - ref[a:b]) / max(np.linalg.norm(ref[a:b]), 1e-30)
        out[name] = float(d)
    return out


@pytest.fixture
def mlp():
    import granular_gpu_gb300 as gg
    m = gg.Mlp(device=0, seed=7)
    yield m
    m.close()


def _dev(a, dtype=None):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 128, 1000, 70_000])
def test_mlp_forward_matches_oracle(mlp, n):
    import torch
    p = _params(11)
    mlp.set_params(p)
    x, _ = _data(n, 12)
    xd = _dev(mo.bf16_bits(x).view(np.int16))
    yd = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    mlp.forward(xd, yd, n)
    y = yd.cpu().numpy()
    ref = mo.forward(p, x)
    err = np.abs(y - ref) / (np.abs(ref) + 0.05)
    assert err.max() < 2e-2, f"max relative error {err.max():.3g}"
    assert np.abs(y - ref).mean() < 2e-3 * (np.abs(ref).mean() + 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [128, 777, 20_000])
def test_mlp_gradient_matches_oracle(mlp, n):
    p = _params(21)
    mlp.set_params(p)
    x, t = _data(n, 22)
    xd = _dev(mo.bf16_bits(x).view(np.int16))
    td = _dev(t.astype(np.float32))
    g, loss = mlp.gradient(xd, td, n)
    lref, gref = mo.loss_and_grad(p, x, t)
    assert abs(loss - lref) <= 1e-3 * lref
    errs = _block_errors(g.astype(np.float64), gref)
    assert max(errs.values()) < 2e-2, errs


@pytest.mark.gpu
def test_mlp_training_reduces_loss(mlp):
    # a smooth target the network can represent: a random linear map of
    # the features through a ReLU
    rng = np.random.default_rng(31)
    n = 8192
    x, _ = _data(n, 32)
    A = rng.normal(0, 0.3, (mo.N_FEAT, mo.N_OUT))
    t = (np.maximum(x @ A, 0) - 0.5).astype(np.float32)
    xd = _dev(mo.bf16_bits(x).view(np.int16))
    td = _dev(t)
    first = mlp.train_step(xd, td, n, lr=3e-3)
    for _ in range(300):
        last = mlp.train_step(xd, td, n, lr=3e-3)
    assert last < 0.1 * first, (first, last)
    # the trained parameters read back and the loss agrees with the oracle
    lref, _ = mo.loss_and_grad(mlp.get_params(), x, t)
    _, loss = mlp.gradient(xd, td, n)
    assert abs(loss - lref) <= 2e-3 * lref + 1e-7
