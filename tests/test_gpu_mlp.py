"""Surrogate MLP kernels (tcgen05) against the CPU FP64 reference (needs a GB300).

Training (the gradient) keeps BF16 activations and weights; the reference
(oracle/mlp_ref.py) rounds to BF16 at the same points, so what remains is FP32
accumulation order and the hardware tanh: gradients per tensor within 3e-2
relative L2 norm with cosine similarity >= 0.999.  Inference runs every layer
with F16 operands and the GELU on packed halves: its outputs are compared with
the unrounded FP64 reference at 5e-3 of max(1, |y|) (F16 keeps 11 significant
bits), and with the training forward at the BF16 level.
"""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu

MEAN = np.array([0.6, 6.0, -1.8, -1.8, -0.05, -2.3, -7.0], dtype=np.float32)
STD = np.array([0.5, 0.7, 0.5, 0.5, 0.02, 0.8, 1.2], dtype=np.float32)


def raw_samples(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(300, 3800, n), 10 ** rng.uniform(4.7, 7, n), rng.uniform(0, .05, n),
                     rng.uniform(0, .05, n), rng.uniform(.85, .95, n), rng.uniform(0, .02, n),
                     10 ** rng.uniform(-9, -5, n)], 1).astype(np.float32)


@pytest.fixture(scope="module")
def net():
    from rocketcombustor_gb300 import surrogate
    m = surrogate.MLP(seed=3)
    m.set_norm(MEAN, STD)
    return m


def test_fused_forward_matches_reference(net):
    import torch
    x = raw_samples(1000, 1)  # not a multiple of 128: a partial last tile
    y = net.forward(torch.tensor(x, device="cuda")).cpu().numpy()
    yr, _ = mlp_ref.forward(net.get_params(), x, MEAN, STD, bf=False)
    assert np.abs(y - yr).max() <= 5e-3 * max(1.0, np.abs(yr).max()), np.abs(y - yr).max()
    yb, _ = mlp_ref.forward(net.get_params(), x, MEAN, STD, bf=True)
    assert np.abs(y - yb).max() <= 1e-2 * max(1.0, np.abs(yb).max()), np.abs(y - yb).max()


def test_gradient_matches_reference(net):
    import torch
    from rocketcombustor_gb300 import surrogate
    n = 512
    x = raw_samples(n, 2)
    t = np.random.default_rng(3).normal(size=(n, 4)).astype(np.float32)
    g, loss = net.gradient(torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda"))
    g = g.cpu().numpy().astype(np.float64)
    lr, gr, _ = mlp_ref.loss_and_grad(net.get_params(), x, t, MEAN, STD, bf=True)
    assert loss == pytest.approx(lr, rel=1e-3)
    for name, (sl, _) in surrogate.param_slices().items():
        a, b = g[sl], gr[sl]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel <= 3e-2 and cos >= 0.999, (name, rel, cos)


def test_training_and_inference_paths_agree(net):
    import torch
    n = 256
    x = torch.tensor(raw_samples(n, 4), device="cuda")
    y = net.forward(x)
    _, loss = net.gradient(x, torch.zeros((n, 4), device="cuda"))
    # the training forward's BF16 activations against the inference's F16 ones
    assert loss == pytest.approx(float((y.double() ** 2).mean()), rel=2e-2)


def test_gradient_is_reproducible(net):
    import torch
    x = torch.tensor(raw_samples(384, 5), device="cuda")
    t = torch.ones((384, 4), device="cuda")
    g1, _ = net.gradient(x, t)
    g2, _ = net.gradient(x, t)
    assert torch.equal(g1, g2)


def test_training_reduces_the_loss():
    import torch
    from rocketcombustor_gb300 import surrogate
    m = surrogate.MLP(seed=4)
    m.set_norm(MEAN, STD)
    x = torch.tensor(raw_samples(8192, 6), device="cuda")
    f = (x[:, 0:1] - 2000) / 1000 * 0.5
    t = torch.cat([torch.tanh(f), f * f, torch.sin(3 * f), 0 * f + 1], 1).contiguous()
    hist = m.train(x, t, steps=300, batch=2048, lr=3e-3, lr_end=3e-4, log_every=50)
    assert hist[-1][1] < 0.05 * hist[0][1], hist


def test_training_is_reproducible_and_checks_its_arguments():
    """rc_mlp_train twice from the same parameters and seed gives the same
    parameters bit for bit (every gradient reduction has a fixed order, the
    weight-gradient branch on its own stream included); a batch that is not a
    multiple of 128 is refused."""
    import ctypes

    import torch
    from rocketcombustor_gb300 import RcError, surrogate
    from rocketcombustor_gb300 import load
    x = torch.tensor(raw_samples(4096, 8), device="cuda")
    t = torch.rand(4096, 4, device="cuda", generator=torch.Generator(device="cuda").manual_seed(2))
    params = []
    for _ in range(2):
        m = surrogate.MLP(seed=5)
        m.set_norm(MEAN, STD)
        m.train(x, t, steps=40, batch=1024, lr=3e-3, lr_end=3e-4, seed=11)
        params.append(m.get_params())
        m.close()
    assert np.array_equal(params[0], params[1])
    m = surrogate.MLP(seed=5)
    st = load().rc_mlp_train(m.handle, x.data_ptr(), t.data_ptr(), 4096, 10, 1000, 1e-3, 1e-4, 0.9, 0.999, 1e-8, 0,
                             None, ctypes.c_void_p(0))
    assert st != 0
    with pytest.raises(RcError):
        m._check(st)
    m.close()
