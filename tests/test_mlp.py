"""The learned-sampler network: the CPU restatement against finite
differences (pins it), then the tensor-core kernels against the restatement:
forward values, one-batch gradients, and a training run that fits a smooth
function of (a, b)."""
import numpy as np
import pytest

from oracle import mlp_ref


def _params(seed=0):
    rng = np.random.default_rng(seed)
    H = mlp_ref.H
    p = np.zeros(mlp_ref.NPARAM)
    p[mlp_ref.oW1:mlp_ref.ob1] = rng.uniform(-1.7, 1.7, 2 * H)
    p[mlp_ref.ob1:mlp_ref.oW2] = rng.uniform(-0.1, 0.1, H)
    p[mlp_ref.oW2:mlp_ref.ob2] = rng.uniform(-0.2, 0.2, H * H)
    p[mlp_ref.ob2:mlp_ref.oW3] = rng.uniform(-0.1, 0.1, H)
    p[mlp_ref.oW3:mlp_ref.ob3] = rng.uniform(-0.2, 0.2, H * H)
    p[mlp_ref.ob3:mlp_ref.ow4] = rng.uniform(-0.1, 0.1, H)
    p[mlp_ref.ow4:mlp_ref.ob4] = rng.uniform(-0.15, 0.15, H)
    p[mlp_ref.ob4] = 0.05
    return p.astype(np.float32).astype(np.float64)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3])
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == 1.0 + 2 ** -7                # rounds up
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(1)
    x = rng.uniform(-1, 1, (16, 2))
    t = rng.normal(size=16)
    g, _ = mlp_ref.gradient(p, x, t, emulate=False)
    idx = np.concatenate([rng.choice(np.arange(s, e), 6, replace=False) for s, e in
                          ((mlp_ref.oW1, mlp_ref.ob1), (mlp_ref.ob1, mlp_ref.oW2), (mlp_ref.oW2, mlp_ref.ob2),
                           (mlp_ref.ob2, mlp_ref.oW3), (mlp_ref.oW3, mlp_ref.ob3), (mlp_ref.ob3, mlp_ref.ow4),
                           (mlp_ref.ow4, mlp_ref.ob4))] + [np.array([mlp_ref.ob4])])
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h; pm[i] -= h
        lp = np.mean((mlp_ref.forward(pp, x, False)[0] - t) ** 2)
        lm = np.mean((mlp_ref.forward(pm, x, False)[0] - t) ** 2)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (i, fd, g[i])


@pytest.fixture(scope="module")
def net(pcl, gpu):
    n = pcl.SamplerNet(seed=3)
    n.set_params(_params(2).astype(np.float32))
    yield n
    n.close()


@pytest.mark.gpu
def test_forward_matches_oracle(pcl, net):
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (1000, 2)).astype(np.float32)   # 8 tiles, last one ragged
    y = net.forward(x)
    yr, _ = mlp_ref.forward(net.params(), x, emulate=True)
    scale = np.abs(yr).max()
    # FP32 accumulation on the device vs Float64 here; the same BF16 roundings
    assert np.max(np.abs(y - yr)) <= 2e-3 * scale + 1e-6, np.max(np.abs(y - yr)) / scale


@pytest.mark.gpu
def test_gradient_matches_oracle(pcl, net):
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (640, 2)).astype(np.float32)
    t = rng.normal(size=640).astype(np.float32)
    g, loss = net.gradient(x, t)
    gr, lr_ = mlp_ref.gradient(net.params(), x, t, emulate=True)
    assert abs(loss - lr_) <= 1e-4 * lr_
    blocks = {"W1": (mlp_ref.oW1, mlp_ref.ob1), "b1": (mlp_ref.ob1, mlp_ref.oW2), "W2": (mlp_ref.oW2, mlp_ref.ob2),
              "b2": (mlp_ref.ob2, mlp_ref.oW3), "W3": (mlp_ref.oW3, mlp_ref.ob3), "b3": (mlp_ref.ob3, mlp_ref.ow4),
              "w4": (mlp_ref.ow4, mlp_ref.ob4), "b4": (mlp_ref.ob4, mlp_ref.ob4 + 1)}
    for name, (a, b) in blocks.items():
        d = np.linalg.norm(g[a:b] - gr[a:b]) / max(np.linalg.norm(gr[a:b]), 1e-30)
        # BF16 roundings of dz3 / dz2 / h1 / h2 can land on the other side of a
        # rounding boundary (FP32 device vs Float64 here): ~1e-3 relative
        assert d < 1e-2, (name, d)


@pytest.mark.gpu
def test_training_fits_smooth_function(pcl, gpu):
    rng = np.random.default_rng(6)
    x = rng.uniform(-1, 1, (200_000, 2)).astype(np.float32)
    t = (np.sin(2.0 * x[:, 0]) * 0.5 + x[:, 1] ** 3 + 0.3 * x[:, 0] * x[:, 1]).astype(np.float32)
    n = pcl.SamplerNet(seed=7)
    y0 = n.forward(x[:4096])
    l0 = float(np.mean((y0 - t[:4096]) ** 2))
    loss = n.train(x, t, steps=1500, batch=4096, lr=2e-3, seed=1)
    y1 = n.forward(x[:4096])
    l1 = float(np.mean((y1 - t[:4096]) ** 2))
    n.close()
    assert l1 < 2e-3 and l1 < 0.01 * l0, (l0, l1, loss)
