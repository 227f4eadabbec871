"""The U-Net oracle's own checks (CPU): analytic gradients against central
finite differences in float64, bf16 rounding, Adam."""
import numpy as np

from oracle import unet_oracle as U


def _case(seed=0, B=1, H=16, W=16):
    rng = np.random.default_rng(seed)
    th = U.init_params(seed + 1).astype(np.float64)
    layout, n = U.param_layout()
    _, wo, nw, bo, _ = layout[-1]
    th[wo:wo + nw] = rng.standard_normal(nw) * 0.1
    th[bo] = 0.05
    x = rng.standard_normal((B, H, W, 3))
    t = rng.standard_normal((B, H, W))
    m = (rng.random((B, H, W)) > 0.2).astype(np.float64)
    return th, x, t, m


def test_gradient_matches_finite_differences():
    th, x, t, m = _case()
    net = U.Net(th, bf16=False)
    _, dout, _ = U.loss_and_grad(net, x, t, m)
    g = net.backward(dout)
    rng = np.random.default_rng(5)
    layout, n = U.param_layout()
    # two weights and the bias of every layer
    idx = []
    for name, wo, nw, bo, cout in layout:
        idx += [wo + int(rng.integers(nw)), wo + int(rng.integers(nw)), bo]
    for i in idx:
        e = 1e-6
        tp, tm = th.copy(), th.copy()
        tp[i] += e
        tm[i] -= e
        fd = (U.loss_and_grad(U.Net(tp, False), x, t, m)[0] - U.loss_and_grad(U.Net(tm, False), x, t, m)[0]) / (2 * e)
        assert abs(g[i] - fd) <= 1e-5 * max(abs(fd), 1e-3), (i, g[i], fd)


def test_bf16_rounding_is_nearest_even():
    a = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e-39, np.inf], np.float32)
    r = U.to_bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.015625) and r[3] == -2.5 and r[5] == np.inf
    assert (r.view(np.uint32) & 0xFFFF == 0).all()


def test_adam_first_step_moves_by_lr():
    th = np.zeros(4, np.float32)
    g = np.array([1.0, -2.0, 0.5, 0.0], np.float32)
    t, m, v = U.adam(th, np.zeros(4, np.float32), np.zeros(4, np.float32), g, 1, lr=1e-3)
    # the first bias-corrected step is lr * sign(g)
    assert np.allclose(t[:3], -1e-3 * np.sign(g[:3]), rtol=1e-5) and t[3] == 0


def test_untrained_head_returns_zero():
    x = np.random.default_rng(0).standard_normal((1, 16, 16, 3))
    out = U.Net(U.init_params(0), bf16=True).forward(x)
    assert not out.any()


def test_host_init_layout_matches_the_oracle():
    from flowlab_gb300 import warmstart

    th = warmstart.he_init(0)
    assert th.size == U.num_params()
    layout, _ = U.param_layout()
    _, wo, nw, bo, _ = layout[-1]
    assert not th[wo:].any()  # zero head: the untrained network predicts no correction


def test_features_follow_the_engine_normalisation():
    from flowlab_gb300 import warmstart

    rng = np.random.default_rng(0)
    b = rng.standard_normal((8, 8)).astype(np.float32)
    p = rng.standard_normal((8, 8)).astype(np.float32)
    label = np.zeros((8, 8), np.uint8)
    label[0, :] = 2
    x, sb, sp = warmstart.features(b, label, p)
    fl = label == 0
    assert abs(sb - np.sqrt(np.mean(b[fl].astype(np.float64) ** 2))) < 1e-12
    assert np.allclose(x[..., 0][fl], b[fl] / sb, rtol=1e-6) and (x[..., 0][~fl] == 0).all()
    assert (x[..., 1] == fl).all()
    _, sb2, sp2 = warmstart.features(b, label, np.zeros_like(p))
    assert sp2 == sb2
