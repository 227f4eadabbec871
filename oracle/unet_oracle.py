"""CPU oracle of the pressure warm-start U-Net (test infrastructure only).

The reference has no learned part (its warm start is the previous step's
pressure, src/core/pressureSolver.ts:28-30); this network is project-defined
and this file restates it from the definitions of its operations, in numpy:

  input  x0 = (b / s_b, mask, p_prev / s_p)        3 channels, NHWC
  enc0   conv3x3(3->32)+ReLU, conv3x3(32->32)+ReLU             -> s0
  enc1   avgpool2, conv3x3(32->64)+ReLU, conv3x3(64->64)+ReLU  -> s1
  enc2   avgpool2, conv3x3(64->96)+ReLU, conv3x3(96->96)+ReLU  -> s2
  mid    avgpool2, conv3x3(96->128)+ReLU, conv3x3(128->128)+ReLU
  dec2   up2 (nearest), concat s2, conv3x3(224->96)+ReLU, conv3x3(96->96)+ReLU
  dec1   up2, concat s1, conv3x3(160->64)+ReLU, conv3x3(64->64)+ReLU
  dec0   up2, concat s0, conv3x3(96->32)+ReLU, conv3x3(32->32)+ReLU
  head   conv1x1(32->1), no ReLU (float32 output)

Convolutions are zero-padded "same" cross-correlations, weights laid out
[cout][ky][kx][cin]. With bf16=True the weights, the input and every stored
activation (after ReLU, pooling and upsampling) are rounded to bfloat16
(round to nearest even) and arithmetic is float32, the precision the CUDA
kernels use; with bf16=False everything is float64 (the reference for the
finite-difference gradient check).

Loss: mean over the masked pixels of (out - target)^2. Adam: the standard
update (Kingma & Ba 2015) with bias correction.
"""
import numpy as np

CH = (32, 64, 96, 128)
IN_CH = 3

# (name, cin, cout, ksize)
LAYERS = [
    ("enc0a", IN_CH, CH[0], 3), ("enc0b", CH[0], CH[0], 3),
    ("enc1a", CH[0], CH[1], 3), ("enc1b", CH[1], CH[1], 3),
    ("enc2a", CH[1], CH[2], 3), ("enc2b", CH[2], CH[2], 3),
    ("mida", CH[2], CH[3], 3), ("midb", CH[3], CH[3], 3),
    ("dec2a", CH[3] + CH[2], CH[2], 3), ("dec2b", CH[2], CH[2], 3),
    ("dec1a", CH[2] + CH[1], CH[1], 3), ("dec1b", CH[1], CH[1], 3),
    ("dec0a", CH[1] + CH[0], CH[0], 3), ("dec0b", CH[0], CH[0], 3),
    ("head", CH[0], 1, 1),
]


def param_layout():
    """[(name, weight offset, weight count, bias offset, cout)] into one flat
    float32 vector: each layer's weights [cout][k][k][cin], then its bias."""
    out, off = [], 0
    for name, cin, cout, k in LAYERS:
        nw = cout * k * k * cin
        out.append((name, off, nw, off + nw, cout))
        off += nw + cout
    return out, off


def num_params():
    return param_layout()[1]


def init_params(seed=0):
    """He-normal weights (std sqrt(2 / fan_in)), zero biases; the head
    starts at zero so the untrained network returns p_prev."""
    rng = np.random.default_rng(seed)
    layout, n = param_layout()
    theta = np.zeros(n, np.float32)
    for (name, cin, cout, k), (_, wo, nw, bo, _) in zip(LAYERS, layout):
        if name == "head":
            continue
        theta[wo:wo + nw] = rng.standard_normal(nw).astype(np.float32) * np.float32(np.sqrt(2.0 / (k * k * cin)))
    return theta


def to_bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    nan = np.isnan(a)
    out = r.astype(np.uint32).view(np.float32).copy()
    out[nan] = np.nan
    return out


class Net:
    def __init__(self, theta, bf16=True):
        self.bf16 = bf16
        self.dt = np.float32 if bf16 else np.float64
        layout, _ = param_layout()
        self.w, self.b = {}, {}
        for (name, cin, cout, k), (_, wo, nw, bo, _) in zip(LAYERS, layout):
            w = np.asarray(theta[wo:wo + nw], self.dt).reshape(cout, k, k, cin)
            self.w[name] = to_bf16(w) if bf16 else w
            self.b[name] = np.asarray(theta[bo:bo + cout], self.dt)
        self.kernel = {name: k for name, _, _, k in LAYERS}

    def q(self, a):
        return to_bf16(a) if self.bf16 else a

    # ------------------------------------------------------------ ops
    def conv(self, x, name):
        w, bias, k = self.w[name], self.b[name], self.kernel[name]
        B, H, W, C = x.shape
        if k == 1:
            return np.einsum("bhwc,oc->bhwo", x, w[:, 0, 0, :]).astype(self.dt) + bias
        xp = np.zeros((B, H + 2, W + 2, C), self.dt)
        xp[:, 1:-1, 1:-1] = x
        y = np.zeros((B, H, W, w.shape[0]), self.dt)
        for ky in range(3):
            for kx in range(3):
                y += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W], w[:, ky, kx, :]).astype(self.dt)
        return y + bias

    def conv_bwd(self, x, dy, name):
        """Returns (dx, dw, db) of y = conv(x) given dy."""
        w, k = self.w[name], self.kernel[name]
        B, H, W, C = x.shape
        db = dy.sum(axis=(0, 1, 2))
        if k == 1:
            dw = np.einsum("bhwo,bhwc->oc", dy, x)[:, None, None, :]
            dx = np.einsum("bhwo,oc->bhwc", dy, w[:, 0, 0, :])
            return dx.astype(self.dt), dw.astype(self.dt), db
        xp = np.zeros((B, H + 2, W + 2, C), self.dt)
        xp[:, 1:-1, 1:-1] = x
        dxp = np.zeros_like(xp)
        dw = np.zeros_like(w)
        for ky in range(3):
            for kx in range(3):
                dw[:, ky, kx, :] = np.einsum("bhwo,bhwc->oc", dy, xp[:, ky:ky + H, kx:kx + W])
                dxp[:, ky:ky + H, kx:kx + W] += np.einsum("bhwo,oc->bhwc", dy, w[:, ky, kx, :]).astype(self.dt)
        return dxp[:, 1:-1, 1:-1], dw, db

    @staticmethod
    def pool(x):
        B, H, W, C = x.shape
        return x.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))

    @staticmethod
    def pool_bwd(dy):
        return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    @staticmethod
    def up_bwd(dy):
        B, H, W, C = dy.shape
        return dy.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))

    # ------------------------------------------------------------ network
    def forward(self, x0):
        """x0 [B,H,W,3] -> out [B,H,W]; keeps what backward needs."""
        t = {}
        r = lambda a: self.q(np.maximum(a, 0))
        t["x0"] = x = self.q(np.asarray(x0, self.dt))
        t["e0a"] = x = r(self.conv(x, "enc0a"))
        t["s0"] = x = r(self.conv(x, "enc0b"))
        t["p0"] = x = self.q(self.pool(x))
        t["e1a"] = x = r(self.conv(x, "enc1a"))
        t["s1"] = x = r(self.conv(x, "enc1b"))
        t["p1"] = x = self.q(self.pool(x))
        t["e2a"] = x = r(self.conv(x, "enc2a"))
        t["s2"] = x = r(self.conv(x, "enc2b"))
        t["p2"] = x = self.q(self.pool(x))
        t["ma"] = x = r(self.conv(x, "mida"))
        t["m"] = x = r(self.conv(x, "midb"))
        t["c2"] = x = np.concatenate([self.up(x), t["s2"]], axis=3)
        t["d2a"] = x = r(self.conv(x, "dec2a"))
        t["d2"] = x = r(self.conv(x, "dec2b"))
        t["c1"] = x = np.concatenate([self.up(x), t["s1"]], axis=3)
        t["d1a"] = x = r(self.conv(x, "dec1a"))
        t["d1"] = x = r(self.conv(x, "dec1b"))
        t["c0"] = x = np.concatenate([self.up(x), t["s0"]], axis=3)
        t["d0a"] = x = r(self.conv(x, "dec0a"))
        t["d0"] = x = r(self.conv(x, "dec0b"))
        out = self.conv(x, "head")[..., 0]
        self.t = t
        return out

    def backward(self, dout):
        """Gradient of the loss with respect to every parameter, as a flat
        vector in param_layout order, given dL/dout [B,H,W]."""
        t = self.t
        g = {}

        def relu_conv_bwd(dy_post, y_post, x_in, name):
            dy = dy_post * (y_post > 0)
            dx, g[name + ".w"], g[name + ".b"] = self.conv_bwd(x_in, dy, name)
            return dx

        dx, g["head.w"], g["head.b"] = self.conv_bwd(t["d0"], dout[..., None], "head")
        dx = relu_conv_bwd(dx, t["d0"], t["d0a"], "dec0b")
        dc = relu_conv_bwd(dx, t["d0a"], t["c0"], "dec0a")
        c = CH[1]
        d_d1, d_s0 = self.up_bwd(dc[..., :c]), dc[..., c:]
        dx = relu_conv_bwd(d_d1, t["d1"], t["d1a"], "dec1b")
        dc = relu_conv_bwd(dx, t["d1a"], t["c1"], "dec1a")
        c = CH[2]
        d_d2, d_s1 = self.up_bwd(dc[..., :c]), dc[..., c:]
        dx = relu_conv_bwd(d_d2, t["d2"], t["d2a"], "dec2b")
        dc = relu_conv_bwd(dx, t["d2a"], t["c2"], "dec2a")
        c = CH[3]
        d_m, d_s2 = self.up_bwd(dc[..., :c]), dc[..., c:]
        dx = relu_conv_bwd(d_m, t["m"], t["ma"], "midb")
        dx = relu_conv_bwd(dx, t["ma"], t["p2"], "mida")
        d_s2 = d_s2 + self.pool_bwd(dx)
        dx = relu_conv_bwd(d_s2, t["s2"], t["e2a"], "enc2b")
        dx = relu_conv_bwd(dx, t["e2a"], t["p1"], "enc2a")
        d_s1 = d_s1 + self.pool_bwd(dx)
        dx = relu_conv_bwd(d_s1, t["s1"], t["e1a"], "enc1b")
        dx = relu_conv_bwd(dx, t["e1a"], t["p0"], "enc1a")
        d_s0 = d_s0 + self.pool_bwd(dx)
        dx = relu_conv_bwd(d_s0, t["s0"], t["e0a"], "enc0b")
        relu_conv_bwd(dx, t["e0a"], t["x0"], "enc0a")
        layout, n = param_layout()
        grad = np.zeros(n, np.float64)
        for name, wo, nw, bo, cout in layout:
            grad[wo:wo + nw] = g[name + ".w"].reshape(-1)
            grad[bo:bo + cout] = g[name + ".b"]
        return grad


def loss_and_grad(net, x0, target, mask):
    """Masked mean squared error and dL/dout."""
    out = net.forward(x0)
    m = np.asarray(mask, out.dtype)
    n = max(1.0, float(m.sum()))
    d = (out - target) * m
    return float((d * d).sum() / n), 2.0 * d / n, out


def adam(theta, m, v, grad, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update in float32 (step counts from 1); returns new arrays."""
    g = np.asarray(grad, np.float32)
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    mh = m / np.float32(1 - b1 ** step)
    vh = v / np.float32(1 - b2 ** step)
    theta = theta - np.float32(lr) * mh / (np.sqrt(vh) + np.float32(eps))
    return theta.astype(np.float32), m.astype(np.float32), v.astype(np.float32)
