"""numpy restatement of the learned preconditioner's U-Net (test infrastructure
only): the forward pass, the relative loss and the hand-derived backward pass of
topoptspline3d_gb300/csrc/unet.cu and k_unet.cu, with the same parameter layout.

With ``bf16=True`` values are rounded to bf16 where the CUDA kernels store bf16
(network input, weights, every layer output, pooled tensors, pre-activation
gradients); everything else is float64.  With ``bf16=False`` it is plain float64,
which is what the finite-difference check of the backward pass uses.
"""
from __future__ import annotations

import numpy as np

# (cin, cout, relu, cin_real, cout_real), same order as unet.cu
LAYERS = [(16, 16, 1, 8, 16), (16, 16, 1, 16, 16), (16, 32, 1, 16, 32), (32, 32, 1, 32, 32),
          (32, 64, 1, 32, 64), (64, 32, 1, 64, 32), (64, 32, 1, 64, 32), (32, 16, 1, 32, 16),
          (32, 16, 1, 32, 16), (16, 16, 0, 16, 3)]
L0A, L0B, L1A, L1B, L2A, L2B, D1A, D1B, D0A, D0B = range(10)


def offsets():
    w, b, o = [], [], 0
    for cin, cout, *_ in LAYERS:
        w.append(o)
        o += cout * 27 * cin
        b.append(o)
        o += cout
    return w, b, o


def num_params() -> int:
    return offsets()[2]


def effective_params() -> int:
    return sum(27 * ci * co + co for _, _, _, ci, co in LAYERS)


def bf16(a):
    """Round to the nearest bf16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    wo, bo, _ = offsets()
    W, B = [], []
    for l, (cin, cout, *_) in enumerate(LAYERS):
        W.append(params[wo[l]:wo[l] + cout * 27 * cin].reshape(cout, 27, cin).astype(np.float64))
        B.append(params[bo[l]:bo[l] + cout].astype(np.float64))
    return W, B


def _shifts(x):
    """x [nb, Z, Y, X, C] -> list of 27 zero-padded shifts x[v + off(tap)]."""
    nb, Z, Y, X, C = x.shape
    p = np.zeros((nb, Z + 2, Y + 2, X + 2, C), dtype=x.dtype)
    p[:, 1:-1, 1:-1, 1:-1] = x
    out = []
    for t in range(27):
        dx, dy, dz = t % 3, (t // 3) % 3, t // 9
        out.append(p[:, dz:dz + Z, dy:dy + Y, dx:dx + X])
    return out


def conv(x, W, b=None):
    """out[v, n] = sum_tap sum_c x[v + off(tap), c] W[n, tap, c] (+ b)."""
    sh = _shifts(x)
    out = np.zeros(x.shape[:4] + (W.shape[0],))
    for t in range(27):
        out += sh[t] @ W[:, t, :].T
    if b is not None:
        out += b
    return out


def conv_wgrad(x, G):
    """dW[n, tap, c] = sum_v G[v, n] x[v + off(tap), c]."""
    sh = _shifts(x)
    n, c = G.shape[-1], x.shape[-1]
    dW = np.zeros((n, 27, c))
    g2 = G.reshape(-1, n)
    for t in range(27):
        dW[:, t, :] = g2.T @ sh[t].reshape(-1, c)
    return dW


def conv_dgrad(G, W):
    """dX[u, c] = sum_tap sum_n G[u - off(tap), n] W[n, tap, c]."""
    Wt = W[:, ::-1, :].transpose(2, 1, 0)  # [c, tap', n] with tap' = 26 - tap
    return conv(G, Wt)


def pool(x):
    nb, Z, Y, X, C = x.shape
    return x.reshape(nb, Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(axis=(2, 4, 6))


def pool_bwd(d):
    return np.repeat(np.repeat(np.repeat(d, 2, axis=1), 2, axis=2), 2, axis=3) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, axis=1), 2, axis=2), 2, axis=3)


def up_bwd(d):
    nb, Z, Y, X, C = d.shape
    return d.reshape(nb, Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(axis=(2, 4, 6))


class UNetOracle:
    def __init__(self, params, bf16_round=True):
        self.params = np.asarray(params, dtype=np.float64)
        self.r = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
        W, B = unpack(self.params)
        self.W = [self.r(w) for w in W]
        self.B = B

    def _layer(self, l, x):
        y = conv(x, self.W[l], self.B[l])
        if LAYERS[l][2]:
            y = np.maximum(y, 0.0)
        return self.r(y)

    def forward(self, x8):
        """x8 [nb, Z, Y, X, 8] -> output [nb, Z, Y, X, 3]; keeps activations."""
        r = self.r
        x0 = np.zeros(x8.shape[:4] + (16,))
        x0[..., :8] = x8
        x0 = r(x0)
        a = {}
        a["x0"] = x0
        a[L0A] = self._layer(L0A, x0)
        a[L0B] = self._layer(L0B, a[L0A])
        a["p0"] = r(pool(a[L0B]))
        a[L1A] = self._layer(L1A, a["p0"])
        a[L1B] = self._layer(L1B, a[L1A])
        a["p1"] = r(pool(a[L1B]))
        a[L2A] = self._layer(L2A, a["p1"])
        a[L2B] = self._layer(L2B, a[L2A])
        a["c1"] = np.concatenate([up(a[L2B]), a[L1B]], axis=-1)
        a[D1A] = self._layer(D1A, a["c1"])
        a[D1B] = self._layer(D1B, a[D1A])
        a["c0"] = np.concatenate([up(a[D1B]), a[L0B]], axis=-1)
        a[D0A] = self._layer(D0A, a["c0"])
        a[D0B] = self._layer(D0B, a[D0A])
        self.a = a
        return a[D0B][..., :3]

    def loss_grad(self, x8, t, m):
        """Relative loss sum m (y - t)^2 / sum m t^2 and the flat parameter gradient."""
        y = self.forward(x8)
        mb = np.stack([(m >> c) & 1 for c in range(3)], axis=-1).astype(np.float64)
        den = float((mb * t * t).sum())
        loss = float((mb * (y - t) ** 2).sum()) / den
        gout = np.zeros(y.shape[:4] + (16,))
        gout[..., :3] = 2.0 * mb * (y - t) / den
        grads = self._backward(gout)
        return loss, grads

    def _bwd_layer(self, l, dY, x, grads, need_dx=True):
        a = self.a
        G = dY * (a[l] > 0) if LAYERS[l][2] else dY
        G = self.r(G)
        grads[l] = (conv_wgrad(x, G), G.reshape(-1, G.shape[-1]).sum(axis=0))
        return conv_dgrad(G, self.W[l]) if need_dx else None

    def _backward(self, gout):
        a, grads = self.a, {}
        d = self._bwd_layer(D0B, gout, a[D0A], grads)
        d = self._bwd_layer(D0A, d, a["c0"], grads)
        gs0 = d[..., 16:].copy()
        d = up_bwd(d[..., :16])
        d = self._bwd_layer(D1B, d, a[D1A], grads)
        d = self._bwd_layer(D1A, d, a["c1"], grads)
        gs1 = d[..., 32:].copy()
        d = up_bwd(d[..., :32])
        d = self._bwd_layer(L2B, d, a[L2A], grads)
        d = self._bwd_layer(L2A, d, a["p1"], grads)
        gs1 = gs1 + pool_bwd(d)
        d = self._bwd_layer(L1B, gs1, a[L1A], grads)
        d = self._bwd_layer(L1A, d, a["p0"], grads)
        gs0 = gs0 + pool_bwd(d)
        d = self._bwd_layer(L0B, gs0, a[L0A], grads)
        self._bwd_layer(L0A, d, a["x0"], grads, need_dx=False)
        wo, bo, n = offsets()
        flat = np.zeros(n)
        for l in range(10):
            dW, db = grads[l]
            flat[wo[l]:wo[l] + dW.size] = dW.ravel()
            flat[bo[l]:bo[l] + db.size] = db
        return flat


def random_params(seed=0, scale=1.0, last_scale=0.3):
    """He-normal weights on the real channels (zero elsewhere), small biases."""
    rng = np.random.default_rng(seed)
    wo, bo, n = offsets()
    p = np.zeros(n)
    for l, (cin, cout, _, ci, co) in enumerate(LAYERS):
        w = np.zeros((cout, 27, cin))
        sd = np.sqrt(2.0 / (27 * ci)) * scale * (last_scale if l == D0B else 1.0)
        w[:co, :, :ci] = rng.standard_normal((co, 27, ci)) * sd
        p[wo[l]:wo[l] + w.size] = w.ravel()
        p[bo[l]:bo[l] + co] = rng.uniform(-0.05, 0.05, co)
    return p
