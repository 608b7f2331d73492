"""CPU oracle of the learned Poisson preconditioner's network (test
infrastructure only: the product path runs the CUDA kernels).

The same four-level U-Net as the library (layer table, NHWC layout, zero
padding, 2x2 average pooling, nearest upsampling, ReLU), in numpy, with the
library's roundings emulated: BF16 (round to nearest even) for the weights,
every stored activation and every stored activation gradient; FP32
accumulation.  Used to check the GPU forward pass and gradients, and
(``bf16=False``) in FP64 against finite differences.

The network has no counterpart in the reference (lapl_lib.F90 hands the
Poisson system to PETSc); parameters are laid out per layer as W[tap][cout][cin]
then b[cout], tap = 3 (dy + 1) + (dx + 1).
"""
import numpy as np

CIN0 = 16
COUT_LAST = 16
NFEAT = 4
# c1, c2, cout, resolution level: a four-level U-Net (16, 32, 64, 64 channels)
LAYERS = [(CIN0, 0, 16, 0), (16, 0, 16, 0),        # enc0a, enc0b (skip s0)
          (16, 0, 32, 1), (32, 0, 32, 1),          # enc1a, enc1b (skip s1)
          (32, 0, 64, 2), (64, 0, 64, 2),          # enc2a, enc2b (skip s2)
          (64, 0, 64, 3), (64, 0, 64, 3),          # bottleneck
          (64, 64, 64, 2), (64, 32, 32, 1), (32, 16, 16, 0),   # decoders [up, skip]
          (16, 0, COUT_LAST, 0)]                   # output (channel 0)


def layout():
    """(w_off, b_off) per layer and the parameter count."""
    off, out = 0, []
    for c1, c2, co, _ in LAYERS:
        nw = 9 * (c1 + c2) * co
        out.append((off, off + nw))
        off += nw + co
    return out, off


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).reshape(a.shape)


class Net:
    def __init__(self, params, use_bf16=True, dtype=np.float32):
        self.p = np.asarray(params, dtype=np.float64)
        self.q = use_bf16
        self.dt = dtype
        self.lay, self.n = layout()

    def _r(self, x):
        x = np.asarray(x, dtype=self.dt)
        return bf16(x) if self.q else x

    def W(self, l):
        c1, c2, co, _ = LAYERS[l]
        wo, bo = self.lay[l]
        w = self.p[wo:bo].reshape(9, co, c1 + c2).astype(self.dt)
        return (bf16(w) if self.q else w), self.p[bo:bo + co].astype(self.dt)

    @staticmethod
    def _shift(x, dy, dx):
        """y[b, i, j] = x[b, i + dy, j + dx] with zero padding."""
        B, H, W, C = x.shape
        out = np.zeros_like(x)
        ys, ye = max(0, -dy), min(H, H - dy)
        xs, xe = max(0, -dx), min(W, W - dx)
        out[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
        return out

    def conv(self, l, x):
        w, b = self.W(l)
        out = np.zeros(x.shape[:3] + (w.shape[1],), dtype=self.dt)
        for t in range(9):
            out += np.einsum("bhwc,oc->bhwo", self._shift(x, t // 3 - 1, t % 3 - 1), w[t])
        return out + b

    def conv_bwd(self, l, x, dout):
        """(dx, dW, db) of out = conv(l, x) given dout."""
        w, _ = self.W(l)
        dw = np.zeros(w.shape, dtype=self.dt)
        dx = np.zeros(x.shape, dtype=self.dt)
        for t in range(9):
            dy_, dx_ = t // 3 - 1, t % 3 - 1
            dw[t] = np.einsum("bhwo,bhwc->oc", dout, self._shift(x, dy_, dx_))
            dx += self._shift(np.einsum("bhwo,oc->bhwc", dout, w[t]), -dy_, -dx_)
        return dx, dw, dout.sum(axis=(0, 1, 2))

    @staticmethod
    def pool(x):
        return 0.25 * (x[:, 0::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 0::2] + x[:, 1::2, 1::2])

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    def forward(self, x0):
        r, relu = self._r, (lambda v: np.maximum(v, 0))
        cat = lambda a, b: np.concatenate([a, b], axis=3)
        A = {}
        A["x0"] = r(x0)
        A["a0"] = r(relu(self.conv(0, A["x0"])))
        A["s0"] = r(relu(self.conv(1, A["a0"])))
        A["p0"] = r(self.pool(A["s0"]))
        A["a1"] = r(relu(self.conv(2, A["p0"])))
        A["s1"] = r(relu(self.conv(3, A["a1"])))
        A["p1"] = r(self.pool(A["s1"]))
        A["a2"] = r(relu(self.conv(4, A["p1"])))
        A["s2"] = r(relu(self.conv(5, A["a2"])))
        A["p2"] = r(self.pool(A["s2"]))
        A["a3"] = r(relu(self.conv(6, A["p2"])))
        A["b3"] = r(relu(self.conv(7, A["a3"])))
        A["u2"] = self.up(A["b3"])
        A["d2"] = r(relu(self.conv(8, cat(A["u2"], A["s2"]))))
        A["u1"] = self.up(A["d2"])
        A["d1"] = r(relu(self.conv(9, cat(A["u1"], A["s1"]))))
        A["u0"] = self.up(A["d1"])
        A["d0"] = r(relu(self.conv(10, cat(A["u0"], A["s0"]))))
        A["y"] = self.conv(11, A["d0"]).astype(self.dt)
        self.A = A
        return A["y"][..., 0]

    def loss_grad(self, x0, tgt, mask):
        """MSE over masked pixels and its gradient w.r.t. all parameters."""
        r = self._r
        y = self.forward(x0)
        A = self.A
        cat = lambda a, b: np.concatenate([a, b], axis=3)
        m = np.broadcast_to(mask, y.shape).astype(self.dt)
        d = y - tgt
        msum = m.sum()
        loss = float((m * d * d).sum() / msum)
        dy = np.zeros(A["y"].shape, dtype=self.dt)
        dy[..., 0] = r(2.0 * m * d / msum)
        g = np.zeros(self.n, dtype=np.float64)

        def put(l, dw, db):
            wo, bo = self.lay[l]
            g[wo:bo] = dw.ravel()
            g[bo:bo + LAYERS[l][2]] = db

        mk = lambda a: (a > 0).astype(self.dt)
        dd0, dw, db = self.conv_bwd(11, A["d0"], dy); put(11, dw, db)
        dd0 = r(dd0 * mk(A["d0"]))
        dcat, dw, db = self.conv_bwd(10, cat(A["u0"], A["s0"]), dd0); put(10, dw, db)
        du0, ds0b = r(dcat[..., :32]), r(dcat[..., 32:])
        dd1 = r(self._upb(du0) * mk(A["d1"]))
        dcat, dw, db = self.conv_bwd(9, cat(A["u1"], A["s1"]), dd1); put(9, dw, db)
        du1, ds1b = r(dcat[..., :64]), r(dcat[..., 64:])
        dd2 = r(self._upb(du1) * mk(A["d2"]))
        dcat, dw, db = self.conv_bwd(8, cat(A["u2"], A["s2"]), dd2); put(8, dw, db)
        du2, ds2b = r(dcat[..., :64]), r(dcat[..., 64:])
        db3 = r(self._upb(du2) * mk(A["b3"]))
        da3, dw, db = self.conv_bwd(7, A["a3"], db3); put(7, dw, db)
        da3 = r(da3 * mk(A["a3"]))
        dp2, dw, db = self.conv_bwd(6, A["p2"], da3); put(6, dw, db)
        ds2 = r((0.25 * self.up(r(dp2)) + ds2b) * mk(A["s2"]))
        da2, dw, db = self.conv_bwd(5, A["a2"], ds2); put(5, dw, db)
        da2 = r(da2 * mk(A["a2"]))
        dp1, dw, db = self.conv_bwd(4, A["p1"], da2); put(4, dw, db)
        ds1 = r((0.25 * self.up(r(dp1)) + ds1b) * mk(A["s1"]))
        da1, dw, db = self.conv_bwd(3, A["a1"], ds1); put(3, dw, db)
        da1 = r(da1 * mk(A["a1"]))
        dp0, dw, db = self.conv_bwd(2, A["p0"], da1); put(2, dw, db)
        ds0 = r((0.25 * self.up(r(dp0)) + ds0b) * mk(A["s0"]))
        da0, dw, db = self.conv_bwd(1, A["a0"], ds0); put(1, dw, db)
        da0 = r(da0 * mk(A["a0"]))
        _, dw, db = self.conv_bwd(0, A["x0"], da0); put(0, dw, db)
        return loss, g

    @staticmethod
    def _upb(du):
        return du[:, 0::2, 0::2] + du[:, 0::2, 1::2] + du[:, 1::2, 0::2] + du[:, 1::2, 1::2]


def init_params(seed=0, scale_last=0.1):
    """He-normal weights (numpy generator; the library has its own seeded init)."""
    lay, n = layout()
    rng = np.random.default_rng(seed)
    p = np.zeros(n)
    for l, (c1, c2, co, _) in enumerate(LAYERS):
        cin = c1 + c2
        cin_eff = NFEAT if l == 0 else cin
        sd = np.sqrt(2.0 / (9 * cin_eff)) * (scale_last if l == len(LAYERS) - 1 else 1.0)
        w = rng.standard_normal((9, co, cin)) * sd
        if l == 0:
            w[:, :, NFEAT:] = 0
        if l == len(LAYERS) - 1:
            w[:, 1:, :] = 0
        wo, bo = lay[l]
        p[wo:bo] = w.ravel()
    return p
