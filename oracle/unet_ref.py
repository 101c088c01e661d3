"""CPU oracle of the learned Poisson preconditioner's network (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels in
icep_kapsel_gb300/csrc/unet.cu (forward values and parameter gradients). It
is not used by the product.

The reference has no learned component; this module states the network the
GPU path implements, so that its kernels can be checked:

  inputs  (coarse grid n^3, n = N/2): channel 0 = eps_c / eps_ref - 1,
          channel 1 = r_c / rms(r); eps_c, r_c are 2x2x2 averages of the
          fine-grid permittivity and residual
  e0 = relu(conv(x, c0a));  e0 = relu(conv(e0, c0b))          16 ch, n^3
  e1 = relu(conv(pool(e0), c1a)); e1 = relu(conv(e1, c1b))     32 ch, (n/2)^3
  e2 = relu(conv(pool(e1), c2a)); e2 = relu(conv(e2, c2b))     64 ch, (n/4)^3
  d1 = relu(conv(cat(e1, up(e2)), c1u))                        32 ch, (n/2)^3
  d0 = relu(conv(cat(e0, up(d1)), c0u))                        16 ch, n^3
  y  = conv(d0, out)                                           1 ch, n^3

conv: 3x3x3, periodic, W[t][ci][co] with tap t = 9(dx+1) + 3(dy+1) + (dz+1)
for the neighbour (x+dx, y+dy, z+dz), plus a bias; pool: mean of the 8
children; up: nearest (child (2X+a) reads parent X). Arrays are [x][y][z][c].
The flat parameter vector holds, layer by layer, W (27*ci*co) then b (co).
"""
import numpy as np

LAYERS = [("c0a", 2, 16), ("c0b", 16, 16), ("c1a", 16, 32), ("c1b", 32, 32), ("c2a", 32, 64), ("c2b", 64, 64),
          ("c1u", 96, 32), ("c0u", 48, 16), ("out", 16, 1)]


def param_offsets():
    off, o = {}, 0
    for name, ci, co in LAYERS:
        off[name] = (o, o + 27 * ci * co, ci, co)  # W start, b start
        o += 27 * ci * co + co
    return off, o


def n_params():
    return param_offsets()[1]


def init_params(seed=0):
    """He-normal weights, zero biases (the GPU initialiser draws its own)."""
    rng = np.random.default_rng(seed)
    off, n = param_offsets()
    p = np.zeros(n)
    for name, ci, co in LAYERS:
        w0, b0, _, _ = off[name]
        p[w0:b0] = rng.standard_normal(27 * ci * co) * np.sqrt(2.0 / (27 * ci))
    return p


def _shifts():
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                yield 9 * (dx + 1) + 3 * (dy + 1) + (dz + 1), dx, dy, dz


def _nb(a, dx, dy, dz):
    """a[(x+dx)%n, (y+dy)%n, (z+dz)%n]"""
    return np.roll(a, shift=(-dx, -dy, -dz), axis=(0, 1, 2))


def conv(a, W, b):
    out = np.broadcast_to(b, a.shape[:3] + (W.shape[2],)).copy()
    for t, dx, dy, dz in _shifts():
        out += _nb(a, dx, dy, dz) @ W[t]
    return out


def conv_backward(a, W, dout):
    """Gradients of conv(a, W, b) given dL/dout: (da, dW, db)."""
    da = np.zeros_like(a)
    dW = np.zeros_like(W)
    for t, dx, dy, dz in _shifts():
        an = _nb(a, dx, dy, dz)
        dW[t] = an.reshape(-1, a.shape[3]).T @ dout.reshape(-1, dout.shape[3])
        # out[v] += a[v + s] W  ->  da[v + s] += dout[v] W^T
        da += _nb(dout @ W[t].T, -dx, -dy, -dz)
    db = dout.sum(axis=(0, 1, 2))
    return da, dW, db


def pool(a):
    n = a.shape[0] // 2
    return a.reshape(n, 2, n, 2, n, 2, -1).mean(axis=(1, 3, 5))


def pool_backward(d):
    return up(d) / 8.0


def up(a):
    return a.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def up_backward(d):
    n = d.shape[0] // 2
    return d.reshape(n, 2, n, 2, n, 2, -1).sum(axis=(1, 3, 5))


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_MMA = ("c0b", "c1a", "c1b", "c2a", "c2b", "c1u", "c0u")


def _layer(p, name, emulate=False):
    off, _ = param_offsets()
    w0, b0, ci, co = off[name]
    W = p[w0:b0].reshape(27, ci, co)
    if emulate and name in _MMA:  # tensor-core layers use BF16 weights
        W = bf16(W)
    return W, p[b0:b0 + co]


def forward(p, x, emulate=False):
    """x: [n][n][n][2]; returns (y [n][n][n], cache). emulate=True rounds to
    BF16 where the GPU stores BF16 (tensor-core weights, activations)."""
    q = bf16 if emulate else (lambda v: v)
    c = {"x": x, "emulate": emulate}
    relu = lambda v: np.maximum(v, 0.0)
    L = lambda name: _layer(p, name, emulate)
    c["e0a"] = q(relu(conv(x, *L("c0a"))))
    c["e0"] = q(relu(conv(c["e0a"], *L("c0b"))))
    c["p1"] = q(pool(c["e0"]))
    c["e1a"] = q(relu(conv(c["p1"], *L("c1a"))))
    c["e1"] = q(relu(conv(c["e1a"], *L("c1b"))))
    c["p2"] = q(pool(c["e1"]))
    c["e2a"] = q(relu(conv(c["p2"], *L("c2a"))))
    c["e2"] = q(relu(conv(c["e2a"], *L("c2b"))))
    c["k1"] = np.concatenate([c["e1"], up(c["e2"])], axis=3)
    c["d1"] = q(relu(conv(c["k1"], *L("c1u"))))
    c["k0"] = np.concatenate([c["e0"], up(c["d1"])], axis=3)
    c["d0"] = q(relu(conv(c["k0"], *L("c0u"))))
    y = conv(c["d0"], *L("out"))[..., 0]
    return y, c


def backward(p, c, dy):
    """dL/dparams (flat, same layout as p) given dL/dy. With an emulating
    cache the masked gradients that feed a convolution are rounded to BF16,
    as on the GPU. ReLU masks come from the activations (relu(z) > 0 iff z > 0)."""
    emulate = c.get("emulate", False)
    q = bf16 if emulate else (lambda v: v)
    L = lambda name: _layer(p, name, emulate)[0]
    off, n = param_offsets()
    g = np.zeros(n)

    def put(name, dW, db):
        w0, b0, ci, co = off[name]
        g[w0:b0] = dW.ravel()
        g[b0:b0 + co] = db

    da, dW, db = conv_backward(c["d0"], L("out"), dy[..., None]); put("out", dW, db)
    dz = q(da * (c["d0"] > 0))
    da, dW, db = conv_backward(c["k0"], L("c0u"), dz); put("c0u", dW, db)
    de0 = da[..., :16].copy()
    dz = q(up_backward(da[..., 16:]) * (c["d1"] > 0))
    da, dW, db = conv_backward(c["k1"], L("c1u"), dz); put("c1u", dW, db)
    de1 = da[..., :32].copy()
    dz = q(up_backward(da[..., 32:]) * (c["e2"] > 0))
    da, dW, db = conv_backward(c["e2a"], L("c2b"), dz); put("c2b", dW, db)
    dz = q(da * (c["e2a"] > 0))
    da, dW, db = conv_backward(c["p2"], L("c2a"), dz); put("c2a", dW, db)
    de1 += pool_backward(da)
    dz = q(de1 * (c["e1"] > 0))
    da, dW, db = conv_backward(c["e1a"], L("c1b"), dz); put("c1b", dW, db)
    dz = q(da * (c["e1a"] > 0))
    da, dW, db = conv_backward(c["p1"], L("c1a"), dz); put("c1a", dW, db)
    de0 += pool_backward(da)
    dz = q(de0 * (c["e0"] > 0))
    da, dW, db = conv_backward(c["e0a"], L("c0b"), dz); put("c0b", dW, db)
    dz = q(da * (c["e0a"] > 0))
    _, dW, db = conv_backward(c["x"], L("c0a"), dz); put("c0a", dW, db)
    return g


def restrict_avg(f):
    """Fine [N][N][N] -> coarse 2x2x2 means."""
    return pool(f[..., None])[..., 0]


def prolong(yc):
    """Coarse -> fine, cell-centred trilinear (weights 3/4, 1/4 per axis, periodic)."""
    out = yc
    for ax in range(3):
        a = np.moveaxis(out, ax, 0)
        lo = 0.75 * a + 0.25 * np.roll(a, 1, axis=0)   # fine child 2X: towards X-1
        hi = 0.75 * a + 0.25 * np.roll(a, -1, axis=0)  # fine child 2X+1: towards X+1
        f = np.empty((2 * a.shape[0],) + a.shape[1:])
        f[0::2] = lo
        f[1::2] = hi
        out = np.moveaxis(f, 0, ax)
    return out


def prolong_adjoint(ff):
    """Transpose of prolong."""
    out = ff
    for ax in range(3):
        a = np.moveaxis(out, ax, 0)
        lo, hi = a[0::2], a[1::2]
        c = 0.75 * lo + 0.25 * np.roll(lo, -1, axis=0) + 0.75 * hi + 0.25 * np.roll(hi, 1, axis=0)
        out = np.moveaxis(c, 0, ax)
    return out


def network_input(eps, r, eps_ref):
    """Fine-grid eps and residual [N][N][N] -> coarse input [n][n][n][2]."""
    rms = np.sqrt(np.mean(r * r))
    x = np.stack([restrict_avg(eps) / eps_ref - 1.0, restrict_avg(r) / (rms if rms > 0 else 1.0)], axis=3)
    return x, rms
