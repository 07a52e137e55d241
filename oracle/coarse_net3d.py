"""CPU oracle of the 3D learned coarse-grid correction network (test infrastructure).

The checker for the 3D variant of the library's coarse-correction network: a
plain NumPy restatement used only by the tests, never by the solver.  Like the
2D network (oracle/coarse_net.py) it has no counterpart in the reference
(Helmholtz.jl recurses to a coarsest LU on every level); this file pins the
library's own definition of the 3D variant, three grid levels with 8-16-32
channels:

  e0 = relu(conv(x, w0))            grid g0          x = (Re r/s, Im r/s, w^2 m h^2, gamma/w)
  e1 = relu(conv(R e0, w1))         g1 = coarsen(g0)
  e2 = relu(conv(R e1, w2))         g2
  d1 = relu(conv([P e2, e1], w3))   g1
  d0 = relu(conv([P d1, e0], w4))   g0
  y  = conv(d0, w5)                 g0
  loss = mean_b ||y_b - t_b||^2 / ||t_b||^2

conv: 3x3x3 cross-correlation with zero padding, weights [cout][27][cin], tap
t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1), dx along axis 1 (the fastest node
index).  R: full weighting (1, 1/2 per axis) normalised by the weights inside
the grid; P: trilinear prolongation (the 2D network's 1D operators on each
axis).  Arrays are (batch, nz, ny, nx, channels).

emulate=True rounds to BF16 where the GPU stores BF16 (the input, the weights,
every stored activation and activation gradient) and to FP32 where it stores
FP32 (the output, the loss gradient before its BF16 rounding); emulate=False
computes everything in FP64 (the finite-difference check of the backward pass).
"""
from __future__ import annotations

import numpy as np

from coarse_net import _fw_1d, _p_1d, bf16, coarse, f32

# (cin, cout) per layer, forward order
LAYERS = [(4, 8), (8, 16), (16, 32), (48, 16), (24, 8), (8, 2)]
TAPS = 27


def num_params() -> int:
    return sum(TAPS * a * b for a, b in LAYERS)


def split(w: np.ndarray) -> list[np.ndarray]:
    """Flat weight vector -> per-layer [cout][27][cin] arrays."""
    out, k = [], 0
    for cin, cout in LAYERS:
        n = TAPS * cin * cout
        out.append(np.asarray(w[k:k + n], dtype=np.float64).reshape(cout, TAPS, cin))
        k += n
    assert k == w.size
    return out


def join(ws: list[np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(a).ravel() for a in ws])


def tap_offset(t: int) -> tuple[int, int, int]:
    """(dx, dy, dz) of tap t."""
    return t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1


def _shift(x: np.ndarray, dx: int, dy: int, dz: int) -> np.ndarray:
    """out[b, k, j, i] = x[b, k + dz, j + dy, i + dx] (zero outside the grid)."""
    out = np.zeros_like(x)
    dst, src = [slice(None)], [slice(None)]
    for d, n in ((dz, x.shape[1]), (dy, x.shape[2]), (dx, x.shape[3])):
        dst.append(slice(max(0, -d), min(n, n - d)))
        src.append(slice(max(0, d), min(n, n + d)))
    out[tuple(dst)] = x[tuple(src)]
    return out


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """3x3x3 same convolution: out[..., co] = sum_t sum_ci w[co, t, ci] x[p + off_t, ci]."""
    out = np.zeros(x.shape[:4] + (w.shape[0],))
    for t in range(TAPS):
        out += _shift(x, *tap_offset(t)) @ w[:, t, :].T
    return out


def conv_t(g: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Adjoint of conv with respect to its input."""
    out = np.zeros(g.shape[:4] + (w.shape[2],))
    for t in range(TAPS):
        dx, dy, dz = tap_offset(t)
        out += _shift(g @ w[:, t, :], -dx, -dy, -dz)
    return out


def conv_wgrad(x: np.ndarray, g: np.ndarray) -> np.ndarray:
    """d/dw of sum(g * conv(x, w))."""
    co, ci = g.shape[4], x.shape[4]
    dw = np.zeros((co, TAPS, ci))
    G = g.reshape(-1, co)
    for t in range(TAPS):
        dw[:, t, :] = G.T @ _shift(x, *tap_offset(t)).reshape(-1, ci)
    return dw


def _apply3(Az: np.ndarray, Ay: np.ndarray, Ax: np.ndarray, x: np.ndarray) -> np.ndarray:
    return np.einsum("Kk,Jj,Ii,bkjic->bKJIc", Az, Ay, Ax, x, optimize=True)


def _weights(nz: int, ny: int, nx: int):
    Rz, Ry, Rx = _fw_1d(nz), _fw_1d(ny), _fw_1d(nx)
    s = Rz.sum(1)[:, None, None] * Ry.sum(1)[None, :, None] * Rx.sum(1)[None, None, :]
    return Rz, Ry, Rx, s[None, ..., None]


def restrict(x: np.ndarray) -> np.ndarray:
    """Full weighting normalised by the 3D weight sum (the product of the 1D sums)."""
    Rz, Ry, Rx, s = _weights(*x.shape[1:4])
    return _apply3(Rz, Ry, Rx, x) / s


def restrict_t(g: np.ndarray, nz: int, ny: int, nx: int) -> np.ndarray:
    Rz, Ry, Rx, s = _weights(nz, ny, nx)
    return _apply3(Rz.T, Ry.T, Rx.T, g / s)


def prolong(x: np.ndarray, nz: int, ny: int, nx: int) -> np.ndarray:
    return _apply3(_p_1d(nz), _p_1d(ny), _p_1d(nx), x)


def prolong_t(g: np.ndarray) -> np.ndarray:
    nz, ny, nx = g.shape[1:4]
    return _apply3(_p_1d(nz).T, _p_1d(ny).T, _p_1d(nx).T, g)


def _grids(nz: int, ny: int, nx: int) -> list[tuple[int, int, int]]:
    g = [(nz, ny, nx)]
    for _ in range(2):
        g.append(tuple(coarse(n) for n in g[-1]))
    return g


def forward(w, x4: np.ndarray, emulate: bool = True):
    """y (batch, nz, ny, nx, 2) and the cache for backward."""
    rb = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    ro = f32 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    W = [rb(a) for a in (split(w) if isinstance(w, np.ndarray) and w.ndim == 1 else w)]
    relu = lambda a: np.maximum(a, 0.0)  # noqa: E731
    X = rb(x4)
    g = _grids(*X.shape[1:4])
    e0 = rb(relu(conv(X, W[0])))
    r0 = rb(restrict(e0))
    e1 = rb(relu(conv(r0, W[1])))
    r1 = rb(restrict(e1))
    e2 = rb(relu(conv(r1, W[2])))
    c1 = np.concatenate([rb(prolong(e2, *g[1])), e1], axis=4)
    d1 = rb(relu(conv(c1, W[3])))
    c0 = np.concatenate([rb(prolong(d1, *g[0])), e0], axis=4)
    d0 = rb(relu(conv(c0, W[4])))
    y = ro(conv(d0, W[5]))
    cache = dict(W=W, X=X, e0=e0, r0=r0, e1=e1, r1=r1, e2=e2, c1=c1, d1=d1, c0=c0, d0=d0, y=y, g=g,
                 emulate=emulate)
    return y, cache


def loss(y: np.ndarray, t: np.ndarray) -> float:
    B = y.shape[0]
    e = ((y - t) ** 2).reshape(B, -1).sum(1)
    tn = (t ** 2).reshape(B, -1).sum(1)
    return float(np.mean(e / np.where(tn > 0, tn, 1.0)))


def backward(cache: dict, t: np.ndarray):
    """(loss, flat weight gradient) of the cached forward pass."""
    em = cache["emulate"]
    rb = bf16 if em else (lambda a: np.asarray(a, dtype=np.float64))
    ro = f32 if em else (lambda a: np.asarray(a, dtype=np.float64))
    W, y, g = cache["W"], cache["y"], cache["g"]
    B = y.shape[0]
    tn = (t.astype(np.float64) ** 2).reshape(B, -1).sum(1)
    tn = np.where(tn > 0, tn, 1.0)
    L = loss(y, t)
    dy = rb(ro(2.0 * (y - t) / tn[:, None, None, None, None] / B))
    msk = lambda a, act: np.where(act > 0, a, 0.0)  # noqa: E731
    gw = [None] * len(LAYERS)
    gw[5] = conv_wgrad(cache["d0"], dy)
    gd0 = rb(msk(conv_t(dy, W[5]), cache["d0"]))
    gw[4] = conv_wgrad(cache["c0"], gd0)
    gc0 = conv_t(gd0, W[4])
    gc0[..., 16:] = msk(gc0[..., 16:], cache["e0"])
    gc0 = rb(gc0)
    gd1 = rb(msk(prolong_t(gc0[..., :16]), cache["d1"]))
    gw[3] = conv_wgrad(cache["c1"], gd1)
    gc1 = conv_t(gd1, W[3])
    gc1[..., 32:] = msk(gc1[..., 32:], cache["e1"])
    gc1 = rb(gc1)
    ge2 = rb(msk(prolong_t(gc1[..., :32]), cache["e2"]))
    gw[2] = conv_wgrad(cache["r1"], ge2)
    gr1 = rb(conv_t(ge2, W[2]))
    ge1 = rb(ro(msk(restrict_t(gr1, *g[1]), cache["e1"])) + gc1[..., 32:])
    gw[1] = conv_wgrad(cache["r0"], ge1)
    gr0 = rb(conv_t(ge1, W[1]))
    ge0 = rb(ro(msk(restrict_t(gr0, *g[0]), cache["e0"])) + gc0[..., 16:])
    gw[0] = conv_wgrad(cache["X"], ge0)
    return L, join(gw)


def he_init(seed: int) -> np.ndarray:
    """Seeded He-normal weights (any initialisation works for the parity tests)."""
    rng = np.random.default_rng(seed)
    ws = []
    for k, (cin, cout) in enumerate(LAYERS):
        sd = np.sqrt(2.0 / (TAPS * cin)) * (0.5 if k == len(LAYERS) - 1 else 1.0)
        ws.append(rng.normal(0.0, sd, size=(cout, TAPS, cin)))
    return join(ws).astype(np.float32)
