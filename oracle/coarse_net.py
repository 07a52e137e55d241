"""CPU oracle of the learned coarse-grid correction network (test infrastructure).

This is the checker for the library's network kernels (forward pass, loss,
backward pass): a plain NumPy restatement of the same encoder-decoder, used only
by the tests and the gradient check, never by the solver.  The network has no
counterpart in the reference (Helmholtz.jl recurses to a coarsest LU on every
level); what this file pins is the library's own definition:

  e0 = relu(conv(x, w0))            grid g0          x = (Re r/s, Im r/s, w^2 m h^2, gamma/w)
  e1 = relu(conv(R e0, w1))         g1 = coarsen(g0)
  e2 = relu(conv(R e1, w2))         g2
  e3 = relu(conv(R e2, w3))         g3
  d2 = relu(conv([P e3, e2], w4))   g2
  d1 = relu(conv([P d2, e1], w5))   g1
  d0 = relu(conv([P d1, e0], w6))   g0
  y  = conv(d0, w7)                 g0
  loss = mean_b ||y_b - t_b||^2 / ||t_b||^2

conv: 3x3 cross-correlation with zero padding, weights [cout][9][cin], tap
t = 3 (dy + 1) + (dx + 1), dx along axis 1 (the fastest node index).  R: full
weighting (1, 1/2 per axis) normalised by the weights inside the grid.  P:
bilinear prolongation.  Arrays are (batch, ny, nx, channels).

emulate=True rounds to BF16 (round to nearest even) exactly where the GPU
stores BF16 (the input, the weights, every stored activation and activation
gradient) and to FP32 where the GPU stores FP32 (the output, the loss
gradient before its BF16 rounding); emulate=False computes everything in
FP64 (used for the finite-difference check of the backward formulas).
"""
from __future__ import annotations

import numpy as np

# (cin, cout) per layer, forward order
LAYERS = [(4, 16), (16, 32), (32, 64), (64, 64), (128, 64), (96, 32), (48, 16), (16, 2)]


def num_params() -> int:
    return sum(9 * a * b for a, b in LAYERS)


def split(w: np.ndarray) -> list[np.ndarray]:
    """Flat weight vector -> per-layer [cout][9][cin] arrays."""
    out, k = [], 0
    for cin, cout in LAYERS:
        n = 9 * cin * cout
        out.append(np.asarray(w[k:k + n], dtype=np.float64).reshape(cout, 9, cin))
        k += n
    assert k == w.size
    return out


def join(ws: list[np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(a).ravel() for a in ws])


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def f32(a) -> np.ndarray:
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def coarse(n: int) -> int:
    return (n - 1) // 2 + 1


def _shift(x: np.ndarray, dx: int, dy: int) -> np.ndarray:
    """out[b, j, i] = x[b, j + dy, i + dx] (zero outside the grid)."""
    out = np.zeros_like(x)
    ny, nx = x.shape[1], x.shape[2]
    jd = slice(max(0, -dy), min(ny, ny - dy))
    js = slice(max(0, dy), min(ny, ny + dy))
    idd = slice(max(0, -dx), min(nx, nx - dx))
    iss = slice(max(0, dx), min(nx, nx + dx))
    out[:, jd, idd] = x[:, js, iss]
    return out


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """3x3 same convolution: out[..., co] = sum_t sum_ci w[co, t, ci] x[p + off_t, ci]."""
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for t in range(9):
        dx, dy = t % 3 - 1, t // 3 - 1
        out += _shift(x, dx, dy) @ w[:, t, :].T
    return out


def conv_t(g: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Adjoint of conv with respect to its input."""
    out = np.zeros(g.shape[:3] + (w.shape[2],))
    for t in range(9):
        dx, dy = t % 3 - 1, t // 3 - 1
        out += _shift(g @ w[:, t, :], -dx, -dy)
    return out


def conv_wgrad(x: np.ndarray, g: np.ndarray) -> np.ndarray:
    """d/dw of sum(g * conv(x, w))."""
    co, ci = g.shape[3], x.shape[3]
    dw = np.zeros((co, 9, ci))
    G = g.reshape(-1, co)
    for t in range(9):
        dx, dy = t % 3 - 1, t // 3 - 1
        dw[:, t, :] = G.T @ _shift(x, dx, dy).reshape(-1, ci)
    return dw


def _fw_1d(nf: int) -> np.ndarray:
    """Full-weighting matrix on one axis (coarse x fine), rows normalised."""
    nc = coarse(nf)
    Rm = np.zeros((nc, nf))
    for I in range(nc):
        for d, wt in ((-1, 0.5), (0, 1.0), (1, 0.5)):
            f = 2 * I + d
            if 0 <= f < nf:
                Rm[I, f] = wt
    return Rm


def _p_1d(nf: int) -> np.ndarray:
    """Linear prolongation on one axis (fine x coarse): (c[i//2] + c[(i+1)//2]) / 2."""
    nc = coarse(nf)
    Pm = np.zeros((nf, nc))
    for i in range(nf):
        Pm[i, i // 2] += 0.5
        Pm[i, (i + 1) // 2] += 0.5
    return Pm


def _apply2(Ay: np.ndarray, Ax: np.ndarray, x: np.ndarray) -> np.ndarray:
    return np.einsum("Jj,Ii,bjic->bJIc", Ay, Ax, x)


def restrict(x: np.ndarray) -> np.ndarray:
    ny, nx = x.shape[1], x.shape[2]
    Ry, Rx = _fw_1d(ny), _fw_1d(nx)
    # normalisation by the 2D weight sum = product of the 1D sums
    sy, sx = Ry.sum(1), Rx.sum(1)
    return _apply2(Ry, Rx, x) / (sy[None, :, None, None] * sx[None, None, :, None])


def restrict_t(g: np.ndarray, ny: int, nx: int) -> np.ndarray:
    Ry, Rx = _fw_1d(ny), _fw_1d(nx)
    sy, sx = Ry.sum(1), Rx.sum(1)
    gs = g / (sy[None, :, None, None] * sx[None, None, :, None])
    return _apply2(Ry.T, Rx.T, gs)


def prolong(x: np.ndarray, ny: int, nx: int) -> np.ndarray:
    return _apply2(_p_1d(ny), _p_1d(nx), x)


def prolong_t(g: np.ndarray) -> np.ndarray:
    ny, nx = g.shape[1], g.shape[2]
    return _apply2(_p_1d(ny).T, _p_1d(nx).T, g)


def forward(w, x4: np.ndarray, emulate: bool = True):
    """y (batch, ny, nx, 2) and the cache for backward."""
    rb = bf16 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    ro = f32 if emulate else (lambda a: np.asarray(a, dtype=np.float64))
    W = [rb(a) for a in (split(w) if isinstance(w, np.ndarray) and w.ndim == 1 else w)]
    relu = lambda a: np.maximum(a, 0.0)
    X = rb(x4)
    ny, nx = X.shape[1], X.shape[2]
    g = [(ny, nx)]
    for _ in range(3):
        g.append((coarse(g[-1][0]), coarse(g[-1][1])))
    e0 = rb(relu(conv(X, W[0])))
    r0 = rb(restrict(e0))
    e1 = rb(relu(conv(r0, W[1])))
    r1 = rb(restrict(e1))
    e2 = rb(relu(conv(r1, W[2])))
    r2 = rb(restrict(e2))
    e3 = rb(relu(conv(r2, W[3])))
    c2 = np.concatenate([rb(prolong(e3, *g[2])), e2], axis=3)
    d2 = rb(relu(conv(c2, W[4])))
    c1 = np.concatenate([rb(prolong(d2, *g[1])), e1], axis=3)
    d1 = rb(relu(conv(c1, W[5])))
    c0 = np.concatenate([rb(prolong(d1, *g[0])), e0], axis=3)
    d0 = rb(relu(conv(c0, W[6])))
    y = ro(conv(d0, W[7]))
    cache = dict(W=W, X=X, e0=e0, r0=r0, e1=e1, r1=r1, e2=e2, r2=r2, e3=e3, c2=c2, d2=d2, c1=c1, d1=d1, c0=c0,
                 d0=d0, y=y, g=g, emulate=emulate)
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
    W, y = cache["W"], cache["y"]
    B = y.shape[0]
    tn = (t.astype(np.float64) ** 2).reshape(B, -1).sum(1)
    tn = np.where(tn > 0, tn, 1.0)
    L = loss(y, t)
    dy = rb(ro(2.0 * (y - t) / tn[:, None, None, None] / B))
    msk = lambda a, act: np.where(act > 0, a, 0.0)
    gw = [None] * 8
    gw[7] = conv_wgrad(cache["d0"], dy)
    gd0 = rb(msk(conv_t(dy, W[7]), cache["d0"]))
    gw[6] = conv_wgrad(cache["c0"], gd0)
    gc0 = conv_t(gd0, W[6])
    gc0[..., 32:] = msk(gc0[..., 32:], cache["e0"])
    gc0 = rb(gc0)
    gd1 = rb(msk(prolong_t(gc0[..., :32]), cache["d1"]))
    gw[5] = conv_wgrad(cache["c1"], gd1)
    gc1 = conv_t(gd1, W[5])
    gc1[..., 64:] = msk(gc1[..., 64:], cache["e1"])
    gc1 = rb(gc1)
    gd2 = rb(msk(prolong_t(gc1[..., :64]), cache["d2"]))
    gw[4] = conv_wgrad(cache["c2"], gd2)
    gc2 = conv_t(gd2, W[4])
    gc2[..., 64:] = msk(gc2[..., 64:], cache["e2"])
    gc2 = rb(gc2)
    ge3 = rb(msk(prolong_t(gc2[..., :64]), cache["e3"]))
    gw[3] = conv_wgrad(cache["r2"], ge3)
    gr2 = rb(conv_t(ge3, W[3]))
    g = cache["g"]
    ge2 = rb(ro(msk(restrict_t(gr2, *g[2]), cache["e2"])) + gc2[..., 64:])
    gw[2] = conv_wgrad(cache["r1"], ge2)
    gr1 = rb(conv_t(ge2, W[2]))
    ge1 = rb(ro(msk(restrict_t(gr1, *g[1]), cache["e1"])) + gc1[..., 64:])
    gw[1] = conv_wgrad(cache["r0"], ge1)
    gr0 = rb(conv_t(ge1, W[1]))
    ge0 = rb(ro(msk(restrict_t(gr0, *g[0]), cache["e0"])) + gc0[..., 32:])
    gw[0] = conv_wgrad(cache["X"], ge0)
    return L, join(gw)


def he_init(seed: int) -> np.ndarray:
    """Seeded He-normal weights (any initialisation works for the parity tests)."""
    rng = np.random.default_rng(seed)
    ws = []
    for k, (cin, cout) in enumerate(LAYERS):
        sd = np.sqrt(2.0 / (9 * cin)) * (0.5 if k == len(LAYERS) - 1 else 1.0)
        ws.append(rng.normal(0.0, sd, size=(cout, 9, cin)))
    return join(ws).astype(np.float32)
