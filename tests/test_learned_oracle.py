"""CPU checks of the learned coarse-correction oracle (oracle/coarse_net.py):
its backward pass against central finite differences in FP64, its convolution
against torch's CPU conv2d, the adjointness of its restriction/prolongation
pairs, and the BF16 rounding helper.  Plus the host-side argument checks of the
network entry points (no GPU work)."""
import numpy as np
import pytest

import coarse_net as CN


def _data(seed, B=2, ny=9, nx=17):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, ny, nx, 4))
    t = rng.normal(size=(B, ny, nx, 2))
    return x, t


def test_backward_matches_finite_differences():
    """Exact (FP64) mode: every layer's gradient entries against central differences."""
    x, t = _data(1)
    w = CN.he_init(3).astype(np.float64)
    y, cache = CN.forward(w, x, emulate=False)
    L0, g = CN.backward(cache, t)
    assert np.isclose(L0, CN.loss(y, t))
    rng = np.random.default_rng(5)
    offs = np.cumsum([0] + [9 * a * b for a, b in CN.LAYERS])
    eps = 1e-6
    for k in range(8):
        for idx in rng.integers(offs[k], offs[k + 1], size=6):
            wp, wm = w.copy(), w.copy()
            wp[idx] += eps
            wm[idx] -= eps
            fd = (CN.loss(CN.forward(wp, x, emulate=False)[0], t) - CN.loss(CN.forward(wm, x, emulate=False)[0], t))
            fd /= 2 * eps
            assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])) + 1e-8, (k, idx, fd, g[idx])


def test_conv_matches_torch_conv2d():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 9, 17, 5))
    w = rng.normal(size=(3, 9, 5))
    ours = CN.conv(x, w)
    # torch: NCHW cross-correlation, weight [cout][cin][ky][kx]; tap t = 3*ky + kx
    wt = torch.tensor(w.reshape(3, 3, 3, 5).transpose(0, 3, 1, 2))
    ref = torch.nn.functional.conv2d(torch.tensor(x.transpose(0, 3, 1, 2)), wt, padding=1)
    np.testing.assert_allclose(ours, ref.numpy().transpose(0, 2, 3, 1), rtol=1e-12, atol=1e-12)


def test_conv_adjoint_and_wgrad():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(2, 9, 17, 4))
    w = rng.normal(size=(6, 9, 4))
    g = rng.normal(size=(2, 9, 17, 6))
    assert np.isclose(np.sum(CN.conv(x, w) * g), np.sum(x * CN.conv_t(g, w)))
    assert np.isclose(np.sum(CN.conv(x, w) * g), np.sum(w * CN.conv_wgrad(x, g)))


@pytest.mark.parametrize("ny,nx", [(9, 17), (17, 9), (33, 17)])
def test_resampling_adjoints(ny, nx):
    rng = np.random.default_rng(4)
    f = rng.normal(size=(2, ny, nx, 3))
    c = rng.normal(size=(2, CN.coarse(ny), CN.coarse(nx), 3))
    assert np.isclose(np.sum(CN.restrict(f) * c), np.sum(f * CN.restrict_t(c, ny, nx)))
    assert np.isclose(np.sum(CN.prolong(c, ny, nx) * f), np.sum(c * CN.prolong_t(f)))
    # full weighting reproduces constants, prolongation interpolates them
    one = np.ones((1, ny, nx, 1))
    np.testing.assert_allclose(CN.restrict(one), 1.0)
    np.testing.assert_allclose(CN.prolong(np.ones((1, CN.coarse(ny), CN.coarse(nx), 1)), ny, nx), 1.0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265, 0.0, 1e-30], dtype=np.float32)
    r = CN.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0          # tie -> even
    assert r[2] == 1.0 + 2 ** -7  # above the tie -> up
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-12
    assert r[5] == 0.0
    # every result is exactly representable in 8 significand bits
    m, e = np.frexp(r[r != 0])
    assert np.all(np.abs(m * 2 ** 8 - np.round(m * 2 ** 8)) == 0)


def test_emulated_forward_close_to_exact():
    x, _ = _data(6)
    w = CN.he_init(7)
    ye, _ = CN.forward(w, x, emulate=True)
    yx, _ = CN.forward(w.astype(np.float64), x, emulate=False)
    assert np.linalg.norm(ye - yx) / np.linalg.norm(yx) < 5e-2


def test_net_entry_points_reject_bad_arguments(hz):
    """Argument errors come back as status codes before any GPU work."""
    lib = hz._lib.load()
    import ctypes as C
    assert lib.hz_net_num_params() == CN.num_params()
    for k, (cin, cout) in enumerate(CN.LAYERS):
        a, b = C.c_int32(), C.c_int32()
        assert lib.hz_net_layer_shape(k, C.byref(a), C.byref(b)) == 0
        assert (a.value, b.value) == (cin, cout)
    a = C.c_int32()
    assert lib.hz_net_layer_shape(8, C.byref(a), C.byref(a)) == hz._lib.HZ_ERR_ARG
    assert lib.hz_net_forward(None, None, None, 17, 17, 1, 0) == hz._lib.HZ_ERR_ARG
    assert lib.hz_net_gradient(None, None, None, 17, 17, 1, 0, None, None) == hz._lib.HZ_ERR_ARG
    assert lib.hz_net_train(None, None, None, 17, 17, 1, 1, 1, 1e-3, 0, None) == hz._lib.HZ_ERR_ARG
    assert lib.hz_attach_net(None, None, 2, 0.5) == hz._lib.HZ_ERR_ARG
    assert lib.hz_collect_pairs(None, None, None, 0, 0, 0, 2, 1, 1, None, None, None, None, None) == \
        hz._lib.HZ_ERR_ARG
    out = C.c_void_p()
    st = lib.hz_net_create(0, 0, C.byref(out))
    assert st in (hz._lib.HZ_OK, hz._lib.HZ_ERR_NO_DEVICE)
    if st == hz._lib.HZ_OK:
        lib.hz_net_destroy(out)


def _net_file(path, layers=None, version=1, magic=b"HZCNET01", nparams=None, step=7, arrays=3, values=None):
    import struct
    layers = layers or CN.LAYERS
    n = CN.num_params() if nparams is None else nparams
    with open(path, "wb") as f:
        f.write(magic)
        f.write(struct.pack("<II", version, len(layers)))
        for a, b in layers:
            f.write(struct.pack("<ii", a, b))
        f.write(struct.pack("<qq", n, step))
        v = np.zeros(n, np.float32) if values is None else values
        for _ in range(arrays):
            f.write(v.astype(np.float32).tobytes())


def test_net_file_format_checks(hz, tmp_path):
    """The saved-network header check runs on the host: a valid file gives its
    parameter count and Adam step; another magic, version or layer shape, or a
    truncated file, is rejected with an error status (no GPU needed)."""
    good = tmp_path / "good.hzn"
    _net_file(good)
    assert hz.learned.file_info(good) == (CN.num_params(), 7)
    bad = {
        "magic": dict(magic=b"NOTANETW"),
        "version": dict(version=2),
        "shape": dict(layers=[(4, 16)] * 8),
        "truncated": dict(arrays=2),
    }
    for name, kw in bad.items():
        p = tmp_path / f"{name}.hzn"
        _net_file(p, **kw)
        with pytest.raises(hz._lib.HelmgpuError):
            hz.learned.file_info(p)
    with pytest.raises(hz._lib.HelmgpuError):
        hz.learned.file_info(tmp_path / "missing.hzn")


def test_backward_matches_torch_autograd():
    """The oracle's hand-written backward against PyTorch CPU autograd of the same
    network (FP64, no rounding): the restriction and prolongation as the same
    separable linear maps, the convolutions as conv2d cross-correlations."""
    torch = pytest.importorskip("torch")
    x, t = _data(11)
    w = CN.he_init(12).astype(np.float64)
    _, cache = CN.forward(w, x, emulate=False)
    L_np, g_np = CN.backward(cache, t)

    ws = [torch.tensor(a, requires_grad=True) for a in CN.split(w)]

    def conv(z, wl):  # z (B, ny, nx, C); wl [cout][9][cin] with tap 3*(dy+1) + (dx+1)
        k = wl.reshape(wl.shape[0], 3, 3, wl.shape[2]).permute(0, 3, 1, 2)
        return torch.nn.functional.conv2d(z.permute(0, 3, 1, 2), k, padding=1).permute(0, 2, 3, 1)

    def lin(Ay, Ax, z):
        return torch.einsum("Jj,Ii,bjic->bJIc", torch.tensor(Ay), torch.tensor(Ax), z)

    def R(z):
        ny, nx = z.shape[1], z.shape[2]
        Ry, Rx = CN._fw_1d(ny), CN._fw_1d(nx)
        return lin(Ry / Ry.sum(1, keepdims=True), Rx / Rx.sum(1, keepdims=True), z)

    def P(z, ny, nx):
        return lin(CN._p_1d(ny), CN._p_1d(nx), z)

    relu = torch.relu
    X = torch.tensor(x)
    ny, nx = X.shape[1], X.shape[2]
    g1 = (CN.coarse(ny), CN.coarse(nx))
    g2 = (CN.coarse(g1[0]), CN.coarse(g1[1]))
    e0 = relu(conv(X, ws[0]))
    e1 = relu(conv(R(e0), ws[1]))
    e2 = relu(conv(R(e1), ws[2]))
    e3 = relu(conv(R(e2), ws[3]))
    d2 = relu(conv(torch.cat([P(e3, *g2), e2], 3), ws[4]))
    d1 = relu(conv(torch.cat([P(d2, *g1), e1], 3), ws[5]))
    d0 = relu(conv(torch.cat([P(d1, ny, nx), e0], 3), ws[6]))
    y = conv(d0, ws[7])
    T = torch.tensor(t)
    B = y.shape[0]
    loss = (((y - T) ** 2).reshape(B, -1).sum(1) / (T ** 2).reshape(B, -1).sum(1)).mean()
    loss.backward()
    g_t = np.concatenate([a.grad.numpy().ravel() for a in ws])
    assert abs(loss.item() - L_np) <= 1e-12 * abs(L_np)
    np.testing.assert_allclose(g_np, g_t, rtol=1e-9, atol=1e-12 * np.abs(g_t).max())
