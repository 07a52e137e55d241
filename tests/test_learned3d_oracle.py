"""CPU checks of the 3D coarse-correction network oracle (oracle/coarse_net3d.py):
its backward pass against central finite differences in FP64 and against
PyTorch CPU autograd, its convolution against torch's conv3d, the adjointness of
its restriction/prolongation pairs, and its BF16-emulated forward pass against
the exact one."""
import numpy as np
import pytest

import coarse_net3d as CN3


def _data(seed, B=2, nz=9, ny=5, nx=9):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(B, nz, ny, nx, 4)), rng.normal(size=(B, nz, ny, nx, 2))


def test_layer_shapes_and_parameter_count():
    assert CN3.LAYERS[0][0] == 4 and CN3.LAYERS[-1][1] == 2
    assert [b for _, b in CN3.LAYERS[:3]] == [8, 16, 32]          # 8-16-32 channels
    assert CN3.LAYERS[3][0] == 32 + 16 and CN3.LAYERS[4][0] == 16 + 8  # skip concatenations
    assert CN3.num_params() == 27 * sum(a * b for a, b in CN3.LAYERS) == 44496
    w = CN3.he_init(1)
    np.testing.assert_array_equal(CN3.join(CN3.split(w)), w.astype(np.float64))


def test_backward_matches_finite_differences():
    x, t = _data(1)
    w = CN3.he_init(3).astype(np.float64)
    y, cache = CN3.forward(w, x, emulate=False)
    L0, g = CN3.backward(cache, t)
    assert np.isclose(L0, CN3.loss(y, t))
    rng = np.random.default_rng(5)
    offs = np.cumsum([0] + [27 * a * b for a, b in CN3.LAYERS])
    eps = 1e-6
    for k in range(len(CN3.LAYERS)):
        for idx in rng.integers(offs[k], offs[k + 1], size=5):
            wp, wm = w.copy(), w.copy()
            wp[idx] += eps
            wm[idx] -= eps
            fd = CN3.loss(CN3.forward(wp, x, emulate=False)[0], t) - CN3.loss(CN3.forward(wm, x, emulate=False)[0], t)
            fd /= 2 * eps
            assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])) + 1e-8, (k, idx, fd, g[idx])


def test_conv_matches_torch_conv3d():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 5, 7, 9, 3))
    w = rng.normal(size=(4, 27, 3))
    ours = CN3.conv(x, w)
    # torch: NCDHW cross-correlation, weight [cout][cin][kz][ky][kx]; tap t = 9 kz + 3 ky + kx
    wt = torch.tensor(w.reshape(4, 3, 3, 3, 3).transpose(0, 4, 1, 2, 3))
    ref = torch.nn.functional.conv3d(torch.tensor(x.transpose(0, 4, 1, 2, 3)), wt, padding=1)
    np.testing.assert_allclose(ours, ref.numpy().transpose(0, 2, 3, 4, 1), rtol=1e-12, atol=1e-12)


def test_conv_adjoint_and_wgrad():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(2, 5, 7, 9, 4))
    w = rng.normal(size=(6, 27, 4))
    g = rng.normal(size=(2, 5, 7, 9, 6))
    assert np.isclose(np.sum(CN3.conv(x, w) * g), np.sum(x * CN3.conv_t(g, w)))
    assert np.isclose(np.sum(CN3.conv(x, w) * g), np.sum(w * CN3.conv_wgrad(x, g)))


@pytest.mark.parametrize("shape", [(9, 9, 9), (5, 9, 17), (17, 5, 9)])
def test_resampling_adjoints(shape):
    rng = np.random.default_rng(4)
    f = rng.normal(size=(2,) + shape + (3,))
    c = rng.normal(size=(2,) + tuple((n - 1) // 2 + 1 for n in shape) + (3,))
    assert np.isclose(np.sum(CN3.restrict(f) * c), np.sum(f * CN3.restrict_t(c, *shape)))
    assert np.isclose(np.sum(CN3.prolong(c, *shape) * f), np.sum(c * CN3.prolong_t(f)))
    np.testing.assert_allclose(CN3.restrict(np.ones((1,) + shape + (1,))), 1.0)
    np.testing.assert_allclose(CN3.prolong(np.ones(c.shape[:1] + c.shape[1:4] + (1,)), *shape), 1.0)


def test_emulated_forward_close_to_exact():
    x, _ = _data(6)
    w = CN3.he_init(7)
    ye, _ = CN3.forward(w, x, emulate=True)
    yx, _ = CN3.forward(w.astype(np.float64), x, emulate=False)
    assert np.linalg.norm(ye - yx) / np.linalg.norm(yx) < 5e-2


def test_backward_matches_torch_autograd():
    """The hand-written backward against PyTorch CPU autograd of the same network
    (FP64): restriction and prolongation as separable linear maps, convolutions
    as conv3d cross-correlations."""
    torch = pytest.importorskip("torch")
    x, t = _data(11)
    w = CN3.he_init(12).astype(np.float64)
    _, cache = CN3.forward(w, x, emulate=False)
    L_np, g_np = CN3.backward(cache, t)
    ws = [torch.tensor(a, requires_grad=True) for a in CN3.split(w)]

    def conv(z, wl):
        k = wl.reshape(wl.shape[0], 3, 3, 3, wl.shape[2]).permute(0, 4, 1, 2, 3)
        return torch.nn.functional.conv3d(z.permute(0, 4, 1, 2, 3), k, padding=1).permute(0, 2, 3, 4, 1)

    def lin(Az, Ay, Ax, z):
        return torch.einsum("Kk,Jj,Ii,bkjic->bKJIc", torch.tensor(Az), torch.tensor(Ay), torch.tensor(Ax), z)

    def R(z):
        A = [CN3._fw_1d(n) for n in z.shape[1:4]]
        return lin(*[a / a.sum(1, keepdims=True) for a in A], z)

    def P(z, *shape):
        return lin(*[CN3._p_1d(n) for n in shape], z)

    X = torch.tensor(x)
    g = CN3._grids(*X.shape[1:4])
    e0 = torch.relu(conv(X, ws[0]))
    e1 = torch.relu(conv(R(e0), ws[1]))
    e2 = torch.relu(conv(R(e1), ws[2]))
    d1 = torch.relu(conv(torch.cat([P(e2, *g[1]), e1], 4), ws[3]))
    d0 = torch.relu(conv(torch.cat([P(d1, *g[0]), e0], 4), ws[4]))
    y = conv(d0, ws[5])
    T = torch.tensor(t)
    B = y.shape[0]
    loss = (((y - T) ** 2).reshape(B, -1).sum(1) / (T ** 2).reshape(B, -1).sum(1)).mean()
    loss.backward()
    g_t = np.concatenate([a.grad.numpy().ravel() for a in ws])
    assert abs(loss.item() - L_np) <= 1e-12 * abs(L_np)
    np.testing.assert_allclose(g_np, g_t, rtol=1e-9, atol=1e-12 * np.abs(g_t).max())
