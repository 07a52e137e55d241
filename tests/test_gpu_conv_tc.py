"""GPU parity of the networks' convolutions on the 5th-generation tensor
cores (tcgen05.mma with the accumulator in tensor memory, operands staged by
the TMA unit) against the CPU oracle (oracle/coarse_net.py,
BF16 rounding emulated) and against the warp-level MMA path: forward output to
relative L2 error <= 1e-2, loss to <= 1e-3, every layer's weight gradient to
<= 3e-2 (the tolerances of the network's other parity tests), on grids whose
tiles are partial at the edges; weight images follow Adam steps."""
import numpy as np
import pytest

import coarse_net as CN

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _x(seed, B, ny, nx):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, ny, nx, 4)).astype(np.float32)
    x[..., 2] = rng.uniform(0.5, 6.0, size=(B, ny, nx))
    x[..., 3] = rng.uniform(0.01, 0.9, size=(B, ny, nx))
    t = rng.normal(size=(B, ny, nx, 2)).astype(np.float32)
    return x, t


def _launches(net, name):
    return sum(r["launches"] for r in net.kernel_times() if r["name"] == name)


PATHS = ["tcgen05"]


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("ny,nx", [(17, 33), (41, 25)])
def test_tcgen05_forward_matches_oracle_and_warp_mma(hz, ny, nx, path):
    net = hz.learned.CoarseNet(seed=11)
    w = net.get_weights()
    x, _ = _x(1, 3, ny, nx)
    net.set_conv_path("mma")
    y_mma = net.forward(x)
    net.set_conv_path(path)
    net.reset_kernel_times()
    y_tc = net.forward(x)
    assert _launches(net, "net_conv_fwd_tc") == 7  # every layer but the 8-channel output layer
    assert _launches(net, "net_conv_fwd") == 1
    yo, _ = CN.forward(w, x.astype(np.float64), emulate=True)
    for b in range(x.shape[0]):
        assert _rel(y_tc[b], yo[b]) <= 1e-2, (b, _rel(y_tc[b], yo[b]))
        assert _rel(y_tc[b], y_mma[b]) <= 1e-2, (b, _rel(y_tc[b], y_mma[b]))


@pytest.mark.parametrize("path", PATHS + ["mma"])
def test_tcgen05_gradient_matches_oracle(hz, path):
    """Loss and weight gradients (weight gradient on tcgen05 with the tensor-core
    path, warp-level with "mma") against the oracle."""
    net = hz.learned.CoarseNet(seed=5)
    net.set_conv_path(path)
    w = net.get_weights()
    x, t = _x(2, 2, 25, 33)
    net.reset_kernel_times()
    loss, g = net.gradient(x, t)
    tc = path != "mma"
    assert _launches(net, "net_conv_bwd_tc") == (7 if tc else 0)  # data gradients of layers 1..7
    assert _launches(net, "net_wgrad_tc") == (8 if tc else 0) and _launches(net, "net_wgrad") == (0 if tc else 8)
    yo, cache = CN.forward(w, x.astype(np.float64), emulate=True)
    lo, go = CN.backward(cache, t.astype(np.float64))
    assert abs(loss - lo) <= 1e-3 * lo
    offs = np.cumsum([0] + [9 * a * b for a, b in CN.LAYERS])
    for k in range(8):
        a, b = g[offs[k]:offs[k + 1]], go[offs[k]:offs[k + 1]]
        assert _rel(a, b) <= 3e-2, (k, _rel(a, b))


def test_tcgen05_path_selection(hz):
    net = hz.learned.CoarseNet(seed=1)
    x, _ = _x(4, 1, 17, 17)
    net.reset_kernel_times()
    net.forward(x)  # the default path: the tensor cores for every 2D layer they support
    assert _launches(net, "net_conv_fwd_tc") == 7 and _launches(net, "net_conv_fwd") == 1
    with pytest.raises(KeyError):
        net.set_conv_path("wmma")


def _x3(seed, B, nz, ny, nx):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, nz, ny, nx, 4)).astype(np.float32)
    x[..., 2] = rng.uniform(0.5, 6.0, size=(B, nz, ny, nx))
    x[..., 3] = rng.uniform(0.01, 0.9, size=(B, nz, ny, nx))
    t = rng.normal(size=(B, nz, ny, nx, 2)).astype(np.float32)
    return x, t


@pytest.mark.parametrize("nz,ny,nx", [(9, 33, 17), (13, 21, 9)])
def test_tcgen05_3d_forward_matches_oracle_and_warp_mma(hz, nz, ny, nx):
    """3x3x3 convolutions: three z-planes per halo tile (the planes outside the grid
    zero-filled by the TMA unit), the 8-channel layers computed 16 wide."""
    import coarse_net3d as CN3
    net = hz.learned.CoarseNet3D(seed=11)
    w = net.get_weights()
    x, _ = _x3(1, 2, nz, ny, nx)
    net.set_conv_path("mma")
    y_mma = net.forward(x)
    net.set_conv_path("tcgen05")
    net.reset_kernel_times()
    y_tc = net.forward(x)
    # every layer on the tensor cores: y-line tiles, and z-line tiles for the last y-rows
    assert _launches(net, "net3_conv_fwd") == 0
    assert _launches(net, "net3_conv_fwd_tc") + _launches(net, "net3_conv_fwd_tc_zlines") >= 6
    assert _launches(net, "net3_conv_fwd_tc_zlines") >= 1
    yo, _ = CN3.forward(w, x.astype(np.float64), emulate=True)
    for b in range(x.shape[0]):
        assert _rel(y_tc[b], yo[b]) <= 1e-2, (b, _rel(y_tc[b], yo[b]))
        assert _rel(y_tc[b], y_mma[b]) <= 1e-2, (b, _rel(y_tc[b], y_mma[b]))


@pytest.mark.parametrize("path", ["tcgen05", "mma"])
def test_tcgen05_3d_gradient_matches_oracle(hz, path):
    import coarse_net3d as CN3
    net = hz.learned.CoarseNet3D(seed=5)
    net.set_conv_path(path)
    w = net.get_weights()
    x, t = _x3(2, 2, 9, 33, 17)
    net.reset_kernel_times()
    loss, g = net.gradient(x, t)
    if path == "tcgen05":  # data and weight gradients on the tensor cores
        assert _launches(net, "net3_conv_bwd") == 0 and _launches(net, "net3_wgrad") == 0
        assert _launches(net, "net3_conv_bwd_tc") + _launches(net, "net3_conv_bwd_tc_zlines") >= 5
        assert _launches(net, "net3_wgrad_tc") == 6
    else:
        assert _launches(net, "net3_wgrad") == 6 and _launches(net, "net3_wgrad_tc") == 0
    yo, cache = CN3.forward(w, x.astype(np.float64), emulate=True)
    lo, go = CN3.backward(cache, t.astype(np.float64))
    assert abs(loss - lo) <= 1e-3 * lo
    offs = np.cumsum([0] + [27 * a * b for a, b in CN3.LAYERS])
    for k in range(len(CN3.LAYERS)):
        a, b = g[offs[k]:offs[k + 1]], go[offs[k]:offs[k + 1]]
        assert _rel(a, b) <= 3e-2, (k, _rel(a, b))


def test_tcgen05_weight_images_follow_training(hz):
    """Adam steps and set_weights on the tensor-core path rewrite the weight
    images: afterwards both paths give the same forward output for the same
    weights."""
    import torch
    x, t = _x(3, 8, 17, 17)
    net = hz.learned.CoarseNet(seed=2)
    net.set_conv_path("tcgen05")
    hist = net.train(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda(), epochs=3, batch=4, lr=1e-3, seed=1)
    assert np.all(np.isfinite(hist))
    y_tc = net.forward(x)
    net.set_conv_path("mma")
    y_mma = net.forward(x)
    assert _rel(y_tc, y_mma) <= 1e-2, _rel(y_tc, y_mma)
    w = net.get_weights()
    net.set_weights(1.5 * w)
    y_mma = net.forward(x)
    for path in PATHS:
        net.set_conv_path(path)
        assert _rel(net.forward(x), y_mma) <= 1e-2, path


def test_auto_path_3d_picks_per_layer(hz):
    """The default path runs a 3D layer on the tensor cores where its tiles waste at
    most 3.5x the work on its grid: on a 17^3-node batch every layer but the one on
    the 5^3 level, which stays warp-level."""
    net = hz.learned.CoarseNet3D(seed=3)
    x, _ = _x3(6, 4, 17, 17, 17)
    net.reset_kernel_times()
    y_auto = net.forward(x)
    tc = _launches(net, "net3_conv_fwd_tc") + _launches(net, "net3_conv_fwd_tc_zlines")
    mma = _launches(net, "net3_conv_fwd")
    assert tc >= 1 and mma >= 1, (tc, mma)
    net.set_conv_path("mma")
    y_mma = net.forward(x)
    assert _rel(y_auto, y_mma) <= 1e-2
