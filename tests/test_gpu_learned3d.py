"""GPU tests of the 3D learned coarse-grid correction.

* The 3D network's kernels (BF16 tensor-core 3x3x3 convolutions, FP32
  accumulation, trilinear transfers) against the CPU oracle
  (oracle/coarse_net3d.py, BF16 rounding emulated at the same points): forward
  output to relative L2 error <= 1e-2, loss to <= 1e-3, the weight gradient of
  every layer to <= 3e-2 (FP32 summation order can flip a BF16 rounding).
* Pairs from the FP64 solver on a 3D hierarchy (targets from restarted two-step
  FGMRES corrections on the network's level), training on the GPU, and the trained
  network inside FGMRES: the learned form reaches the stopping residual with
  error <= 1e-4 against the direct solution, in fewer iterations than the same
  solver without the network.
"""
import numpy as np
import pytest

import coarse_net3d as CN3
import problems as PB

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _x(seed, B=2, nz=9, ny=13, nx=17):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, nz, ny, nx, 4)).astype(np.float32)
    x[..., 2] = rng.uniform(0.5, 6.0, size=(B, nz, ny, nx))   # w^2 m h^2
    x[..., 3] = rng.uniform(0.01, 0.9, size=(B, nz, ny, nx))  # gamma / w
    t = rng.normal(size=(B, nz, ny, nx, 2)).astype(np.float32)
    return x, t


def test_forward_matches_oracle(hz):
    net = hz.learned.CoarseNet3D(seed=11)
    w = net.get_weights()
    assert w.size == CN3.num_params() == hz.learned.num_params_3d()
    assert hz.learned.layer_shapes_3d() == CN3.LAYERS
    x, _ = _x(1)
    y = net.forward(x)
    yo, _ = CN3.forward(w, x.astype(np.float64), emulate=True)
    for b in range(x.shape[0]):
        assert _rel(y[b], yo[b]) <= 1e-2, (b, _rel(y[b], yo[b]))
    import torch
    yd = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    np.testing.assert_array_equal(yd, y)


def test_weights_roundtrip_and_file(hz, tmp_path):
    net = hz.learned.CoarseNet3D(seed=2)
    w = CN3.he_init(9)
    net.set_weights(w)
    np.testing.assert_array_equal(net.get_weights(), w)
    with pytest.raises(ValueError):
        net.set_weights(w[:-1])
    p = tmp_path / "net3.bin"
    net.save(p)
    assert hz.learned.file_info(p) == (CN3.num_params(), 0)
    other = hz.learned.CoarseNet3D(seed=3)
    other.load(p)
    np.testing.assert_array_equal(other.get_weights(), w)
    # a 2D network refuses the 3D file
    with pytest.raises(Exception):
        hz.learned.CoarseNet(seed=1).load(p)


def test_gradient_matches_oracle(hz):
    net = hz.learned.CoarseNet3D(seed=5)
    w = net.get_weights()
    x, t = _x(2, B=2)
    loss, g = net.gradient(x, t)
    yo, cache = CN3.forward(w, x.astype(np.float64), emulate=True)
    lo, go = CN3.backward(cache, t.astype(np.float64))
    assert abs(loss - lo) <= 1e-3 * lo
    offs = np.cumsum([0] + [27 * a * b for a, b in CN3.LAYERS])
    for k in range(len(CN3.LAYERS)):
        a, b = g[offs[k]:offs[k + 1]], go[offs[k]:offs[k + 1]]
        assert _rel(a, b) <= 3e-2, (k, _rel(a, b))
    np.testing.assert_array_equal(net.get_weights(), w)


def _sources3(P, k, seed, pad):
    """k unit point sources at seeded positions outside the absorbing layer of a 3D grid."""
    rng = np.random.default_rng(seed)
    nn = P["M"].n + 1
    h = P["M"].h
    B = np.zeros((int(np.prod(nn)), k), dtype=np.complex128)
    for c in range(k):
        i = rng.integers(pad, nn[0] - pad)
        j = rng.integers(pad, nn[1] - pad)
        kk = rng.integers(1, nn[2] - pad)
        B[i + nn[0] * (j + nn[1] * kk), c] = 1.0 / (h[0] * h[1])
    return B


def _solver(hz, P, precision, cycle="V", levels=4, tol=1e-6, max_outer=60):
    MG = hz.getMGparam(complex, int, levels, 1, max_outer, tol, "Jac-GMRES", 0.8, 1, 1, cycle, "Julia", 0.3, 0.0,
                       precision=precision, relaxFrom=1)
    return hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.3, "GMRES", 10)


@pytest.fixture(scope="module")
def trained3(hz):
    """A 3D network trained on pairs from twelve seeded layered+ellipsoid models (33^3
    nodes, four levels, V-cycle with GMRES smoothing from level 1; the network
    replaces the correction below level 2 = 9^3).  With the K-cycle the plain
    correction there is already within a couple of iterations of an exact
    level-2 solve (CPU oracle: 20 against 19), so the V-cycle is where a
    correction below level 2 has something to gain (49 against 23)."""
    import torch
    xs, ts, pes = [], [], []
    for seed in range(31, 43):
        P = PB.layered((32, 32, 32), seed=seed, pad=4, ellipsoid=True)
        S = _solver(hz, P, "fp64")
        d = hz.learned.collect_pairs(S, _sources3(P, 4, seed, 4), level=2, sweeps=12, max_pairs=400)
        assert d["x"].shape[1:] == (9, 9, 9, 4)
        assert d["target_relres"] < 1e-3, d["target_relres"]
        xs.append(d["x"])
        ts.append(d["t"])
        pes.append(d["plain_err"])
    x = torch.cat(xs).contiguous()
    t = torch.cat(ts).contiguous()
    net = hz.learned.CoarseNet3D(seed=1)
    hist = net.train(x, t, epochs=60, batch=16, lr=3e-3, seed=3)
    return net, x, t, np.concatenate(pes), hist


def test_training_lowers_loss_3d(hz, trained3):
    net, x, t, plain_err, hist = trained3
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.5 * hist[0], hist
    err = hz.learned.pair_errors(net, x, t)
    print(f"3D loss {hist[0]:.3f} -> {hist[-1]:.3f}; median pair error: network {np.median(err):.3f}, "
          f"plain correction {np.median(plain_err):.3f}")
    assert np.median(err) < 0.7, np.median(err)


def test_learned_3d_solve_beats_plain_cycle(hz, O, trained3):
    """Held-out model: the same solver with and without the network below level 2."""
    net = trained3[0]
    P = PB.layered((32, 32, 32), seed=77, pad=4, ellipsoid=True)
    B = _sources3(P, 4, 77, 4)
    Xref = O.direct_solve(P["H"], B)
    iters = {}
    for name, use_net in (("plain", False), ("learned", True)):
        S = _solver(hz, P, "mixed")
        if use_net:
            hz.learned.attach(S, net, level=2, stag_ratio=0.95)
        X, S = hz.solveLinearSystem(None, B, S)
        assert S.last_relres.max() <= 1e-6
        assert max(_rel(X[:, c], Xref[:, c]) for c in range(B.shape[1])) <= 1e-4
        iters[name] = float(np.mean(S.last_iters))
        if use_net:
            calls, _ = hz.learned.learned_stats(S)
            assert calls > 0
    print(f"3D held-out iterations: {iters}")
    assert iters["learned"] < iters["plain"], iters


def test_pairs_on_the_coarsest_level(hz):
    """On the coarsest level the cycle is the band LU: its solve is the target
    (residual at rounding level) and one plain cycle equals it."""
    P = PB.layered((32, 32, 32), seed=5, pad=4, ellipsoid=True)
    S = _solver(hz, P, "fp64", levels=4)  # 33^3, 17^3, 9^3, 5^3
    d = hz.learned.collect_pairs(S, _sources3(P, 2, 5, 4), level=3, sweeps=5, max_pairs=16)
    assert d["x"].shape[1:] == (5, 5, 5, 4)
    assert d["target_relres"] < 1e-10, d["target_relres"]
    assert np.max(d["plain_err"]) < 1e-12
