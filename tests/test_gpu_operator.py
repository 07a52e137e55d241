"""GPU parity of the matrix-free operator apply (kernel K-a) against the
oracle's assembled sparse operators (src/GetHelmholtz.jl:33-50, 81-95)."""
from pathlib import Path

import numpy as np
import pytest

import problems as PB

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "golden.npz"
# FP64 stencil vs CSR product: same terms, different summation order
TOL64 = 1e-13


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_apply_matches_golden_2d_3d(hz):
    g = np.load(GOLD)
    M = hz.getRegularMesh([0.0, 2.0, 0.0, 1.0], [16, 8])
    w = float(g["w2"])
    H, gam = hz.GetHelmholtzOperator(M, g["m2"], w, 0.01 * w * np.ones(g["m2"].size), True, [3, 2], 0.9 * w, True)
    np.testing.assert_allclose(np.ravel(gam, order="F"), g["gamma2"], rtol=1e-15, atol=1e-15 * w)
    assert _rel(H @ g["X2"], g["HX2"]) < TOL64
    assert _rel(H.H @ g["X2"], g["HadjX2"]) < TOL64
    SH = H + hz.GetHelmholtzShiftOP(g["m2"], w, 0.5)
    assert _rel(SH @ g["X2"], g["SHX2"]) < TOL64
    # orderNeumannBC = 1 with Sommerfeld on (order-2 Sommerfeld term, src/GetHelmholtz.jl:45)
    H1 = hz.GetHelmholtzOperator(hz.HelmholtzParam(M, gam, g["m2"], w, True, True), 1)
    assert _rel(H1 @ g["X2"], g["HX2_bc1"]) < TOL64
    M3 = hz.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    w3 = float(g["w3"])
    H3, _ = hz.GetHelmholtzOperator(M3, g["m3"], w3, [], False, [2, 2, 3], 0.9 * w3, True)
    assert _rel(H3 @ g["X3"], g["HX3"]) < TOL64
    assert _rel(H3.H @ g["X3"], g["HadjX3"]) < TOL64


@pytest.mark.parametrize("case", ["2d_neumann", "2d_dirichlet_somm", "3d", "3d_wide", "2d_bc1", "2d_bc1_somm",
                                  "3d_bc1_somm"])
def test_apply_matches_oracle_sparse(hz, O, case):
    if case == "3d":
        P = PB.layered((20, 12, 16), seed=4, pad=3, ellipsoid=True)
    elif case == "3d_wide":
        # more than a warp of nodes along x, sizes that divide nothing evenly
        P = PB.layered((40, 18, 20), seed=4, pad=3, ellipsoid=True)
    elif case == "3d_bc1_somm":
        P = PB.layered((20, 12, 16), seed=6, pad=3, neumann=False, ellipsoid=True)
    elif case in ("2d_dirichlet_somm", "2d_bc1_somm"):
        P = PB.gradient_2d((40, 24), pad=5, neumann=False, sommerfeld=True)
    else:
        P = PB.gradient_2d((40, 24), pad=5, neumann=True, sommerfeld=(case == "2d_neumann"))
    order = 1 if "bc1" in case else 2
    Mo = P["M"]
    Ho = O.GetHelmholtzOperator(Mo, P["m"], P["w"], P["gamma"], P["neumann"], P["sommerfeld"], order)
    if "bc1_somm" in case:
        # the operator assembled term by term, not through the oracle's mass helper:
        # first-order Laplacian rows, order-2 Sommerfeld term (src/GetHelmholtz.jl:45)
        Ho = PB.operator_from_parts(P, order)
    p = PB.hz_param(hz, P)
    H = hz.GetHelmholtzOperator(p, order)
    X = PB.rhs(Ho.shape[0], 5, seed=11)
    assert _rel(H @ X, Ho @ X) < TOL64
    assert _rel(H.H @ X, Ho.conj().T @ X) < TOL64
    # getHelmholtzFun(SH', Shift) evaluates H; with (SH, -Shift) it evaluates H^H
    Sh = hz.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)
    SH = H + Sh
    Hfun = hz.getHelmholtzFun(SH.H, Sh)
    assert _rel(Hfun(X), Ho @ X) < TOL64
    HfunT = hz.getHelmholtzFun(SH, -Sh)
    assert _rel(HfunT(X[:, 0]), Ho.conj().T @ X[:, 0]) < TOL64
    SHo = (Ho + O.GetHelmholtzShiftOP(P["m"], P["w"], 0.5)).tocsr()
    assert _rel(SH @ X, SHo @ X) < TOL64
    assert _rel(SH.H @ X, SHo.conj().T @ X) < TOL64


def test_apply_linearity_large(hz, O):
    """Size-independent check at a larger 2D grid: A(aX + bY) = a AX + b AY, and
    the apply on a device tensor equals the host path."""
    import torch
    P = PB.layered((512, 256), seed=5, pad=16)
    p = PB.hz_param(hz, P)
    H = hz.GetHelmholtzOperator(p)
    n = P["m"].size
    X = PB.rhs(n, 2, seed=1)
    a, b = 0.3 - 1.1j, 2.0 + 0.5j
    lhs = H @ (a * X[:, 0] + b * X[:, 1])
    HX = H @ X
    assert _rel(lhs, a * HX[:, 0] + b * HX[:, 1]) < 1e-13
    Xd = torch.from_numpy(X).to("cuda")
    Yd = H @ Xd
    np.testing.assert_array_equal(Yd.cpu().numpy(), HX)
