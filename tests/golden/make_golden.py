"""Generate tests/golden/golden.npz from the CPU oracle (oracle/helmholtz_oracle.py).

The reference is Julia and cannot run in this container, so these vectors come
from the oracle's restatement of src/GetHelmholtz.jl, src/PlainNodalLaplacian.jl
and src/getPointSource.jl; the oracle itself is pinned by the reference's
manufactured-solution test (tests/test_oracle.py).  Run:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import helmholtz_oracle as O  # noqa: E402


def main():
    out = {}
    rng = np.random.default_rng(20240601)
    # 2D: 16 x 8 cells on [0, 2] x [0, 1], smooth random slowness
    M = O.getRegularMesh([0.0, 2.0, 0.0, 1.0], [16, 8])
    nn = M.n + 1
    N = int(np.prod(nn))
    v = 1.5 + 2.0 * rng.random(N)
    m = 1.0 / v**2
    w = O.getMaximalFrequency(m, M)
    out["m2"], out["w2"] = m, w
    for neu in (0, 1):
        out[f"abl2_neu{neu}"] = O.getABL(nn, bool(neu), [3, 2], 0.9 * w).ravel(order="F")
        out[f"somm2_neu{neu}"] = O.getSommerfeldBC(M, m, w, bool(neu)).ravel(order="F")
    H, g = O.GetHelmholtzOperatorABL(M, m, w, 0.01 * w * np.ones(N), True, [3, 2], 0.9 * w, True)
    out["gamma2"] = np.ravel(g, order="F")
    out["mass2"] = O.helmholtz_mass(M, m, w, g, True, True)
    X = rng.standard_normal((N, 3)) + 1j * rng.standard_normal((N, 3))
    out["X2"] = X
    out["HX2"] = H @ X
    SH = (H + O.GetHelmholtzShiftOP(m, w, 0.5)).tocsr()
    out["SHX2"] = SH @ X
    out["HadjX2"] = H.conj().T @ X
    out["Xsol2"] = O.direct_solve(H, X)
    # orderNeumannBC = 1 with Sommerfeld on: first-order Laplacian rows, and the
    # Sommerfeld term that src/GetHelmholtz.jl:45 builds with getSommerfeldBC's
    # default order 2 (:222), assembled term by term here
    L1 = O.getNodalLaplacianMatrix(M, 1).astype(np.complex128)
    mass1 = -(w**2) * m * (1.0 - 1j * out["gamma2"] / w) - O.getSommerfeldBC(M, m, w, True, 2).ravel(order="F")
    H1 = (L1 + sp.diags(mass1)).tocsr()
    out["HX2_bc1"] = H1 @ X
    q, _ = O.getAcousticPointSource(M, np.complex128)
    out["q2"] = q
    # 3D: 6 x 4 x 8 cells on [0,1.5]x[0,1]x[0,2]
    M3 = O.getRegularMesh([0.0, 1.5, 0.0, 1.0, 0.0, 2.0], [6, 4, 8])
    nn3 = M3.n + 1
    N3 = int(np.prod(nn3))
    m3 = 1.0 / (1.5 + 2.0 * rng.random(N3)) ** 2
    w3 = O.getMaximalFrequency(m3, M3)
    out["m3"], out["w3"] = m3, w3
    for neu in (0, 1):
        out[f"abl3_neu{neu}"] = O.getABL(nn3, bool(neu), [2, 2, 3], 0.9 * w3).ravel(order="F")
        out[f"somm3_neu{neu}"] = O.getSommerfeldBC(M3, m3, w3, bool(neu)).ravel(order="F")
    H3, g3 = O.GetHelmholtzOperatorABL(M3, m3, w3, [], False, [2, 2, 3], 0.9 * w3, True)
    out["gamma3"] = np.ravel(g3, order="F")
    X3 = rng.standard_normal((N3, 2)) + 1j * rng.standard_normal((N3, 2))
    out["X3"], out["HX3"] = X3, H3 @ X3
    out["HadjX3"] = H3.conj().T @ X3
    q3, _ = O.getAcousticPointSource(M3, np.complex128)
    out["q3"] = q3
    out["maxfreq_case"] = np.array([O.getMaximalFrequency(m3, M3)])
    np.savez_compressed(HERE / "golden.npz", **out)
    print("wrote", HERE / "golden.npz", sum(v.nbytes for v in out.values() if hasattr(v, "nbytes")), "bytes")


if __name__ == "__main__":
    main()
