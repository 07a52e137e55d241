"""Seeded synthetic Helmholtz problems shared by the tests (small versions of
the measured workloads: gradient + ellipse 2D model, layered 2D/3D models)."""
from __future__ import annotations

import numpy as np

import helmholtz_oracle as O


def gradient_2d(nc=(64, 64), pad=8, neumann=True, sommerfeld=True):
    """2D [0,1]^2 model v = 1.5 + 3 z with the v=4.5 ellipse; w at 10 points
    per wavelength, quadratic absorbing layer (max 0.95 w) + attenuation 0.01 w."""
    M = O.getRegularMesh([0.0, 1.0, 0.0, 1.0], list(nc))
    nn = M.n + 1
    v = O.model_gradient_ellipse(nn, M.h)
    m = (1.0 / v**2).ravel(order="F")
    w = O.getMaximalFrequency(m, M)
    H, g = O.GetHelmholtzOperatorABL(M, m, w, 0.01 * w * np.ones(m.size), neumann, [pad, pad], 0.95 * w,
                                     sommerfeld)
    return dict(M=M, m=m, w=w, gamma=np.ravel(g, order="F"), H=H, neumann=neumann, sommerfeld=sommerfeld)


def layered(nc, seed=1, pad=6, neumann=True, sommerfeld=True, ellipsoid=False, lengths=None):
    dim = len(nc)
    lengths = lengths or [1.0] * dim
    dom = []
    for L_ in lengths:
        dom += [0.0, L_]
    M = O.getRegularMesh(dom, list(nc))
    nn = M.n + 1
    v = O.model_layered(nn, seed, ellipsoid=ellipsoid)
    m = (1.0 / v**2).ravel(order="F")
    w = O.getMaximalFrequency(m, M)
    H, g = O.GetHelmholtzOperatorABL(M, m, w, 0.01 * w * np.ones(m.size), neumann, [pad] * dim, 0.95 * w,
                                     sommerfeld)
    return dict(M=M, m=m, w=w, gamma=np.ravel(g, order="F"), H=H, neumann=neumann, sommerfeld=sommerfeld)


def operator_from_parts(P, order):
    """H assembled term by term as src/GetHelmholtz.jl:36-49 writes it, without
    the oracle's helmholtz_mass: the order-`order` nodal Laplacian, the mass
    -w^2 m (1 - i gamma / Re w), and the Sommerfeld term of getSommerfeldBC called
    with no order argument (:45), i.e. its default order 2 (:222)."""
    import scipy.sparse as sp
    M, m, w = P["M"], P["m"], P["w"]
    L = O.getNodalLaplacianMatrix(M, order).astype(np.complex128)
    mass = -(w**2) * m * (1.0 - 1j * P["gamma"] / np.real(w))
    if P["sommerfeld"]:
        mass = mass - O.getSommerfeldBC(M, m, np.real(w), P["neumann"], 2).ravel(order="F")
    return (L + sp.diags(mass)).tocsr()


def rhs(n, nrhs, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))


def hz_param(hz, P):
    Mo = P["M"]
    M = hz.getRegularMesh(Mo.domain, Mo.n)
    return hz.HelmholtzParam(M, P["gamma"], P["m"], P["w"], P["neumann"], P["sommerfeld"])
