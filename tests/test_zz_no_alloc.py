"""The allocation-free operator apply (hz_apply_noalloc) gives the same result
as hz_apply.

hz_apply_noalloc exists for callers that cannot allocate GPU memory when they
apply the operator (their own pool already holds the device, their footprint
must stay fixed, or they must avoid cudaMalloc's device-wide synchronisation);
it keeps its scratch column list in a static device array instead.  This file
is collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

import problems as PB

pytestmark = pytest.mark.gpu
TOL64 = 1e-13  # the FP64 apply tolerance of the operator tests


def _handle(hz, P):
    L = hz._lib
    lib = L.load()
    p, keep = hz.api._problem(PB.hz_param(hz, P))
    o = L.hz_options()
    lib.hz_default_options(C.byref(o))
    h = C.c_void_p()
    L.check(lib.hz_create(C.byref(p), C.byref(o), C.byref(h)))
    return lib, h, keep


@pytest.mark.parametrize("case", ["2d", "3d"])
def test_apply_noalloc_matches_apply(hz, case):
    import torch
    L = hz._lib
    P = PB.gradient_2d((48, 40), pad=5) if case == "2d" else PB.layered((16, 12, 20), seed=8, pad=3)
    lib, h, keep = _handle(hz, P)
    try:
        n = P["m"].size
        nrhs = 5
        X = torch.from_numpy(np.ascontiguousarray(PB.rhs(n, nrhs, seed=31).T)).to("cuda")  # column-major n x nrhs
        for op, adj in ((L.HZ_OP_H, 0), (L.HZ_OP_SH, 0), (L.HZ_OP_H, 1), (L.HZ_OP_SH, 1)):
            Yref = torch.empty_like(X)
            L.check(lib.hz_apply(h, op, adj, X.data_ptr(), Yref.data_ptr(), n, nrhs, L.HZ_MEM_DEVICE), h)
            ref = Yref.cpu().numpy()
            for _ in range(2):  # two calls in a row share the static scratch
                Y = torch.full_like(X, complex(float("nan"), float("nan")))
                # X and Y must be complete before the call (the fill runs on torch's stream)
                torch.cuda.synchronize()
                rc = lib.hz_apply_noalloc(h, op, adj, X.data_ptr(), Y.data_ptr(), n, nrhs)
                assert rc == L.HZ_OK, lib.hz_last_error(h)
                got = Y.cpu().numpy()
                assert np.all(np.isfinite(got))
                assert np.linalg.norm(got - ref) <= TOL64 * np.linalg.norm(ref)
        # more columns than the static scratch holds: a clear error, nothing launched
        big = L.HZ_NOALLOC_MAX_COLS + 1
        Y = torch.empty_like(X)
        rc = lib.hz_apply_noalloc(h, L.HZ_OP_H, 0, X.data_ptr(), Y.data_ptr(), n, big)
        assert rc == L.HZ_ERR_ARG
        assert b"columns" in lib.hz_last_error(h)
        # in place (X and Y overlapping) is refused by both entry points
        rc = lib.hz_apply_noalloc(h, L.HZ_OP_H, 0, X.data_ptr(), X.data_ptr(), n, nrhs)
        assert rc == L.HZ_ERR_ARG and b"overlap" in lib.hz_last_error(h)
        rc = lib.hz_apply(h, L.HZ_OP_H, 0, X.data_ptr(), X.data_ptr() + 16, n, nrhs, L.HZ_MEM_DEVICE)
        assert rc == L.HZ_ERR_ARG and b"overlap" in lib.hz_last_error(h)
    finally:
        lib.hz_destroy(h)
