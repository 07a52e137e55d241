"""Stencil launch-shape autotuner: the tuned shapes change how many right-hand
sides a block loops over, never the arithmetic of a column, so solutions are
bit-identical with and without tuning; the choice is reported per handle and
persisted to the file named by HELMGPU_TUNE_CACHE."""
import ctypes as C
import os

import numpy as np
import pytest

import problems as PB

pytestmark = pytest.mark.gpu


def _solver(hz, P, tune, precision):
    MG = hz.getMGparam(complex, int, 4, 1, 60, 1e-6, "Jac", 0.8, 1, 1, "V", "Julia", 0.5, 0.0, precision=precision)
    MG.autotune = tune
    return hz.getShiftedLaplacianMultigridSolver(PB.hz_param(hz, P), MG, 0.5, "GMRES", 10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_bit_identical_and_persisted(hz, tmp_path, precision):
    cache = tmp_path / "tune.txt"
    os.environ["HELMGPU_TUNE_CACHE"] = str(cache)
    try:
        P = PB.layered((136, 72), seed=7, pad=8, lengths=[2.0, 1.0])  # a size no other test uses
        B = PB.rhs(P["m"].size, 5, seed=3)
        S0 = _solver(hz, P, False, precision)
        X0, S0 = hz.solveLinearSystem(None, B, S0)
        S1 = _solver(hz, P, True, precision)
        X1, S1 = hz.solveLinearSystem(None, B, S1)
        np.testing.assert_array_equal(X1, X0)
        lib = hz._lib.load()
        f, r = C.c_int32(), C.c_int32()
        assert lib.hz_tune_info(S1._handle, C.byref(f), C.byref(r)) == 0
        assert lib.hz_tune_info(S0._handle, C.byref(f), C.byref(r)) == hz._lib.HZ_NOT_CONVERGED
        lines = cache.read_text().splitlines()
        assert len(lines) == 1 and "|137x73x1|c5|" in lines[0]
        # a second handle of the same problem takes the cached choice: nothing re-tuned
        S2 = _solver(hz, P, True, precision)
        X2, S2 = hz.solveLinearSystem(None, B, S2)
        np.testing.assert_array_equal(X2, X0)
        assert len(cache.read_text().splitlines()) == 1
    finally:
        os.environ.pop("HELMGPU_TUNE_CACHE", None)
