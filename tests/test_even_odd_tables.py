"""The premise of the double-float assembly's even-odd form (p = 2): which
elements' basis tables are centro-symmetric, N[k][b] = N[2-k][2-b] and
dN[k][b] = -dN[2-k][2-b], to 4e-15 of their largest entry (the criterion
the library applies per element).  Host tables only, no GPU."""
import numpy as np
import pytest

from ads_mpi_gb300 import ads as A


def symmetric_elements(NN, tol=4e-15):
    N, D = NN[..., 0], NN[..., 1]
    en = np.abs(N - N[:, ::-1, ::-1]).max(axis=(1, 2))
    ed = np.abs(D + D[:, ::-1, ::-1]).max(axis=(1, 2))
    return (en <= tol * np.abs(N).max(axis=(1, 2))) & (ed <= tol * np.abs(D).max(axis=(1, 2)))


@pytest.mark.parametrize("E", [16, 64, 256])
def test_uniform_knots_interior_elements_are_symmetric(E):
    """1/E exact in FP32: every element but the first and the last, whose
    basis the open knot vector's end knots bend."""
    t = A.axis_setup(E + 1, 2)
    sym = symmetric_elements(t["NN"].reshape(E, 3, 3, 2))
    assert sym[1:-1].all()
    assert not sym[0] and not sym[-1]


@pytest.mark.parametrize("E", [24, 96])
def test_fp32_rounded_knots_are_not_symmetric(E):
    """Knots i/E rounded to FP32 are not uniform: the general path runs."""
    t = A.axis_setup(E + 1, 2)
    sym = symmetric_elements(t["NN"].reshape(E, 3, 3, 2))
    assert not sym[2:-2].all()
