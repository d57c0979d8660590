"""The premise of the double-float assembly's even-odd form (p = 2 and 3):
which elements' basis tables are centro-symmetric, N[k][b] = N[p-k][p-b] and
dN[k][b] = -dN[p-k][p-b], to 4e-15 of their largest entry (the criterion
the library applies per element).  Host tables only, no GPU."""
import numpy as np
import pytest

from ads_mpi_gb300 import ads as A


def symmetric_elements(NN, tol=4e-15):
    N, D = NN[..., 0], NN[..., 1]
    en = np.abs(N - N[:, ::-1, ::-1]).max(axis=(1, 2))
    ed = np.abs(D + D[:, ::-1, ::-1]).max(axis=(1, 2))
    return (en <= tol * np.abs(N).max(axis=(1, 2))) & (ed <= tol * np.abs(D).max(axis=(1, 2)))


@pytest.mark.parametrize("E,p", [(16, 2), (64, 2), (256, 2), (16, 3), (64, 3), (256, 3)])
def test_uniform_knots_interior_elements_are_symmetric(E, p):
    """1/E exact in FP32: every element but the first and last p - 1, whose
    basis the open knot vector's repeated end knots bend."""
    t = A.axis_setup(E + p - 1, p)
    sym = symmetric_elements(t["NN"].reshape(E, p + 1, p + 1, 2))
    assert sym[p - 1:E - p + 1].all()
    assert not sym[:p - 1].any() and not sym[E - p + 1:].any()


@pytest.mark.parametrize("E,p", [(24, 2), (96, 2), (96, 3)])
def test_fp32_rounded_knots_are_not_symmetric(E, p):
    """Knots i/E rounded to FP32 are not uniform: the general path runs."""
    t = A.axis_setup(E + p - 1, p)
    sym = symmetric_elements(t["NN"].reshape(E, p + 1, p + 1, 2))
    assert not sym[2:-2].all()
