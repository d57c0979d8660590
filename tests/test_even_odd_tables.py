"""The premises of the double-float assembly's shortcuts.  The even-odd form
(p = 2 and 3): which elements' basis tables are centro-symmetric,
N[k][b] = N[p-k][p-b] and dN[k][b] = -dN[p-k][p-b], to 4e-15 of their
largest entry (the criterion the library applies per element).  The x bands
of the constant-conductivity increment: the element stiffness and mass
matrices summed per brick column.  Host tables only, no GPU."""
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


def element_matrices(t, p):
    """Each element's 1-D stiffness and mass matrices, the Gauss sums
    K[b][b'] = sum_k dN[k][b] dN[k][b'] J W(k), M likewise with N."""
    E = t["NN"].shape[0]
    NN = t["NN"].reshape(E, p + 1, p + 1, 2)
    jw = t["J"][:, None] * t["W"][None, :]
    K = np.einsum("ekb,ekc,ek->ebc", NN[..., 1], NN[..., 1], jw)
    M = np.einsum("ekb,ekc,ek->ebc", NN[..., 0], NN[..., 0], jw)
    return K, M


def brick_bands(m, x0, tx, p):
    """The band rows the constant-conductivity x stage applies, one per
    column x0 + c of a brick of elements x0 .. x0 + tx - 1 (c < tx + p):
    band[c][j] couples column x0 + c with x0 + c + j - p, summed over the
    brick's elements on that column."""
    E = m.shape[0]
    band = np.zeros((tx + p, 2 * p + 1))
    for c in range(tx + p):
        for b in range(p + 1):
            e = x0 + c - b
            if 0 <= c - b < tx and e < E:
                for cc in range(p + 1):
                    band[c, cc - b + p] += m[e, b, cc]
    return band


@pytest.mark.parametrize("E,p", [(40, 2), (96, 2), (40, 3), (61, 1), (45, 4)])
def test_x_bands_assemble_the_element_matrices(E, p):
    """The x stage of the constant-conductivity increment multiplies each row
    of points by the brick's stiffness and mass bands (32 - p elements a
    brick).  Over the bricks the bands add up to the 1-D matrices: M to the
    mass band the solve factorises, K with vanishing row sums; and a brick's
    band product equals the sum of its element products."""
    t = A.axis_setup(E + p - 1, p)
    K, M = element_matrices(t, p)
    N, tx = E + p, 32 - p
    for m, ref in ((M, t["band"][:, :N]), (K, None)):
        G = np.zeros((2 * p + 1, N))
        for x0 in range(0, E, tx):
            bb = brick_bands(m, x0, tx, p)
            for c in range(min(tx + p, N - x0)):
                G[:, x0 + c] += bb[c]
        if ref is not None:
            np.testing.assert_allclose(G, ref, rtol=0, atol=1e-15 * np.abs(ref).max())
        else:
            assert np.abs(G.sum(axis=0)).max() <= 1e-12 * np.abs(G).max()
        # one brick: the band product (reads outside the brick's columns
        # clamped into them, against zero coefficients) equals the sum of the
        # element products
        x0 = tx if E > tx else 0
        v = np.random.default_rng(5).standard_normal(tx + p)
        bb = brick_bands(m, x0, tx, p)
        got = np.array([sum(bb[c, j] * v[min(max(c + j - p, 0), tx + p - 1)] for j in range(2 * p + 1))
                        for c in range(tx + p)])
        want = np.zeros(tx + p)
        for e in range(x0, min(x0 + tx, E)):
            want[e - x0:e - x0 + p + 1] += m[e] @ v[e - x0:e - x0 + p + 1]
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(m).max())


@pytest.mark.parametrize("E,p", [(40, 2), (40, 3), (45, 4)])
def test_x_bands_equal_the_pointwise_x_stage(E, p):
    """The banded x stage and the pointwise one it replaces give the same
    H rows: interpolating a row's coefficients to each element's x points,
    weighting by Jx Wx and contracting with the test functions (values for
    the mass part, derivatives for the stiffness part), then adding the
    elements' contributions per DOF column."""
    t = A.axis_setup(E + p - 1, p)
    NN = t["NN"].reshape(E, p + 1, p + 1, 2)
    jw = t["J"][:, None] * t["W"][None, :]
    K, M = element_matrices(t, p)
    tx = 32 - p
    rng = np.random.default_rng(11)
    for x0 in range(0, E, tx):
        v = rng.standard_normal(tx + p)
        for d, m in ((1, K), (0, M)):
            point = np.zeros(tx + p)
            for e in range(x0, min(x0 + tx, E)):
                c = v[e - x0:e - x0 + p + 1]
                at_points = NN[e, :, :, d] @ c                      # interpolation to the x points
                point[e - x0:e - x0 + p + 1] += NN[e, :, :, d].T @ (jw[e] * at_points)  # weighted test
            bb = brick_bands(m, x0, tx, p)
            band = np.array([sum(bb[c, j] * v[min(max(c + j - p, 0), tx + p - 1)] for j in range(2 * p + 1))
                             for c in range(tx + p)])
            np.testing.assert_allclose(band, point, rtol=0, atol=1e-13 * np.abs(point).max())
