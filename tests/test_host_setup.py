"""Host logic of the product without a GPU: the setup tables that ads_create
uploads (ads_axis_setup) against the oracle, FP32-rounded knots, and the LU
factor rows of the banded sweeps."""
import numpy as np
import pytest


@pytest.mark.parametrize("E,p", [(2, 1), (8, 2), (32, 2), (96, 2), (13, 3), (7, 4), (128, 2), (256, 3)])
def test_tables_match_oracle(ads_mod, oracle_mod, E, p):
    n = E + p - 1
    t = ads_mod.axis_setup(n, p)
    o = oracle_mod.Oracle((n, p, p), (p, p, p)) if False else oracle_mod.Oracle((n, n, n), (p, p, p))
    ot = o.axis_tables(0)
    assert np.array_equal(t["U"], ot["U"])
    assert np.array_equal(t["O"], ot["O"])
    assert np.array_equal(t["J"], ot["J"])
    assert np.array_equal(t["W"], ot["W"])
    assert np.abs(t["X"] - ot["X"]).max() < 1e-15
    assert np.abs(t["NN"][..., 0] - ot["NN"][..., 0]).max() < 1e-14
    assert np.abs(t["NN"][..., 1] - ot["NN"][..., 1]).max() < 1e-13 * E


def test_knots_are_fp32_rounded(ads_mod):
    """src/knot_vector.F90:88-90 divides default-kind REALs: at E = 96 the
    knots differ from k/96 in FP64 (by up to ~2e-8)."""
    t = ads_mod.axis_setup(97, 2)
    k = np.arange(1, 96)
    interior = t["U"][3:98]
    assert np.array_equal(interior, (k.astype(np.float32) / np.float32(96)).astype(np.float64))
    assert np.abs(interior - k / 96.0).max() > 1e-9


@pytest.mark.parametrize("E,p", [(9, 1), (16, 2), (11, 3), (6, 4)])
def test_factor_rows_solve_the_mass_matrix(ads_mod, E, p):
    n = E + p - 1
    N = n + 1
    t = ads_mod.axis_setup(n, p)
    M = np.zeros((N, N))
    for m in range(-p, p + 1):
        for i in range(N):
            if 0 <= i + m < N:
                M[i, i + m] = t["band"][m + p, i]
    assert np.allclose(M, M.T, rtol=0, atol=1e-17)
    rng = np.random.default_rng(E)
    b = rng.standard_normal(N)

    def sweep(fac, b):
        y = np.zeros(N)
        for i in range(N):
            acc = fac[0, i] * b[i]
            for m in range(1, p + 1):
                if i - m >= 0:
                    acc -= fac[m, i] * y[i - m]
            y[i] = acc
        x = np.zeros(N)
        for i in range(N - 1, -1, -1):
            acc = fac[p + 1, i] * y[i]
            for m in range(1, p + 1):
                if i + m < N:
                    acc -= fac[p + 1 + m, i] * x[i + m]
            x[i] = acc
        return x

    x = sweep(t["fac"], b)
    assert np.abs(M @ x - b).max() < 1e-12 * np.abs(b).max() / M.diagonal().min()
    xt = sweep(t["tfac"], b)
    assert np.abs(M.T @ xt - b).max() < 1e-12 * np.abs(b).max() / M.diagonal().min()


def test_unsupported_degree_is_rejected(ads_mod):
    with pytest.raises(ads_mod.ADSError) as e:
        ads_mod.axis_setup(10, 5)
    assert e.value.status == 7
