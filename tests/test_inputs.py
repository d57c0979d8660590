"""Seeded synthetic inputs are deterministic and have the stated statistics."""
import numpy as np

from ads_mpi_gb300 import inputs


def test_inputs_are_seeded():
    x = np.linspace(0, 1, 11)[:, None, None]
    y = np.linspace(0, 1, 7)[None, :, None]
    z = np.linspace(0, 1, 5)[None, None, :]
    for fn in (inputs.projection_target, inputs.gaussian_bumps, inputs.gaussian_random_field):
        a = fn(x, y, z, seed=3)
        b = fn(x, y, z, seed=3)
        c = fn(x, y, z, seed=4)
        assert np.array_equal(a, b)
        assert not np.array_equal(a, c)


def test_grf_statistics():
    g = np.linspace(0, 1, 40, endpoint=False)
    x, y, z = g[:, None, None], g[None, :, None], g[None, None, :]
    f = inputs.gaussian_random_field(x, y, z, seed=0, sigma=0.5, corr=0.1, grid=40)
    assert abs(f.std() - 0.5) < 0.05
    # correlation at lag 0.1 ~ exp(-1/2)
    lag = 4
    c = np.mean((f - f.mean()) * (np.roll(f, lag, axis=0) - f.mean())) / f.var()
    assert 0.4 < c < 0.8


def test_bumps_are_positive_and_bounded():
    g = np.linspace(0, 1, 21)
    x, y, z = g[:, None, None], g[None, :, None], g[None, None, :]
    f = inputs.gaussian_bumps(x, y, z, seed=0)
    assert f.min() >= 0.0 and f.max() < 16.0


def test_separable_bumps_match_direct():
    E, q = 5, 3
    rng = np.random.default_rng(0)
    Xx = np.sort(rng.uniform(0, 1, (E, q)), axis=None).reshape(E, q)
    Xy = np.sort(rng.uniform(0, 1, (E + 1, q)), axis=None).reshape(E + 1, q)
    Xz = np.sort(rng.uniform(0, 1, (E + 2, q)), axis=None).reshape(E + 2, q)
    x = Xx[None, None, :, None, None, :]
    y = Xy[None, :, None, None, :, None]
    z = Xz[:, None, None, :, None, None]
    a = inputs.gaussian_bumps(x, y, z, seed=5)
    b = inputs.gaussian_bumps_separable(Xx, Xy, Xz, seed=5)
    assert a.shape == b.shape
    assert np.abs(a - b).max() < 1e-13


def test_random_field_on_qp_grid_matches_pointwise():
    """The separable quadrature-grid evaluation of the Gaussian random field
    equals the pointwise trilinear evaluation at the same points."""
    from ads_mpi_gb300 import inputs
    rng = np.random.default_rng(3)
    q = 3
    Xx, Xy, Xz = (np.sort(rng.uniform(0, 1, (e, q)), axis=None).reshape(e, q) for e in (4, 3, 5))
    a = inputs.gaussian_random_field_qp(Xx, Xy, Xz, seed=1, grid=16)
    x = Xx[None, None, :, None, None, :]
    y = Xy[None, :, None, None, :, None]
    z = Xz[:, None, None, :, None, None]
    b = inputs.gaussian_random_field(x, y, z, seed=1, grid=16)
    assert a.shape == (5, 3, 4, q, q, q)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
