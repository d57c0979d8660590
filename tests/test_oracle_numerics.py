"""CPU checks of the oracle: the reference's L2-projection known answer, Gauss
exactness, partition of unity, polynomial reproduction, the banded solve
against LAPACK (scipy), the reorders, and the heat assembly against explicit
Kronecker-product matrices."""
import numpy as np
import pytest

from conftest import rel_l2


@pytest.mark.parametrize("q", range(1, 11))
def test_gauss_exactness(oracle_mod, q):
    X, W = oracle_mod.gauss_rule(q)
    for deg in range(2 * q):
        exact = 0.0 if deg % 2 else 2.0 / (deg + 1)
        assert abs(np.dot(W, X ** deg) - exact) < 1e-13


@pytest.mark.parametrize("E,p", [(4, 1), (5, 2), (7, 3), (6, 4), (32, 2)])
def test_partition_of_unity(oracle_mod, E, p):
    o = oracle_mod.Oracle((E + p - 1,) * 3, (p,) * 3)
    t = o.axis_tables(0)
    NN = t["NN"]  # (E, q, p+1, 2)
    assert np.abs(NN[..., 0].sum(-1) - 1.0).max() < 1e-14
    assert np.abs(NN[..., 1].sum(-1)).max() < 1e-10 * E


@pytest.mark.parametrize("E,p", [(4, 1), (6, 2), (5, 3), (32, 2)])
def test_l2_projection_known_answer(oracle_mod, E, p):
    """problems/L2Projection/main.F90:62,72-78: projecting f == 1 gives every
    coefficient 1 and l2norm 1, within 1e-10."""
    o = oracle_mod.Oracle((E + p - 1,) * 3, (p,) * 3)
    l2 = o.step(oracle_mod.FORM_PROJECT)
    assert abs(l2 - 1.0) < 1e-10
    assert np.abs(o.coeffs() - 1.0).max() < 1e-10


@pytest.mark.parametrize("p", [1, 2, 3])
def test_projection_reproduces_linear_function(oracle_mod, p):
    """Projecting f = x gives the Greville abscissae as coefficients."""
    E = 6
    n = E + p - 1
    o = oracle_mod.Oracle((n, n, n), (p, p, p))
    X = o.axis_tables(0)["X"]  # (E, q)
    q = p + 1
    x = np.broadcast_to(X[None, None, :, None, None, :], (E, E, E, q, q, q))
    o.step(oracle_mod.FORM_PROJECT, fqp=np.ascontiguousarray(x))
    U = o.axis_tables(0)["U"]
    grev = np.array([U[i + 1:i + p + 1].mean() for i in range(n + 1)])
    u = o.coeffs().reshape(n + 1, n + 1, n + 1)
    assert np.abs(u - grev[None, None, :]).max() < 1e-12


@pytest.mark.parametrize("kl,n,sym", [(1, 12, True), (2, 30, True), (3, 25, False), (2, 40, False)])
def test_banded_solve_matches_lapack(oracle_mod, kl, n, sym):
    scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
    rng = np.random.default_rng(kl * 100 + n)
    ku = kl
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            A[i, j] = rng.uniform(-1, 1)
    if sym:
        A = A + A.T + 4 * kl * np.eye(n)
    AB = np.zeros((2 * kl + ku + 1, n))
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            AB[kl + ku + i - j, j] = A[i, j]
    B = rng.standard_normal((n, 3))
    info, X, piv = oracle_mod.dgbsv(AB, kl, ku, B)
    assert info == 0
    lub, piv2, x2, info2 = scipy_lapack.dgbsv(kl, ku, AB.copy(), B.copy())
    assert info2 == 0
    assert np.abs(X - x2).max() < 1e-12 * max(1.0, np.abs(x2).max())
    assert np.abs(A @ X - B).max() < 1e-10


def test_mass_band_is_spd_and_unpivoted(oracle_mod):
    o = oracle_mod.Oracle((33, 33, 33), (2, 2, 2))
    AB = o.mkbbt_band(0)
    p, n1 = 2, 34
    M = np.zeros((n1, n1))
    for j in range(n1):
        for i in range(max(0, j - p), min(n1, j + p + 1)):
            M[i, j] = AB[2 * p + i - j, j]
    assert np.allclose(M, M.T, atol=1e-16)
    assert np.linalg.eigvalsh(M).min() > 0
    o.step(oracle_mod.FORM_PROJECT)
    assert o.pivoted() == (0, 0, 0)


@pytest.mark.parametrize("s", [(5, 4, 3), (7, 7, 7), (3, 6, 2)])
def test_reorders_are_the_reference_permutations(oracle_mod, s):
    rng = np.random.default_rng(1)
    F = rng.standard_normal(int(np.prod(s)))
    Fa = F.reshape(s[2], s[1], s[0])          # [z][y][x]
    F2 = oracle_mod.reorder("y", s, F)        # F2(y, x + z*Nx)
    assert np.array_equal(F2.reshape(s[2], s[0], s[1]), Fa.transpose(0, 2, 1))
    F3 = oracle_mod.reorder("z", s, F2)       # F3(z, x + y*Nx)
    assert np.array_equal(F3.reshape(s[1], s[0], s[2]), Fa.transpose(1, 2, 0))
    Fb = oracle_mod.reorder("x", s, F3)
    assert np.array_equal(Fb, F)


def _dense_1d(o, axis):
    t = o.axis_tables(axis)
    NN, J, W, O = t["NN"], t["J"], t["W"], t["O"]
    E, q, pp1, _ = NN.shape
    n1 = o.ndof[axis]
    M = np.zeros((n1, n1))
    K = np.zeros((n1, n1))
    for e in range(E):
        for k in range(q):
            v = NN[e, k, :, 0]
            d = NN[e, k, :, 1]
            sl = slice(O[e], O[e] + pp1)
            M[sl, sl] += J[e] * W[k] * np.outer(v, v)
            K[sl, sl] += J[e] * W[k] * np.outer(d, d)
    return M, K


@pytest.mark.parametrize("E,p", [(4, 2), (3, 3), (5, 1)])
def test_heat_assembly_equals_kronecker_operator(oracle_mod, E, p):
    """With exact Gauss quadrature, Form3DRHS of the heat form is
    F = (Mz x My x Mx) u - dt (Kz x My x Mx + Mz x Ky x Mx + Mz x My x Kx) u."""
    n = E + p - 1
    o = oracle_mod.Oracle((n, n, n), (p, p, p))
    rng = np.random.default_rng(E + p)
    u = rng.standard_normal(o.N)
    o.set_coeffs(u)
    dt = 1e-3
    F, l2 = o.assemble(oracle_mod.FORM_HEAT, kappa=1.3, dt=dt)
    Mx, Kx = _dense_1d(o, 0)
    M3 = np.kron(np.kron(Mx, Mx), Mx)
    K3 = (np.kron(np.kron(Kx, Mx), Mx) + np.kron(np.kron(Mx, Kx), Mx) + np.kron(np.kron(Mx, Mx), Kx))
    expect = M3 @ u - dt * 1.3 * (K3 @ u)
    assert rel_l2(F, expect) < 1e-13
    assert abs(l2 - u @ (M3 @ u)) < 1e-12 * abs(u @ (M3 @ u))


def test_heat_step_with_zero_dt_is_identity(oracle_mod):
    o = oracle_mod.Oracle((6, 6, 6), (2, 2, 2))
    u = np.random.default_rng(3).standard_normal(o.N)
    o.set_coeffs(u)
    o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=0.0)
    assert rel_l2(o.coeffs(), u) < 1e-13


def test_mass_apply_matches_dense(oracle_mod):
    o = oracle_mod.Oracle((5, 5, 5), (2, 2, 2))
    u = np.random.default_rng(4).standard_normal(o.N)
    Mx, _ = _dense_1d(o, 0)
    M3 = np.kron(np.kron(Mx, Mx), Mx)
    assert rel_l2(o.apply_mass(u), M3 @ u) < 1e-14


def test_oracle_adjoint_matches_finite_differences(oracle_mod):
    o = oracle_mod.Oracle((5, 5, 5), (2, 2, 2))
    rng = np.random.default_rng(5)
    u0 = rng.standard_normal(o.N)
    ut = rng.standard_normal(o.N)
    kq = np.exp(0.3 * rng.standard_normal(o.nqp))
    dt, K = 2e-3, 3
    loss, g, gk = o.heat_adjoint(K, u0, ut, kappa_qp=kq, dt=dt, want_kappa_grad=True)
    for trial in range(3):
        d = rng.standard_normal(o.N)
        h = 1e-6
        lp, _, _ = o.heat_adjoint(K, u0 + h * d, ut, kappa_qp=kq, dt=dt, want_grad=False)
        lm, _, _ = o.heat_adjoint(K, u0 - h * d, ut, kappa_qp=kq, dt=dt, want_grad=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(fd))
        dk = rng.standard_normal(o.nqp) * kq
        lp, _, _ = o.heat_adjoint(K, u0, ut, kappa_qp=kq + h * dk, dt=dt, want_grad=False)
        lm, _, _ = o.heat_adjoint(K, u0, ut, kappa_qp=kq - h * dk, dt=dt, want_grad=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gk @ dk) <= 1e-6 * max(1.0, abs(fd))
