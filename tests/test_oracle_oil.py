"""The oracle's oil-problem integrand (problems/oil/RHS_eq.F90:69-92) against
its heat integrand, which the L2 known answer and the Kronecker identity pin:
at the quadrature points the oil form is the heat form with
kappa = Kq exp(mu u) and f = pump - max(0, w u), so both assemblies must agree
once u is interpolated at the points.  Also the seeded oil inputs."""
import numpy as np
import pytest

from conftest import rel_l2


def qp_coords(o):
    """x, y, z at the points in the (kx,ky,kz,ex,ey,ez) layout (C shape (Ez,Ey,Ex,q,q,q))."""
    X = [o.axis_tables(d)["X"] for d in range(3)]  # (E, q) per axis
    x = X[0][None, None, :, None, None, :]
    y = X[1][None, :, None, None, :, None]
    z = X[2][:, None, None, :, None, None]
    shape = (X[2].shape[0], X[1].shape[0], X[0].shape[0], X[2].shape[1], X[1].shape[1], X[0].shape[1])
    return [np.broadcast_to(v, shape) for v in (x, y, z)]


def interp_matrix(t, N):
    E, q, p1 = t["NN"].shape[0], t["NN"].shape[1], t["NN"].shape[2]
    B = np.zeros((E * q, N))
    for e in range(E):
        for k in range(q):
            for a in range(p1):
                B[e * q + k, t["O"][e] + a] = t["NN"][e, k, a, 0]
    return B


def u_at_qp(o, u):
    """u at the points, (kx,ky,kz,ex,ey,ez) layout, from x-fastest coefficients."""
    T = [o.axis_tables(d) for d in range(3)]
    Nx, Ny, Nz = o.ndof
    Bx, By, Bz = (interp_matrix(T[d], n) for d, n in enumerate((Nx, Ny, Nz)))
    V = np.einsum("zi,yj,xk,ijk->zyx", Bz, By, Bx, u.reshape(Nz, Ny, Nx))
    Ex, Ey, Ez = (T[d]["NN"].shape[0] for d in range(3))
    q = T[0]["NN"].shape[1]
    return V.reshape(Ez, q, Ey, q, Ex, q).transpose(0, 2, 4, 1, 3, 5)


def jw_at_qp(o):
    T = [o.axis_tables(d) for d in range(3)]
    jw = [T[d]["J"][:, None] * T[d]["W"][None, :] for d in range(3)]  # (E, q)
    return (jw[0][None, None, :, None, None, :] * jw[1][None, :, None, None, :, None]
            * jw[2][:, None, None, :, None, None])


@pytest.mark.parametrize("E,p", [((6, 5, 7), 2), ((5, 4, 4), 3)])
def test_oil_form_is_heat_form_with_pointwise_kappa_and_source(oracle_mod, E, p):
    from ads_mpi_gb300 import inputs
    n = tuple(e + p - 1 for e in E)
    o = oracle_mod.Oracle(n, (p, p, p))
    x, y, z = qp_coords(o)
    f = inputs.oil_fields(x, y, z, seed=3)
    rng = np.random.default_rng(5)
    u = 0.1 * rng.standard_normal(o.N)  # both signs: max(0, w u) is active and inactive
    mu, dt = 4.0, 1e-6
    o.set_coeffs(u)
    F_oil, l2_oil, drained = o.assemble_oil(f["pump"], f["kq"], f["drain"], mu, dt)
    uq = u_at_qp(o, u)
    kappa = f["kq"] * np.exp(mu * uq)
    src = f["pump"] - np.maximum(0.0, f["drain"] * uq)
    o.set_coeffs(u)
    F_heat, l2_heat = o.assemble(oracle_mod.FORM_HEAT, fqp=src, kappa_qp=kappa, dt=dt)
    assert rel_l2(F_oil, F_heat) < 1e-13
    assert abs(l2_oil - l2_heat) <= 1e-13 * abs(l2_heat)
    # drained: sum over points and test functions of J W v dt max(0, w u); the
    # test functions sum to 1 at every point (partition of unity)
    expect = np.sum(jw_at_qp(o) * dt * np.maximum(0.0, f["drain"] * uq))
    assert expect > 0.0
    assert abs(drained - expect) <= 1e-12 * expect


def test_oil_step_with_constant_state_only_drains(oracle_mod):
    """u = c: grad u = 0, so one step solves M u1 = M c + dt M_w-weighted source."""
    from ads_mpi_gb300 import inputs
    E, p = (5, 6, 4), 2
    n = tuple(e + p - 1 for e in E)
    o = oracle_mod.Oracle(n, (p, p, p))
    x, y, z = qp_coords(o)
    f = inputs.oil_fields(x, y, z, seed=1)
    c, dt = 0.05, 1e-3
    o.set_coeffs(np.full(o.N, c))
    F_oil, _, drained = o.assemble_oil(f["pump"], f["kq"], f["drain"], 10.0, dt)
    o.set_coeffs(np.full(o.N, c))
    F_heat, _ = o.assemble(oracle_mod.FORM_HEAT, fqp=f["pump"] - f["drain"] * c, kappa=123.0, dt=dt)
    assert rel_l2(F_oil, F_heat) < 1e-13
    assert abs(drained - np.sum(jw_at_qp(o) * dt * f["drain"] * c)) <= 1e-12 * drained


def test_oil_inputs_are_seeded_and_in_range():
    from ads_mpi_gb300 import inputs
    pts = np.random.default_rng(0).random((500, 3))
    a = inputs.oil_fields(pts[:, 0], pts[:, 1], pts[:, 2], seed=7)
    b = inputs.oil_fields(pts[:, 0], pts[:, 1], pts[:, 2], seed=7)
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert a["kq"].min() >= inputs.OIL_KQMIN and a["kq"].max() <= inputs.OIL_KQMAX
    assert a["pump"].min() >= 0.0 and a["drain"].min() >= 0.0
    assert 0.0 <= a["init"].min() and a["init"].max() <= 0.1
    # the torch path (used for large grids) evaluates the same formulas
    pytest.importorskip("torch")
    c = inputs.oil_fields(pts[:, 0], pts[:, 1], pts[:, 2], seed=7, device="cpu")
    for k in a:
        assert np.allclose(c[k], a[k], rtol=1e-12, atol=1e-12)
    # the curves follow the reference's random walk: consecutive points 0.05 |dx| apart
    c = inputs.oil_curves(7)
    assert c.shape == (30, 16, 3)
    assert np.all(np.linalg.norm(np.diff(c, axis=1), axis=2) < 0.05 * 3.0)
