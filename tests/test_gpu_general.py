"""The general geometry through the C-ABI against the oracle: a separate
degree per axis, as initialize(n(3), p(3), ...) takes it (src/ADS.F90:11), and
axes longer than the tuned sweeps' 448-DOF shared-memory lines.  Both run the
FP64 path (the general assembly and mass product of k_general.cu, banded LU
solves per axis) and must agree with the oracle to 1e-12; mixed precision is
refused there."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12

DEGREES = [((9, 7, 8), (2, 3, 2)), ((6, 8, 5), (1, 2, 3)), ((7, 5, 6), (4, 1, 2)), ((5, 6, 4), (3, 4, 1))]


def make(ads_mod, oracle_mod, E, p, **kw):
    n = tuple(e + q - 1 for e, q in zip(E, p))
    return ads_mod.ADS(n, p, **kw), oracle_mod.Oracle(n, p)


@pytest.mark.parametrize("E,p", DEGREES)
def test_assembly_with_per_axis_degrees(ads_mod, oracle_mod, E, p):
    g, o = make(ads_mod, oracle_mod, E, p)
    assert g.nq == tuple(q + 1 for q in p)
    rng = np.random.default_rng(sum(E) + sum(p))
    u = rng.standard_normal(g.N)
    kq = np.exp(0.4 * rng.standard_normal(g.nqp))
    f = rng.standard_normal(g.nqp)
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, dt=2e-3)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_HEAT, fqp=f, kappa_qp=kq, dt=2e-3)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)
    g.set_form(ads_mod.FORM_HEAT, kappa=0.7, dt=1e-3)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_HEAT, kappa=0.7, dt=1e-3)
    assert rel_l2(F, Fo) < FP64_TOL
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_PROJECT, fqp=f)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


@pytest.mark.parametrize("E,p", DEGREES)
def test_solve_mass_and_reorders_with_per_axis_degrees(ads_mod, oracle_mod, E, p):
    g, o = make(ads_mod, oracle_mod, E, p)
    rng = np.random.default_rng(3 + sum(p))
    F = rng.standard_normal(g.N)
    assert rel_l2(g.solve(F), o.solve(F)) < FP64_TOL
    assert rel_l2(g.apply_mass(F), o.apply_mass(F)) < 1e-14
    for kind, name in ((ads_mod.REORDER_FOR_Y, "y"), (ads_mod.REORDER_FOR_Z, "z"), (ads_mod.REORDER_FOR_X, "x")):
        out = g.reorder(kind, F)
        assert np.array_equal(out, oracle_mod.reorder(name, g.ndof, F))
        F = out


@pytest.mark.parametrize("E,p", DEGREES[:2])
def test_steps_with_per_axis_degrees(ads_mod, oracle_mod, E, p):
    """The L2 projection of 1 (problems/L2Projection/main.F90:62,72-78), then
    a seeded projection and heat steps against the oracle."""
    from ads_mpi_gb300 import inputs
    g, o = make(ads_mod, oracle_mod, E, p)
    g.set_form(ads_mod.FORM_PROJECT)
    assert abs(g.step() - 1.0) < 1e-12
    assert np.abs(g.coeffs() - 1.0).max() < 1e-12
    u0 = inputs.gaussian_bumps(*g.qp_coords(), seed=6)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
    g.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=u0)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-4)
    l2g = g.steps(4)
    l2o = [o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-4) for _ in range(4)]
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert np.abs(l2g - np.array(l2o)).max() < FP64_TOL * max(l2o)


def test_multistep_plot_and_adjoint_with_per_axis_degrees(ads_mod, oracle_mod):
    E, p = (8, 6, 7), (2, 3, 1)
    g, o = make(ads_mod, oracle_mod, E, p)
    rng = np.random.default_rng(17)
    u0 = rng.standard_normal(g.N)
    kq = np.exp(0.3 * rng.standard_normal(g.nqp))
    mix = np.array([[1.0, 0.0, 0.0, 0.0], [0.2, 0.0, 1.0, 0.3], [0.3, 0.01, 1.0, -0.5]])
    g.set_coeffs(u0)
    o.set_coeffs(u0)
    g.set_form(ads_mod.FORM_HEAT, kappa_qp=kq, dt=1e-3)
    l2 = g.multistep(mix)
    l2o = o.multistep(oracle_mod.FORM_HEAT, mix, kappa_qp=kq, dt=1e-3)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)
    v = g.save_spline_plot(res=(13, 17, 11))
    vo = o.eval_spline_grid((0.0, 1.0, 0.0, 1.0, 0.0, 1.0), (13, 17, 11))
    assert np.abs(v - vo).max() <= 1e-13 * np.abs(vo).max()
    ut = rng.standard_normal(g.N)
    loss, gu, gk = g.heat_adjoint(4, 2, u0, ut, grad=True, grad_kappa=True)
    lo, gou, gok = o.heat_adjoint(4, u0, ut, kappa_qp=kq, dt=1e-3, want_kappa_grad=True)
    assert abs(loss - lo) < 1e-12 * abs(lo)
    assert rel_l2(gu, gou) < 1e-11
    assert rel_l2(gk, gok) < 1e-10


@pytest.mark.parametrize("N", [(600, 40, 40), (40, 600, 40), (40, 40, 600)])
def test_long_axis_solve_and_steps(ads_mod, oracle_mod, N):
    """600 DOFs along one axis (beyond the tuned sweeps' 448): banded LU solves
    with the tuned assembly and mass product."""
    from ads_mpi_gb300 import inputs
    p = (2, 2, 2)
    n = tuple(v - 1 for v in N)
    g = ads_mod.ADS(n, p)
    o = oracle_mod.Oracle(n, p)
    assert g.ndof == N
    F = np.random.default_rng(sum(N)).standard_normal(g.N)
    assert rel_l2(g.solve(F), o.solve(F)) < FP64_TOL
    assert rel_l2(g.apply_mass(F), o.apply_mass(F)) < 1e-14
    u0 = inputs.gaussian_bumps(*g.qp_coords(), seed=8)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
    g.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=u0)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-6)
    l2g = g.steps(2)
    l2o = [o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-6) for _ in range(2)]
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert np.abs(l2g - np.array(l2o)).max() < FP64_TOL * max(l2o)


def test_long_axis_with_per_axis_degrees(ads_mod, oracle_mod):
    p = (2, 3, 2)
    N = (520, 24, 20)
    n = tuple(v - 1 for v in N)
    g = ads_mod.ADS(n, p)
    o = oracle_mod.Oracle(n, p)
    rng = np.random.default_rng(23)
    u = rng.standard_normal(g.N)
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-6)
    g.step()
    o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-6)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL


def test_general_geometry_refuses_what_it_does_not_run(ads_mod):
    for n, p in (((9, 10, 8), (2, 3, 2)), ((599, 39, 39), (2, 2, 2))):
        for prec in (ads_mod.PREC_MIXED, ads_mod.PREC_MIXED_FAST):
            with pytest.raises(ads_mod.ADSError) as e:
                ads_mod.ADS(n, p, precision=prec)
            assert e.value.status == 7
    with pytest.raises(ads_mod.ADSError) as e:
        ads_mod.ADS((9, 10, 8), (2, 5, 2))
    assert e.value.status == 7
