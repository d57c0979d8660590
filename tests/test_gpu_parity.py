"""GPU parity: the CUDA path, called through the C-ABI, against the CPU oracle on
the same seeded inputs.  FP64 results must agree to 1e-12 relative L2 (the
bar of the FP64 drop-in); the mixed-precision path (double-float increment
assembly, FP32 sweeps, FP64 refinement to 1e-13 relative residual) must agree
with the FP64 oracle and the FP64 GPU step to 1e-10 relative L2."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
# the mixed-precision step against FP64, relative L2
MIXED_TOL = 1e-10


def make(ads_mod, E, p, prec=0, **kw):
    if isinstance(E, int):
        E = (E, E, E)
    n = tuple(e + p - 1 for e in E)
    return ads_mod.ADS(n, (p, p, p), precision=prec, **kw), n


def oracle_for(oracle_mod, n, p):
    return oracle_mod.Oracle(n, (p, p, p))


# --------------------------------------------------------------------------
# assembly (K1)
# --------------------------------------------------------------------------
@pytest.mark.parametrize("E,p", [((6, 5, 4), 1), ((9, 10, 7), 2), ((40, 19, 11), 2), ((35, 12, 9), 3),
                                 ((8, 9, 6), 4), ((64, 20, 70), 2)])
def test_heat_assembly_matches_oracle(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_for(oracle_mod, n, p)
    rng = np.random.default_rng(sum(E) + p)
    u = rng.standard_normal(g.N)
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_HEAT, kappa=0.7, dt=1e-3)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_HEAT, kappa=0.7, dt=1e-3)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


@pytest.mark.parametrize("E,p", [((10, 9, 12), 2), ((33, 9, 17), 3)])
def test_variable_kappa_and_source_assembly(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_for(oracle_mod, n, p)
    rng = np.random.default_rng(7)
    u = rng.standard_normal(g.N)
    kq = np.exp(0.5 * rng.standard_normal(g.nqp))
    f = rng.standard_normal(g.nqp)
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, dt=2e-3)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_HEAT, fqp=f, kappa_qp=kq, dt=2e-3)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


@pytest.mark.parametrize("E,p", [((7, 6, 5), 2), ((34, 9, 10), 3)])
def test_projection_assembly_matches_oracle(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_for(oracle_mod, n, p)
    f = np.random.default_rng(9).standard_normal(g.nqp)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f)
    F, l2 = g.assemble()
    Fo, l2o = o.assemble(oracle_mod.FORM_PROJECT, fqp=f)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


def test_fp32_assembly_error_bound(ads_mod, oracle_mod):
    g, n = make(ads_mod, (20, 18, 16), 2, prec=1)
    o = oracle_for(oracle_mod, n, 2)
    u = np.random.default_rng(11).standard_normal(g.N)
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-4)
    F, _ = g.assemble()
    Fo, _ = o.assemble(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-4)
    assert rel_l2(F, Fo) < 1e-5


# --------------------------------------------------------------------------
# solve (K3 + K4) and the stand-alone pieces
# --------------------------------------------------------------------------
@pytest.mark.parametrize("E,p", [((6, 7, 8), 1), ((30, 33, 40), 2), ((17, 64, 9), 3), ((12, 11, 10), 4)])
def test_fp64_solve_matches_oracle(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_for(oracle_mod, n, p)
    F = np.random.default_rng(13).standard_normal(g.N)
    u = g.solve(F)
    uo = o.solve(F)
    assert rel_l2(u, uo) < FP64_TOL


@pytest.mark.parametrize("E,p", [((30, 33, 40), 2), ((17, 24, 9), 3)])
def test_mixed_solve_refines_to_tolerance(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p, prec=1)
    o = oracle_for(oracle_mod, n, p)
    F = np.random.default_rng(17).standard_normal(g.N)
    u = g.solve(F)
    st = g.stats()
    assert st["converged"] and st["rel_residual"] <= 1e-13
    assert rel_l2(u, o.solve(F)) < MIXED_TOL


def true_rel_residual(ads_mod, E, p, F, u):
    """||F - M u|| / ||F|| with the FP64 mass operator."""
    g64, _ = make(ads_mod, E, p)
    return np.linalg.norm(F - g64.apply_mass(u)) / np.linalg.norm(F)


def fp64_floor(ads_mod, E, p, F, u):
    """What the certified bound leaves out: the FP64 rounding of the stored
    result and of an FP64 residual, relative to ||F||: K 2^-53 ||M|u||| with
    K = 3 (2p + 2) (three banded passes of 2p + 1 terms and the subtraction)."""
    g64, _ = make(ads_mod, E, p)
    return 3 * (2 * p + 2) * 2.0 ** -53 * np.linalg.norm(g64.apply_mass(np.abs(u))) / np.linalg.norm(F)


@pytest.mark.parametrize("E,p", [((30, 33, 40), 2), ((17, 24, 9), 3), ((64, 20, 70), 2)])
@pytest.mark.parametrize("tol", [1e-10, 1e-13])
def test_mixed_certified_bound_covers_true_residual(ads_mod, E, p, tol):
    """The refinement stops on the certified bound of the updated residual
    r1 - M x1 (M x1 in double-float arithmetic); the FP64 residual of the
    result must lie below that bound.  At p = 2 the bound certifies even
    1e-13 after one correction, so the reported value is the bound (above
    the true residual by at least u ||r1||), not a second FP64 residual."""
    g, _ = make(ads_mod, E, p, prec=1, refine_tol=tol)
    for seed, smooth in ((31, False), (37, True)):
        F = np.random.default_rng(seed).standard_normal(g.N)
        if smooth:
            # coefficients are x fastest: F(x, y + Ny z)
            X, Y, Z = np.meshgrid(*[np.linspace(0, 1, m) for m in g.ndof], indexing="ij")
            bump = np.exp(-20 * ((X - 0.3) ** 2 + (Y - 0.6) ** 2 + (Z - 0.5) ** 2))
            F = bump.ravel(order="F") + 1e-3 * F
        u = g.solve(F)
        st = g.stats()
        assert st["converged"] and 0 < st["rel_residual"] <= tol
        assert st["refinements"] >= 1
        true = true_rel_residual(ads_mod, E, p, F, u)
        assert true <= st["rel_residual"] + fp64_floor(ads_mod, E, p, F, u)
        if p == 2:
            assert st["refinements"] == 1
            assert st["fp64_residuals"] == 1  # the bound decided, not a second FP64 residual
            assert st["rel_residual"] >= true + 1e-15
        assert st["fp64_residuals"] in (st["refinements"], st["refinements"] + 1)


def test_mixed_tolerance_below_one_correction_takes_another_round(ads_mod):
    """With refine_tol below what one correction reaches (~1.6e-14 here, and
    its bound carries u ||r1||, ~2e-14 more), the next round's FP64 residual
    finds the solve unconverged and a second correction follows, whose bound
    certifies; the result meets the tolerance."""
    E, p, tol = (30, 33, 40), 2, 1e-14
    g, _ = make(ads_mod, E, p, prec=1, refine_tol=tol)
    F = np.random.default_rng(41).standard_normal(g.N)
    u = g.solve(F)
    st = g.stats()
    assert st["converged"] and st["rel_residual"] <= tol
    assert st["refinements"] == 2
    assert st["fp64_residuals"] in (st["refinements"], st["refinements"] + 1)
    assert true_rel_residual(ads_mod, E, p, F, u) <= 2 * tol


@pytest.mark.parametrize("s", [(5, 4, 3), (34, 33, 40), (70, 9, 33)])
def test_reorders_match_reference_permutations(ads_mod, oracle_mod, s):
    E = tuple(v - 1 for v in s)
    g, n = make(ads_mod, E, 2)
    F = np.random.default_rng(19).standard_normal(g.N)
    for kind, name in ((ads_mod.REORDER_FOR_Y, "y"), (ads_mod.REORDER_FOR_Z, "z"), (ads_mod.REORDER_FOR_X, "x")):
        out = g.reorder(kind, F)
        assert np.array_equal(out, oracle_mod.reorder(name, g.ndof, F))
        F = out


def test_apply_mass_matches_oracle(ads_mod, oracle_mod):
    g, n = make(ads_mod, (33, 10, 40), 2)
    o = oracle_for(oracle_mod, n, 2)
    u = np.random.default_rng(23).standard_normal(g.N)
    assert rel_l2(g.apply_mass(u), o.apply_mass(u)) < 1e-14


# --------------------------------------------------------------------------
# full steps
# --------------------------------------------------------------------------
# The mixed path refines each Kronecker solve to a relative residual of 1e-13;
# with cond(Mx (x) My (x) Mz) ~ 1.2e3 at p = 2 that bounds the coefficient error
# by ~1.2e-10 (the projection step is assembled in FP64, the heat increments in
# double-float arithmetic, ~1e-13 relative).
MIXED_KAT_TOL = 1e-10


@pytest.mark.parametrize("prec", [0, 1])
def test_l2_projection_known_answer(ads_mod, prec):
    """problems/L2Projection/main.F90:62,72-78 at its 32^3, p=2 size."""
    g, _ = make(ads_mod, 32, 2, prec=prec)
    g.set_form(ads_mod.FORM_PROJECT)
    l2 = g.step()
    tol = 1e-10 if prec == 0 else MIXED_KAT_TOL
    assert abs(l2 - 1.0) < tol
    assert np.abs(g.coeffs() - 1.0).max() < tol
    if prec == 1:
        assert g.stats()["rel_residual"] <= 1e-13


def test_projection_config_matches_oracle(ads_mod, oracle_mod):
    """The L2-projection configuration: E = 32, p = 2, seeded target."""
    from ads_mpi_gb300 import inputs
    g, n = make(ads_mod, 32, 2)
    o = oracle_for(oracle_mod, n, 2)
    f = inputs.projection_target(*g.qp_coords(), seed=0)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f)
    l2 = g.step()
    l2o = o.step(oracle_mod.FORM_PROJECT, fqp=f)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


def test_reference_heat_problem_trajectory(ads_mod, oracle_mod):
    """problems/heat: projection of 2*bump3d(0.05,0.4,x) at t=0, then explicit
    steps with kappa = 1, f = 0 (stable at E = 16, dt = 1e-5)."""
    g, n = make(ads_mod, 16, 2)
    o = oracle_for(oracle_mod, n, 2)
    f0 = o.heat_initial_qp()
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f0)
    l2g = [g.step()]
    l2o = [o.step(oracle_mod.FORM_PROJECT, heat_initial=True)]
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    l2g += list(g.steps(20))
    for _ in range(20):
        l2o.append(o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-5))
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert np.abs(np.array(l2g) - np.array(l2o)).max() < FP64_TOL * max(l2o)


@pytest.mark.parametrize("E,p,dt,K", [(24, 2, 1e-5, 10), (20, 3, 5e-6, 8), ((40, 12, 18), 2, 1e-5, 6)])
def test_heat_steps_match_oracle(ads_mod, oracle_mod, E, p, dt, K):
    from ads_mpi_gb300 import inputs
    g, n = make(ads_mod, E, p)
    o = oracle_for(oracle_mod, n, p)
    u0 = inputs.gaussian_bumps(*g.qp_coords(), seed=1)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
    g.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=u0)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=dt)
    l2g = g.steps(K)
    l2o = [o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=dt) for _ in range(K)]
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert np.abs(l2g - np.array(l2o)).max() < FP64_TOL * max(l2o)


def test_heat_config_size_first_steps(ads_mod, oracle_mod):
    """The 128^3, p=2, dt=1e-5 heat configuration: projection plus two steps
    against the oracle (the explicit scheme is unstable at this dt, which
    amplifies rounding differences by ~10x per step, so only the first steps
    are compared at 1e-12)."""
    from ads_mpi_gb300 import inputs
    g, n = make(ads_mod, 128, 2)
    o = oracle_for(oracle_mod, n, 2)
    u0 = inputs.gaussian_bumps(*g.qp_coords(), seed=0)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
    g.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=u0)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    for _ in range(2):
        g.step()
        o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL


def test_mixed_heat_steps_error_bound(ads_mod, oracle_mod):
    from ads_mpi_gb300 import inputs
    gm, n = make(ads_mod, 24, 2, prec=1)
    o = oracle_for(oracle_mod, n, 2)
    u0 = inputs.gaussian_bumps(*gm.qp_coords(), seed=2)
    gm.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
    gm.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=u0)
    gm.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    for _ in range(5):
        gm.step()
        o.step(oracle_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
        st = gm.stats()
        assert st["converged"] and st["rel_residual"] <= 1e-13
    assert rel_l2(gm.coeffs(), o.coeffs()) < MIXED_TOL


@pytest.mark.parametrize("E,p,var", [(24, 2, False), ((30, 20, 26), 2, True), (20, 3, False), (14, 3, True),
                                     (18, 1, True), (12, 1, False), (10, 4, False)])
def test_mixed_step_matches_fp64_step(ads_mod, E, p, var):
    """Mixed against FP64 on the GPU, step by step at a stable dt, with a
    constant conductivity or per-point conductivity plus a source (every
    variant of the double-float assembly)."""
    from ads_mpi_gb300 import inputs
    gs = [make(ads_mod, E, p, prec=prec)[0] for prec in (0, 1)]
    u0 = inputs.gaussian_bumps(*gs[0].qp_coords(), seed=4)
    rng = np.random.default_rng(5)
    kq = np.exp(0.3 * rng.standard_normal(gs[0].nqp)) if var else None
    f = rng.standard_normal(gs[0].nqp) if var else None
    dt = 2e-6 if p >= 3 else 5e-6
    for g in gs:
        g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
        g.step()
        g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, kappa=1.0, dt=dt)
    for _ in range(4):
        l2 = [g.step() for g in gs]
        assert gs[1].stats()["converged"]
        assert rel_l2(gs[1].coeffs(), gs[0].coeffs()) < MIXED_TOL
        assert abs(l2[1] - l2[0]) < 1e-6 * abs(l2[0])


def test_mixed_fast_step_error_bound(ads_mod):
    """ADS_PREC_MIXED_FAST keeps the plain FP32 increment assembly: its step
    error against FP64 stays of order 1e-8 (FP32 rounding of the increment)."""
    from ads_mpi_gb300 import inputs
    gs = [make(ads_mod, 24, 2, prec=prec)[0] for prec in (0, 2)]
    u0 = inputs.gaussian_bumps(*gs[0].qp_coords(), seed=2)
    for g in gs:
        g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
        g.step()
        g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
        g.steps(3)
    assert rel_l2(gs[1].coeffs(), gs[0].coeffs()) < 1e-6


def test_steps_are_deterministic(ads_mod):
    from ads_mpi_gb300 import inputs
    outs = []
    for _ in range(2):
        g, _ = make(ads_mod, (40, 20, 30), 2)
        g.set_form(ads_mod.FORM_PROJECT, f_qp=inputs.gaussian_bumps(*g.qp_coords(), seed=3))
        g.step()
        g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
        g.steps(3)
        outs.append(g.coeffs())
        g.cleanup()
    assert np.array_equal(outs[0], outs[1])


# --------------------------------------------------------------------------
# properties at the full 256^3 size (too large for the oracle)
# --------------------------------------------------------------------------
@pytest.mark.parametrize("prec", [0, 1])
def test_full_size_projection_of_one(ads_mod, prec):
    g, _ = make(ads_mod, 256, 2, prec=prec)
    g.set_form(ads_mod.FORM_PROJECT)
    l2 = g.step()
    tol = 1e-10 if prec == 0 else MIXED_KAT_TOL
    assert abs(l2 - 1.0) < tol
    assert np.abs(g.coeffs() - 1.0).max() < tol


def _basis_integrals(ads_mod, n, p):
    U = ads_mod.axis_setup(n, p)["U"]
    return np.array([(U[i + p + 1] - U[i]) / (p + 1) for i in range(n + 1)])


@pytest.mark.parametrize("E", [64, 96, 128, 192, 256, (256, 96, 160)])
@pytest.mark.parametrize("prec", [0, 1])
def test_projection_rhs_is_product_of_basis_integrals(ads_mod, E, prec):
    """F_a = integral of the tensor B-spline a = product of 1-D integrals
    (U_{i+p+1} - U_i)/(p+1): an exact check of the assembly at any size."""
    g, n = make(ads_mod, E, 2, prec=prec)
    g.set_form(ads_mod.FORM_PROJECT)
    F, l2 = g.assemble()
    wx, wy, wz = (_basis_integrals(ads_mod, n[d], 2) for d in range(3))
    expect = (wz[:, None, None] * wy[None, :, None] * wx[None, None, :]).ravel()
    assert rel_l2(F, expect) < (1e-13 if prec == 0 else 1e-6)
    assert abs(l2 - 1.0) < (1e-12 if prec == 0 else 1e-6)


@pytest.mark.parametrize("prec", [0, 1])
def test_full_size_constant_state_is_steady(ads_mod, prec):
    """grad u = 0 for u == c, so one explicit heat step returns u == c."""
    g, _ = make(ads_mod, 256, 2, prec=prec)
    g.set_coeffs(np.full(g.N, 2.5))
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    g.step()
    # the derivative tables sum to zero to rounding: ~1e-16 relative in FP64,
    # ~4e-15 in double-float (two floats carry ~48 bits of each FP64 table
    # entry), so the increment is at that level and the state stays constant
    assert np.abs(g.coeffs() - 2.5).max() < (1e-12 if prec == 0 else MIXED_TOL * 2.5)
    if prec == 1:
        assert g.stats()["rel_residual"] <= 1e-13


def test_full_size_step_is_linear(ads_mod):
    rng = np.random.default_rng(29)
    g, _ = make(ads_mod, 256, 2)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-7)
    a = rng.standard_normal(g.N)
    b = rng.standard_normal(g.N)
    res = []
    for u in (a, b, 2.0 * a - 3.0 * b):
        g.set_coeffs(u)
        g.step()
        res.append(g.coeffs())
    assert rel_l2(res[2], 2.0 * res[0] - 3.0 * res[1]) < 1e-12


# --------------------------------------------------------------------------
# errors
# --------------------------------------------------------------------------
def test_errors_are_status_codes(ads_mod):
    with pytest.raises(ads_mod.ADSError) as e:
        ads_mod.ADS((10, 10, 10), (5, 5, 5))
    assert e.value.status == 7
    with pytest.raises(ads_mod.ADSError) as e:
        ads_mod.ADS((10, 10, 10), (2, 5, 2))
    assert e.value.status == 7
    g, _ = make(ads_mod, 6, 2)
    with pytest.raises(ads_mod.ADSError) as e:
        g.step()
    assert e.value.status == 8
    with pytest.raises(ValueError):
        g.set_coeffs(np.zeros(3))
