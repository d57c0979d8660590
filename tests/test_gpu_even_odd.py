"""The double-float assembly's even-odd form (p = 2, 3) against the FP64 step.
With uniform knots (1/E exact in FP32) every brick, element row and layer
whose elements are centro-symmetric runs the even-odd sums, the rest the
direct ones; FP32-rounded knots run the direct sums only.  Either way the
mixed step matches FP64 to 1e-10 (src/ADS.F90:437-461)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-10


@pytest.mark.parametrize("E,p,var", [((64, 32, 16), 2, False), ((64, 32, 16), 2, True), ((96, 24, 12), 2, False),
                                     ((64, 32, 16), 3, False), ((64, 32, 16), 3, True)])
def test_even_odd_mixed_step_matches_fp64(ads_mod, E, p, var):
    from ads_mpi_gb300 import inputs
    n = tuple(e + p - 1 for e in E)
    gs = [ads_mod.ADS(n, (p, p, p), precision=prec, refine_tol=1e-13)
          for prec in (ads_mod.PREC_FP64, ads_mod.PREC_MIXED)]
    u0 = inputs.gaussian_bumps(*gs[0].qp_coords(), seed=4)
    rng = np.random.default_rng(5)
    kq = np.exp(0.3 * rng.standard_normal(gs[0].nqp)) if var else None
    f = rng.standard_normal(gs[0].nqp) if var else None
    for g in gs:
        g.set_form(ads_mod.FORM_PROJECT, f_qp=u0)
        g.step()
        g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, kappa=1.0, dt=2e-6 if p == 2 else 1e-6)
    for _ in range(4):
        l2 = [g.step() for g in gs]
        assert gs[1].stats()["converged"]
        assert rel_l2(gs[1].coeffs(), gs[0].coeffs()) < MIXED_TOL
        assert abs(l2[1] - l2[0]) < 1e-6 * abs(l2[0])


@pytest.mark.parametrize("p", [2, 3])
def test_even_odd_increment_of_a_constant_state_is_zero(ads_mod, p):
    """The heat increment of a constant state vanishes: the even-odd sums of
    the derivative tables cancel as the direct ones do."""
    E = (64, 32, 16)
    n = tuple(e + p - 1 for e in E)
    g = ads_mod.ADS(n, (p, p, p), precision=ads_mod.PREC_MIXED, refine_tol=1e-13)
    g.set_coeffs(np.full(g.N, 0.75))
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    g.step()
    assert np.abs(g.coeffs() - 0.75).max() < 1e-11
