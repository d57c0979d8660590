"""GPU MultiStep (src/ADS.F90:391-429) through the C-ABI against the oracle:
three substeps with general M/K/B/BT mixes, whose banded LU pivots."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

MIXES = np.array([[1.0, 0.0, 0.0, 0.0],
                  [0.2, 0.0, 1.0, 0.3],
                  [0.3, 0.01, 1.0, -0.5]])


def make(ads_mod, E, p, prec=0):
    n = tuple(e + p - 1 for e in E)
    return ads_mod.ADS(n, (p, p, p), precision=prec), n


@pytest.mark.parametrize("E,p", [((9, 10, 7), 2), ((28, 31, 38), 2), ((7, 6, 8), 3), ((6, 5, 4), 1), ((6, 7, 5), 4)])
def test_multistep_heat_matches_oracle(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_mod.Oracle(n, (p, p, p))
    rng = np.random.default_rng(sum(E) + p)
    u0 = rng.standard_normal(g.N)
    kq = np.exp(0.3 * rng.standard_normal(g.nqp))
    f = rng.standard_normal(g.nqp)
    dt = 1e-3
    g.set_coeffs(u0)
    o.set_coeffs(u0)
    g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, dt=dt)
    l2 = g.multistep(MIXES)
    l2o = o.multistep(oracle_mod.FORM_HEAT, MIXES, fqp=f, kappa_qp=kq, dt=dt)
    assert any(o.pivoted())
    assert rel_l2(g.coeffs(), o.coeffs()) < 1e-12
    assert abs(l2 - l2o) < 1e-12 * abs(l2o)
    # a second MultiStep reuses the cached factors
    l2b = g.multistep(MIXES)
    l2ob = o.multistep(oracle_mod.FORM_HEAT, MIXES, fqp=f, kappa_qp=kq, dt=dt)
    assert rel_l2(g.coeffs(), o.coeffs()) < 1e-12
    assert abs(l2b - l2ob) < 1e-12 * abs(l2ob)


def test_multistep_projection_with_mass_mixes_is_a_step(ads_mod):
    g, _ = make(ads_mod, (12, 11, 10), 2)
    f = np.random.default_rng(3).standard_normal(g.nqp)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f)
    g.step()
    ref = g.coeffs()
    g.set_coeffs(np.zeros(g.N))
    g.multistep(np.tile([1.0, 0.0, 0.0, 0.0], (3, 1)))
    assert rel_l2(g.coeffs(), ref) < 1e-13


def test_multistep_runs_fp64_on_a_mixed_handle(ads_mod):
    res = []
    for prec in (0, 1):
        g, _ = make(ads_mod, (10, 9, 11), 2, prec=prec)
        g.set_coeffs(np.random.default_rng(5).standard_normal(g.N))
        g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-3)
        g.multistep(MIXES)
        res.append(g.coeffs())
    assert rel_l2(res[1], res[0]) < 1e-14


def test_multistep_rejects_the_oil_form(ads_mod):
    g, _ = make(ads_mod, (6, 6, 6), 2)
    from ads_mpi_gb300 import inputs
    x, y, z = g.qp_coords()
    fl = inputs.oil_fields(x, y, z)
    g.set_form(ads_mod.FORM_OIL, f_qp=fl["pump"], kappa_qp=fl["kq"], dt=1e-6)
    g.set_oil(fl["drain"])
    with pytest.raises(ads_mod.ADSError) as e:
        g.multistep(MIXES)
    assert e.value.status == 7
