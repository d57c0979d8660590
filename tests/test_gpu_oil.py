"""GPU parity of the oil problem (problems/oil/RHS_eq.F90:69-92) through the
C-ABI against the CPU oracle: the FP64 assembly and steps to 1e-12 relative
L2 together with the `drained` statistic; the mixed-precision steps against
the FP64 ones."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MU = 10.0  # mi of problems/oil/input_data.F90:11


def make(ads_mod, E, p, prec=0):
    n = tuple(e + p - 1 for e in E)
    return ads_mod.ADS(n, (p, p, p), precision=prec), n


def fields(g, seed=0):
    from ads_mpi_gb300 import inputs
    x, y, z = g.qp_coords()
    return inputs.oil_fields(x, y, z, seed=seed)


def stable_dt(g, f):
    """dt with dt * lambda_max(M^-1 K_kappa) ~ 0.5 for kappa up to max Kq exp(mu max u)."""
    lam1 = {1: 12.0, 2: 21.6, 3: 47.2, 4: 100.0}[g.p[0]]
    kmax = f["kq"].max() * np.exp(MU * max(f["init"].max(), 0.1))
    return 0.5 / (3 * lam1 * max(g.nelem) ** 2 * kmax)


@pytest.mark.parametrize("E,p", [((9, 10, 7), 2), ((7, 6, 8), 3), ((40, 19, 11), 2), ((6, 5, 4), 1), ((6, 7, 5), 4)])
def test_oil_assembly_matches_oracle(ads_mod, oracle_mod, E, p):
    g, n = make(ads_mod, E, p)
    o = oracle_mod.Oracle(n, (p, p, p))
    f = fields(g, seed=2)
    u = 0.1 * np.random.default_rng(sum(E) + p).standard_normal(g.N)
    dt = 1e-4
    g.set_coeffs(u)
    o.set_coeffs(u)
    g.set_form(ads_mod.FORM_OIL, f_qp=f["pump"], kappa_qp=f["kq"], dt=dt)
    g.set_oil(f["drain"], mu=MU)
    F, l2 = g.assemble()
    Fo, l2o, _ = o.assemble_oil(f["pump"], f["kq"], f["drain"], MU, dt)
    assert rel_l2(F, Fo) < FP64_TOL
    assert abs(l2 - l2o) < FP64_TOL * abs(l2o)


@pytest.mark.parametrize("E,p", [((12, 10, 9), 2), ((8, 7, 9), 3)])
def test_oil_steps_match_oracle(ads_mod, oracle_mod, E, p):
    """Projection of the oil initial state, then oil steps, with the drained total."""
    g, n = make(ads_mod, E, p)
    o = oracle_mod.Oracle(n, (p, p, p))
    f = fields(g, seed=4)
    g.set_form(ads_mod.FORM_PROJECT, f_qp=f["init"])
    g.step()
    o.step(oracle_mod.FORM_PROJECT, fqp=f["init"])
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    dt = 20 * stable_dt(g, f)  # a visible drain; the few steps stay far from overflow
    g.set_form(ads_mod.FORM_OIL, f_qp=f["pump"], kappa_qp=f["kq"], dt=dt)
    g.set_oil(f["drain"], mu=MU)
    drained_o = 0.0
    for _ in range(3):
        l2 = g.step()
        l2o, dr = o.step_oil(f["pump"], f["kq"], f["drain"], MU, dt)
        drained_o += dr
        assert abs(l2 - l2o) < FP64_TOL * abs(l2o)
    assert rel_l2(g.coeffs(), o.coeffs()) < FP64_TOL
    assert drained_o > 0.0
    assert abs(g.drained() - drained_o) < FP64_TOL * drained_o
    # set_oil starts a new total
    g.set_oil(f["drain"], mu=MU)
    assert g.drained() == 0.0


def test_oil_mixed_steps_track_fp64(ads_mod):
    E, p = (24, 20, 18), 2
    f = None
    res = {}
    for prec in (0, 1):
        g, _ = make(ads_mod, E, p, prec=prec)
        f = fields(g, seed=6) if f is None else f
        g.set_form(ads_mod.FORM_PROJECT, f_qp=f["init"])
        g.step()
        dt = stable_dt(g, f)
        g.set_form(ads_mod.FORM_OIL, f_qp=f["pump"], kappa_qp=f["kq"], dt=dt)
        g.set_oil(f["drain"], mu=MU)
        g.steps(4)
        if prec == 1:
            st = g.stats()
            assert st["converged"] and st["rel_residual"] <= 1e-10
        res[prec] = (g.coeffs(), g.drained())
    assert rel_l2(res[1][0], res[0][0]) < 1e-6
    assert abs(res[1][1] - res[0][1]) < 1e-5 * abs(res[0][1])


def test_oil_form_needs_its_data(ads_mod):
    g, _ = make(ads_mod, (6, 6, 6), 2)
    f = fields(g)
    with pytest.raises(ads_mod.ADSError) as e:
        g.set_form(ads_mod.FORM_OIL, f_qp=f["pump"], dt=1e-6)  # Kq missing
    assert e.value.status == 1
    g.set_form(ads_mod.FORM_OIL, f_qp=f["pump"], kappa_qp=f["kq"], dt=1e-6)
    with pytest.raises(ads_mod.ADSError) as e:
        g.step()  # set_oil missing
    assert e.value.status == 8
