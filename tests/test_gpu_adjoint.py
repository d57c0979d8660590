"""Hand-written adjoint of the explicit heat step (K6) through the C-ABI:
against the oracle's FP64 reference gradient, against central finite
differences (h = 1e-6) along seeded random directions, against the tangent-
linear model (ads_heat_jvp: forward mode, no finite-difference cancellation),
and through a thin torch.autograd.Function checked with
torch.autograd.gradcheck."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def setup(ads_mod, oracle_mod, E=6, p=2, var_kappa=True, seed=0, dt=2e-3):
    n = (E + p - 1,) * 3
    g = ads_mod.ADS(n, (p, p, p))
    o = oracle_mod.Oracle(n, (p, p, p))
    rng = np.random.default_rng(seed)
    kq = np.exp(0.4 * rng.standard_normal(g.nqp)) if var_kappa else None
    g.set_form(ads_mod.FORM_HEAT, kappa_qp=kq, kappa=1.0, dt=dt)
    u0 = rng.standard_normal(g.N)
    ut = rng.standard_normal(g.N)
    return g, o, kq, u0, ut, dt


@pytest.mark.parametrize("K,ck", [(5, 2), (7, 3), (4, 10)])
def test_adjoint_matches_oracle(ads_mod, oracle_mod, K, ck):
    g, o, kq, u0, ut, dt = setup(ads_mod, oracle_mod)
    loss, gu, gk = g.heat_adjoint(K, ck, u0, ut, grad=True, grad_kappa=True)
    lo, gou, gok = o.heat_adjoint(K, u0, ut, kappa_qp=kq, dt=dt, want_kappa_grad=True)
    assert abs(loss - lo) < 1e-12 * abs(lo)
    assert rel_l2(gu, gou) < 1e-11
    assert rel_l2(gk, gok) < 1e-10


def test_adjoint_matches_central_differences(ads_mod, oracle_mod):
    g, o, kq, u0, ut, dt = setup(ads_mod, oracle_mod, E=7, seed=3)
    K = 6
    loss, gu, gk = g.heat_adjoint(K, 2, u0, ut, grad=True, grad_kappa=True)
    rng = np.random.default_rng(11)
    h = 1e-6
    for _ in range(8):
        d = rng.standard_normal(g.N)
        lp, _, _ = g.heat_adjoint(K, 2, u0 + h * d, ut, grad=False)
        lm, _, _ = g.heat_adjoint(K, 2, u0 - h * d, ut, grad=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gu @ d) <= 1e-6 * abs(fd)
    for _ in range(4):
        dk = rng.standard_normal(g.nqp) * kq
        g.set_form(ads_mod.FORM_HEAT, kappa_qp=kq + h * dk, dt=dt)
        lp, _, _ = g.heat_adjoint(K, 2, u0, ut, grad=False)
        g.set_form(ads_mod.FORM_HEAT, kappa_qp=kq - h * dk, dt=dt)
        lm, _, _ = g.heat_adjoint(K, 2, u0, ut, grad=False)
        g.set_form(ads_mod.FORM_HEAT, kappa_qp=kq, dt=dt)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gk @ dk) <= 1e-6 * abs(fd)


@pytest.mark.parametrize("E,p,dt", [(7, 2, 2e-3), ((9, 8, 6), 3, 1e-2), (6, 1, 5e-3)])
def test_tangent_model_matches_adjoint_dot_products(ads_mod, oracle_mod, E, p, dt):
    """Forward-mode (ads_heat_jvp) against reverse mode (ads_heat_adjoint):
    e^T M du^K along (d, dk) equals grad_u0 . d + grad_kappa . dk for any
    direction, to rounding, with a per-point kappa and a source term.  At
    these dt the explicit scheme is unstable (values grow by orders of
    magnitude), which the identity is indifferent to."""
    if isinstance(E, int):
        E = (E, E, E)
    n = tuple(e + p - 1 for e in E)
    g = ads_mod.ADS(n, (p, p, p))
    rng = np.random.default_rng(sum(E) + p)
    kq = np.exp(0.4 * rng.standard_normal(g.nqp))
    f = rng.standard_normal(g.nqp)
    g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa_qp=kq, dt=dt)
    u0 = rng.standard_normal(g.N)
    ut = rng.standard_normal(g.N)
    K = 6
    loss, gu, gk = g.heat_adjoint(K, 2, u0, ut, grad=True, grad_kappa=True)
    g.set_coeffs(u0)
    g.steps(K)
    u_fwd = g.coeffs()
    for _ in range(3):
        d = rng.standard_normal(g.N)
        dk = rng.standard_normal(g.nqp) * kq
        uK, duK = g.heat_jvp(K, u0, du0=d, dkappa=dk)
        assert rel_l2(uK, u_fwd) < 1e-14
        jvp = float((uK - ut) @ g.apply_mass(duK))
        vjp = float(gu @ d + gk @ dk)
        assert abs(jvp - vjp) <= 1e-11 * abs(vjp)
        # each direction on its own
        _, du_only = g.heat_jvp(K, u0, du0=d)
        _, dk_only = g.heat_jvp(K, u0, dkappa=dk)
        assert abs(float((uK - ut) @ g.apply_mass(du_only)) - float(gu @ d)) <= 1e-11 * abs(float(gu @ d))
        assert abs(float((uK - ut) @ g.apply_mass(dk_only)) - float(gk @ dk)) <= 1e-11 * abs(float(gk @ dk))


def test_tangent_model_of_initial_state_is_the_homogeneous_step(ads_mod):
    """Along du0 alone the tangent of the (affine) heat step is the step
    without its source, applied to du0."""
    n = (9, 10, 8)
    g = ads_mod.ADS(n, (2, 2, 2))
    rng = np.random.default_rng(2)
    f = rng.standard_normal(g.nqp)
    u0 = rng.standard_normal(g.N)
    d = rng.standard_normal(g.N)
    g.set_form(ads_mod.FORM_HEAT, f_qp=f, kappa=0.8, dt=1e-3)
    _, duK = g.heat_jvp(4, u0, du0=d)
    g.set_form(ads_mod.FORM_HEAT, kappa=0.8, dt=1e-3)
    g.set_coeffs(d)
    g.steps(4)
    assert rel_l2(duK, g.coeffs()) < 1e-14


def test_adjoint_gradcheck_through_autograd(ads_mod, oracle_mod):
    torch = pytest.importorskip("torch")
    g, o, kq, u0, ut, dt = setup(ads_mod, oracle_mod, E=5, seed=5)
    K, ck = 4, 2

    class HeatLoss(torch.autograd.Function):
        """loss(u0, g) with kappa = exp(g) at the quadrature points; the
        backward is the library's hand-written adjoint."""

        @staticmethod
        def forward(ctx, u0_t, gq_t):
            kappa = np.exp(gq_t.detach().cpu().numpy())
            g.set_form(ads_mod.FORM_HEAT, kappa_qp=kappa, dt=dt)
            loss, gu, gk = g.heat_adjoint(K, ck, u0_t.detach().cpu().numpy(), ut, grad=True, grad_kappa=True)
            ctx.save_for_backward(torch.from_numpy(gu), torch.from_numpy(gk * kappa))
            return torch.tensor(loss, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            gu, gg = ctx.saved_tensors
            return gout * gu, gout * gg

    u0_t = torch.tensor(u0, dtype=torch.float64, requires_grad=True)
    gq_t = torch.tensor(np.log(kq), dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(HeatLoss.apply, (u0_t, gq_t), eps=1e-6, atol=1e-7, rtol=1e-6,
                                    fast_mode=True)


def test_adjoint_with_mixed_forward(ads_mod, oracle_mod):
    """Mixed-precision forward (double-float increments, refinement to 1e-13),
    FP64 backward: the gradient matches the FP64 reference gradient to the
    forward's refinement tolerance."""
    n = (7 + 1,) * 3
    gm = ads_mod.ADS(n, (2, 2, 2), precision=ads_mod.PREC_MIXED)
    o = oracle_mod.Oracle(n, (2, 2, 2))
    rng = np.random.default_rng(21)
    kq = np.exp(0.5 * rng.standard_normal(gm.nqp))
    dt = 1e-3
    gm.set_form(ads_mod.FORM_HEAT, kappa_qp=kq, dt=dt)
    u0 = rng.standard_normal(gm.N)
    ut = rng.standard_normal(gm.N)
    loss, gu, gk = gm.heat_adjoint(5, 2, u0, ut, grad=True, grad_kappa=True)
    lo, gou, gok = o.heat_adjoint(5, u0, ut, kappa_qp=kq, dt=dt, want_kappa_grad=True)
    assert abs(loss - lo) < 1e-10 * abs(lo)
    assert rel_l2(gu, gou) < 1e-10
    assert rel_l2(gk, gok) < 1e-10


def test_adjoint_errors(ads_mod):
    g = ads_mod.ADS((6, 6, 6), (2, 2, 2))
    g.set_form(ads_mod.FORM_PROJECT)
    with pytest.raises(ads_mod.ADSError) as e:
        g.heat_adjoint(3, 1, np.zeros(g.N), np.zeros(g.N))
    assert e.value.status == 8
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-3)
    with pytest.raises(ads_mod.ADSError) as e:
        g.heat_adjoint(3, 1, np.zeros(g.N), np.zeros(g.N), grad_kappa=True)
    assert e.value.status == 8
