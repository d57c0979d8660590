"""One Step on a caller's state arrays (ads_step_host, the reference's Step
updating its state in place, src/ADS.F90:437-461) against ads_set_coeffs +
ads_step + ads_get_coeffs on a second handle: the same coefficients and l2norm
bit for bit, on every route (the step's kernels reading and writing pinned or
pageable buffers in place, the redo after a scale miss, staged copies)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE, P, DT = (21, 20, 19), 2, 1e-5


def _pinned(ads_mod, n):
    torch = pytest.importorskip("torch")
    return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()


def _pair(ads_mod, prec):
    hs = []
    for _ in range(2):
        g = ads_mod.ADS(SHAPE, (P, P, P), precision=prec, refine_tol=1e-13)
        g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=DT)
        hs.append(g)
    return hs


def _staged(g, u):
    g.set_coeffs(u)
    l2 = g.step()
    return g.coeffs(), l2


def _u0(n, seed=3):
    return np.random.default_rng(seed).standard_normal(n)


@pytest.mark.parametrize("buffers", ["pinned", "pinned_in_place", "pageable"])
def test_step_host_matches_three_calls(ads_mod, buffers):
    ref, g = _pair(ads_mod, ads_mod.PREC_MIXED)
    u = _u0(g.N)
    if buffers == "pageable":
        u_in, out = u.copy(), np.empty(g.N)
    else:
        u_in, out = _pinned(ads_mod, g.N), _pinned(ads_mod, g.N)
        u_in[:] = u
    if buffers == "pinned_in_place":
        out = u_in
    want = u
    for step in range(3):
        want, l2_want = _staged(ref, want)
        src = u_in if step == 0 or buffers == "pinned_in_place" else out
        l2 = g.step_host(src, out)
        path = g.stats()["host_path"]
        if buffers == "pageable":
            assert path in (0, 1)  # 1 where the device reads pageable memory
        else:
            assert path == 1
        assert l2 == l2_want
        assert np.array_equal(out, want)
        assert np.array_equal(g.coeffs(), want)  # the handle's state is the step's result
        assert g.stats()["converged"] and g.stats()["fp64_residuals"] == ref.stats()["fp64_residuals"]


@pytest.mark.parametrize("binades,path", [(8, 1), (-8, 1), (9, 2), (40, 2), (-40, 2)])
def test_step_host_scale_window(ads_mod, binades, path):
    """The scale comes from the previous step: within 8 binades of the exact
    one the step runs on it (a power of two commutes with the double-float
    arithmetic's roundings, so the result is the exact scale's); beyond, the
    step is redone on staged copies.  In place, so a redo also shows that the
    discarded attempt wrote nothing."""
    ref, g = _pair(ads_mod, ads_mod.PREC_MIXED)
    base = _u0(g.N)
    buf = _pinned(ads_mod, g.N)
    buf[:] = base
    g.step_host(buf, buf)  # leaves the exact scale of base
    assert g.stats()["host_path"] == 1
    x = np.ldexp(base, binades)
    want, l2_want = _staged(ref, x)
    buf[:] = x
    l2 = g.step_host(buf, buf)
    assert g.stats()["host_path"] == path
    assert l2 == l2_want
    assert np.array_equal(buf, want)
    # the next step starts from the exact scale of what it was given
    want2, l2_want2 = _staged(ref, want)
    assert g.step_host(buf, buf) == l2_want2
    assert g.stats()["host_path"] == 1
    assert np.array_equal(buf, want2)


def test_step_host_zero_state(ads_mod):
    ref, g = _pair(ads_mod, ads_mod.PREC_MIXED)
    buf = _pinned(ads_mod, g.N)
    buf[:] = _u0(g.N)
    g.step_host(buf, buf)
    buf[:] = 0.0
    want, l2_want = _staged(ref, np.zeros(g.N))
    assert g.step_host(buf, buf) == l2_want
    assert g.stats()["host_path"] == 1
    assert np.array_equal(buf, want)


@pytest.mark.parametrize("prec", ["fp64", "mixed_fast"])
def test_step_host_staged_precisions(ads_mod, prec):
    """FP64 and the FP32 increment go through staged copies, with the same
    results as the three calls."""
    pr = {"fp64": ads_mod.PREC_FP64, "mixed_fast": ads_mod.PREC_MIXED_FAST}[prec]
    ref, g = _pair(ads_mod, pr)
    u_in, out = _pinned(ads_mod, g.N), _pinned(ads_mod, g.N)
    u_in[:] = _u0(g.N)
    want, l2_want = _staged(ref, u_in.copy())
    assert g.step_host(u_in, out) == l2_want
    assert g.stats()["host_path"] == 0
    assert np.array_equal(out, want)


def test_step_host_then_graph_steps(ads_mod):
    """A step on host buffers leaves the handle where ads_step continues."""
    ref, g = _pair(ads_mod, ads_mod.PREC_MIXED)
    buf = _pinned(ads_mod, g.N)
    buf[:] = _u0(g.N)
    ref.set_coeffs(buf.copy())
    l2a = [ref.step()] + list(ref.steps(4))
    l2b = [g.step_host(buf, buf)] + list(g.steps(4))
    assert g.stats()["host_path"] == 0
    assert l2a == l2b
    assert np.array_equal(ref.coeffs(), g.coeffs())


def test_step_host_rejects_bad_arrays(ads_mod):
    g = ads_mod.ADS(SHAPE, (P, P, P), precision=ads_mod.PREC_MIXED)
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=DT)
    with pytest.raises(ValueError):
        g.step_host(np.zeros(g.N - 1))
    with pytest.raises(ValueError):
        g.step_host(np.zeros(g.N, dtype=np.float32))
    with pytest.raises(ValueError):
        g.step_host(np.zeros((g.N, 2))[:, 0])


def test_step_host_general_geometry_staged(ads_mod):
    """Unequal degrees per axis (general geometry, FP64) take the staged
    copies, with the three calls' results."""
    hs = []
    for _ in range(2):
        g = ads_mod.ADS((13, 12, 11), (2, 3, 1), precision=ads_mod.PREC_FP64)
        g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=DT)
        hs.append(g)
    ref, g = hs
    u_in, out = _pinned(ads_mod, g.N), _pinned(ads_mod, g.N)
    u_in[:] = _u0(g.N)
    want, l2_want = _staged(ref, u_in.copy())
    assert g.step_host(u_in, out) == l2_want
    assert g.stats()["host_path"] == 0
    assert np.array_equal(out, want)
