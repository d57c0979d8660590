"""Per-phase timers under the reference's PERFORMANCE names
(src/ADS.F90:497-754) through the C-ABI: the phases of a timed step and their
sum against the per-kernel timers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,expect", [
    (0, {"Form 3D RHS", "Solve 1", "Solve 2", "Solve 3"}),
    (1, {"Form 3D RHS", "Solve 1", "Solve 2", "Solve 3", "Refinement", "Update"}),
])
def test_phase_timers_cover_the_step(ads_mod, prec, expect):
    p = 2
    g = ads_mod.ADS((21, 20, 19), (p, p, p), precision=prec)
    g.set_coeffs(np.random.default_rng(1).standard_normal(g.N))
    g.set_form(ads_mod.FORM_HEAT, kappa=1.0, dt=1e-5)
    g.timing(True)
    g.timing_reset()
    g.steps(2)
    kernels = g.timing_read()
    phases = g.phase_timing_read()
    g.timing(False)
    assert expect <= set(phases), phases
    assert set(phases) <= expect | {"Other"}
    assert sum(v[1] for v in phases.values()) == sum(v[1] for v in kernels.values())
    tk = sum(v[0] for v in kernels.values())
    assert abs(sum(v[0] for v in phases.values()) - tk) <= 1e-9 * max(tk, 1.0)
    assert phases["Form 3D RHS"][0] > 0


def test_phase_timers_of_the_banded_solve(ads_mod):
    g = ads_mod.ADS((11, 12, 10), (2, 3, 2))
    g.timing(True)
    g.timing_reset()
    g.solve(np.ones(g.N))
    phases = g.phase_timing_read()
    g.timing(False)
    assert {"Solve 1", "Solve 2", "Solve 3"} <= set(phases)
