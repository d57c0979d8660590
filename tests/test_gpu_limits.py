"""The tuned GPU path at its size limit: 448 DOFs along one axis (the longest
line the sweeps stage in shared memory; the column z sweep then holds 3 tiles
per SM, the skewed sweeps 2), against the oracle; one DOF more switches the
FP64 path to banded LU solves and refuses mixed precision."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [(448, 9, 10), (9, 448, 10), (9, 10, 448)])
@pytest.mark.parametrize("prec", [0, 1])
def test_solve_at_the_axis_limit(ads_mod, oracle_mod, N, prec):
    p = 2
    n = tuple(v - 1 for v in N)  # functions minus one
    g = ads_mod.ADS(n, (p, p, p), precision=prec)
    assert g.ndof == N
    o = oracle_mod.Oracle(n, (p, p, p))
    F = np.random.default_rng(sum(N) + prec).standard_normal(g.N)
    u = g.solve(F)
    uo = o.solve(F)
    if prec == 0:
        assert rel_l2(u, uo) < 1e-12
    else:
        st = g.stats()
        assert st["converged"] and st["rel_residual"] <= 1e-13
        assert rel_l2(u, uo) < 1e-10


def test_one_dof_beyond_the_limit(ads_mod, oracle_mod):
    n = (448, 8, 8)  # 449 DOFs along x
    g = ads_mod.ADS(n, (2, 2, 2))
    o = oracle_mod.Oracle(n, (2, 2, 2))
    F = np.random.default_rng(5).standard_normal(g.N)
    assert rel_l2(g.solve(F), o.solve(F)) < 1e-12
    with pytest.raises(ads_mod.ADSError) as e:
        ads_mod.ADS(n, (2, 2, 2), precision=ads_mod.PREC_MIXED)
    assert e.value.status == 7
