"""The oracle's MultiStep (src/ADS.F90:391-429) against dense Kronecker
algebra: substep s solves (A_s (x) A_s (x) A_s) u_s = F_s, A_s the MKBBT mix
of the substep, with F_s assembled from the start-of-step value (Un) and the
current gradient (dUn of FormUn(s)); the mixes with an advection part make
the banded LU pivot."""
import numpy as np
import pytest

from conftest import rel_l2

# substep rows of (M, K, B, BT) weights; the last two are dominated by the
# advection B, so the LU pivots, and stay well conditioned (1-D cond <= 6e2)
MIXES = np.array([[1.0, 0.0, 0.0, 0.0],
                  [0.2, 0.0, 1.0, 0.3],
                  [0.3, 0.01, 1.0, -0.5]])


def dense_1d(o, axis, mix):
    t = o.axis_tables(axis)
    NN, J, W, O = t["NN"], t["J"], t["W"], t["O"]
    E, q, pp1, _ = NN.shape
    n1 = o.ndof[axis]
    A = np.zeros((n1, n1))
    for e in range(E):
        for k in range(q):
            v, d = NN[e, k, :, 0], NN[e, k, :, 1]
            sl = slice(O[e], O[e] + pp1)
            jw = J[e] * W[k]
            A[sl, sl] += jw * (mix[0] * np.outer(v, v) + mix[1] * np.outer(d, d)
                               + mix[2] * np.outer(d, v) + mix[3] * np.outer(v, d))
    return A


def kron3(o, mix):
    Ax, Ay, Az = (dense_1d(o, d, mix) for d in range(3))
    return np.kron(Az, np.kron(Ay, Ax))   # x fastest


@pytest.mark.parametrize("n,p", [((5, 6, 4), 2), ((4, 4, 5), 3)])
def test_oracle_multistep_heat_matches_dense_algebra(oracle_mod, n, p):
    o = oracle_mod.Oracle(n, (p, p, p))
    u0 = np.random.default_rng(sum(n) + p).standard_normal(o.N)
    kappa, dt = 1.3, 2e-3
    M3 = kron3(o, (1, 0, 0, 0))
    Ms = [dense_1d(o, d, (1, 0, 0, 0)) for d in range(3)]
    Ks = [dense_1d(o, d, (0, 1, 0, 0)) for d in range(3)]
    K3 = (np.kron(Ms[2], np.kron(Ms[1], Ks[0])) + np.kron(Ms[2], np.kron(Ks[1], Ms[0]))
          + np.kron(Ks[2], np.kron(Ms[1], Ms[0])))
    u = u0.copy()
    for s in range(3):
        F = M3 @ u0 - dt * kappa * (K3 @ u)
        u = np.linalg.solve(kron3(o, MIXES[s]), F)
    o.set_coeffs(u0)
    l2 = o.multistep(oracle_mod.FORM_HEAT, MIXES, kappa=kappa, dt=dt)
    assert rel_l2(o.coeffs(), u) < 1e-11
    assert abs(l2 - u0 @ (M3 @ u0)) < 1e-12 * abs(u0 @ (M3 @ u0))
    assert any(o.pivoted())  # the last substep's LU interchanged rows


def test_oracle_multistep_of_projection_with_mass_mixes_is_a_step(oracle_mod):
    o = oracle_mod.Oracle((6, 5, 7), (2, 2, 2))
    f = np.random.default_rng(1).standard_normal(o.nqp)
    o.step(oracle_mod.FORM_PROJECT, fqp=f)
    ref = o.coeffs()
    o.set_coeffs(np.zeros(o.N))
    o.multistep(oracle_mod.FORM_PROJECT, np.tile([1.0, 0.0, 0.0, 0.0], (3, 1)), fqp=f)
    assert rel_l2(o.coeffs(), ref) < 1e-14
