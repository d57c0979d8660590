"""GPU solution output through the C-ABI against the oracle: SaveSplinePlot's
samples of the coefficients (src/plot.F90:111-140) and the .vti file that
PrintSolution writes (src/ADS.F90:955-989, src/vtk.F90:15-77)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("E,p", [((9, 10, 7), 2), ((6, 5, 4), 1), ((7, 6, 8), 3), ((6, 7, 5), 4), ((40, 19, 11), 2)])
def test_spline_samples_match_oracle(ads_mod, oracle_mod, E, p):
    n = tuple(e + p - 1 for e in E)
    g = ads_mod.ADS(n, (p, p, p))
    o = oracle_mod.Oracle(n, (p, p, p))
    u = np.random.default_rng(sum(E) + p).standard_normal(g.N)
    g.set_coeffs(u)
    o.set_coeffs(u)
    for rng, res in (((0.0, 1.0, 0.0, 1.0, 0.0, 1.0), (31, 31, 31)),
                     ((0.1, 0.9, 0.0, 0.5, 0.25, 1.0), (17, 40, 2))):
        v = g.save_spline_plot(rng=rng, res=res)
        vo = o.eval_spline_grid(rng, res)
        assert np.abs(v - vo).max() <= 1e-13 * np.abs(vo).max()


def test_print_solution_writes_the_reference_file(ads_mod, oracle_mod, tmp_path):
    """PrintSolution after an L2 projection of 1 (problems/L2Projection): every
    sample is 1, and the file equals VtkOutput of the returned samples."""
    E, p = (12, 12, 12), 2
    n = tuple(e + p - 1 for e in E)
    g = ads_mod.ADS(n, (p, p, p))
    g.set_form(ads_mod.FORM_PROJECT)
    g.step()
    v = g.print_solution(3, directory=str(tmp_path))
    assert v.shape == (31, 31, 31)
    assert np.abs(v - 1.0).max() < 1e-10
    ads_mod.write_vti(str(tmp_path / "again"), v)
    assert (tmp_path / "step3.vti").read_text() == (tmp_path / "again.vti").read_text()
    lines = (tmp_path / "step3.vti").read_text().splitlines()
    assert len(lines) == 6 + 31 ** 3 + 5
    assert all(s.strip() in ("1.0000000000", "0.9999999999") for s in lines[6:6 + 31 ** 3])


def test_spline_plot_rejects_bad_resolution(ads_mod):
    g = ads_mod.ADS((8, 8, 8), (2, 2, 2))
    with pytest.raises(ads_mod.ADSError) as e:
        g.save_spline_plot(res=(1, 31, 31))
    assert e.value.status == 1
