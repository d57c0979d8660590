"""Solution output (PrintSolution, src/ADS.F90:955-989): the VtkOutput writer
(src/vtk.F90:15-77) without a GPU, and the oracle's SaveSplinePlot sampling
(src/plot.F90:111-140 with EvalSpline, src/basis.F90:323-369) against
scipy's independent B-spline evaluation."""
import numpy as np
import pytest


def test_write_vti_reproduces_vtkoutput_text(ads_mod, tmp_path):
    # values as F30.10 writes them (after adjustl/trim): fixed notation, 10
    # decimals, 30 asterisks when the number does not fit in 30 characters
    cases = [(0.5, "0.5000000000"), (-1.25, "-1.2500000000"), (0.0, "0.0000000000"),
             (1234.56789012344, "1234.5678901234"), (-3e-11, "-0.0000000000"),
             (1e25, "*" * 30), (2.0 / 3.0, "0.6666666667"), (float("nan"), "NaN")]
    vals = np.array([v for v, _ in cases]).reshape(2, 1, 4)  # (resz, resy, resx) = 4 x 1 x 2
    ads_mod.write_vti(str(tmp_path / "step7"), vals)
    text = (tmp_path / "step7.vti").read_text().splitlines()
    extent = "0     3 0     0 0     1"  # ("0 ",I5," 0 ",I5," 0 ",I5) of res - 1
    head = ['<?xml version="1.0"?>', '<VTKFile type="ImageData" version="0.1">',
            f'  <ImageData WholeExtent="{extent}" origin="0 0 0" spacing="1 1 1">',
            f'    <Piece Extent="{extent}">', '      <PointData Scalars="Result">',
            '        <DataArray Name="Result" type="Float32">']
    tail = ['        </DataArray>', '      </PointData>', '    </Piece>', '  </ImageData>', '</VTKFile>']
    assert text == head + ["          " + s for _, s in cases] + tail


def test_write_vti_rejects_bad_arguments(ads_mod, tmp_path):
    with pytest.raises(ads_mod.ADSError):
        ads_mod.write_vti(str(tmp_path / "no_such_dir" / "x"), np.zeros((2, 2, 2)))


@pytest.mark.parametrize("n,p", [((9, 7, 8), 2), ((6, 5, 7), 1), ((8, 9, 6), 3), ((7, 6, 6), 4)])
def test_oracle_spline_samples_match_scipy(oracle_mod, n, p):
    from scipy.interpolate import BSpline
    o = oracle_mod.Oracle(n, (p, p, p))
    u = np.random.default_rng(sum(n) + p).standard_normal(o.N)
    o.set_coeffs(u)
    rng, res = (0.0, 1.0, 0.05, 0.95, 0.0, 1.0), (31, 17, 13)
    vals = o.eval_spline_grid(rng, res)
    B = []
    for d in range(3):
        U = o.axis_tables(d)["U"]
        x = np.array([(1.0 - i / (res[d] - 1)) * rng[2 * d] + i / (res[d] - 1) * rng[2 * d + 1]
                      for i in range(res[d])])
        B.append(BSpline.design_matrix(x, U, p).toarray())
    Nx, Ny, Nz = o.ndof
    ref = np.einsum("zk,yj,xi,kji->zyx", B[2], B[1], B[0], u.reshape(Nz, Ny, Nx))
    assert np.abs(vals - ref).max() <= 1e-13 * np.abs(ref).max()
