// setup.h — host-side setup tables (knots, Gauss rule, basis tables, mass band, LU factors).
#pragma once
#include <vector>

namespace ads {

struct AxisHost {
  int n = 0, p = 0, q = 0, E = 0, N = 0;
  std::vector<double> U;    // n+p+2 knots
  std::vector<int> O;       // first DOF of each element
  std::vector<double> J;    // element Jacobians
  std::vector<double> W;    // Gauss weights
  std::vector<double> X;    // [E][q] Gauss points
  std::vector<double> JW;   // [E][q] J(e) W(k)
  std::vector<double> NN;   // [E][q][p+1][2]
  std::vector<double> DD;   // [E][q][p]: D_b = p N_{j,p-1} / (U_{j+p} - U_j), j = O(e) + b, b = 1..p;
                            // dN_b/dx = D_b - D_{b+1} (D_0 = D_{p+1} = 0)
  std::vector<double> band; // [(m+p)*N + i] = M[i][i+m]
};

void open_knot(int n, int p, std::vector<double>& U);
int gauss_legendre(int q, double* x, double* w);
int axis_setup(int n, int p, AxisHost& a);
// FindSpan (src/basis.F90:226-259): the knot span of x, clamped to [p, n]
int find_span(const AxisHost& a, double x);
// The p+1 nonzero B-splines at the res sample points lerp(i/(res-1), t0, t1)
// of SaveSplinePlot (src/plot.F90:126-133): B[i*(p+1) + r] = N_{first[i]+r}(x_i)
void sample_basis(const AxisHost& a, double t0, double t1, int res, std::vector<double>& B,
                  std::vector<int>& first);
// MKBBT (src/projection_engine.F90:63-132): mix[0] M + mix[1] K + mix[2] B +
// mix[3] BT with B(a, b) = int N_a' N_b, in LAPACK band storage: kl = ku = p,
// ldab = 3p+1, A(i, j) at AB[(2p + i - j) + ldab j] (rows 0..p-1 hold the fill-in
// of the pivoting and start at zero)
void mix_band(const AxisHost& a, const double mix[4], std::vector<double>& AB);
// banded LU with partial pivoting in place (the DGBTF2 algorithm): L below the
// diagonal, U with kl+ku superdiagonals, ipiv 0-based row interchanges;
// returns 0, or j+1 for a zero pivot in column j
int band_lu(int n, int kl, int ku, double* AB, int ldab, int* ipiv);
// LU factors (see ads_internal.cuh) of the mass band; returns 1 on a zero pivot
int band_factor(const AxisHost& a, std::vector<double>& fac, std::vector<double>& tfac);

}  // namespace ads
