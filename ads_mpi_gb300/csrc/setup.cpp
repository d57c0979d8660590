// setup.cpp — host-side setup tables of the GB300 ADS library.
//
// Knot vector (src/knot_vector.F90:43-130), Gauss rule (src/gauss.F90:71-257),
// B-spline values/derivatives at the Gauss points (src/basis.F90:74-112) and
// the 1-D mass matrix band of MKBBT with mix = (1,0,0,0)
// (src/projection_engine.F90:63-132), followed by its banded LU factorisation
// (done once per configuration; the reference re-analyses and re-factorises
// with MUMPS on every substep, src/ADS.F90:306-361).
//
// The basis values use the triangular Cox-de Boor recurrence for degrees p and
// p-1 and obtain derivatives from the standard derivative formula
// N'_{j,p} = p N_{j,p-1}/(U_{j+p}-U_j) - p N_{j+1,p-1}/(U_{j+p+1}-U_{j+1});
// the reference uses the equivalent Piegl-Tiller algorithm A2.3.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "setup.h"

namespace ads {

void open_knot(int n, int p, std::vector<double>& U) {
  // U has n+p+2 entries: p+1 zeros, interior knots (computed in 32-bit float,
  // as the reference's default-kind REAL division does), p+1 ones.
  U.assign((size_t)(n + p + 2), 0.0);
  const int E = n - p + 1;
  for (int k = 0; k < n + p + 2; ++k) {
    if (k <= p) U[k] = 0.0;
    else if (k >= n + 1) U[k] = 1.0;
    else {
      volatile float a = (float)(k - p);
      volatile float b = (float)E;
      U[k] = (double)(a / b);
    }
  }
}

int gauss_legendre(int q, double* x, double* w) {
  switch (q) {
    case 1: x[0] = 0.0; w[0] = 2.0; return 0;
    case 2: {
      const double a = 1.0 / std::sqrt(3.0);
      x[0] = -a; x[1] = a; w[0] = w[1] = 1.0;
      return 0;
    }
    case 3: {
      const double a = std::sqrt(0.6);
      x[0] = -a; x[1] = 0.0; x[2] = a;
      w[0] = w[2] = 5.0 / 9.0; w[1] = 8.0 / 9.0;
      return 0;
    }
    case 4: {
      const double r = 2.0 * std::sqrt(1.2);
      const double a = std::sqrt((3.0 + r) / 7.0), b = std::sqrt((3.0 - r) / 7.0);
      x[0] = -a; x[1] = -b; x[2] = b; x[3] = a;
      const double s30 = std::sqrt(30.0);
      w[0] = w[3] = (18.0 - s30) / 36.0;
      w[1] = w[2] = (18.0 + s30) / 36.0;
      return 0;
    }
    case 5: {
      const double r = 2.0 * std::sqrt(10.0 / 7.0);
      const double a = std::sqrt(5.0 + r) / 3.0, b = std::sqrt(5.0 - r) / 3.0;
      x[0] = -a; x[1] = -b; x[2] = 0.0; x[3] = b; x[4] = a;
      const double s70 = std::sqrt(70.0);
      w[0] = w[4] = (322.0 - 13.0 * s70) / 900.0;
      w[1] = w[3] = (322.0 + 13.0 * s70) / 900.0;
      w[2] = 128.0 / 225.0;
      return 0;
    }
  }
  return 1;
}

// Nonzero B-splines of degree deg on span i (U[i] <= x < U[i+1]) at x:
// N[r] = N_{i-deg+r, deg}(x), r = 0..deg.
static void nonzero_basis(const std::vector<double>& U, int i, int deg, double x, double* N) {
  double left[16], right[16];
  N[0] = 1.0;
  for (int j = 1; j <= deg; ++j) {
    left[j] = x - U[i + 1 - j];
    right[j] = U[i + j] - x;
    double carry = 0.0;
    for (int r = 0; r < j; ++r) {
      const double den = right[r + 1] + left[j - r];
      const double t = N[r] / den;
      N[r] = carry + right[r + 1] * t;
      carry = left[j - r] * t;
    }
    N[j] = carry;
  }
}

int find_span(const AxisHost& a, double x) {
  const int n = a.n, p = a.p;
  const std::vector<double>& U = a.U;
  if (x >= U[n + 1]) return n;
  if (x <= U[p]) return p;
  int low = p, high = n + 1;
  int span = (low + high) / 2;
  while (x < U[span] || x >= U[span + 1]) {
    if (x < U[span]) high = span;
    else low = span;
    span = (low + high) / 2;
  }
  return span;
}

void sample_basis(const AxisHost& a, double t0, double t1, int res, std::vector<double>& B,
                  std::vector<int>& first) {
  B.assign((size_t)res * (a.p + 1), 0.0);
  first.assign(res, 0);
  for (int i = 0; i < res; ++i) {
    const double t = i / (double)(res - 1);
    const double x = (1.0 - t) * t0 + t * t1;  // lerp, src/math.F90:44-51
    const int span = find_span(a, x);
    nonzero_basis(a.U, span, a.p, x, &B[(size_t)i * (a.p + 1)]);
    first[i] = span - a.p;
  }
}

int axis_setup(int n, int p, AxisHost& a) {
  if (p < 1 || p > 4 || n < p) return 1;
  a.n = n; a.p = p; a.q = p + 1;
  open_knot(n, p, a.U);
  // elements = distinct knot spans (uniform open knots: n-p+1 of them)
  a.O.clear();
  for (int i = p; i <= n; ++i)
    if (a.U[i] != a.U[i + 1]) a.O.push_back(i - p);
  a.E = (int)a.O.size();
  a.N = n + 1;
  const int q = a.q;
  double xg[8], wg[8];
  if (gauss_legendre(q, xg, wg)) return 2;
  a.W.assign(wg, wg + q);
  a.J.assign(a.E, 0.0);
  a.X.assign((size_t)a.E * q, 0.0);
  a.NN.assign((size_t)a.E * q * (p + 1) * 2, 0.0);
  a.DD.assign((size_t)a.E * q * p, 0.0);
  a.JW.assign((size_t)a.E * q, 0.0);
  double Np[16], Nm[16];
  for (int e = 0; e < a.E; ++e) {
    const int i = a.O[e] + p;
    const double J = (a.U[i + 1] - a.U[i]) / 2.0;
    a.J[e] = J;
    for (int k = 0; k < q; ++k) {
      const double x = (xg[k] + 1.0) * J + a.U[i];
      a.X[(size_t)e * q + k] = x;
      a.JW[(size_t)e * q + k] = J * wg[k];
      nonzero_basis(a.U, i, p, x, Np);
      nonzero_basis(a.U, i, p - 1, x, Nm);
      for (int r = 0; r <= p; ++r) {
        const int j = i - p + r;  // global function index
        double d = 0.0;
        if (r >= 1) {
          const double den = a.U[j + p] - a.U[j];
          if (den != 0.0) d += p * Nm[r - 1] / den;
        }
        if (r <= p - 1) {
          const double den = a.U[j + p + 1] - a.U[j + 1];
          if (den != 0.0) d -= p * Nm[r] / den;
        }
        a.NN[(((size_t)e * q + k) * (p + 1) + r) * 2 + 0] = Np[r];
        a.NN[(((size_t)e * q + k) * (p + 1) + r) * 2 + 1] = d;
        if (r >= 1) {
          const double den = a.U[j + p] - a.U[j];
          a.DD[((size_t)e * q + k) * p + (r - 1)] = (den != 0.0) ? p * Nm[r - 1] / den : 0.0;
        }
      }
    }
  }
  // mass band M[i][i+m], m = -p..p, as band[(m+p)*N + i]
  const int N = a.N;
  a.band.assign((size_t)(2 * p + 1) * N, 0.0);
  for (int e = 0; e < a.E; ++e)
    for (int k = 0; k < q; ++k)
      for (int c = 0; c <= p; ++c)
        for (int d = 0; d <= p; ++d) {
          const int ia = a.O[e] + c, ib = a.O[e] + d;
          const double vc = a.NN[(((size_t)e * q + k) * (p + 1) + c) * 2];
          const double vd = a.NN[(((size_t)e * q + k) * (p + 1) + d) * 2];
          a.band[(size_t)(ib - ia + p) * N + ia] += vc * vd * a.J[e] * a.W[k];
        }
  return 0;
}

void mix_band(const AxisHost& a, const double mix[4], std::vector<double>& AB) {
  const int p = a.p, n1 = a.N, ldab = 3 * p + 1;
  AB.assign((size_t)ldab * n1, 0.0);
  // contributions summed in MKBBT's order: element, point, row function, column function
  for (int e = 0; e < a.E; ++e)
    for (int k = 0; k < a.q; ++k)
      for (int c = 0; c <= p; ++c)
        for (int d = 0; d <= p; ++d) {
          auto nn = [&](int der, int f) { return a.NN[(((size_t)e * a.q + k) * (p + 1) + f) * 2 + der]; };
          const double M = nn(0, c) * nn(0, d) * a.J[e] * a.W[k];
          const double K = nn(1, c) * nn(1, d) * a.J[e] * a.W[k];
          const double B = nn(1, c) * nn(0, d) * a.J[e] * a.W[k];
          const double BT = nn(0, c) * nn(1, d) * a.J[e] * a.W[k];
          const int ia = a.O[e] + c, ib = a.O[e] + d;
          AB[(size_t)(2 * p + ia - ib) + (size_t)ldab * ib] += mix[0] * M + mix[1] * K + mix[2] * B + mix[3] * BT;
        }
}

int band_lu(int n, int kl, int ku, double* AB, int ldab, int* ipiv) {
  const int kv = ku + kl;
  auto at = [&](int i, int j) -> double& { return AB[(size_t)(kv + i - j) + (size_t)ldab * j]; };
  int ju = 0;  // last column touched by the row interchanges so far
  for (int j = 0; j < n; ++j) {
    const int km = std::min(kl, n - 1 - j);
    int jp = 0;
    double amax = std::fabs(at(j, j));
    for (int i = 1; i <= km; ++i)
      if (std::fabs(at(j + i, j)) > amax) { amax = std::fabs(at(j + i, j)); jp = i; }
    ipiv[j] = j + jp;
    if (at(j + jp, j) == 0.0) return j + 1;
    ju = std::max(ju, std::min(j + ku + jp, n - 1));
    if (jp != 0)
      for (int c = j; c <= ju; ++c) std::swap(at(j + jp, c), at(j, c));
    if (km > 0) {
      const double r = 1.0 / at(j, j);
      for (int i = 1; i <= km; ++i) at(j + i, j) *= r;
      for (int c = j + 1; c <= ju; ++c) {
        const double u = at(j, c);
        if (u != 0.0)
          for (int i = 1; i <= km; ++i) at(j + i, c) += at(j + i, j) * -u;
      }
    }
  }
  return 0;
}

int band_factor(const AxisHost& a, std::vector<double>& fac, std::vector<double>& tfac) {
  const int p = a.p, N = a.N, w = 2 * p + 1;
  // A[i][m+p] = M[i][i+m]
  std::vector<double> A((size_t)N * w);
  for (int i = 0; i < N; ++i)
    for (int m = -p; m <= p; ++m) A[(size_t)i * w + m + p] = a.band[(size_t)(m + p) * N + i];
  double dmax = 0.0;
  for (int i = 0; i < N; ++i) dmax = std::fmax(dmax, std::fabs(A[(size_t)i * w + p]));
  for (int k = 0; k < N; ++k) {
    const double piv = A[(size_t)k * w + p];
    if (!(std::fabs(piv) > 1e-300) || !(std::fabs(piv) > 1e-14 * dmax)) return 1;  // zero pivot
    for (int i = k + 1; i <= std::min(k + p, N - 1); ++i) {
      const double l = A[(size_t)i * w + (k - i + p)] / piv;
      A[(size_t)i * w + (k - i + p)] = l;
      for (int j = k + 1; j <= std::min(k + p, N - 1); ++j) A[(size_t)i * w + (j - i + p)] -= l * A[(size_t)k * w + (j - k + p)];
    }
  }
  auto Lf = [&](int i, int j) { return A[(size_t)i * w + (j - i + p)]; };  // j < i
  auto Uf = [&](int i, int j) { return A[(size_t)i * w + (j - i + p)]; };  // j >= i
  const int rows = 2 * p + 2;
  fac.assign((size_t)rows * N, 0.0);
  tfac.assign((size_t)rows * N, 0.0);
  for (int i = 0; i < N; ++i) {
    const double dinv = 1.0 / Uf(i, i);
    // normal: fs = 1, f[m] = L(i, i-m), bs = 1/U(i,i), g[m] = U(i, i+m)/U(i,i)
    fac[(size_t)0 * N + i] = 1.0;
    fac[(size_t)(p + 1) * N + i] = dinv;
    for (int m = 1; m <= p; ++m) {
      fac[(size_t)m * N + i] = (i - m >= 0) ? Lf(i, i - m) : 0.0;
      fac[(size_t)(p + 1 + m) * N + i] = (i + m < N) ? Uf(i, i + m) * dinv : 0.0;
    }
    // transposed: fs = 1/U(i,i), f[m] = U(i-m, i)/U(i,i), bs = 1, g[m] = L(i+m, i)
    tfac[(size_t)0 * N + i] = dinv;
    tfac[(size_t)(p + 1) * N + i] = 1.0;
    for (int m = 1; m <= p; ++m) {
      tfac[(size_t)m * N + i] = (i - m >= 0) ? Uf(i - m, i) * dinv : 0.0;
      tfac[(size_t)(p + 1 + m) * N + i] = (i + m < N) ? Lf(i + m, i) : 0.0;
    }
  }
  return 0;
}

}  // namespace ads
