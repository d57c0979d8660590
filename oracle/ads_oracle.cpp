// ads_oracle.cpp — CPU ORACLE (test infrastructure only).
//
// A C++ restatement of the IGA-ADS (macwozni/ADS_MPI) FP64 time-step path, used
// only as the correctness checker by tests/, by __graft_entry__.smoke() and as
// the timed CPU baseline leg of bench.py.  Nothing in the product links or
// calls this file.
//
// Parity pinning: the knot routines are checked against the golden vectors of
// tests/test_knot.pf (tests/golden/knot_vectors.json), and the whole path is
// checked against the reference's own known-answer test, the L2 projection of
// f == 1 (problems/L2Projection/main.F90:62,72-78).  Nothing in the reference
// pins the MUMPS solve (src/ADS.F90:294-379) bit for bit; it is replaced here by
// the banded LU with partial pivoting that the comment at src/ADS.F90:288-293
// names (DGBSV semantics).
//
// Every function cites the reference routine it restates.  The loop nests of
// FormUn / Form3DRHS keep the reference's per-point structure (the integrand
// is called through a function pointer once per (quadrature point, test
// function), as the Fortran procedure argument RHS_fun is), and the quadrature
// arrays Un/dUn are materialised with the reference's (ex,ey,ez,kx,ky,kz)
// column-major layout (src/ADS.F90:187-190).
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API extern "C" __attribute__((visibility("default")))

// ---------------------------------------------------------------------------
// knot_vector.F90
// ---------------------------------------------------------------------------

// FillOpenKnot (src/knot_vector.F90:79-92).  U has n+p+2 entries; interior
// knots are computed in default-kind (32-bit) REAL arithmetic and then stored
// in a REAL(8) array, exactly as the Fortran `real(i-p-1)/real(n-p+1)` does.
ORC_API void orc_fill_open_knot(int n, int p, double* U) {
  const int len = n + p + 2;
  for (int i = 1; i <= p + 1; ++i)
    if (i >= 1 && i <= len) U[i - 1] = 0.0;
  for (int i = n + 2; i <= n + p + 2; ++i)
    if (i >= 1 && i <= len) U[i - 1] = 1.0;
  for (int i = p + 2; i <= n + 1; ++i) {
    volatile float num = (float)(i - p - 1);
    volatile float den = (float)(n - p + 1);
    float q = num / den;
    U[i - 1] = (double)q;
  }
}

// CountSpans (src/knot_vector.F90:110-130, identical copy in src/basis.F90:279-299).
// U is indexed 0..n+p+1 as in the Fortran dummy argument.
ORC_API int orc_count_spans(int n, int p, const double* U) {
  int nelem = 0;
  int i = p;
  while (i <= n) {
    while (i < n && U[i] == U[i + 1]) ++i;
    ++nelem;
    ++i;
  }
  return nelem;
}

// PrepareKnot (src/knot_vector.F90:43-59): allocate + fill + count.
ORC_API int orc_prepare_knot(int n, int p, double* U, int* nelem) {
  if (n + p + 2 < 1) return 1;
  orc_fill_open_knot(n, p, U);
  *nelem = orc_count_spans(n, p, U);
  return 0;
}

// ---------------------------------------------------------------------------
// gauss.F90
// ---------------------------------------------------------------------------

// GaussRule (src/gauss.F90:213-257) with the point/weight table of
// src/gauss.F90:71-193.  For 1..5 points the reference uses closed forms, which
// are restated here.  For 6..10 points the reference lists 15-16 digit
// decimals; this oracle computes the Gauss-Legendre nodes by Newton iteration on
// the Legendre polynomial (Golub-Welsch-free textbook method), which agrees with
// those decimals to about 1e-15.  The GPU path supports p <= 4 (q <= 5) only.
ORC_API int orc_gauss_rule(int q, double* X, double* W) {
  switch (q) {
    case 1:
      X[0] = 0.0; W[0] = 2.0; return 0;
    case 2:
      X[0] = -1.0 / std::sqrt(3.0); X[1] = -X[0];
      W[0] = 1.0; W[1] = 1.0; return 0;
    case 3:
      X[0] = -std::sqrt(3.0 / 5.0); X[1] = 0.0; X[2] = -X[0];
      W[0] = 5.0 / 9.0; W[1] = 8.0 / 9.0; W[2] = W[0]; return 0;
    case 4: {
      const double s = 2.0 * std::sqrt(6.0 / 5.0);
      X[0] = -std::sqrt((3.0 + s) / 7.0);
      X[1] = -std::sqrt((3.0 - s) / 7.0);
      X[2] = -X[1]; X[3] = -X[0];
      W[0] = (18.0 - std::sqrt(30.0)) / 36.0;
      W[1] = (18.0 + std::sqrt(30.0)) / 36.0;
      W[2] = W[1]; W[3] = W[0];
      return 0;
    }
    case 5: {
      const double s = 2.0 * std::sqrt(10.0 / 7.0);
      X[0] = -1.0 / 3.0 * std::sqrt(5.0 + s);
      X[1] = -1.0 / 3.0 * std::sqrt(5.0 - s);
      X[2] = 0.0; X[3] = -X[1]; X[4] = -X[0];
      W[0] = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
      W[1] = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0;
      W[2] = 128.0 / 225.0; W[3] = W[1]; W[4] = W[0];
      return 0;
    }
    default:
      break;
  }
  if (q < 1 || q > 10) {
    for (int i = 0; i < (q > 0 ? q : 0); ++i) { X[i] = 0.0; W[i] = 0.0; }
    return 1;
  }
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < q; ++i) {
    // i-th root from the largest, then mirrored so X is ascending.
    double x = std::cos(pi * (i + 0.75) / (q + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= q; ++k) {
        double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = pk;
      }
      dp = q * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    X[q - 1 - i] = x;
    W[q - 1 - i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  for (int i = 0; i < q / 2; ++i) {  // enforce exact symmetry
    double xs = 0.5 * (X[q - 1 - i] - X[i]);
    X[i] = -xs; X[q - 1 - i] = xs;
    double ws = 0.5 * (W[i] + W[q - 1 - i]);
    W[i] = ws; W[q - 1 - i] = ws;
  }
  if (q % 2 == 1) X[q / 2] = 0.0;
  return 0;
}

// ---------------------------------------------------------------------------
// basis.F90
// ---------------------------------------------------------------------------

// DersBasisFuns (src/basis.F90:136-202): values and derivatives up to order d
// of the p+1 B-splines that are nonzero on knot span i, at point uu (the
// Piegl-Tiller algorithm A2.3).  Output ders[(k)*(p+1) + r] = d^k N_{i-p+r}/du^k,
// matching the Fortran ders(0:p, 0:d) column-major layout.
ORC_API void orc_ders_basis_funs(int i, double uu, int p, int d, const double* U,
                                 double* ders) {
  std::vector<double> left(p + 1), right(p + 1);
  std::vector<double> ndu((p + 1) * (p + 1));  // ndu(j, r) -> ndu[j + (p+1)*r]
  std::vector<double> a(2 * (p + 1));          // a(s, j)   -> a[s + 2*j]
  auto NDU = [&](int j, int r) -> double& { return ndu[j + (p + 1) * r]; };
  auto A = [&](int s, int j) -> double& { return a[s + 2 * j]; };

  NDU(0, 0) = 1.0;
  for (int j = 1; j <= p; ++j) {
    left[j] = uu - U[i + 1 - j];
    right[j] = U[i + j] - uu;
    double saved = 0.0;
    for (int r = 0; r <= j - 1; ++r) {
      NDU(j, r) = right[r + 1] + left[j - r];
      double temp = NDU(r, j - 1) / NDU(j, r);
      NDU(r, j) = saved + right[r + 1] * temp;
      saved = left[j - r] * temp;
    }
    NDU(j, j) = saved;
  }
  for (int r = 0; r <= p; ++r) ders[r] = NDU(r, p);

  for (int r = 0; r <= p; ++r) {
    int s1 = 0, s2 = 1;
    A(0, 0) = 1.0;
    for (int k = 1; k <= d; ++k) {
      double der = 0.0;
      const int rk = r - k, pk = p - k;
      if (r >= k) {
        A(s2, 0) = A(s1, 0) / NDU(pk + 1, rk);
        der = A(s2, 0) * NDU(rk, pk);
      }
      const int j1 = (rk > -1) ? 1 : -rk;
      const int j2 = (r - 1 <= pk) ? k - 1 : p - r;
      for (int j = j1; j <= j2; ++j) {
        A(s2, j) = (A(s1, j) - A(s1, j - 1)) / NDU(pk + 1, rk + j);
        der = der + A(s2, j) * NDU(rk + j, pk);
      }
      if (r <= pk) {
        A(s2, k) = -A(s1, k - 1) / NDU(pk + 1, r);
        der = der + A(s2, k) * NDU(r, pk);
      }
      ders[k * (p + 1) + r] = der;
      std::swap(s1, s2);
    }
  }
  int rr = p;
  for (int k = 1; k <= d; ++k) {
    for (int j = 0; j <= p; ++j) ders[k * (p + 1) + j] = ders[k * (p + 1) + j] * rr;
    rr = rr * (p - k);
  }
}

// BasisData (src/basis.F90:74-112).  Outputs, all 0-based:
//   O[e]                         first nonzero basis function of element e
//   J[e]                         (U(i+1)-U(i))/2
//   W[k]                         Gauss weights
//   X[k + q*e]                   Gauss points mapped to element e
//   NN[dd + (d+1)*(a + (p+1)*(k + q*e))]  = NN(dd, a, k, e) of the Fortran.
ORC_API int orc_basis_data(int p, int m, const double* U, int d, int q, int r,
                           int* O, double* J, double* W, double* X, double* NN) {
  int ir = 0;
  for (int i = p; i <= m - p; ++i) {
    if (i + 1 <= m && U[i] != U[i + 1]) {
      if (ir >= r) return 1;
      O[ir++] = i - p;
    }
  }
  std::vector<double> Xg(q);
  if (orc_gauss_rule(q, Xg.data(), W)) return 2;
  std::vector<double> basis((p + 1) * (d + 1));
  for (int e = 0; e < r; ++e) {
    const int i = O[e] + p;
    J[e] = (U[i + 1] - U[i]) / 2.0;
    for (int k = 0; k < q; ++k) X[k + q * e] = (Xg[k] + 1.0) * J[e] + U[i];
    for (int k = 0; k < q; ++k) {
      orc_ders_basis_funs(i, X[k + q * e], p, d, U, basis.data());
      for (int a = 0; a <= p; ++a)
        for (int dd = 0; dd <= d; ++dd)
          NN[dd + (d + 1) * (a + (p + 1) * (k + q * e))] = basis[dd * (p + 1) + a];
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// math.F90 + problems/heat/input_data.F90
// ---------------------------------------------------------------------------

// falloff (src/math.F90:74-88).
static double orc_falloff(double r, double Rr, double t) {
  if (t < r) return 1.0;
  if (t > Rr) return 0.0;
  double h = (t - r) / (Rr - r);
  double b = (h - 1.0) * (h + 1.0);
  return b * b;
}

// bump3d (src/math.F90:173-181) with norm2 (src/math.F90:197-204).
static double orc_bump3d(double r, double Rr, double x, double y, double z) {
  double a = x - 0.5, b = y - 0.5, c = z - 0.5;
  double t = std::sqrt(a * a + b * b + c * c);
  return orc_falloff(r / 2.0, Rr / 2.0, t);
}

// initial_state of the heat problem (problems/heat/input_data.F90:57-70).
ORC_API double orc_heat_initial_state(double x, double y, double z) {
  return 2.0 * orc_bump3d(0.05, 0.4, x, y, z);
}

// ---------------------------------------------------------------------------
// Banded LU with partial pivoting: the DGBSV semantics that src/ADS.F90:288-293
// documents for SolveOneDirection (LAPACK dgbtf2 + dgbtrs, restated).
// AB is the LAPACK band layout with ldab >= 2*kl+ku+1, column-major:
// A(i,j) = AB[(kl+ku+i-j) + ldab*j] (0-based).
// ---------------------------------------------------------------------------

ORC_API int orc_dgbtrf(int n, int kl, int ku, double* AB, int ldab, int* ipiv) {
  const int kv = ku + kl;
  auto ab = [&](int row, int col) -> double& { return AB[row + ldab * col]; };
  // zero the fill-in rows of the first kv columns
  for (int j = ku + 1; j < std::min(kv, n); ++j)
    for (int i = kv - j; i < kl; ++i) ab(i, j) = 0.0;
  int ju = 0, info = 0;
  for (int j = 0; j < n; ++j) {
    if (j + kv < n)
      for (int i = 0; i < kl; ++i) ab(i, j + kv) = 0.0;
    const int km = std::min(kl, n - 1 - j);
    int jp = 0;
    double best = -1.0;
    for (int i = 0; i <= km; ++i) {
      double v = std::fabs(ab(kv + i, j));
      if (v > best) { best = v; jp = i; }
    }
    ipiv[j] = jp + j;
    if (ab(kv + jp, j) != 0.0) {
      ju = std::max(ju, std::min(j + ku + jp, n - 1));
      if (jp != 0) {
        for (int c = 0; c <= ju - j; ++c) {
          double* a1 = &AB[(kv + jp - c) + ldab * (j + c)];
          double* a2 = &AB[(kv - c) + ldab * (j + c)];
          std::swap(*a1, *a2);
        }
      }
      if (km > 0) {
        double inv = 1.0 / ab(kv, j);
        for (int i = 1; i <= km; ++i) ab(kv + i, j) *= inv;
        if (ju > j) {
          for (int c = 1; c <= ju - j; ++c) {
            double f = ab(kv - c, j + c);
            if (f != 0.0)
              for (int i = 1; i <= km; ++i) ab(kv + i - c, j + c) -= ab(kv + i, j) * f;
          }
        }
      }
    } else if (info == 0) {
      info = j + 1;
    }
  }
  return info;
}

// Single right-hand side solve with the factors of orc_dgbtrf (dgbtrs, 'N').
ORC_API void orc_dgbtrs1(int n, int kl, int ku, const double* AB, int ldab,
                         const int* ipiv, double* b) {
  const int kd = ku + kl;
  auto ab = [&](int row, int col) -> double { return AB[row + ldab * col]; };
  if (kl > 0) {
    for (int j = 0; j < n - 1; ++j) {
      const int lm = std::min(kl, n - 1 - j);
      const int l = ipiv[j];
      if (l != j) std::swap(b[l], b[j]);
      const double bj = b[j];
      for (int i = 1; i <= lm; ++i) b[j + i] -= ab(kd + i, j) * bj;
    }
  }
  for (int j = n - 1; j >= 0; --j) {
    if (b[j] != 0.0) {
      b[j] /= ab(kd, j);
      const double bj = b[j];
      const int lm = std::min(j, kd);
      for (int i = 1; i <= lm; ++i) b[j - i] -= ab(kd - i, j) * bj;
    }
  }
}

// Convenience: dgbsv for nrhs right-hand sides stored column-major (ldb >= n).
ORC_API int orc_dgbsv(int n, int kl, int ku, int nrhs, double* AB, int ldab,
                      int* ipiv, double* B, int ldb) {
  int info = orc_dgbtrf(n, kl, ku, AB, ldab, ipiv);
  if (info) return info;
  for (int c = 0; c < nrhs; ++c) orc_dgbtrs1(n, kl, ku, AB, ldab, ipiv, B + (size_t)ldb * c);
  return 0;
}

// ---------------------------------------------------------------------------
// ADS state (src/Setup.F90:29-140 restricted to one rank)
// ---------------------------------------------------------------------------

struct OrcAxis {
  int n = 0, p = 0, nelem = 0, m = 0, ng = 0;
  std::vector<double> U;   // 0..m
  std::vector<int> O;      // nelem
  std::vector<double> J;   // nelem
  std::vector<double> W;   // ng
  std::vector<double> X;   // ng*nelem
  std::vector<double> NN;  // 2*(p+1)*ng*nelem
  double nn(int d, int a, int k, int e) const {
    return NN[d + 2 * (a + (p + 1) * (k + ng * e))];
  }
};

struct OrcADS {
  OrcAxis ax[3];
  int s[3] = {0, 0, 0};  // DOFs per axis (n+1)
  size_t ndof = 0, nqp = 0;
  std::vector<double> F, F2, F3;     // (s1, s2*s3), (s2, s1*s3), (s3, s1*s2)
  std::vector<double> R;             // R(:,2,2,2) at one rank
  std::vector<double> Un, Un13, Un23, dUn;
  // band factors cached per axis for the current matrix mix
  int last_info = 0;
  int pivoted[3] = {0, 0, 0};
  double drained = 0.0;  // oil problem: sum of J W v Dt vdrain of the last assembly
};

// Index of Un(ex,ey,ez,kx,ky,kz) in the Fortran column-major layout (0-based).
static inline size_t un_index(const OrcADS& A, int ex, int ey, int ez, int kx, int ky, int kz) {
  const size_t E1 = A.ax[0].nelem, E2 = A.ax[1].nelem, E3 = A.ax[2].nelem;
  const size_t q1 = A.ax[0].ng, q2 = A.ax[1].ng;
  return ex + E1 * (ey + E2 * (ez + E3 * (kx + q1 * (ky + q2 * (size_t)kz))));
}

// initialize (src/ADS.F90:11-107) for one rank: PrepareKnot x3, BasisData x3,
// AllocateADSdata (src/ADS.F90:178-203) with R zeroed.
ORC_API OrcADS* orc_create(const int n[3], const int p[3]) {
  for (int d = 0; d < 3; ++d)
    if (n[d] < p[d] || p[d] < 0 || p[d] > 9) return nullptr;
  OrcADS* A = new OrcADS();
  for (int d = 0; d < 3; ++d) {
    OrcAxis& X = A->ax[d];
    X.n = n[d]; X.p = p[d];
    X.U.assign(n[d] + p[d] + 2, 0.0);
    orc_prepare_knot(n[d], p[d], X.U.data(), &X.nelem);
    X.m = X.n + X.p + 1;
    X.ng = X.p + 1;
    X.O.assign(X.nelem, 0); X.J.assign(X.nelem, 0.0); X.W.assign(X.ng, 0.0);
    X.X.assign((size_t)X.ng * X.nelem, 0.0);
    X.NN.assign((size_t)2 * (X.p + 1) * X.ng * X.nelem, 0.0);
    if (orc_basis_data(X.p, X.m, X.U.data(), 1, X.ng, X.nelem, X.O.data(), X.J.data(),
                       X.W.data(), X.X.data(), X.NN.data())) {
      delete A;
      return nullptr;
    }
    A->s[d] = n[d] + 1;
  }
  A->ndof = (size_t)A->s[0] * A->s[1] * A->s[2];
  A->nqp = (size_t)A->ax[0].nelem * A->ax[1].nelem * A->ax[2].nelem * A->ax[0].ng *
           A->ax[1].ng * A->ax[2].ng;
  A->F.assign(A->ndof, 0.0);
  A->F2.assign(A->ndof, 0.0);
  A->F3.assign(A->ndof, 0.0);
  A->R.assign(A->ndof, 0.0);
  A->Un.assign(A->nqp, 0.0);
  A->Un13.assign(A->nqp, 0.0);
  A->Un23.assign(A->nqp, 0.0);
  A->dUn.assign(A->nqp * 3, 0.0);
  return A;
}

ORC_API void orc_destroy(OrcADS* A) { delete A; }

ORC_API void orc_dims(const OrcADS* A, int* nelem, int* ndof, int* nq) {
  for (int d = 0; d < 3; ++d) {
    nelem[d] = A->ax[d].nelem; ndof[d] = A->s[d]; nq[d] = A->ax[d].ng;
  }
}

// Basis tables of one axis (for cross-checks of the GPU host setup).
ORC_API void orc_axis_tables(const OrcADS* A, int axis, double* U, int* O, double* J,
                             double* W, double* X, double* NN) {
  const OrcAxis& a = A->ax[axis];
  if (U) std::memcpy(U, a.U.data(), sizeof(double) * a.U.size());
  if (O) std::memcpy(O, a.O.data(), sizeof(int) * a.O.size());
  if (J) std::memcpy(J, a.J.data(), sizeof(double) * a.J.size());
  if (W) std::memcpy(W, a.W.data(), sizeof(double) * a.W.size());
  if (X) std::memcpy(X, a.X.data(), sizeof(double) * a.X.size());
  if (NN) std::memcpy(NN, a.NN.data(), sizeof(double) * a.NN.size());
}

ORC_API void orc_set_coeffs(OrcADS* A, const double* u) {
  std::memcpy(A->R.data(), u, sizeof(double) * A->ndof);
}
ORC_API void orc_get_coeffs(const OrcADS* A, double* u) {
  std::memcpy(u, A->R.data(), sizeof(double) * A->ndof);
}
ORC_API void orc_get_F(const OrcADS* A, double* F) {
  std::memcpy(F, A->F.data(), sizeof(double) * A->ndof);
}

// ---------------------------------------------------------------------------
// projection_engine.F90
// ---------------------------------------------------------------------------

// FormUn (src/projection_engine.F90:306-441) for one rank: u and grad u of
// the spline with coefficients R at every quadrature point, stored in
// Un / Un13 / Un23 (by subun) and dUn with the reference's layout.
// subun = 1, 2, 3 fills Un, Un13 or Un23 with the values; dUn always
// (src/projection_engine.F90:330-340,424-433)
static void orc_form_un(OrcADS& A, int subun = 1) {
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  std::vector<double>& V = (subun == 1) ? A.Un : (subun == 2 ? A.Un13 : A.Un23);
  std::fill(V.begin(), V.end(), 0.0);
  std::fill(A.dUn.begin(), A.dUn.end(), 0.0);
  const int E1 = X.nelem, E2 = Y.nelem, E3 = Z.nelem;
  const long total = (long)E1 * E2 * E3;
  const size_t nqp = A.nqp;
  const size_t sx = A.s[0], sy = A.s[1];
#pragma omp parallel for schedule(static)
  for (long all = 0; all < total; ++all) {
    const int ez = (int)(all % E3);
    const int ey = (int)((all / E3) % E2);
    const int ex = (int)(all / ((long)E3 * E2));
    for (int kx = 0; kx < X.ng; ++kx)
      for (int ky = 0; ky < Y.ng; ++ky)
        for (int kz = 0; kz < Z.ng; ++kz) {
          double Uval = 0.0, dux = 0.0, duy = 0.0, duz = 0.0;
          for (int bx = 0; bx <= X.p; ++bx)
            for (int by = 0; by <= Y.p; ++by)
              for (int bz = 0; bz <= Z.p; ++bz) {
                const size_t ix = X.O[ex] + bx, iy = Y.O[ey] + by, iz = Z.O[ez] + bz;
                const double Ucoeff = A.R[ix + sx * (iy + sy * iz)];
                const double v = X.nn(0, bx, kx, ex) * Y.nn(0, by, ky, ey) * Z.nn(0, bz, kz, ez);
                const double dvx = X.nn(1, bx, kx, ex) * Y.nn(0, by, ky, ey) * Z.nn(0, bz, kz, ez);
                const double dvy = X.nn(0, bx, kx, ex) * Y.nn(1, by, ky, ey) * Z.nn(0, bz, kz, ez);
                const double dvz = X.nn(0, bx, kx, ex) * Y.nn(0, by, ky, ey) * Z.nn(1, bz, kz, ez);
                Uval = Uval + Ucoeff * v;
                dux = dux + Ucoeff * dvx;
                duy = duy + Ucoeff * dvy;
                duz = duz + Ucoeff * dvz;
              }
          const size_t q = un_index(A, ex, ey, ez, kx, ky, kz);
          A.dUn[q] = dux;
          A.dUn[q + nqp] = duy;
          A.dUn[q + 2 * nqp] = duz;
          V[q] = Uval;
        }
  }
}

// Problem integrands (the RHS_fun_int callback, src/Interfaces.F90:52-81).
enum { ORC_FORM_PROJECT = 0, ORC_FORM_HEAT = 1, ORC_FORM_OIL = 2 };

struct OrcFormCtx {
  int form;
  const double* fqp;     // per quadrature point, layout (kx,ky,kz,ex,ey,ez); may be null
  const double* kappa;   // per quadrature point, same layout; may be null
  double kappa_const;
  double dt;
  int heat_initial;      // project the heat problem's own initial_state(X)
  const double* drain;   // oil: draining weight per point, draining(u, X) = drain * u
  double mu;             // oil: exponent of the saturation factor exp(mu u)
};

struct OrcPoint {
  const OrcADS* A;
  double X[3];
  int k[3], e[3], a[3];
  double du[3];
  double un;
  double J, W;
  size_t qp;  // linear (kx,ky,kz,ex,ey,ez) index
};

// extra: a per-call statistic the problem accumulates (the oil problem's
// `drained` module variable); 0 for the other problems
typedef void (*orc_rhs_fun)(const OrcFormCtx*, const OrcPoint*, double* l2norm, double* ret, double* extra);

// L2Projection / heat t=0 integrand:
// problems/L2Projection/RHS_eq.F90:66-70 and problems/heat/RHS_eq.F90:82-85.
__attribute__((noinline)) static void orc_rhs_project(const OrcFormCtx* c, const OrcPoint* P,
                                                      double* l2norm, double* ret, double* extra) {
  const OrcADS& A = *P->A;
  const double v = A.ax[0].nn(0, P->a[0], P->k[0], P->e[0]) *
                   A.ax[1].nn(0, P->a[1], P->k[1], P->e[1]) *
                   A.ax[2].nn(0, P->a[2], P->k[2], P->e[2]);
  double fval;
  if (c->heat_initial) fval = orc_heat_initial_state(P->X[0], P->X[1], P->X[2]);
  else if (c->fqp) fval = c->fqp[P->qp];
  else fval = 1.0;
  *ret = P->J * P->W * v * fval;
  *l2norm = P->J * P->W * v * fval * fval;
  *extra = 0.0;
}

// Heat t>0 integrand: problems/heat/RHS_eq.F90:69-81 (kqval = kappa, fval = f).
__attribute__((noinline)) static void orc_rhs_heat(const OrcFormCtx* c, const OrcPoint* P,
                                                   double* l2norm, double* ret, double* extra) {
  const OrcADS& A = *P->A;
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  const int *a = P->a, *k = P->k, *e = P->e;
  const double v = X.nn(0, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvx = X.nn(1, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvy = X.nn(0, a[0], k[0], e[0]) * Y.nn(1, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvz = X.nn(0, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(1, a[2], k[2], e[2]);
  const double kqval = c->kappa ? c->kappa[P->qp] : c->kappa_const;
  const double fval = c->fqp ? c->fqp[P->qp] : 0.0;
  const double rhs = c->dt * (-kqval * (P->du[0] * dvx + P->du[1] * dvy + P->du[2] * dvz) + v * fval);
  *ret = P->J * P->W * (v * P->un + rhs);
  *l2norm = P->J * P->W * v * P->un * P->un;
  *extra = 0.0;
}

// Oil problem t>0 integrand: problems/oil/RHS_eq.F90:69-92.  The pointwise
// inputs are sampled by the host at the quadrature points: kqval = Kqvals
// (input_data.F90:333-336 through CacheKqValues), vpump = pumping(X)
// (:241-259), and the draining weight w(X) with draining(u, X) = w(X) u
// (:265-283); bq = exp(mi u) (:297-303).  extra receives the `drained`
// increment J W v Dt vdrain.
__attribute__((noinline)) static void orc_rhs_oil(const OrcFormCtx* c, const OrcPoint* P,
                                                  double* l2norm, double* ret, double* extra) {
  const OrcADS& A = *P->A;
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  const int *a = P->a, *k = P->k, *e = P->e;
  const double v = X.nn(0, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvx = X.nn(1, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvy = X.nn(0, a[0], k[0], e[0]) * Y.nn(1, a[1], k[1], e[1]) * Z.nn(0, a[2], k[2], e[2]);
  const double dvz = X.nn(0, a[0], k[0], e[0]) * Y.nn(0, a[1], k[1], e[1]) * Z.nn(1, a[2], k[2], e[2]);
  const double kqval = c->kappa ? c->kappa[P->qp] : c->kappa_const;
  const double vpump = c->fqp ? c->fqp[P->qp] : 0.0;
  const double vdrain = std::max(0.0, (c->drain ? c->drain[P->qp] : 0.0) * P->un);
  const double fval = vpump - vdrain;
  const double rhs =
      c->dt * (-kqval * std::exp(c->mu * P->un) * (P->du[0] * dvx + P->du[1] * dvy + P->du[2] * dvz) + v * fval);
  *ret = P->J * P->W * (v * P->un + rhs);
  *extra = P->J * P->W * v * c->dt * vdrain;
  *l2norm = P->J * P->W * v * P->un * P->un;
}

// Form3DRHS (src/projection_engine.F90:154-284) for one rank.  The reference
// scatters each element's local array under OMP CRITICAL in arbitrary thread
// order; here elements are processed in (p+1)^3 colour classes so the scatter
// is race-free and the sum order is deterministic.
static double orc_form_3d_rhs(OrcADS& A, const OrcFormCtx* ctx, orc_rhs_fun fun) {
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  std::fill(A.F.begin(), A.F.end(), 0.0);
  const int E1 = X.nelem, E2 = Y.nelem, E3 = Z.nelem;
  const size_t nqp = A.nqp;
  const size_t sx = A.s[0], sy = A.s[1];
  double l2total = 0.0, extotal = 0.0;
  const int c1 = X.p + 1, c2 = Y.p + 1, c3 = Z.p + 1;
  for (int colour = 0; colour < c1 * c2 * c3; ++colour) {
    const int ox = colour % c1, oy = (colour / c1) % c2, oz = colour / (c1 * c2);
    const int n1 = (E1 - ox + c1 - 1) / c1, n2 = (E2 - oy + c2 - 1) / c2, n3 = (E3 - oz + c3 - 1) / c3;
    const long total = (long)std::max(n1, 0) * std::max(n2, 0) * std::max(n3, 0);
    double l2colour = 0.0, excolour = 0.0;
#pragma omp parallel reduction(+ : l2colour, excolour)
    {
    std::vector<double> elarr((size_t)c1 * c2 * c3, 0.0);
#pragma omp for schedule(static)
    for (long all = 0; all < total; ++all) {
      const int ez = oz + c3 * (int)(all % n3);
      const int ey = oy + c2 * (int)((all / n3) % n2);
      const int ex = ox + c1 * (int)(all / ((long)n3 * n2));
      std::fill(elarr.begin(), elarr.end(), 0.0);
      OrcPoint P;
      P.A = &A;
      P.e[0] = ex; P.e[1] = ey; P.e[2] = ez;
      P.J = X.J[ex] * Y.J[ey] * Z.J[ez];
      double l2el = 0.0, exel = 0.0;
      for (int kx = 0; kx < X.ng; ++kx)
        for (int ky = 0; ky < Y.ng; ++ky)
          for (int kz = 0; kz < Z.ng; ++kz) {
            P.k[0] = kx; P.k[1] = ky; P.k[2] = kz;
            P.W = X.W[kx] * Y.W[ky] * Z.W[kz];
            const size_t q = un_index(A, ex, ey, ez, kx, ky, kz);
            P.un = A.Un[q];
            (void)A.Un13[q]; (void)A.Un23[q];
            P.du[0] = A.dUn[q]; P.du[1] = A.dUn[q + nqp]; P.du[2] = A.dUn[q + 2 * nqp];
            P.X[0] = X.X[kx + X.ng * ex]; P.X[1] = Y.X[ky + Y.ng * ey]; P.X[2] = Z.X[kz + Z.ng * ez];
            P.qp = kx + (size_t)X.ng * (ky + (size_t)Y.ng * (kz + (size_t)Z.ng *
                   (ex + (size_t)E1 * (ey + (size_t)E2 * ez))));
            for (int ax_ = 0; ax_ <= X.p; ++ax_)
              for (int ay = 0; ay <= Y.p; ++ay)
                for (int az = 0; az <= Z.p; ++az) {
                  P.a[0] = ax_; P.a[1] = ay; P.a[2] = az;
                  double l2tmp, res, extmp;
                  fun(ctx, &P, &l2tmp, &res, &extmp);
                  elarr[ax_ + c1 * (ay + c2 * az)] += res;
                  l2el = l2el + l2tmp;
                  exel = exel + extmp;
                }
          }
      for (int ax_ = 0; ax_ <= X.p; ++ax_)
        for (int ay = 0; ay <= Y.p; ++ay)
          for (int az = 0; az <= Z.p; ++az) {
            const size_t ix = X.O[ex] + ax_, iy = Y.O[ey] + ay, iz = Z.O[ez] + az;
            A.F[ix + sx * (iy + sy * iz)] += elarr[ax_ + c1 * (ay + c2 * az)];
          }
      l2colour += l2el;
      excolour += exel;
    }
    }
    l2total += l2colour;
    extotal += excolour;
  }
  A.drained = extotal;
  return l2total;
}

// MKBBT (src/projection_engine.F90:63-132): the 1-D matrix
// mix(1)*M + mix(2)*K + mix(3)*B + mix(4)*BT in LAPACK band layout with
// kl = ku = p and ldab = 3p+1 (rows 0..p-1 left free for fill-in).
ORC_API void orc_mkbbt_band(const OrcADS* A, int axis, const double mix[4], double* AB) {
  const OrcAxis& X = A->ax[axis];
  const int p = X.p, n1 = X.n + 1, ldab = 3 * p + 1, kl = p, ku = p;
  std::fill(AB, AB + (size_t)ldab * n1, 0.0);
  for (int e = 0; e < X.nelem; ++e)
    for (int i = 0; i < X.ng; ++i)
      for (int c = 0; c <= p; ++c)
        for (int d = 0; d <= p; ++d) {
          const int ia = X.O[e] + c, ib = X.O[e] + d;
          const double M = X.nn(0, c, i, e) * X.nn(0, d, i, e) * X.J[e] * X.W[i];
          const double K = X.nn(1, c, i, e) * X.nn(1, d, i, e) * X.J[e] * X.W[i];
          const double B = X.nn(1, c, i, e) * X.nn(0, d, i, e) * X.J[e] * X.W[i];
          const double BT = X.nn(0, c, i, e) * X.nn(1, d, i, e) * X.J[e] * X.W[i];
          const double val = mix[0] * M + mix[1] * K + mix[2] * B + mix[3] * BT;
          AB[(kl + ku + ia - ib) + (size_t)ldab * ib] += val;
        }
}

// SolveOneDirection (src/ADS.F90:294-379): factor once, then solve each of the
// eqnum right-hand-side columns of RHS(n+1, eqnum) separately (the reference
// calls dmumps(job=3) once per column).  The per-column loop is threaded.
static int orc_solve_one_direction(OrcADS& A, int axis, const double mix[4], double* RHS,
                                   long eqnum) {
  const OrcAxis& X = A.ax[axis];
  const int n1 = X.n + 1, p = X.p, ldab = 3 * p + 1;
  std::vector<double> AB((size_t)ldab * n1);
  orc_mkbbt_band(&A, axis, mix, AB.data());
  std::vector<int> ipiv(n1);
  int info = orc_dgbtrf(n1, p, p, AB.data(), ldab, ipiv.data());
  if (info) return info;
  int piv = 0;
  for (int j = 0; j < n1; ++j) piv |= (ipiv[j] != j);
  A.pivoted[axis] = piv;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < eqnum; ++i)
    orc_dgbtrs1(n1, p, p, AB.data(), ldab, ipiv.data(), RHS + (size_t)n1 * i);
  return 0;
}

// Linearize/Delinearize (src/my_mpi.F90:546-559, 780-793): the single-rank
// effect of Gather/Scatter (src/my_mpi.F90:585-612, 638-702) is two transposing
// copies that compose to the identity.
static void orc_gather_identity(const std::vector<double>& F, std::vector<double>& Fout,
                                long elems, long stride) {
  std::vector<double> lin((size_t)elems * stride);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < elems; ++i)
    for (long j = 0; j < stride; ++j) lin[(size_t)i * stride + j] = F[i + (size_t)elems * j];
#pragma omp parallel for schedule(static)
  for (long i = 0; i < elems; ++i)
    for (long j = 0; j < stride; ++j) Fout[i + (size_t)elems * j] = lin[(size_t)i * stride + j];
}

// ReorderRHSForY / ForZ / ForX (src/reorderRHS.F90:7-93), single rank.
// F(x, y+z*Ny) -> F2(y, x+z*Nx)
ORC_API void orc_reorder_for_y(const int s[3], const double* F, double* F2) {
  const long s1 = s[0], s2 = s[1], s3 = s[2];
#pragma omp parallel for schedule(static)
  for (long ix = 0; ix < s1; ++ix)
    for (long iy = 0; iy < s2; ++iy)
      for (long iz = 0; iz < s3; ++iz)
        F2[iy + s2 * (ix + iz * s1)] = F[ix + s1 * (iy + iz * s2)];
}
// F2(y, x+z*Nx) -> F3(z, x+y*Nx)
ORC_API void orc_reorder_for_z(const int s[3], const double* F2, double* F3) {
  const long s1 = s[0], s2 = s[1], s3 = s[2];
#pragma omp parallel for schedule(static)
  for (long ix = 0; ix < s1; ++ix)
    for (long iy = 0; iy < s2; ++iy)
      for (long iz = 0; iz < s3; ++iz)
        F3[iz + s3 * (ix + iy * s1)] = F2[iy + s2 * (ix + iz * s1)];
}
// F3(z, x+y*Nx) -> F(x, y+z*Ny)
ORC_API void orc_reorder_for_x(const int s[3], const double* F3, double* F) {
  const long s1 = s[0], s2 = s[1], s3 = s[2];
#pragma omp parallel for schedule(static)
  for (long ix = 0; ix < s1; ++ix)
    for (long iy = 0; iy < s2; ++iy)
      for (long iz = 0; iz < s3; ++iz)
        F[ix + s1 * (iy + iz * s2)] = F3[iz + s3 * (ix + iy * s1)];
}

// Kronecker solve part of Sub_Step (src/ADS.F90:518-779) on A.F, one rank:
// x-solve, ReorderRHSForY, y-solve, ReorderRHSForZ, z-solve, ReorderRHSForX,
// then R(:,2,2,2) = F (src/ADS.F90:777-779; DistributeSpline sends nothing).
static int orc_kron_solve(OrcADS& A, const double mix[4]) {
  const long s1 = A.s[0], s2 = A.s[1], s3 = A.s[2];
  std::vector<double> tmp(A.ndof);
  int info;
  orc_gather_identity(A.F, tmp, s1, s2 * s3);
  if ((info = orc_solve_one_direction(A, 0, mix, tmp.data(), s2 * s3))) return info;
  orc_gather_identity(tmp, A.F, s1, s2 * s3);
  orc_reorder_for_y(A.s, A.F.data(), A.F2.data());
  orc_gather_identity(A.F2, tmp, s2, s1 * s3);
  if ((info = orc_solve_one_direction(A, 1, mix, tmp.data(), s1 * s3))) return info;
  orc_gather_identity(tmp, A.F2, s2, s1 * s3);
  orc_reorder_for_z(A.s, A.F2.data(), A.F3.data());
  orc_gather_identity(A.F3, tmp, s3, s1 * s2);
  if ((info = orc_solve_one_direction(A, 2, mix, tmp.data(), s1 * s2))) return info;
  orc_gather_identity(tmp, A.F3, s3, s1 * s2);
  orc_reorder_for_x(A.s, A.F3.data(), A.F.data());
  std::memcpy(A.R.data(), A.F.data(), sizeof(double) * A.ndof);
  return 0;
}

// Step (src/ADS.F90:437-461) with Sub_Step (src/ADS.F90:471-794), one rank,
// mix = (1,0,0,0).  form selects the integrand; returns the status and writes
// the step's l2norm (the per-rank value the drivers MPI_Reduce).
ORC_API int orc_step(OrcADS* A, int form, const double* fqp, const double* kappa_qp,
                     double kappa, double dt, int heat_initial, double* l2norm) {
  std::fill(A->Un13.begin(), A->Un13.end(), 0.0);
  std::fill(A->Un23.begin(), A->Un23.end(), 0.0);
  orc_form_un(*A);
  OrcFormCtx ctx{form, fqp, kappa_qp, kappa, dt, heat_initial, nullptr, 0.0};
  orc_rhs_fun fun = (form == ORC_FORM_HEAT) ? orc_rhs_heat : orc_rhs_project;
  const double l2 = orc_form_3d_rhs(*A, &ctx, fun);
  if (l2norm) *l2norm = l2;
  const double mix[4] = {1.0, 0.0, 0.0, 0.0};
  return orc_kron_solve(*A, mix);
}

// Only the assembly (Form3DRHS after FormUn) of one step, leaving F in place.
ORC_API double orc_assemble(OrcADS* A, int form, const double* fqp, const double* kappa_qp,
                            double kappa, double dt, int heat_initial) {
  orc_form_un(*A);
  OrcFormCtx ctx{form, fqp, kappa_qp, kappa, dt, heat_initial, nullptr, 0.0};
  orc_rhs_fun fun = (form == ORC_FORM_HEAT) ? orc_rhs_heat : orc_rhs_project;
  return orc_form_3d_rhs(*A, &ctx, fun);
}

// One oil-problem step at t > 0 (problems/oil/main.F90 driving Step with the
// oil ComputePointForRHS): pump_qp, kq_qp, drain_qp per quadrature point in
// the (kx,ky,kz,ex,ey,ez) layout.  Writes the step's l2norm and its drained
// increment.
ORC_API int orc_step_oil(OrcADS* A, const double* pump_qp, const double* kq_qp, const double* drain_qp,
                         double mu, double dt, double* l2norm, double* drained) {
  std::fill(A->Un13.begin(), A->Un13.end(), 0.0);
  std::fill(A->Un23.begin(), A->Un23.end(), 0.0);
  orc_form_un(*A);
  OrcFormCtx ctx{ORC_FORM_OIL, pump_qp, kq_qp, 1.0, dt, 0, drain_qp, mu};
  const double l2 = orc_form_3d_rhs(*A, &ctx, orc_rhs_oil);
  if (l2norm) *l2norm = l2;
  if (drained) *drained = A->drained;
  const double mix[4] = {1.0, 0.0, 0.0, 0.0};
  return orc_kron_solve(*A, mix);
}

// Only the oil assembly, leaving F in place; returns the l2norm, writes drained.
ORC_API double orc_assemble_oil(OrcADS* A, const double* pump_qp, const double* kq_qp, const double* drain_qp,
                                double mu, double dt, double* drained) {
  orc_form_un(*A);
  OrcFormCtx ctx{ORC_FORM_OIL, pump_qp, kq_qp, 1.0, dt, 0, drain_qp, mu};
  const double l2 = orc_form_3d_rhs(*A, &ctx, orc_rhs_oil);
  if (drained) *drained = A->drained;
  return l2;
}

// MultiStep (src/ADS.F90:391-429): three substeps; substep s runs FormUn(s)
// (Un, Un13 or Un23 and dUn from the current R), Form3DRHS with the form's
// integrand, and the Kronecker solve with the 1-D mix mix[4s..4s+3].  l2norm
// is the last substep's, as in the reference.
ORC_API int orc_multistep(OrcADS* A, int form, const double* fqp, const double* kappa_qp, double kappa,
                          double dt, const double* mix, double* l2norm) {
  OrcFormCtx ctx{form, fqp, kappa_qp, kappa, dt, 0, nullptr, 0.0};
  orc_rhs_fun fun = (form == ORC_FORM_HEAT) ? orc_rhs_heat : orc_rhs_project;
  double l2 = 0.0;
  for (int s = 1; s <= 3; ++s) {
    orc_form_un(*A, s);
    if (s == 1) {
      std::fill(A->Un13.begin(), A->Un13.end(), 0.0);
      std::fill(A->Un23.begin(), A->Un23.end(), 0.0);
    } else if (s == 2) {
      std::fill(A->Un23.begin(), A->Un23.end(), 0.0);
    }
    l2 = orc_form_3d_rhs(*A, &ctx, fun);
    const int info = orc_kron_solve(*A, mix + 4 * (s - 1));
    if (info) return info;
  }
  if (l2norm) *l2norm = l2;
  return 0;
}

// Only the Kronecker solve of F (mix = (1,0,0,0)); result in R and F.
ORC_API int orc_solve_F(OrcADS* A, double* F) {
  std::memcpy(A->F.data(), F, sizeof(double) * A->ndof);
  const double mix[4] = {1.0, 0.0, 0.0, 0.0};
  int info = orc_kron_solve(*A, mix);
  std::memcpy(F, A->F.data(), sizeof(double) * A->ndof);
  return info;
}

ORC_API void orc_pivoted(const OrcADS* A, int* piv) {
  for (int d = 0; d < 3; ++d) piv[d] = A->pivoted[d];
}

// FindSpan (src/basis.F90:226-259): the knot span of uu, clamped to [p, n],
// by the reference's binary search.
ORC_API int orc_find_span(int n, int p, double uu, const double* U) {
  if (uu >= U[n + 1]) return n;
  if (uu <= U[p]) return p;
  int low = p, high = n + 1;
  int span = (low + high) / 2;
  while (uu < U[span] || uu >= U[span + 1]) {
    if (uu < U[span]) high = span;
    else low = span;
    span = (low + high) / 2;
  }
  return span;
}

// SaveSplinePlot's sampling (src/plot.F90:111-140) with EvalSpline
// (src/basis.F90:323-369, d = 0) on the coefficients R: vals(ix, iy, iz) at
// x = lerp((ix-1)/(resx-1), startx, endx) etc., x fastest.  range =
// (startx, endx, starty, endy, startz, endz).  The plotted array is the one
// GatherFullSolution (src/my_mpi.F90:422-514) collects, at one rank R itself.
ORC_API void orc_eval_spline_grid(const OrcADS* A, const double range[6], const int res[3], double* vals) {
  const OrcAxis &X = A->ax[0], &Y = A->ax[1], &Z = A->ax[2];
  const int sx = A->s[0], sy = A->s[1];
  auto lerp = [](double t, double a, double b) { return (1.0 - t) * a + t * b; };
#pragma omp parallel for schedule(static)
  for (int ix = 1; ix <= res[0]; ++ix) {
    std::vector<double> bx(X.p + 1), by(Y.p + 1), bz(Z.p + 1);
    const double x = lerp((ix - 1) / (double)(res[0] - 1), range[0], range[1]);
    const int xspan = orc_find_span(X.n, X.p, x, X.U.data());
    orc_ders_basis_funs(xspan, x, X.p, 0, X.U.data(), bx.data());
    for (int iy = 1; iy <= res[1]; ++iy) {
      const double y = lerp((iy - 1) / (double)(res[1] - 1), range[2], range[3]);
      const int yspan = orc_find_span(Y.n, Y.p, y, Y.U.data());
      orc_ders_basis_funs(yspan, y, Y.p, 0, Y.U.data(), by.data());
      for (int iz = 1; iz <= res[2]; ++iz) {
        const double z = lerp((iz - 1) / (double)(res[2] - 1), range[4], range[5]);
        const int zspan = orc_find_span(Z.n, Z.p, z, Z.U.data());
        orc_ders_basis_funs(zspan, z, Z.p, 0, Z.U.data(), bz.data());
        const int x0 = xspan - X.p, y0 = yspan - Y.p, z0 = zspan - Z.p;
        double val = 0.0;
        for (int a = 0; a <= X.p; ++a)
          for (int b = 0; b <= Y.p; ++b)
            for (int c = 0; c <= Z.p; ++c) {
              const double w = bx[a] * by[b] * bz[c];
              val = val + w * A->R[(x0 + a) + (size_t)sx * ((y0 + b) + (size_t)sy * (z0 + c))];
            }
        vals[(ix - 1) + (size_t)res[0] * ((iy - 1) + (size_t)res[1] * (iz - 1))] = val;
      }
    }
  }
}

// Heat-problem quadrature-point field of initial_state (problems/heat/input_data.F90:57-70)
// in the (kx,ky,kz,ex,ey,ez) layout.
ORC_API void orc_heat_initial_qp(const OrcADS* A, double* fqp) {
  const OrcAxis &X = A->ax[0], &Y = A->ax[1], &Z = A->ax[2];
  const long E1 = X.nelem, E2 = Y.nelem, E3 = Z.nelem;
#pragma omp parallel for schedule(static)
  for (long ez = 0; ez < E3; ++ez)
    for (long ey = 0; ey < E2; ++ey)
      for (long ex = 0; ex < E1; ++ex)
        for (int kz = 0; kz < Z.ng; ++kz)
          for (int ky = 0; ky < Y.ng; ++ky)
            for (int kx = 0; kx < X.ng; ++kx) {
              const size_t q = kx + (size_t)X.ng * (ky + (size_t)Y.ng * (kz + (size_t)Z.ng *
                               (ex + (size_t)E1 * (ey + (size_t)E2 * ez))));
              fqp[q] = orc_heat_initial_state(X.X[kx + X.ng * ex], Y.X[ky + Y.ng * ey],
                                              Z.X[kz + Z.ng * ez]);
            }
}

// ---------------------------------------------------------------------------
// FP64 reference adjoint of the explicit heat step (checker for the GPU
// adjoint).  Forward: u^{n+1} = M3^{-1} A_kappa u^n with A_kappa the assembled
// heat operator.  Loss L = 1/2 (u^K - ut)^T M3 (u^K - ut).  Backward:
// mu = M3^{-1} lambda^{n+1} (M3 is symmetric), lambda^n = A_kappa mu (A_kappa is
// symmetric), dL/dkappa_q += -dt * J W grad u^n(q) . grad mu(q).
// The whole trajectory is stored (no checkpointing: this is the checker).
// ---------------------------------------------------------------------------

// Apply M3 = Mx (x) My (x) Mz to u (x-fastest layout) with the band of MKBBT.
static void orc_apply_m3(OrcADS& A, const double* u, double* out) {
  const long s1 = A.s[0], s2 = A.s[1], s3 = A.s[2];
  std::vector<double> a(u, u + A.ndof), b(A.ndof, 0.0);
  const double mix[4] = {1.0, 0.0, 0.0, 0.0};
  for (int axis = 0; axis < 3; ++axis) {
    const OrcAxis& X = A.ax[axis];
    const int p = X.p, n1 = X.n + 1, ldab = 3 * p + 1;
    std::vector<double> AB((size_t)ldab * n1);
    orc_mkbbt_band(&A, axis, mix, AB.data());
    const long stride = axis == 0 ? 1 : (axis == 1 ? s1 : s1 * s2);
    const long nlines = A.ndof / n1;
    std::fill(b.begin(), b.end(), 0.0);
#pragma omp parallel for schedule(static)
    for (long l = 0; l < nlines; ++l) {
      long base;
      if (axis == 0) base = l * s1;
      else if (axis == 1) base = (l % s1) + s1 * s2 * (l / s1);
      else base = l;
      for (int i = 0; i < n1; ++i) {
        double acc = 0.0;
        for (int j = std::max(0, i - p); j <= std::min(n1 - 1, i + p); ++j)
          acc += AB[(2 * p + i - j) + (size_t)ldab * j] * a[base + stride * j];
        b[base + stride * i] = acc;
      }
    }
    std::swap(a, b);
  }
  (void)s3;
  std::memcpy(out, a.data(), sizeof(double) * A.ndof);
}

ORC_API void orc_apply_mass(OrcADS* A, const double* u, double* out) { orc_apply_m3(*A, u, out); }

// grad of the spline with coefficients c at every quadrature point, written in
// the (kx,ky,kz,ex,ey,ez) layout as g[3*q + d].
static void orc_grad_qp(OrcADS& A, const double* c, std::vector<double>& g) {
  std::vector<double> saveR = A.R;
  std::memcpy(A.R.data(), c, sizeof(double) * A.ndof);
  orc_form_un(A);
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  g.assign(A.nqp * 3, 0.0);
  for (int ez = 0; ez < Z.nelem; ++ez)
    for (int ey = 0; ey < Y.nelem; ++ey)
      for (int ex = 0; ex < X.nelem; ++ex)
        for (int kz = 0; kz < Z.ng; ++kz)
          for (int ky = 0; ky < Y.ng; ++ky)
            for (int kx = 0; kx < X.ng; ++kx) {
              const size_t q = un_index(A, ex, ey, ez, kx, ky, kz);
              const size_t o = kx + (size_t)X.ng * (ky + (size_t)Y.ng * (kz + (size_t)Z.ng *
                               (ex + (size_t)X.nelem * (ey + (size_t)Y.nelem * ez))));
              for (int d = 0; d < 3; ++d) g[3 * o + d] = A.dUn[q + d * A.nqp];
            }
  A.R = saveR;
}

// JW at each quadrature point in the (kx,ky,kz,ex,ey,ez) layout.
static void orc_jw_qp(const OrcADS& A, std::vector<double>& jw) {
  const OrcAxis &X = A.ax[0], &Y = A.ax[1], &Z = A.ax[2];
  jw.assign(A.nqp, 0.0);
  for (int ez = 0; ez < Z.nelem; ++ez)
    for (int ey = 0; ey < Y.nelem; ++ey)
      for (int ex = 0; ex < X.nelem; ++ex)
        for (int kz = 0; kz < Z.ng; ++kz)
          for (int ky = 0; ky < Y.ng; ++ky)
            for (int kx = 0; kx < X.ng; ++kx) {
              const size_t o = kx + (size_t)X.ng * (ky + (size_t)Y.ng * (kz + (size_t)Z.ng *
                               (ex + (size_t)X.nelem * (ey + (size_t)Y.nelem * ez))));
              jw[o] = (X.J[ex] * Y.J[ey] * Z.J[ez]) * (X.W[kx] * Y.W[ky] * Z.W[kz]);
            }
}

// Forward K heat steps from u0 and the loss against ut; optionally the
// gradients with respect to u0 (coefficients) and kappa at the quadrature
// points.  kappa_qp may be null (constant kappa).
ORC_API int orc_heat_adjoint(OrcADS* A, int K, const double* u0, const double* ut,
                             const double* kappa_qp, double kappa, double dt, double* loss,
                             double* grad_u0, double* grad_kappa) {
  const size_t N = A->ndof;
  std::vector<std::vector<double>> traj(K + 1, std::vector<double>(N));
  std::memcpy(traj[0].data(), u0, sizeof(double) * N);
  for (int n = 0; n < K; ++n) {
    std::memcpy(A->R.data(), traj[n].data(), sizeof(double) * N);
    double l2;
    int info = orc_step(A, ORC_FORM_HEAT, nullptr, kappa_qp, kappa, dt, 0, &l2);
    if (info) return info;
    std::memcpy(traj[n + 1].data(), A->R.data(), sizeof(double) * N);
  }
  std::vector<double> e(N), Me(N);
  for (size_t i = 0; i < N; ++i) e[i] = traj[K][i] - ut[i];
  orc_apply_m3(*A, e.data(), Me.data());
  double L = 0.0;
  for (size_t i = 0; i < N; ++i) L += e[i] * Me[i];
  if (loss) *loss = 0.5 * L;
  if (!grad_u0 && !grad_kappa) return 0;
  std::vector<double> lam = Me, mu(N), jw;
  if (grad_kappa) { std::fill(grad_kappa, grad_kappa + A->nqp, 0.0); orc_jw_qp(*A, jw); }
  std::vector<double> gu, gm;
  for (int n = K - 1; n >= 0; --n) {
    std::vector<double> tmp = lam;
    int info = orc_solve_F(A, tmp.data());
    if (info) return info;
    mu = tmp;
    if (grad_kappa) {
      orc_grad_qp(*A, traj[n].data(), gu);
      orc_grad_qp(*A, mu.data(), gm);
      for (size_t q = 0; q < A->nqp; ++q)
        grad_kappa[q] += -dt * jw[q] *
                         (gu[3 * q] * gm[3 * q] + gu[3 * q + 1] * gm[3 * q + 1] + gu[3 * q + 2] * gm[3 * q + 2]);
    }
    // lambda^n = A_kappa mu (assemble the heat form with coefficients mu)
    std::vector<double> saveR = A->R;
    std::memcpy(A->R.data(), mu.data(), sizeof(double) * N);
    orc_assemble(A, ORC_FORM_HEAT, nullptr, kappa_qp, kappa, dt, 0);
    std::memcpy(lam.data(), A->F.data(), sizeof(double) * N);
    A->R = saveR;
  }
  if (grad_u0) std::memcpy(grad_u0, lam.data(), sizeof(double) * N);
  return 0;
}

ORC_API int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

ORC_API void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
