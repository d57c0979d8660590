// k_assemble_df.cu — the heat increment of the mixed-precision step assembled
// in double-float arithmetic on the FP32 pipe (K1-DF).
//
// Replaces, for the heat integrand at t > 0 (problems/heat/RHS_eq.F90:69-86),
// FormUn (src/projection_engine.F90:306-441) + Form3DRHS (:154-284) minus the
// mass term: with exact Gauss quadrature the J W v u part of F is M u^n, so
// the mixed step assembles only
//
//   G_a = sum_e sum_qp J W (-dt kappa grad u . grad v_a + dt v_a f)
//
// and solves M delta = G with FP64 refinement.  The sums are the FP64
// kernel's (k_assemble.cuh with T = double): sum-factorised one direction at a
// time, the same brick decomposition, coefficient ring, spill shadows and
// fixed-order fixup, the same Gauss rule and basis tables.  Only the
// arithmetic differs: every basis value, weight, coefficient and partial sum is
// a double-float (df32.cuh), so each of the ~800 multiply-adds per element
// costs about twelve FP32 instructions instead of one FP64 instruction, which
// GB300 issues at 1/64 of the FP32 rate.  G comes out with a relative error of
// order 1e-13 (plain FP32 left ~1e-6, which no refinement of the solve can
// remove), so the step matches the FP64 step to the refinement tolerance.
//
//   interpolation   C[bz,by,bx] --z--> ZA,ZB --y--> Y0,Y1,Y2 --x--> du/dx, du/dy, du/dz
//   integrand       g{1,2,3} = -dt kappa J W du/d{x,y,z},  g0 = dt J W f
//   test functions  g --x--> H0,H1,H2 --y--> I0,I1 --z--> G (double-float planes)
//
// The coefficients are scaled by 2^-e (max |u| < 2^e, from the uscale pass,
// or the previous step's scale checked afterwards when a caller's array is
// read in place) so that FP32 never overflows, split once per plane into
// (high, low) floats, and the finished DOF planes are scaled back by 2^e
// exactly.  The l2norm (J W u^2) is accumulated from the high parts in
// compensated FP32.  At p = 2 and 3, elements whose tables are
// centro-symmetric take the even-odd form of the sums (EO below): per layer
// for the z interpolation and test, per element row for the y stages, per
// brick for the x stage.  With a constant conductivity and no source the x
// quadrature is done on the host, per element (its 1-D stiffness and mass
// matrices, the same Gauss sums), and the x stage applies the brick's bands
// of those matrices to each row of points.
#include "df32.cuh"
#include "k_assemble.cuh"

namespace ads {

// ---- even-odd forms of an element's contractions (p = 2 and 3) ----
// For an element whose tables are centro-symmetric, N[k][b] = N[p-k][p-b]
// and dN[k][b] = -dN[p-k][p-b] (Gauss points symmetric about the element's
// centre, basis mirrored: every element of a uniform knot vector but the
// first and last p - 1), the sums over b of an interpolation pair the outputs
// k and p-k.  With s_j = v_j + v_{p-j} and d_j = v_j - v_{p-j},
//   sum_b N[k][b] v[b]:  out_k, out_{p-k} = X_k +- Y_k, X_k = sum_j a_kj s_j, Y_k = sum_j c_kj d_j
//   sum_b dN[k][b] v[b]: out_k, out_{p-k} = X_k +- Y_k, X_k = sum_j c'_kj d_j, Y_k = sum_j a'_kj s_j
// with a_kj, c_kj = (N[k][j] +- N[k][p-j]) / 2 (a', c' the same for dN) and,
// at p = 2, the middle output and middle input folded in; the test
// contractions (sums over k) are the transposes.  A double-float
// multiply-add costs 12 FP32 operations and a sum 8: at p = 2 the forms take
// 52-68 operations for the direct sums' 84, at p = 3 96 for 160.
template <int P>
struct EO {
  static constexpr bool on = false;
  static constexpr int NS = 1;
};

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

template <>
struct EO<2> {
  static constexpr bool on = true;
  static constexpr int NS = 9;  // [a, c, N01, N10, N11, a', c', dN01, dN10]
  struct N { dfl a, c, n01, n10, n11; };
  struct D { dfl a, c, d01, d10; };
  static __device__ __forceinline__ N n(const dfl* t) { return N{t[0], t[1], t[2], t[3], t[4]}; }
  static __device__ __forceinline__ D d(const dfl* t) { return D{t[5], t[6], t[7], t[8]}; }
  // out[k] = sum_b N[k][b] v[b]
  static __device__ __forceinline__ void interp_n(dfl (&out)[3], const dfl (&v)[3], const N& n) {
    const dfl sp = df_add(v[0], v[2]), dm = df_sub(v[0], v[2]);
    const dfl e = df_mac(df_mul(n.a, sp), n.n01, v[1]), d = df_mul(n.c, dm);
    out[0] = df_add(e, d);
    out[2] = df_sub(e, d);
    out[1] = df_mac(df_mul(n.n10, sp), n.n11, v[1]);
  }
  // out[k] = sum_b dN[k][b] v[b]
  static __device__ __forceinline__ void interp_d(dfl (&out)[3], const dfl (&v)[3], const D& dn) {
    const dfl sp = df_add(v[0], v[2]), dm = df_sub(v[0], v[2]);
    const dfl e = df_mac(df_mul(dn.a, sp), dn.d01, v[1]), d = df_mul(dn.c, dm);
    out[0] = df_add(d, e);
    out[2] = df_sub(d, e);
    out[1] = df_mul(dn.d10, dm);
  }
  // both, sharing s and d
  static __device__ __forceinline__ void interp_nd(dfl (&on)[3], dfl (&od)[3], const dfl (&v)[3], const N& n,
                                                   const D& dn) {
    const dfl sp = df_add(v[0], v[2]), dm = df_sub(v[0], v[2]);
    const dfl e = df_mac(df_mul(n.a, sp), n.n01, v[1]), d = df_mul(n.c, dm);
    on[0] = df_add(e, d);
    on[2] = df_sub(e, d);
    on[1] = df_mac(df_mul(n.n10, sp), n.n11, v[1]);
    const dfl e2 = df_mac(df_mul(dn.a, sp), dn.d01, v[1]), d2 = df_mul(dn.c, dm);
    od[0] = df_add(d2, e2);
    od[2] = df_sub(d2, e2);
    od[1] = df_mul(dn.d10, dm);
  }
  // h[b] = sum_k N[k][b] g[k]
  static __device__ __forceinline__ void test_n(dfl (&h)[3], const dfl (&g)[3], const N& n) {
    const dfl sp = df_add(g[0], g[2]), dm = df_sub(g[0], g[2]);
    const dfl e = df_mac(df_mul(n.a, sp), n.n10, g[1]), d = df_mul(n.c, dm);
    h[0] = df_add(e, d);
    h[2] = df_sub(e, d);
    h[1] = df_mac(df_mul(n.n01, sp), n.n11, g[1]);
  }
  // h[b] = sum_k dN[k][b] g[k]
  static __device__ __forceinline__ void test_d(dfl (&h)[3], const dfl (&g)[3], const D& dn) {
    const dfl sp = df_add(g[0], g[2]), dm = df_sub(g[0], g[2]);
    const dfl e = df_mac(df_mul(dn.c, sp), dn.d10, g[1]), d = df_mul(dn.a, dm);
    h[0] = df_add(e, d);
    h[2] = df_sub(d, e);
    h[1] = df_mul(dn.d01, dm);
  }
  // interp_n on the high parts, in FP32 (the l2norm's u at the points)
  static __device__ __forceinline__ void uu(float (&u)[3], const dfl (&v)[3], const N& n) {
    const float sp = v[0].x + v[2].x, dm = v[0].x - v[2].x;
    const float e = fmaf(n.n01.x, v[1].x, n.a.x * sp), d = n.c.x * dm;
    u[0] = e + d;
    u[2] = e - d;
    u[1] = fmaf(n.n11.x, v[1].x, n.n10.x * sp);
  }
  // the z test contraction h[b] += sum_k N[k][b] g0[k] + dN[k][b] g1[k],
  // accumulated over the points in even-odd form: h[0] holds X, h[2] Y and
  // h[1] the middle function until zt_finish sets h[0], h[2] = X +- Y.
  // zt_pair takes the points (k, p - k) = (0, 2), zt_mid the middle point;
  // t holds the even-odd coefficients (the N part, then the dN part)
  static __device__ __forceinline__ void zt_pair(dfl (&h)[3], int, dfl g0a, dfl g0b, dfl g1a, dfl g1b,
                                                 const dfl* t) {
    const dfl s0 = df_add(g0a, g0b), d0 = df_sub(g0a, g0b);
    const dfl s1 = df_add(g1a, g1b), d1 = df_sub(g1a, g1b);
    h[0] = df_mac(df_mac(h[0], t[0], s0), t[5], d1);  // a S0 + a' D1
    h[2] = df_mac(df_mac(h[2], t[1], d0), t[6], s1);  // c D0 + c' S1
    h[1] = df_mac(df_mac(h[1], t[2], s0), t[7], d1);  // N01 S0 + dN01 D1
  }
  static __device__ __forceinline__ void zt_mid(dfl (&h)[3], dfl g0, dfl g1, const dfl* t) {
    h[0] = df_mac(h[0], t[3], g0);  // N10
    h[2] = df_mac(h[2], t[8], g1);  // dN10
    h[1] = df_mac(h[1], t[4], g0);  // N11
  }
  static __device__ __forceinline__ void zt_finish(dfl (&h)[3]) {
    const dfl x = h[0], y = h[2];
    h[0] = df_add(x, y);
    h[2] = df_sub(x, y);
  }
};

template <>
struct EO<3> {
  static constexpr bool on = true;
  static constexpr int NS = 16;  // N: a[k][j] (4), c[k][j] (4); then dN: a', c'
  struct C { dfl a[2][2], c[2][2]; };
  using N = C;
  using D = C;
  static __device__ __forceinline__ C load(const dfl* t) {
    C r;
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        r.a[k][j] = t[2 * k + j];
        r.c[k][j] = t[4 + 2 * k + j];
      }
    return r;
  }
  static __device__ __forceinline__ C n(const dfl* t) { return load(t); }
  static __device__ __forceinline__ C d(const dfl* t) { return load(t + 8); }
  static __device__ __forceinline__ dfl dot2(dfl c0, dfl x0, dfl c1, dfl x1) { return df_mac(df_mul(c0, x0), c1, x1); }
  static __device__ __forceinline__ void sd(dfl (&s)[2], dfl (&d)[2], const dfl (&v)[4]) {
    s[0] = df_add(v[0], v[3]);
    d[0] = df_sub(v[0], v[3]);
    s[1] = df_add(v[1], v[2]);
    d[1] = df_sub(v[1], v[2]);
  }
  static __device__ __forceinline__ void pairs(dfl (&out)[4], const dfl (&X)[2], const dfl (&Y)[2]) {
    out[0] = df_add(X[0], Y[0]);
    out[3] = df_sub(X[0], Y[0]);
    out[1] = df_add(X[1], Y[1]);
    out[2] = df_sub(X[1], Y[1]);
  }
  static __device__ __forceinline__ void interp_n_sd(dfl (&out)[4], const dfl (&s)[2], const dfl (&d)[2], const C& n) {
    dfl X[2], Y[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      X[k] = dot2(n.a[k][0], s[0], n.a[k][1], s[1]);
      Y[k] = dot2(n.c[k][0], d[0], n.c[k][1], d[1]);
    }
    pairs(out, X, Y);
  }
  static __device__ __forceinline__ void interp_d_sd(dfl (&out)[4], const dfl (&s)[2], const dfl (&d)[2], const C& dn) {
    dfl X[2], Y[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      X[k] = dot2(dn.c[k][0], d[0], dn.c[k][1], d[1]);
      Y[k] = dot2(dn.a[k][0], s[0], dn.a[k][1], s[1]);
    }
    pairs(out, X, Y);
  }
  static __device__ __forceinline__ void interp_n(dfl (&out)[4], const dfl (&v)[4], const C& n) {
    dfl s[2], d[2];
    sd(s, d, v);
    interp_n_sd(out, s, d, n);
  }
  static __device__ __forceinline__ void interp_d(dfl (&out)[4], const dfl (&v)[4], const C& dn) {
    dfl s[2], d[2];
    sd(s, d, v);
    interp_d_sd(out, s, d, dn);
  }
  static __device__ __forceinline__ void interp_nd(dfl (&on)[4], dfl (&od)[4], const dfl (&v)[4], const C& n,
                                                   const C& dn) {
    dfl s[2], d[2];
    sd(s, d, v);
    interp_n_sd(on, s, d, n);
    interp_d_sd(od, s, d, dn);
  }
  // h[b] = sum_k N[k][b] g[k]: X_b = sum_k a_kb S_k, Y_b = sum_k c_kb D_k
  static __device__ __forceinline__ void test_n(dfl (&h)[4], const dfl (&g)[4], const C& n) {
    dfl S[2], D[2], X[2], Y[2];
    sd(S, D, g);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      X[b] = dot2(n.a[0][b], S[0], n.a[1][b], S[1]);
      Y[b] = dot2(n.c[0][b], D[0], n.c[1][b], D[1]);
    }
    pairs(h, X, Y);
  }
  // h[b] = sum_k dN[k][b] g[k]: X_b = sum_k a'_kb D_k, Y_b = sum_k c'_kb S_k
  static __device__ __forceinline__ void test_d(dfl (&h)[4], const dfl (&g)[4], const C& dn) {
    dfl S[2], D[2], X[2], Y[2];
    sd(S, D, g);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      X[b] = dot2(dn.a[0][b], D[0], dn.a[1][b], D[1]);
      Y[b] = dot2(dn.c[0][b], S[0], dn.c[1][b], S[1]);
    }
    pairs(h, X, Y);
  }
  static __device__ __forceinline__ void uu(float (&u)[4], const dfl (&v)[4], const C& n) {
    const float s0 = v[0].x + v[3].x, d0 = v[0].x - v[3].x, s1 = v[1].x + v[2].x, d1 = v[1].x - v[2].x;
    const float X0 = fmaf(n.a[0][1].x, s1, n.a[0][0].x * s0), Y0 = fmaf(n.c[0][1].x, d1, n.c[0][0].x * d0);
    const float X1 = fmaf(n.a[1][1].x, s1, n.a[1][0].x * s0), Y1 = fmaf(n.c[1][1].x, d1, n.c[1][0].x * d0);
    u[0] = X0 + Y0;
    u[3] = X0 - Y0;
    u[1] = X1 + Y1;
    u[2] = X1 - Y1;
  }
  // the z test contraction in even-odd form (as EO<2>): h[b] holds X_b and
  // h[3-b] Y_b (b = 0, 1) until zt_finish; zt_pair takes the points (k, 3 - k)
  static __device__ __forceinline__ void zt_pair(dfl (&h)[4], int k, dfl g0a, dfl g0b, dfl g1a, dfl g1b,
                                                 const dfl* t) {
    const dfl s0 = df_add(g0a, g0b), d0 = df_sub(g0a, g0b);
    const dfl s1 = df_add(g1a, g1b), d1 = df_sub(g1a, g1b);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      h[b] = df_mac(df_mac(h[b], t[2 * k + b], s0), t[8 + 2 * k + b], d1);              // a S0 + a' D1
      h[3 - b] = df_mac(df_mac(h[3 - b], t[4 + 2 * k + b], d0), t[12 + 2 * k + b], s1);  // c D0 + c' S1
    }
  }
  static __device__ __forceinline__ void zt_mid(dfl (&)[4], dfl, dfl, const dfl*) {}
  static __device__ __forceinline__ void zt_finish(dfl (&h)[4]) {
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const dfl x = h[b], y = h[3 - b];
      h[b] = df_add(x, y);
      h[3 - b] = df_sub(x, y);
    }
  }
};

template <int P>
struct DfLayout {
  static constexpr int Q = P + 1;
  static constexpr int TX = as_tx(P), TY = AS_TY;
  static constexpr int CX = TX + P;  // == 32: the x footprint is one warp wide
  static constexpr int CY = TY + P;
  static constexpr int NCOL = CX * CY;
  static constexpr int QY = TY * Q;
  static constexpr int RC = P + 2;  // coefficient ring (P+1 planes in use + 1 in flight)
  static constexpr int RF = P + 1;  // accumulator ring
  static constexpr int NT = Q * (P + 1) * 2;
  static_assert(CX == 32, "footprint must be one warp wide");
  static_assert(TY == AS_THREADS / 32, "a warp per element row");
  static constexpr size_t D = sizeof(dfl);
  static constexpr size_t o_cring = 0;                          // double [RC][NCOL] (cp.async target)
  static constexpr size_t o_tring = o_cring + 8 * RC * NCOL;    // dfl [RC][NCOL] split planes
  static constexpr size_t o_fring = o_tring + D * RC * NCOL;    // dfl [RF][NCOL] DOF accumulators
  static constexpr size_t o_z = o_fring + D * RF * NCOL;        // dfl [2][Q][NCOL]
  static constexpr size_t o_y = o_z + D * 2 * Q * NCOL;         // dfl [3][QY][CX]
  static constexpr size_t o_h = o_y + D * 3 * QY * CX;          // dfl [3][QY][CX]
  static constexpr size_t o_ny = o_h + D * 3 * QY * CX;         // dfl [TY][NT]
  static constexpr size_t o_jwy = o_ny + D * TY * NT;           // dfl [TY][Q]
  static constexpr size_t o_nz = o_jwy + D * TY * Q;            // dfl [NT]
  static constexpr size_t o_jwz = o_nz + D * NT;                // dfl [Q]
  static constexpr int NS = EO<P>::NS;                         // even-odd coefficients per element
  static constexpr size_t o_sy = o_jwz + D * Q;                 // dfl [TY][NS]
  static constexpr size_t o_sz = o_sy + D * TY * NS;            // dfl [NS]
  static constexpr size_t o_sf = o_sz + D * NS;                 // int [TY + 1]: rows, then the layer
  // the J W-folded interpolation tables of the constant-kappa increment
  static constexpr size_t o_nyw = (o_sf + 4 * (TY + 1) + 15) / 16 * 16;  // dfl [TY][NT]
  static constexpr size_t o_syw = o_nyw + D * TY * NT;          // dfl [TY][NS]
  static constexpr size_t o_nzw = o_syw + D * TY * NS;          // dfl [NT]
  static constexpr size_t o_szw = o_nzw + D * NT;               // dfl [NS]
  static constexpr size_t o_red = (o_szw + D * NS + 15) / 16 * 16;
  static constexpr size_t bytes = o_red + 3 * sizeof(double) * (AS_THREADS / 32);
};

__device__ __forceinline__ dfl df_split(double d, int sexp) {
  float h, l;
  split_scaled(d, sexp, h, l);
  return df_make(h, l);
}

template <int P, bool HAS_F, bool HAS_K>
__global__ void __launch_bounds__(AS_THREADS, P <= 2 ? 2 : 1)
    k_assemble_df(const AssembleArgs a, const DfTabs3 tb) {
  using L = DfLayout<P>;
  using E = EO<P>;
  constexpr int Q = L::Q, TX = L::TX, TY = L::TY, CX = L::CX;
  constexpr int NS = L::NS;
  // constant conductivity, no source: the point weights Jy Wy and Jz Wz are
  // folded into the y and z interpolation tables, the x quadrature into the
  // brick's x stiffness and mass bands (per element sum_kx of the basis
  // products times Jx Wx, the same Gauss sums in another order, then summed
  // over the elements on a column), and -dt kappa into the written DOFs: the
  // x stage is three banded products per row of points
  constexpr bool FOLD = !HAS_F && !HAS_K;
  // the z test contraction of a symmetric layer in even-odd form (at p = 2
  // with a per-point conductivity or a source its registers would spill)
  constexpr bool ZEO = E::on && (FOLD || P == 3);
  // the x stage's output kept in registers for the y test (constant
  // conductivity at p <= 2; the per-point x stage, or p = 3 with its 4 x 3
  // values a lane, would cost registers the kernel does not have)
  constexpr bool HREG = FOLD && P <= 2;
  constexpr int NCOL = L::NCOL, QY = L::QY, RC = L::RC, RF = L::RF, NT = L::NT;

  extern __shared__ __align__(16) unsigned char smem[];
  double* cring = reinterpret_cast<double*>(smem + L::o_cring);
  dfl* tring = reinterpret_cast<dfl*>(smem + L::o_tring);
  dfl* fring = reinterpret_cast<dfl*>(smem + L::o_fring);
  dfl* ZA = reinterpret_cast<dfl*>(smem + L::o_z);
  dfl* ZB = ZA + Q * NCOL;
  dfl* Y0 = reinterpret_cast<dfl*>(smem + L::o_y);
  dfl* Y1 = Y0 + QY * CX;
  dfl* Y2 = Y1 + QY * CX;
  dfl* H0 = reinterpret_cast<dfl*>(smem + L::o_h);
  dfl* H1 = H0 + QY * CX;
  dfl* H2 = H1 + QY * CX;
  dfl* NYs = reinterpret_cast<dfl*>(smem + L::o_ny);
  dfl* JWYs = reinterpret_cast<dfl*>(smem + L::o_jwy);
  dfl* NZs = reinterpret_cast<dfl*>(smem + L::o_nz);
  dfl* JWZs = reinterpret_cast<dfl*>(smem + L::o_jwz);
  dfl* SYs = reinterpret_cast<dfl*>(smem + L::o_sy);
  dfl* SZs = reinterpret_cast<dfl*>(smem + L::o_sz);
  int* SF = reinterpret_cast<int*>(smem + L::o_sf);
  dfl* NYw = reinterpret_cast<dfl*>(smem + L::o_nyw);
  dfl* SYw = reinterpret_cast<dfl*>(smem + L::o_syw);
  dfl* NZw = reinterpret_cast<dfl*>(smem + L::o_nzw);
  dfl* SZw = reinterpret_cast<dfl*>(smem + L::o_szw);
  // the y and z interpolation tables (J W folded in under FOLD); the y and z
  // test contractions keep NYs, SYs and NZs
  const dfl* NYi = FOLD ? NYw : NYs;
  const dfl* SYi = FOLD ? SYw : SYs;
  const dfl* NZi = FOLD ? NZw : NZs;
  const dfl* SZi = FOLD ? SZw : SZs;
  double* red = reinterpret_cast<double*>(smem + L::o_red);

  const Geometry& g = a.g;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int Ex = g.E[0], Ey = g.E[1], Ez = g.E[2];
  const int Nx = g.N[0], Ny = g.N[1];
  const long long QXt = (long long)Ex * Q, QYt = (long long)Ey * Q;
  const int nitems = a.nix * a.niy * a.niz;
  const int my_ey = tid / CX, my_cx = tid % CX;
  // FOLD: the columns lane - P .. lane + P of a row, clamped into the row
  int xoff[2 * P + 1];
#pragma unroll
  for (int j = 0; j <= 2 * P; ++j) xoff[j] = min(max(lane + j - P, 0), CX - 1);
  // coefficients (and the source) are multiplied by 2^uexp
  const int uexp = pow2_exp(*a.uscale);
  const dfl ndtk = df_split(-a.dt * a.kappa, 0);  // constant conductivity
  const dfl ndt = df_split(-a.dt, 0);             // per-point conductivity
  const dfl dtv = df_split(a.dt, 0);              // source term

  double l2_thread = 0.0;
  unsigned long long amax_bits = 0ull;  // max |written value| as ordered bits
  unsigned long long umax_bits = 0ull;  // max |u| over the coefficients read, as ordered bits

  for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
    const int ix = item % a.nix;
    const int iy = (item / a.nix) % a.niy;
    const int iz = item / (a.nix * a.niy);
    const int x0 = ix * TX, y0 = iy * TY;
    const int ez0 = iz * a.zc;
    const int ez1 = min(ez0 + a.zc, Ez);
    const bool lastx = (ix == a.nix - 1), lasty = (iy == a.niy - 1), lastz = (iz == a.niz - 1);

    __syncthreads();  // previous item fully done with shared memory

    // per-lane x tables for the pointwise x stage (per-point conductivity or
    // a source; element x0 + lane, lanes >= TX have no element).  p = 2, 3:
    // bricks whose elements are all centro-symmetric run it in even-odd form;
    // the table registers then hold the lane's NS even-odd coefficients
    dfl nx[Q][P + 1][2];
    dfl jwx[Q];
    // FOLD: row lane of the brick's x stiffness and mass bands, column
    // x0 + lane against columns x0 + lane - P .. x0 + lane + P: the sums of
    // the element matrices' rows over the brick's elements on that column
    dfl kb[2 * P + 1], mb[2 * P + 1];
    const bool lane_elem = (lane < TX) && (x0 + lane < Ex);
    bool symx = false;
    if constexpr (E::on && !FOLD) {
      if (tb.x.sym != nullptr) symx = __all_sync(0xffffffffu, !lane_elem || tb.x.symf[x0 + lane] != 0);
    }
    if constexpr (FOLD) {
#pragma unroll
      for (int j = 0; j <= 2 * P; ++j) kb[j] = mb[j] = df_zero();
#pragma unroll
      for (int b = 0; b <= P; ++b) {  // element x0 + lane - b, its local function b
        const int e = x0 + lane - b;
        if (lane - b >= 0 && lane - b < TX && e < Ex) {
          const dfl* m = tb.x.mat + (size_t)e * 2 * (P + 1) * (P + 1) + b * (P + 1);
#pragma unroll
          for (int c = 0; c <= P; ++c) {
            kb[c - b + P] = df_add(kb[c - b + P], m[c]);
            mb[c - b + P] = df_add(mb[c - b + P], m[(P + 1) * (P + 1) + c]);
          }
        }
      }
    } else {
      const int ex = x0 + lane;
#pragma unroll
      for (int k = 0; k < Q; ++k) jwx[k] = lane_elem ? tb.x.jw[(size_t)ex * Q + k] : df_zero();
      if (symx) {
        // even-odd coefficients for the interpolation and the test contraction
        dfl* t = &nx[0][0][0];
#pragma unroll
        for (int i = 0; i < Q * (P + 1) * 2; ++i) t[i] = (lane_elem && i < NS) ? tb.x.sym[(size_t)ex * NS + i] : df_zero();
      } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
#pragma unroll
          for (int b = 0; b <= P; ++b) {
            nx[k][b][0] = lane_elem ? tb.x.nn[(((size_t)ex * Q + k) * (P + 1) + b) * 2 + 0] : df_zero();
            nx[k][b][1] = lane_elem ? tb.x.nn[(((size_t)ex * Q + k) * (P + 1) + b) * 2 + 1] : df_zero();
          }
        }
      }
    }
    for (int i = tid; i < TY * NT; i += AS_THREADS) {
      const int ey = y0 + i / NT;
      NYs[i] = (ey < Ey) ? tb.y.nn[(size_t)ey * NT + (i % NT)] : df_zero();
      if constexpr (FOLD) NYw[i] = (ey < Ey) ? tb.y.nnw[(size_t)ey * NT + (i % NT)] : df_zero();
    }
    if constexpr (E::on) {
      // the element rows' even-odd coefficients and flags (the y stage of a
      // row, one warp, takes the even-odd form where its element qualifies)
      const bool ys = tb.y.sym != nullptr;
      for (int i = tid; i < TY * NS; i += AS_THREADS) {
        const int ey = y0 + i / NS;
        SYs[i] = (ys && ey < Ey) ? tb.y.sym[(size_t)ey * NS + (i % NS)] : df_zero();
        if constexpr (FOLD) SYw[i] = (ys && ey < Ey) ? tb.y.symw[(size_t)ey * NS + (i % NS)] : df_zero();
      }
      for (int i = tid; i < TY; i += AS_THREADS) SF[i] = (ys && y0 + i < Ey) ? (int)tb.y.symf[y0 + i] : 0;
    }
    for (int i = tid; i < TY * Q; i += AS_THREADS) {
      const int ey = y0 + i / Q;
      JWYs[i] = (ey < Ey) ? tb.y.jw[(size_t)ey * Q + (i % Q)] : df_zero();
    }
    for (int i = tid; i < RF * NCOL; i += AS_THREADS) fring[i] = df_zero();

    // initial coefficient planes ez0 .. ez0+P
#pragma unroll
    for (int b = 0; b <= P; ++b) issue_plane<P>(cring + ((ez0 + b) % RC) * NCOL, a.u, g, x0, y0, ez0 + b, a.u_px);
    cp_async_commit();

    float l2_item = 0.f, l2_lo = 0.f;

    for (int ez = ez0; ez < ez1; ++ez) {
      float l2_layer = 0.f;
      if (ez + 1 < ez1) issue_plane<P>(cring + ((ez + P + 1) % RC) * NCOL, a.u, g, x0, y0, ez + P + 1, a.u_px);
      cp_async_commit();
      for (int i = tid; i < NT; i += AS_THREADS) {
        NZs[i] = tb.z.nn[(size_t)ez * NT + i];
        if constexpr (FOLD) NZw[i] = tb.z.nnw[(size_t)ez * NT + i];
      }
      for (int i = tid; i < Q; i += AS_THREADS) JWZs[i] = tb.z.jw[(size_t)ez * Q + i];
      if constexpr (E::on) {
        const bool zs = tb.z.sym != nullptr;
        for (int i = tid; i < NS; i += AS_THREADS) {
          SZs[i] = zs ? tb.z.sym[(size_t)ez * NS + i] : df_zero();
          if constexpr (FOLD) SZw[i] = zs ? tb.z.symw[(size_t)ez * NS + i] : df_zero();
        }
        if (tid == 0) SF[TY] = zs ? (int)tb.z.symf[ez] : 0;
      }
      cp_async_wait<1>();
      __syncthreads();
      const bool symz = E::on && SF[TY] != 0;
      const bool symy = E::on && SF[my_ey] != 0;  // warp-uniform: a warp is one element row

      // split each coefficient plane once, when it arrives
      {
        const int zlo = (ez == ez0) ? ez : ez + P;
        for (int z = zlo; z <= ez + P; ++z) {
          const double* src = cring + (z % RC) * NCOL;
          dfl* dst = tring + (z % RC) * NCOL;
          // the brick's own DOFs (those the next brick along an axis does not start with)
          const bool ownz = ((z < ez1) || lastz) && z < g.N[2];
          for (int i = tid; i < NCOL; i += AS_THREADS) {
            const double v = src[i];
            const unsigned long long vb = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
            umax_bits = vb > umax_bits ? vb : umax_bits;
            dst[i] = df_split(v, uexp);
            if (a.u_copy && ownz) {
              const int cy = i / CX, cx = i % CX;
              const int x = x0 + cx, y = y0 + cy;
              if ((cx < TX || lastx) && (cy < TY || lasty) && x < Nx && y < Ny)
                a.u_copy[(size_t)x + (size_t)g.PX * ((size_t)y + (size_t)Ny * z)] = v;
            }
          }
        }
      }
      __syncthreads();

      // ---- z interpolation per column: ZA = sum_b Nz C, ZB = sum_b dNz C ----
      if constexpr (E::on) {
        if (symz) {
          const typename E::N sn = E::n(SZi);
          const typename E::D sd = E::d(SZi);
          for (int col = tid; col < NCOL; col += AS_THREADS) {
            dfl c[P + 1], za[Q], zb[Q];
#pragma unroll
            for (int b = 0; b <= P; ++b) c[b] = tring[((ez + b) % RC) * NCOL + col];
            E::interp_nd(za, zb, c, sn, sd);
#pragma unroll
            for (int kz = 0; kz < Q; ++kz) {
              ZA[kz * NCOL + col] = za[kz];
              ZB[kz * NCOL + col] = zb[kz];
            }
          }
        }
      }
      for (int col = symz ? NCOL : tid; col < NCOL; col += AS_THREADS) {
        dfl c[P + 1];
#pragma unroll
        for (int b = 0; b <= P; ++b) c[b] = tring[((ez + b) % RC) * NCOL + col];
#pragma unroll
        for (int kz = 0; kz < Q; ++kz) {
          dfl za = df_mul(NZi[(kz * (P + 1)) * 2 + 0], c[0]);
          dfl zb = df_mul(NZi[(kz * (P + 1)) * 2 + 1], c[0]);
#pragma unroll
          for (int b = 1; b <= P; ++b) {
            za = df_mac(za, NZi[(kz * (P + 1) + b) * 2 + 0], c[b]);
            zb = df_mac(zb, NZi[(kz * (P + 1) + b) * 2 + 1], c[b]);
          }
          ZA[kz * NCOL + col] = za;
          ZB[kz * NCOL + col] = zb;
        }
      }
      __syncthreads();

      // this thread's partial sums of the layer for DOF rows my_ey+by, planes ez+bz
      dfl acc[P + 1][P + 1];
#pragma unroll
      for (int by = 0; by <= P; ++by)
#pragma unroll
        for (int bz = 0; bz <= P; ++bz) acc[by][bz] = df_zero();

      // the layer's points in the order 0, P, 1, P - 1, ...: a symmetric layer
      // contracts each pair (k, P - k) at once (i0p, i1p hold the first)
      dfl i0p[P + 1], i1p[P + 1];
#pragma unroll 1
      for (int it = 0; it < Q; ++it) {
        const int kz = (it & 1) ? P - (it >> 1) : (it >> 1);
        // ---- y interpolation, one (element row, column) per thread ----
        {
          dfl za[P + 1], zb[P + 1];
#pragma unroll
          for (int b = 0; b <= P; ++b) {
            za[b] = ZA[kz * NCOL + (my_ey + b) * CX + my_cx];
            zb[b] = ZB[kz * NCOL + (my_ey + b) * CX + my_cx];
          }
          if constexpr (E::on) {
            if (symy) {
              const typename E::N sn = E::n(SYi + my_ey * NS);
              const typename E::D sd = E::d(SYi + my_ey * NS);
              dfl y0v[Q], y1v[Q], y2v[Q];
              E::interp_nd(y0v, y1v, za, sn, sd);
              E::interp_n(y2v, zb, sn);
#pragma unroll
              for (int ky = 0; ky < Q; ++ky) {
                const int qy = my_ey * Q + ky;
                Y0[qy * CX + my_cx] = y0v[ky];
                Y1[qy * CX + my_cx] = y1v[ky];
                Y2[qy * CX + my_cx] = y2v[ky];
              }
            }
          }
          if (!symy) {
#pragma unroll
            for (int ky = 0; ky < Q; ++ky) {
              const dfl* ny = NYi + my_ey * NT + ky * (P + 1) * 2;
              dfl y0v = df_mul(ny[0], za[0]);
              dfl y1v = df_mul(ny[1], za[0]);
              dfl y2v = df_mul(ny[0], zb[0]);
#pragma unroll
              for (int b = 1; b <= P; ++b) {
                y0v = df_mac(y0v, ny[2 * b], za[b]);
                y1v = df_mac(y1v, ny[2 * b + 1], za[b]);
                y2v = df_mac(y2v, ny[2 * b], zb[b]);
              }
              const int qy = my_ey * Q + ky;
              Y0[qy * CX + my_cx] = y0v;
              Y1[qy * CX + my_cx] = y1v;
              Y2[qy * CX + my_cx] = y2v;
            }
          }
        }
        // warp w is element row w in all three stages of a point layer: it
        // writes the Y rows of its Q points, runs the x stage on them and
        // reads the H rows it wrote, so the stages meet at warp barriers
        __syncwarp();

        // ---- x stage (warp per row): the bands' products under FOLD, else x
        // interpolation + integrand + x test contraction ----
        // HREG: this lane's column of the warp's H rows stays in registers for
        // the y test; otherwise the rows go through shared memory
        dfl hr0[Q], hr1[Q], hr2[Q];
#pragma unroll (HREG ? Q : 1)
        for (int kyr = 0; kyr < Q; ++kyr) {
          const int qy = warp * Q + kyr;
          const int ey_l = warp;
          const bool elem_ok = lane_elem && (y0 + ey_l < Ey);
          const dfl jwyz = FOLD ? df_zero() : df_mul(JWYs[qy], JWZs[kz]);
          const dfl cyz = FOLD ? df_zero() : df_mul(ndtk, jwyz);
          // under FOLD the interpolated values carry Jy Wy Jz Wz: the l2norm's
          // J W u^2 is Jx Wx u'^2 / (Jy Wy Jz Wz)
          const float jyz = JWYs[qy].x * JWZs[kz].x;  // 0 on rows past the mesh
          const float wr = (FOLD && jyz > 0.f) ? __frcp_rn(jyz) : 0.f;
          // this lane's P + 1 values of a y-interpolated plane
          auto yrow = [&](const dfl* Yp, dfl (&v)[P + 1]) {
#pragma unroll
            for (int b = 0; b <= P; ++b) v[b] = lane_elem ? Yp[qy * CX + lane + b] : df_zero();
          };
          const long long qyg = (long long)y0 * Q + qy;
          const long long qzg = (long long)ez * Q + kz;
          if constexpr (FOLD) {
            // H0 = Kx Y0, H1 = Mx Y1, H2 = Mx Y2 along the row with the brick's
            // bands (column lane), and the l2norm's row term Y0' Mx Y0 from
            // the high parts.  Columns outside the row carry zero coefficients:
            // their reads are clamped into it.
            const dfl* r0 = Y0 + qy * CX;
            const dfl* r1 = Y1 + qy * CX;
            const dfl* r2 = Y2 + qy * CX;
            dfl a0 = df_mul(kb[0], r0[xoff[0]]);
            dfl a1 = df_mul(mb[0], r1[xoff[0]]);
            dfl a2 = df_mul(mb[0], r2[xoff[0]]);
            float t = mb[0].x * r0[xoff[0]].x;
#pragma unroll
            for (int j = 1; j <= 2 * P; ++j) {
              const dfl v0 = r0[xoff[j]];
              a0 = df_mac(a0, kb[j], v0);
              a1 = df_mac(a1, mb[j], r1[xoff[j]]);
              a2 = df_mac(a2, mb[j], r2[xoff[j]]);
              t = fmaf(mb[j].x, v0.x, t);
            }
            l2_layer = fmaf(wr * r0[lane].x, t, l2_layer);
            if constexpr (HREG) {
              hr0[kyr] = a0;
              hr1[kyr] = a1;
              hr2[kyr] = a2;
            } else {
              H0[qy * CX + lane] = a0;
              H1[qy * CX + lane] = a1;
              H2[qy * CX + lane] = a2;
            }
          } else {
            dfl h0[P + 1], h1[P + 1], h2[P + 1];
            if constexpr (E::on && !FOLD) {
              if (symx) {
                const typename E::N sn = E::n(&nx[0][0][0]);
                const typename E::D sd = E::d(&nx[0][0][0]);
                // the point weights, then one gradient component at a time:
                // interpolate, weight, contract
                dfl cw[Q];
                float sx[Q];
                dfl g0[Q];
#pragma unroll
                for (int kx = 0; kx < Q; ++kx) {
                  const long long qidx = ((long long)(x0 + lane) * Q + kx) + QXt * (qyg + QYt * qzg);
                  if constexpr (HAS_K || HAS_F) {
                    const dfl s = df_mul(jwx[kx], jwyz);
                    sx[kx] = s.x;
                    if constexpr (HAS_K) cw[kx] = df_mul(df_mul(ndt, elem_ok ? df_split(a.kqp[qidx], 0) : df_zero()), s);
                    if constexpr (HAS_F) g0[kx] = df_mul(df_mul(s, dtv), elem_ok ? df_split(a.fqp[qidx], uexp) : df_zero());
                  } else {
                    sx[kx] = jwx[kx].x * jwyz.x;  // the l2norm's weight: high parts suffice
                  }
                  if constexpr (!HAS_K) cw[kx] = df_mul(jwx[kx], cyz);
                }
                dfl yv0[P + 1];
                yrow(Y0, yv0);
                {
                  // u at the points from the high parts (the l2norm), the same even-odd form
                  float u[Q];
                  E::uu(u, yv0, sn);
#pragma unroll
                  for (int kx = 0; kx < Q; ++kx) l2_layer = fmaf(sx[kx] * u[kx], u[kx], l2_layer);
                }
                {
                  dfl du[Q];
                  E::interp_d(du, yv0, sd);
#pragma unroll
                  for (int kx = 0; kx < Q; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                  E::test_d(h0, du, sd);
                }
                {
                  dfl du[Q], yv1[P + 1];
                  yrow(Y1, yv1);
                  E::interp_n(du, yv1, sn);
#pragma unroll
                  for (int kx = 0; kx < Q; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                  E::test_n(h1, du, sn);
                }
                {
                  dfl du[Q], yv2[P + 1];
                  yrow(Y2, yv2);
                  E::interp_n(du, yv2, sn);
#pragma unroll
                  for (int kx = 0; kx < Q; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                  E::test_n(h2, du, sn);
                }
                if constexpr (HAS_F) {
                  dfl hf[P + 1];
                  E::test_n(hf, g0, sn);
#pragma unroll
                  for (int b = 0; b <= P; ++b) h0[b] = df_add(h0[b], hf[b]);
                }
              }
            }
            if (!symx && !FOLD) {
            dfl yv0[P + 1], yv1[P + 1], yv2[P + 1];
            yrow(Y0, yv0);
            yrow(Y1, yv1);
            yrow(Y2, yv2);
#pragma unroll
            for (int kx = 0; kx < Q; ++kx) {
              dfl dux = df_mul(nx[kx][0][1], yv0[0]);
              dfl duy = df_mul(nx[kx][0][0], yv1[0]);
              dfl duz = df_mul(nx[kx][0][0], yv2[0]);
              float uu = nx[kx][0][0].x * yv0[0].x;
#pragma unroll
              for (int b = 1; b <= P; ++b) {
                dux = df_mac(dux, nx[kx][b][1], yv0[b]);
                duy = df_mac(duy, nx[kx][b][0], yv1[b]);
                duz = df_mac(duz, nx[kx][b][0], yv2[b]);
                uu = fmaf(nx[kx][b][0].x, yv0[b].x, uu);
              }
              const long long qidx = ((long long)(x0 + lane) * Q + kx) + QXt * (qyg + QYt * qzg);
              dfl c;
              dfl g0 = df_zero();
              {
                const dfl s = df_mul(jwx[kx], jwyz);
                if constexpr (HAS_K) c = df_mul(df_mul(ndt, elem_ok ? df_split(a.kqp[qidx], 0) : df_zero()), s);
                else c = df_mul(jwx[kx], cyz);
                l2_layer = fmaf(s.x * uu, uu, l2_layer);
                if constexpr (HAS_F) g0 = df_mul(df_mul(s, dtv), elem_ok ? df_split(a.fqp[qidx], uexp) : df_zero());
              }
              const dfl g1 = df_mul(c, dux), g2 = df_mul(c, duy), g3 = df_mul(c, duz);
#pragma unroll
              for (int b = 0; b <= P; ++b) {
                if (kx == 0) {
                  h0[b] = df_mul(nx[kx][b][1], g1);
                  h1[b] = df_mul(nx[kx][b][0], g2);
                  h2[b] = df_mul(nx[kx][b][0], g3);
                } else {
                  h0[b] = df_mac(h0[b], nx[kx][b][1], g1);
                  h1[b] = df_mac(h1[b], nx[kx][b][0], g2);
                  h2[b] = df_mac(h2[b], nx[kx][b][0], g3);
                }
                if constexpr (HAS_F) h0[b] = df_mac(h0[b], nx[kx][b][0], g0);
              }
            }
            }  // !symx && !FOLD
            // column cx = lane receives local function b of element lane - b
            dfl v0 = h0[0], v1 = h1[0], v2 = h2[0];
#pragma unroll
            for (int b = 1; b <= P; ++b) {
              const dfl s0 = df_shfl_up(h0[b], b);
              const dfl s1 = df_shfl_up(h1[b], b);
              const dfl s2 = df_shfl_up(h2[b], b);
              if (lane >= b) { v0 = df_add(v0, s0); v1 = df_add(v1, s1); v2 = df_add(v2, s2); }
            }
            H0[qy * CX + lane] = v0;
            H1[qy * CX + lane] = v1;
            H2[qy * CX + lane] = v2;
          }
        }
        __syncwarp();

        // ---- y test contraction of this thread's element row, then z ----
        {
          dfl i0[P + 1], i1[P + 1];
          if constexpr (E::on) {
            if (symy) {
              const typename E::N sn = E::n(SYs + my_ey * NS);
              const typename E::D sd = E::d(SYs + my_ey * NS);
              dfl hv0[Q], hv1[Q], hv2[Q], ta[P + 1], tb1[P + 1];
#pragma unroll
              for (int ky = 0; ky < Q; ++ky) {
                const int qy = my_ey * Q + ky;
                hv0[ky] = HREG ? hr0[ky] : H0[qy * CX + my_cx];
                hv1[ky] = HREG ? hr1[ky] : H1[qy * CX + my_cx];
                hv2[ky] = HREG ? hr2[ky] : H2[qy * CX + my_cx];
              }
              E::test_n(ta, hv0, sn);
              E::test_d(tb1, hv1, sd);
#pragma unroll
              for (int by = 0; by <= P; ++by) i0[by] = df_add(ta[by], tb1[by]);
              E::test_n(i1, hv2, sn);
            }
          }
          if (!symy) {
#pragma unroll
          for (int ky = 0; ky < Q; ++ky) {
            const int qy = my_ey * Q + ky;
            const dfl hv0 = HREG ? hr0[ky] : H0[qy * CX + my_cx];
            const dfl hv1 = HREG ? hr1[ky] : H1[qy * CX + my_cx];
            const dfl hv2 = HREG ? hr2[ky] : H2[qy * CX + my_cx];
            const dfl* ny = NYs + my_ey * NT + ky * (P + 1) * 2;
#pragma unroll
            for (int by = 0; by <= P; ++by) {
              if (ky == 0) {
                i0[by] = df_mul(ny[2 * by], hv0);
                i1[by] = df_mul(ny[2 * by], hv2);
              } else {
                i0[by] = df_mac(i0[by], ny[2 * by], hv0);
                i1[by] = df_mac(i1[by], ny[2 * by], hv2);
              }
              i0[by] = df_mac(i0[by], ny[2 * by + 1], hv1);
            }
          }
          }  // !symy
          if constexpr (ZEO) {
            if (symz) {
              if (it & 1) {
#pragma unroll
                for (int by = 0; by <= P; ++by) E::zt_pair(acc[by], it >> 1, i0p[by], i0[by], i1p[by], i1[by], SZs);
              } else if (2 * kz == P) {
#pragma unroll
                for (int by = 0; by <= P; ++by) E::zt_mid(acc[by], i0[by], i1[by], SZs);
              } else {
#pragma unroll
                for (int by = 0; by <= P; ++by) { i0p[by] = i0[by]; i1p[by] = i1[by]; }
              }
            }
          }
          if (!ZEO || !symz) {
#pragma unroll
            for (int bz = 0; bz <= P; ++bz) {
              const dfl nz0 = NZs[(kz * (P + 1) + bz) * 2 + 0];
              const dfl nz1 = NZs[(kz * (P + 1) + bz) * 2 + 1];
#pragma unroll
              for (int by = 0; by <= P; ++by) acc[by][bz] = df_mac(df_mac(acc[by][bz], nz0, i0[by]), nz1, i1[by]);
            }
          }
        }
      }  // kz
      if constexpr (ZEO) {
        if (symz) {
#pragma unroll
          for (int by = 0; by <= P; ++by) E::zt_finish(acc[by]);
        }
      }

      // compensated FP32 sum of the l2 layers
      {
        const float t = l2_item + l2_layer;
        const float bp = t - l2_item;
        l2_lo += (l2_item - (t - bp)) + (l2_layer - bp);
        l2_item = t;
      }

      // accumulate this layer's element partials into the DOF planes, one
      // element-row offset at a time so no two threads touch the same entry
#pragma unroll
      for (int by = 0; by <= P; ++by) {
        const int row = my_ey + by;
#pragma unroll
        for (int bz = 0; bz <= P; ++bz) {
          const int o = ((ez + bz) % RF) * NCOL + row * CX + my_cx;
          fring[o] = df_add(fring[o], acc[by][bz]);
        }
        __syncthreads();
      }

      // DOF plane ez is complete: write it out (scaled back) and clear its slot
      {
        const int cz = ez;
        const bool ownz = (cz < ez1) || lastz;
        const int slot = (cz % RF) * NCOL;
        for (int it = tid; it < NCOL; it += AS_THREADS) {
          const int cy = it / CX, cx = it % CX;
          const int x = x0 + cx, y = y0 + cy;
          dfl f = fring[slot + it];
          fring[slot + it] = df_zero();
          if constexpr (FOLD) f = df_mul(f, ndtk);  // -dt kappa, kept out of the point sums
          if (x < Nx && y < Ny) {
            const double v = f2d_scaled(f.x, -uexp) + f2d_scaled(f.y, -uexp);
            const bool ownx = (cx < TX) || lastx, owny = (cy < TY) || lasty;
            const int cls = (ownx ? 0 : 1) | (owny ? 0 : 2) | (ownz ? 0 : 4);
            double* dst = (cls == 0) ? a.F : a.shadow + (size_t)(cls - 1) * a.shadow_stride;
            dst[(size_t)x + (size_t)g.PX * ((size_t)y + (size_t)Ny * cz)] = v;
            const unsigned long long vb = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
            amax_bits = vb > amax_bits ? vb : amax_bits;
          }
        }
      }
      __syncthreads();
    }  // ez

    // remaining planes ez1 .. ez1+P-1
    for (int cz = ez1; cz < ez1 + P; ++cz) {
      const bool ownz = lastz;
      const int slot = (cz % RF) * NCOL;
      for (int it = tid; it < NCOL; it += AS_THREADS) {
        const int cy = it / CX, cx = it % CX;
        const int x = x0 + cx, y = y0 + cy;
        if (x < Nx && y < Ny && cz < g.N[2]) {
          dfl f = fring[slot + it];
          if constexpr (FOLD) f = df_mul(f, ndtk);  // -dt kappa, kept out of the point sums
          const double v = f2d_scaled(f.x, -uexp) + f2d_scaled(f.y, -uexp);
          const bool ownx = (cx < TX) || lastx, owny = (cy < TY) || lasty;
          const int cls = (ownx ? 0 : 1) | (owny ? 0 : 2) | (ownz ? 0 : 4);
          double* dst = (cls == 0) ? a.F : a.shadow + (size_t)(cls - 1) * a.shadow_stride;
          dst[(size_t)x + (size_t)g.PX * ((size_t)y + (size_t)Ny * cz)] = v;
          const unsigned long long vb = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
          amax_bits = vb > amax_bits ? vb : amax_bits;
        }
      }
    }
    l2_thread += (double)l2_item + (double)l2_lo;
    cp_async_wait<0>();
  }  // item

  // deterministic block reduction of the l2 partial and of max |value|
  double v = l2_thread;
  unsigned long long mb = amax_bits, ub = umax_bits;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_down_sync(0xffffffffu, v, o);
    const unsigned long long ob = __shfl_down_sync(0xffffffffu, mb, o);
    mb = ob > mb ? ob : mb;
    const unsigned long long oub = __shfl_down_sync(0xffffffffu, ub, o);
    ub = oub > ub ? oub : ub;
  }
  __syncthreads();
  unsigned long long* redm = reinterpret_cast<unsigned long long*>(red + AS_THREADS / 32);
  unsigned long long* redu = redm + AS_THREADS / 32;
  if (lane == 0) { red[warp] = v; redm[warp] = mb; redu[warp] = ub; }
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    unsigned long long m = 0ull, mu = 0ull;
    for (int w = 0; w < AS_THREADS / 32; ++w) {
      t += red[w];
      m = redm[w] > m ? redm[w] : m;
      mu = redu[w] > mu ? redu[w] : mu;
    }
    // the high parts integrated (2^uexp u)^2
    a.l2part[blockIdx.x] = t * ldexp(1.0, -2 * uexp);
    a.l2part[gridDim.x + blockIdx.x] = __longlong_as_double((long long)m);
    a.l2part[2 * gridDim.x + blockIdx.x] = 0.0;
    a.l2part[3 * gridDim.x + blockIdx.x] = __longlong_as_double((long long)mu);
  }
}

template <int P, bool HF, bool HK>
static cudaError_t launch_df(const AssembleArgs& a, const DfTabs3& tb, int grid, int* used_grid, cudaStream_t s) {
  using L = DfLayout<P>;
  auto kern = k_assemble_df<P, HF, HK>;
  const size_t bytes = L::bytes;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, AS_THREADS, bytes);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int items = a.nix * a.niy * a.niz;
  int gr = std::min(std::min(grid, items), nsm * per_sm);
  if (gr < 1) gr = 1;
  *used_grid = gr;
  kern<<<gr, AS_THREADS, bytes, s>>>(a, tb);
  return cudaGetLastError();
}

template <int P>
static cudaError_t dispatch_df(const AssembleArgs& a, const DfTabs3& tb, int grid, int* used_grid, cudaStream_t s) {
  const bool hf = a.fqp != nullptr, hk = a.kqp != nullptr;
  if (hf && hk) return launch_df<P, true, true>(a, tb, grid, used_grid, s);
  if (hf) return launch_df<P, true, false>(a, tb, grid, used_grid, s);
  if (hk) return launch_df<P, false, true>(a, tb, grid, used_grid, s);
  return launch_df<P, false, false>(a, tb, grid, used_grid, s);
}

cudaError_t launch_assemble_df(const AssembleArgs& a, const DfTabs3& tb, int grid, int* used_grid, cudaStream_t s) {
  if (a.form != ADS_FORM_HEAT) return cudaErrorInvalidValue;
  switch (a.g.P) {
    case 1: return dispatch_df<1>(a, tb, grid, used_grid, s);
    case 2: return dispatch_df<2>(a, tb, grid, used_grid, s);
    case 3: return dispatch_df<3>(a, tb, grid, used_grid, s);
    case 4: return dispatch_df<4>(a, tb, grid, used_grid, s);
    default: return cudaErrorInvalidValue;
  }
}

size_t assemble_df_smem_bytes(int P) {
  switch (P) {
    case 1: return DfLayout<1>::bytes;
    case 2: return DfLayout<2>::bytes;
    case 3: return DfLayout<3>::bytes;
    case 4: return DfLayout<4>::bytes;
  }
  return 0;
}

}  // namespace ads
