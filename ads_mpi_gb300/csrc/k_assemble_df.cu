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
// The coefficients are scaled by 2^-e (max |u| < 2^e, from the uscale pass)
// so that FP32 never overflows, split once per plane into (high, low) floats,
// and the finished DOF planes are scaled back by 2^e exactly.  The l2norm
// (J W u^2) is accumulated from the high parts in compensated FP32.
#include "df32.cuh"
#include "k_assemble.cuh"

namespace ads {

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
  static constexpr size_t o_sy = o_jwz + D * Q;                 // dfl [TY][DF_SYM] (p = 2)
  static constexpr size_t o_sz = o_sy + D * TY * DF_SYM;        // dfl [DF_SYM]
  static constexpr size_t o_sf = o_sz + D * DF_SYM;             // int [TY + 1]: rows, then the layer
  static constexpr size_t o_red = (o_sf + 4 * (TY + 1) + 15) / 16 * 16;
  static constexpr size_t bytes = o_red + 3 * sizeof(double) * (AS_THREADS / 32);
};

__device__ __forceinline__ dfl df_split(double d, int sexp) {
  float h, l;
  split_scaled(d, sexp, h, l);
  return df_make(h, l);
}

// ---- even-odd forms of an element's 3 x 3 contractions (p = 2) ----
// For an element whose tables are centro-symmetric, N[k][b] = N[2-k][2-b]
// and dN[k][b] = -dN[2-k][2-b] (Gauss points symmetric about the element's
// centre, basis mirrored: every element of a uniform knot vector but the
// first and the last), the sums over b of an interpolation pair the outputs k
// and 2-k: with s = v0 + v2 and d = v0 - v2,
//   sum_b N[k][b] v[b]:  out0,2 = (a s + N01 v1) +- c d,  out1 = N10 s + N11 v1
//   sum_b dN[k][b] v[b]: out0,2 = a' s + dN01 v1 ... (signs below), out1 = dN10 d
// with a = (N00 + N02)/2, c = (N00 - N02)/2 (a', c' the same for dN); the
// test contractions (sums over k) are the transposes.  A double-float
// multiply-add costs 12 FP32 operations and a sum 8, so the forms below take
// 52-68 operations for what the direct sums do in 84.
struct SymN { dfl a, c, n01, n10, n11; };
struct SymD { dfl a, c, d01, d10; };

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

// out[k] = sum_b N[k][b] v[b]
__device__ __forceinline__ void eo_interp_n(dfl (&out)[3], const dfl (&v)[3], const SymN& n) {
  const dfl sp = df_add(v[0], v[2]), dm = df_sub(v[0], v[2]);
  const dfl e = df_mac(df_mul(n.a, sp), n.n01, v[1]), d = df_mul(n.c, dm);
  out[0] = df_add(e, d);
  out[2] = df_sub(e, d);
  out[1] = df_mac(df_mul(n.n10, sp), n.n11, v[1]);
}
// on[k] = sum_b N[k][b] v[b], od[k] = sum_b dN[k][b] v[b] (s and d shared)
__device__ __forceinline__ void eo_interp_nd(dfl (&on)[3], dfl (&od)[3], const dfl (&v)[3], const SymN& n,
                                             const SymD& dn) {
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
// out[k] = sum_b dN[k][b] v[b]
__device__ __forceinline__ void eo_interp_d(dfl (&out)[3], const dfl (&v)[3], const SymD& dn) {
  const dfl sp = df_add(v[0], v[2]), dm = df_sub(v[0], v[2]);
  const dfl e = df_mac(df_mul(dn.a, sp), dn.d01, v[1]), d = df_mul(dn.c, dm);
  out[0] = df_add(d, e);
  out[2] = df_sub(d, e);
  out[1] = df_mul(dn.d10, dm);
}
// h[b] = sum_k N[k][b] g[k]
__device__ __forceinline__ void eo_test_n(dfl (&h)[3], const dfl (&g)[3], const SymN& n) {
  const dfl sp = df_add(g[0], g[2]), dm = df_sub(g[0], g[2]);
  const dfl e = df_mac(df_mul(n.a, sp), n.n10, g[1]), d = df_mul(n.c, dm);
  h[0] = df_add(e, d);
  h[2] = df_sub(e, d);
  h[1] = df_mac(df_mul(n.n01, sp), n.n11, g[1]);
}
// h[b] = sum_k dN[k][b] g[k]
__device__ __forceinline__ void eo_test_d(dfl (&h)[3], const dfl (&g)[3], const SymD& dn) {
  const dfl sp = df_add(g[0], g[2]), dm = df_sub(g[0], g[2]);
  const dfl e = df_mac(df_mul(dn.c, sp), dn.d10, g[1]), d = df_mul(dn.a, dm);
  h[0] = df_add(e, d);
  h[2] = df_sub(d, e);
  h[1] = df_mul(dn.d01, dm);
}
__device__ __forceinline__ SymN sym_n(const dfl* t) { return SymN{t[0], t[1], t[2], t[3], t[4]}; }
__device__ __forceinline__ SymD sym_d(const dfl* t) { return SymD{t[5], t[6], t[7], t[8]}; }

template <int P, bool HAS_F, bool HAS_K>
__global__ void __launch_bounds__(AS_THREADS, P <= 2 ? 2 : 1)
    k_assemble_df(const AssembleArgs a, const DfTabs3 tb) {
  using L = DfLayout<P>;
  constexpr int Q = L::Q, TX = L::TX, TY = L::TY, CX = L::CX;
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
  double* red = reinterpret_cast<double*>(smem + L::o_red);

  const Geometry& g = a.g;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int Ex = g.E[0], Ey = g.E[1], Ez = g.E[2];
  const int Nx = g.N[0], Ny = g.N[1];
  const long long QXt = (long long)Ex * Q, QYt = (long long)Ey * Q;
  const int nitems = a.nix * a.niy * a.niz;
  const int my_ey = tid / CX, my_cx = tid % CX;
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

    // per-lane x tables (element x0 + lane; lanes >= TX have no element).
    // p = 2 bricks whose elements are all centro-symmetric run the x stage in
    // even-odd form; the table registers then hold the lane's DF_SYM
    // even-odd coefficients
    dfl nx[Q][P + 1][2];
    dfl jwx[Q];
    const bool lane_elem = (lane < TX) && (x0 + lane < Ex);
    bool symx = false;
    if constexpr (P == 2) {
      if (tb.x.sym != nullptr) symx = __all_sync(0xffffffffu, !lane_elem || tb.x.symf[x0 + lane] != 0);
    }
    {
      const int ex = x0 + lane;
#pragma unroll
      for (int k = 0; k < Q; ++k) jwx[k] = lane_elem ? tb.x.jw[(size_t)ex * Q + k] : df_zero();
      if (symx) {
        dfl* t = &nx[0][0][0];
#pragma unroll
        for (int i = 0; i < Q * (P + 1) * 2; ++i)
          t[i] = (i < DF_SYM && lane_elem) ? tb.x.sym[(size_t)ex * DF_SYM + i] : df_zero();
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
    }
    if constexpr (P == 2) {
      // the element rows' even-odd coefficients and flags (the y stage of a
      // row, one warp, takes the even-odd form where its element qualifies)
      const bool ys = tb.y.sym != nullptr;
      for (int i = tid; i < TY * DF_SYM; i += AS_THREADS) {
        const int ey = y0 + i / DF_SYM;
        SYs[i] = (ys && ey < Ey) ? tb.y.sym[(size_t)ey * DF_SYM + (i % DF_SYM)] : df_zero();
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
      for (int i = tid; i < NT; i += AS_THREADS) NZs[i] = tb.z.nn[(size_t)ez * NT + i];
      for (int i = tid; i < Q; i += AS_THREADS) JWZs[i] = tb.z.jw[(size_t)ez * Q + i];
      if constexpr (P == 2) {
        const bool zs = tb.z.sym != nullptr;
        for (int i = tid; i < DF_SYM; i += AS_THREADS) SZs[i] = zs ? tb.z.sym[(size_t)ez * DF_SYM + i] : df_zero();
        if (tid == 0) SF[TY] = zs ? (int)tb.z.symf[ez] : 0;
      }
      cp_async_wait<1>();
      __syncthreads();
      const bool symz = (P == 2) && SF[TY] != 0;
      const bool symy = (P == 2) && SF[my_ey] != 0;  // warp-uniform: a warp is one element row

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
      if constexpr (P == 2) {
        if (symz) {
          const SymN sn = sym_n(SZs);
          const SymD sd = sym_d(SZs);
          for (int col = tid; col < NCOL; col += AS_THREADS) {
            dfl c[3], za[3], zb[3];
#pragma unroll
            for (int b = 0; b < 3; ++b) c[b] = tring[((ez + b) % RC) * NCOL + col];
            eo_interp_nd(za, zb, c, sn, sd);
#pragma unroll
            for (int kz = 0; kz < 3; ++kz) {
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
          dfl za = df_mul(NZs[(kz * (P + 1)) * 2 + 0], c[0]);
          dfl zb = df_mul(NZs[(kz * (P + 1)) * 2 + 1], c[0]);
#pragma unroll
          for (int b = 1; b <= P; ++b) {
            za = df_mac(za, NZs[(kz * (P + 1) + b) * 2 + 0], c[b]);
            zb = df_mac(zb, NZs[(kz * (P + 1) + b) * 2 + 1], c[b]);
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

#pragma unroll 1
      for (int kz = 0; kz < Q; ++kz) {
        // ---- y interpolation, one (element row, column) per thread ----
        {
          dfl za[P + 1], zb[P + 1];
#pragma unroll
          for (int b = 0; b <= P; ++b) {
            za[b] = ZA[kz * NCOL + (my_ey + b) * CX + my_cx];
            zb[b] = ZB[kz * NCOL + (my_ey + b) * CX + my_cx];
          }
          if constexpr (P == 2) {
            if (symy) {
              const SymN sn = sym_n(SYs + my_ey * DF_SYM);
              const SymD sd = sym_d(SYs + my_ey * DF_SYM);
              dfl y0v[3], y1v[3], y2v[3];
              eo_interp_nd(y0v, y1v, za, sn, sd);
              eo_interp_n(y2v, zb, sn);
#pragma unroll
              for (int ky = 0; ky < 3; ++ky) {
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
              const dfl* ny = NYs + my_ey * NT + ky * (P + 1) * 2;
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
        __syncthreads();

        // ---- x interpolation + integrand + x test contraction (warp per row) ----
        for (int qy = warp; qy < QY; qy += AS_THREADS / 32) {
          const int ey_l = qy / Q;
          const bool elem_ok = lane_elem && (y0 + ey_l < Ey);
          const dfl jwyz = df_mul(JWYs[qy], JWZs[kz]);
          const dfl cyz = df_mul(ndtk, jwyz);
          // this lane's P + 1 values of a y-interpolated plane
          auto yrow = [&](const dfl* Yp, dfl (&v)[P + 1]) {
#pragma unroll
            for (int b = 0; b <= P; ++b) v[b] = lane_elem ? Yp[qy * CX + lane + b] : df_zero();
          };
          const long long qyg = (long long)y0 * Q + qy;
          const long long qzg = (long long)ez * Q + kz;
          dfl h0[P + 1], h1[P + 1], h2[P + 1];
          if constexpr (P == 2) {
            if (symx) {
              const SymN sn = sym_n(&nx[0][0][0]);
              const SymD sd = sym_d(&nx[0][0][0]);
              // the point weights, then one gradient component at a time:
              // interpolate, weight, contract
              dfl cw[3];
              float sx[3];
              dfl g0[3];
#pragma unroll
              for (int kx = 0; kx < 3; ++kx) {
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
              dfl yv0[3];
              yrow(Y0, yv0);
              {
                // u at the points from the high parts (the l2norm), the same even-odd form
                const float sp = yv0[0].x + yv0[2].x, dm = yv0[0].x - yv0[2].x;
                const float e = fmaf(sn.n01.x, yv0[1].x, sn.a.x * sp), d = sn.c.x * dm;
                const float u0 = e + d, u2 = e - d, u1 = fmaf(sn.n11.x, yv0[1].x, sn.n10.x * sp);
                l2_layer = fmaf(sx[0] * u0, u0, l2_layer);
                l2_layer = fmaf(sx[1] * u1, u1, l2_layer);
                l2_layer = fmaf(sx[2] * u2, u2, l2_layer);
              }
              {
                dfl du[3];
                eo_interp_d(du, yv0, sd);
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                eo_test_d(h0, du, sd);
              }
              {
                dfl du[3], yv1[3];
                yrow(Y1, yv1);
                eo_interp_n(du, yv1, sn);
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                eo_test_n(h1, du, sn);
              }
              {
                dfl du[3], yv2[3];
                yrow(Y2, yv2);
                eo_interp_n(du, yv2, sn);
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) du[kx] = df_mul(cw[kx], du[kx]);
                eo_test_n(h2, du, sn);
              }
              if constexpr (HAS_F) {
                dfl hf[3];
                eo_test_n(hf, g0, sn);
#pragma unroll
                for (int b = 0; b < 3; ++b) h0[b] = df_add(h0[b], hf[b]);
              }
            }
          }
          if (!symx) {
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
            const dfl s = df_mul(jwx[kx], jwyz);
            dfl c;
            if constexpr (HAS_K) c = df_mul(df_mul(ndt, elem_ok ? df_split(a.kqp[qidx], 0) : df_zero()), s);
            else c = df_mul(jwx[kx], cyz);
            const dfl g1 = df_mul(c, dux), g2 = df_mul(c, duy), g3 = df_mul(c, duz);
            l2_layer = fmaf(s.x * uu, uu, l2_layer);
            dfl g0 = df_zero();
            if constexpr (HAS_F) g0 = df_mul(df_mul(s, dtv), elem_ok ? df_split(a.fqp[qidx], uexp) : df_zero());
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
          }  // !symx
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
        __syncthreads();

        // ---- y test contraction of this thread's element row, then z ----
        {
          dfl i0[P + 1], i1[P + 1];
          if constexpr (P == 2) {
            if (symy) {
              const SymN sn = sym_n(SYs + my_ey * DF_SYM);
              const SymD sd = sym_d(SYs + my_ey * DF_SYM);
              dfl hv0[3], hv1[3], hv2[3], ta[3], tb1[3];
#pragma unroll
              for (int ky = 0; ky < 3; ++ky) {
                const int qy = my_ey * Q + ky;
                hv0[ky] = H0[qy * CX + my_cx];
                hv1[ky] = H1[qy * CX + my_cx];
                hv2[ky] = H2[qy * CX + my_cx];
              }
              eo_test_n(ta, hv0, sn);
              eo_test_d(tb1, hv1, sd);
#pragma unroll
              for (int by = 0; by < 3; ++by) i0[by] = df_add(ta[by], tb1[by]);
              eo_test_n(i1, hv2, sn);
            }
          }
          if (!symy) {
#pragma unroll
          for (int ky = 0; ky < Q; ++ky) {
            const int qy = my_ey * Q + ky;
            const dfl hv0 = H0[qy * CX + my_cx];
            const dfl hv1 = H1[qy * CX + my_cx];
            const dfl hv2 = H2[qy * CX + my_cx];
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
#pragma unroll
          for (int bz = 0; bz <= P; ++bz) {
            const dfl nz0 = NZs[(kz * (P + 1) + bz) * 2 + 0];
            const dfl nz1 = NZs[(kz * (P + 1) + bz) * 2 + 1];
#pragma unroll
            for (int by = 0; by <= P; ++by) acc[by][bz] = df_mac(df_mac(acc[by][bz], nz0, i0[by]), nz1, i1[by]);
          }
        }
      }  // kz

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
          const dfl f = fring[slot + it];
          fring[slot + it] = df_zero();
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
          const dfl f = fring[slot + it];
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
