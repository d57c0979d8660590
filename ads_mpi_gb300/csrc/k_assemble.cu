// k_assemble.cu — Gauss-quadrature right-hand-side assembly (K1).
//
// Replaces FormUn (src/projection_engine.F90:306-441) followed by Form3DRHS
// (src/projection_engine.F90:154-284) with the integrands of
// problems/heat/RHS_eq.F90:69-86 and problems/L2Projection/RHS_eq.F90:66-70.
//
// The reference evaluates u and grad u at every quadrature point with
// (p+1)^3 basis products per point, stores them in Un/dUn, and then calls the
// integrand once per (point, test function).  Here the same sums are
// sum-factorised one direction at a time and fused into one kernel; nothing is
// materialised per quadrature point:
//
//   interpolation   C[bz,by,bx] --z--> ZA,ZB --y--> Y0,Y1,Y2 --x--> u, du/dx, du/dy, du/dz
//   integrand       g0 = JW (u + dt f),  g{1,2,3} = -dt kappa JW du/d{x,y,z}     (heat)
//                   g0 = JW f                                                   (projection)
//   test functions  g --x--> H0,H1,H2 --y--> I0,I1 --z--> F (accumulated in FP64)
//
// Work decomposition: a CTA owns a brick of (32-p) x AS_TY elements in x/y and
// a chunk of element layers in z, which it streams layer by layer with a ring
// of p+2 coefficient planes (prefetched with cp.async) and a ring of p+1 FP64
// accumulator planes.  A DOF plane is complete once the layer with the same
// index is done and is then written out.  DOFs of the brick's footprint that
// belong to the next brick in x, y or z ("spill" DOFs, p wide) go to one of
// seven shadow arrays instead; k_fixup adds them in a fixed order, so the
// result is deterministic and no atomics are used.
//
// The integrand's l2norm (J W u^2 for heat, J W f^2 for projection; the
// reference sums J W v u^2 over the test functions v, which is the same by the
// partition of unity) is reduced per CTA and finished by k_fixup.
#include "k_assemble.cuh"

namespace ads {

// The assembly's partials: the l2norm, the drained statistic (oil form), max
// |F| and the power-of-two scale of the FP32 solve (from the largest value the
// assembly wrote, which is within a factor 8 of max |F|: a DOF sums at most 8
// written parts).
__global__ void k_fixup_scale(const FixupArgs a) {
  const int lane = threadIdx.x & 31;
  double t = 0.0, d = 0.0;
  unsigned long long m = 0ull;
  for (int i = lane; i < a.nl2; i += 32) {
    t += a.l2part[i];
    d += a.l2part[2 * a.nl2 + i];
    const unsigned long long b = (unsigned long long)__double_as_longlong(a.l2part[a.nl2 + i]);
    m = b > m ? b : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_down_sync(0xffffffffu, t, o);
    d += __shfl_down_sync(0xffffffffu, d, o);
    const unsigned long long ob = __shfl_down_sync(0xffffffffu, m, o);
    m = ob > m ? ob : m;
  }
  if (lane == 0) {
    const double fm = __longlong_as_double((long long)m);
    int e = 0;
    if (fm > 0.0 && fm <= 1.7976931348623157e308) (void)frexp(fm, &e);
    a.scal[SC_L2] = t;
    a.scal[SC_DRAINED] = d;
    a.scal[SC_FMAX] = fm;
    a.scal[SC_OUT_SCALE] = ldexp(1.0, e);
    a.scal[SC_IN_SCALE] = ldexp(1.0, -e);
  }
  if (a.umiss) {
    // The assembly ran on coefficients scaled by a guessed 2^-eg.  A power of
    // two commutes with every rounding of the double-float arithmetic while the
    // intermediates stay normal and finite, so within a few binades of the
    // exact scale (max |u| < 2^e) the increment is the one the exact scale
    // gives; outside the window, or with a non-finite F, the step is redone.
    unsigned long long mu = 0ull;
    for (int i = lane; i < a.nl2; i += 32) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(a.l2part[3 * a.nl2 + i]);
      mu = b > mu ? b : mu;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_down_sync(0xffffffffu, mu, o);
      mu = ob > mu ? ob : mu;
    }
    if (lane == 0) {
      const double um = __longlong_as_double((long long)mu);
      const double fm = __longlong_as_double((long long)m);
      const int eg = -pow2_exp(a.scal[SC_USCALE]);
      int eu = 0;
      const bool ufin = um <= 1.7976931348623157e308;
      if (um > 0.0 && ufin) (void)frexp(um, &eu);
      const int off = eu - eg;
      const bool miss = !ufin || !(fm <= 1.7976931348623157e308) ||
                        (um > 0.0 && (off > USCALE_WINDOW || off < -USCALE_WINDOW));
      if (miss) *a.umiss = 1;
      a.scal[SC_USCALE] = ldexp(1.0, -eu);
    }
  }
}

// F += shadow contributions, in class order.  One CTA per (y, z) row.  FP64
// adds issue per warp at 1/64 of the FP32 rate whatever the active lanes, so
// the work is arranged to keep warp-level DADDs few: (1) the row's x-slab
// entries (a host-built list of at most 2 per brick boundary) are finished by
// one thread each; (2) if the row lies in a y or z slab, every other entry
// adds the classes of that (row-uniform) zone, one thread per 4 consecutive x
// (32-byte aligned: pitches are multiples of 8).  With g32 set (the mixed heat
// step) every entry of the final F is also written as float(F * 2^-e), the
// FP32 solve's scaled input.  No integer division in the kernel.
__global__ void k_fixup(const FixupArgs a) {
  const Geometry& g = a.g;
  const int Nx = g.N[0], Ny = g.N[1];
  const int y = blockIdx.y, z = blockIdx.z;
  const int zyz = (a.slab[Nx + y] ? 2 : 0) | (a.slab[Nx + Ny + z] ? 4 : 0);
  const size_t rb = (size_t)g.PX * ((size_t)y + (size_t)Ny * z);
  // (1) x-slab entries: zone = 1 | zyz, classes in fixed order
  if ((int)threadIdx.x < a.nxslab) {
    const size_t o = rb + (size_t)a.xslab[threadIdx.x];
    const int zone = 1 | zyz;
    double v = a.F[o];
    for (int cls = 1; cls < 8; ++cls)
      if ((cls & zone) == cls) v += a.shadow[(size_t)(cls - 1) * a.shadow_stride + o];
    a.F[o] = v;
  }
  if (a.g32 == nullptr && zyz == 0) return;
  __syncthreads();  // the x-slab entries are final before the row is read
  const int x0 = 4 * threadIdx.x;
  if (x0 >= (int)g.PX) return;
  const size_t o = rb + (size_t)x0;
  const double2 v01 = *reinterpret_cast<const double2*>(a.F + o);
  const double2 v23 = *reinterpret_cast<const double2*>(a.F + o + 2);
  double v[4] = {v01.x, v01.y, v23.x, v23.y};
  if (zyz != 0) {
    // (2) entries not in an x slab (those are final already): classes of zyz
    bool own[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) own[k] = (x0 + k < Nx) && a.slab[x0 + k] == 0;
#pragma unroll
    for (int cls = 2; cls < 8; cls += 2) {
      if ((cls & zyz) != cls) continue;  // row-uniform
      const double* sh = a.shadow + (size_t)(cls - 1) * a.shadow_stride + o;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (own[k]) v[k] += sh[k];
    }
    *reinterpret_cast<double2*>(a.F + o) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(a.F + o + 2) = make_double2(v[2], v[3]);
  }
  if (a.g32 != nullptr) {
    const int sexp = pow2_exp(a.scal[SC_IN_SCALE]);
    *reinterpret_cast<float4*>(a.g32 + o) =
        make_float4(d2f_scaled(v[0], sexp), d2f_scaled(v[1], sexp), d2f_scaled(v[2], sexp), d2f_scaled(v[3], sexp));
  }
}

template <int P, typename T, bool INCR>
static cudaError_t dispatch_heat(const AssembleArgs& a, const void* tx, const void* ty, const void* tz,
                                 int grid, int* used_grid, cudaStream_t s) {
  const bool hf = a.fqp != nullptr, hk = a.kqp != nullptr;
  if (hf && hk) return launch_one<P, T, ADS_FORM_HEAT, true, true, INCR>(a, tx, ty, tz, grid, used_grid, s);
  if (hf) return launch_one<P, T, ADS_FORM_HEAT, true, false, INCR>(a, tx, ty, tz, grid, used_grid, s);
  if (hk) return launch_one<P, T, ADS_FORM_HEAT, false, true, INCR>(a, tx, ty, tz, grid, used_grid, s);
  return launch_one<P, T, ADS_FORM_HEAT, false, false, INCR>(a, tx, ty, tz, grid, used_grid, s);
}

template <int P>
static cudaError_t dispatch_form(bool fp32, bool incr, const AssembleArgs& a, const void* tx,
                                 const void* ty, const void* tz, int grid, int* used_grid, cudaStream_t s) {
  if (a.form == ADS_FORM_OIL) return launch_assemble_oil(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
  const bool hf = a.fqp != nullptr;
  if (a.form == ADS_FORM_PROJECT) {
    if (fp32)
      return hf ? launch_one<P, float, ADS_FORM_PROJECT, true, false, false>(a, tx, ty, tz, grid, used_grid, s)
                : launch_one<P, float, ADS_FORM_PROJECT, false, false, false>(a, tx, ty, tz, grid, used_grid, s);
    return hf ? launch_one<P, double, ADS_FORM_PROJECT, true, false, false>(a, tx, ty, tz, grid, used_grid, s)
              : launch_one<P, double, ADS_FORM_PROJECT, false, false, false>(a, tx, ty, tz, grid, used_grid, s);
  }
  if (fp32) return incr ? dispatch_heat<P, float, true>(a, tx, ty, tz, grid, used_grid, s)
                        : dispatch_heat<P, float, false>(a, tx, ty, tz, grid, used_grid, s);
  // FP64 increment form: -dt K(kappa) u alone, with a per-point kappa and no
  // source (the tangent model's conductivity term)
  if (incr) {
    if (a.fqp != nullptr || a.kqp == nullptr) return cudaErrorInvalidValue;
    return launch_one<P, double, ADS_FORM_HEAT, false, true, true>(a, tx, ty, tz, grid, used_grid, s);
  }
  return dispatch_heat<P, double, false>(a, tx, ty, tz, grid, used_grid, s);
}

cudaError_t launch_assemble(bool fp32, bool incr, const AssembleArgs& a, const void* tx, const void* ty,
                            const void* tz, int grid, int* used_grid, cudaStream_t s) {
  switch (a.g.P) {
    case 1: return dispatch_form<1>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 2: return dispatch_form<2>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 3: return dispatch_form<3>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 4: return dispatch_form<4>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    default: return cudaErrorInvalidValue;
  }
}

size_t assemble_smem_bytes(int P, bool fp32) {
  switch (P) {
    case 1: return fp32 ? AsmLayout<1, float>::bytes : AsmLayout<1, double>::bytes;
    case 2: return fp32 ? AsmLayout<2, float>::bytes : AsmLayout<2, double>::bytes;
    case 3: return fp32 ? AsmLayout<3, float>::bytes : AsmLayout<3, double>::bytes;
    case 4: return fp32 ? AsmLayout<4, float>::bytes : AsmLayout<4, double>::bytes;
  }
  return 0;
}

cudaError_t launch_fixup(const FixupArgs& a, cudaStream_t s) {
  k_fixup_scale<<<1, 32, 0, s>>>(a);
  const int nq = (int)(a.g.PX / 4);
  const int nthr = std::max(nq, a.nxslab);
  const dim3 grid(1, a.g.N[1], a.g.N[2]);
  k_fixup<<<grid, (nthr + 31) / 32 * 32, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace ads
