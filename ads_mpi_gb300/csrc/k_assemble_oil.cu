// k_assemble_oil.cu — the assembly kernel (K1) instantiated for the oil
// problem's integrand (problems/oil/RHS_eq.F90:69-92):
//   J W (v u + dt (-Kq exp(mu u) grad u . grad v + v (pump - max(0, w u))))
// with Kq, pump and the draining weight w sampled per quadrature point by the
// host.  Kept apart from k_assemble.cu so both compile in parallel.
#include "k_assemble.cuh"

namespace ads {

template <int P>
static cudaError_t dispatch_oil(bool fp32, bool incr, const AssembleArgs& a, const void* tx, const void* ty,
                                const void* tz, int grid, int* used_grid, cudaStream_t s) {
  if (fp32)
    return incr ? launch_one<P, float, ADS_FORM_OIL, true, true, true>(a, tx, ty, tz, grid, used_grid, s)
                : launch_one<P, float, ADS_FORM_OIL, true, true, false>(a, tx, ty, tz, grid, used_grid, s);
  return launch_one<P, double, ADS_FORM_OIL, true, true, false>(a, tx, ty, tz, grid, used_grid, s);
}

cudaError_t launch_assemble_oil(bool fp32, bool incr, const AssembleArgs& a, const void* tx, const void* ty,
                                const void* tz, int grid, int* used_grid, cudaStream_t s) {
  if (a.fqp == nullptr || a.kqp == nullptr || a.dqp == nullptr) return cudaErrorInvalidValue;
  switch (a.g.P) {
    case 1: return dispatch_oil<1>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 2: return dispatch_oil<2>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 3: return dispatch_oil<3>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    case 4: return dispatch_oil<4>(fp32, incr, a, tx, ty, tz, grid, used_grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ads
