// noalloc.cu — ads_residual_noalloc: the mass-matrix residual of a handle for
// callers that must not allocate device memory.
//
// Which callers cannot allocate, and why: a host program that hands out all of
// its device memory up front through its own pool (every byte it may touch is
// reserved before the time loop starts, so a library that calls cudaMalloc
// breaks its budget), and a program that keeps other streams busy while it
// calls in (cudaFree synchronises the whole device and would stall them).
// This entry point works on the caller's device arrays.  Its only working
// storage — one partial sum triple per CTA of the residual kernel and the
// three reduced values — is the file-scope array below, of a fixed size that
// every GPU loading the library holds until the process exits.  It calls no
// cudaMalloc, cudaFree or allocating library routine.
//
// The array is shared by every call on every handle of a device and keeps the
// last call's contents.  Calls whose kernels overlap on the GPU (two host
// threads, or two handles on different streams of the same device) race on it:
// serialise them on one stream or with events.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address once (cudaGetSymbolAddress; this also loads the
// module holding the array if it is not loaded yet).  Make that first call
// before any stream capture.  The address is kept per device ordinal for the
// life of the process: do not use this entry point on a device after a
// cudaDeviceReset of it (the kept address would belong to the destroyed
// context).
#include <cuda_runtime.h>

#include <mutex>

#include "ads_internal.cuh"

namespace {

// largest residual grid the scratch covers: one CTA per tile of 32 x 8 x 32
// DOFs, ceil(Nx/32) * ceil(Ny/8) * ceil(Nz/32) <= 8192 (the largest cube is
// 384^3 DOFs: 12 * 48 * 12 = 6912 tiles; 385^3 needs 13 * 49 * 13 = 8281)
constexpr int kMaxCtas = ADS_NOALLOC_MAX_CTAS;
constexpr int kResultOffset = 3 * kMaxCtas;          // [rr, ff, rmax] after the partials
constexpr int kScratchDoubles = 3 * kMaxCtas + 8;    // 196,672 bytes

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// the device address of the scratch array on the current device (set up once)
cudaError_t scratch_for_device(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

// fixed-order reduction of the residual kernel's per-CTA partials into
// out = [sum rr, sum ff, max rmax]; every value read was written by the same
// call's residual kernel, so nothing has to be cleared beforehand
__global__ void __launch_bounds__(256) k_noalloc_reduce(const double* part, int n, double* out) {
  __shared__ double s0[256], s1[256];
  __shared__ unsigned long long s2[256];
  double rr = 0.0, ff = 0.0;
  unsigned long long m = 0ull;  // max of non-negative doubles, compared as bits
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    rr += part[3 * i];
    ff += part[3 * i + 1];
    const unsigned long long b = (unsigned long long)__double_as_longlong(part[3 * i + 2]);
    m = b > m ? b : m;
  }
  s0[threadIdx.x] = rr;
  s1[threadIdx.x] = ff;
  s2[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s0[threadIdx.x] += s0[threadIdx.x + w];
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] = s2[threadIdx.x + w] > s2[threadIdx.x] ? s2[threadIdx.x + w] : s2[threadIdx.x];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s0[0];
    out[1] = s1[0];
    out[2] = __longlong_as_double((long long)s2[0]);
  }
}

}  // namespace

extern "C" int ads_residual_noalloc(ads_handle* h, const double* d_F, const double* d_u, double* d_r,
                                    double norms[3]) {
  if (!h || !d_u || !d_r) return ADS_ERR_ARG;
  ads::NoallocView v;
  ads::handle_noalloc_view(h, &v);
  if (v.general)
    return ads::handle_fail(h, ADS_ERR_UNSUPPORTED, "ads_residual_noalloc needs equal degrees on all axes");
  cudaError_t e = cudaSetDevice(v.dev);
  if (e != cudaSuccess) return ads::handle_cuda_fail(h, e, "ads_residual_noalloc: cudaSetDevice");
  if (v.grid > kMaxCtas)
    return ads::handle_fail(h, ADS_ERR_ARG,
                            "ads_residual_noalloc: the residual needs " + std::to_string(v.grid) +
                                " CTAs (tiles of 32x8x32 DOFs) but its fixed scratch holds " +
                                std::to_string(kMaxCtas) + "; use ads_apply_mass for this size");
  double* scratch = nullptr;
  if ((e = scratch_for_device(v.dev, &scratch)) != cudaSuccess)
    return ads::handle_cuda_fail(h, e, "ads_residual_noalloc: cudaGetSymbolAddress");

  ads::ResidualArgs a = v.args;  // dense x-fastest layout of the caller's arrays
  a.u = d_u;
  a.F = d_F;
  a.r = d_r;
  a.part = scratch;
  a.skip_flag = nullptr;
  a.want_ff = d_F != nullptr ? 1 : 0;
  if ((e = ads::launch_residual(v.P, a, v.grid, v.stream)) != cudaSuccess)
    return ads::handle_cuda_fail(h, e, "ads_residual_noalloc: residual");
  k_noalloc_reduce<<<1, 256, 0, v.stream>>>(scratch, v.grid, scratch + kResultOffset);
  if ((e = cudaGetLastError()) != cudaSuccess) return ads::handle_cuda_fail(h, e, "ads_residual_noalloc: reduce");
  *v.launches += 2;
  if (norms != nullptr) {
    if ((e = cudaMemcpyAsync(norms, scratch + kResultOffset, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                             v.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(v.stream)) != cudaSuccess)
      return ads::handle_cuda_fail(h, e, "ads_residual_noalloc: reading the norms");
  }
  return ADS_OK;
}
