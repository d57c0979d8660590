// k_sweep.cu — batched banded LU sweeps (K3) with the 3-D transposes between
// them (K4) fused into the TMA-staged epilogue.
//
// Replaces SolveOneDirection (src/ADS.F90:294-379: one dmumps job=3 call per
// right-hand-side column) and the reorders between the three directions
// (src/reorderRHS.F90:7-93, plus the identity Gather/Scatter copies of
// src/my_mpi.F90:585-702 at one rank).
//
// One warp solves 32 lines ("right-hand sides").  The lines of a tile are
// contiguous in the input layout; TMA loads them into shared memory as boxes
// of SW_CH positions x 32 lines ([chunk][line][pos]).  Lane j solves line j
// with its forward and backward recurrences in registers, lagging j steps
// behind lane 0 (a skewed wavefront), so that at every step the 32 lanes touch
// 32 different shared-memory banks.  The backward pass writes the solution
// transposed, [pos][line], which is exactly the box layout of the NEXT
// direction's array (the lines of this tile become 32 consecutive entries of
// the next layout's contiguous dimension), and TMA stores it there:
//
//   x sweep: L0 (x fastest) -> L1 (y fastest)   = solve + ReorderRHSForY
//   y sweep: L1 (y fastest) -> L2 (z fastest)   = solve + ReorderRHSForZ
//   z sweep: L2 (z fastest) -> L0 (x fastest)   = solve + ReorderRHSForX
//
// Mode 3 skips the solve and is the plain TMA-staged transpose used by
// ads_reorder.  Modes 1 and 2 finish the z sweep with coalesced plain stores
// into the FP64 state (u = s*x, or u += s*x for a refinement correction).
//
// Every wait on the TMA mbarrier is bounded by ~1 s of %globaltimer; on time-out
// the kernel sets an error bit, waits (again bounded) for its copies and returns.
#include "ads_internal.cuh"

#include <algorithm>

namespace ads {

__device__ __forceinline__ unsigned sw_smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(sw_smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sw_smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sw_smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: true on completion, false after ~1 s
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (gtimer_ns() - t0 > 1000000000ull) return false;
  }
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(sw_smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(sw_smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* tm, int c0, int c1, int c2, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                   reinterpret_cast<unsigned long long>(tm)),
               "r"(c0), "r"(c1), "r"(c2), "r"(sw_smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

constexpr int SW_RING = 3;  // output chunks in flight per warp

template <typename TIn, typename TC>
struct SweepSmem {
  __host__ __device__ static size_t s_bytes(int nchunk) { return sizeof(TIn) * (size_t)SW_LANES * SW_CH * nchunk; }
  __host__ __device__ static size_t t_bytes() { return sizeof(TC) * (size_t)SW_LANES * SW_CH * SW_RING; }
  __host__ __device__ static size_t f_bytes(int P, int L) {
    return (sizeof(TC) * (size_t)(2 * P + 2) * L + 15) / 16 * 16;
  }
  __host__ __device__ static size_t total(int P, int L, int nchunk) {
    return 128 + s_bytes(nchunk) + t_bytes() + f_bytes(P, L) + 16;
  }
};

// Position i of line j in the staged input: [chunk][line][pos within chunk].
__device__ __forceinline__ int s_index(int i, int j) {
  return (i / SW_CH) * (SW_LANES * SW_CH) + j * SW_CH + (i % SW_CH);
}

template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}

// One warp per CTA, persistent over tiles of 32 lines.  Shared memory holds
// the staged lines S (the forward pass overwrites them with y in place), a
// ring of SW_RING transposed output chunks, and the factor rows.
template <typename TIn, typename TC, int P, int MODE, bool TRANS>
__global__ void __launch_bounds__(SW_LANES)
    k_sweep(const __grid_constant__ CUtensorMap tmin, const __grid_constant__ CUtensorMap tmout,
            const SweepArgs a) {
  extern __shared__ unsigned char smem_dyn[];
  if (a.skip_flag != nullptr && *a.skip_flag != 0) return;

  const int j = threadIdx.x;
  const int L = a.L;
  const int nchunk = a.nchunk;
  const unsigned base = sw_smem_u32(smem_dyn);
  const unsigned pad = (128u - (base & 127u)) & 127u;
  unsigned char* p0 = smem_dyn + pad;
  TIn* S = reinterpret_cast<TIn*>(p0);
  TC* T = reinterpret_cast<TC*>(p0 + SweepSmem<TIn, TC>::s_bytes(nchunk));
  TC* Fs = reinterpret_cast<TC*>(p0 + SweepSmem<TIn, TC>::s_bytes(nchunk) + SweepSmem<TIn, TC>::t_bytes());
  uint64_t* bar = reinterpret_cast<uint64_t*>(p0 + SweepSmem<TIn, TC>::s_bytes(nchunk) +
                                              SweepSmem<TIn, TC>::t_bytes() + SweepSmem<TIn, TC>::f_bytes(P, L));

  // factor rows -> shared memory, once per CTA
  if (MODE != 3) {
    const TC* fac = static_cast<const TC*>(a.fac);
    for (int idx = j; idx < (2 * P + 2) * L; idx += SW_LANES) Fs[idx] = fac[idx];
  }
  if (j == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncwarp();

  const double isd = (a.in_scale_dev != nullptr) ? *a.in_scale_dev : a.in_scale;
  const bool scaled = (isd != 1.0);
  const TC in_scale = (TC)isd;
  const double osd = (a.out_scale_dev != nullptr) ? *a.out_scale_dev : a.out_scale;

  const int ntiles = a.tiles_lane * ((MODE == 1 || MODE == 2) ? a.out_third_extent : a.third_extent);
  unsigned phase = 0;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int tl = tile % a.tiles_lane;
    const int t3 = tile / a.tiles_lane;
    const int lane_base = tl * SW_LANES;

    // S is rewritten by the async proxy: order the generic accesses of the
    // previous tile before the new load
    fence_proxy_async();
    __syncwarp();
    if (j == 0) {
      mbar_arrive_expect_tx(bar, (unsigned)(nchunk * SW_LANES * SW_CH * sizeof(TIn)));
      const int c1 = (a.lane_dim == 1) ? lane_base : t3;
      const int c2 = (a.lane_dim == 1) ? t3 : lane_base;
      for (int c = 0; c < nchunk; ++c) tma_load_3d(S + c * SW_LANES * SW_CH, &tmin, c * SW_CH, c1, c2, bar);
    }
    if (!mbar_wait_bounded(bar, phase)) {
      if (j == 0) atomicOr(a.err, ERRF_TMA_TIMEOUT);
      (void)mbar_wait_bounded(bar, phase);
      break;
    }
    phase ^= 1u;

    // ---- forward recurrence: y_i = fs_i b_i - sum_m f[m]_i y_{i-m}, in place ----
    if (MODE != 3) {
      TC prev[P];
#pragma unroll
      for (int m = 0; m < P; ++m) prev[m] = TC(0);
      auto fstep = [&](int i) {
        const int si = s_index(i, j);
        TC b = (TC)S[si];
        if (scaled) b *= in_scale;
        TC y = TRANS ? Fs[i] * b : b;
#pragma unroll
        for (int m = P; m >= 2; --m) y -= Fs[m * L + i] * prev[m - 1];
        y -= Fs[L + i] * prev[0];
#pragma unroll
        for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
        prev[0] = y;
        S[si] = (TIn)y;
      };
      const int ramp = SW_LANES - 1;
      for (int s = 0; s < ramp; ++s) {
        const int i = s - j;
        if (i >= 0 && i < L) fstep(i);
      }
#pragma unroll 4
      for (int s = ramp; s < L; ++s) fstep(s - j);
      for (int s = (L > ramp ? L : ramp); s < L + ramp; ++s) {
        const int i = s - j;
        if (i >= 0 && i < L) fstep(i);
      }
    }

    // ---- backward recurrence: x_i = bs_i y_i - sum_m g[m]_i x_{i+m}, written
    //      transposed into the output ring; a chunk leaves as soon as the
    //      slowest lane (31) has passed its lowest position ----
    {
      TC nxt[P];
#pragma unroll
      for (int m = 0; m < P; ++m) nxt[m] = TC(0);
      int next_done = nchunk - 1;    // next chunk to complete
      int next_start = nchunk - 2;   // next chunk lane 0 starts writing (top one starts at s = 0)
      const int steps = L + SW_LANES - 1;
      for (int s = 0; s < steps; ++s) {
        // before lane 0 enters chunk next_start, its ring slot must be free
        if (next_start >= 0 && s == L - (next_start + 1) * SW_CH) {
          if (MODE == 0 || MODE == 3) {
            if (next_start + SW_RING <= nchunk - 1 && j == 0) bulk_wait_read<1>();
          }
          __syncwarp();
          --next_start;
        }
        const int i = L - 1 - (s - j);
        if (i >= 0 && i < L) {
          TC x;
          if (MODE == 3) {
            x = (TC)S[s_index(i, j)];
          } else {
            const TC y = (TC)S[s_index(i, j)];
            x = TRANS ? y : Fs[(P + 1) * L + i] * y;
#pragma unroll
            for (int m = P; m >= 2; --m) x -= Fs[(P + 1 + m) * L + i] * nxt[m - 1];
            x -= Fs[(P + 2) * L + i] * nxt[0];
#pragma unroll
            for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
            nxt[0] = x;
          }
          T[((i / SW_CH) % SW_RING) * (SW_CH * SW_LANES) + (i % SW_CH) * SW_LANES + j] = x;
        }
        // chunk next_done is complete after lane 31 wrote its lowest position
        if (next_done >= 0 && s == L - 1 - next_done * SW_CH + (SW_LANES - 1)) {
          const int c = next_done;
          TC* slot = T + (c % SW_RING) * (SW_CH * SW_LANES);
          if (MODE == 0 || MODE == 3) {
            fence_proxy_async();
            __syncwarp();
            if (j == 0) {
              if (a.out_line_dim == 1) tma_store_3d(&tmout, lane_base, c * SW_CH, t3, slot);
              else tma_store_3d(&tmout, lane_base, t3, c * SW_CH, slot);
              bulk_commit();
            }
          } else {
            __syncwarp();
            // final z sweep: lanes are x, positions are z, t3 is y
            const int x = lane_base + j;
            if (x < a.lanes_total) {
              double* o = a.out + (size_t)x + (size_t)a.out_pitch * (size_t)t3;
              const int r1 = min(SW_CH, L - c * SW_CH);
              for (int r = 0; r < r1; ++r) {
                const double v = osd * (double)slot[r * SW_LANES + j];
                double* d = o + (size_t)a.out_slice * (size_t)(c * SW_CH + r);
                if (MODE == 2) *d += v;
                else *d = v;
              }
            }
            __syncwarp();
          }
          --next_done;
        }
      }
    }
    if (MODE == 0 || MODE == 3) {
      if (j == 0) bulk_wait_read<0>();
    }
    __syncwarp();
  }
  if (MODE == 0 || MODE == 3) {
    if (j == 0) bulk_wait_all();
  }
  __syncwarp();
}

template <typename TIn, typename TC, int P, int MODE, bool TRANS>
static cudaError_t launch_t(const CUtensorMap* tmin, const CUtensorMap* tmout, const SweepArgs& a,
                            int grid, cudaStream_t s) {
  auto kern = k_sweep<TIn, TC, P, MODE, TRANS>;
  const size_t bytes = SweepSmem<TIn, TC>::total(P, a.L, a.nchunk);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  // persistent: as many CTAs as fit at once, each looping over tiles
  int per_sm = 0, dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SW_LANES, bytes);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int g = std::min(grid, nsm * per_sm);
  kern<<<g, SW_LANES, bytes, s>>>(*tmin, *tmout, a);
  return cudaGetLastError();
}

template <int P, int MODE, bool TRANS>
static cudaError_t launch_types(int tin, int tc, const CUtensorMap* tmin, const CUtensorMap* tmout,
                                const SweepArgs& a, int grid, cudaStream_t s) {
  if (tin == 0 && tc == 0) return launch_t<double, double, P, MODE, TRANS>(tmin, tmout, a, grid, s);
  if (tin == 0 && tc == 1) return launch_t<double, float, P, MODE, TRANS>(tmin, tmout, a, grid, s);
  if (tin == 1 && tc == 1) return launch_t<float, float, P, MODE, TRANS>(tmin, tmout, a, grid, s);
  return cudaErrorInvalidValue;
}

template <int P>
static cudaError_t launch_mode(int tin, int tc, int mode, bool trans, const CUtensorMap* tmin,
                               const CUtensorMap* tmout, const SweepArgs& a, int grid, cudaStream_t s) {
  switch (mode) {
    case 0: return trans ? launch_types<P, 0, true>(tin, tc, tmin, tmout, a, grid, s)
                         : launch_types<P, 0, false>(tin, tc, tmin, tmout, a, grid, s);
    case 1: return trans ? launch_types<P, 1, true>(tin, tc, tmin, tmout, a, grid, s)
                         : launch_types<P, 1, false>(tin, tc, tmin, tmout, a, grid, s);
    case 2: return trans ? launch_types<P, 2, true>(tin, tc, tmin, tmout, a, grid, s)
                         : launch_types<P, 2, false>(tin, tc, tmin, tmout, a, grid, s);
    case 3: return launch_types<P, 3, false>(tin, tc, tmin, tmout, a, grid, s);
  }
  return cudaErrorInvalidValue;
}

size_t sweep_smem_bytes(int tin, int tc, int P, int L, int nchunk) {
  if (tin == 0 && tc == 0) return SweepSmem<double, double>::total(P, L, nchunk);
  if (tin == 0 && tc == 1) return SweepSmem<double, float>::total(P, L, nchunk);
  return SweepSmem<float, float>::total(P, L, nchunk);
}

cudaError_t launch_sweep(int P, int tin, int tc, int mode, bool trans, const CUtensorMap* tmin,
                         const CUtensorMap* tmout, const SweepArgs& a, int grid, cudaStream_t s) {
  switch (P) {
    case 1: return launch_mode<1>(tin, tc, mode, trans, tmin, tmout, a, grid, s);
    case 2: return launch_mode<2>(tin, tc, mode, trans, tmin, tmout, a, grid, s);
    case 3: return launch_mode<3>(tin, tc, mode, trans, tmin, tmout, a, grid, s);
    case 4: return launch_mode<4>(tin, tc, mode, trans, tmin, tmout, a, grid, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace ads
