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

template <typename TC, typename TIn>
__device__ __forceinline__ TC load_in(TIn v, int sexp, TC scale) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) return d2f_scaled((double)v, sexp);
  else return (TC)v * scale;
}
// The forward pass keeps y in place of its input.  An FP32 y in an FP64 input
// slot goes into the slot's first word as it is: a float <-> double
// conversion would run on the FP64 pipe (1/64 of the FP32 rate on GB300).
template <typename TC, typename TIn>
__device__ __forceinline__ void store_y(TIn* S, int si, TC y) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) reinterpret_cast<float*>(S + si)[0] = y;
  else S[si] = (TIn)y;
}
template <typename TC, typename TIn>
__device__ __forceinline__ TC load_y(const TIn* S, int si) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) return reinterpret_cast<const float*>(S + si)[0];
  else return (TC)S[si];
}
constexpr int SW_BLK = 8;  // steps per software-pipelined block

// One warp per CTA, persistent over tiles of 32 lines.  Shared memory holds
// the staged lines S (the forward pass overwrites them with y in place), a
// ring of SW_RING transposed output chunks, and the factor rows.  The
// recurrences run in blocks of SW_BLK steps: all loads of a block first,
// then the dependent FMA chain, then the stores.
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
  const int in_exp = pow2_exp(isd);
  const TC in_scale = (TC)isd;
  const double osd = (a.out_scale_dev != nullptr) ? *a.out_scale_dev : a.out_scale;
  const int out_exp = pow2_exp(osd);
  const TC* F1 = Fs + L;               // f[1]
  const TC* BS = Fs + (P + 1) * L;     // bs
  const TC* G1 = Fs + (P + 2) * L;     // g[1]

  const int ntiles = a.tiles_lane * a.third_extent;
  unsigned phase = 0;
  constexpr int RAMP = SW_LANES - 1;

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int tl = tile % a.tiles_lane;
    const int t3 = tile / a.tiles_lane;
    const int lane_base = tl * SW_LANES;

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
        const TC b = load_in<TC>(S[si], in_exp, in_scale);
        TC y = TRANS ? Fs[i] * b : b;
#pragma unroll
        for (int m = P; m >= 2; --m) y -= Fs[m * L + i] * prev[m - 1];
        y -= F1[i] * prev[0];
#pragma unroll
        for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
        prev[0] = y;
        store_y(S, si, y);
      };
      int s = 0;
      for (; s < RAMP && s < L + RAMP; ++s) {
        const int i = s - j;
        if (i >= 0 && i < L) fstep(i);
      }
      // steady state, all lanes active: blocks of SW_BLK steps
      for (; s + SW_BLK <= L; s += SW_BLK) {
        TC bv[SW_BLK], fv[SW_BLK][P + 1];
        int si[SW_BLK];
#pragma unroll
        for (int t = 0; t < SW_BLK; ++t) {
          const int i = s + t - j;
          si[t] = s_index(i, j);
          bv[t] = load_in<TC>(S[si[t]], in_exp, in_scale);
          fv[t][0] = TRANS ? Fs[i] : TC(1);
#pragma unroll
          for (int m = 1; m <= P; ++m) fv[t][m] = Fs[m * L + i];
        }
#pragma unroll
        for (int t = 0; t < SW_BLK; ++t) {
          TC y = TRANS ? fv[t][0] * bv[t] : bv[t];
#pragma unroll
          for (int m = P; m >= 2; --m) y -= fv[t][m] * prev[m - 1];
          y -= fv[t][1] * prev[0];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
          prev[0] = y;
          bv[t] = y;
        }
#pragma unroll
        for (int t = 0; t < SW_BLK; ++t) store_y(S, si[t], bv[t]);
      }
      for (; s < L + RAMP; ++s) {
        const int i = s - j;
        if (i >= 0 && i < L) fstep(i);
      }
    }

    // ---- backward recurrence: x_i = bs_i y_i - sum_m g[m]_i x_{i+m}, written
    //      transposed into the output ring.  Chunk c is complete right after
    //      step L-1-c*CH+31 (lane 31 passes its lowest position); the loop
    //      runs in segments that end exactly at those steps. ----
    {
      TC nxt[P];
#pragma unroll
      for (int m = 0; m < P; ++m) nxt[m] = TC(0);
      auto tslot = [&](int i) -> TC* {
        return T + ((i / SW_CH) % SW_RING) * (SW_CH * SW_LANES) + (i % SW_CH) * SW_LANES + j;
      };
      auto bstep = [&](int i) {
        TC x;
        if (MODE == 3) {
          x = load_in<TC>(S[s_index(i, j)], 0, TC(1));
        } else {
          const TC y = load_y<TC>(S, s_index(i, j));
          x = TRANS ? y : BS[i] * y;
#pragma unroll
          for (int m = P; m >= 2; --m) x -= Fs[(P + 1 + m) * L + i] * nxt[m - 1];
          x -= G1[i] * nxt[0];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
          nxt[0] = x;
        }
        *tslot(i) = x;
      };
      auto run = [&](int sa, int sb) {
        int s = sa;
        const int lo = (sa > RAMP) ? sa : RAMP;  // steady range [lo, hi): every lane in range
        const int hi = (sb < L) ? sb : L;
        for (; s < sb && s < lo; ++s) {
          const int i = L - 1 - (s - j);
          if (i >= 0 && i < L) bstep(i);
        }
        for (; s + SW_BLK <= hi; s += SW_BLK) {
          TC yv[SW_BLK], gv[SW_BLK][P + 1];
#pragma unroll
          for (int t = 0; t < SW_BLK; ++t) {
            const int i = L - 1 - (s + t - j);
            if (MODE == 3) yv[t] = load_in<TC>(S[s_index(i, j)], 0, TC(1));
            else yv[t] = load_y<TC>(S, s_index(i, j));
            if (MODE != 3) {
              gv[t][0] = TRANS ? TC(1) : BS[i];
#pragma unroll
              for (int m = 1; m <= P; ++m) gv[t][m] = Fs[(P + 1 + m) * L + i];
            }
          }
          if (MODE != 3) {
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              TC x = TRANS ? yv[t] : gv[t][0] * yv[t];
#pragma unroll
              for (int m = P; m >= 2; --m) x -= gv[t][m] * nxt[m - 1];
              x -= gv[t][1] * nxt[0];
#pragma unroll
              for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
              nxt[0] = x;
              yv[t] = x;
            }
          }
#pragma unroll
          for (int t = 0; t < SW_BLK; ++t) *tslot(L - 1 - (s + t - j)) = yv[t];
        }
        for (; s < sb; ++s) {
          const int i = L - 1 - (s - j);
          if (i >= 0 && i < L) bstep(i);
        }
      };
      int s = 0;
      for (int c = nchunk - 1; c >= 0; --c) {
        const int se = L - 1 - c * SW_CH + (SW_LANES - 1);
        run(s, se + 1);
        s = se + 1;
        TC* slot = T + (c % SW_RING) * (SW_CH * SW_LANES);
        if (MODE == 0 || MODE == 3) {
          fence_proxy_async();
          __syncwarp();
          if (j == 0) {
            if (a.out_line_dim == 1) tma_store_3d(&tmout, lane_base, c * SW_CH, t3, slot);
            else tma_store_3d(&tmout, lane_base, t3, c * SW_CH, slot);
            bulk_commit();
            // lane 0 enters chunk c-2 (slot of chunk c+1) two steps after the
            // next completion; keep only this chunk's store outstanding
            bulk_wait_read<1>();
          }
          __syncwarp();
        } else {
          __syncwarp();
          // final z sweep: lanes are x, positions are z, t3 is y; rows of 32 x are coalesced
          const int x = lane_base + j;
          if (x < a.lanes_total) {
            double* o = a.out + (size_t)x + (size_t)a.out_pitch * (size_t)t3 + (size_t)a.out_slice * (size_t)(c * SW_CH);
            const int r1 = min(SW_CH, L - c * SW_CH);
            double old[SW_CH];
            if (MODE == 2) {
#pragma unroll
              for (int r = 0; r < SW_CH; ++r)
                if (r < r1) old[r] = o[(size_t)a.out_slice * r];
            }
#pragma unroll
            for (int r = 0; r < SW_CH; ++r) {
              if (r < r1) {
                const double v = f2d_scaled(slot[r * SW_LANES + j], out_exp);
                o[(size_t)a.out_slice * r] = (MODE == 2) ? old[r] + v : v;
              }
            }
          }
          __syncwarp();
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
