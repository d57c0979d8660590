// k_sweep.cu — batched banded LU sweeps (K3) with the 3-D transposes between
// them (K4) fused into the TMA-staged epilogue.
//
// Replaces SolveOneDirection (src/ADS.F90:294-379: one dmumps job=3 call per
// right-hand-side column) and the reorders between the three directions
// (src/reorderRHS.F90:7-93, plus the identity Gather/Scatter copies of
// src/my_mpi.F90:585-702 at one rank).
//
// One warp solves 32 lines ("right-hand sides").  The lines of a tile are
// contiguous in the input layout; 16-byte cp.async copies stage them in shared
// memory line-major, S[line][pos] with an even row stride LS, in four position
// groups so the forward pass starts while the rest is still arriving.  Lane j
// solves line j with its forward and backward recurrences in registers,
// lagging j steps behind lane 0 (a skewed wavefront): with LS even the 32
// lanes then touch 32 different banks at every step, and every address of a
// step is a fixed offset from a per-lane pointer.  The backward pass writes the
// solution transposed, [pos][line], into a ring of four 32-position chunks,
// which is exactly the box layout of the NEXT direction's array (the lines of
// this tile become 32 consecutive entries of the next layout's contiguous
// dimension), and TMA stores each chunk there as soon as it is complete:
//
//   x sweep: L0 (x fastest) -> L1 (y fastest)   = solve + ReorderRHSForY
//   y sweep: L1 (y fastest) -> L2 (z fastest)   = solve + ReorderRHSForZ
//   z sweep: L2 (z fastest) -> L0 (x fastest)   = solve + ReorderRHSForX
//
// Mode 3 skips the solve and is the plain staged transpose used by
// ads_reorder.  Mode 4 solves without the transpose: the chunks keep the
// positions contiguous and go back into the input's layout (the mixed step's
// FP32 x sweep, L0 -> L0, whose y and z sweeps then run in column form).
// No wait in this kernel spins: cp.async and bulk-group waits complete in
// hardware.
#include "ads_internal.cuh"

#include <algorithm>

namespace ads {

__device__ __forceinline__ unsigned sw_smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* tm, int c0, int c1, int c2, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                   reinterpret_cast<unsigned long long>(tm)),
               "r"(c0), "r"(c1), "r"(c2), "r"(sw_smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// 16-byte global -> shared copy (L2 only: the tile is read once)
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sw_smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit_group() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int SW_RING = 4;       // transposed output chunks per warp (power of two)
constexpr int SW_GROUPS = 4;     // position groups of the staged input
constexpr int SW_BLK = 32;       // steps per software-pipelined block

// The factors of one position packed for one vector load per step: forward
// (f1..fP) in KF entries, backward (bs, g1..gP) in KB entries (powers of two),
// plus the forward scales fs as a row of their own (transposed solve only).
__host__ __device__ constexpr int sw_kf(int P) { return P <= 1 ? 1 : (P <= 2 ? 2 : 4); }
__host__ __device__ constexpr int sw_kb(int P) { return P + 1 <= 2 ? 2 : (P + 1 <= 4 ? 4 : 8); }

// Shared memory of one CTA (one warp): staged lines S[32][LS] (TIn), the
// output ring T[SW_RING * 32 positions][32 lines] (TC), the packed factors
// (KF + KB + 1 entries per position, TC).  LS = L rounded up to a multiple of
// 4: even (so the skewed accesses are conflict-free) and a whole number of
// 16-byte copies.
template <typename TIn, typename TC>
struct SweepSmem {
  __host__ __device__ static int ls(int L) { return (L + 3) / 4 * 4; }
  __host__ __device__ static size_t s_bytes(int L) { return sizeof(TIn) * (size_t)SW_LANES * ls(L); }
  __host__ __device__ static size_t t_bytes() { return sizeof(TC) * (size_t)SW_LANES * SW_CH * SW_RING; }
  // forward vectors, then backward vectors (16-byte aligned), then fs
  __host__ __device__ static size_t fw_bytes(int P, int L) {
    return (sizeof(TC) * (size_t)sw_kf(P) * L + 15) / 16 * 16;
  }
  __host__ __device__ static size_t bw_bytes(int P, int L) {
    return (sizeof(TC) * (size_t)sw_kb(P) * L + 15) / 16 * 16;
  }
  __host__ __device__ static size_t f_bytes(int P, int L, bool trans) {
    return fw_bytes(P, L) + bw_bytes(P, L) + (trans ? (sizeof(TC) * (size_t)L + 15) / 16 * 16 : 0);
  }
  __host__ __device__ static size_t total(int P, int L, bool trans) {
    return 128 + s_bytes(L) + t_bytes() + f_bytes(P, L, trans);
  }
};

// K consecutive entries as one or more 8/16-byte loads (p aligned to their size)
template <typename TC, int K>
__device__ __forceinline__ void sw_ldk(const TC* p, TC (&v)[K]) {
  constexpr int B = (int)sizeof(TC) * K;
  if constexpr (B == 4) {
    v[0] = p[0];
  } else if constexpr (B == 8) {
    if constexpr (sizeof(TC) == 4) {
      const float2 t = *reinterpret_cast<const float2*>(p);
      v[0] = t.x; v[1] = t.y;
    } else {
      v[0] = p[0];
    }
  } else {
#pragma unroll
    for (int h = 0; h < B / 16; ++h) {
      if constexpr (sizeof(TC) == 4) {
        const float4 t = reinterpret_cast<const float4*>(p)[h];
        v[4 * h] = t.x; v[4 * h + 1] = t.y; v[4 * h + 2] = t.z; v[4 * h + 3] = t.w;
      } else {
        const double2 t = reinterpret_cast<const double2*>(p)[h];
        v[2 * h] = t.x; v[2 * h + 1] = t.y;
      }
    }
  }
}

// An input of the compute type is used as it is (launch_sweep rejects an
// input scale for it); an FP64 input of an FP32 solve is scaled by 2^sexp.
template <typename TC, typename TIn>
__device__ __forceinline__ TC load_in(TIn v, int sexp, TC scale) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) return d2f_scaled((double)v, sexp);
  else return (TC)v;
}
// The forward pass keeps y in place of its input.  An FP32 y in an FP64 input
// slot goes into the slot's first word as it is: a float <-> double
// conversion would run on the FP64 pipe (1/64 of the FP32 rate on GB300).
template <typename TC, typename TIn>
__device__ __forceinline__ void store_y(TIn* p, TC y) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) reinterpret_cast<float*>(p)[0] = y;
  else *p = (TIn)y;
}
template <typename TC, typename TIn>
__device__ __forceinline__ TC load_y(const TIn* p) {
  if constexpr (sizeof(TIn) == 8 && sizeof(TC) == 4) return reinterpret_cast<const float*>(p)[0];
  else return (TC)*p;
}

// Slot of position i of lane j in the output ring.  Modes 0 and 3 write the
// chunk transposed, [position][line] (the lines become the next layout's
// contiguous dimension); mode 4 solves like mode 0 but keeps the positions
// contiguous, [line][position], for an output in the input's own layout.
template <int MODE>
__device__ __forceinline__ int sw_tidx(int i, int j) {
  constexpr int RMASK = SW_RING * SW_CH - 1;
  if constexpr (MODE == 4) return ((i & RMASK) & ~(SW_CH - 1)) * SW_LANES + j * SW_CH + (i & (SW_CH - 1));
  else return ((i & RMASK) << 5) + j;
}

// One warp per CTA, persistent over tiles of 32 lines.  The recurrences run in
// blocks of SW_BLK steps once every lane is inside its line: all loads of a
// block first, then the dependent FMA chain, then the stores.
template <typename TIn, typename TC, int P, int MODE, bool TRANS>
__global__ void __launch_bounds__(SW_LANES)
    k_sweep(const __grid_constant__ CUtensorMap tmout, const SweepArgs a) {
  extern __shared__ unsigned char smem_dyn[];
  if (a.skip_flag != nullptr && *a.skip_flag != 0) return;

  using SM = SweepSmem<TIn, TC>;
  const int j = threadIdx.x;
  const int L = a.L;
  const int LS = SM::ls(L);
  const int nchunk = (L + SW_CH - 1) / SW_CH;
  const unsigned base = sw_smem_u32(smem_dyn);
  const unsigned pad = (128u - (base & 127u)) & 127u;
  unsigned char* p0 = smem_dyn + pad;
  TIn* S = reinterpret_cast<TIn*>(p0);
  TC* T = reinterpret_cast<TC*>(p0 + SM::s_bytes(L));
  constexpr int KF = sw_kf(P), KB = sw_kb(P);
  TC* FW = reinterpret_cast<TC*>(p0 + SM::s_bytes(L) + SM::t_bytes());  // [L][KF]: f1..fP
  TC* BW = reinterpret_cast<TC*>(reinterpret_cast<unsigned char*>(FW) + SM::fw_bytes(P, L));  // [L][KB]: bs, g
  TC* FS = reinterpret_cast<TC*>(reinterpret_cast<unsigned char*>(BW) + SM::bw_bytes(P, L));  // [L]: fs (TRANS)

  if (MODE != 3) {
    // factor rows (global [row][L]): 0 fs, 1..P f, P+1 bs, P+2..2P+1 g
    const TC* fac = static_cast<const TC*>(a.fac);
    for (int i = j; i < L; i += SW_LANES) {
#pragma unroll
      for (int m = 0; m < KF; ++m) FW[(size_t)i * KF + m] = (m < P) ? fac[(size_t)(1 + m) * L + i] : TC(0);
#pragma unroll
      for (int m = 0; m < KB; ++m) BW[(size_t)i * KB + m] = (m <= P) ? fac[(size_t)(P + 1 + m) * L + i] : TC(0);
      if (TRANS) FS[i] = fac[i];
    }
  }
  __syncwarp();

  const double isd = (a.in_scale_dev != nullptr) ? *a.in_scale_dev : a.in_scale;
  const int in_exp = pow2_exp(isd);
  const TC in_scale = (TC)isd;

  constexpr int V = 16 / (int)sizeof(TIn);          // elements per 16-byte copy
  const int nv = LS / V;                             // copies per line
  constexpr int GA = SW_BLK / V;                    // group sizes in whole blocks of steps
  const int gcp = ((nv + SW_GROUPS - 1) / SW_GROUPS + GA - 1) / GA * GA;  // copies per line and group
  const int GP = gcp * V;                            // positions per group
  const TIn* in = static_cast<const TIn*>(a.in);
  const int ntiles = a.tiles_lane * a.third_extent;
  constexpr int RAMP = SW_LANES - 1;
  TIn* const Sj = S + (size_t)j * LS;  // this lane's line

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int tl = tile % a.tiles_lane;
    const int t3 = tile / a.tiles_lane;
    const int lane_base = tl * SW_LANES;
    const int nl = min(SW_LANES, a.lanes_total - lane_base);
    const TIn* src = in + (size_t)t3 * a.in_t3s + (size_t)lane_base * a.in_ls;

    // ---- stage the tile: group g holds positions [g*GP, (g+1)*GP) of every line ----
    __syncwarp();  // the previous tile's backward pass is done with S
#pragma unroll 1
    for (int g = 0; g < SW_GROUPS; ++g) {
      const int k0 = g * gcp;
      const int kc = min(gcp, nv - k0);
      if (kc > 0) {
        const int q = SW_LANES / kc, r = SW_LANES % kc;
        int l = j / kc, k = j % kc;
        while (l < nl) {
          cp_async16(S + (size_t)l * LS + (size_t)(k0 + k) * V, src + (size_t)l * a.in_ls + (size_t)(k0 + k) * V);
          k += r;
          l += q;
          if (k >= kc) { k -= kc; ++l; }
        }
      }
      cp_async_commit_group();
    }

    // ---- forward recurrence: y_i = fs_i b_i - sum_m f[m]_i y_{i-m}, in place ----
    if (MODE != 3) {
      TC prev[P];
#pragma unroll
      for (int m = 0; m < P; ++m) prev[m] = TC(0);
      auto fstep = [&](int i) {
        TIn* yp = Sj + i;
        const TC b = load_in<TC>(*yp, in_exp, in_scale);
        TC f[KF];
        sw_ldk<TC, KF>(FW + (size_t)i * KF, f);
        TC y = TRANS ? FS[i] * b : b;
#pragma unroll
        for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
#pragma unroll
        for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
        prev[0] = y;
        store_y(yp, y);
      };
      int s = 0;
#pragma unroll 1
      for (int g = 0; g < SW_GROUPS; ++g) {
        // lane 0 reaches group g at step g*GP; the other lanes later
        switch (g) {
          case 0: cp_async_wait_group<SW_GROUPS - 1>(); break;
          case 1: cp_async_wait_group<SW_GROUPS - 2>(); break;
          case 2: cp_async_wait_group<SW_GROUPS - 3>(); break;
          default: cp_async_wait_group<0>(); break;
        }
        __syncwarp();
        const int sb = (g == SW_GROUPS - 1) ? L + RAMP : min((g + 1) * GP, L + RAMP);
        const int sbl = min(sb, L);
        while (s < sb) {
          if (s >= RAMP && s + SW_BLK <= sbl) {
            const int i0 = s - j;
            TIn* yp = Sj + i0;
            TC bv[SW_BLK], fv[SW_BLK][KF], fsv[SW_BLK];
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              bv[t] = load_in<TC>(yp[t], in_exp, in_scale);
              sw_ldk<TC, KF>(FW + (size_t)(i0 + t) * KF, fv[t]);
              fsv[t] = TRANS ? FS[i0 + t] : TC(1);
            }
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              TC y = TRANS ? fsv[t] * bv[t] : bv[t];
#pragma unroll
              for (int m = P; m >= 1; --m) y -= fv[t][m - 1] * prev[m - 1];
#pragma unroll
              for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
              prev[0] = y;
              bv[t] = y;
            }
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) store_y(yp + t, bv[t]);
            s += SW_BLK;
          } else if (s + SW_BLK <= sb) {
            // ramp block: lanes outside their line read a clamped position,
            // keep y = 0 (so the recurrence starts from zero) and store nothing
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              const int i = s + t - j;
              const bool act = (i >= 0) && (i < L);
              const int ic = min(max(i, 0), L - 1);
              const TC b = load_in<TC>(Sj[ic], in_exp, in_scale);
              TC f[KF];
              sw_ldk<TC, KF>(FW + (size_t)ic * KF, f);
              TC y = TRANS ? FS[ic] * b : b;
#pragma unroll
              for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
              y = act ? y : TC(0);
#pragma unroll
              for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
              prev[0] = y;
              if (act) store_y(Sj + ic, y);
            }
            s += SW_BLK;
          } else {
            const int i = s - j;
            if (i >= 0 && i < L) fstep(i);
            ++s;
          }
        }
      }
    } else {
      cp_async_wait_group<0>();
      __syncwarp();
    }

    // ---- backward recurrence: x_i = bs_i y_i - sum_m g[m]_i x_{i+m}, written
    //      transposed into the output ring (row i mod 128).  Chunk c is
    //      complete right after step L-1-c*CH+31 (lane 31 passes its lowest
    //      position); the loop runs in segments that end at those steps. ----
    if (j == 0) bulk_wait_read<0>();  // the previous tile's stores are done reading the ring
    __syncwarp();
    {
      TC nxt[P];
#pragma unroll
      for (int m = 0; m < P; ++m) nxt[m] = TC(0);
      auto bstep = [&](int i) {
        TC x;
        if (MODE == 3) {
          x = load_in<TC>(Sj[i], 0, TC(1));
        } else {
          const TC y = load_y<TC>(Sj + i);
          TC gb[KB];
          sw_ldk<TC, KB>(BW + (size_t)i * KB, gb);
          x = TRANS ? y : gb[0] * y;
#pragma unroll
          for (int m = P; m >= 1; --m) x -= gb[m] * nxt[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
          nxt[0] = x;
        }
        T[sw_tidx<MODE>(i, j)] = x;
      };
      int s = 0;
      for (int c = nchunk - 1; c >= 0; --c) {
        const int se = L - 1 - c * SW_CH + RAMP;  // last step of chunk c
        const int sb = se + 1;
        const int sbl = min(sb, L);
        while (s < sb) {
          if (s >= RAMP && s + SW_BLK <= sbl) {
            const int i0 = L - 1 - (s - j);
            const TIn* yp = Sj + i0;
            TC yv[SW_BLK];
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              if (MODE == 3) yv[t] = load_in<TC>(yp[-t], 0, TC(1));
              else yv[t] = load_y<TC>(yp - t);
            }
            if (MODE != 3) {
              TC gv[SW_BLK][KB];
#pragma unroll
              for (int t = 0; t < SW_BLK; ++t) sw_ldk<TC, KB>(BW + (size_t)(i0 - t) * KB, gv[t]);
#pragma unroll
              for (int t = 0; t < SW_BLK; ++t) {
                TC x = TRANS ? yv[t] : gv[t][0] * yv[t];
#pragma unroll
                for (int m = P; m >= 1; --m) x -= gv[t][m] * nxt[m - 1];
#pragma unroll
                for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
                nxt[0] = x;
                yv[t] = x;
              }
            }
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) T[sw_tidx<MODE>(i0 - t, j)] = yv[t];
            s += SW_BLK;
          } else if (s + SW_BLK <= sb) {
            // ramp block: lanes outside their line read a clamped position,
            // keep x = 0 and store nothing (the ring slots of other chunks
            // may still be read by their stores)
#pragma unroll
            for (int t = 0; t < SW_BLK; ++t) {
              const int i = L - 1 - (s + t - j);
              const bool act = (i >= 0) && (i < L);
              const int ic = min(max(i, 0), L - 1);
              TC x;
              if (MODE == 3) {
                x = load_in<TC>(Sj[ic], 0, TC(1));
              } else {
                const TC y = load_y<TC>(Sj + ic);
                TC gb[KB];
                sw_ldk<TC, KB>(BW + (size_t)ic * KB, gb);
                x = TRANS ? y : gb[0] * y;
#pragma unroll
                for (int m = P; m >= 1; --m) x -= gb[m] * nxt[m - 1];
                x = act ? x : TC(0);
#pragma unroll
                for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
                nxt[0] = x;
              }
              if (act) T[sw_tidx<MODE>(ic, j)] = x;
            }
            s += SW_BLK;
          } else {
            const int i = L - 1 - (s - j);
            if (i >= 0 && i < L) bstep(i);
            ++s;
          }
        }
        TC* slot = T + (c & (SW_RING - 1)) * (SW_CH * SW_LANES);
        fence_proxy_async();
        __syncwarp();
        if (j == 0) {
          if (MODE == 4) tma_store_3d(&tmout, c * SW_CH, lane_base, t3, slot);
          else if (a.out_line_dim == 1) tma_store_3d(&tmout, lane_base, c * SW_CH, t3, slot);
          else tma_store_3d(&tmout, lane_base, t3, c * SW_CH, slot);
          bulk_commit();
          // lane 0 enters chunk c-2 two steps after this event; its slot was
          // last stored from for chunk c+2, two commits ago
          bulk_wait_read<SW_RING - 2>();
        }
        __syncwarp();
      }
    }
  }
  if (j == 0) bulk_wait_all();
  __syncwarp();
}

template <typename TIn, typename TC, int P, int MODE, bool TRANS>
static cudaError_t launch_t(const CUtensorMap* tmout, const SweepArgs& a, int grid, cudaStream_t s) {
  auto kern = k_sweep<TIn, TC, P, MODE, TRANS>;
  const size_t bytes = SweepSmem<TIn, TC>::total(P, a.L, TRANS);
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
  kern<<<g, SW_LANES, bytes, s>>>(*tmout, a);
  return cudaGetLastError();
}

// The combinations the solves use: modes 0 and 3 in FP64 (the FP64 solves,
// the adjoint's transposed solve, ads_reorder), mode 4 from FP64 or FP32 input
// in FP32 (the mixed step's x sweep).
template <int P>
static cudaError_t launch_mode(int tin, int tc, int mode, bool trans, const CUtensorMap* tmout,
                               const SweepArgs& a, int grid, cudaStream_t s) {
  switch (mode) {
    case 0:
      if (tin != 0 || tc != 0) return cudaErrorInvalidValue;
      if (trans) return launch_t<double, double, P, 0, true>(tmout, a, grid, s);
      return launch_t<double, double, P, 0, false>(tmout, a, grid, s);
    case 3:
      if (tin != 0 || tc != 0) return cudaErrorInvalidValue;
      return launch_t<double, double, P, 3, false>(tmout, a, grid, s);
    case 4:  // FP32 solve, output in the input's layout
      if (trans) return cudaErrorInvalidValue;
      if (tin == 0 && tc == 1) return launch_t<double, float, P, 4, false>(tmout, a, grid, s);
      if (tin == 1 && tc == 1) return launch_t<float, float, P, 4, false>(tmout, a, grid, s);
      return cudaErrorInvalidValue;
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep(int P, int tin, int tc, int mode, bool trans, const CUtensorMap* tmout,
                         const SweepArgs& a, int grid, cudaStream_t s) {
  if (a.in == nullptr) return cudaErrorInvalidValue;
  if (tin == tc && (a.in_scale != 1.0 || a.in_scale_dev != nullptr)) return cudaErrorInvalidValue;
  switch (P) {
    case 1: return launch_mode<1>(tin, tc, mode, trans, tmout, a, grid, s);
    case 2: return launch_mode<2>(tin, tc, mode, trans, tmout, a, grid, s);
    case 3: return launch_mode<3>(tin, tc, mode, trans, tmout, a, grid, s);
    case 4: return launch_mode<4>(tin, tc, mode, trans, tmout, a, grid, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace ads
