// k_csweep.cu — the FP32 y and z sweeps of the mixed step in column form.
//
// Replaces SolveOneDirection (src/ADS.F90:294-379) along y and z, and the
// reorders between the directions (src/reorderRHS.F90:7-93), for the FP32
// solves: both sweeps read and write the x-fastest layout L0, the y sweep in
// place.  In L0 the lines of a y or z tile are contiguous: 32 consecutive x
// form a 128-byte row at every position.  One warp solves 32 lines with the
// lanes ACROSS the lines: at every step all 32 lanes are at the same
// position, so
//   * the tile is staged position-major by 16-byte copies, S[pos][line] in
//     128-byte rows: a row of 32 lanes hits 32 different banks;
//   * the last blocks of every line skip shared memory: their rows are loaded
//     straight into registers, which also keep their forward results;
//   * the LU factors of a position are the same for every lane: one
//     broadcast vector load per step from a per-CTA table;
//   * there is no wavefront skew, so no ramp steps;
//   * each block of solution rows (32 consecutive x) is stored straight to
//     global memory, coalesced, during the backward pass: FP32, or the FP64
//     state 2^e x.
// (The x sweep reads lines whose positions are contiguous; staging those
// position-major would take 4-byte transposing copies, so k_xsweep below
// stages them line-major instead.)  A CTA holds as many warps
// (tiles) as shared memory allows next to one copy of the factor tables;
// warps loop over tiles on their own.  No wait spins: cp.async groups
// complete in hardware.
#include "ads_internal.cuh"

#include <algorithm>
#include <type_traits>

namespace ads {

constexpr int CS_BLK = 16;        // steps per software-pipelined block
constexpr int CS_GROUPS = 4;      // position groups of the staged input
constexpr int CS_MAX_WARPS = 8;
constexpr int CS_TAIL_BLKS = 3;   // blocks at the end of a line held in registers
constexpr int CS_SROW = 32;       // floats per staged row: 128 bytes, 32 lanes on 32 banks

__device__ __forceinline__ unsigned cs_smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cs_cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(cs_smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cs_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// bytes (a multiple of 16) from a 16-byte aligned global address into L2
__device__ __forceinline__ void cs_prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(__cvta_generic_to_global(p)), "r"(bytes)
               : "memory");
}
template <int N>
__device__ __forceinline__ void cs_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// factor table of one position: forward f[1..P] in VF float4, backward
// (bs, g[1..P]) in VB float4
template <int P>
struct CsTab {
  static constexpr int VF = (P + 3) / 4;
  static constexpr int VB = (P + 1 + 3) / 4;
  __host__ __device__ static size_t bytes(int L) { return sizeof(float4) * (size_t)(VF + VB) * L; }
};

// The last cs_tail_blocks(L) blocks of every line never touch shared memory:
// their input rows are loaded into registers at the start of the tile, and
// their forward results stay there for the backward pass.  The rest, Ls
// positions, is staged.
__host__ __device__ inline int cs_tail_blocks(int L) {
  return (L / CS_BLK < CS_TAIL_BLKS) ? L / CS_BLK : CS_TAIL_BLKS;
}
size_t csweep_warp_bytes(int L) {
  return sizeof(float) * (size_t)(L - CS_BLK * cs_tail_blocks(L)) * CS_SROW;
}

// A block of 16 solution rows (rows i0 .. i0 + 15 of this lane's line) out:
// FP32 as it is, or the FP64 state 2^e x.  The row pointer steps by the
// pitch, one 64-bit add per row.  In FP64 the conversion takes the integer
// fast path for the whole block (normal floats and zeros; `hi_add` holds
// (896 + e) << 20 for the exponent, valid for |e| <= 896) and falls back to
// f2d_scaled for every row if any value is subnormal, infinite or NaN.
template <int MODE>
__device__ __forceinline__ void cs_store_block(void* out, size_t i0, size_t ops, const float (&v)[CS_BLK],
                                               int out_exp, bool fast_ok, unsigned hi_add) {
  if constexpr (MODE == 1) {
    double* q = static_cast<double*>(out) + i0 * ops;
    double d[CS_BLK];
    bool rare = !fast_ok;
#pragma unroll
    for (int t = 0; t < CS_BLK; ++t) {
      const unsigned b = __float_as_uint(v[t]);
      const unsigned m = b & 0x7fffffffu;
      rare |= (m - 0x00800000u >= 0x7f000000u) && m != 0u;  // subnormal, inf or NaN
      const unsigned hi = (m == 0u ? 0u : (m >> 3) + hi_add) | (b & 0x80000000u);
      d[t] = __hiloint2double((int)hi, (int)(b << 29));
    }
    if (rare) {
#pragma unroll
      for (int t = 0; t < CS_BLK; ++t) d[t] = f2d_scaled(v[t], out_exp);
    }
#pragma unroll
    for (int t = 0; t < CS_BLK; ++t) {
      *q = d[t];
      q += ops;
    }
  } else {
    float* q = static_cast<float*>(out) + i0 * ops;
#pragma unroll
    for (int t = 0; t < CS_BLK; ++t) {
      *q = v[t];
      q += ops;
    }
  }
}

template <int P, int MODE>
__global__ void __launch_bounds__(CS_MAX_WARPS * 32) k_csweep(const CSweepArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (a.skip_flag != nullptr && *a.skip_flag != 0) return;
  using Tab = CsTab<P>;
  constexpr int VF = Tab::VF, VB = Tab::VB;
  constexpr int NTB = CS_TAIL_BLKS;
  const int L = a.L;
  const int nt = cs_tail_blocks(L);
  const int Ls = L - CS_BLK * nt;  // staged positions [0, Ls); the tail [Ls, L) is in registers
  const int j = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  constexpr int srow = CS_SROW;
  float4* FT = reinterpret_cast<float4*>(smem);      // [L][VF]
  float4* BT = FT + (size_t)VF * L;                  // [L][VB]
  float* S = reinterpret_cast<float*>(smem + Tab::bytes(L)) + (size_t)warp * Ls * srow;

  // factor rows (global [row][L]): row 0 fs (1 here), 1..P f, P+1 bs, P+2.. g
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    float fw[4 * VF], bw[4 * VB];
#pragma unroll
    for (int m = 0; m < 4 * VF; ++m) fw[m] = (m < P) ? a.fac[(size_t)(1 + m) * L + i] : 0.f;
#pragma unroll
    for (int m = 0; m < 4 * VB; ++m) bw[m] = (m <= P) ? a.fac[(size_t)(P + 1 + m) * L + i] : 0.f;
#pragma unroll
    for (int v = 0; v < VF; ++v) FT[(size_t)i * VF + v] = make_float4(fw[4 * v], fw[4 * v + 1], fw[4 * v + 2], fw[4 * v + 3]);
#pragma unroll
    for (int v = 0; v < VB; ++v) BT[(size_t)i * VB + v] = make_float4(bw[4 * v], bw[4 * v + 1], bw[4 * v + 2], bw[4 * v + 3]);
  }
  __syncthreads();

  const double osd = (MODE == 1) ? *a.out_scale_dev : 1.0;
  const int out_exp = pow2_exp(osd);
  const bool fast_ok = out_exp >= -896 && out_exp <= 896;
  const unsigned hi_add = fast_ok ? (unsigned)(896 + out_exp) << 20 : 0u;
  const int tiles_l = (a.nl + 31) / 32;
  const int ntiles = tiles_l * a.n3;
  const int GP = ((Ls + CS_GROUPS - 1) / CS_GROUPS + CS_BLK - 1) / CS_BLK * CS_BLK;  // positions per group

  for (int tile = blockIdx.x * nwarps + warp; tile < ntiles; tile += gridDim.x * nwarps) {
    const int tl = tile % tiles_l, t3 = tile / tiles_l;
    const int l0 = tl * 32;
    const int nlv = min(32, a.nl - l0);
    const bool act = j < nlv;
    const float* src = a.in + (size_t)t3 * a.in_ts + (size_t)l0 * a.in_ls;

    // the tail rows, coalesced, straight into registers (lanes beyond the
    // tile's lines load nothing); they are first used after the staged part
    float yt[NTB][CS_BLK];
    {
      const float* q = src + (size_t)Ls * a.in_ps + j;  // steps one row per position
#pragma unroll
      for (int b = 0; b < NTB; ++b)
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t) {
          yt[b][t] = (b < nt && act) ? *q : 0.f;
          q += a.in_ps;
        }
    }

    __syncwarp();  // the previous tile is done with S
    // ---- stage: group g holds positions [g*GP, (g+1)*GP) of every line ----
#pragma unroll 1
    for (int g = 0; g < CS_GROUPS; ++g) {
      const int p0 = g * GP, p1 = min(Ls, p0 + GP);
      // 16-byte copies of the line-contiguous rows (lines up to a multiple
      // of 4: within the row's padded pitch)
      const int nc = (nlv + 3) / 4;
      if (nc == 8) {  // whole tile: 4 rows per warp-wide copy
        for (int i = p0 + (j >> 3); i < p1; i += 4)
          cs_cp16(S + (size_t)i * srow + 4 * (j & 7), src + (size_t)i * a.in_ps + 4 * (j & 7));
      } else {
        for (int idx = j; idx < (p1 - p0) * nc; idx += 32) {
          const int i = p0 + idx / nc, c = idx % nc;
          cs_cp16(S + (size_t)i * srow + 4 * c, src + (size_t)i * a.in_ps + 4 * c);
        }
      }
      cs_commit();
    }

    float* Sj = S + j;
    // ---- forward: y_i = b_i - sum_m f[m]_i y_{i-m}, in place ----
    float prev[P];
#pragma unroll
    for (int m = 0; m < P; ++m) prev[m] = 0.f;
    {
      int i = 0;
#pragma unroll 1
      for (int g = 0; g < CS_GROUPS; ++g) {
        switch (g) {
          case 0: cs_wait<CS_GROUPS - 1>(); break;
          case 1: cs_wait<CS_GROUPS - 2>(); break;
          case 2: cs_wait<CS_GROUPS - 3>(); break;
          default: cs_wait<0>(); break;
        }
        __syncwarp();
        const int ie = min(Ls, (g + 1) * GP);
#pragma unroll 1
        for (; i + CS_BLK <= ie; i += CS_BLK) {
          float* yp = Sj + (size_t)i * srow;
          const float4* fp = FT + (size_t)i * VF;
          float bv[CS_BLK];
          float4 fv[CS_BLK][VF];
#pragma unroll
          for (int t = 0; t < CS_BLK; ++t) {
            bv[t] = yp[t * srow];
#pragma unroll
            for (int v = 0; v < VF; ++v) fv[t][v] = fp[t * VF + v];
          }
#pragma unroll
          for (int t = 0; t < CS_BLK; ++t) {
            const float* f = reinterpret_cast<const float*>(fv[t]);
            float y = bv[t];
#pragma unroll
            for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
#pragma unroll
            for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
            prev[0] = y;
            bv[t] = y;
          }
#pragma unroll
          for (int t = 0; t < CS_BLK; ++t) yp[t * srow] = bv[t];
        }
#pragma unroll 1
        for (; i < ie; ++i) {
          float4 fv[VF];
#pragma unroll
          for (int v = 0; v < VF; ++v) fv[v] = FT[(size_t)i * VF + v];
          const float* f = reinterpret_cast<const float*>(fv);
          float y = Sj[(size_t)i * srow];
#pragma unroll
          for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
          prev[0] = y;
          Sj[(size_t)i * srow] = y;
        }
      }
    }
    // the tail, in registers
#pragma unroll
    for (int b = 0; b < NTB; ++b) {
      if (b < nt) {
        const int i0 = Ls + b * CS_BLK;
        float4 fv[CS_BLK][VF];
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t)
#pragma unroll
          for (int v = 0; v < VF; ++v) fv[t][v] = FT[(size_t)(i0 + t) * VF + v];
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t) {
          const float* f = reinterpret_cast<const float*>(fv[t]);
          float y = yt[b][t];
#pragma unroll
          for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
          prev[0] = y;
          yt[b][t] = y;
        }
      }
    }

    // ---- backward: x_i = bs_i y_i - sum_m g[m]_i x_{i+m}; row i goes out ----
    using TO = typename std::conditional<MODE == 1, double, float>::type;
    TO* op = static_cast<TO*>(a.out) + (size_t)t3 * a.out_ts + (size_t)(l0 + j);
    const size_t ops = (size_t)a.out_ps;
    float nxt[P];
#pragma unroll
    for (int m = 0; m < P; ++m) nxt[m] = 0.f;
    // the tail first, from the registers
#pragma unroll
    for (int b = NTB - 1; b >= 0; --b) {
      if (b < nt) {
        const int i0 = Ls + b * CS_BLK;
        float4 bw[CS_BLK][VB];
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t)
#pragma unroll
          for (int v = 0; v < VB; ++v) bw[t][v] = BT[(size_t)(i0 + t) * VB + v];
#pragma unroll
        for (int t = CS_BLK - 1; t >= 0; --t) {
          const float* c = reinterpret_cast<const float*>(bw[t]);
          float x = c[0] * yt[b][t];
#pragma unroll
          for (int m = P; m >= 1; --m) x -= c[m] * nxt[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
          nxt[0] = x;
          yt[b][t] = x;
        }
        if (act) cs_store_block<MODE>(op, (size_t)i0, ops, yt[b], out_exp, fast_ok, hi_add);
      }
    }
    // then the staged part
    {
      int i = Ls;
      const int rem = Ls % CS_BLK;
#pragma unroll 1
      for (int r = 0; r < rem; ++r) {
        --i;
        float4 bw[VB];
#pragma unroll
        for (int v = 0; v < VB; ++v) bw[v] = BT[(size_t)i * VB + v];
        const float* c = reinterpret_cast<const float*>(bw);
        float x = c[0] * Sj[(size_t)i * srow];
#pragma unroll
        for (int m = P; m >= 1; --m) x -= c[m] * nxt[m - 1];
#pragma unroll
        for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
        nxt[0] = x;
        if (act) {
          if constexpr (MODE == 1) op[(size_t)i * ops] = f2d_scaled(x, out_exp);
          else op[(size_t)i * ops] = x;
        }
      }
#pragma unroll 1
      for (; i >= CS_BLK; i -= CS_BLK) {
        const int ib = i - CS_BLK;  // block [ib, i), processed downwards
        const float* yp = Sj + (size_t)ib * srow;
        const float4* bp = BT + (size_t)ib * VB;
        float yv[CS_BLK];
        float4 bw[CS_BLK][VB];
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t) {
          yv[t] = yp[t * srow];
#pragma unroll
          for (int v = 0; v < VB; ++v) bw[t][v] = bp[t * VB + v];
        }
#pragma unroll
        for (int t = CS_BLK - 1; t >= 0; --t) {
          const float* c = reinterpret_cast<const float*>(bw[t]);
          float x = c[0] * yv[t];
#pragma unroll
          for (int m = P; m >= 1; --m) x -= c[m] * nxt[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
          nxt[0] = x;
          yv[t] = x;
        }
        if (act) cs_store_block<MODE>(op, (size_t)ib, ops, yv, out_exp, fast_ok, hi_add);
      }
    }
  }
  cs_wait<0>();
}

// ---------------------------------------------------------------------------
// The FP32 x sweep (k_xsweep): the banded LU solve along x, where the
// positions of a line are contiguous in memory.  A warp solves a tile of 32
// lines (32 consecutive y at one z), lane j line j, in blocks of XS_BLK
// positions.  Only a ring of XS_RING staged blocks and, per block, the P
// forward values it starts from (a checkpoint) stay on chip, so an SM holds
// two to three times the lines that staging whole lines allowed, and the line
// length is not bounded by shared memory.  The tile's input is first
// prefetched into L2 in bulk, a line per lane.
//   forward   blocks 0..nb-1 are staged XS_RING-1 ahead by 16-byte cp.async
//             copies (a copy instruction moves 64 contiguous bytes of each of
//             eight lines) into rows of XS_PITCH floats, five 16-byte chunks,
//             so the eight lines a quarter-warp touches sit on different bank
//             quads; each lane runs y_i = b_i - sum_m f[m]_i y_{i-m} over the
//             block from four 128-bit reads of its row, keeping only the block
//             checkpoint;
//   backward  block b, from the top down, re-derives its forward values from
//             its checkpoint and staged input (the last XS_RING blocks are
//             still staged, earlier ones are staged again, from L2, XS_RING
//             blocks ahead), runs x_i = bs_i y_i - sum_m g[m]_i x_{i+m} into
//             its row, and leaves by 16-byte stores the way it came.
// Positions past L are zero in the factor tables and in the staged values,
// so they neither feed nor take anything.  No wait spins: cp.async groups
// complete in hardware.
// ---------------------------------------------------------------------------
constexpr int XS_BLK = 16;        // positions per block
constexpr int XS_RING = 3;        // staged blocks per warp
constexpr int XS_PITCH = 20;      // floats per line of a staged block: four chunks and a spare
constexpr int XS_MAX_WARPS = 8;   // warps per CTA (the launch picks the count that fits most per SM)

template <int P>
struct XsLayout {
  __host__ __device__ static int blocks(int L) { return (L + XS_BLK - 1) / XS_BLK; }
  // the CTA's factor tables, dense per position: forward f[1..P] at [i][P],
  // backward (bs, g[1..P]) at [i][P + 1], nb * XS_BLK positions
  __host__ __device__ static size_t tab_bytes(int L) {
    return sizeof(float) * (size_t)(2 * P + 1) * blocks(L) * XS_BLK;
  }
  // per warp: the ring [XS_RING][32][XS_PITCH] and the checkpoints [nb][P][32]
  __host__ __device__ static size_t warp_floats(int L) {
    return (size_t)XS_RING * 32 * XS_PITCH + (size_t)blocks(L) * P * 32;
  }
};

__device__ __forceinline__ void xs_load_row(float (&v)[XS_BLK], const float* row) {
#pragma unroll
  for (int q = 0; q < XS_BLK / 4; ++q) {
    const float4 t = reinterpret_cast<const float4*>(row)[q];
    v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
  }
}
__device__ __forceinline__ void xs_store_row(float* row, const float (&v)[XS_BLK]) {
#pragma unroll
  for (int q = 0; q < XS_BLK / 4; ++q)
    reinterpret_cast<float4*>(row)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}
// N floats (a multiple of 4) from a 16-byte aligned table, by 128-bit loads
template <int N>
__device__ __forceinline__ void xs_load_tab(float (&f)[N], const float* p) {
#pragma unroll
  for (int q = 0; q < N / 4; ++q) {
    const float4 t = reinterpret_cast<const float4*>(p)[q];
    f[4 * q] = t.x; f[4 * q + 1] = t.y; f[4 * q + 2] = t.z; f[4 * q + 3] = t.w;
  }
}
// forward recurrence over one block in place; prev[m] = y_{i-1-m} on entry and exit
template <int P>
__device__ __forceinline__ void xs_forward(float (&v)[XS_BLK], float (&prev)[P], const float* fp) {
  float f[XS_BLK * P];
  xs_load_tab(f, fp);
#pragma unroll
  for (int t = 0; t < XS_BLK; ++t) {
    float y = v[t];
#pragma unroll
    for (int m = P; m >= 1; --m) y -= f[t * P + m - 1] * prev[m - 1];
#pragma unroll
    for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
    prev[0] = y;
    v[t] = y;
  }
}
// backward recurrence over one block in place, top down; nxt[m] = x_{i+1+m}
template <int P>
__device__ __forceinline__ void xs_backward(float (&v)[XS_BLK], float (&nxt)[P], const float* bp) {
  float c[XS_BLK * (P + 1)];
  xs_load_tab(c, bp);
#pragma unroll
  for (int t = XS_BLK - 1; t >= 0; --t) {
    float x = c[t * (P + 1)] * v[t];
#pragma unroll
    for (int m = P; m >= 1; --m) x -= c[t * (P + 1) + m] * nxt[m - 1];
#pragma unroll
    for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
    nxt[0] = x;
    v[t] = x;
  }
}

template <int P>
__global__ void __launch_bounds__(XS_MAX_WARPS * 32, 2) k_xsweep(const CSweepArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (a.skip_flag != nullptr && *a.skip_flag != 0) return;
  using Lay = XsLayout<P>;
  constexpr int SLOT = 32 * XS_PITCH;  // floats per staged block
  const int L = a.L;
  const int nb = Lay::blocks(L);
  const int NP = nb * XS_BLK;
  const int nch = (L + 3) / 4;  // 16-byte chunks of a line
  const int j = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int cq = j >> 3, cl = j & 7;  // copies: chunk cq of lines cl, cl + 8, cl + 16, cl + 24
  float* FT = reinterpret_cast<float*>(smem);  // [NP][P]
  float* BT = FT + (size_t)P * NP;             // [NP][P + 1]
  float* ring = BT + (size_t)(P + 1) * NP + (size_t)warp * Lay::warp_floats(L);
  float* ck = ring + XS_RING * SLOT;  // [nb][P][32]

  // factor rows (global [row][L]): row 0 fs (1 here), 1..P f, P+1 bs, P+2.. g;
  // zero past L
  for (int i = threadIdx.x; i < NP; i += blockDim.x) {
    const bool in = i < L;
#pragma unroll
    for (int m = 0; m < P; ++m) FT[(size_t)i * P + m] = in ? a.fac[(size_t)(1 + m) * L + i] : 0.f;
#pragma unroll
    for (int m = 0; m <= P; ++m) BT[(size_t)i * (P + 1) + m] = in ? a.fac[(size_t)(P + 1 + m) * L + i] : 0.f;
  }
  __syncthreads();

  float* out = static_cast<float*>(a.out);
  const int tiles_l = (a.nl + 31) / 32;
  const int ntiles = tiles_l * a.n3;
  for (int tile = blockIdx.x * nwarps + warp; tile < ntiles; tile += gridDim.x * nwarps) {
    const int tl = tile % tiles_l, t3 = tile / tiles_l;
    const int l0 = tl * 32;
    const int nlv = min(32, a.nl - l0);
    const float* src = a.in + (size_t)t3 * a.in_ts + (size_t)l0 * a.in_ls;
    float* dst = out + (size_t)t3 * a.out_ts + (size_t)l0 * a.out_ls;

    // this lane's copies: chunk cq of lines cl + 8k; block b adds 16 b floats
    const float* sp[4];
    float* dp[4];
    bool lv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int l = cl + 8 * k;
      lv[k] = l < nlv;
      sp[k] = src + (size_t)l * a.in_ls + 4 * cq;
      dp[k] = dst + (size_t)l * a.out_ls + 4 * cq;
    }
    const int so = cl * XS_PITCH + 4 * cq;  // slot offset of line cl, chunk cq (line cl + 8k: + 8k XS_PITCH)
    // block b of the tile's lines into the ring slot at sl
    auto stage = [&](int b, float* sl) {
      if (4 * b + cq < nch) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (lv[k]) cs_cp16(sl + so + 8 * k * XS_PITCH, sp[k] + XS_BLK * b);
      }
    };
    // the solved block b out of its slot sl, then block b - XS_RING into the slot
    auto flush = [&](int b, float* sl) {
      __syncwarp();
      if (4 * b + cq < nch) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (lv[k])
            *reinterpret_cast<float4*>(dp[k] + XS_BLK * b) =
                *reinterpret_cast<const float4*>(sl + so + 8 * k * XS_PITCH);
      }
      __syncwarp();
      if (b >= XS_RING) stage(b - XS_RING, sl);
      cs_commit();
    };

    // the tile's input into L2 at once (a line per lane), so that staging
    // waits on L2 rather than DRAM latency; the backward pass's second
    // staging finds it there too
    if (j < nlv) cs_prefetch_l2(src + (size_t)j * a.in_ls, 16u * (unsigned)nch);

    __syncwarp();  // the previous tile is done with the ring
#pragma unroll 1
    for (int b = 0; b < XS_RING - 1; ++b) {
      if (b < nb) stage(b, ring + b * SLOT);
      cs_commit();
    }

    // ---- forward; the last block turns straight into the backward pass ----
    float prev[P], nxt[P];
#pragma unroll
    for (int m = 0; m < P; ++m) prev[m] = nxt[m] = 0.f;
    int sb = 0;  // ring slot of block b
#pragma unroll 1
    for (int b = 0; b < nb; ++b) {
      __syncwarp();  // every lane is done with block b-1, whose slot block b+XS_RING-1 takes
      const int sn = (sb == 0) ? XS_RING - 1 : sb - 1;
      if (b + XS_RING - 1 < nb) stage(b + XS_RING - 1, ring + sn * SLOT);
      cs_commit();
      cs_wait<XS_RING - 1>();
      __syncwarp();
      float* row = ring + sb * SLOT + j * XS_PITCH;
      float v[XS_BLK];
      xs_load_row(v, row);
      if (b < nb - 1) {
#pragma unroll
        for (int m = 0; m < P; ++m) ck[(b * P + m) * 32 + j] = prev[m];
        xs_forward<P>(v, prev, FT + (size_t)b * XS_BLK * P);
        sb = (sb == XS_RING - 1) ? 0 : sb + 1;
      } else {
#pragma unroll
        for (int t = 0; t < XS_BLK; ++t)
          if (b * XS_BLK + t >= L) v[t] = 0.f;
        xs_forward<P>(v, prev, FT + (size_t)b * XS_BLK * P);
        xs_backward<P>(v, nxt, BT + (size_t)b * XS_BLK * (P + 1));
        xs_store_row(row, v);
      }
    }
    flush(nb - 1, ring + sb * SLOT);

    // ---- backward over the other blocks ----
#pragma unroll 1
    for (int b = nb - 2; b >= 0; --b) {
      sb = (sb == 0) ? XS_RING - 1 : sb - 1;
      cs_wait<XS_RING - 1>();  // block b's staging (from flush(b + XS_RING)) has landed
      __syncwarp();
      float* sl = ring + sb * SLOT;
      float* row = sl + j * XS_PITCH;
      float v[XS_BLK], pv[P];
      xs_load_row(v, row);
#pragma unroll
      for (int m = 0; m < P; ++m) pv[m] = ck[(b * P + m) * 32 + j];
      xs_forward<P>(v, pv, FT + (size_t)b * XS_BLK * P);
      xs_backward<P>(v, nxt, BT + (size_t)b * XS_BLK * (P + 1));
      xs_store_row(row, v);
      flush(b, sl);
    }
  }
  cs_wait<0>();
}

template <int P>
static cudaError_t launch_xs(const CSweepArgs& a, cudaStream_t s) {
  auto kern = k_xsweep<P>;
  int dev = 0, nsm = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t tab = XsLayout<P>::tab_bytes(a.L), per = sizeof(float) * XsLayout<P>::warp_floats(a.L);
  if (tab + per > (size_t)smem_max) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
  if (e != cudaSuccess) return e;
  // the warps per CTA that put the most warps on an SM (the factor tables are per CTA)
  int best_w = 1, best_total = 0;
  for (int w = XS_MAX_WARPS; w >= 1; --w) {
    const size_t bytes = tab + per * w;
    if (bytes > (size_t)smem_max) continue;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, w * 32, bytes);
    if (e != cudaSuccess) return e;
    if (per_sm * w > best_total) { best_total = per_sm * w; best_w = w; }
  }
  const size_t bytes = tab + per * best_w;
  const int per_sm = std::max(1, best_total / best_w);
  const int tiles = (a.nl + 31) / 32 * a.n3;
  const int grid = std::max(1, std::min(nsm * per_sm, (tiles + best_w - 1) / best_w));
  kern<<<grid, best_w * 32, bytes, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_xsweep(int P, const CSweepArgs& a, cudaStream_t s) {
  if (a.in == nullptr || a.out == nullptr || a.fac == nullptr) return cudaErrorInvalidValue;
  // positions contiguous; lines and planes 16-byte aligned with room for
  // round_up(L, 4) entries per line
  const long long Lr = (a.L + 3) / 4 * 4;
  if (a.in_ps != 1 || a.in_ls % 4 != 0 || a.in_ts % 4 != 0 || a.out_ls % 4 != 0 || a.out_ts % 4 != 0 ||
      a.in_ls < Lr || a.out_ls < Lr)
    return cudaErrorInvalidValue;
  switch (P) {
    case 1: return launch_xs<1>(a, s);
    case 2: return launch_xs<2>(a, s);
    case 3: return launch_xs<3>(a, s);
    case 4: return launch_xs<4>(a, s);
  }
  return cudaErrorInvalidValue;
}

template <int P, int MODE>
static cudaError_t launch_cs(const CSweepArgs& a, cudaStream_t s) {
  auto kern = k_csweep<P, MODE>;
  int dev = 0, nsm = 0, smem_max = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t tab = CsTab<P>::bytes(a.L), per = csweep_warp_bytes(a.L);
  if (tab + per > (size_t)smem_max) return cudaErrorInvalidValue;
  const int nw = (per == 0) ? CS_MAX_WARPS : (int)std::min<size_t>(CS_MAX_WARPS, ((size_t)smem_max - tab) / per);
  const size_t bytes = tab + per * nw;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  const int tiles = (a.nl + 31) / 32 * a.n3;
  const int grid = std::max(1, std::min(nsm, (tiles + nw - 1) / nw));
  kern<<<grid, 32 * nw, bytes, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_csweep(int P, int mode, const CSweepArgs& a, cudaStream_t s) {
  if (a.in == nullptr || a.out == nullptr || a.fac == nullptr || (mode == 1 && a.out_scale_dev == nullptr))
    return cudaErrorInvalidValue;
  // lines contiguous, rows 16-byte aligned (pitches are multiples of 8 entries)
  if (a.in_ls != 1 || (a.in_ps % 4) != 0 || (a.in_ts % 4) != 0) return cudaErrorInvalidValue;
  switch (P * 2 + mode) {
    case 2: return launch_cs<1, 0>(a, s);
    case 3: return launch_cs<1, 1>(a, s);
    case 4: return launch_cs<2, 0>(a, s);
    case 5: return launch_cs<2, 1>(a, s);
    case 6: return launch_cs<3, 0>(a, s);
    case 7: return launch_cs<3, 1>(a, s);
    case 8: return launch_cs<4, 0>(a, s);
    case 9: return launch_cs<4, 1>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace ads
