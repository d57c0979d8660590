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
// The FP32 x sweep in column form (k_xsweep).  Along x the positions of a line
// are contiguous, so a tile of 32 lines (32 consecutive y) is staged LINE-major
// by 16-byte cp.async copies (coalesced: consecutive lanes copy consecutive
// chunks of a line) into rows whose pitch is an odd number of 16-byte chunks.
// Lane j then reads its own line four positions at a time: the eight lanes of
// a quarter-warp read the same chunk index of eight rows, which the odd pitch
// puts on eight different bank quads, so the 128-bit loads and stores are
// conflict-free.  The lanes run across the lines as in k_csweep (all at the
// same position, the LU factors of a position one broadcast load), forward and
// backward in place in the staged rows, and the finished rows leave by 16-byte
// stores, coalesced again.  Positions are processed in software-pipelined
// blocks of 16; the input is staged in four position groups (separate commit
// groups) so the forward pass starts when the first group has landed.  No wait
// spins: cp.async groups complete in hardware.
// ---------------------------------------------------------------------------
constexpr int XS_MAX_WARPS = 8;
constexpr int XS_GROUPS = 4;

// staged row pitch in floats: round_up(L, 4) positions, as an odd number of
// 16-byte chunks
__host__ __device__ inline int xs_pitch(int L) {
  int c = (L + 3) / 4;
  if ((c & 1) == 0) ++c;
  return 4 * c;
}
size_t xsweep_warp_bytes(int L) { return sizeof(float) * 32 * (size_t)xs_pitch(L); }

template <int P>
__global__ void __launch_bounds__(XS_MAX_WARPS * 32) k_xsweep(const CSweepArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (a.skip_flag != nullptr && *a.skip_flag != 0) return;
  using Tab = CsTab<P>;
  constexpr int VF = Tab::VF, VB = Tab::VB;
  const int L = a.L;
  const int Lp = xs_pitch(L);
  const int nch = (L + 3) / 4;  // 16-byte chunks of a line
  const int j = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  float4* FT = reinterpret_cast<float4*>(smem);  // [L][VF]
  float4* BT = FT + (size_t)VF * L;              // [L][VB]
  float* S = reinterpret_cast<float*>(smem + Tab::bytes(L)) + (size_t)warp * 32 * Lp;

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

  float* out = static_cast<float*>(a.out);
  const int tiles_l = (a.nl + 31) / 32;
  const int ntiles = tiles_l * a.n3;
  const int GP = ((L + XS_GROUPS - 1) / XS_GROUPS + CS_BLK - 1) / CS_BLK * CS_BLK;  // positions per group

  for (int tile = blockIdx.x * nwarps + warp; tile < ntiles; tile += gridDim.x * nwarps) {
    const int tl = tile % tiles_l, t3 = tile / tiles_l;
    const int l0 = tl * 32;
    const int nlv = min(32, a.nl - l0);
    const float* src = a.in + (size_t)t3 * a.in_ts + (size_t)l0 * a.in_ls;

    __syncwarp();  // the previous tile is done with S
    // ---- stage: group g holds chunks [g*GP/4, (g+1)*GP/4) of every line ----
#pragma unroll 1
    for (int g = 0; g < XS_GROUPS; ++g) {
      const int c0 = g * (GP / 4), c1 = min(nch, (g + 1) * (GP / 4));
      const int ncg = c1 - c0;
      for (int idx = j; idx < nlv * ncg; idx += 32) {
        const int l = idx / ncg, c = c0 + idx % ncg;
        cs_cp16(S + (size_t)l * Lp + 4 * c, src + (size_t)l * a.in_ls + 4 * c);
      }
      cs_commit();
    }

    float* Sj = S + (size_t)j * Lp;
    // ---- forward: y_i = b_i - sum_m f[m]_i y_{i-m}, in place ----
    float prev[P];
#pragma unroll
    for (int m = 0; m < P; ++m) prev[m] = 0.f;
    {
      int i = 0;
#pragma unroll 1
      for (int g = 0; g < XS_GROUPS; ++g) {
        switch (g) {
          case 0: cs_wait<XS_GROUPS - 1>(); break;
          case 1: cs_wait<XS_GROUPS - 2>(); break;
          case 2: cs_wait<XS_GROUPS - 3>(); break;
          default: cs_wait<0>(); break;
        }
        __syncwarp();
        const int ie = min(L, (g + 1) * GP);
#pragma unroll 1
        for (; i + CS_BLK <= ie; i += CS_BLK) {
          float4* yp = reinterpret_cast<float4*>(Sj + i);
          const float4* fp = FT + (size_t)i * VF;
          float bv[CS_BLK];
          float4 fv[CS_BLK][VF];
#pragma unroll
          for (int q = 0; q < CS_BLK / 4; ++q) {
            const float4 v4 = yp[q];
            bv[4 * q] = v4.x; bv[4 * q + 1] = v4.y; bv[4 * q + 2] = v4.z; bv[4 * q + 3] = v4.w;
          }
#pragma unroll
          for (int t = 0; t < CS_BLK; ++t)
#pragma unroll
            for (int v = 0; v < VF; ++v) fv[t][v] = fp[t * VF + v];
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
          for (int q = 0; q < CS_BLK / 4; ++q) yp[q] = make_float4(bv[4 * q], bv[4 * q + 1], bv[4 * q + 2], bv[4 * q + 3]);
        }
#pragma unroll 1
        for (; i < ie; ++i) {
          float4 fv[VF];
#pragma unroll
          for (int v = 0; v < VF; ++v) fv[v] = FT[(size_t)i * VF + v];
          const float* f = reinterpret_cast<const float*>(fv);
          float y = Sj[i];
#pragma unroll
          for (int m = P; m >= 1; --m) y -= f[m - 1] * prev[m - 1];
#pragma unroll
          for (int m = P - 1; m >= 1; --m) prev[m] = prev[m - 1];
          prev[0] = y;
          Sj[i] = y;
        }
      }
    }

    // ---- backward: x_i = bs_i y_i - sum_m g[m]_i x_{i+m}, in place ----
    {
      float nxt[P];
#pragma unroll
      for (int m = 0; m < P; ++m) nxt[m] = 0.f;
      int i = L;
      const int rem = L % CS_BLK;
#pragma unroll 1
      for (int r = 0; r < rem; ++r) {
        --i;
        float4 bw[VB];
#pragma unroll
        for (int v = 0; v < VB; ++v) bw[v] = BT[(size_t)i * VB + v];
        const float* c = reinterpret_cast<const float*>(bw);
        float x = c[0] * Sj[i];
#pragma unroll
        for (int m = P; m >= 1; --m) x -= c[m] * nxt[m - 1];
#pragma unroll
        for (int m = P - 1; m >= 1; --m) nxt[m] = nxt[m - 1];
        nxt[0] = x;
        Sj[i] = x;
      }
#pragma unroll 1
      for (; i >= CS_BLK; i -= CS_BLK) {
        const int ib = i - CS_BLK;  // block [ib, i), processed downwards
        float4* yp = reinterpret_cast<float4*>(Sj + ib);
        const float4* bp = BT + (size_t)ib * VB;
        float yv[CS_BLK];
        float4 bw[CS_BLK][VB];
#pragma unroll
        for (int q = 0; q < CS_BLK / 4; ++q) {
          const float4 v4 = yp[q];
          yv[4 * q] = v4.x; yv[4 * q + 1] = v4.y; yv[4 * q + 2] = v4.z; yv[4 * q + 3] = v4.w;
        }
#pragma unroll
        for (int t = 0; t < CS_BLK; ++t)
#pragma unroll
          for (int v = 0; v < VB; ++v) bw[t][v] = bp[t * VB + v];
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
#pragma unroll
        for (int q = 0; q < CS_BLK / 4; ++q) yp[q] = make_float4(yv[4 * q], yv[4 * q + 1], yv[4 * q + 2], yv[4 * q + 3]);
      }
    }

    // ---- the solved rows out, 16-byte coalesced stores ----
    __syncwarp();
    float* dst = out + (size_t)t3 * a.out_ts + (size_t)l0 * a.out_ls;
    for (int idx = j; idx < nlv * nch; idx += 32) {
      const int l = idx / nch, c = idx % nch;
      *reinterpret_cast<float4*>(dst + (size_t)l * a.out_ls + 4 * c) =
          *reinterpret_cast<const float4*>(S + (size_t)l * Lp + 4 * c);
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
  const size_t tab = CsTab<P>::bytes(a.L), per = xsweep_warp_bytes(a.L);
  if (tab + per > (size_t)smem_max) return cudaErrorInvalidValue;
  const int nw = (int)std::min<size_t>(XS_MAX_WARPS, ((size_t)smem_max - tab) / per);
  const size_t bytes = tab + per * nw;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  const int tiles = (a.nl + 31) / 32 * a.n3;
  const int grid = std::max(1, std::min(nsm, (tiles + nw - 1) / nw));
  kern<<<grid, 32 * nw, bytes, s>>>(a);
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
