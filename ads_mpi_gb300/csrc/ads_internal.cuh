// ads_internal.cuh — shared declarations of the GB300 ADS library.
#pragma once

#include <cuda.h>  // CUtensorMap type only; the driver entry point is fetched at run time
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/ads_gpu.h"

namespace ads {

// ---------------------------------------------------------------------------
// Tiling constants
// ---------------------------------------------------------------------------
// Assembly: a CTA owns a brick of as_tx(p) x AS_TY elements in x/y and streams
// a chunk of element layers along z.  as_tx(p) = 32 - p makes the brick's DOF
// footprint in x exactly 32 wide (one warp); 256 threads = 8 warps = one
// thread per (element row, footprint column) in the y/z stages.
constexpr int AS_TY = 8;
constexpr int AS_THREADS = 256;
__host__ __device__ constexpr int as_tx(int p) { return 32 - p; }

// Banded sweeps: one warp solves SW_LANES lines staged in shared memory; the
// transposed output leaves in chunks of SW_CH positions (TMA store boxes).
constexpr int SW_LANES = 32;
// largest DOF count per axis the GPU kernels take (sweep shared memory, fixup tables)
constexpr int ADS_MAX_AXIS_DOFS = 448;
constexpr int SW_CH = 32;

// Residual (Kronecker mat-vec) tile in x/y, streamed along z.
constexpr int RS_TX = 32;
constexpr int RS_TY = 8;
constexpr int RS_THREADS = 256;

// ---------------------------------------------------------------------------
// Device-side per-axis tables
// ---------------------------------------------------------------------------
template <typename T>
struct AxisTab {
  const T* nn;   // [E][Q][P+1][2]: value (d=0) and derivative (d=1) of local function a at point k
  const T* jw;   // [E][Q]: J(e) * W(k)
  const T* dd;   // [E][Q][P]: difference weights D_b, b = 1..P (dN_b = D_b - D_{b+1})
};

// The same tables as double-floats (float2: high part, low part) for the
// double-float heat increment assembly (k_assemble_df.cu)
struct DfTab {
  const float2* nn;  // [E][Q][P+1][2]
  const float2* jw;  // [E][Q]
  // p = 2 and 3: per element, the even-odd coefficients of its
  // centro-symmetric tables (N[k][b] = N[p-k][p-b], dN[k][b] = -dN[p-k][p-b]),
  //   p = 2: [(N00+N02)/2, (N00-N02)/2, N01, N10, N11, (dN00+dN02)/2, (dN00-dN02)/2, dN01, dN10]
  //   p = 3: a[k][j] = (N[k][j] + N[k][3-j])/2, c[k][j] = (N[k][j] - N[k][3-j])/2 (k, j < 2),
  //          then the same for dN: [a00 a01 a10 a11 c00 c01 c10 c11 a' c']
  // and symf[e] = 1 where the element's tables are symmetric (null: none are)
  const float2* sym;           // [E][df_sym_count(p)]
  const unsigned char* symf;   // [E]
  // the tables with the point weights J W folded in, nnw[e][k][b][d] =
  // nn[e][k][b][d] J(e) W(k) (null: not built), and their even-odd
  // coefficients (symw; the flags are symf's, W being symmetric): the
  // constant-kappa heat increment interpolates with them along y and z (x
  // takes the element matrices below), so that no per-point product remains
  const float2* nnw;           // [E][Q][P+1][2]
  const float2* symw;          // [E][df_sym_count(p)]
  // x only, for the same increment: each element's 1-D stiffness and mass
  // matrices, K[b][b'] = sum_k dN[k][b] dN[k][b'] J W(k) and M[b][b'] =
  // sum_k N[k][b] N[k][b'] J W(k) (row-major, K then M)
  const float2* mat;           // [E][2][P+1][P+1]
};
constexpr int df_sym_count(int p) { return p == 2 ? 9 : (p == 3 ? 16 : 0); }
struct DfTabs3 {
  DfTab x, y, z;
};

// Factors of the banded LU of one 1-D matrix, as rows of length N:
//   row 0        : fs[i]     forward scale
//   rows 1..P    : f[m][i]   forward coefficients (y_i -= f[m][i] * y_{i-m})
//   row P+1      : bs[i]     backward scale
//   rows P+2..2P+1: g[m][i]  backward coefficients (x_i -= g[m][i] * x_{i+m})
// Normal solve (M = L U, no pivoting): fs = 1, f = L, bs = 1/U_ii, g = U_{i,i+m}/U_ii.
// Transposed solve (M^T = U^T L^T):     fs = 1/U_ii, f = U_{i-m,i}/U_ii, bs = 1, g = L_{i+m,i}.

// ---------------------------------------------------------------------------
// Launch descriptors
// ---------------------------------------------------------------------------
struct Geometry {
  int E[3];      // elements per axis
  int N[3];      // DOFs per axis (E + p)
  int P, Q;      // the common degree and Gauss points per axis (the largest if they differ)
  int p[3], q[3];  // degree and Gauss points of each axis
  long long PX, PY, PZ;  // padded pitches of the three layouts (elements)
  // L0 index: x + PX*(y + Ny*z); L1 index: y + PY*(x + Nx*z); L2 index: z + PZ*(x + Nx*y)
};

struct AssembleArgs {
  Geometry g;
  int form;            // ADS_FORM_*
  int zc;              // element layers per z-chunk
  int nix, niy, niz;   // items per axis
  double dt, kappa;
  const double* u;     // L0 coefficients (FP64)
  long long u_px;      // row pitch of u in entries: g.PX for a device array, g.N[0] for a
                       // caller's unpadded array read in place (the double-float assembly only)
  double* u_copy;      // if set (double-float assembly): every coefficient read, once, into
                       // this padded array (rows of g.PX)
  double* F;           // L0 output (owned DOFs)
  double* shadow;      // 7 spill classes, each an L0-sized array
  long long shadow_stride;
  const double* fqp;   // qp-grid layout (qx + QX*(qy + QY*qz)), may be null
  const double* kqp;   // same layout, may be null
  const double* dqp;   // oil form: draining weight w (draining(u, X) = w u), same layout
  double mu;           // oil form: exponent of exp(mu u)
  double* l2part;      // per CTA: l2 partial at [cta], max |written value| at [grid + cta],
                       // drained partial (oil form; else 0) at [2 grid + cta]
  const double* uscale;  // FP32 heat form: 2^-e with max |u| < 2^e (coefficients are scaled by it)
  int* err;
};

struct FixupArgs {
  Geometry g;
  int zc, nix, niy, niz;
  double* F;
  const double* shadow;
  long long shadow_stride;
  const double* l2part;  // [nl2] l2 partials, [nl2] max |value| partials, [nl2] drained partials
  int nl2;
  double* scal;          // device scalars (SC_*)
  float* g32;            // if set: every entry of the final F also as float(F * SC_IN_SCALE)
  const unsigned char* slab;  // 1 where a DOF index lies in a spill slab: x [Nx], then y [Ny], then z [Nz]
  const int* xslab;           // the x indices of the x slabs, ascending
  int nxslab;
  int* umiss;                 // if set (double-float assembly on a guessed scale): the max |u| the
                              // assembly saw (l2part segment 3) is checked against SC_USCALE and
                              // *umiss set when the scale was off by more than USCALE_WINDOW binades
                              // or F is not finite; SC_USCALE then becomes the exact scale
};

struct SweepArgs {
  int L;            // line length
  const void* in;   // input array (TIn): position p of line l of the tile at (l, t3) is
                    // in[t3 * in_t3s + l * in_ls + p]; lines padded to a multiple of 8 entries
  long long in_ls, in_t3s;
  int lanes_total;  // extent of the lane dimension
  int tiles_lane;   // ceil(lanes_total / SW_LANES)
  int lane_dim;     // 1 or 2: which input tensor dimension carries the lanes
  const void* fac;  // factor rows (TC), (2P+2) x L
  double in_scale;  // multiply the input by this before the solve
  const double* in_scale_dev;   // if set, in_scale = *in_scale_dev (refinement)
  const int* skip_flag;         // if set and *skip_flag != 0, the kernel returns at once
  int out_line_dim;      // TMA store: 1 -> coords (lanes, line, third); 2 -> (lanes, third, line)
  int third_extent;      // extent of the tile's fixed (third) dimension
  int* err;
};

// Column-form FP32 sweep (k_csweep.cu): lines l in [0, nl) in tiles of 32,
// positions i in [0, L), third index t in [0, n3).  Element (l, i, t) of the
// input is in[l*in_ls + i*in_ps + t*in_ts] (in_ls == 1: lines contiguous), of the
// output out[l + i*out_ps + t*out_ts]: float (mode 0) or, in mode 1, the FP64
// state 2^e x with 2^e = *out_scale_dev.  In mode 0 out may be in (a tile
// reads all of its input before it writes).
struct CSweepArgs {
  int L, nl, n3;
  const float* in;
  long long in_ls, in_ps, in_ts;
  void* out;
  long long out_ps, out_ts;
  long long out_ls;              // k_xsweep only: the output's line stride
  const float* fac;              // factor rows (2P+2) x L, as for k_sweep
  const double* out_scale_dev;
  const int* skip_flag;
};

struct ResidualArgs {
  Geometry g;
  int zc, nix, niy, niz;
  const double* u;    // L0
  const double* F;    // L0 (may be null: plain mat-vec)
  double* r;          // L0 output: F - M u (or M u)
  float* r32;         // if set, r is written here as float(r * *r32_scale) instead
  const double* r32_scale;
  const double* band[3];  // per axis, (2P+1) x N: band[(m+P)*N + i] = M_{i,i+m}
  double* part;       // per CTA: [rr, ff, rmax]
  const int* skip_flag;
  int want_ff;        // also reduce ||F||^2 (the first residual of a solve)
  int* err;
};

// Updated residual of an FP32 correction (mixed solve).  r1 = float(r 2^-e)
// is the scaled FP64 residual that the correction x1 (FP32) was solved for:
// delta += 2^e x1, r2 = r1 - M x1 with M x1 in double-float arithmetic (FP32
// at P = 4), and a = M |x1| in FP32, for the certified bound of k_certify.
struct UpdateArgs {
  Geometry g;
  int zc, nix, niy, niz;
  const float* x1;           // L0: the correction's FP32 solution
  const float* r1;           // L0: the scaled FP32 residual it solved for
  double* delta;             // L0: += 2^e x1
  const double* out_scale;   // 2^e
  const float2* band[3];     // double-float copies of the 1-D mass bands (.x: the FP32 rounding)
  double* part;              // per CTA: [sum (2^24 r2)^2, sum a^2, sum r1^2]
  const int* skip_flag;
};

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
// incr (FP32 heat form only): leave out the mass term J W v u, i.e. assemble
// G = F - M u instead of F
// grid: upper bound of persistent CTAs (size of the partial arrays); the grid
// actually launched (resident CTAs, at most the work items) is returned
cudaError_t launch_assemble(bool fp32, bool incr, const AssembleArgs& a, const void* tabs_x,
                            const void* tabs_y, const void* tabs_z, int grid, int* used_grid, cudaStream_t s);
// the oil form (k_assemble_oil.cu): pump (fqp), Kq (kqp) and w (dqp) all required
cudaError_t launch_assemble_oil(bool fp32, bool incr, const AssembleArgs& a, const void* tabs_x,
                                const void* tabs_y, const void* tabs_z, int grid, int* used_grid, cudaStream_t s);
cudaError_t launch_fixup(const FixupArgs& a, cudaStream_t s);
// the heat increment G = F - M u (form HEAT only) in double-float arithmetic
// on the FP32 pipe, from coefficients scaled by *a.uscale (k_assemble_df.cu)
cudaError_t launch_assemble_df(const AssembleArgs& a, const DfTabs3& tb, int grid, int* used_grid, cudaStream_t s);
size_t assemble_df_smem_bytes(int P);

// kind: 0 = x sweep (L0 -> L1), 1 = y sweep (L1 -> L2), 2 = z sweep (L2 -> L0)
// mode: 0 = TMA store to the next layout through tmout, 3 = identity transpose
//       (no solve), both FP64; 4 = FP32 solve stored back into the input's
//       layout through tmout (box: SW_CH positions by SW_LANES lines); trans
//       (the adjoint's transposed solve) in mode 0 only
// tin: 0 = double input, 1 = float input; tc: 0 = double compute, 1 = float compute
// The input is read through a.in (set with sweep_input in the host code).
cudaError_t launch_sweep(int P, int tin, int tc, int mode, bool trans, const CUtensorMap* tmout,
                         const SweepArgs& a, int grid, cudaStream_t s);

// device scalar slots (double) and flag slots (int) of a handle
enum ScalarSlot {
  SC_L2 = 0,        // l2norm of the last assembly
  SC_FF,            // ||F||_2^2
  SC_FMAX,          // max |F|
  SC_RR,            // ||r||_2^2 of the last residual
  SC_RELRES,        // ||r|| / ||F|| of the last residual
  SC_IN_SCALE,      // first solve: input scale 2^-e (max|F| ~ 2^e)
  SC_OUT_SCALE,     // first solve: output scale 2^e
  SC_DOT,           // result of launch_dot
  SC_USCALE,        // 2^-e with max |u| < 2^e, for the FP32 assembly
  SC_DRAINED,       // oil form: drained statistic of the last assembly
  SC_DRAINED_TOTAL, // oil form: drained summed over the steps since ads_set_oil
  SC_COUNT = 16
};
// doubles per step in the history the step kernels record
constexpr int HIST_W = 5;
enum FlagSlot {
  FL_ERR = 0,       // error bits (ERRF_*)
  FL_CONV,          // refinement converged
  FL_ITERS,         // corrections applied in the current solve
  FL_HIST,          // number of recorded steps
  FL_RESID,         // FP64 residuals that ran in the current solve
  FL_UMISS,         // the step on a caller's buffers found its guessed coefficient scale off
  FL_COUNT = 8
};

cudaError_t launch_residual(int P, const ResidualArgs& a, int grid, cudaStream_t s);
// resident k_residual CTAs per SM (1 if the query fails)
int residual_ctas_per_sm(int P);
// reduce residual partials; sets SC_RR, SC_RELRES, FL_CONV and
// (if count_iter and not converged) FL_ITERS += 1.  Skipped when FL_CONV is set.
// use_ff: take ||F||^2 from the partials (and store it) instead of SC_FF
cudaError_t launch_decide(const double* part, int n, double tol, bool count_iter, bool use_ff, double* scal,
                          int* flags, cudaStream_t s);
cudaError_t launch_resid_update(int P, const UpdateArgs& a, int grid, cudaStream_t s);
// DOF rows (y) of one k_resid_update tile; its x width is RS_TX, its z chunk UpdateArgs::zc
int resid_update_rows();
// from the k_resid_update partials: SC_RELRES = an upper bound of ||F - M x|| / ||F||
// after the correction, FL_CONV if it is <= tol.  Skipped when FL_CONV is set.
cudaError_t launch_certify(const double* part, int n, int P, long long ndof, double tol, double* scal, int* flags,
                           cudaStream_t s);
// ||F||^2, max|F| and the first-solve scales
cudaError_t launch_norm_f(const double* F, const Geometry& g, double* part, int nparts, double* scal,
                          cudaStream_t s);
cudaError_t launch_step_reset(double* scal, int* flags, cudaStream_t s);
// scal[SC_USCALE] = 2^-e for max |u| over n entries (power-of-two scale of the FP32 assembly)
cudaError_t launch_uscale(const double* u, long long n, double* part, int nparts, double* scal, cudaStream_t s);
// hist row of the step; adds the oil drained statistic to its running total
cudaError_t launch_record(double* scal, int* flags, double* hist, int cap, cudaStream_t s);

// the spline of the L0 coefficients u at an rx x ry x rz sample grid (x fastest);
// tab/first: the per-axis sample tables of sample_basis, x then y then z
cudaError_t launch_eval_grid(const double* u, const Geometry& g, const double* tab, const int* first, int rx,
                             int ry, int rz, double* vals, cudaStream_t s);
// MultiStep: the pivoted band solve (band_lu factors) along one direction of an
// FP64 L0 array, lines (l1, l2) at b + l1*s1 + l2*s2, positions ps apart
cudaError_t launch_band_solve(double* b, long long n1, long long n2, long long s1, long long s2, long long ps, int n,
                              int kl, int ku, const double* AB, const int* ipiv, cudaStream_t s);
// packed coefficients (dense Nx) -> padded L0 (to_padded) or back
cudaError_t launch_repack(const double* src, double* dst, const Geometry& g, bool to_padded, cudaStream_t s);
// layout conversions between the per-point (kx,ky,kz,ex,ey,ez) layout and the
// quadrature grid layout qx + QX*(qy + QY*qz)
cudaError_t launch_qp_to_grid(const double* src, double* dst, const Geometry& g, cudaStream_t s);
cudaError_t launch_grid_to_qp(const double* src, double* dst, const Geometry& g, cudaStream_t s);
// y = alpha*x + beta*y over n entries
// y += x
cudaError_t launch_add(double* y, const double* x, long long n, cudaStream_t s);
// d_u += delta, also into u_out: d_u and delta padded (rows of PX), u_out an
// unpadded array (rows of N[0]) a caller owns, written in place.  Writes
// nothing when *skip is set.
cudaError_t launch_update_host(const double* delta, double* d_u, double* u_out, const Geometry& g,
                               const int* skip, cudaStream_t s);
// binades by which the guessed coefficient scale of a step on a caller's
// buffers may differ from the exact one
constexpr int USCALE_WINDOW = 8;
cudaError_t launch_axpby(double* y, const double* x, double alpha, double beta, long long n,
                         cudaStream_t s);
// out = sum x*y over n entries (deterministic two-stage)
cudaError_t launch_dot(const double* x, const double* y, long long n, double* part, int nparts,
                       double* out, cudaStream_t s);

// adjoint: gk[q] += -dt * J W grad u(q) . grad mu(q) on the quadrature grid layout
cudaError_t launch_kappa_grad(const Geometry& g, const double* u, const double* mu, double dt,
                              double* gk, const AxisTab<double>& tx, const AxisTab<double>& ty,
                              const AxisTab<double>& tz, cudaStream_t s);

// ---------------------------------------------------------------------------
// General geometry (k_general.cu): per-axis degrees p[3] (1..4 each, not all
// equal).  FP64 kernels with the degrees as run-time values: one thread per
// element of one colour class for the assembly (elements of a class share no
// DOF, so the scatter needs no atomics and the sum order is fixed), one thread
// per DOF for the mass product.
// ---------------------------------------------------------------------------
struct GenAssembleArgs {
  Geometry g;
  int form;             // ADS_FORM_PROJECT or ADS_FORM_HEAT
  int incr;             // heat: leave out the mass term J W v u
  double dt, kappa;
  const double* u;      // L0 coefficients
  double* F;            // L0 output, accumulated (zeroed before the first colour)
  const double* fqp;    // qp-grid layout, may be null
  const double* kqp;    // qp-grid layout, may be null
  const double* nn[3];  // per axis [E][q][p+1][2]
  const double* jw[3];  // per axis [E][q]
  double* part;         // l2 partial per (colour, block)
};
// all colour classes in order, then the l2norm into scal[SC_L2]
cudaError_t launch_assemble_gen(const GenAssembleArgs& a, double* scal, cudaStream_t s);
// partials needed by launch_assemble_gen
long long assemble_gen_parts(const Geometry& g);
// r = F - (Mx (x) My (x) Mz) u (or M u with F null), band[d][(m+p_d)*N_d + i] = M_{i,i+m}
cudaError_t launch_residual_gen(const Geometry& g, const double* u, const double* F, double* r,
                                const double* const band[3], cudaStream_t s);
// dL/dkappa at the points, as launch_kappa_grad
cudaError_t launch_kappa_grad_gen(const Geometry& g, const double* u, const double* mu, double dt, double* gk,
                                  const AxisTab<double>& tx, const AxisTab<double>& ty, const AxisTab<double>& tz,
                                  cudaStream_t s);
// the reorders of ReorderRHSFor{Y,Z,X} as plain permutations (kind: ADS_REORDER_*),
// dense arrays in and out
cudaError_t launch_permute(const double* in, double* out, const Geometry& g, int kind, cudaStream_t s);

// FMA throughput of the FP32 or FP64 pipe (TFLOP/s, an FMA counted as 2 flops)
cudaError_t measure_fma_peak(bool fp64, double* tflops);

size_t assemble_smem_bytes(int P, bool fp32);

// What ads_residual_noalloc (noalloc.cu) reads from a handle: the residual
// kernel's tiling, the mass bands and a geometry whose x pitch is the dense
// Nx of caller-owned arrays.  No buffer of the handle is used.
struct NoallocView {
  int dev = 0, P = 0, grid = 0;
  bool general = false;  // unequal degrees: the tuned residual does not apply
  cudaStream_t stream = nullptr;
  ResidualArgs args{};
  long long* launches = nullptr;
};
void handle_noalloc_view(ads_handle* h, NoallocView* v);
int handle_fail(ads_handle* h, int code, const std::string& msg);
int handle_cuda_fail(ads_handle* h, cudaError_t e, const char* where);

// ---------------------------------------------------------------------------
// FP64 <-> FP32 conversions with integer operations only (GB300 runs FP64 at
// 1/64 of the FP32 rate, conversions included), with a power-of-two scale
// 2^sexp folded into the exponent.  Every case is integer work, so no FP64
// instruction is ever issued for them: values below the target's normal range
// flush to signed zero, overflow gives infinity, inf and NaN map to inf and
// (quiet) NaN.
// ---------------------------------------------------------------------------
// The rare cases (zero, subnormal, inf, NaN, out of range) live in separate,
// non-inlined functions so the common path is a short branch-free sequence.
static __device__ __noinline__ float d2f_scaled_rare(double d, int sexp) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int ed = (int)((b >> 52) & 0x7ffull);
  const unsigned long long m = b & 0xfffffffffffffull;
  if (ed == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m != 0ull ? 0x400000u : 0u));
  const int ef = ed + sexp - 896;
  if (ed == 0 || ef < 1) return __uint_as_float(sign);
  return __uint_as_float(sign | 0x7f800000u);  // ef > 254: overflow
}

__device__ __forceinline__ float d2f_scaled(double d, int sexp) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int ed = (int)((b >> 52) & 0x7ffull);
  const int ef = ed + sexp - 896;  // biased float exponent after scaling (1023 - 127)
  if ((unsigned)(ed - 1) >= 2046u || (unsigned)(ef - 1) >= 254u) {
    // zeros (and double subnormals, which flush) inline: no call for the common zero
    if (ed == 0) return __uint_as_float((unsigned)(b >> 63) << 31);
    return d2f_scaled_rare(d, sexp);
  }
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned m23 = (unsigned)(b >> 29) & 0x7fffffu;
  const unsigned rem = (unsigned)b & 0x1fffffffu;
  unsigned r = sign | ((unsigned)ef << 23) | m23;
  if (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) r += 1u;  // a carry rounds into the exponent
  return __uint_as_float(r);
}

static __device__ __noinline__ double f2d_scaled_rare(float f, int sexp) {
  const unsigned b = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  int e = (int)((b >> 23) & 0xffu);
  unsigned m23 = b & 0x7fffffu;
  if (e == 0xff) return __longlong_as_double((long long)(sign | (0x7ffull << 52) | ((unsigned long long)m23 << 29)));
  if (e == 0) {
    if (m23 == 0u) return __longlong_as_double((long long)sign);
    const int sh = __clz(m23) - 8;  // float subnormal: normalise
    m23 = (m23 << sh) & 0x7fffffu;
    e = 1 - sh;
  }
  const int ed = e + 896 + sexp;
  if (ed < 1) return __longlong_as_double((long long)sign);
  if (ed > 2046) return __longlong_as_double((long long)(sign | (0x7ffull << 52)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)ed << 52) | ((unsigned long long)m23 << 29)));
}

// float -> double (exact) times 2^sexp
__device__ __forceinline__ double f2d_scaled(float f, int sexp) {
  const unsigned b = __float_as_uint(f);
  const unsigned e8 = (b >> 23) & 0xffu;
  const int edn = (int)e8 + 896 + sexp;
  if (e8 - 1u >= 254u || (unsigned)(edn - 1) >= 2046u) {
    if ((b << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)(b >> 31) << 63));  // zero inline
    return f2d_scaled_rare(f, sexp);
  }
  return __longlong_as_double((long long)(((unsigned long long)(b >> 31) << 63) | ((unsigned long long)edn << 52) |
                                          ((unsigned long long)(b & 0x7fffffu) << 29)));
}

// d * 2^sexp = hi + lo with hi the nearest float and lo the float nearest to
// the remainder (hi + lo carries ~48 bits); both zero below the float range
__device__ __forceinline__ void split_scaled(double d, int sexp, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int ed = (int)((b >> 52) & 0x7ffull);
  const int ef = ed + sexp - 896;
  lo = 0.f;
  if ((unsigned)(ed - 1) >= 2046u || (unsigned)(ef - 1) >= 254u) {
    // zero (inline), inf, NaN, under- or overflow: lo = 0
    hi = (ed == 0) ? __uint_as_float((unsigned)(b >> 63) << 31) : d2f_scaled_rare(d, sexp);
    return;
  }
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned m23 = (unsigned)(b >> 29) & 0x7fffffu;
  const unsigned rem = (unsigned)b & 0x1fffffffu;
  const bool up = rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u));
  hi = __uint_as_float((sign | ((unsigned)ef << 23) | m23) + (up ? 1u : 0u));
  // remainder in units of the double's last mantissa bit, 2^(ef - 179)
  const int rs = (int)rem - (up ? (1 << 29) : 0);
  if (rs != 0 && ef >= 53) {
    const float unit = __uint_as_float((unsigned)(ef - 52) << 23);
    const float v = (float)rs * unit;
    lo = sign ? -v : v;
  }
}

__device__ __forceinline__ int pow2_exp(double s) {
  return (int)(((unsigned long long)__double_as_longlong(s) >> 52) & 0x7ffull) - 1023;
}
cudaError_t launch_csweep(int P, int mode, const CSweepArgs& a, cudaStream_t s);
// The FP32 x sweep of the mixed step in column form (k_csweep.cu): lines l
// (y) in tiles of 32, positions i (x) contiguous, in[l*in_ls + i + t*in_ts] ->
// out[l*out_ls + i + t*out_ts] (FP32; out may be in); in_ls, out_ls, in_ts and
// out_ts multiples of 4 entries with at least round_up(L, 4) entries per line
cudaError_t launch_xsweep(int P, const CSweepArgs& a, cudaStream_t s);

}  // namespace ads
