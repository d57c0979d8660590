// ads_api.cu — the C-ABI (include/ads_gpu.h): handle, device memory, step
// orchestration, refinement control, adjoint driver, timing.
//
// One handle = one configuration on one GPU (the reference's ADS_setup +
// ADS_compute_data, src/Setup.F90:29-140, for one rank).  Device layouts:
//   L0: x fastest, pitch PX  (coefficients u, assembled F, residual r)
//   L1: y fastest, pitch PY  (after the x sweep; the reference's F2)
//   L2: z fastest, pitch PZ  (after the y sweep; the reference's F3)
// Pitches are rounded up to 8 entries so every TMA stride is a multiple of 16 B.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "ads_internal.cuh"
#include "setup.h"

using namespace ads;

namespace {

typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

PFN_encodeTiled get_encode() {
  static PFN_encodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_encodeTiled>(p);
  }
  return fn;
}

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

}  // namespace

struct ads_handle {
  int n[3] = {0, 0, 0}, p[3] = {0, 0, 0};
  int P = 0, Q = 0;
  ads_opts opts{};
  int dev = 0;
  bool pageable = false;  // the device reads pageable host memory (cudaDevAttrPageableMemoryAccess)
  bool uscale_set = false;  // SC_USCALE holds the scale of some coefficients (a uscale pass ran)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;

  AxisHost ax[3];
  Geometry g{};
  size_t n0 = 0, n1 = 0, n2 = 0;  // padded element counts of L0/L1/L2
  long long nqp = 0;

  // device tables
  double* d_nn64[3] = {nullptr, nullptr, nullptr};
  double* d_jw64[3] = {nullptr, nullptr, nullptr};
  float* d_nn32[3] = {nullptr, nullptr, nullptr};
  float* d_jw32[3] = {nullptr, nullptr, nullptr};
  double* d_dd64[3] = {nullptr, nullptr, nullptr};
  float* d_dd32[3] = {nullptr, nullptr, nullptr};
  double* d_fac64[3] = {nullptr, nullptr, nullptr};
  double* d_tfac64[3] = {nullptr, nullptr, nullptr};
  float* d_fac32[3] = {nullptr, nullptr, nullptr};
  double* d_band[3] = {nullptr, nullptr, nullptr};
  float2* d_nndf[3] = {nullptr, nullptr, nullptr};  // double-float tables (ADS_PREC_MIXED)
  // general geometry: unequal degrees (general) or an axis longer than the
  // sweeps' shared-memory lines (banded: every solve by k_band_solve with the
  // mass matrix's banded LU, d_gab/d_gpiv per axis)
  bool general = false, banded = false;
  double* d_gab[3] = {nullptr, nullptr, nullptr};
  int* d_gpiv[3] = {nullptr, nullptr, nullptr};
  double* d_gpart = nullptr;  // l2 partials of the general assembly
  float2* d_jwdf[3] = {nullptr, nullptr, nullptr};
  float2* d_symdf[3] = {nullptr, nullptr, nullptr};        // p = 2, 3: even-odd coefficients per element
  unsigned char* d_symf[3] = {nullptr, nullptr, nullptr};  // ... and which elements are symmetric
  float2* d_nnwdf[3] = {nullptr, nullptr, nullptr};        // double-float tables times J W
  float2* d_symwdf[3] = {nullptr, nullptr, nullptr};       // ... and their even-odd coefficients
  float2* d_matdf = nullptr;   // x: element stiffness and mass matrices (double-float)
  float2* d_band32[3] = {nullptr, nullptr, nullptr};  // double-float copies for the updated residual

  // device buffers
  double* d_u = nullptr;
  double* d_F = nullptr;
  double* d_r = nullptr;
  double* d_delta = nullptr;  // mixed: increment of the heat step
  float* d_g32 = nullptr;     // mixed: the FP32 solve's scaled input (G, then each residual), L0
  float* d_x32 = nullptr;     // mixed: the FP32 correction x1, L0
  float* d_wC = nullptr;      // mixed: the FP32 x and y sweeps' output, L0
  double* d_wA = nullptr;  // L1 (double-sized; float view uses the same memory)
  double* d_wB = nullptr;  // L2
  double* d_shadow = nullptr;
  double* d_fqp = nullptr;
  double* d_kqp = nullptr;
  double* d_dqp = nullptr;  // oil: draining weight per point (qp grid layout)
  double* d_l2part = nullptr;
  double* d_stage = nullptr;        // packed copy of one coefficient array (host transfers)
  // MultiStep: the start-of-step state, a work array, and per axis the
  // pivoted LU of the last matrix mix
  double* d_un = nullptr;
  double* d_ms = nullptr;
  double* d_mab[3] = {nullptr, nullptr, nullptr};
  int* d_mpiv[3] = {nullptr, nullptr, nullptr};
  double mab_mix[3][4] = {};
  bool mab_valid[3] = {false, false, false};
  unsigned char* d_slab = nullptr;  // spill-slab flags per DOF index (x, y, z)
  int* d_xslab = nullptr;           // x indices of the x slabs
  int nxslab = 0;
  double* d_part = nullptr;
  double* d_scal = nullptr;
  int* d_flags = nullptr;
  double* d_hist = nullptr;
  int hist_cap = 0;
  int npart = 0;

  // launch geometry
  int asm_grid = 0, asm_zc = 0, asm_nix = 0, asm_niy = 0, asm_niz = 0;
  int res_grid = 0, res_zc = 0, res_nix = 0, res_niy = 0, res_niz = 0;  // 32-plane chunks
  int rsd_grid = 0, rsd_zc = 0, rsd_niz = 0;  // k_residual's own z chunking (whole waves)
  int upd_grid = 0, upd_niy = 0;  // k_resid_update: the x and z tiling of res_*, its own rows
  int norm_parts = 0;

  // tensor maps
  // TMA store maps of the sweeps' transposed outputs
  CUtensorMap tm_u_out64{}, tm_r_out64{};
  CUtensorMap tm_wA_out64{}, tm_wB_out64{};
  CUtensorMap tm_wC_out32{};

  // form
  bool has_form = false;
  int form = ADS_FORM_PROJECT;
  double kappa = 1.0, dt = 0.0;
  bool has_f = false, has_k = false;
  bool has_oil = false;  // oil: ads_set_oil was called
  double mu = 0.0;

  ads_stats last{};

  // timing: one event pair per timed launch, resolved when the totals are read
  bool timing = false;
  std::vector<std::string> tnames;
  std::vector<double> tms;
  std::vector<int> tcount;
  std::vector<cudaEvent_t> evpool;
  std::vector<int> pending;  // kernel index of each recorded event pair
  // phases under the reference's PERFORMANCE names (src/ADS.F90:497-754):
  // the current one, and the per-phase totals of the timed launches
  const char* phase = "Other";
  std::vector<std::string> pnames;
  std::vector<double> pms;
  std::vector<int> pcount;
  std::vector<int> ppending;  // phase index of each recorded event pair
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  long long launches = 0;

  // graph of one step
  cudaGraphExec_t gexec = nullptr;
  bool graph_valid = false;
  long long graph_launches = 0;
};

namespace {

int fail(ads_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

// FP32 sweeps with FP64 refinement (either mixed precision)
bool is_mixed(const ads_handle* h) { return h->opts.precision != ADS_PREC_FP64; }
// the heat increment assembled in double-float arithmetic
bool df_increment(const ads_handle* h) { return h->opts.precision == ADS_PREC_MIXED && h->form == ADS_FORM_HEAT; }

int cuda_fail(ads_handle* h, cudaError_t e, const char* where) {
  return fail(h, ADS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define ADS_CUDA(h, call)                               \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

// resolve recorded event pairs into the per-kernel totals
void resolve_timing(ads_handle* h) {
  if (h->pending.empty()) return;
  cudaStreamSynchronize(h->stream);
  for (size_t i = 0; i < h->pending.size(); ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->evpool[2 * i], h->evpool[2 * i + 1]) == cudaSuccess) {
      h->tms[h->pending[i]] += ms;
      h->tcount[h->pending[i]] += 1;
      h->pms[h->ppending[i]] += ms;
      h->pcount[h->ppending[i]] += 1;
    }
  }
  h->pending.clear();
  h->ppending.clear();
}

// A phase of the step named as the reference's PERFORMANCE output names it
// ("Form 3D RHS", "Solve 1", ...): an NVTX range over its launches and the
// phase that the per-kernel timers also add into.
struct Phase {
  ads_handle* h;
  const char* prev;
  Phase(ads_handle* hh, const char* name) : h(hh), prev(hh->phase) {
    h->phase = name;
    nvtxRangePushA(name);
  }
  ~Phase() {
    nvtxRangePop();
    h->phase = prev;
  }
};

template <typename F>
int run_kernel(ads_handle* h, const char* name, int nlaunch, F&& f) {
  cudaError_t e;
  if (h->timing) {
    size_t k = 0;
    for (; k < h->tnames.size(); ++k)
      if (h->tnames[k] == name) break;
    if (k == h->tnames.size()) {
      h->tnames.push_back(name);
      h->tms.push_back(0.0);
      h->tcount.push_back(0);
    }
    if (h->pending.size() >= 4096) resolve_timing(h);
    size_t pk = 0;
    for (; pk < h->pnames.size(); ++pk)
      if (h->pnames[pk] == h->phase) break;
    if (pk == h->pnames.size()) {
      h->pnames.push_back(h->phase);
      h->pms.push_back(0.0);
      h->pcount.push_back(0);
    }
    const size_t i = h->pending.size();
    while (h->evpool.size() < 2 * (i + 1)) {
      cudaEvent_t ev;
      if (cudaEventCreate(&ev) != cudaSuccess) break;
      h->evpool.push_back(ev);
    }
    const bool have = h->evpool.size() >= 2 * (i + 1);
    if (have) cudaEventRecord(h->evpool[2 * i], h->stream);
    e = f();
    if (have) {
      cudaEventRecord(h->evpool[2 * i + 1], h->stream);
      h->pending.push_back((int)k);
      h->ppending.push_back((int)pk);
    }
  } else {
    e = f();
  }
  h->launches += nlaunch;
  if (e != cudaSuccess) return cuda_fail(h, e, name);
  return ADS_OK;
}

#define RUN(h, name, n, expr)                                               \
  do {                                                                      \
    int st_ = run_kernel(h, name, n, [&]() -> cudaError_t { return (expr); }); \
    if (st_ != ADS_OK) return st_;                                          \
  } while (0)

template <typename T>
int upload(ads_handle* h, T** d, const std::vector<T>& v) {
  ADS_CUDA(h, cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(v.size(), 1)));
  ADS_CUDA(h, cudaMemcpy(*d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return ADS_OK;
}

// p = 2 and 3 (p + 1 Gauss points): the even-odd coefficients of each
// element's value and derivative tables (DfTab::sym) and whether they may
// stand for the tables.  An element qualifies when N[k][b] = N[p-k][p-b] and
// dN[k][b] = -dN[p-k][p-b] hold to 4e-15 of the table's largest entry (about
// the double-float tables' own precision): the elements of a knot vector that
// is uniform in FP64, except the first and last p - 1, whose basis the open
// knot vector's repeated end knots bend.
void even_odd_tables(const AxisHost& a, std::vector<double>& sc, std::vector<unsigned char>& sf) {
  const int E = a.E, p = a.p, q = p + 1, ns = df_sym_count(p);
  sc.assign((size_t)E * ns, 0.0);
  sf.assign((size_t)E, 0);
  for (int e = 0; e < E; ++e) {
    auto N = [&](int k, int b, int d) { return a.NN[(((size_t)e * q + k) * (p + 1) + b) * 2 + d]; };
    double mn = 0.0, md = 0.0, en = 0.0, ed = 0.0;  // largest entries, largest departures from the symmetry
    for (int k = 0; k < q; ++k)
      for (int b = 0; b <= p; ++b) {
        mn = std::max(mn, std::fabs(N(k, b, 0)));
        md = std::max(md, std::fabs(N(k, b, 1)));
        en = std::max(en, std::fabs(N(k, b, 0) - N(p - k, p - b, 0)));
        ed = std::max(ed, std::fabs(N(k, b, 1) + N(p - k, p - b, 1)));
      }
    double* c = &sc[(size_t)e * ns];
    if (p == 2) {
      c[0] = 0.5 * (N(0, 0, 0) + N(0, 2, 0));
      c[1] = 0.5 * (N(0, 0, 0) - N(0, 2, 0));
      c[2] = N(0, 1, 0);
      c[3] = N(1, 0, 0);
      c[4] = N(1, 1, 0);
      c[5] = 0.5 * (N(0, 0, 1) + N(0, 2, 1));
      c[6] = 0.5 * (N(0, 0, 1) - N(0, 2, 1));
      c[7] = N(0, 1, 1);
      c[8] = N(1, 0, 1);
    } else {
      for (int d = 0; d < 2; ++d)
        for (int k = 0; k < 2; ++k)
          for (int j = 0; j < 2; ++j) {
            c[8 * d + 2 * k + j] = 0.5 * (N(k, j, d) + N(k, 3 - j, d));
            c[8 * d + 4 + 2 * k + j] = 0.5 * (N(k, j, d) - N(k, 3 - j, d));
          }
    }
    sf[e] = (en <= 4e-15 * mn && ed <= 4e-15 * md) ? 1 : 0;
  }
}

// Each element's 1-D stiffness and mass matrices along an axis, K[b][b'] =
// sum_k dN[k][b] dN[k][b'] J W(k), M[b][b'] = sum_k N[k][b] N[k][b'] J W(k)
// (the same Gauss rule, in FP64; row-major, K then M: DfTab::mat).
std::vector<double> element_matrices(const AxisHost& a) {
  const int E = a.E, p = a.p, q = p + 1, nb = p + 1;
  std::vector<double> m((size_t)E * 2 * nb * nb, 0.0);
  for (int e = 0; e < E; ++e) {
    auto N = [&](int k, int b, int d) { return a.NN[(((size_t)e * q + k) * (p + 1) + b) * 2 + d]; };
    for (int t = 0; t < 2; ++t) {  // t = 0: stiffness (derivatives), 1: mass (values)
      const int d = t == 0 ? 1 : 0;
      double* M = &m[((size_t)e * 2 + t) * nb * nb];
      for (int b = 0; b < nb; ++b)
        for (int bb = 0; bb < nb; ++bb) {
          double s = 0.0;
          for (int k = 0; k < q; ++k) s += N(k, b, d) * N(k, bb, d) * a.JW[(size_t)e * q + k];
          M[b * nb + bb] = s;
        }
    }
  }
  return m;
}

bool encode(CUtensorMap* m, void* base, bool fp32, cuuint64_t d0, cuuint64_t d1, cuuint64_t d2,
            long long pitch, cuuint32_t b0, cuuint32_t b1, cuuint32_t b2) {
  PFN_encodeTiled fn = get_encode();
  if (!fn) return false;
  const size_t es = fp32 ? 4 : 8;
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * es), (cuuint64_t)(pitch * d1 * es)};
  cuuint32_t box[3] = {b0, b1, b2};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Layout maps: L0 dims (Nx,Ny,Nz) pitch PX; L1 (Ny,Nx,Nz) pitch PY; L2 (Nz,Nx,Ny) pitch PZ.
// Sweep input boxes are (CH, lanes...) and output boxes (32 lanes, line...).
bool make_l0_out(const ads_handle* h, CUtensorMap* m, void* base, bool f32) {
  return encode(m, base, f32, h->g.N[0], h->g.N[1], h->g.N[2], h->g.PX, SW_LANES, 1, SW_CH);
}
bool make_l1_out(const ads_handle* h, CUtensorMap* m, void* base, bool f32) {
  return encode(m, base, f32, h->g.N[1], h->g.N[0], h->g.N[2], h->g.PY, SW_LANES, SW_CH, 1);
}
bool make_l2_out(const ads_handle* h, CUtensorMap* m, void* base, bool f32) {
  return encode(m, base, f32, h->g.N[2], h->g.N[0], h->g.N[1], h->g.PZ, SW_LANES, 1, SW_CH);
}

// sweep along `axis` (0: x, L0->L1; 1: y, L1->L2; 2: z, L2->L0) reading `in`,
// an array in that axis' input layout (L0, L1 or L2)
SweepArgs sweep_args(const ads_handle* h, int axis, const void* fac, const void* in) {
  SweepArgs a{};
  const int* N = h->g.N;
  const Geometry& g = h->g;
  a.L = N[axis];
  a.in = in;
  if (axis == 0) {  // lines y, tiles over z: x + PX (y + Ny z)
    a.lanes_total = N[1]; a.lane_dim = 1; a.out_line_dim = 1; a.third_extent = N[2];
    a.in_ls = g.PX; a.in_t3s = g.PX * (long long)N[1];
  }
  if (axis == 1) {  // lines z, tiles over x: y + PY (x + Nx z)
    a.lanes_total = N[2]; a.lane_dim = 2; a.out_line_dim = 2; a.third_extent = N[0];
    a.in_ls = g.PY * (long long)N[0]; a.in_t3s = g.PY;
  }
  if (axis == 2) {  // lines x, tiles over y: z + PZ (x + Nx y)
    a.lanes_total = N[0]; a.lane_dim = 1; a.out_line_dim = 2; a.third_extent = N[1];
    a.in_ls = g.PZ; a.in_t3s = g.PZ * (long long)N[0];
  }
  a.tiles_lane = (a.lanes_total + SW_LANES - 1) / SW_LANES;
  a.fac = fac;
  a.in_scale = 1.0;
  a.err = h->d_flags + FL_ERR;
  return a;
}
int sweep_grid(const ads_handle* h, int axis) {
  const int* N = h->g.N;
  if (axis == 0) return ((N[1] + SW_LANES - 1) / SW_LANES) * N[2];
  if (axis == 1) return ((N[2] + SW_LANES - 1) / SW_LANES) * N[0];
  return ((N[0] + SW_LANES - 1) / SW_LANES) * N[1];
}

AssembleArgs assemble_args(const ads_handle* h, const double* u, double* F, bool with_f) {
  AssembleArgs a{};
  a.g = h->g;
  a.form = h->form;
  a.zc = h->asm_zc;
  a.nix = h->asm_nix; a.niy = h->asm_niy; a.niz = h->asm_niz;
  a.dt = h->dt;
  a.kappa = h->kappa;
  a.u = u;
  a.u_px = h->g.PX;
  a.F = F;
  a.shadow = h->d_shadow;
  a.shadow_stride = (long long)h->n0;
  a.fqp = (with_f && h->has_f) ? h->d_fqp : nullptr;
  a.kqp = h->has_k ? h->d_kqp : nullptr;
  a.dqp = h->has_oil ? h->d_dqp : nullptr;
  a.mu = h->mu;
  a.l2part = h->d_l2part;
  a.err = h->d_flags + FL_ERR;
  return a;
}

FixupArgs fixup_args(const ads_handle* h, double* F) {
  FixupArgs f{};
  f.g = h->g;
  f.zc = h->asm_zc;
  f.nix = h->asm_nix; f.niy = h->asm_niy; f.niz = h->asm_niz;
  f.F = F;
  f.shadow = h->d_shadow;
  f.shadow_stride = (long long)h->n0;
  f.l2part = h->d_l2part;
  f.nl2 = h->asm_grid;
  f.scal = h->d_scal;
  f.slab = h->d_slab;
  f.xslab = h->d_xslab;
  f.nxslab = h->nxslab;
  return f;
}

ResidualArgs residual_args(const ads_handle* h, const double* u, const double* F, double* r) {
  ResidualArgs a{};
  a.g = h->g;
  a.zc = h->rsd_zc;
  a.nix = h->res_nix; a.niy = h->res_niy; a.niz = h->rsd_niz;
  a.u = u; a.F = F; a.r = r;
  for (int d = 0; d < 3; ++d) a.band[d] = h->d_band[d];
  a.part = h->d_part;
  a.err = h->d_flags + FL_ERR;
  return a;
}

// r = F - (Mx (x) My (x) Mz) u, or M u with F null (FP64)
int enqueue_mass(ads_handle* h, const double* u, const double* F, double* r, const char* name) {
  if (h->general) {
    RUN(h, name, 1, launch_residual_gen(h->g, u, F, r, h->d_band, h->stream));
    return ADS_OK;
  }
  ResidualArgs ra = residual_args(h, u, F, r);
  RUN(h, name, 1, launch_residual(h->P, ra, h->rsd_grid, h->stream));
  return ADS_OK;
}

// assembly (+ fixup) of F from coefficients u with the handle's form
// the general-geometry assembly (k_general.cu), FP64
int enqueue_assemble_gen(ads_handle* h, const double* u, double* F, bool incr, bool with_f, const double* kqp_override) {
  if (h->form == ADS_FORM_OIL)
    return fail(h, ADS_ERR_UNSUPPORTED, "the oil form needs equal degrees on all axes");
  GenAssembleArgs a{};
  a.g = h->g;
  a.form = h->form;
  a.incr = incr ? 1 : 0;
  a.dt = h->dt;
  a.kappa = h->kappa;
  a.u = u;
  a.F = F;
  a.fqp = (with_f && h->has_f) ? h->d_fqp : nullptr;
  a.kqp = kqp_override ? kqp_override : (h->has_k ? h->d_kqp : nullptr);
  for (int d = 0; d < 3; ++d) { a.nn[d] = h->d_nn64[d]; a.jw[d] = h->d_jw64[d]; }
  a.part = h->d_gpart;
  const int ncol = (h->p[0] + 1) * (h->p[1] + 1) * (h->p[2] + 1);
  RUN(h, "assemble_gen", ncol + 1, launch_assemble_gen(a, h->d_scal, h->stream));
  return ADS_OK;
}

DfTabs3 df_tabs(const ads_handle* h) {
  DfTabs3 tb;
  DfTab* t[3] = {&tb.x, &tb.y, &tb.z};
  for (int d = 0; d < 3; ++d) {
    t[d]->nn = h->d_nndf[d];
    t[d]->jw = h->d_jwdf[d];
    t[d]->sym = h->d_symdf[d];
    t[d]->symf = h->d_symf[d];
    t[d]->nnw = h->d_nnwdf[d];
    t[d]->symw = h->d_symwdf[d];
    t[d]->mat = d == 0 ? h->d_matdf : nullptr;
  }
  return tb;
}

int enqueue_assemble(ads_handle* h, const double* u, double* F, bool fp32, bool incr, bool with_f,
                     const double* kqp_override = nullptr) {
  Phase ph(h, "Form 3D RHS");
  if (h->general) return enqueue_assemble_gen(h, u, F, incr, with_f, kqp_override);
  AssembleArgs a = assemble_args(h, u, F, with_f);
  if (kqp_override) a.kqp = kqp_override;
  AxisTab<double> t64[3];
  AxisTab<float> t32[3];
  for (int d = 0; d < 3; ++d) {
    t64[d].nn = h->d_nn64[d]; t64[d].jw = h->d_jw64[d]; t64[d].dd = h->d_dd64[d];
    t32[d].nn = h->d_nn32[d]; t32[d].jw = h->d_jw32[d]; t32[d].dd = h->d_dd32[d];
  }
  // the FP32 heat assembly works on coefficients scaled by a power of two
  if (fp32 && (h->form == ADS_FORM_HEAT || h->form == ADS_FORM_OIL)) {
    RUN(h, "uscale", 2, launch_uscale(u, (long long)h->n0, h->d_part, h->norm_parts, h->d_scal, h->stream));
    h->uscale_set = true;
  }
  a.uscale = h->d_scal + SC_USCALE;
  int used = h->asm_grid;
  if (fp32 && incr && df_increment(h)) {
    RUN(h, "assemble_df", 1, launch_assemble_df(a, df_tabs(h), h->asm_grid, &used, h->stream));
  } else {
    const void* tx = fp32 ? (const void*)&t32[0] : (const void*)&t64[0];
    const void* ty = fp32 ? (const void*)&t32[1] : (const void*)&t64[1];
    const void* tz = fp32 ? (const void*)&t32[2] : (const void*)&t64[2];
    RUN(h, fp32 ? "assemble_f32" : "assemble_f64", 1,
        launch_assemble(fp32, incr, a, tx, ty, tz, h->asm_grid, &used, h->stream));
  }
  FixupArgs f = fixup_args(h, F);
  f.nl2 = used;
  if (fp32 && incr) f.g32 = h->d_g32;  // the heat increment also feeds the FP32 solve as float
  RUN(h, "fixup", 2, launch_fixup(f, h->stream));
  return ADS_OK;
}

// The double-float increment assembly of a step on a caller's array u
// (unpadded rows of N[0], read in place), on the coefficient scale the last
// assembly left in SC_USCALE instead of a pass over u: the fixup checks it
// against the max |u| the assembly saw, sets FL_UMISS when it was off and
// leaves the exact scale of u for the next step.
int enqueue_assemble_host(ads_handle* h, const double* u) {
  Phase ph(h, "Form 3D RHS");
  if (!h->uscale_set) {
    // no scale to start from yet: a pass over u (through the host link)
    const long long n = (long long)h->g.N[0] * h->g.N[1] * h->g.N[2];
    RUN(h, "uscale", 2, launch_uscale(u, n, h->d_part, h->norm_parts, h->d_scal, h->stream));
    h->uscale_set = true;
  }
  AssembleArgs a = assemble_args(h, u, h->d_F, true);
  a.u_px = h->g.N[0];
  a.u_copy = h->d_u;  // u becomes the handle's coefficients on the way (HBM writes)
  a.uscale = h->d_scal + SC_USCALE;
  int used = h->asm_grid;
  RUN(h, "assemble_df", 1, launch_assemble_df(a, df_tabs(h), h->asm_grid, &used, h->stream));
  FixupArgs f = fixup_args(h, h->d_F);
  f.nl2 = used;
  f.g32 = h->d_g32;
  f.umiss = h->d_flags + FL_UMISS;
  RUN(h, "fixup", 2, launch_fixup(f, h->stream));
  return ADS_OK;
}

// FP64 Kronecker solve: in (L0) -> out (L0, through the map tm_out on the
// sweep path).  Banded geometry: in is copied to out and each direction is
// solved in place by k_band_solve with the mass matrix's LU (M is symmetric,
// so the transposed solve is the same).
int enqueue_solve64(ads_handle* h, const double* in, const CUtensorMap* tm_out, bool trans, double* out) {
  if (h->banded) {
    const Geometry& g = h->g;
    const long long Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
    if (in != out) ADS_CUDA(h, cudaMemcpyAsync(out, in, sizeof(double) * h->n0, cudaMemcpyDeviceToDevice, h->stream));
    { Phase ph(h, "Solve 1"); RUN(h, "band_solve_x", 1, launch_band_solve(out, Ny, Nz, g.PX, g.PX * Ny, 1, (int)Nx, h->p[0], h->p[0],
                                                h->d_gab[0], h->d_gpiv[0], h->stream)); }
    { Phase ph(h, "Solve 2"); RUN(h, "band_solve_y", 1, launch_band_solve(out, Nx, Nz, 1, g.PX * Ny, g.PX, (int)Ny, h->p[1], h->p[1],
                                                h->d_gab[1], h->d_gpiv[1], h->stream)); }
    { Phase ph(h, "Solve 3"); RUN(h, "band_solve_z", 1, launch_band_solve(out, Nx, Ny, 1, g.PX, g.PX * Ny, (int)Nz, h->p[2], h->p[2],
                                                h->d_gab[2], h->d_gpiv[2], h->stream)); }
    return ADS_OK;
  }
  double* const* fac = trans ? h->d_tfac64 : h->d_fac64;
  SweepArgs ax = sweep_args(h, 0, fac[0], in);
  { Phase ph(h, "Solve 1"); RUN(h, "sweep_x_f64", 1, launch_sweep(h->P, 0, 0, 0, trans, &h->tm_wA_out64, ax, sweep_grid(h, 0), h->stream)); }
  SweepArgs ay = sweep_args(h, 1, fac[1], h->d_wA);
  { Phase ph(h, "Solve 2"); RUN(h, "sweep_y_f64", 1, launch_sweep(h->P, 0, 0, 0, trans, &h->tm_wB_out64, ay, sweep_grid(h, 1), h->stream)); }
  SweepArgs az = sweep_args(h, 2, fac[2], h->d_wB);
  { Phase ph(h, "Solve 3"); RUN(h, "sweep_z_f64", 1, launch_sweep(h->P, 0, 0, 0, trans, tm_out, az, sweep_grid(h, 2), h->stream)); }
  return ADS_OK;
}

// FP32 Kronecker solve of an L0 input (tin 0: double, scaled by *in_scale on
// load; tin 1: float, already scaled): final_mode 1 writes out = s x (FP64),
// final_mode 0 writes x itself (FP32) into d_x32.  x sweep L0 -> L1 (wA) and
// y sweep L1 -> L0 (wC) in the skewed form of k_sweep (their lines are
// contiguous along the solve direction), the y sweep with its lanes along x
// so that its TMA-stored chunks land in L0; z sweep L0 -> L0 in the column
// form of k_csweep (lines x contiguous: 16-byte row copies, each solution
// row stored straight out).
int enqueue_solve32(ads_handle* h, const void* in, int tin, const double* in_scale, const double* out_scale,
                    int final_mode, const int* skip, const char* tag, double* out) {
  const Geometry& g = h->g;
  const long long Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
  std::string nx = std::string("sweep_x_f32") + tag, ny = std::string("sweep_y_f32") + tag,
              nz = std::string("sweep_z_f32") + tag;
  SweepArgs ax = sweep_args(h, 0, h->d_fac32[0], in);
  ax.in_scale_dev = in_scale;
  ax.skip_flag = skip;
  // x: skewed, without the transpose, into wC (L0)
  const bool corr = tag[0] != '\0';  // a refinement correction, not the first solve
  if (tin == 1) {
    // FP32 input: the column-form x sweep (lines y, positions x contiguous) into wC
    CSweepArgs cx{};
    cx.L = (int)Nx; cx.nl = (int)Ny; cx.n3 = (int)Nz;
    cx.in = static_cast<const float*>(in);
    cx.in_ls = g.PX; cx.in_ps = 1; cx.in_ts = g.PX * Ny;
    cx.out = h->d_wC;
    cx.out_ls = g.PX; cx.out_ps = 1; cx.out_ts = g.PX * Ny;
    cx.fac = h->d_fac32[0];
    cx.skip_flag = skip;
    Phase ph(h, corr ? "Refinement" : "Solve 1");
    RUN(h, nx.c_str(), 1, launch_xsweep(h->P, cx, h->stream));
  } else {
    // FP64 input (a caller's right-hand side), scaled on load: the skewed form
    Phase ph(h, corr ? "Refinement" : "Solve 1");
    RUN(h, nx.c_str(), 1, launch_sweep(h->P, tin, 1, 4, false, &h->tm_wC_out32, ax, sweep_grid(h, 0), h->stream));
  }
  // y: column form in place on wC (lines x contiguous, positions y at stride PX, tiles over z)
  CSweepArgs cy{};
  cy.L = (int)Ny; cy.nl = (int)Nx; cy.n3 = (int)Nz;
  cy.in = h->d_wC;
  cy.in_ls = 1; cy.in_ps = g.PX; cy.in_ts = g.PX * Ny;
  cy.out = h->d_wC;
  cy.out_ps = g.PX; cy.out_ts = g.PX * Ny;
  cy.fac = h->d_fac32[1];
  cy.skip_flag = skip;
  { Phase ph(h, corr ? "Refinement" : "Solve 2"); RUN(h, ny.c_str(), 1, launch_csweep(h->P, 0, cy, h->stream)); }
  CSweepArgs cz{};
  cz.L = (int)Nz; cz.nl = (int)Nx; cz.n3 = (int)Ny;
  cz.in = h->d_wC;
  cz.in_ls = 1; cz.in_ps = g.PX * Ny; cz.in_ts = g.PX;
  cz.out = final_mode == 1 ? static_cast<void*>(out) : static_cast<void*>(h->d_x32);
  cz.out_ps = g.PX * Ny; cz.out_ts = g.PX;
  cz.fac = h->d_fac32[2];
  cz.out_scale_dev = out_scale;
  cz.skip_flag = skip;
  { Phase ph(h, corr ? "Refinement" : "Solve 3"); RUN(h, nz.c_str(), 1, launch_csweep(h->P, final_mode, cz, h->stream)); }
  return ADS_OK;
}

// Mixed-precision Kronecker solve of d_F into x with FP64 iterative refinement:
// x = M^{-1} F by FP32 sweeps, then up to max_refine rounds of: FP64 residual
// r = F - M x, FP32 correction x1 = M^{-1} r, x += x1 and the updated residual
// r - M x1 with its certified bound (k_resid_update, k_certify), stopping once
// the bound, or an FP64 residual, is <= refine_tol ||F||.
// f32_input: the fixup already wrote F 2^-e as float into d_g32 (the heat
// increment); otherwise the first x sweep reads FP64 F and scales it on load.
// Each FP64 residual is written to d_g32 with the same scale 2^-e.
int enqueue_solve_mixed(ads_handle* h, double* x, bool scales_ready, bool f32_input) {
  // the first solve's scale comes from the assembly (fixup) or, for a caller's F, from a norm pass
  if (!scales_ready) RUN(h, "norm_f", 2, launch_norm_f(h->d_F, h->g, h->d_part, h->norm_parts, h->d_scal, h->stream));
  const double* in_s = h->d_scal + SC_IN_SCALE;
  const double* out_s = h->d_scal + SC_OUT_SCALE;
  int st = f32_input ? enqueue_solve32(h, h->d_g32, 1, nullptr, out_s, 1, nullptr, "", x)
                     : enqueue_solve32(h, h->d_F, 0, in_s, out_s, 1, nullptr, "", x);
  if (st) return st;
  const int* conv = h->d_flags + FL_CONV;
  Phase ph(h, "Refinement");
  // launches of the first round keep the plain timer names; those of later
  // rounds (which return at once once the refinement has converged) are
  // timed as *_late, so a timer never mixes working and returning launches
  auto residual = [&](bool want_ff, bool late) -> int {
    ResidualArgs ra = residual_args(h, x, h->d_F, h->d_r);
    ra.skip_flag = conv;
    ra.want_ff = want_ff;
    ra.r32 = h->d_g32;
    ra.r32_scale = in_s;
    RUN(h, late ? "residual_f64_late" : "residual_f64", 1, launch_residual(h->P, ra, h->rsd_grid, h->stream));
    return ADS_OK;
  };
  UpdateArgs ua{};
  ua.g = h->g;
  ua.zc = h->res_zc;
  ua.nix = h->res_nix; ua.niy = h->upd_niy; ua.niz = h->res_niz;
  ua.x1 = h->d_x32;
  ua.r1 = h->d_g32;
  ua.delta = x;
  ua.out_scale = out_s;
  for (int d = 0; d < 3; ++d) ua.band[d] = h->d_band32[d];
  ua.part = h->d_part;
  ua.skip_flag = conv;
  const long long ndof = (long long)h->g.N[0] * h->g.N[1] * h->g.N[2];
  for (int k = 0; k < h->opts.max_refine; ++k) {
    const bool late = k > 0;
    if ((st = residual(k == 0, late))) return st;
    RUN(h, late ? "decide_late" : "decide", 1,
        launch_decide(h->d_part, h->rsd_grid, h->opts.refine_tol, true, k == 0, h->d_scal, h->d_flags, h->stream));
    if ((st = enqueue_solve32(h, h->d_g32, 1, nullptr, nullptr, 0, conv, late ? "_corr_late" : "_corr", nullptr)))
      return st;
    RUN(h, late ? "resid_update_late" : "resid_update", 1, launch_resid_update(h->P, ua, h->upd_grid, h->stream));
    RUN(h, late ? "certify_late" : "certify", 1,
        launch_certify(h->d_part, h->upd_grid, h->P, ndof, h->opts.refine_tol, h->d_scal, h->d_flags, h->stream));
  }
  const bool late = h->opts.max_refine > 0;
  if ((st = residual(!late, late))) return st;
  RUN(h, late ? "decide_late" : "decide", 1,
      launch_decide(h->d_part, h->rsd_grid, h->opts.refine_tol, false, !late, h->d_scal, h->d_flags, h->stream));
  return ADS_OK;
}

int enqueue_solve(ads_handle* h) {
  if (is_mixed(h)) return enqueue_solve_mixed(h, h->d_u, false, false);
  return enqueue_solve64(h, h->d_F, &h->tm_u_out64, false, h->d_u);
}

// one Step (src/ADS.F90:437-461): FormUn+Form3DRHS, three sweeps, R := F.
// FP64: assemble F, solve M u = F.
// Mixed, heat form (increment form): with exact Gauss quadrature the mass part
// of F is M u^n, so G = F - M u^n is assembled in FP32 from the remaining
// terms, M delta = G is solved with FP64 refinement, and u^{n+1} = u^n + delta
// in FP64; the FP32 rounding then scales with |delta|, not |u|.
// Mixed, projection form (the t = 0 step): F in FP64, refined solve into u.
int enqueue_step(ads_handle* h) {
  RUN(h, "step_reset", 1, launch_step_reset(h->d_scal, h->d_flags, h->stream));
  int st;
  if (is_mixed(h) && (h->form == ADS_FORM_HEAT || h->form == ADS_FORM_OIL)) {
    if ((st = enqueue_assemble(h, h->d_u, h->d_F, true, true, true))) return st;
    if ((st = enqueue_solve_mixed(h, h->d_delta, true, true))) return st;
    Phase ph(h, "Update");
    RUN(h, "update", 1, launch_add(h->d_u, h->d_delta, (long long)h->n0, h->stream));
  } else if (is_mixed(h)) {
    if ((st = enqueue_assemble(h, h->d_u, h->d_F, false, false, true))) return st;
    if ((st = enqueue_solve_mixed(h, h->d_u, true, false))) return st;
  } else {
    if ((st = enqueue_assemble(h, h->d_u, h->d_F, false, false, true))) return st;
    if ((st = enqueue_solve64(h, h->d_F, &h->tm_u_out64, false, h->d_u))) return st;
  }
  RUN(h, "record", 1, launch_record(h->d_scal, h->d_flags, h->d_hist, h->hist_cap, h->stream));
  return ADS_OK;
}

// The mixed heat step on a caller's arrays (device-addressable, unpadded):
// the assembly reads u_in in place and copies it into d_u, the update writes
// d_u + delta into d_u and u_out, unless the scale check failed (then the
// update writes nothing).
int enqueue_step_host(ads_handle* h, const double* u_in, double* u_out) {
  RUN(h, "step_reset", 1, launch_step_reset(h->d_scal, h->d_flags, h->stream));
  int st;
  if ((st = enqueue_assemble_host(h, u_in))) return st;
  if ((st = enqueue_solve_mixed(h, h->d_delta, true, true))) return st;
  {
    Phase ph(h, "Update");
    RUN(h, "update_host", 1, launch_update_host(h->d_delta, h->d_u, u_out, h->g, h->d_flags + FL_UMISS, h->stream));
  }
  RUN(h, "record", 1, launch_record(h->d_scal, h->d_flags, h->d_hist, h->hist_cap, h->stream));
  return ADS_OK;
}

int check_flags(ads_handle* h) {
  int fl[FL_COUNT];
  ADS_CUDA(h, cudaMemcpyAsync(fl, h->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, h->stream));
  ADS_CUDA(h, cudaStreamSynchronize(h->stream));
  if (fl[FL_ERR]) return fail(h, ADS_ERR_DEVICE, "a kernel reported error bits " + std::to_string(fl[FL_ERR]));
  return ADS_OK;
}

int ensure_hist(ads_handle* h, int cap) {
  if (cap <= h->hist_cap) return ADS_OK;
  if (h->d_hist) cudaFree(h->d_hist);
  h->d_hist = nullptr;
  ADS_CUDA(h, cudaMalloc(&h->d_hist, sizeof(double) * HIST_W * (size_t)cap));
  h->hist_cap = cap;
  h->graph_valid = false;
  return ADS_OK;
}

void invalidate_graph(ads_handle* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  h->gexec = nullptr;
  h->graph_valid = false;
}

int build_graph(ads_handle* h) {
  invalidate_graph(h);
  cudaGraph_t graph = nullptr;
  ADS_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
  const long long before = h->launches;
  int st = enqueue_step(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  if (st) { if (graph) cudaGraphDestroy(graph); return st; }
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
  h->graph_launches = h->launches - before;
  h->launches = before;
  e = cudaGraphInstantiate(&h->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
  h->graph_valid = true;
  return ADS_OK;
}

int finish_stats(ads_handle* h, int k, double* l2norms) {
  int st = check_flags(h);
  if (st) return st;
  std::vector<double> hist((size_t)HIST_W * k);
  ADS_CUDA(h, cudaMemcpy(hist.data(), h->d_hist, sizeof(double) * HIST_W * (size_t)k, cudaMemcpyDeviceToHost));
  for (int i = 0; i < k; ++i)
    if (l2norms) l2norms[i] = hist[HIST_W * i];
  const double* last = &hist[HIST_W * (size_t)(k - 1)];
  h->last.l2norm = last[0];
  const bool mixed = is_mixed(h);
  h->last.rel_residual = mixed ? last[1] : 0.0;
  h->last.refinements = mixed ? (int)last[2] : 0;
  h->last.converged = mixed ? (int)last[3] : 1;
  h->last.fp64_residuals = mixed ? (int)last[4] : 0;
  h->last.host_path = 0;
  for (int i = 0; i < k; ++i)
    if (!std::isfinite(hist[HIST_W * i])) return fail(h, ADS_ERR_NONFINITE, "non-finite l2norm");
  if (mixed) {
    for (int i = 0; i < k; ++i)
      if (hist[HIST_W * i + 3] == 0.0)
        return fail(h, ADS_ERR_NOCONV, "iterative refinement did not reach refine_tol (relative residual " +
                                          std::to_string(hist[HIST_W * i + 1]) + ")");
  }
  return ADS_OK;
}

// element layers per z-chunk of the assembly: halve until there are enough
// work items, but never below p (the z spill of a chunk, p DOF planes, must
// lie inside the next chunk) nor below 4
int pick_zc(int E, int per_xy, int resident, int zmin) {
  int zc = E;
  while (true) {
    const int next = (zc + 1) / 2;
    if (next < zmin || next >= zc) break;
    if ((long long)per_xy * ((E + zc - 1) / zc) >= 4LL * resident) break;
    zc = next;
  }
  return zc;
}

void free_all(ads_handle* h) {
  invalidate_graph(h);
  for (int d = 0; d < 3; ++d) {
    cudaFree(h->d_nn64[d]); cudaFree(h->d_jw64[d]); cudaFree(h->d_nn32[d]); cudaFree(h->d_jw32[d]);
    cudaFree(h->d_dd64[d]); cudaFree(h->d_dd32[d]);
    cudaFree(h->d_fac64[d]); cudaFree(h->d_tfac64[d]); cudaFree(h->d_fac32[d]); cudaFree(h->d_band[d]);
    cudaFree(h->d_band32[d]); cudaFree(h->d_nndf[d]); cudaFree(h->d_jwdf[d]);
    cudaFree(h->d_symdf[d]); cudaFree(h->d_symf[d]); cudaFree(h->d_nnwdf[d]); cudaFree(h->d_symwdf[d]);
    if (d == 0) cudaFree(h->d_matdf);
    cudaFree(h->d_gab[d]); cudaFree(h->d_gpiv[d]);
  }
  cudaFree(h->d_gpart);
  cudaFree(h->d_u); cudaFree(h->d_F); cudaFree(h->d_r); cudaFree(h->d_delta); cudaFree(h->d_g32); cudaFree(h->d_x32); cudaFree(h->d_wC); cudaFree(h->d_wA); cudaFree(h->d_wB);
  cudaFree(h->d_shadow); cudaFree(h->d_fqp); cudaFree(h->d_kqp); cudaFree(h->d_dqp); cudaFree(h->d_l2part); cudaFree(h->d_stage); cudaFree(h->d_un); cudaFree(h->d_ms);
  for (int d = 0; d < 3; ++d) { cudaFree(h->d_mab[d]); cudaFree(h->d_mpiv[d]); } cudaFree(h->d_slab); cudaFree(h->d_xslab);
  cudaFree(h->d_part); cudaFree(h->d_scal); cudaFree(h->d_flags); cudaFree(h->d_hist);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (cudaEvent_t ev : h->evpool) cudaEventDestroy(ev);
  h->evpool.clear();
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

int create_impl(ads_handle* h) {
  ADS_CUDA(h, cudaSetDevice(h->dev));
  ADS_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->own_stream = true;
  ADS_CUDA(h, cudaEventCreate(&h->ev0));
  ADS_CUDA(h, cudaEventCreate(&h->ev1));
  if (!get_encode()) return fail(h, ADS_ERR_CUDA, "cuTensorMapEncodeTiled is not available");

  for (int d = 0; d < 3; ++d) {
    if (axis_setup(h->n[d], h->p[d], h->ax[d])) return fail(h, ADS_ERR_UNSUPPORTED, "axis setup failed");
    if (h->ax[d].E < 2) return fail(h, ADS_ERR_UNSUPPORTED, "the GPU path needs at least 2 elements per axis");
  }
  Geometry& g = h->g;
  g.P = h->P;
  g.Q = h->Q;
  for (int d = 0; d < 3; ++d) {
    g.E[d] = h->ax[d].E;
    g.N[d] = h->ax[d].N;
    g.p[d] = h->p[d];
    g.q[d] = h->p[d] + 1;
  }
  // unequal degrees: the general kernels; an axis longer than the sweeps'
  // shared-memory lines: banded solves (with the tuned assembly and residual
  // when the degrees are equal).  Both are FP64 paths.
  // (and an x axis beyond the fixup's one-CTA rows of 4096 DOFs)
  h->general = !(h->p[0] == h->p[1] && h->p[1] == h->p[2]) || g.N[0] > 4096;
  h->banded = h->general;
  for (int d = 0; d < 3; ++d)
    if (g.N[d] > ADS_MAX_AXIS_DOFS) h->banded = true;
  if (h->banded && is_mixed(h))
    return fail(h, ADS_ERR_UNSUPPORTED, "mixed precision needs equal degrees and at most 448 DOFs per axis");
  g.PX = round_up(g.N[0], 8);
  g.PY = round_up(g.N[1], 8);
  g.PZ = round_up(g.N[2], 8);
  h->n0 = (size_t)g.PX * g.N[1] * g.N[2];
  h->n1 = (size_t)g.PY * g.N[0] * g.N[2];
  h->n2 = (size_t)g.PZ * g.N[0] * g.N[1];
  h->nqp = (long long)g.E[0] * g.E[1] * g.E[2] * g.q[0] * g.q[1] * g.q[2];

  for (int d = 0; d < 3; ++d) {
    const AxisHost& a = h->ax[d];
    std::vector<double> fac, tfac;
    if (band_factor(a, fac, tfac)) return fail(h, ADS_ERR_ZERO_PIVOT, "zero pivot in the 1-D mass matrix");
    if (h->banded) {
      // the mass matrix in LAPACK band storage with its banded LU (MKBBT's
      // mass mix; the mass matrix is SPD, so the LU does not pivot)
      const double mass[4] = {1.0, 0.0, 0.0, 0.0};
      std::vector<double> AB;
      mix_band(a, mass, AB);
      std::vector<int> ipiv(a.N);
      if (band_lu(a.N, a.p, a.p, AB.data(), 3 * a.p + 1, ipiv.data()))
        return fail(h, ADS_ERR_ZERO_PIVOT, "zero pivot in the 1-D mass matrix");
      int st;
      if ((st = upload(h, &h->d_gab[d], AB))) return st;
      if ((st = upload(h, &h->d_gpiv[d], ipiv))) return st;
    }
    std::vector<float> nn32(a.NN.begin(), a.NN.end()), jw32(a.JW.begin(), a.JW.end()), fac32(fac.begin(), fac.end());
    std::vector<float> dd32(a.DD.begin(), a.DD.end());
    // double-float copy of a table: the nearest float and the float nearest to the remainder
    auto split = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const float hi = (float)v[i];
        o[i] = make_float2(hi, (float)(v[i] - (double)hi));
      }
      return o;
    };
    int st;
    if ((st = upload(h, &h->d_nn64[d], a.NN))) return st;
    if ((st = upload(h, &h->d_jw64[d], a.JW))) return st;
    if ((st = upload(h, &h->d_nn32[d], nn32))) return st;
    if ((st = upload(h, &h->d_jw32[d], jw32))) return st;
    if ((st = upload(h, &h->d_dd64[d], a.DD))) return st;
    if ((st = upload(h, &h->d_dd32[d], dd32))) return st;
    if ((st = upload(h, &h->d_fac64[d], fac))) return st;
    if ((st = upload(h, &h->d_tfac64[d], tfac))) return st;
    if ((st = upload(h, &h->d_fac32[d], fac32))) return st;
    if ((st = upload(h, &h->d_band[d], a.band))) return st;
    if ((st = upload(h, &h->d_band32[d], split(a.band)))) return st;
    if (h->opts.precision == ADS_PREC_MIXED) {
      if ((st = upload(h, &h->d_nndf[d], split(a.NN)))) return st;
      if ((st = upload(h, &h->d_jwdf[d], split(a.JW)))) return st;
      // the tables with J W folded in: N[e][k][b] J(e) W(k)
      AxisHost aw = a;
      for (int e = 0; e < a.E; ++e)
        for (int k = 0; k < a.q; ++k)
          for (int i = 0; i < (a.p + 1) * 2; ++i) aw.NN[((size_t)e * a.q + k) * (a.p + 1) * 2 + i] *= a.JW[(size_t)e * a.q + k];
      if ((st = upload(h, &h->d_nnwdf[d], split(aw.NN)))) return st;
      if (d == 0 && (st = upload(h, &h->d_matdf, split(element_matrices(a))))) return st;
      if (df_sym_count(a.p) > 0) {
        std::vector<double> sc, scw;
        std::vector<unsigned char> sf, sfw;
        even_odd_tables(a, sc, sf);
        even_odd_tables(aw, scw, sfw);
        for (size_t e = 0; e < sf.size(); ++e) sf[e] = sf[e] && sfw[e];
        if ((st = upload(h, &h->d_symdf[d], split(sc)))) return st;
        if ((st = upload(h, &h->d_symwdf[d], split(scw)))) return st;
        if ((st = upload(h, &h->d_symf[d], sf))) return st;
      }
    }
  }

  auto zalloc = [&](double** p, size_t n) -> int {
    ADS_CUDA(h, cudaMalloc((void**)p, sizeof(double) * std::max<size_t>(n, 1)));
    ADS_CUDA(h, cudaMemset(*p, 0, sizeof(double) * std::max<size_t>(n, 1)));
    return ADS_OK;
  };
  int st;
  if ((st = zalloc(&h->d_u, h->n0))) return st;
  if ((st = zalloc(&h->d_F, h->n0))) return st;
  if ((st = zalloc(&h->d_r, h->n0))) return st;
  if (is_mixed(h) && (st = zalloc(&h->d_delta, h->n0))) return st;
  if (is_mixed(h)) {
    double* g32 = nullptr;
    if ((st = zalloc(&g32, (h->n0 + 1) / 2))) return st;
    h->d_g32 = reinterpret_cast<float*>(g32);
    double* x32 = nullptr;
    if ((st = zalloc(&x32, (h->n0 + 1) / 2))) return st;
    h->d_x32 = reinterpret_cast<float*>(x32);
    double* wc = nullptr;
    if ((st = zalloc(&wc, (h->n0 + 1) / 2))) return st;
    h->d_wC = reinterpret_cast<float*>(wc);
  }
  if (!h->banded && (st = zalloc(&h->d_wA, h->n1))) return st;
  if (!h->banded && (st = zalloc(&h->d_wB, h->n2))) return st;
  if (!h->general && (st = zalloc(&h->d_shadow, 7 * h->n0))) return st;
  if (h->general && (st = zalloc(&h->d_gpart, (size_t)assemble_gen_parts(g)))) return st;

  // assembly launch geometry
  cudaDeviceProp prop;
  ADS_CUDA(h, cudaGetDeviceProperties(&prop, h->dev));
  const int nsm = prop.multiProcessorCount;
  const size_t smem_max = prop.sharedMemPerMultiprocessor;
  int pageable = 0;
  ADS_CUDA(h, cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->dev));
  h->pageable = pageable != 0;
  if (!h->general) {
    // expected residency of the step's assembly: the FP32 kernel 3 CTAs/SM at
    // p <= 2, else 2; the double-float and FP64 kernels 2 at p <= 2, else 1
    // (registers)
    const bool f32 = h->opts.precision == ADS_PREC_MIXED_FAST;
    const bool df = h->opts.precision == ADS_PREC_MIXED;
    const size_t b = (df ? assemble_df_smem_bytes(h->P) : assemble_smem_bytes(h->P, f32)) + 1024;
    int per_sm = (int)std::min<size_t>(smem_max / b, f32 ? (h->P <= 2 ? 3 : 2) : (h->P <= 2 ? 2 : 1));
    if (per_sm < 1) per_sm = 1;
    const int resident = nsm * per_sm;
    h->asm_nix = (g.E[0] + as_tx(h->P) - 1) / as_tx(h->P);
    h->asm_niy = (g.E[1] + AS_TY - 1) / AS_TY;
    h->asm_zc = pick_zc(g.E[2], h->asm_nix * h->asm_niy, resident, std::max(h->P, 4));
    h->asm_niz = (g.E[2] + h->asm_zc - 1) / h->asm_zc;
    h->asm_grid = nsm * 8;  // bound of persistent CTAs; the launch uses the real residency
  }
  if (!h->general) {
    h->res_nix = (g.N[0] + RS_TX - 1) / RS_TX;
    h->res_niy = (g.N[1] + RS_TY - 1) / RS_TY;
    h->res_zc = std::min(g.N[2], 32);
    h->res_niz = (g.N[2] + h->res_zc - 1) / h->res_zc;
    h->res_grid = h->res_nix * h->res_niy * h->res_niz;
    h->upd_niy = (g.N[1] + resid_update_rows() - 1) / resid_update_rows();
    h->upd_grid = h->res_nix * h->upd_niy * h->res_niz;
    // k_residual streams its chunk plus a p-plane halo on each side: pick the
    // chunk that fills whole waves of resident CTAs with the least halo work,
    // min over zc of ceil(CTAs / resident) * (zc + 2p)
    const int resident = nsm * std::max(1, residual_ctas_per_sm(h->P));
    long long best = -1;
    for (int zc = std::min(g.N[2], std::max(8, 2 * h->P)); zc <= std::min(g.N[2], 128); ++zc) {
      const int niz = (g.N[2] + zc - 1) / zc;
      const long long ctas = (long long)h->res_nix * h->res_niy * niz;
      const long long cost = (ctas + resident - 1) / resident * (long long)(zc + 2 * h->P);
      if (best < 0 || cost < best) { best = cost; h->rsd_zc = zc; }
    }
    h->rsd_niz = (g.N[2] + h->rsd_zc - 1) / h->rsd_zc;
    h->rsd_grid = h->res_nix * h->res_niy * h->rsd_niz;
  }
  if (!h->general) {
    // spill-slab membership of each DOF index (the assembly's bricks spill the
    // first p DOFs of every brick after the first one into the shadows)
    auto in_slab = [&](int v, int tile, int nitems) { return v >= tile && (v % tile) < h->P && (v / tile) <= nitems - 1; };
    std::vector<unsigned char> sl((size_t)g.N[0] + g.N[1] + g.N[2], 0);
    for (int x = 0; x < g.N[0]; ++x) sl[x] = in_slab(x, as_tx(h->P), h->asm_nix) ? 1 : 0;
    for (int y = 0; y < g.N[1]; ++y) sl[g.N[0] + y] = in_slab(y, AS_TY, h->asm_niy) ? 1 : 0;
    for (int z = 0; z < g.N[2]; ++z) sl[g.N[0] + g.N[1] + z] = in_slab(z, h->asm_zc, h->asm_niz) ? 1 : 0;
    ADS_CUDA(h, cudaMalloc(&h->d_slab, sl.size()));
    ADS_CUDA(h, cudaMemcpy(h->d_slab, sl.data(), sl.size(), cudaMemcpyHostToDevice));
    std::vector<int> xs;
    for (int x = 0; x < g.N[0]; ++x)
      if (sl[x]) xs.push_back(x);
    h->nxslab = (int)xs.size();
    ADS_CUDA(h, cudaMalloc(&h->d_xslab, sizeof(int) * std::max<size_t>(xs.size(), 1)));
    if (!xs.empty()) ADS_CUDA(h, cudaMemcpy(h->d_xslab, xs.data(), sizeof(int) * xs.size(), cudaMemcpyHostToDevice));
  }
  h->norm_parts = 4 * nsm;
  h->npart = std::max(3 * std::max(std::max(h->res_grid, h->rsd_grid), h->upd_grid), 2 * h->norm_parts);
  if ((st = zalloc(&h->d_l2part, 4 * (size_t)h->asm_grid))) return st;
  if ((st = zalloc(&h->d_part, (size_t)h->npart))) return st;
  if ((st = zalloc(&h->d_scal, SC_COUNT))) return st;
  ADS_CUDA(h, cudaMalloc(&h->d_flags, sizeof(int) * FL_COUNT));
  ADS_CUDA(h, cudaMemset(h->d_flags, 0, sizeof(int) * FL_COUNT));
  if ((st = ensure_hist(h, 64))) return st;

  if (h->banded) return ADS_OK;  // no sweep, no tensor map
  bool ok = true;
  ok &= make_l0_out(h, &h->tm_u_out64, h->d_u, false);
  ok &= make_l0_out(h, &h->tm_r_out64, h->d_r, false);
  ok &= make_l1_out(h, &h->tm_wA_out64, h->d_wA, false);
  ok &= make_l2_out(h, &h->tm_wB_out64, h->d_wB, false);
  // the FP32 x sweep's output: L0 chunks of SW_CH x (positions) by 32 y (lines)
  if (h->d_wC) ok &= encode(&h->tm_wC_out32, h->d_wC, true, h->g.N[0], h->g.N[1], h->g.N[2], h->g.PX, SW_CH, SW_LANES, 1);
  if (!ok) return fail(h, ADS_ERR_CUDA, "cuTensorMapEncodeTiled rejected a layout");
  return ADS_OK;
}

// host <-> device copies between the packed user layouts and the padded ones
// Host copies go through a packed device buffer with one contiguous copy each
// (a pitched 2-D copy moves the 2 KB rows one by one over the host link) and
// an on-device repack; a caller's device array is repacked directly.
int ensure_stage(ads_handle* h) {
  if (h->d_stage) return ADS_OK;
  const size_t n = (size_t)h->g.N[0] * h->g.N[1] * h->g.N[2];
  ADS_CUDA(h, cudaMalloc((void**)&h->d_stage, sizeof(double) * n));
  return ADS_OK;
}
// A pointer the handle's device can dereference for a caller's buffer of
// doubles: the device pointer of pinned or registered host memory mapped for
// this device, device memory of this device, managed memory, or pageable host
// memory itself where the device reads pageable memory; null otherwise.
const double* device_view(const ads_handle* h, const void* p) {
  if (reinterpret_cast<uintptr_t>(p) % alignof(double)) return nullptr;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeUnregistered) return h->pageable ? static_cast<const double*>(p) : nullptr;
  if (at.type == cudaMemoryTypeDevice && at.device != h->dev) return nullptr;
  return static_cast<const double*>(at.devicePointer);
}

int copy_l0_in(ads_handle* h, double* d, const double* src, cudaMemcpyKind kind) {
  const size_t bytes = sizeof(double) * (size_t)h->g.N[0] * h->g.N[1] * h->g.N[2];
  if (kind == cudaMemcpyDeviceToDevice) {
    RUN(h, "repack", 1, launch_repack(src, d, h->g, true, h->stream));
    return ADS_OK;
  }
  int st = ensure_stage(h);
  if (st) return st;
  ADS_CUDA(h, cudaMemcpyAsync(h->d_stage, src, bytes, kind, h->stream));
  RUN(h, "repack", 1, launch_repack(h->d_stage, d, h->g, true, h->stream));
  return ADS_OK;
}
int copy_l0_out(ads_handle* h, double* dst, const double* d, cudaMemcpyKind kind) {
  const size_t bytes = sizeof(double) * (size_t)h->g.N[0] * h->g.N[1] * h->g.N[2];
  if (kind == cudaMemcpyDeviceToDevice) {
    RUN(h, "repack", 1, launch_repack(d, dst, h->g, false, h->stream));
    return ADS_OK;
  }
  int st = ensure_stage(h);
  if (st) return st;
  RUN(h, "repack", 1, launch_repack(d, h->d_stage, h->g, false, h->stream));
  ADS_CUDA(h, cudaMemcpyAsync(dst, h->d_stage, bytes, kind, h->stream));
  return ADS_OK;
}

}  // namespace

extern "C" {

int ads_default_opts(ads_opts* o) {
  if (!o) return ADS_ERR_ARG;
  o->precision = ADS_PREC_FP64;
  o->refine_tol = 1e-13;
  o->max_refine = 3;
  o->device = 0;
  return ADS_OK;
}

const char* ads_status_string(int s) {
  switch (s) {
    case ADS_OK: return "ok";
    case ADS_ERR_ARG: return "invalid argument";
    case ADS_ERR_CUDA: return "CUDA error";
    case ADS_ERR_ZERO_PIVOT: return "zero pivot";
    case ADS_ERR_NONFINITE: return "non-finite value";
    case ADS_ERR_NOCONV: return "refinement did not converge";
    case ADS_ERR_TIMEOUT: return "device wait timed out";
    case ADS_ERR_UNSUPPORTED: return "unsupported configuration";
    case ADS_ERR_STATE: return "call out of order";
    case ADS_ERR_ALLOC: return "allocation failed";
    case ADS_ERR_DEVICE: return "device error flag";
  }
  return "unknown status";
}

int ads_create(const int n[3], const int p[3], const ads_opts* opts, ads_handle** out) {
  if (!n || !p || !out) return ADS_ERR_ARG;
  *out = nullptr;
  for (int d = 0; d < 3; ++d)
    if (p[d] < 0 || n[d] < p[d]) return ADS_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (p[d] < 1 || p[d] > 4) return ADS_ERR_UNSUPPORTED;
  ads_handle* h = new (std::nothrow) ads_handle();
  if (!h) return ADS_ERR_ALLOC;
  for (int d = 0; d < 3; ++d) { h->n[d] = n[d]; h->p[d] = p[d]; }
  h->P = std::max(p[0], std::max(p[1], p[2]));
  h->Q = h->P + 1;
  if (opts) h->opts = *opts;
  else ads_default_opts(&h->opts);
  if (h->opts.precision != ADS_PREC_FP64 && h->opts.precision != ADS_PREC_MIXED &&
      h->opts.precision != ADS_PREC_MIXED_FAST) { delete h; return ADS_ERR_ARG; }
  if (h->opts.max_refine < 0 || h->opts.max_refine > 16 || !(h->opts.refine_tol >= 0.0)) { delete h; return ADS_ERR_ARG; }
  h->dev = h->opts.device;
  int st = create_impl(h);
  if (st) {
    free_all(h);
    delete h;
    return st;
  }
  *out = h;
  return ADS_OK;
}

int ads_destroy(ads_handle* h) {
  if (!h) return ADS_ERR_ARG;
  cudaSetDevice(h->dev);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return ADS_OK;
}

const char* ads_last_error(const ads_handle* h) { return h ? h->err.c_str() : "null handle"; }

int ads_dims(const ads_handle* h, int nelem[3], int ndof[3], int nq[3]) {
  if (!h) return ADS_ERR_ARG;
  for (int d = 0; d < 3; ++d) {
    if (nelem) nelem[d] = h->g.E[d];
    if (ndof) ndof[d] = h->g.N[d];
    if (nq) nq[d] = h->g.q[d];
  }
  return ADS_OK;
}

int ads_qp_points(const ads_handle* h, int axis, double* X) {
  if (!h || !X || axis < 0 || axis > 2) return ADS_ERR_ARG;
  std::memcpy(X, h->ax[axis].X.data(), sizeof(double) * h->ax[axis].X.size());
  return ADS_OK;
}

int ads_axis_tables(const ads_handle* h, int axis, double* U, int* O, double* J, double* W, double* NN) {
  if (!h || axis < 0 || axis > 2) return ADS_ERR_ARG;
  const AxisHost& a = h->ax[axis];
  if (U) std::memcpy(U, a.U.data(), sizeof(double) * a.U.size());
  if (O) std::memcpy(O, a.O.data(), sizeof(int) * a.O.size());
  if (J) std::memcpy(J, a.J.data(), sizeof(double) * a.J.size());
  if (W) std::memcpy(W, a.W.data(), sizeof(double) * a.W.size());
  if (NN) std::memcpy(NN, a.NN.data(), sizeof(double) * a.NN.size());
  return ADS_OK;
}

int ads_set_form(ads_handle* h, int form, const double* f_qp, const double* kappa_qp, double kappa, double dt) {
  if (!h) return ADS_ERR_ARG;
  if (form != ADS_FORM_PROJECT && form != ADS_FORM_HEAT && form != ADS_FORM_OIL) return fail(h, ADS_ERR_ARG, "unknown form");
  if (form == ADS_FORM_OIL && (!f_qp || !kappa_qp))
    return fail(h, ADS_ERR_ARG, "the oil form needs pumping (f_qp) and Kq (kappa_qp) at the points");
  if (!std::isfinite(kappa) || !std::isfinite(dt)) return fail(h, ADS_ERR_NONFINITE, "non-finite kappa or dt");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const size_t bytes = sizeof(double) * (size_t)h->nqp;
  double* stage = nullptr;
  auto load = [&](const double* src, double** dst) -> int {
    if (!*dst) ADS_CUDA(h, cudaMalloc((void**)dst, bytes));
    if (!stage) ADS_CUDA(h, cudaMalloc((void**)&stage, bytes));
    ADS_CUDA(h, cudaMemcpyAsync(stage, src, bytes, cudaMemcpyHostToDevice, h->stream));
    RUN(h, "qp_to_grid", 1, launch_qp_to_grid(stage, *dst, h->g, h->stream));
    return ADS_OK;
  };
  int st = ADS_OK;
  if (f_qp) st = load(f_qp, &h->d_fqp);
  if (!st && kappa_qp) st = load(kappa_qp, &h->d_kqp);
  if (!st) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) st = cuda_fail(h, e, "ads_set_form");
  }
  if (stage) cudaFree(stage);
  if (st) return st;
  h->form = form;
  h->has_f = f_qp != nullptr;
  h->has_k = (form == ADS_FORM_HEAT || form == ADS_FORM_OIL) && kappa_qp != nullptr;
  h->kappa = kappa;
  h->dt = dt;
  h->has_form = true;
  invalidate_graph(h);
  return ADS_OK;
}

int ads_set_oil(ads_handle* h, const double* drain_qp, double mu) {
  if (!h || !drain_qp) return ADS_ERR_ARG;
  if (!std::isfinite(mu)) return fail(h, ADS_ERR_NONFINITE, "non-finite mu");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const size_t bytes = sizeof(double) * (size_t)h->nqp;
  if (!h->d_dqp) ADS_CUDA(h, cudaMalloc((void**)&h->d_dqp, bytes));
  double* stage = nullptr;
  ADS_CUDA(h, cudaMalloc((void**)&stage, bytes));
  int st = ADS_OK;
  cudaError_t e = cudaMemcpyAsync(stage, drain_qp, bytes, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_qp_to_grid(stage, h->d_dqp, h->g, h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->d_scal + SC_DRAINED_TOTAL, 0, sizeof(double), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) st = cuda_fail(h, e, "ads_set_oil");
  cudaFree(stage);
  if (st) return st;
  h->mu = mu;
  h->has_oil = true;
  invalidate_graph(h);
  return ADS_OK;
}

// One value as Fortran's F30.10 edit descriptor writes it, after adjustl and
// trim (src/vtk.F90:57-58): fixed notation with 10 decimals, asterisks when it
// does not fit in 30 characters, Infinity / NaN spelled out.
static std::string f30_10(double v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.10f", v);
  if (std::strlen(buf) > 30) return std::string(30, '*');
  return buf;
}

int ads_write_vti(const char* name, const int res[3], const double* vals) {
  if (!name || !res || !vals) return ADS_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (res[d] < 1 || res[d] > 99999) return ADS_ERR_ARG;
  const std::string path = std::string(name) + ".vti";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return ADS_ERR_ARG;
  char extent[64];
  std::snprintf(extent, sizeof extent, "0 %5d 0 %5d 0 %5d", res[0] - 1, res[1] - 1, res[2] - 1);
  std::fprintf(f, "<?xml version=\"1.0\"?>\n");
  std::fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\">\n");
  std::fprintf(f, "  <ImageData WholeExtent=\"%s\" origin=\"0 0 0\" spacing=\"1 1 1\">\n", extent);
  std::fprintf(f, "    <Piece Extent=\"%s\">\n", extent);
  std::fprintf(f, "      <PointData Scalars=\"Result\">\n");
  std::fprintf(f, "        <DataArray Name=\"Result\" type=\"Float32\">\n");
  const size_t n = (size_t)res[0] * res[1] * res[2];
  for (size_t i = 0; i < n; ++i) std::fprintf(f, "          %s\n", f30_10(vals[i]).c_str());
  std::fprintf(f, "        </DataArray>\n");
  std::fprintf(f, "      </PointData>\n");
  std::fprintf(f, "    </Piece>\n");
  std::fprintf(f, "  </ImageData>\n");
  std::fprintf(f, "</VTKFile>\n");
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? ADS_OK : ADS_ERR_ARG;
}

int ads_save_spline_plot(ads_handle* h, const char* name, const double range[6], const int res[3], double* vals) {
  if (!h || !range || !res) return ADS_ERR_ARG;
  for (int d = 0; d < 3; ++d)
    if (res[d] < 2 || res[d] > 4096) return fail(h, ADS_ERR_ARG, "plot resolution must be 2..4096 per axis");
  for (int i = 0; i < 6; ++i)
    if (!std::isfinite(range[i])) return fail(h, ADS_ERR_NONFINITE, "non-finite plot range");
  const long long n = (long long)res[0] * res[1] * res[2];
  if (n > (1ll << 28)) return fail(h, ADS_ERR_ARG, "plot grid too large (more than 2^28 samples)");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  std::vector<double> tab;
  std::vector<int> first;
  for (int d = 0; d < 3; ++d) {
    std::vector<double> B;
    std::vector<int> F;
    sample_basis(h->ax[d], range[2 * d], range[2 * d + 1], res[d], B, F);
    tab.insert(tab.end(), B.begin(), B.end());
    first.insert(first.end(), F.begin(), F.end());
  }
  std::vector<double> host;
  double* out = vals;
  if (!out) {
    host.resize((size_t)n);
    out = host.data();
  }
  double *d_tab = nullptr, *d_vals = nullptr;
  int* d_first = nullptr;
  int st = ADS_OK;
  cudaError_t e = cudaMalloc((void**)&d_tab, sizeof(double) * tab.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_first, sizeof(int) * first.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_vals, sizeof(double) * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    st = run_kernel(h, "eval_grid", 1, [&]() -> cudaError_t {
      return launch_eval_grid(h->d_u, h->g, d_tab, d_first, res[0], res[1], res[2], d_vals, h->stream);
    });
  }
  if (e == cudaSuccess && !st) e = cudaMemcpyAsync(out, d_vals, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && !st) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess && !st) st = cuda_fail(h, e, "ads_save_spline_plot");
  cudaFree(d_tab);
  cudaFree(d_first);
  cudaFree(d_vals);
  if (st) return st;
  if (name && ads_write_vti(name, res, out) != ADS_OK)
    return fail(h, ADS_ERR_ARG, std::string("cannot write ") + name + ".vti");
  return ADS_OK;
}

// the pivoted LU of mix along axis d, cached per mix
static int multistep_factors(ads_handle* h, int d, const double mix[4]) {
  if (h->mab_valid[d] && std::memcmp(h->mab_mix[d], mix, sizeof(double) * 4) == 0) return ADS_OK;
  const AxisHost& a = h->ax[d];
  std::vector<double> AB;
  mix_band(a, mix, AB);
  std::vector<int> ipiv(a.N);
  if (band_lu(a.N, a.p, a.p, AB.data(), 3 * a.p + 1, ipiv.data()))
    return fail(h, ADS_ERR_ZERO_PIVOT, "zero pivot in the 1-D matrix of the MultiStep mix");
  if (!h->d_mab[d]) ADS_CUDA(h, cudaMalloc((void**)&h->d_mab[d], sizeof(double) * AB.size()));
  if (!h->d_mpiv[d]) ADS_CUDA(h, cudaMalloc((void**)&h->d_mpiv[d], sizeof(int) * ipiv.size()));
  // in stream order: the previous substep's solves on this stream may still
  // read the old factors (a pageable source is staged before the call returns)
  ADS_CUDA(h, cudaMemcpyAsync(h->d_mab[d], AB.data(), sizeof(double) * AB.size(), cudaMemcpyHostToDevice, h->stream));
  ADS_CUDA(h, cudaMemcpyAsync(h->d_mpiv[d], ipiv.data(), sizeof(int) * ipiv.size(), cudaMemcpyHostToDevice, h->stream));
  std::memcpy(h->mab_mix[d], mix, sizeof(double) * 4);
  h->mab_valid[d] = true;
  return ADS_OK;
}

int ads_multistep(ads_handle* h, const double mix[12], double* l2norm) {
  if (!h || !mix) return ADS_ERR_ARG;
  if (!h->has_form) return fail(h, ADS_ERR_STATE, "ads_set_form must be called before stepping");
  if (h->form == ADS_FORM_OIL)
    return fail(h, ADS_ERR_UNSUPPORTED, "MultiStep supports the projection and heat forms (the oil integrand "
                                        "would need its value and gradient from different coefficient sets)");
  for (int i = 0; i < 12; ++i)
    if (!std::isfinite(mix[i])) return fail(h, ADS_ERR_NONFINITE, "non-finite MultiStep mix");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const Geometry& g = h->g;
  const long long Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
  const size_t bytes = sizeof(double) * h->n0;
  for (double** p : {&h->d_un, &h->d_ms}) {
    if (!*p) {
      ADS_CUDA(h, cudaMalloc((void**)p, bytes));
      ADS_CUDA(h, cudaMemset(*p, 0, bytes));
    }
  }
  int st;
  ADS_CUDA(h, cudaMemcpyAsync(h->d_un, h->d_u, bytes, cudaMemcpyDeviceToDevice, h->stream));
  double l2 = 0.0;
  for (int sub = 0; sub < 3; ++sub) {
    const double* mx = mix + 4 * sub;
    for (int d = 0; d < 3; ++d)
      if ((st = multistep_factors(h, d, mx))) return st;
    // FormUn(sub) + Form3DRHS: the integrand sees u from the start of the
    // step (Un) and grad u of the current coefficients (dUn); the heat form
    // is linear in both, so F = F(current) + M (u^n - current)
    if ((st = enqueue_assemble(h, h->d_u, h->d_F, false, false, true))) return st;
    if (sub == 0) {
      // the l2norm integrates Un, the same in every substep
      ADS_CUDA(h, cudaMemcpyAsync(&l2, h->d_scal + SC_L2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else if (h->form == ADS_FORM_HEAT) {
      ADS_CUDA(h, cudaMemcpyAsync(h->d_ms, h->d_un, bytes, cudaMemcpyDeviceToDevice, h->stream));
      RUN(h, "axpby", 1, launch_axpby(h->d_ms, h->d_u, -1.0, 1.0, (long long)h->n0, h->stream));
      if ((st = enqueue_mass(h, h->d_ms, nullptr, h->d_r, "mass_apply"))) return st;  // d_r = M (u^n - current)
      RUN(h, "add", 1, launch_add(h->d_F, h->d_r, (long long)h->n0, h->stream));
    }
    // Sub_Step's three solves with the mix, in place on F (L0)
    Phase phx(h, "Solve 1");
    RUN(h, "band_solve_x", 1, launch_band_solve(h->d_F, Ny, Nz, g.PX, g.PX * Ny, 1, (int)Nx, h->p[0], h->p[0],
                                                h->d_mab[0], h->d_mpiv[0], h->stream));
    Phase phy(h, "Solve 2");
    RUN(h, "band_solve_y", 1, launch_band_solve(h->d_F, Nx, Nz, 1, g.PX * Ny, g.PX, (int)Ny, h->p[1], h->p[1],
                                                h->d_mab[1], h->d_mpiv[1], h->stream));
    Phase phz(h, "Solve 3");
    RUN(h, "band_solve_z", 1, launch_band_solve(h->d_F, Nx, Ny, 1, g.PX, g.PX * Ny, (int)Nz, h->p[2], h->p[2],
                                                h->d_mab[2], h->d_mpiv[2], h->stream));
    ADS_CUDA(h, cudaMemcpyAsync(h->d_u, h->d_F, bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  ADS_CUDA(h, cudaStreamSynchronize(h->stream));
  if ((st = check_flags(h))) return st;
  if (!std::isfinite(l2)) return fail(h, ADS_ERR_NONFINITE, "non-finite l2norm");
  h->last.l2norm = l2;
  h->last.rel_residual = 0.0;
  h->last.refinements = 0;
  h->last.converged = 1;
  h->last.fp64_residuals = 0;
  h->last.host_path = 0;
  if (l2norm) *l2norm = l2;
  return ADS_OK;
}

int ads_get_drained(const ads_handle* h, double* drained) {
  if (!h || !drained) return ADS_ERR_ARG;
  ads_handle* hm = const_cast<ads_handle*>(h);
  ADS_CUDA(hm, cudaSetDevice(h->dev));
  ADS_CUDA(hm, cudaMemcpyAsync(drained, h->d_scal + SC_DRAINED_TOTAL, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  ADS_CUDA(hm, cudaStreamSynchronize(h->stream));
  return ADS_OK;
}

int ads_set_coeffs(ads_handle* h, const double* u) {
  if (!h || !u) return ADS_ERR_ARG;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = copy_l0_in(h, h->d_u, u, cudaMemcpyHostToDevice);
  if (st) return st;
  ADS_CUDA(h, cudaStreamSynchronize(h->stream));
  return ADS_OK;
}

int ads_get_coeffs(ads_handle* h, double* u) {
  if (!h || !u) return ADS_ERR_ARG;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = copy_l0_out(h, u, h->d_u, cudaMemcpyDeviceToHost);
  if (st) return st;
  ADS_CUDA(h, cudaStreamSynchronize(h->stream));
  return ADS_OK;
}

int ads_set_coeffs_device(ads_handle* h, const double* d_u) {
  if (!h || !d_u) return ADS_ERR_ARG;
  return copy_l0_in(h, h->d_u, d_u, cudaMemcpyDeviceToDevice);
}

int ads_get_coeffs_device(ads_handle* h, double* d_u) {
  if (!h || !d_u) return ADS_ERR_ARG;
  return copy_l0_out(h, d_u, h->d_u, cudaMemcpyDeviceToDevice);
}

int ads_steps(ads_handle* h, int k, double* l2norms) {
  if (!h || k < 0) return ADS_ERR_ARG;
  if (!h->has_form) return fail(h, ADS_ERR_STATE, "ads_set_form must be called before stepping");
  if (h->form == ADS_FORM_OIL && !h->has_oil) return fail(h, ADS_ERR_STATE, "ads_set_oil must be called before stepping the oil form");
  if (k == 0) return ADS_OK;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = ensure_hist(h, std::max(k, 64));
  if (st) return st;
  ADS_CUDA(h, cudaMemsetAsync(h->d_flags + FL_HIST, 0, sizeof(int), h->stream));
  if (h->timing) {
    for (int i = 0; i < k; ++i)
      if ((st = enqueue_step(h))) return st;
  } else {
    if (!h->graph_valid && (st = build_graph(h))) return st;
    for (int i = 0; i < k; ++i) {
      ADS_CUDA(h, cudaGraphLaunch(h->gexec, h->stream));
      h->launches += h->graph_launches;
    }
  }
  return finish_stats(h, k, l2norms);
}

int ads_step(ads_handle* h, double* l2norm) {
  double l2 = 0.0;
  int st = ads_steps(h, 1, &l2);
  if (l2norm) *l2norm = l2;
  return st;
}

int ads_step_host(ads_handle* h, const double* u_in, double* u_out, double* l2norm) {
  if (!h || !u_in || !u_out) return ADS_ERR_ARG;
  if (!h->has_form) return fail(h, ADS_ERR_STATE, "ads_set_form must be called before stepping");
  if (h->form == ADS_FORM_OIL && !h->has_oil) return fail(h, ADS_ERR_STATE, "ads_set_oil must be called before stepping the oil form");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  auto staged = [&](int path) -> int {
    int s = ads_set_coeffs(h, u_in);
    if (!s) s = ads_step(h, l2norm);
    if (!s) s = ads_get_coeffs(h, u_out);
    h->last.host_path = path;
    return s;
  };
  const double* din = nullptr;
  double* dout = nullptr;
  if (df_increment(h) && !h->general) {
    din = device_view(h, u_in);
    dout = const_cast<double*>(device_view(h, u_out));
  }
  if (!din || !dout) return staged(0);
  int st = ensure_hist(h, 64);
  if (st) return st;
  ADS_CUDA(h, cudaMemsetAsync(h->d_flags + FL_HIST, 0, sizeof(int), h->stream));
  if ((st = enqueue_step_host(h, din, dout))) return st;
  int fl[FL_COUNT];
  ADS_CUDA(h, cudaMemcpyAsync(fl, h->d_flags, sizeof(fl), cudaMemcpyDeviceToHost, h->stream));
  ADS_CUDA(h, cudaStreamSynchronize(h->stream));
  if (fl[FL_UMISS]) {
    // u_out was not written (d_u holds u_in); errors of the discarded attempt are dropped
    ADS_CUDA(h, cudaMemsetAsync(h->d_flags + FL_ERR, 0, sizeof(int), h->stream));
    return staged(2);
  }
  double l2 = 0.0;
  if ((st = finish_stats(h, 1, &l2))) return st;
  if (l2norm) *l2norm = l2;
  h->last.host_path = 1;
  return ADS_OK;
}

int ads_get_stats(const ads_handle* h, ads_stats* s) {
  if (!h || !s) return ADS_ERR_ARG;
  *s = h->last;
  return ADS_OK;
}

int ads_assemble(ads_handle* h, double* F_out, double* l2norm) {
  if (!h || !F_out) return ADS_ERR_ARG;
  if (!h->has_form) return fail(h, ADS_ERR_STATE, "ads_set_form must be called before assembling");
  if (h->form == ADS_FORM_OIL && !h->has_oil) return fail(h, ADS_ERR_STATE, "ads_set_oil must be called before assembling the oil form");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = enqueue_assemble(h, h->d_u, h->d_F, is_mixed(h), false, true);
  if (st) return st;
  if ((st = copy_l0_out(h, F_out, h->d_F, cudaMemcpyDeviceToHost))) return st;
  double l2 = 0.0;
  ADS_CUDA(h, cudaMemcpyAsync(&l2, h->d_scal + SC_L2, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((st = check_flags(h))) return st;
  if (l2norm) *l2norm = l2;
  return ADS_OK;
}

int ads_solve(ads_handle* h, const double* F, double* u_out) {
  if (!h || !F) return ADS_ERR_ARG;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = copy_l0_in(h, h->d_F, F, cudaMemcpyHostToDevice);
  if (st) return st;
  RUN(h, "step_reset", 1, launch_step_reset(h->d_scal, h->d_flags, h->stream));
  if ((st = enqueue_solve(h))) return st;
  if (u_out && (st = copy_l0_out(h, u_out, h->d_u, cudaMemcpyDeviceToHost))) return st;
  if ((st = check_flags(h))) return st;
  double sc[SC_COUNT];
  int fl[FL_COUNT];
  ADS_CUDA(h, cudaMemcpy(sc, h->d_scal, sizeof(sc), cudaMemcpyDeviceToHost));
  ADS_CUDA(h, cudaMemcpy(fl, h->d_flags, sizeof(fl), cudaMemcpyDeviceToHost));
  const bool mixed = is_mixed(h);
  h->last.rel_residual = mixed ? sc[SC_RELRES] : 0.0;
  h->last.refinements = mixed ? fl[FL_ITERS] : 0;
  h->last.converged = mixed ? fl[FL_CONV] : 1;
  h->last.fp64_residuals = mixed ? fl[FL_RESID] : 0;
  if (mixed && !fl[FL_CONV]) return fail(h, ADS_ERR_NOCONV, "iterative refinement did not reach refine_tol");
  return ADS_OK;
}

int ads_apply_mass(ads_handle* h, const double* u, double* out) {
  if (!h || !u || !out) return ADS_ERR_ARG;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  int st = copy_l0_in(h, h->d_F, u, cudaMemcpyHostToDevice);
  if (st) return st;
  if ((st = enqueue_mass(h, h->d_F, nullptr, h->d_r, "residual_f64"))) return st;
  if ((st = copy_l0_out(h, out, h->d_r, cudaMemcpyDeviceToHost))) return st;
  return check_flags(h);
}

int ads_reorder(ads_handle* h, int kind, const double* in, double* out) {
  if (!h || !in || !out) return ADS_ERR_ARG;
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const Geometry& g = h->g;
  const int Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
  if (kind != ADS_REORDER_FOR_Y && kind != ADS_REORDER_FOR_Z && kind != ADS_REORDER_FOR_X)
    return fail(h, ADS_ERR_ARG, "unknown reorder kind");
  if (h->banded) {
    // no transposing sweeps here: a plain permutation of dense arrays (the
    // packed stage buffer in, d_r as a dense out)
    int st = ensure_stage(h);
    if (st) return st;
    const size_t bytes = sizeof(double) * (size_t)Nx * Ny * Nz;
    ADS_CUDA(h, cudaMemcpyAsync(h->d_stage, in, bytes, cudaMemcpyHostToDevice, h->stream));
    RUN(h, "permute", 1, launch_permute(h->d_stage, h->d_r, g, kind, h->stream));
    ADS_CUDA(h, cudaMemcpyAsync(out, h->d_r, bytes, cudaMemcpyDeviceToHost, h->stream));
    return check_flags(h);
  }
  const CUtensorMap* tout;
  const double* src;
  double* dst;
  int axis;
  if (kind == ADS_REORDER_FOR_Y) {  // L0 -> L1
    ADS_CUDA(h, cudaMemcpy2DAsync(h->d_F, g.PX * 8, in, (size_t)Nx * 8, (size_t)Nx * 8, (size_t)Ny * Nz,
                                  cudaMemcpyHostToDevice, h->stream));
    src = h->d_F; tout = &h->tm_wA_out64; dst = h->d_wA; axis = 0;
  } else if (kind == ADS_REORDER_FOR_Z) {  // L1 -> L2
    ADS_CUDA(h, cudaMemcpy2DAsync(h->d_wA, g.PY * 8, in, (size_t)Ny * 8, (size_t)Ny * 8, (size_t)Nx * Nz,
                                  cudaMemcpyHostToDevice, h->stream));
    src = h->d_wA; tout = &h->tm_wB_out64; dst = h->d_wB; axis = 1;
  } else if (kind == ADS_REORDER_FOR_X) {  // L2 -> L0
    ADS_CUDA(h, cudaMemcpy2DAsync(h->d_wB, g.PZ * 8, in, (size_t)Nz * 8, (size_t)Nz * 8, (size_t)Nx * Ny,
                                  cudaMemcpyHostToDevice, h->stream));
    src = h->d_wB; tout = &h->tm_r_out64; dst = h->d_r; axis = 2;
  } else {
    return fail(h, ADS_ERR_ARG, "unknown reorder kind");
  }
  SweepArgs a = sweep_args(h, axis, h->d_fac64[axis], src);
  RUN(h, "transpose_f64", 1, launch_sweep(h->P, 0, 0, 3, false, tout, a, sweep_grid(h, axis), h->stream));
  if (kind == ADS_REORDER_FOR_Y) {
    ADS_CUDA(h, cudaMemcpy2DAsync(out, (size_t)Ny * 8, dst, g.PY * 8, (size_t)Ny * 8, (size_t)Nx * Nz,
                                  cudaMemcpyDeviceToHost, h->stream));
  } else if (kind == ADS_REORDER_FOR_Z) {
    ADS_CUDA(h, cudaMemcpy2DAsync(out, (size_t)Nz * 8, dst, g.PZ * 8, (size_t)Nz * 8, (size_t)Nx * Ny,
                                  cudaMemcpyDeviceToHost, h->stream));
  } else {
    ADS_CUDA(h, cudaMemcpy2DAsync(out, (size_t)Nx * 8, dst, g.PX * 8, (size_t)Nx * 8, (size_t)Ny * Nz,
                                  cudaMemcpyDeviceToHost, h->stream));
  }
  return check_flags(h);
}

int ads_heat_adjoint(ads_handle* h, int K, int ck, const double* u0, const double* ut, double* loss,
                     double* grad_u0, double* grad_kappa_qp) {
  if (!h || !u0 || !ut || K < 1 || ck < 1) return ADS_ERR_ARG;
  if (!h->has_form || h->form != ADS_FORM_HEAT) return fail(h, ADS_ERR_STATE, "the adjoint needs the HEAT form");
  if (grad_kappa_qp && !h->has_k) return fail(h, ADS_ERR_STATE, "dL/dkappa needs a per-point kappa");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const size_t n0 = h->n0;
  const int ncp = (K + ck - 1) / ck;
  std::vector<double*> bufs;
  auto alloc = [&](size_t n) -> double* {
    double* p = nullptr;
    if (cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(double) * std::max<size_t>(n, 1));
    bufs.push_back(p);
    return p;
  };
  auto cleanup = [&]() { for (double* p : bufs) cudaFree(p); };
  double* cps = alloc(n0 * ncp);
  double* seg = alloc(n0 * ck);
  double* lam = alloc(n0);
  double* mu = alloc(n0);
  double* e = alloc(n0);
  double* d_ut = alloc(n0);
  double* gk = grad_kappa_qp ? alloc((size_t)h->nqp) : nullptr;
  double* dpart = alloc(1024);
  if (!cps || !seg || !lam || !mu || !e || !d_ut || !dpart || (grad_kappa_qp && !gk)) {
    cleanup();
    return fail(h, ADS_ERR_ALLOC, "adjoint buffers");
  }
  CUtensorMap tm_mu_out;
  if (!make_l0_out(h, &tm_mu_out, mu, false)) {
    cleanup();
    return fail(h, ADS_ERR_CUDA, "adjoint tensor maps");
  }
  int st = ADS_OK;
  auto body = [&]() -> int {
    int s;
    if ((s = copy_l0_in(h, h->d_u, u0, cudaMemcpyHostToDevice))) return s;
    if ((s = copy_l0_in(h, d_ut, ut, cudaMemcpyHostToDevice))) return s;
    if ((s = ensure_hist(h, std::max(64, K + 1)))) return s;
    ADS_CUDA(h, cudaMemsetAsync(h->d_flags + FL_HIST, 0, sizeof(int), h->stream));
    // forward with checkpoints
    for (int n = 0; n < K; ++n) {
      if (n % ck == 0)
        ADS_CUDA(h, cudaMemcpyAsync(cps + (size_t)(n / ck) * n0, h->d_u, sizeof(double) * n0,
                                    cudaMemcpyDeviceToDevice, h->stream));
      if ((s = enqueue_step(h))) return s;
    }
    // loss = 1/2 e^T M e, e = u^K - ut; lambda^K = M e
    ADS_CUDA(h, cudaMemcpyAsync(e, h->d_u, sizeof(double) * n0, cudaMemcpyDeviceToDevice, h->stream));
    RUN(h, "axpby", 1, launch_axpby(e, d_ut, -1.0, 1.0, (long long)n0, h->stream));
    if ((s = enqueue_mass(h, e, nullptr, lam, "residual_f64"))) return s;
    RUN(h, "dot", 2, launch_dot(e, lam, (long long)n0, dpart, 512, h->d_scal + SC_DOT, h->stream));
    double Lval = 0.0;
    ADS_CUDA(h, cudaMemcpyAsync(&Lval, h->d_scal + SC_DOT, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ADS_CUDA(h, cudaStreamSynchronize(h->stream));
    if (loss) *loss = 0.5 * Lval;
    if (!grad_u0 && !grad_kappa_qp) return ADS_OK;
    AxisTab<double> t64[3];
    for (int d = 0; d < 3; ++d) { t64[d].nn = h->d_nn64[d]; t64[d].jw = h->d_jw64[d]; t64[d].dd = h->d_dd64[d]; }
    for (int c = ncp - 1; c >= 0; --c) {
      const int s0 = c * ck, s1 = std::min(s0 + ck, K);
      // recompute the segment's states u^{s0} .. u^{s1-1}
      ADS_CUDA(h, cudaMemcpyAsync(h->d_u, cps + (size_t)c * n0, sizeof(double) * n0, cudaMemcpyDeviceToDevice, h->stream));
      for (int n = s0; n < s1; ++n) {
        ADS_CUDA(h, cudaMemcpyAsync(seg + (size_t)(n - s0) * n0, h->d_u, sizeof(double) * n0,
                                    cudaMemcpyDeviceToDevice, h->stream));
        if (n + 1 < s1 && (s = enqueue_step(h))) return s;
      }
      for (int n = s1 - 1; n >= s0; --n) {
        // mu = M^{-T} lambda (transposed sweeps, FP64)
        if ((s = enqueue_solve64(h, lam, &tm_mu_out, true, mu))) return s;
        if (gk) {
          const double* un = seg + (size_t)(n - s0) * n0;
          if (h->general)
            RUN(h, "kappa_grad", 1, launch_kappa_grad_gen(h->g, un, mu, h->dt, gk, t64[0], t64[1], t64[2], h->stream));
          else
            RUN(h, "kappa_grad", 1, launch_kappa_grad(h->g, un, mu, h->dt, gk, t64[0], t64[1], t64[2], h->stream));
        }
        // lambda = A^T mu: the heat operator is symmetric, so the same assembly
        // kernels apply it (the source term does not depend on u and is left out)
        if ((s = enqueue_assemble(h, mu, lam, false, false, false))) return s;
      }
    }
    if (grad_u0 && (s = copy_l0_out(h, grad_u0, lam, cudaMemcpyDeviceToHost))) return s;
    if (gk) {
      double* qp = alloc((size_t)h->nqp);
      if (!qp) return fail(h, ADS_ERR_ALLOC, "adjoint buffers");
      RUN(h, "grid_to_qp", 1, launch_grid_to_qp(gk, qp, h->g, h->stream));
      ADS_CUDA(h, cudaMemcpyAsync(grad_kappa_qp, qp, sizeof(double) * (size_t)h->nqp, cudaMemcpyDeviceToHost, h->stream));
    }
    return check_flags(h);
  };
  st = body();
  cudaStreamSynchronize(h->stream);
  cleanup();
  return st;
}

// Tangent-linear model of K explicit heat steps, run beside the forward:
//   u^{n+1} = M^{-1} (A(kappa) u^n + dt F_f),   A(kappa) = M - dt K(kappa)
//   w^{n+1} = M^{-1} (A(kappa) w^n - dt K(dkappa) u^n),   w^0 = du0
// so w^K = du^K/d(u0, kappa) . (du0, dkappa).  The FP64 assembly applies
// A(kappa) to w (source left out); -dt K(dkappa) u^n is the FP64 assembly in
// increment form with the per-point conductivity dkappa, and the sum is
// solved with the FP64 sweeps.  The forward uses the handle's precision.
int ads_heat_jvp(ads_handle* h, int K, const double* u0, const double* du0, const double* dkappa_qp,
                 double* uK, double* duK) {
  if (!h || !u0 || K < 0) return ADS_ERR_ARG;
  if (!h->has_form || h->form != ADS_FORM_HEAT) return fail(h, ADS_ERR_STATE, "the tangent model needs the HEAT form");
  ADS_CUDA(h, cudaSetDevice(h->dev));
  const size_t n0 = h->n0;
  std::vector<double*> bufs;
  auto alloc = [&](size_t n) -> double* {
    double* p = nullptr;
    if (cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, sizeof(double) * std::max<size_t>(n, 1));
    bufs.push_back(p);
    return p;
  };
  auto cleanup = [&]() { for (double* p : bufs) cudaFree(p); };
  double* w = alloc(n0);
  double* t = dkappa_qp ? alloc(n0) : nullptr;
  double* dk = dkappa_qp ? alloc((size_t)h->nqp) : nullptr;
  if (!w || (dkappa_qp && (!t || !dk))) {
    cleanup();
    return fail(h, ADS_ERR_ALLOC, "tangent buffers");
  }
  CUtensorMap tm_w_out;
  if (!make_l0_out(h, &tm_w_out, w, false)) {
    cleanup();
    return fail(h, ADS_ERR_CUDA, "tangent tensor maps");
  }
  auto body = [&]() -> int {
    int s;
    if ((s = copy_l0_in(h, h->d_u, u0, cudaMemcpyHostToDevice))) return s;
    if (du0 && (s = copy_l0_in(h, w, du0, cudaMemcpyHostToDevice))) return s;
    if (dkappa_qp) {
      double* stage = alloc((size_t)h->nqp);
      if (!stage) return fail(h, ADS_ERR_ALLOC, "tangent buffers");
      ADS_CUDA(h, cudaMemcpyAsync(stage, dkappa_qp, sizeof(double) * (size_t)h->nqp, cudaMemcpyHostToDevice, h->stream));
      RUN(h, "qp_to_grid", 1, launch_qp_to_grid(stage, dk, h->g, h->stream));
    }
    if ((s = ensure_hist(h, std::max(64, K + 1)))) return s;
    ADS_CUDA(h, cudaMemsetAsync(h->d_flags + FL_HIST, 0, sizeof(int), h->stream));
    for (int n = 0; n < K; ++n) {
      // t = -dt K(dkappa) u^n: the FP64 assembly in increment form (no mass
      // term to cancel) with the per-point conductivity dkappa and no source
      if (dkappa_qp && (s = enqueue_assemble(h, h->d_u, t, false, true, false, dk))) return s;
      // A w^n (+ t), solved into w^{n+1}
      if ((s = enqueue_assemble(h, w, h->d_F, false, false, false))) return s;
      if (dkappa_qp) RUN(h, "add", 1, launch_add(h->d_F, t, (long long)n0, h->stream));
      if ((s = enqueue_solve64(h, h->d_F, &tm_w_out, false, w))) return s;
      // the forward step u^n -> u^{n+1}
      if ((s = enqueue_step(h))) return s;
    }
    if (uK && (s = copy_l0_out(h, uK, h->d_u, cudaMemcpyDeviceToHost))) return s;
    if (duK && (s = copy_l0_out(h, duK, w, cudaMemcpyDeviceToHost))) return s;
    return check_flags(h);
  };
  int st = body();
  cudaStreamSynchronize(h->stream);
  cleanup();
  return st;
}

int ads_axis_setup(int n, int p, double* U, int* O, double* J, double* W, double* X, double* NN,
                   double* band, double* fac, double* tfac) {
  if (p < 1 || p > 4) return ADS_ERR_UNSUPPORTED;
  if (n < p) return ADS_ERR_ARG;
  AxisHost a;
  if (axis_setup(n, p, a)) return ADS_ERR_UNSUPPORTED;
  if (U) std::memcpy(U, a.U.data(), sizeof(double) * a.U.size());
  if (O) std::memcpy(O, a.O.data(), sizeof(int) * a.O.size());
  if (J) std::memcpy(J, a.J.data(), sizeof(double) * a.J.size());
  if (W) std::memcpy(W, a.W.data(), sizeof(double) * a.W.size());
  if (X) std::memcpy(X, a.X.data(), sizeof(double) * a.X.size());
  if (NN) std::memcpy(NN, a.NN.data(), sizeof(double) * a.NN.size());
  if (band) std::memcpy(band, a.band.data(), sizeof(double) * a.band.size());
  if (fac || tfac) {
    std::vector<double> f, t;
    if (band_factor(a, f, t)) return ADS_ERR_ZERO_PIVOT;
    if (fac) std::memcpy(fac, f.data(), sizeof(double) * f.size());
    if (tfac) std::memcpy(tfac, t.data(), sizeof(double) * t.size());
  }
  return ADS_OK;
}

int ads_fma_peak(int device, int fp64, double* tflops) {
  if (!tflops) return ADS_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return ADS_ERR_CUDA;
  double t = 0.0;
  cudaError_t e = measure_fma_peak(fp64 != 0, &t);
  if (e != cudaSuccess) return ADS_ERR_CUDA;
  *tflops = t;
  return ADS_OK;
}

void* ads_get_stream(const ads_handle* h) { return h ? (void*)h->stream : nullptr; }

int ads_set_stream(ads_handle* h, void* stream) {
  if (!h) return ADS_ERR_ARG;
  cudaSetDevice(h->dev);
  cudaStreamSynchronize(h->stream);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->own_stream = false;
  h->stream = (cudaStream_t)stream;
  invalidate_graph(h);
  return ADS_OK;
}

int ads_timing_enable(ads_handle* h, int on) {
  if (!h) return ADS_ERR_ARG;
  h->timing = on != 0;
  return ADS_OK;
}

int ads_timing_reset(ads_handle* h) {
  if (!h) return ADS_ERR_ARG;
  resolve_timing(h);
  h->tnames.clear(); h->tms.clear(); h->tcount.clear();
  h->pnames.clear(); h->pms.clear(); h->pcount.clear();
  return ADS_OK;
}

int ads_phase_timing_read(ads_handle* h, char* names, int names_len, double* times_ms, int* launches,
                          int max_phases, int* n_phases) {
  if (!h) return ADS_ERR_ARG;
  resolve_timing(h);
  const int n = (int)std::min<size_t>(h->pnames.size(), (size_t)std::max(max_phases, 0));
  std::string all;
  for (int i = 0; i < n; ++i) {
    if (i) all += ",";
    all += h->pnames[i];
    if (times_ms) times_ms[i] = h->pms[i];
    if (launches) launches[i] = h->pcount[i];
  }
  if (names && names_len > 0) {
    std::strncpy(names, all.c_str(), (size_t)names_len - 1);
    names[names_len - 1] = '\0';
  }
  if (n_phases) *n_phases = n;
  return ADS_OK;
}

int ads_timing_read(ads_handle* h, char* names, int names_len, double* times_ms, int* launches,
                    int max_kernels, int* n_kernels) {
  if (!h) return ADS_ERR_ARG;
  resolve_timing(h);
  const int n = (int)std::min<size_t>(h->tnames.size(), (size_t)std::max(max_kernels, 0));
  std::string all;
  for (int i = 0; i < n; ++i) {
    if (i) all += ",";
    all += h->tnames[i];
    if (times_ms) times_ms[i] = h->tms[i];
    if (launches) launches[i] = h->tcount[i];
  }
  if (names && names_len > 0) {
    std::strncpy(names, all.c_str(), (size_t)names_len - 1);
    names[names_len - 1] = '\0';
  }
  if (n_kernels) *n_kernels = n;
  return ADS_OK;
}

long long ads_launch_count(const ads_handle* h) { return h ? h->launches : -1; }

int ads_launch_count_reset(ads_handle* h) {
  if (!h) return ADS_ERR_ARG;
  h->launches = 0;
  return ADS_OK;
}

}  // extern "C"

namespace ads {

void handle_noalloc_view(ads_handle* h, NoallocView* v) {
  v->dev = h->dev;
  v->P = h->P;
  v->general = h->general;
  v->grid = h->res_grid;  // the 32-plane chunks: the scratch limit is stated in them
  v->stream = h->stream;
  v->args = residual_args(h, nullptr, nullptr, nullptr);
  v->args.zc = h->res_zc;
  v->args.niz = h->res_niz;
  v->args.g.PX = h->g.N[0];
  v->args.part = nullptr;
  v->args.err = nullptr;
  v->launches = &h->launches;
}

int handle_fail(ads_handle* h, int code, const std::string& msg) { return fail(h, code, msg); }

int handle_cuda_fail(ads_handle* h, cudaError_t e, const char* where) { return cuda_fail(h, e, where); }

}  // namespace ads
