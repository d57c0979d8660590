/*
 * ads_gpu.h — C-ABI of the GB300 implementation of the IGA-ADS explicit time
 * step (macwozni/ADS_MPI).  Plain C types only; every entry point returns an
 * int status (ADS_OK == 0) and never exits the process.
 *
 * Reference interface that each entry point replaces (paths are relative to the
 * reference project):
 *   ads_create          initialize(n, p, ads, ads_data, mierr)     src/ADS.F90:11-107
 *   ads_destroy         Cleanup(ads, ads_data, mierr)               src/ADS.F90:802-863
 *   ads_set_form        the RHS_fun procedure argument of Step      src/Interfaces.F90:52-81
 *                       (integrands problems/heat/RHS_eq.F90:69-86,
 *                        problems/L2Projection/RHS_eq.F90:66-70)
 *   ads_step            Step(iter, RHS_fun, ads, ads_data, l2norm, mierr)  src/ADS.F90:437-461
 *   ads_steps           the time loop of problems/heat/main.F90:49-60 (Step + MPI_Reduce)
 *   ads_multistep       MultiStep(iter, mix, RHS_fun, ...)          src/ADS.F90:391-429
 *   ads_get_coeffs      ads_data%F after Step / R(:,2,2,2)          src/ADS.F90:777-779
 *   ads_set_coeffs      R(:,2,2,2) before FormUn                    src/projection_engine.F90:412
 *   ads_qp_points       ads%Xx/Xy/Xz (BasisData X output)           src/basis.F90:74-112
 *   ads_axis_tables     ads%Ox,Jx,Wx,NNx (BasisData outputs)        src/basis.F90:74-112
 *   ads_assemble        FormUn + Form3DRHS                          src/projection_engine.F90:154-441
 *   ads_solve           the Kronecker solve of Sub_Step             src/ADS.F90:518-779
 *   ads_reorder         ReorderRHSForY / ForZ / ForX                src/reorderRHS.F90:7-93
 *   ads_apply_mass      (Mx (x) My (x) Mz) u with MKBBT's mass band  src/projection_engine.F90:63-132
 *   ads_set_oil         the oil problem's pointwise data and mi      problems/oil/input_data.F90:6-20,265-303
 *   ads_get_drained     the `drained` statistic (ComputeResults)     problems/oil/input_data.F90:83-99
 *   ads_save_spline_plot  SaveSplinePlot + VtkOutput of PrintSolution  src/ADS.F90:955-989
 *   ads_write_vti       VtkOutput                                    src/vtk.F90:15-77
 *   ads_heat_adjoint    new: hand-written adjoint of the explicit heat step
 *   ads_heat_jvp        new: tangent-linear model of the explicit heat step
 *
 * Layouts.  Coefficient vectors are x-fastest, u[x + Nx*(y + Ny*z)], which is
 * the Fortran F(x, y+z*Ny) and R(:,2,2,2) of the reference.  Quadrature-point
 * arrays use the (kx,ky,kz,ex,ey,ez) column-major layout of the reference's
 * per-point caches (problems/oil/RHS_eq.F90:78): index
 * kx + q*(ky + q*(kz + q*(ex + Ex*(ey + Ey*ez)))).
 *
 * Index convention (src/knot_vector.F90): n is the number of basis functions
 * minus one per axis; an axis has n-p+1 elements and n+1 DOFs.
 *
 * Threading: a handle is used by one host thread at a time.  All device work
 * of a handle runs on one CUDA stream (ads_get_stream / ads_set_stream); calls
 * that return host data synchronise that stream.
 */
#ifndef ADS_GPU_H
#define ADS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* status codes */
#define ADS_OK 0
#define ADS_ERR_ARG 1          /* invalid argument (sizes, degree, null pointer) */
#define ADS_ERR_CUDA 2         /* a CUDA runtime call failed */
#define ADS_ERR_ZERO_PIVOT 3   /* zero pivot in the banded LU factorisation */
#define ADS_ERR_NONFINITE 4    /* non-finite value in an input or result */
#define ADS_ERR_NOCONV 5       /* iterative refinement did not reach the tolerance */
#define ADS_ERR_TIMEOUT 6      /* reserved for a bounded device-side wait that gives up: no kernel of
                                  this library spins on a device-side condition, so no call returns it */
#define ADS_ERR_UNSUPPORTED 7  /* valid but not supported by the GPU path (e.g. p > 4) */
#define ADS_ERR_STATE 8        /* call out of order (no form set, ...) */
#define ADS_ERR_ALLOC 9        /* device or host allocation failed */
#define ADS_ERR_DEVICE 10      /* a kernel reported an error flag */

/* precision of the time step */
#define ADS_PREC_FP64 0        /* FP64 assembly and FP64 banded sweeps (the drop-in) */
#define ADS_PREC_MIXED 1       /* heat increment assembled in double-float arithmetic on the
                                  FP32 pipe (~44 bits), FP32 banded sweeps, FP64 residual and
                                  iterative refinement: the step matches FP64 to the
                                  refinement tolerance (the oil form's increment is
                                  assembled in plain FP32, as in ADS_PREC_MIXED_FAST) */
#define ADS_PREC_MIXED_FAST 2  /* as ADS_PREC_MIXED with the increment assembled in plain
                                  FP32: faster, but its rounding (~1e-7 relative in the
                                  increment) stays in the step */

/* integrand forms (replace the RHS_fun callback) */
#define ADS_FORM_PROJECT 0  /* J W v f: L2Projection, heat at t = 0 */
#define ADS_FORM_HEAT 1     /* J W (v u + dt (-kappa grad u . grad v + v f)): heat at t > 0 */
#define ADS_FORM_OIL 2      /* J W (v u + dt (-Kq exp(mu u) grad u . grad v + v (pump - max(0, w u)))):
                               the oil problem at t > 0, problems/oil/RHS_eq.F90:69-92 */

/* 3-D permutations of ReorderRHSFor{Y,Z,X} */
#define ADS_REORDER_FOR_Y 0 /* F(x, y+z*Ny) -> F2(y, x+z*Nx) */
#define ADS_REORDER_FOR_Z 1 /* F2(y, x+z*Nx) -> F3(z, x+y*Nx) */
#define ADS_REORDER_FOR_X 2 /* F3(z, x+y*Nx) -> F(x, y+z*Ny) */

typedef struct ads_opts {
  int precision;      /* ADS_PREC_FP64, ADS_PREC_MIXED or ADS_PREC_MIXED_FAST */
  double refine_tol;  /* mixed: stop when ||F - M u||_2 <= refine_tol * ||F||_2 (default 1e-13) */
  int max_refine;     /* mixed: maximum refinement corrections per solve */
  int device;         /* CUDA device ordinal */
} ads_opts;

typedef struct ads_handle ads_handle;

/* per-step statistics of the last ads_step / ads_steps call */
typedef struct ads_stats {
  double l2norm;        /* the step's l2norm (problems/heat/main.F90:53) */
  double rel_residual;  /* mixed: an upper bound of the final ||F - M u|| / ||F|| (the
                           certified bound of the FP32 updated residual, or the FP64
                           residual where that decided); 0 for FP64 */
  int refinements;      /* corrections applied in the last solve (mixed) */
  int converged;        /* 1 if the refinement reached refine_tol (mixed), 1 for FP64 */
  int fp64_residuals;   /* FP64 residuals that ran in the last solve (mixed): one per
                           correction, plus one more where the certified bound stayed
                           above refine_tol and an FP64 residual decided; 0 for FP64 */
  int host_path;        /* the last ads_step_host: 1 = the step's kernels read u_in and wrote
                           u_out in place, 2 = they did, found the coefficient scale guessed
                           from the previous step off and the step was redone on staged
                           copies, 0 = staged copies (ads_set_coeffs, ads_step,
                           ads_get_coeffs); 0 after any other call that steps */
} ads_stats;

int ads_default_opts(ads_opts* opts);

/* initialize: n[3] = functions minus one per axis, p[3] = degrees.
 * Each degree must be in {1,2,3,4} and each axis needs >= 2 elements; anything
 * else returns ADS_ERR_UNSUPPORTED.  Equal degrees with at most 448 DOFs per
 * axis run the tuned kernels in every precision.  Unequal degrees, or a longer
 * axis, run FP64 only (general assembly and mass kernels for unequal degrees,
 * banded LU solves along every axis): ADS_PREC_MIXED and ADS_PREC_MIXED_FAST
 * return ADS_ERR_UNSUPPORTED there, as do the oil form and
 * ads_residual_noalloc with unequal degrees. */
int ads_create(const int n[3], const int p[3], const ads_opts* opts, ads_handle** out);
int ads_destroy(ads_handle* h);
const char* ads_last_error(const ads_handle* h);
const char* ads_status_string(int status);

int ads_dims(const ads_handle* h, int nelem[3], int ndof[3], int nq[3]);
/* X[k + q*e] for axis 0/1/2 (Gauss points of element e, BasisData's X) */
int ads_qp_points(const ads_handle* h, int axis, double* X);
/* knots U[n+p+2], O[E], J[E], W[q], NN[((e*q + k)*(p+1) + a)*2 + d] */
int ads_axis_tables(const ads_handle* h, int axis, double* U, int* O, double* J, double* W,
                    double* NN);

/* Select the integrand.  f_qp: projection target (PROJECT) or source term
 * (HEAT, may be NULL = 0) or pumping(X) (OIL, required).  kappa_qp:
 * per-point conductivity (HEAT, may be NULL, then kappa is used) or Kq(X)
 * (OIL, required: the Kqvals cache of problems/oil/input_data.F90:333-395).
 * Arrays are copied; the caller keeps ownership. */
int ads_set_form(ads_handle* h, int form, const double* f_qp, const double* kappa_qp,
                 double kappa, double dt);
/* The rest of the oil problem's pointwise data (problems/oil/input_data.F90):
 * drain_qp = the draining weight w(X) with draining(u, X) = w(X) u (:265-283),
 * mu = the exponent of bq = exp(mu u) (:297-303; mi = 10 there).  Needed
 * before stepping with ADS_FORM_OIL; resets the drained total. */
int ads_set_oil(ads_handle* h, const double* drain_qp, double mu);
/* SaveSplinePlot + EvalSpline (src/plot.F90:111-140, src/basis.F90:323-369)
 * on the current coefficients: vals[ix + res0*(iy + res1*iz)] = the spline at
 * x = lerp(ix/(res0-1), range[0], range[1]), y from range[2..3], z from
 * range[4..5] (res 2..4096 per axis).  With name non-NULL the samples are
 * also written to name.vti as VtkOutput does (src/vtk.F90:15-77).  vals may
 * be NULL.  PrintSolution (src/ADS.F90:955-989) is name "step<iter>", range
 * [0,1]^3, res 31^3. */
int ads_save_spline_plot(ads_handle* h, const char* name, const double range[6], const int res[3],
                         double* vals);
/* VtkOutput (src/vtk.F90:15-77) alone: an ASCII VTK ImageData file name.vti
 * with the res0 x res1 x res2 samples (x fastest) in F30.10 notation.  No
 * handle or GPU needed. */
int ads_write_vti(const char* name, const int res[3], const double* vals);
/* The oil problem's `drained` statistic (problems/oil/RHS_eq.F90:87, printed
 * by ComputeResults, problems/oil/input_data.F90:83-99): the sum over the
 * steps since ads_set_oil of J W v dt max(0, w u) over points and test
 * functions. */
int ads_get_drained(const ads_handle* h, double* drained);

/* Coefficient state (host buffers, x-fastest). */
int ads_set_coeffs(ads_handle* h, const double* u);
int ads_get_coeffs(ads_handle* h, double* u);

/* One Step: assemble with the current form from the current coefficients,
 * Kronecker solve, store the solution as the new coefficients.  l2norm may be
 * NULL; it is the step's sum of J W v u^2 over points and test functions,
 * the integral of the input state squared: FP64 sums with ADS_PREC_FP64;
 * with the mixed precisions it is accumulated from the coefficients' FP32
 * high parts (relative error ~1e-7, while the new state itself matches the
 * FP64 step to ~1e-13). */
int ads_step(ads_handle* h, double* l2norm);
/* One Step on a caller's state arrays, as Step (src/ADS.F90:437-461) updates
 * the state it is given: u_out = the step from u_in (both host layout,
 * x-fastest, ndof entries; u_out may be u_in), the handle's coefficients
 * become u_out, l2norm as ads_step (may be NULL).  The results are those of
 * ads_set_coeffs(u_in), ads_step, ads_get_coeffs(u_out).  With the mixed
 * heat step on a regular geometry, and buffers the device can address
 * (pinned or registered host memory, device memory of the handle's GPU, or
 * any host memory where the device reads pageable memory), the increment
 * assembly reads u_in in place (its transfer hidden behind the assembly's
 * arithmetic) and keeps it as the handle's coefficients, and the final
 * update writes u_out in place; the coefficient scale comes from the
 * previous step and is checked, and a step whose scale was off is redone on
 * staged copies (ads_stats.host_path). */
int ads_step_host(ads_handle* h, const double* u_in, double* u_out, double* l2norm);
/* MultiStep(iter, mix, RHS_fun, ...) (src/ADS.F90:391-429): three substeps,
 * substep s assembling with the form (u from the start of the step, grad u
 * from the current coefficients, as FormUn(s) provides them) and solving
 * (A_s (x) A_s (x) A_s) u = F with A_s = mix[4s] M + mix[4s+1] K +
 * mix[4s+2] B + mix[4s+3] BT (MKBBT, src/projection_engine.F90:63-132), by
 * a banded LU with partial pivoting.  mix is the reference's mix(4,3) in
 * column order.  FP64 on both precisions; PROJECT and HEAT forms.  l2norm
 * (may be NULL) is the step's, which integrates the start-of-step state. */
int ads_multistep(ads_handle* h, const double mix[12], double* l2norm);
/* k Steps; l2norms (k entries) may be NULL.  Runs without host round trips. */
int ads_steps(ads_handle* h, int k, double* l2norms);
int ads_get_stats(const ads_handle* h, ads_stats* st);

/* Parts of the step, host buffers in and out. */
int ads_assemble(ads_handle* h, double* F_out, double* l2norm);  /* from current coeffs */
int ads_solve(ads_handle* h, const double* F, double* u_out);    /* (Mx(x)My(x)Mz) u = F */
int ads_apply_mass(ads_handle* h, const double* u, double* out); /* (Mx(x)My(x)Mz) u     */
int ads_reorder(ads_handle* h, int kind, const double* in, double* out);

/* Device-resident variants: pointers are device addresses of x-fastest
 * double arrays of ndof entries (ads_set/get with copies on the handle's
 * stream, no host synchronisation). */
int ads_set_coeffs_device(ads_handle* h, const double* d_u);
int ads_get_coeffs_device(ads_handle* h, double* d_u);

/* No counterpart in the reference.  For callers that must not allocate device
 * memory — a program whose device memory is all reserved up front by its own
 * pool, or one that keeps other streams busy and cannot take the device-wide
 * synchronisation of cudaFree — the residual r = F - (Mx(x)My(x)Mz) u of the
 * handle's mass matrix on caller-owned device arrays (dense, x fastest, ndof
 * doubles each; d_F may be NULL for r = M u; d_r may equal d_F but must not
 * overlap d_u).  norms (host, may be NULL) receives ||r||^2, ||F||^2 and
 * max|r|; when it is given the call waits for the handle's stream, otherwise
 * it only enqueues.  Its working storage is a fixed device array compiled
 * into the library (3 * ADS_NOALLOC_MAX_CTAS + 8 doubles, 196,672 bytes per
 * GPU, held until exit); it calls no cudaMalloc, cudaFree or allocating
 * library routine.  Sizes needing more than ADS_NOALLOC_MAX_CTAS residual
 * tiles of 32 x 8 x 32 DOFs, ceil(Nx/32) * ceil(Ny/8) * ceil(Nz/32) > 8192
 * (the largest cube is 384^3 DOFs), return ADS_ERR_ARG.  The array is shared
 * by all calls on a device and keeps the last call's contents: calls that
 * overlap on the GPU race on it.  The first call on each device looks up the
 * array's address and keeps it for the process: make that call before any
 * stream capture, and do not call again on a device after a cudaDeviceReset
 * of it. */
#define ADS_NOALLOC_MAX_CTAS 8192
int ads_residual_noalloc(ads_handle* h, const double* d_F, const double* d_u, double* d_r,
                         double norms[3]);

/* Adjoint of K explicit heat steps from u0 with the current HEAT form:
 * loss = 1/2 (u^K - u_target)^T (Mx(x)My(x)Mz) (u^K - u_target).
 * grad_u0 (ndof) and grad_kappa_qp (quadrature-point layout; only with a
 * per-point kappa) may be NULL.  States are checkpointed every
 * checkpoint_every steps and recomputed segment by segment.  The forward
 * uses the handle's precision; the backward runs in FP64. */
int ads_heat_adjoint(ads_handle* h, int K, int checkpoint_every, const double* u0,
                     const double* u_target, double* loss, double* grad_u0,
                     double* grad_kappa_qp);

/* Tangent-linear (forward-mode) model of K explicit heat steps from u0 with
 * the current HEAT form, the companion of ads_heat_adjoint: duK (ndof) =
 * d u^K along the direction (du0, dkappa_qp) of the initial state (ndof, may
 * be NULL = 0) and of the per-point conductivity (quadrature-point layout,
 * may be NULL = 0; needs no per-point kappa in the form).  uK (may be NULL)
 * receives u^K.  Each step assembles A w^n with the FP64 kernels (the source
 * does not depend on u0 or kappa and is left out), adds -dt K(dkappa) u^n,
 * and solves with the FP64 sweeps; the forward uses the handle's precision.
 * With loss L = 1/2 e^T M e, e = u^K - u_target, the directional derivative
 * is e^T M duK: no finite-difference cancellation at any step size. */
int ads_heat_jvp(ads_handle* h, int K, const double* u0, const double* du0, const double* dkappa_qp,
                 double* uK, double* duK);

/* Host-only setup helpers (no GPU needed): the tables ads_create builds for
 * one axis.  U[n+p+2], O[E], J[E], W[p+1], X[E*(p+1)], NN[E*(p+1)*(p+1)*2],
 * band[(2p+1)*(n+1)] with band[(m+p)*(n+1) + i] = M[i][i+m] (MKBBT mass
 * matrix, src/projection_engine.F90:63-132), fac/tfac[(2p+2)*(n+1)] the LU
 * factor rows of the normal and transposed banded solves.  Any output may be
 * NULL.  Returns ADS_ERR_UNSUPPORTED for p outside 1..4. */
int ads_axis_setup(int n, int p, double* U, int* O, double* J, double* W, double* X, double* NN,
                   double* band, double* fac, double* tfac);

/* Diagnostic with no counterpart in the reference: measured FMA throughput of
 * the FP32 (fp64 = 0) or FP64 (fp64 = 1) pipe of a device, in TFLOP/s
 * (an FMA counts as two flops).  Used as the roofline denominator of the
 * SIMT-bound assembly kernel. */
int ads_fma_peak(int device, int fp64, double* tflops);

/* Stream interop and per-kernel timing (CUDA events on the handle's stream). */
void* ads_get_stream(const ads_handle* h);
int ads_set_stream(ads_handle* h, void* stream);
int ads_timing_enable(ads_handle* h, int on);
/* names: comma-separated kernel names; times_ms/launches: per kernel totals */
int ads_timing_read(ads_handle* h, char* names, int names_len, double* times_ms, int* launches,
                    int max_kernels, int* n_kernels);
int ads_timing_reset(ads_handle* h);
/* The same timings summed per phase of the step, named as the reference's
 * PERFORMANCE output names them (src/ADS.F90:497-754): "Form 3D RHS"
 * (FormUn + Form3DRHS, with the FP32/double-float scaling pass and the
 * fixup), "Solve 1", "Solve 2", "Solve 3" (each direction's sweep, which also
 * does that direction's Gather, Scatter and ReorderRHSFor*: they have no
 * launches of their own), and, with no counterpart in the reference,
 * "Refinement" (the mixed solve's FP64 residuals and corrections), "Update"
 * (u += delta of the mixed heat step) and "Other" (bookkeeping).  The mass
 * matrices are factorised once at ads_create (the reference's "Mass matrix n"
 * rebuilds them every substep), so that phase never appears.  Each phase
 * is also an NVTX range around its launches. */
int ads_phase_timing_read(ads_handle* h, char* names, int names_len, double* times_ms, int* launches,
                          int max_phases, int* n_phases);
/* number of this library's kernel launches since the last reset */
long long ads_launch_count(const ads_handle* h);
int ads_launch_count_reset(ads_handle* h);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* ADS_GPU_H */
