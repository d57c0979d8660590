#!/usr/bin/env python3
"""Benchmark of the explicit ADS heat step on GB300.

Metric: DOF-updates/s per ADS step at 256^3 elements, p = 2,
FP64 vs mixed precision: the heat increment assembled in double-float
arithmetic on the FP32 pipe, FP32 banded sweeps, and FP64 iterative
refinement of each Kronecker solve to <= 1e-13 relative residual, so that the
step matches the FP64 step to ~1e-13 relative L2 (reported per step).  Workload: heat equation, kappa = 1, dt = 1e-5, initial
state = L2 projection of 16 seeded Gaussian bumps (synthetic, seed 0).

`value` is the mixed-precision step with its state resident in HBM, timed with
CUDA events over exactly --steps steps (graph-launched); the FP64 drop-in step
and the plain-FP32-assembly variant (ADS_PREC_MIXED_FAST) are timed the same
way and reported inside "config" with the mixed path's error against FP64 and
against the oracle.  `e2e` times the same steps
through the C-ABI with host buffers: every step copies the coefficients in
from pinned host memory, steps, and copies the solution back.  A separate pass
with per-kernel CUDA events gives the roofline of the dominant kernel.

--impl reference times the oracle (a C++ restatement of the reference's
Fortran FP64 path; the Fortran itself cannot be built here) on the host cores.

Multi-GPU: the step does not shard here (one GPU per ADS instance), so N > 1
runs N independent replicas, one per rank; value = all ranks' DOF-updates
divided by the slowest rank's time.
"""
import argparse
import math
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-updates/s per ADS step, 256³ p=2: FP64 vs FP32+refine at ≤1e-10 rel err"
UNIT = "DOF-updates/s"
HBM_FALLBACK_GBS = 6800.0

# DRAM traffic per launch of the dominant kernels from ncu captures
# (dram__bytes_read.sum + dram__bytes_write.sum, bytes), keyed by (kernel,
# workload); the captures and the commands are summarised in profiles/.  Writes
# still held in L2 when a kernel ends are not counted by the capture.
NCU_TRAFFIC = {
    ("assemble_df", "heat256p2"): 163.093760e6 + 163.435776e6,
    ("assemble_f32", "heat256p2"): 164.389888e6 + 163.244544e6,
    ("assemble_f64", "heat256p2"): 167.988992e6 + 164.684544e6,
    ("residual_f64", "heat256p2"): 291.368960e6 + 57.232128e6,
    ("resid_update", "heat256p2"): 280.538112e6 + 91.008256e6,
    ("fixup", "heat256p2"): 272.985600e6 + 90.721024e6,
    ("sweep_z_f32", "heat256p2"): 71.630592e6 + 80.654592e6,
    ("sweep_z_f32_corr", "heat256p2"): 70.957568e6 + 19.331328e6,
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--elements", type=int, default=256)
    ap.add_argument("--degree", type=int, default=2)
    ap.add_argument("--dt", type=float, default=1e-5)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-aux", action="store_true",
                    help="skip the adjoint (96^3), variable-conductivity (128^3) and 256^3 p=3 measurements")
    ap.add_argument("--ref-slab", type=int, default=32,
                    help="reference arm: z elements of the 256x256xS sample per step")
    ap.add_argument("--only", choices=["mixed", "fp64", "mixed_fast"], default=None,
                    help="profiling case: set up one precision and run warmup + steps only (for ncu)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v, device):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f), "measured"
        except Exception:
            pass
    return None, "fallback"


def hbm_peak():
    peaks, src = load_peaks()
    if peaks:
        for k in ("hbm_gbs", "hbm_GBs", "hbm_gb_s"):
            if k in peaks:
                v = peaks[k]
                if isinstance(v, dict):
                    v = v.get("burst", v.get("value"))
                return float(v), "of measured"
    return HBM_FALLBACK_GBS, "of fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_ready(self, timeout=5.0):
        """Until the first sample is in: nvidia-smi's start-up (NVML
        initialisation) then lies before, not inside, a timed region."""
        t_end = time.perf_counter() + timeout
        while self.proc is not None and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.01)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0=None, t1=None):
        rows = []
        for t, line in self.lines:
            if t0 is not None and (t < t0 or t > t1):
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_assembly_flops(P, nelem):
    """Flops of the sum-factorised heat assembly per launch: per element
    interpolation (2q + 3q^2 + 4q^3)(p+1) FMA, test contraction the same,
    and 9 flops per quadrature point for the integrand."""
    q = P + 1
    fma = 2 * (2 * q + 3 * q * q + 4 * q ** 3) * (P + 1)
    return (2 * fma + 9 * q ** 3) * nelem


# FP32 instructions of the double-float operations of k_assemble_df
# (df32.cuh): product = FMUL + 3 FFMA, multiply-add = product + two-sum
# (6 FADD/FSUB) + 2 FADD, sum = two-sum + 2 FADD
DF_MUL, DF_MAC, DF_ADD = 4, 12, 8


def df_assembly_ops(P, nelem, sym=(0.0, 0.0, 0.0), fold=False):
    """FP32 operations (each FFMA, FADD or FMUL one operation) of the
    double-float heat increment assembly per launch, counted from the kernel's
    stages for the work each element needs (the brick halo's repeated columns
    are not counted): the z interpolation of one DOF column per element layer,
    the y interpolation and the y/z test contraction of one (element row, DOF
    column) pair, the x stage of one element, and the DOF-plane accumulation.
    At p = 2, sym = the fractions of the x stage, element rows and layers
    that run the even-odd form (centro-symmetric elements), whose sums cost
    less: an interpolation pair 52-68 operations where the direct sums take 84.
    fold: constant conductivity and no source, where the y and z point weights
    sit in the tables, the x quadrature in the brick's x stiffness and mass
    bands, and -dt kappa multiplies each written DOF, so the x stage is three
    banded products (2P + 1 wide) per row of points and DOF column."""
    q = P + 1
    z = q * (2 * DF_MUL + 2 * P * DF_MAC)
    y = q * q * (3 * DF_MUL + 3 * P * DF_MAC)
    weights = 3 if fold else DF_MUL + DF_MUL + 2      # l2 weight (and c = Jx Wx Jy Wy Jz Wz (-dt kappa))
    per_kx = (3 * DF_MUL + 3 * P * DF_MAC) + (1 + P) + weights + 3 * DF_MUL
    contraction = 3 * (P + 1) * DF_MUL + (q - 1) * 3 * (P + 1) * DF_MAC
    row = 0 if fold else 2 * DF_MUL                    # Jy Wy Jz Wz and its -dt kappa per row
    x = q * q * (row + q * per_kx + contraction + 3 * P * DF_ADD)
    if fold:
        # per row and DOF column: the reciprocal of Jy Wy Jz Wz, the l2norm's
        # Y0 (Mx Y0) in FP32, then Kx Y0, Mx Y1, Mx Y2 in double-float
        x = q * q * (3 + (2 * P + 1) + 2 + 3 * (DF_MUL + 2 * P * DF_MAC))
    yt = q * ((P + 1) * (2 * DF_MUL + DF_MAC) + (q - 1) * (P + 1) * 3 * DF_MAC)   # y test
    za = q * (P + 1) ** 2 * 2 * DF_MAC                                            # z test
    acc = (P + 1) ** 2 * DF_ADD + (DF_MUL if fold else 0)
    if P == 2:
        fx, fy, fz = sym
        # even-odd sums: s and d of the inputs (2 sums), per output pair a
        # product and a multiply-add plus a product, the pair's 2 sums, the
        # middle output a product and a multiply-add (N) or a product (dN)
        eo_n = 2 * DF_ADD + (DF_MUL + DF_MAC) + DF_MUL + 2 * DF_ADD + (DF_MUL + DF_MAC)   # 68
        eo_d = 2 * DF_ADD + (DF_MUL + DF_MAC) + DF_MUL + 2 * DF_ADD + DF_MUL               # 56
        eo_nd = eo_n + eo_d - 2 * DF_ADD                                                   # 108: s, d shared
        z_eo = eo_nd
        y_eo = q * (eo_nd + eo_n)
        if fold:
            x_row = None  # the banded x stage has no even-odd form
        else:
            x_row = 2 * DF_MUL + q * (DF_MUL + 1) + 15 + (eo_d + 3 * DF_MUL + eo_d) + 2 * (eo_n + 3 * DF_MUL + eo_n)
        x_eo = x if fold else q * q * (x_row + 3 * P * DF_ADD)
        yt_eo = q * (eo_n + eo_d + 3 * DF_ADD + eo_n)
        # fold: the z test over the point pair (0, 2) and the middle point in
        # even-odd form: per DOF row the pair's 4 sums and 6 multiply-adds, the
        # middle's 3 multiply-adds, and the final 2 sums
        za_eo = (P + 1) * (4 * DF_ADD + 9 * DF_MAC + 2 * DF_ADD) if fold else za
        z = fz * z_eo + (1 - fz) * z
        y = fy * y_eo + (1 - fy) * y
        x = fx * x_eo + (1 - fx) * x
        yt = fy * yt_eo + (1 - fy) * yt
        za = fz * za_eo + (1 - fz) * za
    return (z + y + x + yt + za + acc) * nelem


def even_odd_fractions(A, E, p):
    """Fractions of the x stage (bricks of 32 - p elements, all of them
    centro-symmetric), of element rows and of layers that the double-float
    assembly runs in even-odd form at p = 2 (the library's criterion,
    4e-15 of a table's largest entry)."""
    import numpy as np
    if p != 2:
        return (0.0, 0.0, 0.0)
    NN = A.axis_setup(E + p - 1, p)["NN"].reshape(E, 3, 3, 2)
    N, D = NN[..., 0], NN[..., 1]
    en = np.abs(N - N[:, ::-1, ::-1]).max(axis=(1, 2))
    ed = np.abs(D + D[:, ::-1, ::-1]).max(axis=(1, 2))
    sym = (en <= 4e-15 * np.abs(N).max(axis=(1, 2))) & (ed <= 4e-15 * np.abs(D).max(axis=(1, 2)))
    tx = 32 - p
    fx = sum(min(tx, E - x0) for x0 in range(0, E, tx) if sym[x0:x0 + tx].all()) / E
    f = float(sym.mean())
    return (fx, f, f)


def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    import numpy as np
    from ads_mpi_gb300 import inputs
    O.build()
    E, p = args.elements, args.degree
    S = max(2, min(args.ref_slab, E))
    n = (E + p - 1, E + p - 1, S + p - 1)
    o = O.Oracle(n, (p, p, p))
    X = o.axis_tables(0)["X"]
    Z = o.axis_tables(2)["X"]
    u0 = inputs.gaussian_bumps_separable(X, X, Z, seed=args.seed)
    o.step(O.FORM_PROJECT, fqp=u0)
    for _ in range(args.warmup):
        o.step(O.FORM_HEAT, kappa=1.0, dt=args.dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(O.FORM_HEAT, kappa=1.0, dt=args.dt)
    dt_s = time.perf_counter() - t0
    value = o.N * args.steps / dt_s
    cores = O.num_threads()
    sample = (f"oracle (C++ restatement of the reference FP64 path, 1 rank, OpenMP {cores} threads) on a "
              f"{E}x{E}x{S}-element slab of the {E}^3 p={p} heat step per step")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"heat {E}^3 elements p={p} dt={args.dt} kappa=1 (sample {E}x{E}x{S})",
                   "elements": [E, E, S], "degree": p, "dofs_per_step": o.N},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_device_steps(torch, g, K):
    ext = torch.cuda.ExternalStream(g.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(ext)
    g.steps(K)
    e1.record(ext)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def time_e2e(torch, g, K, host_in, host_out, three_calls=False):
    """K steps from the pinned host state host_in into host_out through the
    C-ABI: ads_step_host (the step's kernels read host_in and write host_out),
    or ads_set_coeffs + ads_step + ads_get_coeffs."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        if three_calls:
            g.set_coeffs(host_in)
            g.step()
            g.coeffs_into(host_out)
        else:
            g.step_host(host_in, host_out)
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def kernel_profile(g, K, phases=None):
    g.timing(True)
    g.timing_reset()
    g.steps(K)
    t = g.timing_read()
    if phases is not None:
        phases.update(g.phase_timing_read())
    g.timing(False)
    return t


def run_only(args, local):
    """Minimal case for ncu: one handle of the chosen precision, the seeded
    initial state, --warmup + --steps eager steps, nothing else."""
    import ads_mpi_gb300 as A
    from ads_mpi_gb300 import inputs
    E, p = args.elements, args.degree
    n = (E + p - 1,) * 3
    prec = {"mixed": A.PREC_MIXED, "fp64": A.PREC_FP64, "mixed_fast": A.PREC_MIXED_FAST}[args.only]
    g = A.ADS(n, (p, p, p), precision=prec, refine_tol=REFINE_TOL, device=local)
    X = [g.qp_points(a) for a in range(3)]
    f = inputs.gaussian_bumps_separable(X[0], X[1], X[2], seed=args.seed)
    g.set_form(A.FORM_PROJECT, f_qp=f)
    del f
    g.step()
    g.set_form(A.FORM_HEAT, kappa=1.0, dt=args.dt)
    g.timing(True)  # eager launches, one kernel at a time
    g.steps(args.warmup + args.steps)
    t = g.timing_read()
    print(json.dumps({"only": args.only, "elements": E, "degree": p, "kernels_ms": t}), flush=True)


def finite_or_none(v):
    """JSON-safe copy: non-finite floats become null."""
    if isinstance(v, dict):
        return {k: finite_or_none(x) for k, x in v.items()}
    if isinstance(v, (list, tuple)):
        return [finite_or_none(x) for x in v]
    if isinstance(v, float) and not math.isfinite(v):
        return None
    return v


REFINE_TOL = 1e-13
STABLE_DT = {2: 1e-7, 3: 5e-8}   # dt * lambda_max = 0.43 (p = 2) and 0.46 (p = 3) at 256^3


def greville_bumps(A, n, p, seed):
    """The seeded bumps sampled at the Greville abscissae (coefficients of a
    quasi-interpolant; used where a projection would need a multi-GB array of
    quadrature values on the host)."""
    import numpy as np
    U = A.axis_setup(n, p)["U"]
    xi = np.array([U[i + 1:i + p + 1].mean() for i in range(n + 1)])
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.0, 1.0, 16)
    cen = rng.uniform(0.2, 0.8, (16, 3))
    u0 = np.zeros((n + 1,) * 3)
    for b in range(16):
        gx, gy, gz = (np.exp(-(xi - cen[b, d]) ** 2 / (2 * 0.05 ** 2)) for d in range(3))
        u0 += amp[b] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return u0.ravel()


class DevDiff:
    """Relative L2 difference of two handles' coefficients, on the device."""

    def __init__(self, torch, N, dev):
        self.torch = torch
        self.a = torch.empty(N, dtype=torch.float64, device=f"cuda:{dev}")
        self.b = torch.empty(N, dtype=torch.float64, device=f"cuda:{dev}")

    def __call__(self, g, gref):
        g.get_coeffs_device(self.a.data_ptr())
        gref.get_coeffs_device(self.b.data_ptr())
        self.torch.cuda.synchronize()
        return float(self.torch.linalg.norm(self.a - self.b) / self.torch.linalg.norm(self.b))


def side_by_side(torch, A, dev, n, p, u0, dt, steps, precs):
    """Step FP64 and the given precisions from u0 side by side: per-step
    relative L2 difference of each against FP64."""
    hs = {0: A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)}
    for pr in precs:
        hs[pr] = A.ADS(n, (p, p, p), precision=pr, refine_tol=REFINE_TOL, max_refine=3, device=dev)
    diff = DevDiff(torch, hs[0].N, dev)
    errs = {pr: [] for pr in precs}
    for g in hs.values():
        g.set_form(A.FORM_HEAT, kappa=1.0, dt=dt)
        g.set_coeffs(u0)
    conv = True
    for _ in range(steps):
        for g in hs.values():
            g.step()
        for pr in precs:
            errs[pr].append(diff(hs[pr], hs[0]))
            conv = conv and bool(hs[pr].stats()["converged"])
    for g in hs.values():
        g.cleanup()
    return errs, conv


def aux_runs(args, dev):
    """The other configurations of the workload family, measured after the
    headline step (rank 0 only):
      C1 the 32^3 p=2 L2 projection (one assembly + one solve) against the oracle;
      C2 heat 128^3 p=2 FP64, dt = 1e-5, 200 steps;
      C3 heat 256^3, p = 2 and 3: mixed against FP64 step by step (100 steps at a
         stable dt, the first steps at the configured dt) and the p = 3 timings;
      C4 the FP64 adjoint at 96^3 (50 steps, checkpoint every 10) against the
         tangent-linear model (forward mode, no finite-difference cancellation)
         and central finite differences (h = 1e-6) along 8 seeded directions;
      C5 the conductivity gradient at 128^3 (kappa = exp(g), g a seeded Gaussian
         random field, 100 steps, mixed forward + FP64 adjoint) against an
         all-FP64 gradient, with the inputs scaled by a power of two at the
         configured dt so the loss stays finite;
      the oil problem at 128^3 (mixed against FP64, with its drained statistic)."""
    import numpy as np
    import torch
    import ads_mpi_gb300 as A
    from ads_mpi_gb300 import inputs
    from oracle import oracle as O
    out = {}
    dtv = args.dt

    def sync_time(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    def bumps_state(g, seed):
        X = [g.qp_points(a) for a in range(3)]
        f = inputs.gaussian_bumps_separable(X[0], X[1], X[2], seed=seed, device=f"cuda:{dev}")
        g.set_form(A.FORM_PROJECT, f_qp=f)
        del f
        g.step()
        return g.coeffs()

    # ---- C1: L2 projection 32^3 p=2 (problems/L2Projection/main.F90:43-57) ----
    E, p, reps = 32, 2, 20
    n = (E + p - 1,) * 3
    g = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    f = inputs.projection_target(*g.qp_coords(), seed=args.seed)
    g.set_form(A.FORM_PROJECT, f_qp=f)
    l2 = g.step()
    secs = time_device_steps(torch, g, reps)   # the projection step does not depend on u: same work each time
    o = O.Oracle(n, (p, p, p))
    l2o = o.step(O.FORM_PROJECT, fqp=f)
    err = float(np.linalg.norm(g.coeffs() - o.coeffs()) / np.linalg.norm(o.coeffs()))
    g.set_form(A.FORM_PROJECT)
    l2one = g.step()
    kat = float(np.abs(g.coeffs() - 1.0).max())
    out["c1_projection_32p2"] = {
        "config": "L2 projection 32^3 p=2 FP64 of sin(2 pi x)sin(2 pi y)sin(2 pi z) + 0.1 sum_8 a_k exp(-|x-c_k|^2/0.01) "
                  "(seeded): one assembly + one solve", "unit": UNIT,
        "value": g.N * reps / secs, "ms_per_projection": 1e3 * secs / reps,
        "rel_err_vs_oracle": err, "l2norm_rel_err_vs_oracle": abs(l2 - l2o) / abs(l2o),
        "known_answer_f1_max_abs_err": kat, "known_answer_l2norm_err": abs(l2one - 1.0)}
    o.close()
    g.cleanup()

    # ---- C2: heat 128^3 p=2 FP64, dt = 1e-5, 200 steps (problems/heat/main.F90:49-60) ----
    # dt lambda_max = 10.6: rounding seeds the unstable modes, which grow by
    # ~9.6x per step until the l2norm (an integral of u^2) overflows.  The
    # overflow step is found by stepping the configured state; the 200 steps
    # are timed from the same state scaled by 2^-600 (the step is linear, so
    # the trajectory is the same up to that scale and stays finite).
    E, p, K2 = 128, 2, 200
    n = (E + p - 1,) * 3
    g = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    u0 = bumps_state(g, args.seed)
    g.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
    g.set_coeffs(u0)
    overflow_step = None
    l2s = []
    for i in range(K2):
        try:
            l2s.append(g.step())
        except A.ADSError as e:
            if e.status != 4:
                raise
            overflow_step = i + 1
            break
    sc = 2.0 ** -600
    g.set_coeffs(u0 * sc)
    g.steps(3)
    g.set_coeffs(u0 * sc)
    t0 = time.perf_counter()
    secs = time_device_steps(torch, g, K2)
    wall = time.perf_counter() - t0
    uK = g.coeffs()
    row = {"config": "heat 128^3 p=2 FP64, kappa=1, dt=1e-5, 200 steps from the projection of 16 seeded bumps",
           "unit": UNIT, "value": g.N * K2 / secs, "ms_per_step": 1e3 * secs / K2, "wall_s": wall,
           "dt_lambda_max": dtv * 3 * 21.6 * E * E,
           "l2norm_overflow_step_unscaled": overflow_step,
           "l2norm_steps_1_10_50": [l2s[i] for i in (0, 9, 49) if i < len(l2s)],
           "timed_from_state_scaled_by": "2^-600", "scaled_final_finite": bool(np.isfinite(uK).all()),
           "scaled_final_max_abs_u": float(np.abs(uK).max())}
    gm = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=REFINE_TOL, device=dev)
    gm.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
    gm.set_coeffs(u0 * sc)
    gm.steps(3)
    gm.set_coeffs(u0 * sc)
    row["mixed_value"] = gm.N * K2 / time_device_steps(torch, gm, K2)
    gm.cleanup()
    out["c2_heat_128p2_fp64"] = row
    g.cleanup()

    # ---- C3: 256^3 p=2 and p=3, mixed vs FP64 step by step ----
    c3 = {}
    for p in (2, 3):
        E = 256
        n = (E + p - 1,) * 3
        u0 = greville_bumps(A, n[0], p, args.seed)
        K3 = 100
        errs_s, conv_s = side_by_side(torch, A, dev, n, p, u0, STABLE_DT[p], K3, (A.PREC_MIXED, A.PREC_MIXED_FAST))
        errs_c, conv_c = side_by_side(torch, A, dev, n, p, u0, dtv, 5, (A.PREC_MIXED, A.PREC_MIXED_FAST))
        row = {"stable_dt": STABLE_DT[p], "steps": K3,
               "mixed_rel_err_per_step_stable_dt_max": max(errs_s[A.PREC_MIXED]),
               "mixed_rel_err_stable_dt_steps_1_10_50_100": [errs_s[A.PREC_MIXED][i] for i in (0, 9, 49, 99)],
               "mixed_fast_rel_err_per_step_stable_dt_max": max(errs_s[A.PREC_MIXED_FAST]),
               "configured_dt": dtv,
               "mixed_rel_err_first_steps_configured_dt": errs_c[A.PREC_MIXED],
               "mixed_fast_rel_err_first_steps_configured_dt": errs_c[A.PREC_MIXED_FAST],
               "all_converged": conv_s and conv_c}
        if p == 3:
            Ks = 10
            for name, pr in (("mixed", A.PREC_MIXED), ("fp64", A.PREC_FP64), ("mixed_fast", A.PREC_MIXED_FAST)):
                gg = A.ADS(n, (p, p, p), precision=pr, refine_tol=REFINE_TOL, device=dev)
                gg.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
                gg.set_coeffs(u0)
                gg.steps(3)
                gg.set_coeffs(u0)
                row[name] = gg.N * Ks / time_device_steps(torch, gg, Ks)
                gg.cleanup()
            row["unit"] = UNIT
            row["mixed_over_fp64"] = row["mixed"] / row["fp64"]
        c3[f"p{p}"] = row
    out["c3_heat_256_mixed_vs_fp64"] = c3

    # ---- C4: adjoint 96^3 p=2 FP64, 50 steps, checkpoint every 10 ----
    def adjoint_check(dtv, fd):
        E, p, K, ck = 96, 2, 50, 10
        n = (E + p - 1,) * 3
        g = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
        u0 = bumps_state(g, args.seed)
        ut_src = bumps_state(g, args.seed + 1)   # perturbed initial state
        g.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
        g.set_coeffs(ut_src)
        g.steps(K)
        u_target = g.coeffs()
        (loss, gu, _), t_adj = sync_time(lambda: g.heat_adjoint(K, ck, u0, u_target, grad=True))
        rng = np.random.default_rng(args.seed + 7)
        h = 1e-6
        jv, fdr = [], []
        for _ in range(8):
            d = rng.standard_normal(g.N)   # entries N(0, 1)
            ad = float(np.dot(gu, d))
            uK, duK = g.heat_jvp(K, u0, du0=d)
            jvp = float((uK - u_target) @ g.apply_mass(duK))
            jv.append(abs(jvp - ad) / max(abs(jvp), abs(ad), 1e-300))
            if fd:
                lp, _, _ = g.heat_adjoint(K, ck, u0 + h * d, u_target, grad=False)
                lm, _, _ = g.heat_adjoint(K, ck, u0 - h * d, u_target, grad=False)
                fdv = (lp - lm) / (2 * h)
                fdr.append(abs(fdv - ad) / max(abs(fdv), abs(ad), 1e-300))
        g.cleanup()
        r = {"dt": dtv, "loss": loss, "forward_backward_s": t_adj, "jvp_rel_err_max": max(jv), "jvp_rel_err": jv}
        if fd:
            r["fd_rel_err_max"] = max(fdr)
            r["fd_rel_err"] = fdr
        return r

    out["c4_adjoint_96p2"] = {
        "config": "heat 96^3 p=2 FP64, 50 steps, checkpoint every 10; loss 1/2||u^50 - u_target||_M^2, "
                  "u_target from a seeded forward run of a perturbed initial state; <grad L, d> along 8 seeded "
                  "N(0,1) directions against the tangent-linear model (ads_heat_jvp) and central FD h=1e-6",
        "configured_dt": adjoint_check(dtv, True), "stable_dt": adjoint_check(1e-6, True), "target_rel_err": 1e-6}

    # ---- C5: variable conductivity, 128^3 p=2, 100 steps: dL/dg, g -> kappa = exp(g) ----
    E, p = 128, 2
    n = (E + p - 1,) * 3
    g0 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    X = [g0.qp_points(a) for a in range(3)]
    g0.cleanup()
    gq = inputs.gaussian_random_field_qp(X[0], X[1], X[2], seed=args.seed, sigma=0.5, corr=0.1,
                                         device=f"cuda:{dev}")
    kappa = np.exp(gq).ravel()
    del gq
    lam = 3 * 21.6 * E * E * float(kappa.max())   # lambda_max of M^-1 K, p = 2
    dt_stable = float(f"{1.5 / lam:.0e}")

    def kappa_check(dtv, K=100, ck=10):
        # the states grow by up to |1 - dt lambda_max| per step; scaling u0 and
        # u_target by 2^-k (k from that bound) keeps u^K, the loss and the
        # adjoint in range; dL/dg scales by 2^-2k
        growth = max(abs(1.0 - dtv * lam), 1.0)
        k = int(math.ceil(K * math.log2(growth))) if growth > 1.0 else 0
        sc = 2.0 ** -k
        g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
        u0 = bumps_state(g64, args.seed) * sc
        g64.set_coeffs(bumps_state(g64, args.seed + 1) * sc)
        g64.set_form(A.FORM_HEAT, kappa_qp=kappa, dt=dtv)
        g64.steps(K)
        u_target = g64.coeffs()
        (l64, _, gk64), t64 = sync_time(lambda: g64.heat_adjoint(K, ck, u0, u_target, grad=False, grad_kappa=True))
        # forward-mode check of the FP64 gradient along one seeded direction of g
        dg = np.random.default_rng(args.seed + 11).standard_normal(kappa.size)
        uK, duK = g64.heat_jvp(K, u0, dkappa=dg * kappa)
        jvp = float((uK - u_target) @ g64.apply_mass(duK))
        vjp = float(gk64 @ (dg * kappa))
        gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=REFINE_TOL, max_refine=3, device=dev)
        gmx.set_form(A.FORM_HEAT, kappa_qp=kappa, dt=dtv)
        (lmx, _, gkmx), tmx = sync_time(lambda: gmx.heat_adjoint(K, ck, u0, u_target, grad=False, grad_kappa=True))
        dg64 = gk64 * kappa    # dL/dg = dL/dkappa * kappa
        dgmx = gkmx * kappa
        n64 = float(np.linalg.norm(dg64))
        err = float(np.linalg.norm(dgmx - dg64) / n64) if np.isfinite(n64) and n64 > 0 else None
        gmx.cleanup()
        g64.cleanup()
        return {"dt": dtv, "input_scale_log2": -k, "loss_mixed": lmx, "loss_fp64": l64,
                "dLdg_rel_l2_err_mixed_vs_fp64": err, "dLdg_norm_scaled": n64,
                "dLdg_norm_log10_unscaled": (math.log10(n64) + 2 * k * math.log10(2.0)) if n64 > 0 else None,
                "jvp_vs_adjoint_rel_err_fp64": abs(jvp - vjp) / max(abs(jvp), abs(vjp), 1e-300),
                "forward_backward_s_mixed": tmx, "forward_backward_s_fp64": t64}

    out["c5_var_kappa_128p2"] = {
        "config": "heat 128^3 p=2, kappa = exp(g), g Gaussian random field sigma 0.5 corr 0.1 at the quadrature "
                  "points, 100 steps, checkpoint every 10; mixed forward (double-float increments, FP64 "
                  "refinement), FP64 adjoint, against an all-FP64 reference gradient",
        "kappa_max": float(kappa.max()), "dt_lambda_max_at_configured_dt": dtv * lam,
        "configured_dt": kappa_check(dtv), "stable_dt": kappa_check(dt_stable)}

    # ---- oil problem (problems/oil/RHS_eq.F90:69-92), 128^3 p=2: mixed vs FP64 ----
    # seeded curves (Kq), pumps and drains; mi = 10; dt at half the explicit
    # limit for the largest Kq exp(mi u) (u stays below 0.1).  The oil
    # increment is assembled in plain FP32 in both mixed modes.
    E, p, Ko, mu = 128, 2, 10, 10.0
    n = (E + p - 1,) * 3
    g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=REFINE_TOL, max_refine=3, device=dev)
    x, y, z = g64.qp_coords()
    of = inputs.oil_fields(x, y, z, seed=args.seed, device=f"cuda:{dev}")
    del x, y, z
    lam = 3 * 21.6 * E * E * float(of["kq"].max()) * float(np.exp(mu * 0.1))
    dto = float(f"{0.5 / lam:.0e}")
    row = {"dt": dto, "mu": mu, "steps": Ko}
    res = {}
    for name, gg in (("fp64", g64), ("mixed", gmx)):
        gg.set_form(A.FORM_PROJECT, f_qp=of["init"])
        gg.step()
        gg.set_form(A.FORM_OIL, f_qp=of["pump"], kappa_qp=of["kq"], dt=dto)
        gg.set_oil(of["drain"], mu=mu)
        gg.steps(2)
        secs = time_device_steps(torch, gg, Ko)
        row[name] = gg.N * Ko / secs
        res[name] = (gg.coeffs(), gg.drained())
    a64 = res["fp64"][0]
    row["mixed_rel_err_vs_fp64"] = float(np.linalg.norm(res["mixed"][0] - a64) / np.linalg.norm(a64))
    row["drained_fp64"], row["drained_mixed"] = res["fp64"][1], res["mixed"][1]
    row["mixed_rel_residual"] = gmx.stats()["rel_residual"]
    out["oil_128p2"] = {"config": "oil problem 128^3 p=2: Kq from 30 seeded curves (Kq in [1, 1000]), 2 pumps, "
                                  "2 drains, mi = 10, projection of the initial state then 2 + 10 steps",
                        "unit": UNIT, **row, "mixed_over_fp64": row["mixed"] / row["fp64"]}
    del of
    gmx.cleanup()
    g64.cleanup()
    return out


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    import ads_mpi_gb300 as A
    from ads_mpi_gb300 import inputs

    A.load()
    dev = local
    torch.cuda.set_device(dev)
    E, p = args.elements, args.degree
    n = (E + p - 1,) * 3
    K, W = args.steps, args.warmup

    # initial state: FP64 projection of the seeded bumps
    g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    X = [g64.qp_points(a) for a in range(3)]
    f = inputs.gaussian_bumps_separable(X[0], X[1], X[2], seed=args.seed, device=f"cuda:{dev}")
    g64.set_form(A.FORM_PROJECT, f_qp=f)
    del f
    g64.step()
    u0 = g64.coeffs()
    N = g64.N
    g64.set_form(A.FORM_HEAT, kappa=1.0, dt=args.dt)

    gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=REFINE_TOL, max_refine=3, device=dev)
    gmx.set_form(A.FORM_HEAT, kappa=1.0, dt=args.dt)
    gfa = A.ADS(n, (p, p, p), precision=A.PREC_MIXED_FAST, refine_tol=REFINE_TOL, max_refine=3, device=dev)
    gfa.set_form(A.FORM_HEAT, kappa=1.0, dt=args.dt)
    handles = (("mixed", gmx), ("fp64", g64), ("mixed_fast", gfa))

    clocks = ClockSampler(dev)
    clocks.start()
    clocks.wait_ready()
    res = {}
    for name, g in handles:
        g.set_coeffs(u0)
        g.steps(W)
        barrier(world)
        g.launch_count_reset()
        t0 = time.perf_counter()
        secs = time_device_steps(torch, g, K)
        t1 = time.perf_counter()
        launches = g.launch_count()
        st = g.stats()
        secs = max_over_ranks(world, secs, f"cuda:{dev}")
        res[name] = dict(secs=secs, launches=launches, stats=st, window=(t0, t1))
    clocks.stop()

    # one step from the same state: the mixed paths against FP64 (the oracle
    # step below is compared with the same results)
    one = {}
    for name, g in handles:
        g.set_coeffs(u0)
        g.step()
        one[name] = g.coeffs()
    a64 = one["fp64"]
    err1 = float(np.linalg.norm(one["mixed"] - a64) / np.linalg.norm(a64))
    err1_fast = float(np.linalg.norm(one["mixed_fast"] - a64) / np.linalg.norm(a64))
    mixed_stats = gmx.stats()
    # side by side from that step: the configured dt is beyond the explicit
    # stability limit, so differences grow by about |1 - dt lambda_max| per step
    diff = DevDiff(torch, N, dev)
    err_steps = [err1]
    for _ in range(4):
        g64.step()
        gmx.step()
        err_steps.append(diff(gmx, g64))

    # end to end through the C-ABI with pinned host buffers
    host_in = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_in[:] = u0
    e2e, e2e_route = {}, {}
    for name, g in handles:
        time_e2e(torch, g, min(W, 2), host_in, host_out)
        barrier(world)
        secs = time_e2e(torch, g, K, host_in, host_out)
        secs = max_over_ranks(world, secs, f"cuda:{dev}")
        e2e[name] = world * N * K / secs
        e2e_route[name] = g.stats()["host_path"]
    # the same steps as three calls with staged copies, for comparison
    gm = dict(handles)["mixed"]
    time_e2e(torch, gm, min(W, 2), host_in, host_out, three_calls=True)
    barrier(world)
    secs = max_over_ranks(world, time_e2e(torch, gm, K, host_in, host_out, three_calls=True), f"cuda:{dev}")
    e2e_three_calls = world * N * K / secs

    # per-kernel CUDA events (a separate pass over the same steps)
    prof = {}
    phases = {}
    for name, g in handles:
        g.set_coeffs(u0)
        phases[name] = {}
        prof[name] = kernel_profile(g, K, phases[name])

    if rank != 0:
        return
    gfa.cleanup()
    aux = None if args.no_aux else aux_runs(args, dev)

    nelem = E ** 3
    fp32_peak = A.fma_peak(False, dev)
    fp64_peak = A.fma_peak(True, dev)
    hbm, hbm_src = hbm_peak()
    peak_src = ("measured on this GPU by ads_fma_peak, live: a grid of 8 CTAs x 256 threads per SM, each thread "
                "running 16 independent FMA chains for 4096 iterations; an FMA counts as 2 flops")

    def roofline_for(pr, kname, steps, real_launches=None):
        tot, cnt = pr[kname]
        # correction sweeps and residuals of refinement rounds after convergence
        # return at once; average over the launches that did work
        n_real = real_launches if real_launches else cnt
        avg = tot / max(n_real, 1) * 1e-3
        traffic = NCU_TRAFFIC.get((kname, f"heat{E}p{p}"))
        if kname.startswith("residual"):
            # three banded mat-vecs (2p+1 FMA each) + r = f - Mu, r^2, f^2 per DOF
            flops = N * (3 * 2 * (2 * p + 1) + 5)
            achieved = flops / avg / 1e12
            return {"kernel": kname, "bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                    "unit": "TFLOP/s", "frac": achieved / fp64_peak, "peak_source": peak_src, "traffic": traffic,
                    "algorithmic_flops_per_launch": flops, "avg_launch_ms": avg * 1e3}
        if kname == "assemble_df":
            # FP32 operations of the double-float algorithm against the FP32
            # pipe's instruction rate (half the FMA flop rate)
            eo = even_odd_fractions(A, E, p)
            ops = df_assembly_ops(p, nelem, eo, fold=True)  # the timed step: kappa = 1, no source
            achieved = ops / avg / 1e12
            peak = fp32_peak / 2
            return {"kernel": kname, "bound": "fp32-pipe", "achieved": achieved, "peak": peak, "unit": "Top/s",
                    "frac": achieved / peak, "peak_source": peak_src + "; peak = FP32 instruction rate = flop rate / 2",
                    "traffic": traffic, "algorithmic_fp32_ops_per_launch": ops,
                    "even_odd_fractions_x_rows_layers": eo,
                    "fp64_equivalent_tflops": algorithmic_assembly_flops(p, nelem) / avg / 1e12,
                    "fp64_pipe_peak_tflops": fp64_peak, "avg_launch_ms": avg * 1e3}
        if kname.startswith("assemble"):
            flops = algorithmic_assembly_flops(p, nelem)
            achieved = flops / avg / 1e12
            peak = fp32_peak if kname.endswith("f32") else fp64_peak
            return {"kernel": kname, "bound": "fp32" if kname.endswith("f32") else "fp64",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "peak_source": peak_src, "traffic": traffic,
                    "algorithmic_flops_per_launch": flops, "avg_launch_ms": avg * 1e3}
        s_in, s_out = 8, 8
        if "f32" in kname:
            # the mixed heat step feeds every sweep FP32 (G and the residuals as
            # scaled floats); the first solve's z sweep writes the FP64 increment,
            # the correction's z sweep its FP32 solution
            s_in = 4
            s_out = 8 if kname == "sweep_z_f32" else 4
        if kname == "resid_update":
            # x1 and r1 (FP32) in, the increment (FP64) read and written
            s_in, s_out = 4 + 4 + 8, 8
        bytes_ = N * (s_in + s_out)
        achieved = bytes_ / avg / 1e9
        return {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": hbm_src, "traffic": traffic,
                "algorithmic_bytes_per_launch": bytes_, "avg_launch_ms": avg * 1e3}

    pm = prof["mixed"]
    ncorr = max(int(mixed_stats["refinements"]), 1)
    nres = max(int(mixed_stats["fp64_residuals"]), 1)

    # launches that did work per step: the first refinement round keeps the
    # plain timer names, later rounds (which return at once after convergence)
    # are timed as *_late; the library counts corrections and FP64 residuals
    def real(k):
        if k.endswith("_corr") or k == "resid_update":
            return K
        if k.endswith("_late") and ("_corr" in k or k.startswith("resid_update")):
            return K * (ncorr - 1)
        if k == "residual_f64":
            return K
        if k == "residual_f64_late":
            return K * (nres - 1)
        return None

    dominant = max(pm, key=lambda k: pm[k][0])
    roof = roofline_for(pm, dominant, K, real(dominant))
    sweeps = {k: roofline_for(pm, k, K, real(k)) for k in pm
              if (k.startswith("sweep") or k.startswith("resid_update")) and pm[k][1] > 0
              and real(k) != 0}
    # launches of later refinement rounds that returned at once (converged)
    late_ms = sum(v[0] for k, v in pm.items() if k.endswith("_late")) / K
    late_n = sum(v[1] for k, v in pm.items() if k.endswith("_late")) // K
    roof_res = roofline_for(pm, "residual_f64", K, real("residual_f64")) if "residual_f64" in pm else None
    p64 = prof["fp64"]
    dom64 = max(p64, key=lambda k: p64[k][0])
    roof64 = roofline_for(p64, dom64, K)
    pf = prof["mixed_fast"]
    roof_fast = roofline_for(pf, "assemble_f32", K) if "assemble_f32" in pf else None

    # CPU baseline: one oracle step at the full size on all host cores, from
    # the same state; its result also checks both GPU paths at full size
    cpu = None
    vs_oracle = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        o = O.Oracle(n, (p, p, p))
        o.set_coeffs(u0)
        t0 = time.perf_counter()
        o.step(O.FORM_HEAT, kappa=1.0, dt=args.dt)
        dt_s = time.perf_counter() - t0
        uo = o.coeffs()
        no = np.linalg.norm(uo)
        vs_oracle = {k: float(np.linalg.norm(one[k] - uo) / no) for k in ("fp64", "mixed", "mixed_fast")}
        cores = O.num_threads()
        cpu = {"value": o.N / dt_s, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"one {E}^3 p={p} heat step of the oracle (C++ restatement of the reference FP64 path), "
                         f"1 rank, OpenMP {cores} threads, {dt_s:.1f} s"}
        o.close()

    secs = res["mixed"]["secs"]
    ck = clocks.summary(*res["mixed"]["window"]) or clocks.summary()
    c3 = (aux or {}).get("c3_heat_256_mixed_vs_fp64", {})
    summary = {
        "fp64_step": {"value": world * N * K / res["fp64"]["secs"], "ms_per_step": 1e3 * res["fp64"]["secs"] / K,
                      "e2e": e2e["fp64"], "gpu_launches": res["fp64"]["launches"]},
        "mixed_over_fp64": res["fp64"]["secs"] / secs,
        "e2e_mixed_over_fp64": e2e["mixed"] / e2e["fp64"],
        "e2e_route": {"call": "ads_step_host(h, u_in, u_out, &l2) with pinned u_in, u_out",
                      "host_path": e2e_route,
                      "mixed_three_calls": {"value": e2e_three_calls, "calls": "ads_set_coeffs + ads_step + "
                                            "ads_get_coeffs (staged copies)"}},
        "mixed_rel_err_vs_fp64": {
            "one_step": err1, "steps_1_to_5_configured_dt": err_steps,
            "stable_dt_100_steps_max": c3.get("p2", {}).get("mixed_rel_err_per_step_stable_dt_max"),
            "stable_dt": STABLE_DT[2]},
        "rel_err_vs_oracle_one_step": vs_oracle,
        "refinement": {"tol": REFINE_TOL, "rel_residual": mixed_stats["rel_residual"],
                       "corrections": mixed_stats["refinements"], "fp64_residuals": mixed_stats["fp64_residuals"],
                       "converged": mixed_stats["converged"]},
        "mixed_fast_step": {"value": world * N * K / res["mixed_fast"]["secs"], "e2e": e2e["mixed_fast"],
                            "one_step_rel_err_vs_fp64": err1_fast},
    }
    if "p3" in c3:
        r3 = c3["p3"]
        summary["p3"] = {k: r3.get(k) for k in ("mixed", "fp64", "mixed_over_fp64",
                                               "mixed_rel_err_first_steps_configured_dt",
                                               "mixed_rel_err_per_step_stable_dt_max")}
    line = {
        "metric": METRIC,
        "value": world * N * K / secs,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": 1e3 * secs / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (double-float assembly) + f64 refinement",
        "data": "synthetic",
        "config": {"workload": f"heat {E}^3 elements p={p} dt={args.dt} kappa=1, mixed precision: increment "
                               f"assembled in double-float arithmetic on the FP32 pipe, FP32 banded sweeps, FP64 "
                               f"residual refinement to {REFINE_TOL:g}; the FP64 drop-in step timed alongside",
                   "elements": E, "degree": p, "dofs": N, "parallelism": f"replicas{world}",
                   "l2_flush": "inputs larger than L2 (FP64 state 137 MB; step working set > 500 MB)",
                   "initial_state": "L2 projection of 16 seeded Gaussian bumps, seed 0",
                   **summary},
        "e2e": {"value": e2e["mixed"], "unit": UNIT, "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N + 8},
        "roofline": roof,
        "roofline_fp64_step": roof64,
        "roofline_mixed_fast_assembly": roof_fast,
        "roofline_sweeps": sweeps,
        "roofline_residual": roof_res,
        "kernel_ms_per_step": {k: v[0] / K for k, v in sorted(pm.items(), key=lambda kv: -kv[1][0])},
        # the *_late timers: launches of refinement rounds 2.. (eager, one event
        # pair each) that returned at once because the first round converged
        "refinement_late_launches": {"launches_per_step": late_n, "ms_per_step": late_ms},
        # the same CUDA-event timings per phase, under the reference's PERFORMANCE names
        "phase_ms_per_step": {name: {k: v[0] / K for k, v in ph.items()} for name, ph in phases.items()},
        "gpu_launches": res["mixed"]["launches"],
        "cpu_baseline": cpu,
        "other_configs": finite_or_none(aux),
        "clocks": ck,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.only:
        run_only(args, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
