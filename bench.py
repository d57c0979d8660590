#!/usr/bin/env python3
"""Benchmark of the explicit ADS heat step on GB300.

Metric: DOF-updates/s per ADS step at 256^3 elements, p = 2,
FP64 vs FP32 + FP64 refinement (each Kronecker solve refined to <= 1e-10
relative residual).  Workload: heat equation, kappa = 1, dt = 1e-5, initial
state = L2 projection of 16 seeded Gaussian bumps (synthetic, seed 0).

`value` is the mixed-precision step with its state resident in HBM, timed with
CUDA events over exactly --steps steps (graph-launched); the FP64 drop-in step
is timed the same way and reported under "fp64".  `e2e` times the same steps
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
    ap.add_argument("--only", choices=["mixed", "fp64"], default=None,
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


def time_e2e(torch, g, K, host_in, host_out):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        g.set_coeffs(host_in)
        g.step()
        g.coeffs_into(host_out)
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def kernel_profile(g, K):
    g.timing(True)
    g.timing_reset()
    g.steps(K)
    t = g.timing_read()
    g.timing(False)
    return t


def run_only(args, local):
    """Minimal case for ncu: one handle of the chosen precision, the seeded
    initial state, --warmup + --steps eager steps, nothing else."""
    import ads_mpi_gb300 as A
    from ads_mpi_gb300 import inputs
    E, p = args.elements, args.degree
    n = (E + p - 1,) * 3
    prec = A.PREC_MIXED if args.only == "mixed" else A.PREC_FP64
    g = A.ADS(n, (p, p, p), precision=prec, device=local)
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


def aux_runs(args, dev):
    """The other configurations of the workload family, measured after the
    headline step (rank 0 only): the FP64 adjoint at 96^3 (50 steps,
    checkpoint every 10, central finite differences h = 1e-6 along 8 seeded
    directions), the variable-conductivity gradient at 128^3 (kappa = exp(g),
    g a seeded Gaussian random field, 100 steps, mixed forward + FP64
    adjoint against an all-FP64 reference gradient), and the mixed step
    against FP64 at 256^3 p = 3 plus the per-step error of the mixed path
    over the first steps at 256^3 p = 2, and the oil problem at 128^3
    (mixed against FP64, with its drained statistic)."""
    import numpy as np
    import torch
    import ads_mpi_gb300 as A
    from ads_mpi_gb300 import inputs
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

    # The configured dt = 1e-5 is beyond the explicit stability limit at these
    # sizes (dt * lambda_max = 5.97 at 96^3 and 10.6 at 128^3 with kappa = 1):
    # the loss then grows by ~|1 - dt lambda_max|^(2K), a finite difference at
    # h = 1e-6 is swamped by the FP64 rounding of the loss, and at 128^3 / 100
    # steps the gradient overflows.  Each check therefore runs at the
    # configured dt and at a stable dt: 1e-6 for the adjoint
    # (dt * lambda_max = 0.60), and for the variable conductivity 1.5 /
    # lambda_max rounded to one digit, lambda_max scaled by the largest kappa.
    def adjoint_check(dtv):
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
        rows = []
        for _ in range(8):
            d = rng.standard_normal(g.N)   # entries N(0, 1), h = 1e-6 per entry
            lp, _, _ = g.heat_adjoint(K, ck, u0 + h * d, u_target, grad=False)
            lm, _, _ = g.heat_adjoint(K, ck, u0 - h * d, u_target, grad=False)
            fd = (lp - lm) / (2 * h)
            ad = float(np.dot(gu, d))
            rows.append(abs(fd - ad) / max(abs(fd), abs(ad), 1e-300))
        g.cleanup()
        return {"dt": dtv, "loss": loss, "forward_backward_s": t_adj, "fd_rel_err_max": max(rows),
                "fd_rel_err": rows}

    out["adjoint_96p2"] = {
        "config": "heat 96^3 p=2 FP64, 50 steps, checkpoint every 10; loss 1/2||u^50 - u_target||_M^2, "
                  "u_target from a seeded forward run of a perturbed initial state; central FD h=1e-6 along "
                  "8 seeded random directions with N(0,1) entries",
        "configured_dt": adjoint_check(dtv), "stable_dt": adjoint_check(1e-6), "target_fd_rel_err": 1e-6}

    # ---- variable conductivity, 128^3 p=2, 100 steps: dL/dg, g -> kappa = exp(g) ----
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

    def kappa_check(dtv):
        K, ck = 100, 10
        g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
        u0 = bumps_state(g64, args.seed)
        g64.set_coeffs(bumps_state(g64, args.seed + 1))
        g64.set_form(A.FORM_HEAT, kappa_qp=kappa, dt=dtv)
        g64.steps(K)
        u_target = g64.coeffs()
        (l64, _, gk64), t64 = sync_time(lambda: g64.heat_adjoint(K, ck, u0, u_target, grad=False, grad_kappa=True))
        gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=1e-10, max_refine=3, device=dev)
        gmx.set_form(A.FORM_HEAT, kappa_qp=kappa, dt=dtv)
        (lmx, _, gkmx), tmx = sync_time(lambda: gmx.heat_adjoint(K, ck, u0, u_target, grad=False, grad_kappa=True))
        dg64 = gk64 * kappa    # dL/dg = dL/dkappa * kappa
        dgmx = gkmx * kappa
        n64 = float(np.linalg.norm(dg64))
        err = float(np.linalg.norm(dgmx - dg64) / n64) if np.isfinite(n64) and n64 > 0 else None
        gmx.cleanup()
        g64.cleanup()
        return {"dt": dtv, "loss_mixed": lmx, "loss_fp64": l64, "dLdg_rel_l2_err_vs_fp64": err,
                "dLdg_norm": n64, "forward_backward_s_mixed": tmx, "forward_backward_s_fp64": t64}

    out["var_kappa_128p2"] = {
        "config": "heat 128^3 p=2, kappa = exp(g), g Gaussian random field sigma 0.5 corr 0.1 at the quadrature "
                  "points, 100 steps, checkpoint every 10; mixed (FP32 + FP64 refinement) forward, FP64 adjoint, "
                  "against an all-FP64 reference gradient",
        "kappa_max": float(kappa.max()), "dt_lambda_max_at_configured_dt": dtv * lam,
        "configured_dt": kappa_check(dtv), "stable_dt": kappa_check(dt_stable)}

    # ---- oil problem (problems/oil/RHS_eq.F90:69-92), 128^3 p=2: mixed vs FP64 ----
    # seeded curves (Kq), pumps and drains; mi = 10; dt at half the explicit
    # limit for the largest Kq exp(mi u) (u stays below 0.1)
    E, p, Ko, mu = 128, 2, 10, 10.0
    n = (E + p - 1,) * 3
    g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=1e-10, max_refine=3, device=dev)
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

    # ---- 256^3 p=3: mixed vs FP64 step time ----
    # initial coefficients: the seeded bumps at the Greville abscissae (a
    # projection would need 64 quadrature values per element on the host)
    E, p, Ks = 256, 3, 5
    n = (E + p - 1,) * 3
    U = A.axis_setup(n[0], p)["U"]
    xi = np.array([U[i + 1:i + p + 1].mean() for i in range(n[0] + 1)])
    rng = np.random.default_rng(args.seed)
    amp = rng.uniform(0.0, 1.0, 16)
    cen = rng.uniform(0.2, 0.8, (16, 3))
    u0 = np.zeros((n[0] + 1,) * 3)
    for b in range(16):
        gx, gy, gz = (np.exp(-(xi - cen[b, d]) ** 2 / (2 * 0.05 ** 2)) for d in range(3))
        u0 += amp[b] * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    u0 = u0.ravel()
    g64 = A.ADS(n, (p, p, p), precision=A.PREC_FP64, device=dev)
    g64.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
    gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=1e-10, max_refine=3, device=dev)
    gmx.set_form(A.FORM_HEAT, kappa=1.0, dt=dtv)
    row = {}
    for name, gg in (("mixed", gmx), ("fp64", g64)):
        gg.set_coeffs(u0)
        gg.steps(2)
        secs = time_device_steps(torch, gg, Ks)
        row[name] = g64.N * Ks / secs
    g64.set_coeffs(u0)
    gmx.set_coeffs(u0)
    g64.step()
    gmx.step()
    a64 = g64.coeffs()
    row["mixed_rel_err_vs_fp64_one_step"] = float(np.linalg.norm(gmx.coeffs() - a64) / np.linalg.norm(a64))
    row["mixed_rel_residual"] = gmx.stats()["rel_residual"]
    out["heat_256p3"] = {"unit": UNIT, "steps": Ks, **row, "mixed_over_fp64": row["mixed"] / row["fp64"]}
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

    gmx = A.ADS(n, (p, p, p), precision=A.PREC_MIXED, refine_tol=1e-10, max_refine=3, device=dev)
    gmx.set_form(A.FORM_HEAT, kappa=1.0, dt=args.dt)

    clocks = ClockSampler(dev)
    clocks.start()
    res = {}
    for name, g in (("mixed", gmx), ("fp64", g64)):
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

    # error of the mixed step against the FP64 step, one step from the same state
    g64.set_coeffs(u0)
    gmx.set_coeffs(u0)
    g64.step()
    gmx.step()
    a64 = g64.coeffs()
    amx = gmx.coeffs()
    err1 = float(np.linalg.norm(amx - a64) / np.linalg.norm(a64))
    mixed_stats = gmx.stats()
    # the two paths stepped side by side: relative error per step (the
    # configured dt is beyond the explicit stability limit, so differences
    # grow by about |1 - dt lambda_max| per step)
    err_steps = [err1]
    for _ in range(4):
        g64.step()
        gmx.step()
        a64 = g64.coeffs()
        err_steps.append(float(np.linalg.norm(gmx.coeffs() - a64) / np.linalg.norm(a64)))

    # end to end through the C-ABI with pinned host buffers
    host_in = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_in[:] = u0
    e2e = {}
    for name, g in (("mixed", gmx), ("fp64", g64)):
        time_e2e(torch, g, min(W, 2), host_in, host_out)
        barrier(world)
        secs = time_e2e(torch, g, K, host_in, host_out)
        secs = max_over_ranks(world, secs, f"cuda:{dev}")
        e2e[name] = world * N * K / secs

    # per-kernel CUDA events (a separate pass over the same steps)
    prof = {}
    for name, g in (("mixed", gmx), ("fp64", g64)):
        g.set_coeffs(u0)
        prof[name] = kernel_profile(g, K)

    if rank != 0:
        return
    aux = None if args.no_aux else aux_runs(args, dev)

    nelem = E ** 3
    fp32_peak = A.fma_peak(False, dev)
    fp64_peak = A.fma_peak(True, dev)
    hbm, hbm_src = hbm_peak()

    def roofline_for(pr, kname, steps, real_launches=None):
        tot, cnt = pr[kname]
        # correction sweeps and residuals of refinement rounds after convergence
        # return at once; average over the launches that did work
        n_real = real_launches if real_launches else cnt
        avg = tot / max(n_real, 1) * 1e-3
        if kname.startswith("residual"):
            # three banded mat-vecs (2p+1 FMA each) + r = f - Mu, r^2, f^2 per DOF
            flops = N * (3 * 2 * (2 * p + 1) + 5)
            achieved = flops / avg / 1e12
            return {"kernel": kname, "bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                    "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                    "peak_source": "measured FMA-pipe throughput on this GPU (ads_fma_peak), live",
                    "traffic": NCU_TRAFFIC.get((kname, f"heat{E}p{p}")),
                    "algorithmic_flops_per_launch": flops, "avg_launch_ms": avg * 1e3}
        if kname.startswith("assemble"):
            flops = algorithmic_assembly_flops(p, nelem)
            achieved = flops / avg / 1e12
            peak = fp32_peak if kname.endswith("f32") else fp64_peak
            return {"kernel": kname, "bound": "fp32" if kname.endswith("f32") else "fp64",
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "peak_source": "measured FMA-pipe throughput on this GPU (ads_fma_peak), live",
                    "traffic": NCU_TRAFFIC.get((kname, f"heat{E}p{p}")),
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
                "frac": achieved / hbm, "peak_source": hbm_src, "traffic": NCU_TRAFFIC.get((kname, f"heat{E}p{p}")),
                "algorithmic_bytes_per_launch": bytes_, "avg_launch_ms": avg * 1e3}

    pm = prof["mixed"]
    ncorr = max(int(mixed_stats["refinements"]), 1)

    def real(k):
        # one FP64 residual per correction: the certified bound of the updated
        # residual (resid_update) ends the refinement
        if k.endswith("_corr") or k.startswith("residual") or k == "resid_update":
            return K * ncorr
        return None

    dominant = max(pm, key=lambda k: pm[k][0])
    roof = roofline_for(pm, dominant, K, real(dominant))
    sweeps = {k: roofline_for(pm, k, K, real(k)) for k in pm
              if (k.startswith("sweep") or k == "resid_update") and pm[k][1] > 0}
    roof_res = roofline_for(pm, "residual_f64", K, real("residual_f64")) if "residual_f64" in pm else None
    p64 = prof["fp64"]
    dom64 = max(p64, key=lambda k: p64[k][0])
    roof64 = roofline_for(p64, dom64, K)

    # CPU baseline: one oracle step at the full size on all host cores
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        o = O.Oracle(n, (p, p, p))
        o.set_coeffs(u0)
        t0 = time.perf_counter()
        o.step(O.FORM_HEAT, kappa=1.0, dt=args.dt)
        dt_s = time.perf_counter() - t0
        cores = O.num_threads()
        cpu = {"value": o.N / dt_s, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"one {E}^3 p={p} heat step of the oracle (C++ restatement of the reference FP64 path), "
                         f"1 rank, OpenMP {cores} threads, {dt_s:.1f} s"}
        o.close()

    secs = res["mixed"]["secs"]
    ck = clocks.summary(*res["mixed"]["window"]) or clocks.summary()
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
        "dtype": "f32+f64-refine",
        "data": "synthetic",
        "config": {"workload": f"heat {E}^3 elements p={p} dt={args.dt} kappa=1, mixed precision "
                               f"(FP32 assembly and sweeps, FP64 residual refinement to 1e-10)",
                   "elements": E, "degree": p, "dofs": N, "parallelism": f"replicas{world}",
                   "l2_flush": "inputs larger than L2 (FP64 state 137 MB; step working set > 500 MB)",
                   "initial_state": "L2 projection of 16 seeded Gaussian bumps, seed 0"},
        "fp64": {"value": world * N * K / res["fp64"]["secs"], "unit": UNIT,
                 "ms_per_step": 1e3 * res["fp64"]["secs"] / K, "e2e": e2e["fp64"], "roofline": roof64,
                 "gpu_launches": res["fp64"]["launches"]},
        "mixed_over_fp64": res["fp64"]["secs"] / secs,
        "mixed_rel_err_vs_fp64_one_step": err1,
        "mixed_rel_err_vs_fp64_per_step": err_steps,
        "mixed_refinement": {"rel_residual": mixed_stats["rel_residual"], "corrections": mixed_stats["refinements"],
                             "converged": mixed_stats["converged"], "tol": 1e-10},
        "e2e": {"value": e2e["mixed"], "unit": UNIT, "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * N + 8},
        "roofline": roof,
        "roofline_sweeps": sweeps,
        "roofline_residual": roof_res,
        "kernel_ms_per_step": {k: v[0] / K for k, v in sorted(pm.items(), key=lambda kv: -kv[1][0])},
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
