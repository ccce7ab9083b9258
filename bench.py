"""Benchmark: SIMP cantilever design evaluations on one GB300.

Workload: HEX8 SIMP cantilever 128x64x64 (524,288 elements, 1,635,075 dofs),
densities iid U[0.01, 1] (numpy default_rng(0), element order x-fastest),
E0 = 1, Emin = 1e-9, nu = 0.3, p = 3, x = 0 face clamped, unit -z load spread
over the 65 nodes of the x = max, z = 0 edge.  One step = one design
evaluation: solve to 1e-8 relative FP64 residual ||f - K u|| / ||f||, then the
compliance f.u and dC/drho for all elements.

value  -- solves/s of the mixed-precision form (tcgen05 split-TF32 matrix-free
          operator, FP32 CG preconditioned by a geometric multigrid V-cycle whose
          smoothers use the same tensor-core operator, FP64 refinement), inputs
          resident in HBM, L2 flushed between steps.
e2e    -- the same through the C ABI with host buffers: densities and initial
          guess copied in, solution and sensitivities copied out, every step.
plain_fp64 -- the FP64 CSR Jacobi-PCG form on the same GPU (the 5x target's base).
cpu_baseline -- the FP64 CPU restatement (oracle: assembly + Jacobi-PCG to 1e-8, all
          host threads), one full solve timed; beside it a one-core figure (assembly
          and a bounded number of PCG iterations on one thread, scaled to the full
          iteration count, labelled as such).

--impl reference runs that CPU implementation alone (the reference arm): every timed
step is one full oracle solve of the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "mast-multiphysics_gb300"))

NX, NY, NZ, SEED = 128, 64, 64, 0
WORKLOAD = "simp_cantilever_hex8_128x64x64"
METRIC = "solves/s @1e-8 FP64 residual (SIMP cantilever design evaluation)"
GOLDEN = os.path.join(REPO, "tests", "golden", "simp_128x64x64_seed0.npz")


def bench_config(world):
    """The workload description both arms print under "config" (identical keys and
    values, so the two lines describe the same job)."""
    return {"workload": WORKLOAD, "n_dofs": 1635075, "n_elems": 524288, "rtol": 1e-8,
            "load": "unit -z over the 65 nodes of the x = max, z = 0 edge; x = 0 clamped",
            "l2": "GPU arm: flushed between timed steps (512 MB write)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="tf32x3", choices=["tf32", "bf16", "bf16x3", "tf32x3"])
    ap.add_argument("--preconditioner", default="multigrid", choices=["multigrid", "jacobi"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-design batch section")
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop section")
    ap.add_argument("--no-small", action="store_true", help="skip the 24x12x12 and heat-conduction lines")
    ap.add_argument("--no-bf16", action="store_true", help="skip the split-BF16 line")
    ap.add_argument("--ks-stress", action="store_true",
                    help="only time the KS-aggregated von Mises stress output (value; value and "
                         "adjoint density sensitivity) on a 64x32x32 cantilever and print one JSON line")
    ap.add_argument("--opt", action="append", default=[],
                    help="mg_solve_opts field=value for the solve (with --no-autotune: a fixed schedule)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="solve the headline problem with the default schedule instead of the autotuned one")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="requests per arrival rate of the sweep")
    ap.add_argument("--serve-full", type=int, default=10000,
                    help="requests of the full-length stream (at the sweep's highest rate; 0: skip)")
    ap.add_argument("--kernel-only", default=None, choices=["mixed", "plain", "factored"],
                    help="only launch one kernel (tensor-core column operator, FP64 CG SpMV or the "
                         "factored multigrid level operator) --steps times after --warmup "
                         "launches; for profilers")
    ap.add_argument("--nonlinear-assembly", action="store_true",
                    help="only time the Green-Lagrange HEX8 residual + tangent assembly "
                         "(64x32x32 cantilever) and print one JSON line")
    return ap.parse_args()


def nonlinear_assembly(args, M):
    """Time the nonlinear-strain HEX8 assembly (residual and tangent of every colour,
    scattered into the CSR) on a 64x32x32 cantilever at a random 1e-3-strain state.
    FP64 operations per element, from the per-pair formulation of the element:
    tangent blocks 64 pairs x 8 points x 82 = 41,984; Jacobians, gradients, stresses,
    projections and forces about 10,000: about 52,000 in all.  Bytes per element: the 576-entry tangent scattered as
    read-modify-write (9,216 B), 24 residual entries (384 B), coordinates, state,
    connectivity and modulus (424 B)."""
    import torch
    nx, ny, nz = 64, 32, 32
    prob = M.simp_cantilever(nx, ny, nz, physics=M.PHYS_HEX8_NONLINEAR, load=0.01)
    rng = np.random.default_rng(SEED)
    prob.set_design(rng.uniform(0.3, 1.0, nx * ny * nz))
    X = np.ascontiguousarray(rng.normal(scale=1e-3, size=prob.n_dofs))
    stream = torch.cuda.ExternalStream(prob.stream)
    L = M.lib()
    M.check(L.mg_debug_launch_assembly(prob.h, M._p(X), max(3, args.warmup)), "warm")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = max(1, args.steps)
    e0.record(stream)
    M.check(L.mg_debug_launch_assembly(prob.h, None, reps), "assembly")
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    n_el = nx * ny * nz
    flops = 52000.0 * n_el
    bytes_ = (9216 + 384 + 424) * n_el
    pk = peaks()
    print(json.dumps({
        "metric": "nonlinear_hex8_assembly", "workload": "Green-Lagrange HEX8 residual + tangent, "
        "cantilever 64x32x32 (%d elements, %d colours)" % (n_el, prob.n_colors),
        "ms_per_assembly": ms, "elements_per_s": n_el / (ms * 1e-3),
        "fp64_gflops": flops / (ms * 1e-3) / 1e9, "fp64_peak_nominal_gflops": 1250.0,
        "fp64_frac_of_nominal": flops / (ms * 1e-3) / 1e9 / 1250.0,
        "GBps": bytes_ / (ms * 1e-3) / 1e9, "hbm_frac": bytes_ / (ms * 1e-3) / 1e9 / pk.get("hbm_gbs", 6800.0),
        "reps": reps, "dtype": "f64"}))
    prob.close()


def ks_stress_timing(args, M):
    """Time mg_ks_stress on a 64x32x32 cantilever (65,536 elements) at its solved state:
    the value pass (Gauss-point stresses of every element, the KS and max reductions) and
    the value with the total density sensitivity (value pass, gradient scatter, adjoint
    CG solve of the plain FP64 form, element sensitivities).  Wall-clock per call through
    the ABI (each call synchronises)."""
    nx, ny, nz = 64, 32, 32
    prob = M.simp_cantilever(nx, ny, nz)
    rho = np.random.default_rng(SEED).uniform(0.3, 1.0, nx * ny * nz)
    prob.set_design(rho)
    u, rep = prob.solve(M.default_opts(rtol=1e-10))
    for _ in range(max(1, args.warmup)):
        prob.ks_stress(8.0, 1.0, 3.0, want_sens=True)
    reps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(reps):
        q, vmax, _ = prob.ks_stress(8.0, 1.0, 3.0, want_sens=False)
    t_val = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        prob.ks_stress(8.0, 1.0, 3.0, want_sens=True)
    t_sens = (time.perf_counter() - t0) / reps
    n_el = nx * ny * nz
    print(json.dumps({
        "metric": "ks_stress_output", "workload": "KS-aggregated von Mises stress, p = 8, SIMP "
        "cantilever 64x32x32 (%d elements), FP64" % n_el,
        "ms_per_value": t_val * 1e3, "ms_per_value_and_sensitivity": t_sens * 1e3,
        "elements_per_s_value": n_el / t_val, "adjoint_cg_iterations_of_the_solve": rep.krylov_iterations,
        "ks": q, "max_von_mises": vmax, "reps": reps, "dtype": "f64"}))
    prob.close()


PROFILE = os.path.join(REPO, "profiles", "mf_col_kernel_tf32x3_128x64x64.txt")


def profiled_traffic():
    """DRAM bytes per launch of the column operator from the committed ncu
    summary (line 'dram_bytes_per_launch = N'), or None."""
    try:
        for line in open(PROFILE):
            if line.strip().startswith("dram_bytes_per_launch"):
                return int(line.split("=")[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def kernel_only(args, M, prob, prec, rho):
    """Launch only the dominant kernel (no solve) so that a profiler sees a
    short, regular launch list: setup, then --warmup + --steps launches."""
    import torch
    prob.set_design(rho)  # the plain launch hook assembles the CSR on first use
    p = {"plain": M.PLAIN_FP64, "factored": M.OPERATOR_FACTORED_FP32}.get(args.kernel_only, prec)
    M.check(M.lib().mg_debug_launch_apply(prob.h, p, max(1, args.warmup)), "warm")
    torch.cuda.synchronize()
    M.check(M.lib().mg_debug_launch_apply(prob.h, p, max(1, args.steps)), "launch")
    torch.cuda.synchronize()
    print(json.dumps({"kernel_only": args.kernel_only, "launches": args.warmup + args.steps}))


def plain_time_per_size(M, sizes, rtol=1e-8):
    """Seconds of one plain FP64 CSR Jacobi-PCG solve (one load case over the full
    x = max, z = 0 edge, densities U[0.01,1]) per grid size, on this GPU."""
    out = {}
    for (nx, ny, nz) in sizes:
        rho = np.random.default_rng(1).uniform(0.01, 1.0, nx * ny * nz)
        with M.simp_cantilever(nx, ny, nz) as p:
            p.set_design(rho)
            o = M.default_opts(precision=M.PLAIN_FP64, rtol=rtol, timeout_s=600.0)
            p.solve(o)  # assembly, graph capture
            t0 = time.perf_counter()
            p.solve(o)
            p.compliance()
            out[(nx, ny, nz)] = time.perf_counter() - t0
    return out


def bench_small_configs(M, with_cpu=True):
    """Configs 0 and 1 through the plain FP64 form (GPU), beside the oracle on the
    host cores: config 0 = 24x12x12 HEX8 cantilever, rho = 0.5, Jacobi-PCG to 1e-10,
    compliance and dC/drho; config 1 = QUAD4 200x200 k(T) conduction, Newton with
    Jacobi-PCG to 1e-10, mean temperature and its adjoint sensitivities."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    out = {}
    rho = np.full(24 * 12 * 12, 0.5)
    with M.simp_cantilever(24, 12, 12) as p:
        o = M.default_opts(precision=M.PLAIN_FP64, rtol=1e-10)
        p.set_design(rho)
        p.solve(o)
        p.compliance()
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            p.set_design(rho)
            u, rep = p.solve(o)
            c, dc = p.compliance()
            ts.append(time.perf_counter() - t0)
    g = {"gpu_ms_per_solve": 1e3 * min(ts), "iterations": rep.krylov_iterations, "relres": rep.relres,
         "compliance": c}
    if with_cpu:
        t0 = time.perf_counter()
        _, dc_ref, r = O.simp_solve(O.simp_desc(24, 12, 12, rtol=1e-10), rho)
        g["cpu_ms_per_solve"] = 1e3 * (time.perf_counter() - t0)
        g["cpu_threads"] = O.max_threads()
        g["compliance_rel_err_vs_oracle"] = abs(c - r.compliance) / r.compliance
        g["sens_rel_err_vs_oracle"] = float(np.abs(dc - dc_ref).max() / np.abs(dc_ref).max())
    out["config0_hex8_24x12x12"] = g
    with M.heat_square() as p:
        o = M.default_opts(precision=M.PLAIN_FP64, rtol=1e-10, newton_rtol=1e-10, krylov=M.KRYLOV_CG)
        oa = M.default_opts(precision=M.PLAIN_FP64, rtol=1e-10, krylov=M.KRYLOV_BICGSTAB)  # adjoint
        p.solve(o, X=np.zeros(p.n_dofs))
        p.mean_temperature(opts=oa)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            T, rep = p.solve(o, X=np.zeros(p.n_dofs))
            q, dk0, ds = p.mean_temperature(opts=oa)
            ts.append(time.perf_counter() - t0)
    h = {"gpu_ms_per_solve": 1e3 * min(ts), "newton_iterations": rep.newton_iterations,
         "krylov_iterations": rep.krylov_iterations, "mean_temperature": q}
    if with_cpu:
        t0 = time.perf_counter()
        _, ds_ref, r = O.heat_solve(O.heat_desc(krylov=0), q_elem=O.heat_source_field(200, 200))
        h["cpu_ms_per_solve"] = 1e3 * (time.perf_counter() - t0)
        h["mean_temperature_rel_err_vs_oracle"] = abs(q - r.mean_temperature) / abs(r.mean_temperature)
        h["dq_dk0_rel_err_vs_oracle"] = abs(dk0 - r.dq_dk0) / abs(r.dq_dk0)
        h["dq_ds_rel_err_vs_oracle"] = float(np.abs(ds - ds_ref).max() / np.abs(ds_ref).max())
    out["config1_quad4_heat_200x200"] = h
    return out


def bench_batch(M, n_designs=256, seed=0):
    """Batched design evaluations: n_designs SIMP cantilevers of mixed sizes with
    1-4 load cases each, all solved together (mixed form, autotuned schedule)."""
    designs = M.batch_designs(n_designs, seed=seed)
    b = M.Batch(designs)
    o = M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=600.0)
    t0 = time.perf_counter()
    o, trial_s = b.autotune(o, max_trials=12)
    tune_s = time.perf_counter() - t0
    b.solve(o)  # warm-up: graph capture
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        rc, reps = b.solve(o)
        times.append(time.perf_counter() - t0)
    t = min(times)
    relres = max(r.relres for r in reps)
    # oracle checks outside the timed solves: the first design of every grid size (its
    # first load case) and every load case of the first multi-case design of the two
    # smallest sizes, each against an FP64 oracle solve to 1e-10 with sensitivities
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    picks = {}
    for d, x in enumerate(designs):
        key = (x["nx"], x["ny"], x["nz"])
        if key not in picks:
            picks[key] = (d, [0])
    multi = next(d for d, x in enumerate(designs)
                 if len(x["spans"]) > 1 and (x["nx"], x["ny"], x["nz"]) in M.BATCH_SIZES[:2])
    checks = list(picks.values()) + [(multi, list(range(len(designs[multi]["spans"]))))]
    ce, se, checked = 0.0, 0.0, []
    t_or = time.perf_counter()
    for d, cases in checks:
        x = designs[d]
        comp, dc, _ = b.results(d)
        for k in cases:
            j0, j1 = x["spans"][k]
            _, dc_ref, r = O.simp_solve(O.simp_desc(x["nx"], x["ny"], x["nz"], load_y0=j0, load_y1=j1,
                                                    rtol=1e-10, maxit=10 ** 6), x["rho"])
            ce = max(ce, abs(comp[k] - r.compliance) / abs(r.compliance))
            se = max(se, float(np.abs(dc[k] - dc_ref).max() / np.abs(dc_ref).max()))
            checked.append("design %d case %d (%dx%dx%d)" % (d, k, x["nx"], x["ny"], x["nz"]))
    oracle_check = {"checked": checked, "compliance_rel_err_max": ce, "sens_rel_err_max": se,
                    "oracle": "FP64 Jacobi-PCG to 1e-10, all host threads", "seconds": time.perf_counter() - t_or}
    # plain FP64 estimate: one solve per problem at that problem's size
    sizes = sorted({(d["nx"], d["ny"], d["nz"]) for d in designs})
    tp = plain_time_per_size(M, sizes)
    t_plain = sum(tp[(d["nx"], d["ny"], d["nz"])] * len(d["spans"]) for d in designs)
    res = {"workload": "simp_batch_%d_designs_mixed_sizes" % n_designs,
           "n_designs": b.n_designs, "n_problems": b.n_problems, "n_dofs": b.n_dofs,
           "seconds": t, "solves_per_s": b.n_problems / t, "designs_per_s": b.n_designs / t,
           "dofs_per_s": b.n_dofs / t, "max_relres_fp64": relres,
           "all_converged": all(r.status == 0 for r in reps),
           "autotuned": {"precision": o.precision, "smooth_degree": o.smooth_degree,
                         "coarse_degree": o.coarse_degree, "graph_chunk": o.graph_chunk,
                         "vec_blocks_per_sm": o.vec_blocks_per_sm, "inner_rtol": o.inner_rtol,
                         "tuning_seconds": tune_s},
           "oracle_check": oracle_check,
           "plain_fp64_est_solves_per_s": b.n_problems / t_plain,
           "plain_fp64_method": "one timed plain solve per grid size x the batch's load cases",
           "speedup_vs_plain_fp64": t_plain / t}
    b.close()
    return res


def bench_serve(M, rates, n_requests, big=True, seed=0, n_check=6):
    """Request loop: Poisson streams over 64 design chains (config-4 mix).  After each
    stream, the first n_check completed requests on grids up to 48x24x24 are checked
    against the FP64 oracle (every load case: compliance)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    o = M.default_opts(precision=M.MIXED_TF32X3, rtol=1e-8, inner_rtol=1e-3, timeout_s=600.0)
    sweep = []
    for rate, n in zip(rates, n_requests):
        kw = dict(n_chains=64, big_fraction=0.02 if big else 0.0, seed=seed)
        with M.Server(o, hbm_cap_bytes=150 << 30) as s:
            st, comp = s.run_synthetic(n, rate=rate, **kw)
        desc = M.synthetic_desc(n, rate, **kw)
        err, checked, i = 0.0, 0, 0
        while checked < n_check and i < n:
            r = M.synthetic_request(desc, i, want_rho=False)
            if r["grid"][0] <= 48:
                r = M.synthetic_request(desc, i)
                nx, ny, nz = r["grid"]
                for k, (j0, j1) in enumerate(r["spans"]):
                    _, _, ref = O.simp_solve(O.simp_desc(nx, ny, nz, load_y0=j0, load_y1=j1, rtol=1e-10,
                                                         maxit=10 ** 6), r["rho"], want_sens=False)
                    err = max(err, abs(comp[i, k] - ref.compliance) / abs(ref.compliance))
                checked += 1
            i += 1
        sweep.append({"rate_req_per_s": rate, "n_requests": n, "completed": st["completed"],
                      "failed": st["failed"], "p50_ms": st["p50_s"] * 1e3, "p99_ms": st["p99_s"] * 1e3,
                      "mean_ms": st["mean_s"] * 1e3, "requests_per_s": st["solves_per_s"],
                      "dofs_per_s": st["dofs_per_s"], "peak_inflight": st["peak_inflight"],
                      "rebuilds": st["rebuilds"], "peak_resident_GB": st["peak_resident_bytes"] / 1e9,
                      "oracle_checked_requests": checked, "compliance_rel_err_vs_oracle": err})
    return {"workload": "simp_serving_64_chains_poisson", "hbm_cap_GB": 150, "sweep": sweep}


def replicas_throughput(ms_local, world, device=None):
    """Whole-job throughput of `world` independent replicas that each time one solve
    per step: the slowest rank's mean step time (max over ranks through the process
    group: CPU tensors under gloo, CUDA tensors under NCCL) and world solves per that
    time.  Every rank must call it (it is a collective when world > 1)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * 1e3 / ms


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "mastgpu_clocks_%d.csv" % os.getpid())
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            # start timing only once the sampler is producing lines
            t0 = time.time()
            while time.time() - t0 < 3.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_full_solve(O, rho):
    """One full oracle solve of the 128x64x64 problem to 1e-8 (FP64 assembly +
    Jacobi-PCG on all host threads), timed; returns (seconds, report)."""
    d = O.simp_desc(NX, NY, NZ, rtol=1e-8, maxit=10 ** 6)
    t0 = time.time()
    _, _, rep = O.simp_solve(d, rho, want_sens=False)
    return time.time() - t0, rep


def cpu_baseline(one_core_iters=20):
    """The CPU baseline on this host: one full oracle solve on all host threads
    (measured), and the one-core figure: assembly + `one_core_iters` PCG iterations on
    one thread, scaled to the full solve's iteration count (an extrapolation, stated)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    rho = np.random.default_rng(SEED).uniform(0.01, 1.0, NX * NY * NZ)
    cores = O.max_threads()
    secs, rep = cpu_full_solve(O, rho)
    O.set_threads(1)
    try:
        d1 = O.simp_desc(NX, NY, NZ, rtol=1e-8, maxit=one_core_iters)
        t0 = time.time()
        _, _, r1 = O.simp_solve(d1, rho, want_sens=False)
        wall1 = time.time() - t0
    finally:
        O.set_threads(cores)
    t1 = r1.t_assemble + rep.iterations * r1.t_solve / max(r1.iterations, 1)
    return {"value": 1.0 / secs, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "one full solve of the 128x64x64 problem to 1e-8 (FP64 assembly + %d "
                      "Jacobi-PCG iterations, %.1f s, relres %.2e), measured"
                      % (rep.iterations, secs, rep.relres),
            "seconds_per_solve": secs, "iterations": rep.iterations,
            "one_core": {"solves_per_s": 1.0 / t1, "seconds_per_solve": t1, "cores": 1,
                         "method": "extrapolated: assembly %.2f s + %d iterations x %.1f ms "
                                   "(%d iterations timed on one thread, %.1f s)"
                                   % (r1.t_assemble, rep.iterations,
                                      1e3 * r1.t_solve / max(r1.iterations, 1), r1.iterations,
                                      wall1)}}


def run_reference(args):
    """The reference arm: the FP64 CPU restatement on all host threads, each timed step
    one full solve to 1e-8 of the same workload (warm-up steps: assembly plus a few PCG
    iterations, which only page the oracle in and start its threads)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    rho = np.random.default_rng(SEED).uniform(0.01, 1.0, NX * NY * NZ)
    for _ in range(args.warmup):
        O.simp_solve(O.simp_desc(NX, NY, NZ, rtol=1e-8, maxit=5), rho, want_sens=False)
    secs = []
    t0 = time.time()
    for _ in range(args.steps):
        t, rep = cpu_full_solve(O, rho)
        secs.append(t)
    wall = time.time() - t0
    ms = 1e3 * sum(secs) / len(secs)
    v = 1e3 / ms
    cb = {"value": v, "unit": "solves/s", "cores": O.max_threads(), "kind": "port",
          "sample": "every step one full solve of the 128x64x64 problem to 1e-8 (FP64 assembly "
                    "+ %d Jacobi-PCG iterations, relres %.2e), measured; warm-up steps: assembly "
                    "+ 5 iterations" % (rep.iterations, rep.relres)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (CPU restatement: CSR assembly + Jacobi-PCG)",
            "data": "synthetic (seeded U[0.01,1] densities, default_rng(0))",
            "config": bench_config(world), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "step_s": [round(x, 3) for x in secs], "wall_s": wall}
    print(json.dumps(line), flush=True)


def tune_schedule(M, opts, rho):
    """The solver schedule (smoother and coarse degrees, smoother operator, CG
    steps per graph, vector-kernel CTAs, inner tolerance) that the library's
    autotuner picks for this grid: a one-design batch of the same cantilever,
    tuned once before the timed region."""
    b = M.Batch([dict(nx=NX, ny=NY, nz=NZ, rho=rho, spans=[(0, NY)])])
    t0 = time.perf_counter()
    o, _ = b.autotune(opts, max_trials=14)
    secs = time.perf_counter() - t0
    b.close()
    sched = {"smooth_degree": o.smooth_degree, "coarse_degree": o.coarse_degree,
             "smoother_operator": "factored" if o.smoother_operator == M.SMOOTHER_FACTORED else "tensor",
             "graph_chunk": o.graph_chunk, "vec_blocks_per_sm": o.vec_blocks_per_sm,
             "inner_rtol": o.inner_rtol, "precision": o.precision, "tuning_seconds": secs}
    return o, sched


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import mastgpu as M

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    prec = {"tf32": M.MIXED_TF32, "bf16": M.MIXED_BF16,
            "bf16x3": M.MIXED_BF16X3,
            "tf32x3": M.MIXED_TF32X3}[args.precision]
    rho = np.random.default_rng(SEED).uniform(0.01, 1.0, NX * NY * NZ)
    prob = M.simp_cantilever(NX, NY, NZ)
    stream = torch.cuda.ExternalStream(prob.stream)
    d_rho = torch.from_numpy(rho).to(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 512 MB > L2
    pc = M.PC_MULTIGRID if args.preconditioner == "multigrid" else M.PC_JACOBI
    opts = M.default_opts(precision=prec, rtol=1e-8, inner_rtol=1e-3, timeout_s=600.0,
                          preconditioner=pc)
    for kv in args.opt:
        k, v = kv.split("=")
        setattr(opts, k, type(getattr(opts, k))(float(v)) if isinstance(getattr(opts, k), float) else int(v))
    if args.kernel_only:
        kernel_only(args, M, prob, prec, rho)
        prob.close()
        return
    if args.nonlinear_assembly:
        prob.close()
        nonlinear_assembly(args, M)
        return
    if args.ks_stress:
        prob.close()
        ks_stress_timing(args, M)
        return
    def step_resident(o=None):
        prob.set_design_device(d_rho.data_ptr())
        rc, rep = prob.solve_resident(opts if o is None else o)
        M.check(rc, "mg_solve")
        c = ctypes.c_double()
        M.check(M.lib().mg_compliance_resident(prob.h, ctypes.byref(c)), "mg_compliance_resident")
        return rep, c.value

    schedule = {"autotuned": False}
    if not args.no_autotune:
        default = M.default_opts(precision=prec, rtol=1e-8, inner_rtol=1e-3, timeout_s=600.0, preconditioner=pc)
        tuned, schedule = tune_schedule(M, opts, rho)
        schedule["autotuned"] = True
        # the tuner times one-design batch solves; confirm its pick on this path
        # (resident solve + compliance, CUDA events) against the default schedule
        best = None
        for name, o in (("tuned", tuned), ("default", default)):
            step_resident(o)  # graph capture
            t = []
            for _ in range(2):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                a0 = torch.cuda.Event(enable_timing=True)
                a1 = torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                step_resident(o)
                a1.record(stream)
                torch.cuda.synchronize()
                t.append(a0.elapsed_time(a1))
            schedule["confirm_ms_" + name] = min(t)
            if best is None or min(t) < best[0]:
                best = (min(t), name, o)
        schedule["used"] = best[1]
        opts = best[2]

    # ---------------- value: resident inputs, per-step CUDA events on the library stream
    for _ in range(args.warmup):
        step_resident()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(local)
    # one more untimed step once the sampler runs: the GPU idled while nvidia-smi
    # started, and its first queries land here rather than in a timed step
    step_resident()
    torch.cuda.synchronize()
    launches0 = M.lib().mg_launch_count()
    ev = []
    reps = []
    torch.cuda.synchronize()
    t_wall0 = time.time()
    for _ in range(args.steps):
        flush.fill_(1.0)  # evict L2 between steps (outside the events)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rep, comp = step_resident()
        e1.record(stream)
        ev.append((e0, e1))
        reps.append((rep.krylov_iterations, rep.refinements, rep.relres, comp))
    torch.cuda.synchronize()
    t_wall = time.time() - t_wall0
    launches = M.lib().mg_launch_count() - launches0
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    ms_step, value = replicas_throughput(sum(ms) / len(ms), world, dev)

    g = np.load(GOLDEN)
    comp_err = abs(reps[-1][3] - float(g["compliance"])) / float(g["compliance"])
    # ---------------- e2e: pinned host buffers through the C ABI, every step:
    # densities in (mg_set_design), a cold solve (mg_solve without an initial
    # guess), the solution, compliance and dC/drho out
    rho_h = torch.from_numpy(rho).pin_memory()
    X_h = torch.empty(prob.n_dofs, dtype=torch.float64).pin_memory()
    dc_h = torch.empty(NX * NY * NZ, dtype=torch.float64).pin_memory()
    L = M.lib()
    e2e_ms = []
    for i in range(0 if args.no_e2e else max(1, args.steps)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        M.check(L.mg_set_design(prob.h, ctypes.c_void_p(rho_h.data_ptr())), "mg_set_design")
        rep = M.SolveReport()
        M.check(L.mg_solve(prob.h, ctypes.byref(opts), None, ctypes.byref(rep)), "mg_solve")
        M.check(L.mg_get_solution(prob.h, ctypes.c_void_p(X_h.data_ptr())), "mg_get_solution")
        cc_ = ctypes.c_double()
        M.check(L.mg_compliance(prob.h, None, ctypes.byref(cc_), ctypes.c_void_p(dc_h.data_ptr())),
                "mg_compliance")
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if args.no_e2e:
        c, dch = prob.compliance()
        e2e = None
    else:
        c, dch = cc_.value, dc_h.numpy().copy()
        e2e = {"value": replicas_throughput(sum(e2e_ms) / len(e2e_ms), world, dev)[1], "unit": "solves/s",
               "h2d_bytes_per_step": int(rho.nbytes),
               "d2h_bytes_per_step": int(prob.n_dofs * 8 + NX * NY * NZ * 8 + 8),
               "host_buffers": "pinned"}
    dc_err = float(np.abs(dch - g["dc"]).max() / np.abs(g["dc"]).max())

    # ---------------- the BF16-input variant on the same workload: split BF16 tensor-core
    # operator (three BF16 products, FP32 accumulation), the same schedule otherwise;
    # inputs resident, CUDA events, L2 flushed between solves; errors against the fixture
    bf16 = None
    if prec != M.MIXED_BF16X3 and not args.no_bf16:
        ob = M.SolveOpts.from_buffer_copy(opts)
        ob.precision = M.MIXED_BF16X3
        step_resident(ob)  # graph capture
        bt, brep = [], None
        for _ in range(3):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            b0 = torch.cuda.Event(enable_timing=True)
            b1 = torch.cuda.Event(enable_timing=True)
            b0.record(stream)
            brep, bc = step_resident(ob)
            b1.record(stream)
            torch.cuda.synchronize()
            bt.append(b0.elapsed_time(b1))
        _, bdc = prob.compliance()
        bf16 = {"precision": "bf16x3", "solves_per_s": 1e3 * len(bt) / sum(bt),
                "ms_per_solve": sum(bt) / len(bt), "status": brep.status,
                "iterations": brep.krylov_iterations, "refinements": brep.refinements,
                "relres_fp64": brep.relres,
                "compliance_rel_err_vs_oracle": abs(bc - float(g["compliance"])) / float(g["compliance"]),
                "sens_rel_err_vs_oracle": float(np.abs(bdc - g["dc"]).max() / np.abs(g["dc"]).max())}

    # ---------------- dominant kernel: tensor-core column operator, timed alone
    n = prob.n_dofs
    n_el = NX * NY * NZ
    reps_k = 50
    k0 = torch.cuda.Event(enable_timing=True)
    k1 = torch.cuda.Event(enable_timing=True)
    M.check(M.lib().mg_debug_launch_apply(prob.h, prec, 5), "warm")
    torch.cuda.synchronize()
    k0.record(stream)
    M.check(M.lib().mg_debug_launch_apply(prob.h, prec, reps_k), "apply")
    k1.record(stream)
    torch.cuda.synchronize()
    k_ms = k0.elapsed_time(k1) / reps_k
    # algorithmic bytes per launch: read z, p_old (4 B each per dof), write p_new, q,
    # read E (4 B per element) and the node Dirichlet mask (1 B per node)
    alg_bytes = 16 * n + 4 * n_el + n // 3
    pk = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    roof = {"kernel": "mf_col_kernel (tcgen05 %s column operator, CG step)" % args.precision,
            "bound": "hbm", "achieved": alg_bytes / (k_ms * 1e-3) / 1e9, "peak": peak,
            "unit": "GB/s", "frac": alg_bytes / (k_ms * 1e-3) / 1e9 / peak,
            "traffic": profiled_traffic(), "traffic_source": os.path.relpath(PROFILE, REPO),
            "bytes_per_launch": alg_bytes, "us_per_launch": k_ms * 1e3,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in pk else "fallback"}
    # the multigrid level operator (factored FP32, CUDA cores) on the same grid: y = A x,
    # read x, D^-1 (4 B per dof each), E (4 B per element), write y
    M.check(M.lib().mg_debug_launch_apply(prob.h, M.OPERATOR_FACTORED_FP32, 5), "warm")
    torch.cuda.synchronize()
    k0.record(stream)
    M.check(M.lib().mg_debug_launch_apply(prob.h, M.OPERATOR_FACTORED_FP32, reps_k), "apply")
    k1.record(stream)
    torch.cuda.synchronize()
    f_ms = k0.elapsed_time(k1) / reps_k
    f_bytes = 12 * n + 4 * n_el
    roof_fac = {"kernel": "mf_fac_kernel<3> (factored FP32 multigrid level operator, y = A x)",
                "bound": "hbm", "achieved": f_bytes / (f_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": f_bytes / (f_ms * 1e-3) / 1e9 / peak, "bytes_per_launch": f_bytes,
                "us_per_launch": f_ms * 1e3}

    # ---------------- plain FP64 form on the same GPU
    plain = None
    if not args.no_plain:
        popts = M.default_opts(precision=M.PLAIN_FP64, rtol=1e-8, timeout_s=600.0)
        prob.set_design(rho)
        prob.solve(popts)  # assemble + warm
        pt = []
        for _ in range(2):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            prob.set_design_device(d_rho.data_ptr())
            rc, prep = prob.solve_resident(popts)
            M.check(M.lib().mg_compliance_resident(prob.h, ctypes.byref(ctypes.c_double())), "c")
            p1.record(stream)
            torch.cuda.synchronize()
            pt.append(p0.elapsed_time(p1))
        sp0 = torch.cuda.Event(enable_timing=True)
        sp1 = torch.cuda.Event(enable_timing=True)
        M.check(M.lib().mg_debug_launch_apply(prob.h, M.PLAIN_FP64, 3), "spmv warm")
        torch.cuda.synchronize()
        sp0.record(stream)
        M.check(M.lib().mg_debug_launch_apply(prob.h, M.PLAIN_FP64, 20), "spmv")
        sp1.record(stream)
        torch.cuda.synchronize()
        sp_ms = sp0.elapsed_time(sp1) / 20
        nnz = prob.nnz
        sp_bytes = 8 * nnz + 4 * nnz // 3 + 4 * (n // 3) + 32 * n
        plain = {"solves_per_s": 1e3 / statistics.median(pt), "ms_per_solve": statistics.median(pt),
                 "iterations": prep.krylov_iterations, "relres": prep.relres,
                 "spmv_us": sp_ms * 1e3, "spmv_GBps": sp_bytes / (sp_ms * 1e-3) / 1e9,
                 "spmv_frac": sp_bytes / (sp_ms * 1e-3) / 1e9 / peak}

    small = None if args.no_small else bench_small_configs(M, with_cpu=not args.no_cpu)
    batch = None if args.no_batch else bench_batch(M)
    serve = None
    if not args.no_serve:
        rates = [50, 200, 500, 1000, 2000]
        counts = [args.serve_requests] * len(rates)
        if args.serve_full:
            rates.append(2000)
            counts.append(args.serve_full)
        serve = bench_serve(M, rates, counts)
        plain_sz = plain_time_per_size(M, list(M.BATCH_SIZES) + [(192, 96, 96)])
        # request mix: chain grids uniform over the five sizes, 2 % of chains on
        # 192x96x96, 2.5 load cases on average
        mean_t = 0.98 * sum(plain_sz[sz] for sz in M.BATCH_SIZES) / 5 + 0.02 * plain_sz[(192, 96, 96)]
        serve["plain_fp64_est_requests_per_s"] = 1.0 / (2.5 * mean_t)
        serve["plain_fp64_method"] = ("cold plain solve per grid size, weighted by the request mix "
                                      "(2.5 load cases per request)")

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (TF32 tensor-core operator) / f64 refinement" if args.precision.startswith("tf32")
                else "f32 (BF16 tensor-core operator) / f64 refinement",
                "data": "synthetic (seeded U[0.01,1] densities, default_rng(0))",
                "config": bench_config(world),
                "solver": {"precision": args.precision, "inner_rtol": opts.inner_rtol,
                           "preconditioner": args.preconditioner, "schedule": schedule},
                "step_ms": [round(x, 3) for x in ms],
                "dof_per_s": value * n,
                "iterations": reps[-1][0], "refinements": reps[-1][1],
                "relres_fp64": reps[-1][2], "compliance_rel_err_vs_oracle": comp_err,
                "sens_rel_err_vs_oracle": dc_err,
                "e2e": e2e,
                "roofline": roof, "roofline_level_operator": roof_fac, "plain_fp64": plain,
                "speedup_vs_plain_fp64": (value / plain["solves_per_s"]) if plain else None,
                "bf16x3": bf16,
                "small_configs": small, "batch": batch, "serving": serve,
                "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
                "wall_s_timed": t_wall}
        print(json.dumps(line), flush=True)
    prob.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
