"""Benchmark: systems solved per second at relative residual 1e-10.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--quick]

Headline workload: ParILU(0) (5 sweeps) + ISAI(L, U on |T|^2) preconditioned
BiCGSTAB of 4096 FP64 systems on a 3D 7-point 10x10x10 pattern (n = 1000,
nnz = 6400), seeded synthetic values, relative tolerance 1e-10.  One step =
one solve of the whole batch (preconditioner generation + iteration) through
the library's C ABI.  `value` is measured with the inputs resident in HBM;
`e2e` adds the pinned host->device copy of the step's values and right-hand
sides and the device->host copy of the solutions and per-system results.

Under torchrun (N > 1) rank r solves systems r*B .. (r+1)*B-1 of one seeded
global batch on its own GPU (shard.py; weak scaling, no collective on the data
path); the step time is the maximum over ranks.

--impl reference times the CPU restatement of the reference's solver (the
reference has no CPU path of its own: ILU_0_Factorization_Cpu is declared at
ILU_0.h:7 and never defined) on all host cores, on the same headline batch and
config, 4096 systems per step.  Its line also carries the reference's own GPU
kernels (compiled from its sources into oracle/_ref) timed on the one workload
they can run: the merged ILU(0) BiCGSTAB of 16384 2D 5-point 16x16 systems
(the reference's solvers need n <= 512 and, for ISAI, n <= 54 by their static
shared memory, so they cannot run the headline's n = 1000).
"""
import argparse
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _sub in ("merging-ilu0_gb300", "oracle", "tests"):
    sys.path.insert(0, os.path.join(ROOT, _sub))

SEED = 20261203
METRIC = "systems solved/sec at rel. residual 1e-10: chosen vs plain form, % HBM roofline"

# workloads: (kind, gx, gy, gz, nsys, options)
HEADLINE = dict(name="parilu5_isai_3d7_10x10x10", kind=2, grid=(10, 10, 10), nsys=4096, autotune=True,
                desc="ParILU(0) 5 sweeps + ISAI(L,U on |T|^2) BiCGSTAB, ISAI computed, stored and applied in FP32 "
                     "(A*x, inner products, recurrences, ParILU in FP64), 4096 FP64 systems, 3D 7-point 10x10x10 "
                     "(n=1000, nnz=6400), Peclet skew U(0,0.5), rel. tol 1e-10, max 500 iterations",
                opts=dict(precond=4, parilu_sweeps=5, isai_power=2, tol_mode=1, tol=1e-10, max_iter=500,
                          reduction=1, factor_precision=1), fwd_sample=32)
SECONDARY = [
    dict(name="parilu5_isai_3d7_10x10x10_fp64", kind=2, grid=(10, 10, 10), nsys=4096, autotune=True,
         desc="headline workload with FP64 ISAI values",
         opts=dict(precond=4, parilu_sweeps=5, isai_power=2, tol_mode=1, tol=1e-10, reduction=1, factor_precision=0)),
    dict(name="plain_ilu0_3d7_10x10x10", kind=2, grid=(10, 10, 10), nsys=4096, autotune=True,
         desc="plain form on the headline systems: merged FP64 ILU(0) BiCGSTAB, FAST order (register-resident "
              "kernel: ILU(0) and the factors in shared memory, vectors in registers)",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1)),
    dict(name="fp32_ilu0_3d7_10x10x10", kind=2, grid=(10, 10, 10), nsys=4096, autotune=True,
         desc="headline systems, merged ILU(0) with the factors stored and applied in FP32 (FP64 factorisation, "
              "A*x, inner products, recurrences), FAST order",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1), fwd_sample=32),
    dict(name="plain_ilu0_2d5_16x16_fast", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="plain form: merged FP64 ILU(0) BiCGSTAB, 16384 FP64 systems, 2D 5-point 16x16, rel 1e-10, FAST order "
              "(register-resident kernel)",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1)),
    dict(name="fp32_ilu0_2d5_16x16", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="16384 2D 5-point 16x16 systems, merged ILU(0) with FP32-stored factors, FAST order",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1)),
    dict(name="fp32_isai_2d5_16x16", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="16384 2D 5-point 16x16 systems, ILU(0) + ISAI stored and applied in FP32 (FP64 A*x, inner products, "
              "recurrences), FAST order",
         opts=dict(precond=3, ilu_approach=3, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1)),
    dict(name="plain_ilu0_2d5_16x16_ref", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="plain form in the reference's operation order (bit-identical iterates; register-resident one-warp "
              "kernel)",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=0)),
    dict(name="ref_rule_merged_ilu0_2d5_16x16_ref", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="the reference merged kernel's workload and stopping rule (absolute 1e-11 on the recursive residual, "
              "500 iterations): merged FP64 ILU(0) BiCGSTAB of 16384 2D 5-point 16x16 systems in the reference's "
              "operation order (bit-identical to the reference kernel)",
         opts=dict(precond=0, tol_mode=0, tol=1e-11, reduction=0)),
    dict(name="ref_rule_merged_ilu0_2d5_16x16_fast", kind=1, grid=(16, 16, 1), nsys=16384, autotune=True,
         desc="the same batch and stopping rule in FAST order (register-resident kernel)",
         opts=dict(precond=0, tol_mode=0, tol=1e-11, reduction=1)),
    dict(name="fp32_isai_cd2d_24x24", kind=4, grid=(24, 24, 1), nsys=32768, autotune=True,
         desc="ILU(0) + ISAI stored and applied in FP32 (FP64 A*x, inner products, recurrences), 32768 "
              "convection-diffusion systems 24x24",
         opts=dict(precond=3, ilu_approach=3, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1), fwd_sample=256),
    dict(name="fp32_ilu0_cd2d_24x24", kind=4, grid=(24, 24, 1), nsys=32768, autotune=True,
         desc="FP32-stored ILU(0) factors (FP64 recurrences), 32768 convection-diffusion systems 24x24",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1), fwd_sample=256),
    dict(name="fp64_ilu0_cd2d_24x24", kind=4, grid=(24, 24, 1), nsys=32768, autotune=True,
         desc="same workload with FP64 factors",
         opts=dict(precond=0, tol_mode=1, tol=1e-10, reduction=1, factor_precision=0), fwd_sample=256),
]


# ncu figures of one register-resident solver launch on the headline workload in the configuration the
# autotuner chooses there on GB300 (the occupancy variant with 4 rows per thread: 256 threads per system,
# 4 CTAs per SM, operands read through L1; smem_staging 16): DRAM bytes (dram__bytes_read.sum +
# dram__bytes_write.sum) of a 3072-system launch divided by 3072 -- the traffic grows in proportion to the
# systems of a launch -- and the FP64 pipe (sm__pipe_fp64_cycles_active, percent of peak sustained active).
RR_NCU = {"kernel": "k_bicgstab_rr_occ<4, 1, float>", "threads_per_system": 256, "smem_staging": 16,
          "sm__pipe_fp64_cycles_active_pct": 62.5, "dram_bytes_per_system": 195_600,
          "source": "profiles/k_bicgstab_rr_occ_parilu5_isai_fp32_3d7_10x10x10.md (3072 systems)"}

# systems of the headline workload that both CPU timings run (the GPU line's cpu_baseline and every step of
# --impl reference): the whole 4096-system batch, so that the two samples are the same work
CPU_SAMPLE = 4096


def bytes_per_system(n, nnz):
    """Compulsory HBM bytes of one solved system: A values, b, x, 24 B of results."""
    return 8 * nnz + 16 * n + 24


def fp64_flops_per_iter(n, nnz, prec_nnz, precond):
    """FP64 operations of one full BiCGSTAB iteration (2 per FMA): two SpMVs with A, two
    preconditioner applications (ISAI: two SpMVs; LU: two triangular solves), six inner products
    and the vector updates."""
    fma = 2 * nnz + 6 * n + 6 * n
    fma += 2 * prec_nnz
    return 2 * fma


def solver_kernel_name(info, n, opts):
    """The solver kernel a plan launches, from its configuration (bilu_plan_get_info)."""
    if info["solver_kernel"] != 1:
        return "k_bicgstab (shared-memory solver)"
    rows = next(r for r in (1, 2, 4, 8) if r * info["threads"] >= n)
    pv = {0: 3, 1: 3, 2: 3, 3: 1, 4: 1, 5: 0, 6: 2}[opts["precond"]]
    ft = "float" if opts.get("factor_precision", 0) == 1 and pv else "double"
    if info["operands_in_smem"] & 16:
        return f"k_bicgstab_rr_occ<{rows}, {pv}, {ft}> (register-resident solver, occupancy variant, " \
               f"{info['threads']} threads per system)"
    return f"k_bicgstab_rr<{rows}, {pv}, {ft}> (register-resident solver, {info['threads']} threads per system)"


def launches_per_step(info):
    """Kernels one headline solve launches: ParILU sweeps, ISAI, the solver, plus one SELL-32 copy each of A
    and aiU when the plan reads them that way and does not stage them in shared memory."""
    ops = info["operands_in_smem"]
    n = 3
    if ops & 8:
        n += (0 if ops & 1 else 1) + (0 if ops & 4 else 1)
    return n


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_info():
    """Host cores and CPU model name of the machine the CPU timings run on."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for ln in open("/proc/cpuinfo"):
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    import platform
    return {"nproc": os.cpu_count(), "model": model or platform.processor() or platform.machine(),
            "arch": platform.machine()}


def headline_config(world=1):
    """The `config` of both arms' JSON lines (the same workload, so the same dict)."""
    import bilu
    kind, (gx, gy, gz) = HEADLINE["kind"], HEADLINE["grid"]
    rp, ci, _, _ = bilu.gen_stencil(kind, gx, gy, gz, 0, SEED)
    n, nnz, nsys = len(rp) - 1, len(ci), HEADLINE["nsys"]
    fp32 = HEADLINE["opts"].get("factor_precision", 0) == 1
    return {"workload": HEADLINE["desc"], "nsys": nsys, "n": n, "nnz": nnz,
            "reduction": "fast" if HEADLINE["opts"].get("reduction", 0) == 1 else "reference",
            "factor_precision": "fp32 ISAI (FP64 A*x, inner products, recurrences, ParILU)" if fp32 else "fp64",
            "l2": "inputs larger than L2: A values %.0f MB per step" % (nsys * nnz * 8 / 1e6),
            "parallelism": f"weak: {world} slab(s) of {nsys} systems of one seeded batch, one per GPU, "
                           f"no collective on the data path"}


def headline_dtype():
    return "f64 (ISAI FP32)" if HEADLINE["opts"].get("factor_precision", 0) == 1 else "f64"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_port_rate(wl, sample, threads=None):
    """Systems/s of the oracle (CPU restatement of the reference path) on a bounded sample.  The
    pattern-only work (diagonal insertion, L/U split, ISAI patterns) runs once before the timed call,
    as the GPU arm's plan does it once before its timed steps; the timed call runs the per-system
    arithmetic: factorisation, ISAI values, BiCGSTAB and the true residual."""
    import bilu
    import helpers as H
    import oracle as O
    if threads:
        O.set_num_threads(threads)
    kind, (gx, gy, gz) = wl["kind"], wl["grid"]
    rp, ci, v, b = bilu.gen_stencil(kind, gx, gy, gz, sample, SEED)
    o = wl["opts"]
    kw = dict(approach=o.get("ilu_approach", 1), sweeps=o.get("parilu_sweeps", 5),
              fp32=o.get("factor_precision", 0) == 1, tol_mode=o.get("tol_mode", 0), tol=o.get("tol", 1e-11),
              max_iter=o.get("max_iter", 500), isai_power=o.get("isai_power", 2))
    patterns = {}
    H.oracle_pipeline(rp, ci, v[:1], b[:1], o["precond"], patterns=patterns, **kw)
    t0 = time.perf_counter()
    r = H.oracle_pipeline(rp, ci, v, b, o["precond"], patterns=patterns, **kw)
    dt = time.perf_counter() - t0
    return sample / dt, dt, O.num_threads(), float(r["iters"].mean())


def reference_gpu_kernels(steps, warmup):
    """The reference's own merged ILU(0) BiCGSTAB kernel (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:249-538,
    compiled from its sources into oracle/_ref, launched as its helper does at :568-577) on 16384 2D 5-point 16x16
    systems with the reference's stopping rule (absolute 1e-11 on the recursive residual, 500 iterations), timed
    with CUDA events.  Its busy-wait triangular solves need n <= 512 and converging systems, so it runs only
    after the oracle's reference-order solve of the same batch has converged everywhere with finite values."""
    try:
        import torch
        import ref as R
    except ImportError as ex:
        return {"unavailable": f"import failed: {ex}"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    if not R.available():
        return {"unavailable": "reference kernels not built (oracle/_ref; oracle/build_ref.py builds them where the "
                               "reference sources are present)"}
    import bilu
    import helpers as H
    import oracle as O
    nsys = 16384
    rp, ci, v, b = bilu.gen_stencil(1, 16, 16, 1, nsys, SEED)
    n, nnz = len(rp) - 1, len(ci)
    gate = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, tol_mode=0, tol=1e-11, max_iter=500)
    if not (np.all(gate["conv"] == 1) and np.all(np.isfinite(gate["x"]))):
        return {"unavailable": "the oracle's reference-order solve did not converge everywhere: the reference's "
                               "busy-wait triangular solves are not run on this batch"}
    dev = torch.device("cuda", 0)
    T = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    RP, CI, D = T(rp, torch.int32), T(ci, torch.int32), T(O.find_diag(rp, ci), torch.int32)
    V, B = T(v, torch.float64), T(b, torch.float64)
    X = torch.zeros_like(B)
    F = torch.empty_like(V)
    it = torch.zeros(nsys, dtype=torch.float32, device=dev)
    cv = torch.zeros(nsys, dtype=torch.int32, device=dev)
    rs = torch.zeros(nsys, dtype=torch.float64, device=dev)
    L = R.lib()
    args = (L.ref_merged, n, nnz, nsys, RP, CI, V, B, X, F, D, it, cv, rs)
    for _ in range(max(warmup, 1)):
        R._call(*args)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        R._call(*args)  # the reference's kernel on the legacy default stream (torch's current stream here)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    iters = it.cpu().numpy()
    same = bool(np.array_equal(iters, gate["iters"]) and np.array_equal(X.cpu().numpy(), gate["x"]))
    return {"workload": "merged ILU(0) BiCGSTAB (the reference's namesake kernel), 16384 FP64 systems, 2D 5-point "
                        "16x16 (n=256, nnz=1216), absolute tol 1e-11 on the recursive residual, max 500 iterations",
            "kernel": "KernelBatchedPreconditionedBiCGSTAB_ILU (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu), "
                      "built for sm_103a from the reference sources, 16384 CTAs of 512 threads",
            "systems_per_s": nsys / (ms / 1e3), "ms_per_step": ms, "steps": steps, "mean_iters": float(iters.mean()),
            "converged": int((cv == 1).sum().item()), "bit_identical_to_oracle_reference_order": same,
            "compare_with": "the GPU arm's secondary lines ref_rule_merged_ilu0_2d5_16x16_ref and _fast: the library "
                            "on the same batch and stopping rule"}


def run_reference_arm(args):
    """--impl reference: the CPU restatement of the reference's solver on all host cores, on the headline
    batch (CPU_SAMPLE systems per step); the reference's own GPU kernels on the one workload they can run."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle as O
    wl = HEADLINE
    for _ in range(args.warmup):
        cpu_port_rate(wl, 64)
    rates, secs = [], []
    for _ in range(args.steps):
        rate, dt, cores, _ = cpu_port_rate(wl, CPU_SAMPLE)
        rates.append(rate)
        secs.append(dt)
    value = statistics.median(rates)
    host = cpu_info()
    line = {"metric": METRIC, "value": value, "unit": "systems/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * statistics.median(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": headline_dtype(),
            "data": "synthetic", "config": headline_config(int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": value, "unit": "systems/s", "cores": O.num_threads(), "kind": "port",
                             "host": host,
                             "sample": f"the headline batch ({CPU_SAMPLE} systems) per step, full pipeline (ParILU "
                                       f"sweeps, ISAI, BiCGSTAB) in the reference's operation order, OpenMP over "
                                       f"systems on {O.num_threads()} threads of {host['nproc']} host cores "
                                       f"({host['model']}); the pattern work runs once per step, untimed, as in "
                                       f"the GPU arm's plan; value = median over the steps"},
            "e2e": {"value": value, "unit": "systems/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu_kernels": reference_gpu_kernels(args.steps, args.warmup)}
    print(json.dumps(line))


def measure(wl, steps, warmup, dev, stream, sampler=None, e2e=False, timed_hook=None, first=0):
    """first: index of this rank's first system in the seeded global batch (its slab)."""
    import torch
    import bilu
    kind, (gx, gy, gz), nsys = wl["kind"], wl["grid"], wl["nsys"]
    rp, ci, v, b = bilu.gen_stencil(kind, gx, gy, gz, nsys, SEED, first=first)
    n, nnz = len(rp) - 1, len(ci)
    plan = bilu.Plan(rp, ci, **wl["opts"])
    plan.enable_timing(True)
    V = torch.from_numpy(v).to(dev)
    B = torch.from_numpy(b).to(dev)
    X = torch.empty_like(B)
    it = torch.empty(nsys, dtype=torch.float32, device=dev)
    cv = torch.empty(nsys, dtype=torch.int32, device=dev)
    rs = torch.empty(nsys, dtype=torch.float64, device=dev)
    tr = torch.empty(nsys, dtype=torch.float64, device=dev)
    st = torch.empty(nsys, dtype=torch.int32, device=dev)
    del v, b
    with torch.cuda.stream(stream):
        if wl.get("autotune"):
            plan.autotune(V, B, X, stream=stream)  # configuration search, outside the timed region
        for _ in range(warmup):
            plan.solve(V, B, X, it, cv, rs, tr, st, stream=stream)
        torch.cuda.synchronize()
        setup, solve = [], []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if timed_hook:
            timed_hook("begin")
        if sampler:
            sampler.start()
        e0.record(stream)
        for _ in range(steps):
            plan.solve(V, B, X, it, cv, rs, tr, st, stream=stream)
            t = plan.last_timing()
            setup.append(t["setup_ms"])
            solve.append(t["solve_ms"])
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        if timed_hook:
            timed_hook("end")
        ms = e0.elapsed_time(e1)
    fwd = None
    if wl.get("fwd_sample"):
        ids = np.arange(0, nsys, max(1, nsys // wl["fwd_sample"]), dtype=np.int32)[: wl["fwd_sample"]]
        fe = plan.forward_error(V, B, X, ids)
        fwd = {"systems": len(ids), "median": float(np.median(fe)), "max": float(fe.max()),
               "oracle": "FP64 dense LU with partial pivoting on the GPU (bilu_forward_error)"}
    iters = it.cpu().numpy()
    conv = cv.cpu().numpy()
    trn = tr.cpu().numpy()
    bn = B.norm(dim=1).cpu().numpy()
    info = plan.info()
    out = {"name": wl["name"], "nsys": nsys, "n": n, "nnz": nnz, "ms_total": ms, "steps": steps,
           "systems_per_s": nsys * steps / (ms / 1e3), "setup_ms": statistics.mean(setup),
           "solve_ms": statistics.mean(solve), "mean_iters": float(iters.mean()), "max_iters": float(iters.max()),
           "converged": int((conv == 1).sum()), "max_rel_true_res": float((trn / bn).max()), "info": info,
           "clocks": clocks, "forward_error": fwd}
    if e2e:
        # End to end through the C ABI with host buffers: every step copies its values and right-hand sides
        # host -> device and reads x and the per-system results back, all inside the timed region.  Two
        # device buffer sets and two copy streams pipeline the steps: the inputs of step k+1 travel and the
        # results of step k-1 come back while step k solves.
        hv = torch.empty(V.shape, dtype=V.dtype, pin_memory=True)
        hv.copy_(V)
        hb = torch.empty(B.shape, dtype=B.dtype, pin_memory=True)
        hb.copy_(B)
        hx = torch.empty(B.shape, dtype=B.dtype, pin_memory=True)
        hit = torch.empty(nsys, dtype=torch.float32, pin_memory=True)
        hcv = torch.empty(nsys, dtype=torch.int32, pin_memory=True)
        hrs = torch.empty(nsys, dtype=torch.float64, pin_memory=True)
        bufs = [(V, B, X, it, cv, rs)] + [(torch.empty_like(V), torch.empty_like(B), torch.empty_like(X),
                                           torch.empty_like(it), torch.empty_like(cv), torch.empty_like(rs))]
        h2d_s, d2h_s = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        ready = [torch.cuda.Event() for _ in range(2)]
        solved = [torch.cuda.Event() for _ in range(2)]
        free = [torch.cuda.Event() for _ in range(2)]
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)

        def h2d(k):
            Vk, Bk = bufs[k % 2][0], bufs[k % 2][1]
            h2d_s.wait_event(f0)
            if k >= 2:
                h2d_s.wait_event(free[k % 2])  # step k-2 solved and read back
            with torch.cuda.stream(h2d_s):
                Vk.copy_(hv, non_blocking=True)
                Bk.copy_(hb, non_blocking=True)
            ready[k % 2].record(h2d_s)

        h2d(0)
        for k in range(steps):
            Vk, Bk, Xk, itk, cvk, rsk = bufs[k % 2]
            if k + 1 < steps:
                h2d(k + 1)
            stream.wait_event(ready[k % 2])
            plan.solve(Vk, Bk, Xk, itk, cvk, rsk, tr, st, stream=stream)
            solved[k % 2].record(stream)
            d2h_s.wait_event(solved[k % 2])
            with torch.cuda.stream(d2h_s):
                hx.copy_(Xk, non_blocking=True)
                hit.copy_(itk, non_blocking=True)
                hcv.copy_(cvk, non_blocking=True)
                hrs.copy_(rsk, non_blocking=True)
            free[k % 2].record(d2h_s)
        stream.wait_stream(d2h_s)
        f1.record(stream)
        torch.cuda.synchronize()
        ems = f0.elapsed_time(f1)
        out["e2e"] = {"value": nsys * steps / (ems / 1e3), "unit": "systems/s",
                      "h2d_bytes_per_step": int(hv.numel() * 8 + hb.numel() * 8),
                      "d2h_bytes_per_step": int(hx.numel() * 8 + nsys * (4 + 4 + 8)),
                      "pipelining": "double-buffered: H2D of step k+1 and D2H of step k-1 overlap the solve of step k"}
        if not (conv == 1).all():
            out["e2e"]["note"] = "not every system converged"
    plan.close()
    return out


def measure_uneven(dev, stream, nsys=8192, steps=3, warmup=2, fp32=False):
    """Uneven batch: 8192 systems, n log-uniform in [64, 1024], own random pattern each (5-12 off-diagonals
    per row), merged ILU(0) with FP64 (plain) or FP32-stored factors, FAST order, rel. tol 1e-10; autotuned
    buckets, one CUDA-graph launch per step."""
    import torch
    import bilu
    sn, sz, rp, ci, v, b = bilu.gen_uneven(nsys, SEED, 64, 1024, 5, 12)
    plan = bilu.UnevenPlan(sn, sz, rp, ci, tol_mode=1, tol=1e-10, reduction=1, factor_precision=1 if fp32 else 0)
    V = torch.from_numpy(v).to(dev)
    B = torch.from_numpy(b).to(dev)
    X = torch.empty_like(B)
    it = torch.empty(nsys, dtype=torch.float32, device=dev)
    cv = torch.empty(nsys, dtype=torch.int32, device=dev)
    rs = torch.empty(nsys, dtype=torch.float64, device=dev)
    tr = torch.empty(nsys, dtype=torch.float64, device=dev)
    st = torch.empty(nsys, dtype=torch.int32, device=dev)
    with torch.cuda.stream(stream):
        plan.autotune(V, B, X, stream=stream)
        for _ in range(warmup):
            plan.solve(V, B, X, it, cv, rs, tr, st, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            plan.solve(V, B, X, it, cv, rs, tr, st, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    info = plan.info()
    plan.close()
    bpsys = (12 * sz + 20 * sn + 4 + 28).astype(np.float64)  # values+cols, b/x/row ptrs, results
    return {"name": "uneven_ilu0_n64_1024" + ("_fp32" if fp32 else ""), "nsys": nsys, "steps": steps,
            "systems_per_s": nsys * steps / (ms / 1e3),
            "ms_per_step": ms / steps, "mean_iters": float(it.mean().item()), "converged": int((cv == 1).sum().item()),
            "mean_n": float(sn.mean()), "total_nnz": int(sz.sum()), "bytes_per_step": float(bpsys.sum()),
            "buckets": [{k: i[k] for k in ("n_hi", "systems", "threads", "grid", "smem_bytes", "tuned_ms")}
                        for i in info if i["systems"]],
            "workload": "uneven batch: 8192 FP64 systems, n log-uniform in [64,1024], 5-12 random off-diagonals per "
                        "row, diag 1.2x abs row sum with random sign, merged ILU(0) with %s factors, FAST order "
                        "(register-resident solver, one CTA per system), rel 1e-10, autotuned threads per system per "
                        "size bucket, one CUDA-graph launch per step" % ("FP32-stored" if fp32 else "FP64")}


def measure_learned(dev, stream, ntrain=65536, neval=16384, train_steps=1500, batch=65536, steps=3):
    """Learned ParILU warm start on 3D 7-point 7x7x7 systems: train the MLP on the converged ParILU(0)
    factors of `ntrain` systems, then solve `neval` fresh systems with ParILU sweeps until the ILU residual is
    <= 1e-6 (at most 40) + ISAI in FP32 + BiCGSTAB (FAST order, rel 1e-10), with the plain A-value start and
    with the learned warm start (fallback to A values when its ILU residual exceeds 1e-3)."""
    import torch
    import bilu
    rp, ci, v, _ = bilu.gen_stencil(5, 7, 7, 7, ntrain, SEED + 1)
    opts = dict(precond=4, parilu_sweeps=40, parilu_res_tol=1e-6, tol_mode=1, tol=1e-10, reduction=1,
                factor_precision=1)
    plan = bilu.Plan(rp, ci, **opts)
    V = torch.from_numpy(v).to(dev)
    del v
    LU = torch.empty_like(V)
    plan.parilu0(V, LU, 40, stream=stream)
    torch.cuda.synchronize()
    m = bilu.Mlp(seed=SEED)
    t0 = time.perf_counter()
    losses = m.train(plan, V, LU, train_steps, batch, 2e-3, seed=SEED, stream=stream)
    train_s = time.perf_counter() - t0
    del V, LU
    _, _, v2, b2 = bilu.gen_stencil(5, 7, 7, 7, neval, SEED + 2)
    V2 = torch.from_numpy(v2).to(dev)
    B2 = torch.from_numpy(b2).to(dev)
    X = torch.empty_like(B2)
    it = torch.empty(neval, dtype=torch.float32, device=dev)
    cv = torch.empty(neval, dtype=torch.int32, device=dev)
    sw = torch.empty(neval, dtype=torch.int32, device=dev)
    LU0 = torch.empty_like(V2)
    res = torch.empty(neval, dtype=torch.float64, device=dev)
    used = torch.empty(neval, dtype=torch.int32, device=dev)
    with torch.cuda.stream(stream):
        plan.autotune(V2, B2, X, stream=stream)
    out = {"name": "learned_warm_start_3d7_7x7x7", "ntrain": ntrain, "neval": neval, "train_steps": train_steps,
           "batch": batch, "train_s": train_s, "loss_first": float(losses[:10].mean()),
           "loss_last": float(losses[-10:].mean())}
    # inference alone: the warm start of all evaluation systems (both layers on the tensor cores)
    with torch.cuda.stream(stream):
        for _ in range(3):
            m.warm_start(plan, V2, LU0, 1e-3, res, used, stream=stream)
        torch.cuda.synchronize()
        w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0.record(stream)
        for _ in range(steps):
            m.warm_start(plan, V2, LU0, 1e-3, res, used, stream=stream)
        w1.record(stream)
        torch.cuda.synchronize()
    out["warm_start_ms"] = w0.elapsed_time(w1) / steps
    out["train_ms_per_step"] = 1e3 * train_s / train_steps
    with torch.cuda.stream(stream):
        for mode in ("plain", "learned"):
            def step():
                if mode == "plain":
                    plan.solve(V2, B2, X, it, cv, sweeps=sw, stream=stream)
                else:
                    m.warm_start(plan, V2, LU0, 1e-3, res, used, stream=stream)
                    plan.solve(V2, B2, X, it, cv, sweeps=sw, lu_init=LU0, stream=stream)
            step()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            out[mode] = {"systems_per_s": neval / (ms / 1e3), "ms_per_step": ms,
                         "mean_sweeps": float(sw.float().mean().item()), "mean_iters": float(it.mean().item()),
                         "converged": int((cv == 1).sum().item())}
            if mode == "learned":
                out[mode]["warm_start_accepted"] = float(used.float().mean().item())
                out[mode]["median_warm_ilu_residual"] = float(res.median().item())
    # the plain form on the same systems: merged FP64 ILU(0) + BiCGSTAB
    pl = bilu.Plan(rp, ci, precond=0, tol_mode=1, tol=1e-10, reduction=1)
    with torch.cuda.stream(stream):
        pl.solve(V2, B2, X, it, cv, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            pl.solve(V2, B2, X, it, cv, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out["plain_ilu0_fp64"] = {"systems_per_s": neval / (ms / 1e3), "ms_per_step": ms,
                              "mean_iters": float(it.mean().item()), "converged": int((cv == 1).sum().item())}
    pl.close()
    out["speedup_learned_vs_plain"] = out["learned"]["systems_per_s"] / out["plain"]["systems_per_s"]
    out["speedup_chosen_vs_plain_ilu0_fp64"] = (out["learned"]["systems_per_s"] /
                                                out["plain_ilu0_fp64"]["systems_per_s"])
    out["workload"] = ("learned ParILU warm start: MLP 9-64-64-1 (GELU, BF16 weights, FP32 accumulation) trained on "
                       "65536 3D 7-point 7x7x7 systems' converged ParILU(0) factors; 16384 fresh systems, ParILU "
                       "sweeps to ILU residual 1e-6 + ISAI(L,U) stored and applied in FP32 + BiCGSTAB, rel 1e-10")
    m.close()
    plan.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline only, no secondary workloads")
    ap.add_argument("--kernel-only", action="store_true",
                    help="headline solve only: no e2e pass, secondary workloads or CPU baseline (profiling runs)")
    ap.add_argument("--nsys", type=int, default=0, help="override the headline batch size (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the plan's default solver configuration (profiling runs: fixed launch sequence)")
    ap.add_argument("--smem-staging", type=int, default=-1,
                    help="with --no-autotune: the solver configuration mask (bilu_options.smem_staging), e.g. the "
                         "one the autotuner chooses, so that a profiling run launches that kernel")
    ap.add_argument("--threads", type=int, default=0,
                    help="with --no-autotune: threads per system of the solver (profiling runs)")
    ap.add_argument("--workload", default="",
                    help="with --kernel-only: measure this secondary workload (by name) instead of the headline "
                         "(profiling runs)")
    args = ap.parse_args()
    learned_only = args.workload == "learned_warm_start_3d7_7x7x7"
    if args.workload and not learned_only:
        found = [w for w in SECONDARY if w["name"] == args.workload]
        if not found or not args.kernel_only:
            ap.error("--workload needs --kernel-only and one of: " + ", ".join(
                [w["name"] for w in SECONDARY] + ["learned_warm_start_3d7_7x7x7"]))
        HEADLINE.clear()
        HEADLINE.update(found[0])
    if learned_only and not args.kernel_only:
        ap.error("--workload learned_warm_start_3d7_7x7x7 needs --kernel-only")
    if args.no_autotune:
        HEADLINE["autotune"] = False
    if args.smem_staging >= 0:
        if not args.no_autotune:
            ap.error("--smem-staging needs --no-autotune")
        HEADLINE["opts"] = dict(HEADLINE["opts"], smem_staging=args.smem_staging)
    if args.threads > 0:
        if not args.no_autotune:
            ap.error("--threads needs --no-autotune")
        HEADLINE["opts"] = dict(HEADLINE["opts"], threads_per_system=args.threads)
    if args.nsys > 0:
        HEADLINE["desc"] = HEADLINE["desc"].replace(f"{HEADLINE['nsys']} FP64", f"{args.nsys} FP64")
        HEADLINE["nsys"] = args.nsys
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch
    import bilu
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream(dev)

    def barrier(_what):
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    if learned_only:  # profiling runs of the learned warm start: training, inference, the solves
        if rank == 0:
            print(json.dumps(measure_learned(dev, stream, steps=args.steps)))
        return
    sampler = ClockSampler(local)
    import shard
    first, _ = shard.slab(HEADLINE["nsys"] * world, rank, world)  # B systems per rank (weak scaling)
    res = measure(HEADLINE, args.steps, max(args.warmup, 3), dev, stream, sampler=sampler,
                  e2e=not args.kernel_only, timed_hook=barrier, first=first)
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({k: res[k] for k in ("name", "nsys", "ms_total", "steps", "systems_per_s", "setup_ms",
                                                  "solve_ms", "mean_iters", "converged", "max_rel_true_res")}))
        return
    ms = res["ms_total"]
    if dist:
        ms = shard.max_over_ranks(ms, device=dev)
        e = torch.tensor([res["e2e"]["value"]], device=dev)
        dist.all_reduce(e, op=dist.ReduceOp.SUM)
        res["e2e"]["value"] = float(e.item())
    value = HEADLINE["nsys"] * args.steps * world / (ms / 1e3)
    secondary = []
    if rank == 0 and not args.quick:
        for wl in SECONDARY:
            try:
                r = measure(wl, args.steps, max(args.warmup, 1), dev, stream)
                secondary.append({k: r[k] for k in ("name", "nsys", "steps", "systems_per_s", "setup_ms", "solve_ms",
                                                    "mean_iters", "converged", "max_rel_true_res",
                                                    "forward_error")} |
                                 {"workload": wl["desc"]})
            except Exception as ex:  # a secondary workload never hides the headline
                secondary.append({"name": wl["name"], "error": str(ex)})
        for f32 in (False, True):
            try:
                secondary.append(measure_uneven(dev, stream, steps=args.steps, warmup=max(args.warmup, 1), fp32=f32))
            except Exception as ex:
                secondary.append({"name": "uneven_ilu0_n64_1024" + ("_fp32" if f32 else ""), "error": str(ex)})
        try:
            secondary.append(measure_learned(dev, stream, steps=args.steps))
        except Exception as ex:
            secondary.append({"name": "learned_warm_start_3d7_7x7x7", "error": str(ex)})
    if rank != 0:
        return
    # FP64 FMA issue rate of this GPU, measured now (bilu_probe_fp64_rate): the FP64 roofline's peak
    fp64_peak, fp64_probe_mhz = bilu.probe_fp64_rate()
    chosen = {}
    by_name = {sc.get("name"): sc for sc in secondary if "systems_per_s" in sc}
    plain = by_name.get("plain_ilu0_3d7_10x10x10")
    if plain:
        # FP64 operations of the plain form: A*x, two triangular solves on the in-place factors (nnz entries),
        # inner products and vector updates per iteration
        pfl = fp64_flops_per_iter(res["n"], res["nnz"], res["nnz"], 0) * plain["mean_iters"] * plain["nsys"]
        chosen["headline_3d7_10x10x10"] = {
            "workload": HEADLINE["desc"], "plain_form": "merged FP64 ILU(0) + BiCGSTAB on the same systems",
            "plain_systems_per_s": plain["systems_per_s"],
            "plain_roofline_fp64_frac": pfl / (plain["solve_ms"] / 1e3) / 1e9 / fp64_peak,
            "chosen_form": "ParILU(5) + ISAI stored and applied in FP32, register-resident solver",
            "chosen_systems_per_s": res["systems_per_s"], "ratio": res["systems_per_s"] / plain["systems_per_s"]}
        f32 = by_name.get("fp32_ilu0_3d7_10x10x10")
        if f32:
            chosen["fp32_factors_3d7_10x10x10"] = {
                "workload": "the headline systems", "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
                "plain_systems_per_s": plain["systems_per_s"],
                "chosen_form": "merged ILU(0), factors stored and applied in FP32",
                "chosen_systems_per_s": f32["systems_per_s"], "ratio": f32["systems_per_s"] / plain["systems_per_s"]}
    p16, f16 = by_name.get("plain_ilu0_2d5_16x16_fast"), by_name.get("fp32_ilu0_2d5_16x16")
    if p16 and f16:
        chosen["fp32_factors_2d5_16x16"] = {
            "workload": "16384 2D 5-point 16x16 systems", "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
            "plain_systems_per_s": p16["systems_per_s"], "chosen_form": "merged ILU(0), FP32-stored factors",
            "chosen_systems_per_s": f16["systems_per_s"], "ratio": f16["systems_per_s"] / p16["systems_per_s"]}
    i16 = by_name.get("fp32_isai_2d5_16x16")
    if p16 and i16:
        chosen["fp32_isai_2d5_16x16"] = {
            "workload": "16384 2D 5-point 16x16 systems", "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
            "plain_systems_per_s": p16["systems_per_s"], "chosen_form": "ILU(0) + ISAI stored and applied in FP32",
            "chosen_systems_per_s": i16["systems_per_s"], "ratio": i16["systems_per_s"] / p16["systems_per_s"]}
    p24, i24 = by_name.get("fp64_ilu0_cd2d_24x24"), by_name.get("fp32_isai_cd2d_24x24")
    if p24 and i24:
        chosen["fp32_isai_cd2d_24x24"] = {
            "workload": "32768 convection-diffusion systems 24x24", "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
            "plain_systems_per_s": p24["systems_per_s"], "chosen_form": "ILU(0) + ISAI stored and applied in FP32",
            "chosen_systems_per_s": i24["systems_per_s"], "ratio": i24["systems_per_s"] / p24["systems_per_s"]}
    pu, fu = by_name.get("uneven_ilu0_n64_1024"), by_name.get("uneven_ilu0_n64_1024_fp32")
    if pu and fu:
        chosen["uneven_n64_1024"] = {
            "workload": "8192 uneven systems (n log-uniform in [64,1024], own random pattern each), one CUDA-graph "
                        "launch per step", "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
            "plain_systems_per_s": pu["systems_per_s"], "chosen_form": "merged ILU(0), FP32-stored factors",
            "chosen_systems_per_s": fu["systems_per_s"], "ratio": fu["systems_per_s"] / pu["systems_per_s"]}
    for sc in secondary:
        if sc.get("name") == "learned_warm_start_3d7_7x7x7" and "learned" in sc:
            chosen["learned_3d7_7x7x7"] = {
                "workload": "16384 fresh 3D 7-point 7x7x7 systems (n=343), rel. tol 1e-10",
                "plain_form": "merged FP64 ILU(0) + BiCGSTAB",
                "plain_systems_per_s": sc["plain_ilu0_fp64"]["systems_per_s"],
                "chosen_form": "learned warm start + ParILU sweeps to ILU residual 1e-6 + ISAI in FP32",
                "chosen_systems_per_s": sc["learned"]["systems_per_s"],
                "ratio": sc["speedup_chosen_vs_plain_ilu0_fp64"]}
    n, nnz, nsys = res["n"], res["nnz"], res["nsys"]
    info = res["info"]
    hbm, peak_kind = load_peaks()
    bps = bytes_per_system(n, nnz)
    solve_s = res["solve_ms"] / 1e3
    achieved = bps * nsys / solve_s / 1e9
    fp32_prec = HEADLINE["opts"].get("factor_precision", 0) == 1
    prec_nnz = 0 if fp32_prec else info["nnz_isai_L"] + info["nnz_isai_U"]  # FP32 ISAI work is not FP64
    flops = fp64_flops_per_iter(n, nnz, prec_nnz, HEADLINE["opts"]["precond"]) * res["mean_iters"] * nsys
    host = cpu_info()
    rate, dt, used, _ = cpu_port_rate(HEADLINE, CPU_SAMPLE)
    kernel = solver_kernel_name(info, n, HEADLINE["opts"])
    # the ncu figures hold for the configuration they were captured in
    captured = (info["solver_kernel"] == 1 and fp32_prec and info["threads"] == RR_NCU["threads_per_system"]
                and info["operands_in_smem"] == RR_NCU["smem_staging"])
    line = {
        "metric": METRIC, "value": value, "unit": "systems/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": headline_dtype(), "data": "synthetic",
        "config": headline_config(world),
        "kernel_config": {"solver_kernel": kernel, "threads_per_system": info["threads"],
                          "smem_bytes_per_system": info["smem_bytes"], "smem_staging": info["operands_in_smem"],
                          "chosen_by": "bilu_plan_autotune on the batch, before the timed region"},
        "clocks": res["clocks"],
        "e2e": res["e2e"],
        "gpu_launches": launches_per_step(info) * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": RR_NCU["dram_bytes_per_system"] * nsys
                     if captured and RR_NCU["dram_bytes_per_system"] else None,
                     "traffic_source": RR_NCU["source"] + ", scaled per system", "peak_kind": peak_kind,
                     "kernel": kernel, "bytes_per_system": bps,
                     "achieved_from": "bytes_per_system x nsys / the solver launch's CUDA-event time (stages_ms.solve)"},
        "roofline_fp64": {"achieved": flops / solve_s / 1e9, "peak": fp64_peak, "unit": "GFLOP/s",
                          "frac": flops / solve_s / 1e9 / fp64_peak,
                          "peak_kind": "measured in this run: bilu_probe_fp64_rate (independent DFMA chains on every "
                                       "SM, CUDA events, best of 3 launch shapes x 5 launches)",
                          "peak_sm_mhz": fp64_probe_mhz,
                          "counted": "FP64 operations of the BiCGSTAB iterations (bench.fp64_flops_per_iter x mean "
                                     "iterations x systems); FP32 ISAI work not counted",
                          "ncu": RR_NCU if captured else None,
                          "note": "FP64 issue, not HBM, bounds this kernel on GB300"},
        "stages_ms": {"setup": res["setup_ms"], "solve": res["solve_ms"]},
        "solve_quality": {"mean_iters": res["mean_iters"], "max_iters": res["max_iters"],
                          "converged": res["converged"], "max_rel_true_residual": res["max_rel_true_res"],
                          "forward_error": res["forward_error"]},
        "cpu_baseline": {"value": rate, "unit": "systems/s", "cores": used, "kind": "port", "host": host,
                         "sample": f"the headline batch ({CPU_SAMPLE} systems) through the CPU restatement, the same "
                                   f"sample as each step of --impl reference ({dt:.2f} s, {used} OpenMP threads of "
                                   f"{host['nproc']} host cores, {host['model']}; the pattern work runs once, "
                                   f"untimed, as in the GPU arm's plan)"},
        "chosen_vs_plain": chosen or None,
        "secondary": secondary,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
