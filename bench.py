#!/usr/bin/env python
"""Benchmark of the DMRG sweep hot path: sigma = H psi throughput and sweep time.

Headline workload (one step = one sigma = H psi product): the two-site
superblock at the middle bond (L = orbitals 0..14) of the synthetic
30-orbital / 30-electron Cholesky Hamiltonian (60 vectors, seed 30, S=0,
C1), with left and right blocks renormalised to M=2000 multiplets from
seeded warm-up rotations.  The metric is FP64-equivalent sigma TFLOP/s (the
algorithmic flop count of every sector GEMM, counted by the library's
schedule compiler) of the split-precision path (bf16 slices on the tensor
cores, "bf16x3tc"), together with sweep wall times.

The line also carries: the plain FP64 path's sigma on the same superblock
(time and the split product's error), a Davidson solve of the superblock in
split precision with defect correction against FP64 residuals (its FP64
counterpart is derived from the measured FP64 product time unless
--fp64-davidson runs it), the CPU oracle's sigma (cpu_baseline), FP64-path
parity against the oracle on the 24-orbital M=500 superblock, and whole
sweeps: the 12-site Hubbard chain in FP64, split precision and on the CPU
oracle, and one sweep of the 30-orbital M=2000 system in split precision
(its FP64 sweep time derived from the per-step FP64 product times unless
--sweep-fp64 runs it).  `batching` repeats the sigma measurement, with its
schedule comparisons, on the batching case: the middle bond of the
30-orbital Hamiltonian with D2h irreps at M=1500 (many small uneven
sectors), persistent launches with stacked stage-1 products against the
unstacked plan and the per-sector-launch baseline.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--precision fp64|bf16x3|bf16x6|bf16x3tc|fp16x2tc] [--conf PATH --partition P]
                  [--sweep-conf PATH --sweep-precisions fp64,split] [--big-sweep-conf PATH] [--sweep-fp64]

With torchrun (N > 1) every rank runs an independent replica on its own GPU
("replicas only": the sigma of one superblock is not sharded).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# 30 orbitals, M=2000: the headline superblock (middle bond)
DEFAULT_CONF = os.path.join(GOLDEN, "syn30", "dmrg.conf")
DEFAULT_PARTITION = 14
# 24 orbitals, M=500: FP64 parity of the GPU sigma against the oracle
PARITY_CONF, PARITY_PARTITION = os.path.join(GOLDEN, "syn24", "dmrg.conf"), 11
# 12-site Hubbard chain, M 50 -> 100, 4 sweeps (GPU FP64, GPU split, CPU oracle)
SWEEP_CONF = os.path.join(GOLDEN, "hubbard12", "dmrg.conf")
# 30 orbitals, M=2000: warm-up and one sweep
BIG_SWEEP_CONF = os.path.join(GOLDEN, "syn30_sweep1", "dmrg.conf")
# 30 orbitals with D2h irreps, M=1500: the batching case (many small sectors)
BATCH_CONF, BATCH_PARTITION = os.path.join(GOLDEN, "syn30_d2h", "dmrg.conf"), 14
METRIC = "sigma TFLOP/s & sweep time: split-prec batched vs FP64 GPU at |dE|<=1e-6 Eh"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16x3tc",
                    choices=["fp64", "bf16x3", "bf16x6", "bf16x3tc", "fp16x2tc", "exacttc"])
    ap.add_argument("--conf", default=DEFAULT_CONF)
    ap.add_argument("--partition", type=int, default=DEFAULT_PARTITION)
    ap.add_argument("--no-davidson", action="store_true", help="skip the Davidson solve")
    ap.add_argument("--fp64-davidson", action="store_true",
                    help="also run the FP64 Davidson solve (minutes at M=2000) instead of deriving its time")
    ap.add_argument("--cpu-reps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the FP64 parity check against the oracle")
    ap.add_argument("--no-autotune", action="store_true",
                    help="default schedule knobs instead of the autotuner's (tensor-core paths)")
    ap.add_argument("--no-schedules", action="store_true",
                    help="skip the per-sector-launch baseline and default-knob comparison")
    ap.add_argument("--no-sweeps", action="store_true", help="skip every sweep")
    ap.add_argument("--sweep-conf", default=SWEEP_CONF,
                    help="dmrg.conf of the small sweep comparison (GPU FP64, GPU split, CPU oracle)")
    ap.add_argument("--sweep-precisions", default="fp64,split",
                    help="comma list of the small sweep comparison's GPU arithmetics: fp64, split")
    ap.add_argument("--big-sweep-conf", default=BIG_SWEEP_CONF,
                    help="dmrg.conf of the large split-precision sweep ('none' to skip)")
    ap.add_argument("--sweep-fp64", action="store_true",
                    help="also run the large sweep in FP64 (close to an hour at M=2000) for a measured ratio and dE")
    ap.add_argument("--no-exact", action="store_true", help="skip the exact-slice tensor-core product")
    ap.add_argument("--profile", action="store_true",
                    help="open the CUDA profiler range around the device-timed steps only")
    ap.add_argument("--no-batching", action="store_true",
                    help="skip the batching case (D2h superblock, schedule comparisons)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def whole_job(flops_per_step, t_step, t_e2e_step, dist=None, device="cuda"):
    """Replicas only: every rank ran `flops_per_step` per step; the job's
    step time is the slowest rank's (max over ranks), and the whole-job
    throughput counts the work of all ranks.  Returns (t_step, t_e2e_step,
    value, e2e) with the throughputs in TFLOP/s."""
    world = 1
    if dist is not None:
        import torch

        world = dist.get_world_size()
        tt = torch.tensor([t_step, t_e2e_step], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step, t_e2e_step = tt.tolist()
    return t_step, t_e2e_step, world * flops_per_step / t_step / 1e12, world * flops_per_step / t_e2e_step / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.strip().split(", ") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(rows), "reasons": sorted(reasons)}


def fp64_peak_tflops():
    """cuBLAS DGEMM throughput on this GPU (denominator of the FP64 roofline)."""
    try:
        import torch

        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = 1e30
        for _ in range(3):
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    except Exception:
        return None


# DRAM bytes (read + write) of the two tensor-core sigma kernels per product,
# from ncu captures of this bench's workloads (profiles/tc_sigma_*.md), made
# before the stage-1 products of small blocks were stacked (at M=2000 the
# stacks replace 37 % of the phase-1 tiles, all of small blocks; the
# operands they read are the same bytes)
NCU_TRAFFIC = {("tests/golden/syn24/dmrg.conf", 11, "bf16x3tc"): 3.275e9,
               ("tests/golden/syn30/dmrg.conf", 14, "bf16x3tc"): 244.19e9}
NCU_TRAFFIC_NOTE = "ncu capture before stacked stage-1 tiles (profiles/tc_sigma_bf16x3tc_syn30_m2000.md)"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build()
    return pyoracle


def cpu_sample(conf, partition, reps):
    """The oracle's sigma (OpenMP over operator pairs with a tuned DGEMM, as
    the reference links one) on a superblock with the benchmark's sectors,
    catalogue and pair list and seeded random operator values: sigma's cost
    does not depend on the values, and skipping the warm-up arithmetic keeps
    the sample to about one product's worth of CPU time."""
    po = oracle()
    blas = po.enable_blas()
    r = po.sample_sigma(conf, partition, threads=0, reps=reps)
    r["dgemm"] = blas
    return r


def conf_M(conf):
    with open(conf) as f:
        lines = [l.split() for l in f if l.strip()]
    for i, t in enumerate(lines):
        if t[0].lower() == "schedule" and i + 1 < len(lines):
            return int(lines[i + 1][1])
    return None


def conf_model(conf):
    """(norb, nelec, nchol, seed, group) of a dmrg.conf whose orbitals line
    names a generated Hamiltonian, else None."""
    for line in open(conf):
        t = line.split()
        if len(t) >= 2 and t[0] == "orbitals" and t[1].startswith("synthetic:"):
            f = t[1].split(":")
            return int(f[1]), int(f[2]), int(f[3]), int(f[4]), ("D2h" if len(f) > 5 and f[5] == "1" else "C1")
    return None


def config_dict(conf, partition, n, prec, arena_mb):
    M = conf_M(conf)
    model = conf_model(conf)
    if model:
        norb, nelec, nchol, seed, grp = model
        what = ("the synthetic %d-orbital/%d-electron Cholesky Hamiltonian (%d vectors, seed %d, S=0, %s)"
                % (norb, nelec, nchol, seed, grp))
    else:
        norb = nelec = None
        what = "the Hamiltonian of %s" % os.path.relpath(conf, ROOT)
    return {"workload": "sigma = H psi at the middle bond (L=[0..%d]) of %s, blocks renormalised to M=%s"
                        % (partition, what, M),
            "conf": os.path.relpath(conf, ROOT), "norb": norb, "nelec": nelec, "M": M, "partition": partition,
            "psi_elems": n, "precision": prec,
            "l2": "inputs larger than L2: operator arenas %.0f MB per step" % arena_mb}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    r = cpu_sample(a.conf, a.partition, max(1, min(a.steps, 2)))
    v = r["flops"] / r["seconds"] / 1e12
    sample = ("%d sigma product(s) on a superblock with the benchmark's sectors, operator catalogue and pair list "
              "and seeded random operator values (CPU oracle, OpenMP over operator pairs, per-thread sigma copies)"
              % max(1, min(a.steps, 2)))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": r["seconds"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(a.conf, a.partition, r["psi"], "fp64", 8.0 * r["arena"] / 1e6),
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": r["threads"] or threads, "kind": "port",
                             "sample": sample, "dgemm": r["dgemm"]},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def sweep_entry(ctx, conf, st, seconds, e):
    out = {"seconds": seconds, "energies": [float(x) for x in e], "sweeps": st["sweeps"],
           "sweep_energies": [float(x) for x in st["sweep_energies"]],
           "sigma_calls": st["sigma_calls"], "sigma_seconds": st["sigma_seconds"],
           "split_sigma_calls": st["split_sigma_calls"], "split_sigma_seconds": st["split_sigma_seconds"],
           "fp64_sigma_calls": st["fp64_sigma_calls"], "fp64_sigma_seconds": st["fp64_sigma_seconds"],
           "defect_rounds": st["defect_rounds"], "discarded": st["discarded"],
           "warmup_seconds": st["warmup_seconds"], "sweep_seconds": [float(t) for t in st["sweep_seconds"]],
           "phase_seconds": {k: st[k] for k in ("build_seconds", "solve_seconds", "density_seconds", "renorm_seconds")}}
    return out


def run_sweep(ctx, conf, prec):
    ctx.set_precision(prec)
    t0 = time.perf_counter()
    e, st = ctx.run_dmrg(conf)
    return sweep_entry(ctx, conf, st, time.perf_counter() - t0, e), st


def run_ours(a):
    import numpy as np

    import block_gb300

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    ctx = block_gb300.Context(local)
    ctx.set_precision(a.precision)
    tc_path = a.precision in ("bf16x3tc", "fp16x2tc")
    split = a.precision != "fp64"
    if tc_path and not a.no_autotune:
        # schedule knobs chosen by timing candidates on the first product
        # (untimed warm-up), keyed on the sector-size histogram
        ctx.set_autotune(True)
    t_prep = time.perf_counter()
    sb, n = ctx.prepare_superblock(a.conf, a.partition)
    t_prep = time.perf_counter() - t_prep
    flops, nbytes = ctx.superblock_work(sb)
    launches = ctx.superblock_launches(sb)
    rng = np.random.default_rng(1234)
    psi = rng.standard_normal(n)
    psi /= np.linalg.norm(psi)
    x = ctx.device_alloc(n)
    y = ctx.device_alloc(n)
    ctx.to_device(x, psi)
    ctx.sigma_timed(sb, x, y, max(3, a.warmup))
    if dist:
        dist.barrier()
    ctx.synchronize()
    # end-to-end host buffers: page-locked ones from the library
    # (bgpu_host_alloc), as a caller keeping its wavefunctions there would;
    # ordinary arrays if they cannot be had
    try:
        h_in, h_out = ctx.host_array(n), ctx.host_array(n)
        h_in[:] = psi
        host_buffers = "page-locked (bgpu_host_alloc)"
    except Exception:
        h_in, h_out, host_buffers = psi, np.empty(n), "pageable"
    ctx.sigma(sb, h_in, out=h_out)  # untimed: first use of the buffers
    with ClockSampler(local) as clk:
        if a.profile:
            ctx.profiler_start()
        ms = ctx.sigma_timed(sb, x, y, a.steps)
        if a.profile:
            ctx.profiler_stop()
        # end-to-end through the host-buffer C ABI call (H2D psi, D2H sigma per step)
        t0 = time.perf_counter()
        for _ in range(a.steps):
            ctx.sigma(sb, h_in, out=h_out)
        t_e2e = time.perf_counter() - t0
    ctx.synchronize()
    if host_buffers != "pageable":
        ctx.host_free(h_in)
        ctx.host_free(h_out)
    clocks = clk.summary()
    t_step = ms[0] / a.steps * 1e-3
    t_step, t_e2e_step, value, e2e = whole_job(flops, t_step, t_e2e / a.steps, dist)
    kern_ms = (ms[1] if split else ms[1] + ms[2]) / a.steps
    achieved = flops / (kern_ms * 1e-3) / 1e12
    peaks = measured_peaks()
    fp64 = fp64_peak_tflops()
    if not split:
        roof = {"bound": "tensor", "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
                "frac": (achieved / fp64) if fp64 else None, "traffic": None,
                "kernel": "gemm_fp64_kernel (sigma stages 1+2)",
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 has no entry in MEASURED_PEAKS.json)",
                "frac_of_bf16_measured": achieved / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                "algorithmic_bytes_per_step": nbytes}
    else:
        pk = peaks.get("bf16_tflops", 1900.0)
        prods = {"bf16x6": 6, "exacttc": 21}.get(a.precision, 3)
        kname = ("tc_sigma_kernel<1>+<2> (tcgen05/TMEM two-phase sector GEMMs, bf16 slices)" if tc_path else
                 "tcx_sigma_kernel<1>+<2> (tcgen05/TMEM exact-slice sector GEMMs, 6 bf16 digits, FP64 sums)"
                 if a.precision == "exacttc" else "fused_sigma_kernel (two-stage sector GEMMs, bf16 slices)")
        traffic = NCU_TRAFFIC.get((os.path.relpath(a.conf, ROOT), a.partition, a.precision))
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk, "unit": "TFLOP/s", "frac": achieved / pk,
                "traffic": traffic, "traffic_unit": "bytes per sigma (both tensor-core kernels, ncu)",
                "traffic_source": NCU_TRAFFIC_NOTE if traffic else None,
                "hbm_time_of_traffic_ms": (traffic / (peaks.get("hbm_gbs", 6800.0) * 1e9) * 1e3) if traffic else None,
                "kernel": kname,
                "peak_source": ("bf16_tflops of measured" if peaks else "fallback 1900"),
                "products_per_logical_product": prods,
                "tensor_issued_tflops": prods * achieved, "tensor_issued_frac": prods * achieved / pk,
                "note_issued": "bf16 products per logical FP64 product, without tile padding",
                "fp64_peak_tflops_in_run": fp64, "algorithmic_bytes_per_step": nbytes}
    if tc_path:
        info = ctx.superblock_info(sb)
        roof["tc_mma_issued_tflops"] = info["tc_mma_flops"] / (kern_ms * 1e-3) / 1e12
        roof["tc_mma_issued_frac"] = roof["tc_mma_issued_tflops"] / roof["peak"]
        roof["tc_plan"] = {k: v for k, v in info.items() if k.startswith("tc_")}
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp16x2tc": "fp16 slices, f32 accumulate",
                      "exacttc": "bf16 digit slices, exact f32 accumulate, f64 sums"}.get(a.precision,
                                                                                          "bf16 slices, f32 accumulate"),
            "data": "synthetic",
            "config": config_dict(a.conf, a.partition, n, a.precision, nbytes / 1e6),
            "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                    "host_buffers": host_buffers},
            "gpu_launches": launches * a.steps, "clocks": clocks, "roofline": roof,
            "sigma_flops_per_step": flops, "kernel_ms_per_step": [ms[1] / a.steps, ms[2] / a.steps],
            "prepare_seconds": t_prep}
    if tc_path and not a.no_schedules:
        # one persistent launch per phase against the per-sector-launch
        # baseline (one launch per sector, one block per tile), and the
        # autotuned knobs against the defaults
        sched = {"autotuned": not a.no_autotune,
                 "knobs": {k: info[k] for k in ("tc_item_cost", "tc_split", "tc_group", "tc_nb")},
                 "launches_per_sigma": info["launches"], "ms_per_sigma": t_step * 1e3,
                 "stacks": {k: info[k] for k in ("tc_stacks", "tc_stacked_items", "tc_phase1_tasks")}}
        reps = 2
        ctx.set_autotune(False)
        ctx.set_tc_schedule(True)
        ms_ps = ctx.sigma_timed(sb, x, y, reps)
        sched["per_sector"] = {"ms_per_sigma": ms_ps[0] / reps,
                               "launches_per_sigma": ctx.superblock_info(sb)["launches"],
                               "slowdown_vs_persistent": (ms_ps[0] / reps) / (t_step * 1e3)}
        ctx.set_tc_schedule(False)
        ms_d = ctx.sigma_timed(sb, x, y, reps)
        info_d = ctx.superblock_info(sb)
        sched["default_knobs"] = {"ms_per_sigma": ms_d[0] / reps,
                                  "knobs": {k: info_d[k] for k in ("tc_item_cost", "tc_split", "tc_group", "tc_nb")}}
        # stage-1 products of small blocks one tile each (no stacking)
        ctx.set_tc_stacking(0)
        ms_u = ctx.sigma_timed(sb, x, y, reps)
        sched["unstacked"] = {"ms_per_sigma": ms_u[0] / reps,
                              "phase1_tasks": ctx.superblock_info(sb)["tc_phase1_tasks"]}
        ctx.set_tc_stacking(64)
        if not a.no_autotune:
            ctx.set_autotune(True)
            ctx.sigma_timed(sb, x, y, 1)  # cached knobs back on the plan
            tuned, cached, secs = ctx.autotune_stats()
            sched["tuning"] = {"histograms_tuned": tuned, "seconds": secs}
        line["schedules"] = sched
    ms64 = None
    ref64 = None
    if split:
        # plain FP64 path on the same superblock and input: one device-timed
        # product, whose result is also the reference for the split error
        sp = ctx.to_host(y, n)  # the split product of the timed steps
        ctx.set_precision("fp64")
        y64 = ctx.device_alloc(n)
        ms64 = ctx.sigma_timed(sb, x, y64, 1)[0]
        ref64 = ctx.to_host(y64, n)
        ctx.device_free(y64)
        ctx.set_precision(a.precision)
        line["fp64_path"] = {"ms_per_step": ms64, "tflops": flops / (ms64 * 1e-3) / 1e12,
                             "speedup_of_split": ms64 / (t_step * 1e3),
                             "split_sigma_rel_err": float(np.linalg.norm(sp - ref64) / np.linalg.norm(ref64))}
    if split and ref64 is not None and not a.no_exact and a.precision != "exacttc":
        # the exact-slice tensor-core product (FP64-level, the restart
        # products of defect correction) on the same superblock and input
        ctx.set_precision("exacttc")
        yx = ctx.device_alloc(n)
        msx = ctx.sigma_timed(sb, x, yx, 2)[0] / 2
        px = ctx.to_host(yx, n)
        ctx.device_free(yx)
        ctx.set_precision(a.precision)
        ctx.sigma_timed(sb, x, y, 1)  # back to the split pools (frees the exact ones)
        line["exact_path"] = {"ms_per_step": msx, "tflops": flops / (msx * 1e-3) / 1e12,
                              "speedup_vs_fp64": ms64 / msx,
                              "sigma_rel_err_vs_fp64": float(np.linalg.norm(px - ref64) / np.linalg.norm(ref64)),
                              "products_per_logical_product": 21}
    if not a.no_davidson:
        # Davidson solve of the superblock (tol 1e-8 on the squared residual,
        # as in the schedule); split precision with defect correction against
        # FP64 residuals
        dv = {}
        runs = [(a.precision, "defect")] + ([(a.precision, "exact")] if split and a.precision != "exacttc" else []) + \
               ([("fp64", "defect")] if split and a.fp64_davidson else [])
        for prec, refine in runs:
            ctx.set_precision(prec)
            ctx.set_refinement(refine)
            r0, f0, _ = ctx.refinement_stats()
            t0 = time.perf_counter()
            e, _, it = ctx.davidson(sb, n, nroots=1, tol=1e-8)
            r1, f1, ver = ctx.refinement_stats()
            key = prec if refine == "defect" else prec + "+exact_restarts"
            dv[key] = {"seconds": time.perf_counter() - t0, "iterations": it, "energy": float(e[0]),
                       "graph_launches": ctx.davidson_graph_launches()}
            if prec != "fp64":
                dv[key].update(defect_rounds=r1 - r0, restart_products=f1 - f0, fp64_residual_verified=bool(ver),
                               verified_on=["none", "fp64 residuals", "fp64 residual bounds"][ver],
                               restart_products_on="tensor cores, exact slices" if refine == "exact" else "FP64 pipe")
        ctx.set_refinement("defect")
        ctx.set_precision(a.precision)
        if split and ms64 is not None:
            if "fp64" in dv:
                dv["dE_split_minus_fp64"] = dv[a.precision]["energy"] - dv["fp64"]["energy"]
                dv["speedup"] = dv["fp64"]["seconds"] / dv[a.precision]["seconds"]
            else:
                # the FP64 solve takes about as many products as the split
                # one; its time is derived from the measured FP64 product
                prods = dv[a.precision]["iterations"] + dv[a.precision]["restart_products"]
                dv["fp64_derived_seconds"] = prods * ms64 * 1e-3
                dv["speedup_vs_derived_fp64"] = dv["fp64_derived_seconds"] / dv[a.precision]["seconds"]
        line["davidson"] = dv
    if rank == 0 and not a.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r = cpu_sample(a.conf, a.partition, a.cpu_reps)
        line["cpu_baseline"] = {"value": r["flops"] / r["seconds"] / 1e12, "unit": "TFLOP/s",
                                "cores": r["threads"] or threads, "kind": "port",
                                "sample": "%d sigma product(s) on a superblock with the benchmark's sectors, "
                                          "operator catalogue and pair list and seeded random operator values "
                                          "(CPU oracle, OpenMP over operator pairs, per-thread sigma copies)"
                                          % a.cpu_reps,
                                "dgemm": r["dgemm"],
                                "flops_match_gpu_plan": bool(abs(r["flops"] - flops) <= 1e-9 * flops)}
    if rank == 0 and not a.no_parity:
        # FP64 parity of the GPU sigma with the oracle's on the same inputs
        # (the oracle builds its own 24-orbital M=500 superblock)
        po = oracle()
        po.enable_blas()
        snap = po.prepare(PARITY_CONF, PARITY_PARTITION, threads=0, reps=1)
        # FP64 run: the warm-up's renormalisations on the FP64 pipe, as the
        # oracle's (split-precision runs renormalise with exact slices)
        ctx.set_precision("fp64")
        sb2, n2 = ctx.prepare_superblock(PARITY_CONF, PARITY_PARTITION)
        err = float(np.linalg.norm(ctx.sigma(sb2, snap["psi"]) - snap["sigma"]) / np.linalg.norm(snap["sigma"]))
        ctx.set_precision(a.precision)
        err_s = float(np.linalg.norm(ctx.sigma(sb2, snap["psi"]) - snap["sigma"]) / np.linalg.norm(snap["sigma"]))
        line["parity"] = {"conf": os.path.relpath(PARITY_CONF, ROOT), "partition": PARITY_PARTITION, "psi_elems": n2,
                          "fp64_sigma_rel_err_vs_oracle": err, "split_sigma_rel_err_vs_oracle": err_s}
    if rank == 0 and not a.no_sweeps:
        ctx.set_autotune(False)  # sweeps with the default schedule knobs, as bgpu_run_dmrg runs them
        sweeps = {}
        # small system: GPU FP64 and split precision beside the CPU oracle
        sw = {"conf": os.path.relpath(a.sweep_conf, ROOT)}
        wanted = [p.strip() for p in a.sweep_precisions.split(",") if p.strip()]
        for prec in dict.fromkeys({"split": a.precision}.get(p, p) for p in wanted):
            sw[prec], _ = run_sweep(ctx, a.sweep_conf, prec)
        if "fp64" in sw and a.precision in sw and a.precision != "fp64":
            sw["dE_split_minus_fp64"] = sw[a.precision]["energies"][0] - sw["fp64"]["energies"][0]
            sw["dE_per_sweep_split_minus_fp64"] = [s - f for s, f in zip(sw[a.precision]["sweep_energies"],
                                                                         sw["fp64"]["sweep_energies"])]
        if not a.no_cpu_baseline and "fp64" in sw:
            po = oracle()
            po.enable_blas()
            t0 = time.perf_counter()
            # transformed guesses, as the GPU sweeps (the reference's default)
            e, st = po.run(a.sweep_conf, guess=True)
            sw["cpu_oracle"] = {"seconds": time.perf_counter() - t0, "energies": [float(v) for v in e],
                                "sweep_energies": [float(v) for v in st["sweep_energies"]],
                                "sweeps": st["sweeps"], "cores": os.cpu_count() or 1,
                                "sigma_calls": st["sigma_calls"], "guess": "transformed"}
            sw["dE_fp64_minus_cpu"] = sw["fp64"]["energies"][0] - sw["cpu_oracle"]["energies"][0]
            sw["dE_per_sweep_fp64_minus_cpu"] = [g - c for g, c in zip(sw["fp64"]["sweep_energies"],
                                                                       sw["cpu_oracle"]["sweep_energies"])]
        sweeps["small"] = sw
        # large system: split precision with defect correction; its FP64
        # sweep time is derived from the per-step FP64 product times unless
        # --sweep-fp64 measures it
        if split and a.big_sweep_conf != "none":
            # a fresh context: the large sweep's blocks and pools get the
            # whole device, not what the superblocks measured above left
            ctx.device_free(x)
            ctx.device_free(y)
            ctx.close()
            ctx = block_gb300.Context(local)
            x = ctx.device_alloc(1)
            y = ctx.device_alloc(1)
            bw = {"conf": os.path.relpath(a.big_sweep_conf, ROOT)}
            bw[a.precision], st = run_sweep(ctx, a.big_sweep_conf, a.precision)
            s = bw[a.precision]
            sweep_s = sum(s["sweep_seconds"])
            # renormalisation on the FP64 pipe at the FP64 product rate
            # measured in the same run, in place of the exact-slice one
            # the FP64 path at the FP64 rate measured on the bench superblock
            # (the largest products; smaller ones run below it, so this
            # underestimates the FP64 sweep)
            r64 = flops / (ms64 * 1e-3) if ms64 else (st["fp64_rate"] or None)
            sigma64 = st["sigma_flops"] / r64 if r64 else st["derived_fp64_sigma_seconds"]
            exact_r = st["renorm_exact"] and r64
            renorm64 = st["sweep_renorm_flops"] / r64 if exact_r else 0.0
            renorm_x = st["sweep_renorm_device_seconds"] if exact_r else 0.0
            derived = sweep_s - s["sigma_seconds"] + sigma64 - renorm_x + renorm64
            bw["sweep_seconds"] = sweep_s
            bw["fp64_derived_sweep_seconds"] = derived
            bw["fp64_derived_renorm_seconds"] = renorm64
            bw["fp64_derived_sigma_seconds"] = sigma64
            bw["fp64_derived_note"] = ("the split sweep's wall time (warm-up excluded) with its sigma time (split, "
                                       "exact and FP64 products) and its exact-slice renormalisation device time "
                                       "replaced by their flops at the FP64 rate measured on the bench superblock "
                                       "(fp64_path): a lower bound of the FP64 sweep")
            bw["speedup_vs_derived_fp64"] = derived / sweep_s
            if a.sweep_fp64:
                bw["fp64"], _ = run_sweep(ctx, a.big_sweep_conf, "fp64")
                bw["speedup"] = sum(bw["fp64"]["sweep_seconds"]) / sweep_s
                bw["dE_per_sweep_split_minus_fp64"] = [x - y for x, y in zip(s["sweep_energies"],
                                                                            bw["fp64"]["sweep_energies"])]
            sweeps["large"] = bw
        ctx.set_precision(a.precision)
        line["sweeps"] = sweeps
    ctx.device_free(x)
    ctx.device_free(y)
    ctx.close()
    if tc_path and world == 1 and not a.no_batching and not a.no_schedules and \
            os.path.abspath(a.conf) == os.path.abspath(DEFAULT_CONF):
        line["batching"] = run_batching(a)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_batching(a):
    """The sigma measurement of this script on the batching superblock, in a
    child process that gets the whole device (the headline superblock's
    context is closed by then); returns its schedules and timings."""
    cmd = [sys.executable, os.path.abspath(__file__), "--conf", BATCH_CONF, "--partition", str(BATCH_PARTITION),
           "--precision", a.precision, "--steps", "10", "--warmup", "3", "--no-cpu-baseline", "--no-parity",
           "--no-davidson", "--no-sweeps", "--no-exact", "--big-sweep-conf", "none", "--no-batching"]
    t0 = time.perf_counter()
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        rec = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    except Exception as e:  # the headline line stands without this entry
        return {"conf": os.path.relpath(BATCH_CONF, ROOT), "error": repr(e)[:300]}
    info = rec["roofline"].get("tc_plan", {})
    return {"conf": os.path.relpath(BATCH_CONF, ROOT), "partition": BATCH_PARTITION,
            "workload": rec["config"]["workload"], "psi_elems": rec["config"]["psi_elems"],
            "sigma_flops_per_step": rec["sigma_flops_per_step"], "ms_per_sigma": rec["ms_per_step"],
            "tflops": rec["value"], "e2e_tflops": rec["e2e"]["value"], "clocks": rec["clocks"],
            "tc_mma_flops": info.get("tc_mma_flops"), "tc_mma_issued_frac": rec["roofline"].get("tc_mma_issued_frac"),
            "schedules": rec.get("schedules"), "fp64_path": rec.get("fp64_path"),
            "prepare_seconds": rec.get("prepare_seconds"), "seconds": time.perf_counter() - t0}


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
