"""Benchmark: mixed-precision FMM-BEM matvec on the 81,920-triangle sphere (8 kHz).

Workload (the mixed-precision-vs-FP64 configuration): rigid sphere r = 0.3 m meshed as an
icosphere with 6 subdivisions (81,920 flat triangles), k = 2 pi 8000/343 (ka = 44), octree
depth 6, truncation p = 40/30/20/14/10 at levels 2..6, the reference's 3x3 collapsed Gauss
rule, operator (1/2) I - M of the exterior Neumann problem, input densities with real and
imaginary parts i.i.d. N(0,1) from seed 0 (synthetic data; the reference publishes no
dataset or numbers).

A step is one matvec.  ``value`` is matvec/s of the mixed-precision path with inputs
resident in HBM, timed with CUDA events on the plan's stream around each step, with L2
flushed between steps (a 512 MiB write).  ``e2e`` is the same metric through the public
C ABI with host buffers (H2D of x and D2H of y inside the timed region).  Also reported:
FP64-plain matvec/s, the mixed-vs-FP64 relative error, and an IR-GMRES solve of the
plane-wave problem to 1e-6 in both precisions.

``--impl reference`` times the CPU restatement of the reference algorithm (the oracle port,
FP64, all host cores) on the same workload.
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

SUBDIV, RADIUS, FREQ, DEPTH = 6, 0.3, 8000.0, 6
P_LEVELS = {2: 40, 3: 30, 4: 20, 5: 14, 6: 10}
METRIC = "solve s & matvec/s, mixed-prec batched vs FP64 plain at 1e-5 rel err, 1 GB300"
UNIT = "matvec/s"
# FP32 SIMT nominal of a GB300: 152 SMs x 128 FMA lanes x 2 flops x 2.07 GHz
FP32_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12


def f_rcr(p):
    """Algorithmic flops of one RCR translation at order p (8 flops per complex MAC)."""
    return 8.0 * (10.0 * p ** 3 - p) / 3.0


def workload_config(extra=None):
    cfg = {"workload": "rigid sphere r=0.3 m, icosphere-6 (81920 tri), 8 kHz (ka=44), depth 6, "
                       "p=40/30/20/14/10, 3x3 collapsed Gauss, operator I/2 - M, N(0,1) densities seed 0",
           "num_elements": 81920, "depth": DEPTH, "p_levels": [P_LEVELS[l] for l in range(2, 7)],
           "l2_flush_between_steps": True}
    if extra:
        cfg.update(extra)
    return cfg


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        # the raw samples go to FMMBEM_CLOCKS_DIR (default: the system's temporary directory)
        out = os.environ.get("FMMBEM_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, "fmmbem_clocks_rank%d_%d.csv" % (gpu, os.getpid()))

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes of the translation passes per matvec (all launches of rcr_tile_kernel and
    tc_dense_kernel) from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "translation_passes_traffic_cfg2.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_matvec:"):
            try:
                return float(line.split(":")[1].split()[0])
            except ValueError:
                return None
    return None


def make_mesh(fm):
    return fm.icosphere(SUBDIV, RADIUS)


def cpu_mesh():
    """The same icosphere as fm.icosphere (vertices rounded to 9 significant digits), built in
    NumPy so that the CPU arm loads no library of this package."""
    import meshes
    return meshes.roundtrip(*meshes.icosphere(SUBDIV, RADIUS))


# Leaf-level boxes on which the octree port runs FMMLevelSetNumSR (every k-th box; the
# coarser levels run in full); its time is scaled to all boxes of the level.
OCTREE_SR_SAMPLE = 4096


def cpu_baseline_sample(steps=None, warmup=0):
    """The CPU baseline on the machine's host cores: the reference's CPU path as far as it exists
    (its octree build) plus a CPU matvec.  The reference's own sources are not on this machine,
    so both are ports (test infrastructure under oracle/):

    * matvec: the FP64 CPU restatement of the FMM (oracle/fmm_oracle.c) on all host cores
      (bounded to ~10 s, or `steps` matvecs after `warmup`), and one matvec on one core;
    * octree: oracle/octree_port.c, srcBoxes (fixed depth) + FMMLevelSet + FMMLevelSetNumSR
      with the reference's own quadratic set algebra, on one core (the reference is serial),
      FMMLevelSetNumSR of the leaf level on a strided sample of boxes, scaled.

    Returns the cpu_baseline dict (value = all-cores matvec/s) and the all-cores time per
    matvec."""
    from oracle import oracle_py as O
    V, F = cpu_mesh()
    k = 2 * np.pi * FREQ / 343.0
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    T = O.tree_for_fmm(V, F, depth=DEPTH)
    f = O.FMM(V, F, k, T, [P_LEVELS[l] for l in range(2, 7)], a=0.5, b=0.0, c=-1.0, rule=0, nthreads=cores)
    fmm_setup = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    x = rng.standard_normal(len(F)) + 1j * rng.standard_normal(len(F))
    for _ in range(max(warmup, 1)):
        f.apply(x)
    n, t0 = 0, time.perf_counter()
    if steps:
        for _ in range(steps):
            f.apply(x)
        n = steps
    else:
        while time.perf_counter() - t0 < 10.0 and n < 50:
            f.apply(x)
            n += 1
    dt = time.perf_counter() - t0
    del f
    f1 = O.FMM(V, F, k, T, [P_LEVELS[l] for l in range(2, 7)], a=0.5, b=0.0, c=-1.0, rule=0, nthreads=1)
    t1 = time.perf_counter()
    f1.apply(x)
    dt1 = time.perf_counter() - t1
    del f1
    oc = O.port_octree(V, F, depth=DEPTH, sr_sample=OCTREE_SR_SAMPLE)
    ot = oc["times"]
    octree_s = ot["src_boxes_s"] + ot["level_sets_s"] + ot["sr_lists_s"]
    leaf_ran = int((oc["srnum_%d" % DEPTH] >= 0).sum())
    base = {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "full workload, %d FP64 matvecs of the CPU restatement (oracle) on %d threads in %.1f s"
                      % (n, cores, dt),
            "single_thread": {"value": 1.0 / dt1, "unit": UNIT, "cores": 1,
                              "sample": "one FP64 matvec of the CPU restatement on 1 thread in %.1f s" % dt1},
            "octree_build_s": octree_s,
            "octree_build": {"cores": 1, "kind": "port", "lmax": oc["lmax"],
                             "src_boxes_s": ot["src_boxes_s"], "level_sets_s": ot["level_sets_s"],
                             "sr_lists_s": ot["sr_lists_s"], "sr_lists_s_run": ot["sr_lists_s_run"],
                             "sample": "srcBoxes (depth %d) + FMMLevelSet + FMMLevelSetNumSR with the reference's "
                                       "quadratic set algebra (oracle/octree_port.c); FMMLevelSetNumSR on levels 2-%d in "
                                       "full and on %d of %d level-%d boxes (every k-th), scaled"
                                       % (DEPTH, DEPTH - 1, leaf_ran, len(oc["set_%d" % DEPTH]), DEPTH)},
            "fmm_setup_s": fmm_setup}
    return base, dt / n


def cpu_reference_arm(args, world, rank):
    """--impl reference: the reference's CPU path on the machine's host cores (see
    cpu_baseline_sample); `value` is the all-cores CPU matvec rate, steps and warm-up as given.
    Loads no library of this package: the mesh is built in NumPy, and only oracle/ runs."""
    if rank != 0:
        return
    base, t_step = cpu_baseline_sample(steps=args.steps, warmup=args.warmup)
    v = base["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic", "config": workload_config(),
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def gpu_arm(args, world, rank, local):
    import torch
    import fmbem_gpu_c_gb300 as fm

    torch.cuda.set_device(local)
    V, F = make_mesh(fm)
    k = 2 * np.pi * FREQ / 343.0
    t0 = time.perf_counter()
    plan = fm.Plan(V, F, k=k, depth=DEPTH, p_levels=P_LEVELS, rule=fm.RULE_GAUSS3, a=0.5, b=0.0, c=-1.0,
                   device=local)
    setup_s = time.perf_counter() - t0
    info = plan.info
    nf = plan.nf
    rng = np.random.default_rng(rank)
    xh = rng.standard_normal(nf) + 1j * rng.standard_normal(nf)
    x = torch.from_numpy(xh).to("cuda")
    y = torch.empty_like(x)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # warm-up
    for _ in range(args.warmup):
        plan.matvec(x, fm.FMM_MIXED, out=y)
    torch.cuda.synchronize()

    # timed mixed-precision steps: the plan's whole-matvec CUDA events on its own stream
    # (profiling mode 2 keeps the translation passes on their replayed CUDA graph)
    plan.set_profiling(2)
    step_ms = []
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            plan.matvec(x, fm.FMM_MIXED, out=y)
            step_ms.append(dict(plan.timings())["matvec"])
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    barrier(world)
    t_step = max_over_ranks(world, float(np.mean(step_ms)) / 1e3)
    value = world / t_step

    # per-kernel split, outside the timed region: per-pass timers (direct launches)
    plan.set_profiling(1)
    kernel_ms = {}
    for _ in range(min(args.steps, 5)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        plan.matvec(x, fm.FMM_MIXED, out=y)
        tm = plan.timings()
        for name, ms in tm:
            if name != "matvec":
                kernel_ms.setdefault(name, []).append(ms)
    plan.set_profiling(False)
    launches_per_step = len(tm) - 2  # kernel timers (less the "translations" and "matvec" spans)

    # dominant kernel: the batched RCR translations (rcr_tile_kernel: M2M, M2L, L2L at every
    # level); algorithmic flops = one RCR at the pass's order per translation
    m2l_flops = sum(info.num_m2l[l] * f_rcr(info.p_level[l]) for l in range(info.lmin, info.lmax + 1))
    l2l_flops = sum(info.num_box[l] * f_rcr(info.p_level[l - 1]) for l in range(info.lmin + 1, info.lmax + 1))
    m2m_flops = l2l_flops
    rcr_flops = m2l_flops + l2l_flops + m2m_flops
    rcr_ms = float(np.mean(kernel_ms["translations"]))  # the M2M/M2L/L2L phase as a whole
    bf16_peak, hbm_peak, peak_kind = peaks()
    achieved_tflops = rcr_flops / (rcr_ms / 1e3) / 1e12
    # the M2L levels on the tensor cores (tc_dense_kernel): split-TF32 GEMMs over dense operators,
    # 3 MMAs of 128 x Nmma x 8 per 8 of K for every 128 translations and output half
    tc_levels = [l for l in range(info.lmin, info.lmax + 1) if info.m2l_tensor[l]]
    tc = None
    if tc_levels:
        ex = 0.0
        for l in tc_levels:
            p = info.p_level[l]
            nhalf = 1
            while True:
                ch = -(-p * p // nhalf)
                nmma = (2 * ch + 15) // 16 * 16
                if nmma <= 256:
                    break
                nhalf += 1
            nch = -(-2 * p * p // 16)
            ex += info.num_m2l[l] * nhalf * nch * 16 * 6 * nmma
        tc_ms = sum(float(np.mean(kernel_ms["m2l_l%d" % l])) for l in tc_levels)
        tc_alg = sum(info.num_m2l[l] * f_rcr(info.p_level[l]) for l in tc_levels)
        tc = {"kernel": "tc_dense_kernel (tcgen05.mma kind::tf32, split TF32, TMEM accumulators)", "levels": tc_levels,
              "ms_per_matvec": tc_ms, "executed_tf32_flops": ex, "executed_tflops": ex / (tc_ms / 1e3) / 1e12,
              "tf32_peak_from_measured_bf16": bf16_peak / 2,
              "executed_frac_of_tf32": ex / (tc_ms / 1e3) / 1e12 / (bf16_peak / 2),
              "algorithmic_flops": tc_alg, "algorithmic_tflops": tc_alg / (tc_ms / 1e3) / 1e12,
              "note": "per-pass times from direct launches with the other levels' passes running beside them"}

    # FP64 plain path and accuracy
    plan.matvec(x, fm.FMM_FP64, out=y)
    torch.cuda.synchronize()
    t64 = []
    y64 = torch.empty_like(x)
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = time.perf_counter()
        plan.matvec(x, fm.FMM_FP64, out=y64)
        torch.cuda.synchronize()
        t64.append(time.perf_counter() - a)
    plan.matvec(x, fm.FMM_MIXED, out=y)
    torch.cuda.synchronize()
    rel_err = float((torch.linalg.norm(y - y64) / torch.linalg.norm(y64)).item())
    fp64_rate = 1.0 / float(np.median(t64))
    # the FP64-quality matvec the refined solvers use for residuals (translations in float-float)
    yff = torch.empty_like(x)
    plan.matvec(x, fm.FMM_FLOAT2, out=yff)
    torch.cuda.synchronize()
    tff = []
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = time.perf_counter()
        plan.matvec(x, fm.FMM_FLOAT2, out=yff)
        torch.cuda.synchronize()
        tff.append(time.perf_counter() - a)
    float2 = {"value": 1.0 / float(np.median(tff)), "unit": UNIT,
              "rel_err_vs_fp64": float((torch.linalg.norm(yff - y64) / torch.linalg.norm(y64)).item()),
              "note": "FMM_FLOAT2: M2M, M2L and L2L in float-float on the FP32 pipes, the rest FP64"}

    # batching path: NB columns in one mixed pass (device buffers), columns per second
    NB = 16
    xb = torch.from_numpy(np.concatenate([np.roll(xh, 7 * r) for r in range(NB)])).to("cuda")
    yb = torch.empty_like(xb)
    plan.matvec(xb, fm.FMM_MIXED, out=yb)
    torch.cuda.synchronize()
    plan.matvec(xb, fm.FMM_MIXED, out=yb)  # second call captures the graph for 16 columns
    plan.set_profiling(2)
    tb = []
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        plan.matvec(xb, fm.FMM_MIXED, out=yb)
        tb.append(dict(plan.timings())["matvec"])
    plan.set_profiling(False)
    y0 = yb[:nf]
    batched_err = float((torch.linalg.norm(y0 - y) / torch.linalg.norm(y)).item())
    batched = {"nrhs": NB, "value": NB / (float(np.mean(tb)) / 1e3), "unit": "matvec/s (columns)",
               "ms_per_batch": float(np.mean(tb)), "column0_vs_single_rel_err": batched_err}
    del xb, yb

    # end to end through the C ABI with host buffers
    yh = np.empty_like(xh)
    plan.matvec(xh, fm.FMM_MIXED, out=yh)
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = time.perf_counter()
        plan.matvec(xh, fm.FMM_MIXED, out=yh)
        e2e_t.append(time.perf_counter() - a)
    e2e_value = world / max_over_ranks(world, float(np.mean(e2e_t)))

    solve = None
    if args.solve:
        # Plane wave exp(ikz).  Both paths solve to a residual of 1e-7 (at ka = 44 the operator
        # is ill-conditioned enough that 1e-6 leaves ~2e-5 in the far field); the far fields
        # are compared with an FP64 reference solved to 1e-10 (FP64 residual, refinement).
        b = plan.plane_wave((0.0, 0.0, 1.0))
        tol = 1e-7
        a = time.perf_counter()
        x64, it64, rr64, ok64 = plan.gmres(b, tol=tol, restart=60, maxit=600, precision=fm.FMM_FP64)
        t_plain = time.perf_counter() - a
        a = time.perf_counter()
        xmx, itmx, rrmx, okmx = plan.gmres(b, tol=tol, restart=60, maxit=600, precision=fm.FMM_MIXED)
        t_mixed = time.perf_counter() - a
        xref, itr, rrr, okr = plan.gmres(b, x0=xmx, tol=1e-10, restart=60, maxit=600, precision=fm.FMM_MIXED)
        pts = fm.fibonacci_sphere(64, 2.0)
        ffr = plan.far_field(xref, pts)
        ff64 = plan.far_field(x64, pts)
        ffmx = plan.far_field(xmx, pts)
        nr = np.linalg.norm(ffr)
        solve = {"tol": tol, "plain_fp64_s": t_plain, "plain_iters": it64, "plain_relres": rr64,
                 "mixed_ir_s": t_mixed, "mixed_inner_iters": itmx, "mixed_relres": rrmx, "speedup": t_plain / t_mixed,
                 "far_field_rel_err_mixed": float(np.linalg.norm(ffmx - ffr) / nr),
                 "far_field_rel_err_plain": float(np.linalg.norm(ff64 - ffr) / nr),
                 "reference": "FP64-residual refinement to 1e-10 (%d inner iterations)" % itr}

    # the metric's batched configuration (64 right-hand sides on the 200,000-triangle body),
    # after the timed region and on its own clock record
    head64 = None if args.no_head64 else head64_run(local)

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        cpu, _ = cpu_baseline_sample()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 (FP32 translations and near field, FP64 input/output)", "data": "synthetic",
        "config": workload_config(),
        "run": {"setup_s": setup_s, "parallelism": "replicas" if world > 1 else "single", "wall_s_timed_region": wall},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nf * 16, "d2h_bytes_per_step": nf * 16},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "tensor",
                     "kernel": "translation passes: rcr_tile_kernel (M2M, L2L, M2L) + tc_dense_kernel (M2L at levels %s)"
                               % tc_levels,
                     "achieved": achieved_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": achieved_tflops / bf16_peak, "peak_source": peak_kind + " bf16 burst",
                     "fp32_simt_nominal_tflops": FP32_NOMINAL, "fp32_simt_frac": achieved_tflops / FP32_NOMINAL,
                     "traffic": ncu_traffic(), "algorithmic_flops_per_matvec": rcr_flops,
                     "ms_per_matvec": rcr_ms, "tensor_core_m2l": tc},
        "kernels_ms": {n: float(np.mean(v)) for n, v in kernel_ms.items()},
        "batched": batched,
        "fp64_plain": {"value": fp64_rate, "unit": UNIT, "mixed_speedup": value / world / fp64_rate,
                       "mixed_vs_fp64_rel_err": rel_err, "float2": float2},
        "solve": solve,
        "head64": head64,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    plan.close()


def head64_run(local):
    """The batched right-hand-side workload: a head-like body (ellipsoid 0.075/0.09/0.11 m with
    seeded degree-8 spherical-harmonic bumps of 1.5 mm, 200,000 triangles), 20 kHz, 64 plane
    waves on a Fibonacci sphere solved together (fmm_solve_batched, mixed precision with FP64
    refinement).  The plain FP64 path solves a subset of the columns (its cost per column does
    not depend on how many are solved together), scaled to 64.  Far-field errors at 32 points
    against an FP64 reference refined to 1e-10 from the mixed solution.  Returns the result
    dict (solve seconds; lower is better)."""
    import torch
    import fmbem_gpu_c_gb300 as fm
    torch.cuda.set_device(local)
    V, F = fm.ellipsoid(100, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=2026)
    k = 2 * np.pi * 20000.0 / 343.0
    t0 = time.perf_counter()
    # Burton-Miller coupling alpha = i/k: at ka ~ 37 the conventional equation I/2 - M sits
    # among interior eigenfrequencies of the body and GMRES stalls (relative residual 2.6e-4
    # after 400 iterations on one column); the combined equation converges in ~45
    plan = fm.Plan(V, F, k=k, depth=7, p_levels={2: 40, 3: 30, 4: 20, 5: 14, 6: 10, 7: 8}, rule=0, a=0.5, b=0.0,
                   c=-1.0, alpha=1j / k, device=local)
    setup_s = time.perf_counter() - t0
    dirs = fm.fibonacci_sphere(64, 1.0)
    B = np.stack([plan.plane_wave(d) for d in dirs])
    tol, nsub = 1e-6, 4
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        Xm, itm, rrm, okm = plan.solve_batched(B, tol=tol, restart=60, maxit=2000, precision=fm.FMM_MIXED)
        t_mixed = time.perf_counter() - t0
        t0 = time.perf_counter()
        Xp, itp, rrp, okp = plan.solve_batched(B[:nsub], tol=tol, restart=60, maxit=2000, precision=fm.FMM_FP64)
        t_plain_sub = time.perf_counter() - t0
    Xr, itr, rrr, okr = plan.solve_batched(B[:nsub], X0=Xm[:nsub], tol=1e-10, restart=60, maxit=2000,
                                           precision=fm.FMM_MIXED)
    pts = fm.fibonacci_sphere(32, 1.0)
    err_m, err_p = [], []
    for r in range(nsub):
        ref = plan.far_field(Xr[r], pts)
        nr = np.linalg.norm(ref)
        err_m.append(float(np.linalg.norm(plan.far_field(Xm[r], pts) - ref) / nr))
        err_p.append(float(np.linalg.norm(plan.far_field(Xp[r], pts) - ref) / nr))
    info = plan.info
    t_plain = t_plain_sub * 64 / nsub
    plan.close()
    return {
        "metric": "solve s, 64 plane waves, mixed-prec batched vs FP64 plain at 1e-5 rel far-field err, 1 GB300",
        "value": t_mixed, "unit": "s", "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
        "config": {"workload": "head-like bumped ellipsoid 0.075/0.09/0.11 m, 200,000 tri, 20 kHz (k = %.1f), "
                               "64 Fibonacci plane waves, depth 7, p = 40/30/20/14/10/8, Burton-Miller operator "
                               "(I/2 - M) - (i/k) N" % k,
                   "num_elements": len(F), "lmax": info.lmax, "tol": tol},
        "setup_s": setup_s,
        "mixed": {"solve_s": t_mixed, "converged": bool(okm), "iters_max": int(itm.max()),
                  "relres_max": float(rrm.max()), "far_field_rel_err_max": max(err_m),
                  "far_field_columns_checked": nsub},
        "plain_fp64": {"solve_s_extrapolated": t_plain, "columns_timed": nsub, "solve_s_timed": t_plain_sub,
                       "scaling": "x 64/%d (each column costs the same whether solved alone or together)" % nsub,
                       "converged": bool(okp), "iters_max": int(itp.max()), "far_field_rel_err_max": max(err_p)},
        "speedup": t_plain / t_mixed,
        "reference": "FP64-residual refinement to 1e-10 of %d columns (converged %s)" % (nsub, bool(okr)),
        "clocks": clk.summary(),
    }


def head64_arm(args, world, rank, local):
    line = head64_run(local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def vjp_arm(args, world, rank, local):
    """The adjoint workload: the head-like body (200,000 triangles) at 10 kHz with the admittance
    boundary dp/dn = i k beta p, beta = 0.1 + 0.05i, Burton-Miller operator; J = sum |p_scat|^2 at
    32 far points; one solve, one fmm_vjp (adjoint solve + all vertex derivative passes) and one
    fmm_vjp_admittance (the admittance derivative from the same adjoint solution), timed; the
    gradients checked against central differences (h = 1e-6 m on 20 seeded vertices; h = 1e-6
    in Re and Im beta) of the same pipeline on a 5,120-triangle copy of the body."""
    import torch
    import fmbem_gpu_c_gb300 as fm
    torch.cuda.set_device(local)
    k = 2 * np.pi * 10000.0 / 343.0
    beta = 0.1 + 0.05j
    alpha = 1j / k
    pts = fm.fibonacci_sphere(32, 1.0)
    d = (0.0, 0.0, 1.0)

    def opts(bt, depth, pl):
        b = 1j * k * bt
        return dict(k=k, depth=depth, p_levels=pl, rule=0, a=0.5 * (1 + alpha * b), b=b, c=-1.0, alpha=alpha)

    V, F = fm.ellipsoid(100, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=2026)
    pl_big = {2: 30, 3: 22, 4: 16, 5: 12, 6: 10, 7: 8}
    t0 = time.perf_counter()
    plan = fm.Plan(V, F, device=local, **opts(beta, 7, pl_big))
    setup_s = time.perf_counter() - t0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, it, rr, ok = plan.gmres(plan.plane_wave(d), tol=1e-8, maxit=3000, restart=100, precision=fm.FMM_MIXED)
        t_solve = time.perf_counter() - t0
        pf = plan.far_field(x, pts)
        t0 = time.perf_counter()
        grad, lam = plan.vjp(x, pts, pf, direction=d, tol=1e-8, precision=fm.FMM_MIXED)
        t_vjp = time.perf_counter() - t0
        t0 = time.perf_counter()
        g_beta, dj_beta = plan.vjp_admittance(x, pts, pf, lam)
        t_adm = time.perf_counter() - t0
    plan.close()

    # central differences on a 5,120-triangle copy (FP64 pipeline, tight tolerance)
    Vs, Fs = fm.ellipsoid(16, (0.075, 0.09, 0.11), lmax=8, sigma=1.5e-3, seed=2026)
    Vs = Vs + np.array([0.0031, -0.0017, 0.0023])
    pl_small = {2: 16, 3: 14, 4: 12}

    def J_of(Vx, bt=beta, want_grad=False):
        pl = fm.Plan(Vx, Fs, device=local, build_mixed=False, **opts(bt, 4, pl_small))
        xs, _, _, oks = pl.gmres(pl.plane_wave(d), tol=1e-12, maxit=4000, restart=120, precision=fm.FMM_FP64)
        p_ = pl.far_field(xs, pts)
        g_ = gb_ = None
        if want_grad:
            g_, lam_ = pl.vjp(xs, pts, p_, direction=d, tol=1e-12)
            gb_ = pl.vjp_admittance(xs, pts, p_, lam_)[1]
        pl.close()
        return float(np.sum(np.abs(p_) ** 2)), g_, gb_, oks

    J0, g0, gb0, ok0 = J_of(Vs, want_grad=True)
    rng = np.random.default_rng(5)
    h, worst = 1e-6, 0.0
    scale = float(np.abs(g0).max())
    nvert = 20
    for v in rng.choice(len(Vs), nvert, replace=False):
        e = rng.standard_normal(3)
        e /= np.linalg.norm(e)
        Vp, Vm = Vs.copy(), Vs.copy()
        Vp[v] += h * e
        Vm[v] -= h * e
        fd = (J_of(Vp)[0] - J_of(Vm)[0]) / (2 * h)
        worst = max(worst, abs(float(g0[v] @ e) - fd) / scale)
    fdb = [(J_of(Vs, beta + st)[0] - J_of(Vs, beta - st)[0]) / (2 * h) for st in (h, 1j * h)]
    worst_b = float(np.abs(np.array(fdb) - gb0).max() / np.abs(fdb).max())
    line = {
        "metric": "adjoint: vertex and admittance gradient of J = sum |p_scat|^2 (fmm_vjp + fmm_vjp_admittance), "
                  "s per gradient, 1 GB300",
        "value": t_vjp + t_adm, "unit": "s", "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
        "config": {"workload": "head-like bumped ellipsoid 0.075/0.09/0.11 m, 200,000 tri, 10 kHz (k = %.1f), admittance "
                               "beta = 0.1 + 0.05i, Burton-Miller alpha = i/k, depth 7, p = 30/22/16/12/10/8, 32 far points"
                               % k, "num_elements": len(F), "setup_s": setup_s},
        "forward_solve": {"s": t_solve, "iters": it, "relres": rr, "converged": bool(ok), "precision": "mixed IR"},
        "vjp": {"s": t_vjp, "grad_norm": float(np.linalg.norm(grad)), "finite": bool(np.isfinite(grad).all()),
                "adjoint_tol": 1e-8, "precision": "mixed IR"},
        "vjp_admittance": {"s": t_adm, "dJ_dbeta": [float(v) for v in dj_beta],
                           "finite": bool(np.isfinite(g_beta).all())},
        "fd_check": {"mesh_triangles": len(Fs), "vertices": nvert, "h": h,
                     "max_abs_err_over_max_grad": worst, "admittance_rel_err": worst_b,
                     "admittance_fd": [float(v) for v in fdb], "admittance_grad": [float(v) for v in gb0],
                     "tolerance": 1e-4, "pass": bool(worst <= 1e-4 and worst_b <= 1e-4)},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def bodies_arm(args, world, rank, local):
    """The many-body workload: a seeded scene of --bodies bodies (spheres, bumped ellipsoids with
    semi-axes in [0.02, 0.2] m, boxes with edges of 10-100 mm; triangle counts log-uniform in
    [500, 20,000]), each at its own frequency U(0.5, 10) kHz with one plane wave, Burton-Miller
    rigid operator; all solved in lockstep by fmm_scene_solve (one set of launches per Krylov
    step for all bodies; the reported value), by fmm_solve_many (host thread pool, every plan
    on its own streams) and one after another.  --body-tri sets the range of triangle counts."""
    import torch
    import fmbem_gpu_c_gb300 as fm
    torch.cuda.set_device(local)
    rng = np.random.default_rng(2026)
    d = np.array([0.0, 0.6, 0.8])
    tri_lo, tri_hi = (float(v) for v in args.body_tri.split(","))
    plans, rhs, ns, kinds = [], [], [], []
    t0 = time.perf_counter()
    for i in range(args.bodies):
        n_target = float(np.exp(rng.uniform(np.log(tri_lo), np.log(tri_hi))))
        kind = i % 3
        if kind == 0:
            freq = max(5, int(round(np.sqrt(n_target / 20.0))))
            V, F = fm.geodesic_sphere(freq, rng.uniform(0.02, 0.2))
        elif kind == 1:
            freq = max(5, int(round(np.sqrt(n_target / 20.0))))
            ax = rng.uniform(0.02, 0.2, 3)
            V, F = fm.ellipsoid(freq, ax, lmax=8, sigma=0.03 * ax.min(), seed=int(rng.integers(1 << 30)))
        else:
            nb = max(3, int(round(np.sqrt(n_target / 12.0))))
            V, F = fm.box(nb, rng.uniform(0.01, 0.1, 3))
        k = 2 * np.pi * rng.uniform(500.0, 10000.0) / 343.0
        plan = fm.Plan(V, F, k=k, depth=-1, s=5, rule=fm.RULE_GAUSS3, a=0.5, b=0.0, c=-1.0, alpha=1j / k, device=local)
        plans.append(plan)
        rhs.append(plan.plane_wave(d))
        ns.append(len(F))
        kinds.append(kind)
    setup_s = time.perf_counter() - t0
    tol = 1e-6
    t0 = time.perf_counter()
    scene = fm.Scene(plans)
    xw = np.zeros(scene.n, dtype=np.complex128)
    scene.matvec(xw)
    scene.matvec(xw)  # the second call captures the scene's graph
    scene_setup_s = time.perf_counter() - t0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xsc, it_sc, rr_sc, ok_sc = scene.solve(rhs, tol=tol, maxit=3000, restart=100, precision=fm.FMM_MIXED)
        t_scene = time.perf_counter() - t0
        scene_t = scene.timings()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xs, it, rr, st = fm.solve_many(plans, rhs, tol=tol, maxit=3000, restart=100, precision=fm.FMM_MIXED, nthreads=16)
        t_conc = time.perf_counter() - t0
        t0 = time.perf_counter()
        diff, ok_seq = 0.0, True
        for i, plan in enumerate(plans):
            prec = fm.FMM_MIXED if max(plan.info.m2l_columns) > 0 else fm.FMM_FP64
            x, _, r, ok = plan.gmres(rhs[i], tol=tol, maxit=3000, restart=100, precision=prec)
            ok_seq = ok_seq and ok
            diff = max(diff, float(np.linalg.norm(x - xs[i]) / np.linalg.norm(x)))
        t_seq = time.perf_counter() - t0
    mixed = sum(1 for p in plans if max(p.info.m2l_columns) > 0)
    tensor = sum(1 for p in plans if max(p.info.m2l_tensor) > 0)
    scaled = sum(1 for p in plans if p.info.expansions_scaled)
    scene_diff = max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(scene.split(xsc), xs))
    scene.close()
    for p in plans:
        p.close()
    line = {
        "metric": "scene solve s, %d bodies (one plane wave each), lockstep fmm_scene_solve, 1 GB300" % args.bodies,
        "value": t_scene, "unit": "s", "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
        "config": {"workload": "seeded scene: spheres / bumped ellipsoids (0.02-0.2 m) / boxes (10-100 mm), N log-uniform "
                               "in [%g, %g], f ~ U(0.5, 10) kHz, Burton-Miller rigid, tol %g" % (tri_lo, tri_hi, tol),
                   "bodies": args.bodies, "triangles_total": int(sum(ns)), "triangles_min": int(min(ns)),
                   "triangles_max": int(max(ns)), "setup_s": setup_s, "plans_mixed": mixed, "plans_with_tensor_m2l": tensor,
                   "plans_with_scaled_expansions": scaled},
        "scene": {"s": t_scene, "setup_s": scene_setup_s, "converged": bool(ok_sc), "iters_max": int(it_sc.max()),
                  "iters_sum": int(it_sc.sum()), "relres_max": float(rr_sc.max()),
                  "max_rel_diff_to_concurrent": scene_diff, "matvec_device_time": scene_t},
        "concurrent": {"s": t_conc, "threads": 16, "converged": int((st == 0).sum()), "iters_max": int(it.max()),
                       "iters_sum": int(it.sum()), "relres_max": float(rr.max())},
        "sequential": {"s": t_seq, "all_converged": bool(ok_seq), "max_rel_diff_to_concurrent": diff},
        "speedup_scene_vs_concurrent": t_conc / t_scene,
        "speedup_scene_vs_sequential": t_seq / t_scene,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-solve", dest="solve", action="store_false")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-head64", action="store_true", help="leave out the 64-plane-wave batched solve of the default line")
    ap.add_argument("--bodies", type=int, default=256, help="bodies of --workload bodies")
    ap.add_argument("--body-tri", default="500,20000", help="--workload bodies: range of the log-uniform triangle counts")
    ap.add_argument("--workload", default="sphere-cfg2", choices=["sphere-cfg2", "head64", "vjp", "bodies"],
                    help="head64: the 64-plane-wave batched solve on the 200k-triangle head-like body; vjp: the "
                         "vertex gradient on that body at 10 kHz with an admittance boundary; bodies: a scene of many "
                         "bodies solved concurrently (extra lines)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_init()
    if args.workload == "head64":
        head64_arm(args, world, rank, local)
    elif args.workload == "vjp":
        vjp_arm(args, world, rank, local)
    elif args.workload == "bodies":
        bodies_arm(args, world, rank, local)
    elif args.impl == "reference":
        cpu_reference_arm(args, world, rank)
    else:
        gpu_arm(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
