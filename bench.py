"""Benchmark of the osinco3d hot path on GB300: Mpt-steps/s of whole time
steps (predictor, projection with the pressure Poisson solve, correction and
the per-step diagnostics) on the Taylor-Green vortex at 256^3, Re = 1600,
AB3, CFL 0.2, Poisson eps = 1e-8.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One JSON line on stdout (rank 0).  `value` is the mixed-precision method
(FP32 stencils and V-cycles inside the FP64 defect-correction loop); the
plain-FP64 multigrid and red-black SOR steps are in `variants`.  With
--impl reference the FP64 CPU restatement of the reference (the oracle; the
Fortran reference has no compiler here) is timed on the host cores instead.

With N > 1 (torchrun) every rank runs an independent replica of the same
workload on its own GPU (the path has no data exchange): value = all points
x steps over the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
EPS = 1e-8
METRIC = "Mpt-steps/s at 256^3; Poisson s/step learned+mixed vs plain FP64 at same eps"
WORKLOAD = ("Taylor-Green vortex 256^3 periodic [0,2pi)^3 (xlx = 2pi*255/256), Re=1600, AB3, "
            "CFL=0.2 (dt=0.2*2pi/256), Poisson eps=1e-8, no LES, no scalar")

# algorithmic bytes per grid point of one launch (float32 storage)
PRED_BYTES_PER_PT = 15 * 4   # read u,v,w + 6 history, write 3 u* + 3 fluxes

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# 256^3 launches, from the ncu captures summarised in profiles/
TRAFFIC_PER_LAUNCH: dict = {
    "mg_down": (73.19936 + 32.406016) * 1e6,      # k_mg_down_tgv256.md
    "mg_up": (288.510464 + 152.460032) * 1e6,     # k_mg_up_tgv256.md
    "predict": (424.591104 + 348.993024) * 1e6,   # k_predict25v_tgv256.md
    "rhs": (208.823552 + 43.305472) * 1e6,        # k_div25v_tgv256.md (the rhs-writing launch)
    "correct": (278.680320 + 155.391744) * 1e6,   # k_correct25vf_tgv256.md
    "mg_pre": (68.070656 + 25.961216) * 1e6,      # k_lvl25_tgv256.md
    "mg_resid": (138.118144 + 39.967488) * 1e6,   # k_lvl25_tgv256.md
    "resid64": (202.877952 + 45.707520) * 1e6,    # k_resid25_tgv256.md
    "mg_post": (268.986368 + 87.478272) * 1e6,    # k_smooth_upd_tgv256.md
    "mg_prolong": (75.505920 + 11.468032) * 1e6,  # k_smooth_upd_tgv256.md (the finest k_prolong_cell)
}


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        if self.path and os.path.exists(self.path):
            for ln in open(self.path):
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
_PINNED: list = []


def pinned_field(shape):
    """Fortran-ordered float64 array in page-locked host memory."""
    import numpy as np
    import torch

    n = shape[0] * shape[1] * shape[2]
    t = torch.empty(n, dtype=torch.float64, pin_memory=True)
    _PINNED.append(t)  # the numpy view does not own the page-locked memory
    return t.numpy().reshape(shape, order="F")


def make_context(o3d, weights=None, **kw):
    """Context of the 256^3 workload; with the learned guess, the trained
    network is loaded and attached (owned by the context)."""
    p = o3d.tgv_params(N, eps=EPS, **kw)
    ctx = o3d.Context(p)
    if kw.get("guess") == o3d.GUESS_LEARNED:
        from osinco3d_gb300 import learn

        ctx._net_owned = learn.load(weights, ctx.guess_grid())
        ctx.attach_unet(ctx._net_owned)
    return p, ctx


def run_variant(o3d, name: str, steps: int, warmup: int, world: int, weights=None, **kw) -> dict:
    p, ctx = make_context(o3d, weights, **kw)
    ux, uy, uz, pp = o3d.tgv_fields(p)
    for nm, f in zip(("ux", "uy", "uz", "pp"), (ux, uy, uz, pp)):
        ctx.upload(nm, f)
    it = 0
    for _ in range(warmup):
        it += 1
        ctx.step(it)
    barrier(world)
    l0 = ctx.launches
    ms, pms, iters, cyc, res = [], [], [], [], []
    t0 = time.perf_counter()
    for _ in range(steps):
        it += 1
        info = ctx.step(it)
        ms.append(info.step_ms)
        pms.append(info.poisson_ms)
        iters.append(info.poisson_iters)
        cyc.append(info.poisson_cycles)
        res.append(info.poisson_res_inf)
    wall = time.perf_counter() - t0
    launches = ctx.launches - l0
    dev_s = max_over_ranks(sum(ms) / 1e3, world)
    out = {
        "name": name,
        "ms_per_step": 1e3 * dev_s / steps,
        "mpts_per_s": world * (N ** 3) * steps / dev_s / 1e6,
        "wall_ms_per_step": 1e3 * wall / steps,
        "poisson_s_per_step": sum(pms) / 1e3 / steps,
        "poisson_iters_per_step": sum(iters) / steps,
        "vcycles_per_step": sum(cyc) / steps,
        "poisson_res_inf_last": res[-1],
        "gpu_launches": launches,
    }
    return out, ctx, it


def gpu_local_cpus(local: int):
    """CPUs attached to the GPU's PCI device (its NUMA neighbourhood), from
    sysfs; None when they cannot be found."""
    try:
        out = subprocess.run(["nvidia-smi", "-i", str(local), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout.strip()
        dom, bus, rest = out.split(":")
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{bus.lower()}:{rest.lower()}/local_cpulist"
        cpus = set()
        for part in open(path).read().strip().split(","):
            a, _, b = part.partition("-")
            cpus.update(range(int(a), int(b or a) + 1))
        return cpus or None
    except Exception:
        return None


def measure_e2e(o3d, steps: int, warmup: int, world: int, weights=None, local: int = 0, **kw) -> dict:
    """Same steps through o3d_step_host: the driver's host arrays (page-locked)
    are copied in before and out after every step.  The host thread runs on
    the GPU's local CPUs while the arrays are allocated and copied, so that
    they sit in the memory next to the GPU (as a driver process bound to its
    GPU's NUMA node would have them)."""
    saved = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") else None
    cpus = gpu_local_cpus(local)
    if cpus and saved is not None:
        try:
            os.sched_setaffinity(0, cpus & set(range(os.cpu_count() or 1)) or cpus)
        except OSError:
            cpus = None
    try:
        return _measure_e2e(o3d, steps, warmup, world, weights, **kw)
    finally:
        if cpus and saved is not None:
            os.sched_setaffinity(0, saved)


def _measure_e2e(o3d, steps: int, warmup: int, world: int, weights=None, **kw) -> dict:
    p, ctx = make_context(o3d, weights, **kw)
    ux0, uy0, uz0, pp0 = o3d.tgv_fields(p)
    bufs = [pinned_field(ux0.shape) for _ in range(4)]
    for b, f in zip(bufs, (ux0, uy0, uz0, pp0)):
        b[...] = f
    with ctx:
        it = 0
        for _ in range(warmup):
            it += 1
            ctx.step_host(it, *bufs)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            it += 1
            ctx.step_host(it, *bufs)
        wall = max_over_ranks(time.perf_counter() - t0, world)
    nbytes = 4 * (N ** 3) * 8
    return {"value": world * (N ** 3) * steps / wall / 1e6, "unit": "Mpt-steps/s",
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
            "ms_per_step": 1e3 * wall / steps, "link": link_rates(bufs[0])}


def link_rates(host) -> dict:
    """Plain copies of one pinned FP64 field (the e2e run's own host buffer)
    to and from the device, timed with CUDA events: the host link's rate on
    this box, against which the e2e copies are judged."""
    import torch

    h = torch.from_numpy(host.reshape(-1, order="F"))  # a view: the page-locked memory itself
    d = torch.empty(h.numel(), dtype=torch.float64, device="cuda")
    nb = h.numel() * 8
    out = {}
    for name, fn in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            fn()
        e1.record()
        e1.synchronize()
        out[name] = 5 * nb / (e0.elapsed_time(e1) * 1e-3) / 1e9
    return out


# algorithmic bytes per grid point of the hot kernels (float32 storage)
KERNEL_BYTES = {
    "predict": (PRED_BYTES_PER_PT, "k_predict25v<float> (two x-adjacent points per thread)"),
    # read r, write e and the coarse rhs (1/8)
    "mg_down": (4 + 4 + 0.5, "k_mg_down<2,zero> (pre-smoothing + residual + restriction, finest level; "
                             "the step runs mg_pre and mg_resid there instead)"),
    # the finest level's first sweep from e = 0 (read r, write e) and its residual (read e, r; write t),
    # the 2.5D one-pass kernels the step runs before the fused up kernel
    "mg_pre": (4 + 4, "k_lvl25p<1> (first red-black sweep from e = 0, finest level)"),
    "mg_resid": (4 + 4 + 4, "k_lvl25p<2> (level residual, finest level)"),
    # read e, r, p and the coarse correction (1/8), write e and p
    "mg_up": (4 + 4 + 8 + 0.5 + 4 + 8, "k_mg_up<2,update> (prolongation + post-smoothing + p += e, finest; "
                                       "mg_kernels = 2 only, the step runs mg_prolong, mg_red and mg_post there)"),
    # the post-smoothing of the step's finest level as one-pass kernels: the prolongation-add (read e and
    # the coarse correction, write e), the red pass (read e, r; write e) and the black pass with the
    # pressure pair's update (read e, r and the pair; write the pair)
    "mg_prolong": (4 + 0.5 + 4, "k_prolong_cell (prolongation-add, finest level)"),
    "mg_red": (4 + 4 + 4, "k_smooth<float> colour 0 (red pass, finest level)"),
    "mg_post": (4 + 4 + 8 + 8, "k_smooth_upd (black pass + p += e on the pressure pair + max|e|, finest level)"),
    # read u* (3 x FP32), write the FP32 rhs (its trapezoid-weighted sums ride along)
    "rhs": (4 * 3 + 4, "k_div25v<float> (Poisson rhs, FP32, with its weighted sums)"),
    # read u* (3 x FP32) and the pressure's FP32 high plane, write u (3 x FP32)
    "correct": (4 * 6 + 4, "k_correct25vf (FP32 high plane of the pressure pair, FP32 velocity)"),
    # read the pressure pair (2 x FP32) and the FP32 rhs, write r (FP32)
    "resid64": (8 + 4 + 4, "k_resid25p (double-float residual from the pressure pair, two points per thread)"),
}
# the kernel the roofline entry describes: the outer iteration's
# double-float residual, three launches per step and the largest share of it
ROOF_KERNEL = "resid64"


def kernel_roofline(o3d, ctx, peaks: dict) -> dict:
    """Device time per launch of the hot kernels on the live state (CUDA events
    on the context's stream, averaged over repeated launches) and their
    achieved algorithmic bandwidth."""
    peak = peaks.get("hbm_gbs")
    out = {}
    for name, (bpp, label) in KERNEL_BYTES.items():
        t = ctx.time_kernel(name, 20)
        gbs = bpp * N ** 3 / (t * 1e-3) / 1e9
        out[name] = {"kernel": label, "ms": t, "bytes_per_point": bpp, "achieved": gbs,
                     "frac": gbs / peak if peak else None}
    for name, v in out.items():
        v["traffic"] = TRAFFIC_PER_LAUNCH.get(name)
    return out


# Lexicographic SOR sweeps the reference's solver takes per step of this
# workload at eps = 1e-8 (omega = 2/(1 + sin(2 pi^2 / 256)), starting from the
# previous pressure): the oracle's exit iterations on steps 1-5 were 338,
# 346, 243, 236 and 240; the AB3 steps settle at about 240.
# `python bench.py --cpu-full-steps 5` runs those steps to convergence again.
K_LEX = 240


def _cpu_case(orc, kmax):
    L = 2 * math.pi * (N - 1) / N
    return orc.Case(N, N, N, L, L, L, dt=0.2 * 2 * math.pi / N,
                    omega=2.0 / (1.0 + math.sin(math.pi * 2 * math.pi / N)), eps=EPS, kmax=kmax)


def cpu_sweep_seconds(sweeps: int = 10) -> float:
    """Seconds per lexicographic SOR sweep of the oracle at 256^3 (the
    reference's poisson_solver_0000 loop; serial as in the reference)."""
    import numpy as np

    from oracle import oracle as orc

    orc.build()
    case = _cpu_case(orc, sweeps)
    rng = np.random.default_rng(0)
    rhs = np.asfortranarray(rng.standard_normal(case.shape))
    pp = orc.field3(case.shape)
    t0 = time.perf_counter()
    orc.poisson_sor(case, pp, rhs, case.omega, 0.0, sweeps)  # eps = 0: exactly `sweeps` sweeps
    return (time.perf_counter() - t0) / sweeps


def cpu_step_seconds(omp: bool, sweeps: int = 10) -> float:
    """Seconds of one 256^3 step of the oracle (predictor, divergence,
    correction, diagnostics) with its SOR capped at `sweeps` sweeps."""
    from oracle import oracle as orc

    orc.build()
    case = _cpu_case(orc, sweeps)
    st = orc.State.zeros(case)
    orc.init_tgv(case, st, omp=omp)
    r = orc.Runner(case, st, omp=omp)
    t0 = time.perf_counter()
    r.step(1)
    return time.perf_counter() - t0


def cpu_baseline_oracle(omp: bool = False, sweeps: int = 10) -> dict:
    """The FP64 oracle (the C restatement of the reference) on a bounded
    sample of the workload, extrapolated to a full step: one 256^3 step with
    the lexicographic SOR capped at `sweeps` sweeps, plus `sweeps` sweeps of
    the solver timed alone; a full step is that step plus K_LEX - sweeps more
    sweeps."""
    t_cap = cpu_step_seconds(omp, sweeps)
    t_sweep = cpu_sweep_seconds(sweeps)
    t_step = t_cap + (K_LEX - sweeps) * t_sweep
    cores = (os.cpu_count() or 1) if omp else 1
    return {"value": N ** 3 / t_step / 1e6, "unit": "Mpt-steps/s", "cores": cores, "kind": "port",
            "sample": (f"extrapolated full step: 1 step of the 256^3 workload in FP64 on the oracle (C restatement) "
                       f"with the lexicographic SOR capped at {sweeps} sweeps ({t_cap:.2f} s), plus {sweeps} "
                       f"sweeps timed alone ({t_sweep:.3f} s each), scaled to {K_LEX} sweeps per step (the "
                       f"reference solver's exit iteration on this workload) = {t_step:.1f} s per step"),
            "seconds_sampled": t_cap + sweeps * t_sweep, "seconds_per_step": t_step, "sweep_s": t_sweep,
            "sweeps_per_step": K_LEX}


def cpu_full_steps(nsteps: int, omp: bool) -> dict:
    """Full steps of the oracle with the SOR to convergence: the exit
    iteration and the time of each (about a minute per step at 256^3)."""
    from oracle import oracle as orc

    orc.build()
    case = _cpu_case(orc, 100000)
    st = orc.State.zeros(case)
    orc.init_tgv(case, st, omp=omp)
    r = orc.Runner(case, st, omp=omp)
    out = []
    for it in range(1, nsteps + 1):
        t0 = time.perf_counter()
        info = r.step(it)
        out.append({"step": it, "sor_status": info.sor_status, "sweeps": info.sor_iters,
                    "seconds": time.perf_counter() - t0})
    return {"workload": WORKLOAD, "omp_cores": (os.cpu_count() or 1) if omp else 1, "steps": out}


GUESS_DESC = {"mixed_mg_learned": "learned (U-Net correction of the linearly extrapolated pressure)",
              "mixed_mg": "previous pressure"}


def load_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def gpu_arm(args, rank, world, local):
    from osinco3d_gb300 import learn, o3d

    o3d.lib()
    peaks = load_peaks()
    variants = {}
    weights = learn.WEIGHTS if os.path.exists(learn.WEIGHTS) else None
    mixed = dict(precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, kmax=100)
    if weights:
        head_name, head_kw = "mixed_mg_learned", dict(mixed, guess=o3d.GUESS_LEARNED)
    else:
        head_name, head_kw = "mixed_mg", mixed
    with ClockSampler(local) as clk:
        head, ctx, _ = run_variant(o3d, head_name, args.steps, args.warmup, world, weights=weights, **head_kw)
    clocks = clk.summary()
    roof = None if args.no_roofline else kernel_roofline(o3d, ctx, peaks)
    ctx.close()
    variants[head_name] = head
    # end to end right after the headline, on the same configuration
    e2e = None if args.no_e2e else measure_e2e(o3d, max(3, args.steps // 2), 3, world, weights=weights, local=local,
                                                **head_kw)
    if not args.quick:
        fp64 = dict(precision=o3d.PREC_FP64, solver=o3d.SOLVER_MG, kmax=100)
        for name, kw in (("mixed_mg", mixed), ("mixed_mg_extrapolated", dict(mixed, guess=o3d.GUESS_EXTRAPOLATED)),
                         ("mixed_mg_zero", dict(mixed, guess=o3d.GUESS_ZERO)),
                         # one kernel per multigrid pass instead of the fused level kernels
                         ("mixed_mg_unfused", dict(mixed, mg_kernels=1)),
                         # the plain method: FP64 V(2,2) Gauss-Seidel from the previous pressure
                         ("fp64_mg", fp64),
                         # FP64 with the mixed method's smoother settings and extrapolated guess
                         ("fp64_mg_v11_om1.25_extrapolated",
                          dict(fp64, mg_pre=1, mg_post=1, mg_omega=1.25, guess=o3d.GUESS_EXTRAPOLATED)),
                         # linear extrapolation with its best cycle: V(2,1), omega 1.3
                         ("mixed_mg_extrapolated_v21_om1.3",
                          dict(mixed, mg_pre=2, mg_post=1, mg_omega=1.3, guess=o3d.GUESS_EXTRAPOLATED)),
                         # quadratic extrapolation in time with the default V(1,1)
                         ("mixed_mg_extrapolated2", dict(mixed, guess=o3d.GUESS_EXTRAPOLATED2))):
            if name in variants:
                continue
            v, cx, _ = run_variant(o3d, name, args.steps, args.warmup, world, **kw)
            cx.close()
            variants[name] = v
        sor_steps = max(2, args.steps // 4)
        v, c3, _ = run_variant(o3d, "fp64_rbsor", sor_steps, min(args.warmup, 3), world,
                               precision=o3d.PREC_FP64, solver=o3d.SOLVER_SOR, kmax=20000)
        c3.close()
        variants["fp64_rbsor"] = v
    line = {
        "metric": METRIC,
        "value": head["mpts_per_s"],
        "unit": "Mpt-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 stencils/V-cycles + fp64 defect correction",
        "data": "synthetic (analytic Taylor-Green initial state)",
        "config": {"workload": WORKLOAD, "grid": [N, N, N], "poisson": ("FP32 multigrid V(1,1), red-black smoother omega=1.25, one V-cycle per FP64 residual "
                               "(defect correction); initial guess: " + GUESS_DESC[head_name]),
                   "parallelism": f"replicas x{world}", "l2": "no flush: every step streams > 1 GB, far above the 129 MB L2"},
        "e2e": e2e,
        "gpu_launches": head["gpu_launches"],
        "clocks": clocks,
        "variants": variants,
    }
    if roof:
        top = roof[ROOF_KERNEL]
        line["roofline"] = {"bound": "hbm", "achieved": top["achieved"], "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                            "frac": top["frac"], "traffic": TRAFFIC_PER_LAUNCH.get(ROOF_KERNEL),
                            "kernel": top["kernel"], "bytes_per_point": top["bytes_per_point"], "ms": top["ms"],
                            "peak_source": peaks.get("source"),
                            "others": {k: v for k, v in roof.items() if k != ROOF_KERNEL}}
    if "fp64_mg" in variants:
        line["speedup_mixed_vs_fp64_mg"] = variants["fp64_mg"]["ms_per_step"] / head["ms_per_step"]
        line["speedup_mixed_vs_fp64_rbsor"] = variants["fp64_rbsor"]["ms_per_step"] / head["ms_per_step"]
        line["poisson_s_per_step"] = {k: v["poisson_s_per_step"] for k, v in variants.items()}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_oracle()
    return line


def reference_arm(args, rank, world):
    """The reference's CPU implementation of the path on the host cores: the
    oracle with OpenMP on its stencil passes (the lexicographic SOR stays
    serial, as in the reference), each step a bounded sample extrapolated to
    a full step (cpu_baseline_oracle)."""
    if rank != 0:
        return None
    t_sweep = cpu_sweep_seconds()
    caps = []
    for k in range(args.warmup + args.steps):
        t = cpu_step_seconds(True)
        if k >= args.warmup:
            caps.append(t)
    t_step = sum(caps) / len(caps) + (K_LEX - 10) * t_sweep
    val = N ** 3 / t_step / 1e6
    cb = {"value": val, "unit": "Mpt-steps/s", "cores": os.cpu_count() or 1, "kind": "port",
          "sample": (f"per step: 1 time step of the 256^3 workload in FP64 on the oracle (C restatement, OpenMP on "
                     f"the stencil passes, lexicographic SOR serial as in the reference) with the SOR capped at 10 "
                     f"sweeps (mean {sum(caps) / len(caps):.2f} s), extrapolated to {K_LEX} sweeps per step with "
                     f"{t_sweep:.3f} s per sweep timed alone = {t_step:.1f} s per step")}
    return {"metric": METRIC, "value": val, "unit": "Mpt-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [N, N, N]}, "impl": "reference",
            "cpu_baseline": cb, "e2e": {"value": val, "unit": "Mpt-steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline variant only")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end run")
    ap.add_argument("--cpu-full-steps", type=int, default=0,
                    help="run this many full 256^3 steps of the oracle (SOR to convergence) and print them")
    ap.add_argument("--no-roofline", action="store_true",
                    help="skip the per-kernel timing launches (for a launch list of the steps alone)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.cpu_full_steps:
        print(json.dumps(cpu_full_steps(args.cpu_full_steps, omp=True)), flush=True)
        return
    rank, world, local = dist_setup()
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
    else:
        line = gpu_arm(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
