#!/usr/bin/env python
"""Benchmark: IISPH particle-steps/s on the 1,000,000-fluid-particle dam break
with WKBB18 implicit viscosity (IISPH + PCG, dt 5e-4 s), one GB300.

A step is one pass of the reference driver loop
(share/scripts/prtcl-lua.example.lua:363-461) over the resident scene: grid
update (permute every 8 steps), density, gravity, velocity integration,
IISPH set-up + relaxed Jacobi to 0.1 % average density error (<= 100
iterations), velocity integration, WKBB18 diagonal + PCG (tolerance 1e-4,
<= 100 iterations), velocity integration, position integration.

Arms:
  default            the CUDA library through its C ABI.  `value` is timed
                     with CUDA events on the model's stream around K steps of
                     the resident scene; `e2e` is the same metric through the
                     public API with host buffers: the scene is uploaded from
                     pinned host memory inside the timed region and every
                     step downloads the fluid positions (a frame) to pinned
                     host memory.
  --impl reference   the CPU oracle (OpenMP restatement of the reference's
                     procedures, f32 reductions, per-procedure neighbour
                     re-query) on all host threads, same scene and metric.

Extra measurements in the same line (rank 0, one GPU; --no-extras skips them):
  long_run  the 1M dam break over all 500 steps of its configuration: rate and
            iteration counts over steps 1-250 and 251-500
  plain_27k the reference's plain 27k dam break (IISPH), beside the CPU oracle
  search    neighbour search only, 4M points (uniform / 64 Gaussian blobs),
            radius for 40 mean neighbours, GB/s of algorithmic bytes vs HBM
  batched   256 mixed-size dam-break scenes stepped together by one batch,
            against the same scenes through the plain single-scene path
  serving   Poisson arrivals of dam-break requests, continuous batching,
            throughput and p50 / p99 latency

Prints one JSON line (rank 0).  Inputs are larger than L2 (the 1.36M-particle
working set is ~270 MB), so no explicit L2 flush is done between steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from prtcl_gb300 import driver, scenes, tune  # noqa: E402

METRIC = "IISPH particle-steps/s, plain vs batched, at <=0.1% density error; serve p99"
UNIT = "particle-steps/s"

# algorithmic bytes per kernel launch: each reference field read or written
# once per kernel (f32: real 4 B, real[3] 12 B, real[3][3] 36 B); neighbour
# re-reads and neighbour-list traffic excluded.  (per fluid item, per
# boundary item)
ALGO_BYTES = {
    "density": (20, 16),        # x, m -> rho ; boundary x, V
    "iisph_setup": (88, 32),    # x, v, m, rho -> c, p, s, AA ; boundary x, V (both passes)
    "iisph_accel": (36, 16),    # x, m, p, rho -> a
    "iisph_pressure": (52, 16),  # x, m, a, rho, s, AA, p -> Ap, p
    "wkbb18_diag": (56, 16),    # x, m, rho -> sp
    "pcg_init": (116, 16),      # x, m, rho, x0, v, sp -> r, y, p
    "pcg_q": (44, 16),          # x, m, rho, p -> q
    "pcg_update": (120, 0),     # x, p, r, q, sp -> x, r, y
    "pcg_p": (36, 0),           # y, p -> p
    "integrate_velocity": (40, 0),  # v, a, t_birth -> v
    "integrate_position": (36, 0),  # x, v -> x
    "gravity": (12, 0),
}
# list build (nhood_lists): per fluid query and per listed pair
LIST_BYTES_PER_QUERY, LIST_BYTES_PER_PAIR = 16, 8


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    """Per-launch DRAM bytes (dram__bytes_read.sum + write.sum) of kernels
    captured with ncu, with the capture's command and the commit of the
    build it ran on (profiles/ncu_traffic.json)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


TRAFFIC_1M = "dam break 1M fluid + 363,436 boundary"


def roofline_block(name, launches, ms, algo_bytes_total, peak, peak_kind, timing, workload=None):
    """Achieved algorithmic GB/s of one kernel (its algorithmic bytes over
    all launches / its total CUDA-event time) against the HBM peak; the
    measured DRAM traffic per launch where a capture of this kernel on this
    workload is recorded."""
    avg_s = ms / 1e3 / launches
    per_launch = algo_bytes_total / launches
    ach = per_launch / avg_s / 1e9
    tr = load_traffic()
    rec = tr.get("kernels", {}).get(name)
    if rec is not None and rec.get("workload") != workload:
        rec = None
    return {"bound": "hbm", "kernel": name, "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 4), "traffic": rec["dram_bytes_per_launch"] if rec else None,
            "traffic_source": (f"profiles/ncu_traffic.json: {rec['workload']}, captured at commit {tr.get('commit')}"
                               if rec else None),
            "peak_kind": peak_kind, "algorithmic_bytes_per_launch": int(per_launch),
            "avg_launch_us": round(avg_s * 1e6, 2), "launches": launches, "timing": timing}


def kernel_bytes(name, launches, nf, nb):
    """Algorithmic bytes of `launches` launches of a kernel over nf fluid and
    nb boundary items each (None for kernels without a formula)."""
    if name not in ALGO_BYTES:
        return None
    bf, bb = ALGO_BYTES[name]
    return launches * (bf * nf + bb * nb)


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"prtcl_gb300_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("LOCAL_RANK", "0")],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    smax = float(c[2])
                except ValueError:
                    continue
                for n, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return rank, world, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def nvtx_range(name):
    """An NVTX range around a measured pass (profile_pass: every kernel of
    the headline's profile steps is its own launch; search_uniform,
    search_blobs: the timed searches; batched_profile_pass), so that a
    profiler can select exactly those launches."""
    try:
        import torch
        torch.cuda.nvtx.range_push(name)
        return True
    except Exception:
        return False


def nvtx_end(opened):
    if opened:
        import torch
        torch.cuda.nvtx.range_pop()


def timed_steps(d, loop, K):
    """K quiet steps (no host round trip inside a step) bracketed by CUDA
    events recorded on the model's stream (the stream every kernel of the
    step is launched on)."""
    import torch

    from prtcl_gb300 import _lib
    s = torch.cuda.ExternalStream(d.model.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    d.synchronize()
    torch.cuda.synchronize()
    l0 = _lib.load().prtcl_gpu_launch_count()
    e0.record(s)
    t0 = time.perf_counter()
    for _ in range(K):
        loop.step(quiet=True)
    e1.record(s)
    e1.synchronize()
    wall = time.perf_counter() - t0
    d.synchronize()
    launches = _lib.load().prtcl_gpu_launch_count() - l0
    return e0.elapsed_time(e1) / 1e3, wall, launches


def config_of(args, nf, nb, world):
    """The workload description both arms print (identical keys and values
    for the same arguments)."""
    return {"workload": ("dam break 1M fluid + %d boundary, IISPH + WKBB18 PCG, dt 5e-4 s" % nb)
            if args.config == "1m" else "dam break 27k fluid + %d boundary, IISPH + WKBB18 PCG, dt 1e-3 s" % nb,
            "fluid_particles": nf, "boundary_particles": nb, "replicas": world,
            "parallelism": "replicas only" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (no flush)", "steps_timed": f"{args.steps} after {args.warmup} warm-up"}


def workload(args):
    if args.config == "1m":
        return scenes.dam_break_1m(), driver.DAM_BREAK_1M
    return scenes.dam_break(), dict(driver.DAM_BREAK_27K, viscosity=True)


def tuned(kind, sc, p):
    """The autotuner's knob choice for a workload (tuned on a copy of it
    unless cached) and how it was obtained."""
    t0 = time.perf_counter()
    if kind == "plain":
        choice, source, _ = tune.tune_plain(sc, p)
        wl = tune.workload_class("plain", len(sc["fluid"]))
    else:
        choice, source, _ = tune.tune_batched(sc, p)
        wl = tune.workload_class("batched", sum(len(x["fluid"]) for x in sc), len(sc))
    return choice, {"choice": choice, "source": source, "workload_class": wl,
                    "seconds": round(time.perf_counter() - t0, 2)}


def run_ours(args, rank, world, dist):
    from prtcl_gb300.core import DeviceScene
    sc, p = workload(args)
    nf, nb = len(sc["fluid"]), len(sc["boundary"])
    if args.no_tune:
        choice, tuning = dict(tune.DEFAULTS), {"choice": dict(tune.DEFAULTS), "source": "defaults (--no-tune)"}
    else:
        choice, tuning = tuned("plain", sc, p)
    if args.knob:
        choice = dict(choice, **args.knob)
        tuning = dict(tuning, choice=choice, overrides=args.knob)

    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    tune.apply(d.model, choice)
    loop = driver.StepLoop(d, p, device_loop=True)
    for _ in range(args.warmup):
        loop.step(quiet=True)
    d.model.stats(reset=True)
    clocks = Clocks()
    barrier(dist)
    clocks.start()
    secs, wall, launches = timed_steps(d, loop, args.steps)
    clk = clocks.stop()
    st = d.model.stats(reset=True)
    secs = max_over_ranks(dist, secs)
    value = nf * args.steps * world / secs

    # per-kernel CUDA-event timing, live in this process: a few more steps
    # with timing events around every launch (device loops driven from the
    # host so that each launch is timed; same kernels)
    nvtx = nvtx_range("profile_pass")
    prof = profile_pass(d, loop, args.profile_steps)
    nvtx_end(nvtx)

    peak, peak_kind = load_peaks()
    roof = plain_roofline(d, prof, nf, nb, peak, peak_kind,
                          f"CUDA events around each launch over {args.profile_steps} extra steps",
                          TRAFFIC_1M if args.config == "1m" else None)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, sc, p, nf, dist, world, choice)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, p, nf, steps=args.cpu_steps)

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        legs = {"long_run": lambda: run_long(peak),
                "plain_27k": lambda: run_plain_27k(args.no_cpu_baseline, peak=peak, peak_kind=peak_kind),
                "search": lambda: run_search(peak, no_cpu=args.no_cpu_baseline),
                "batched": lambda: run_batched(peak=peak, peak_kind=peak_kind, no_cpu=args.no_cpu_baseline),
                "serving": run_serving}
        for name, leg in legs.items():
            if args.extras is None or name in args.extras:
                extras[name] = leg()

    solves = max(st["jacobi_solves"], 1.0)
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(secs * 1e3 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 convergence reductions)",
        "data": "synthetic (seeded lattice dam break generated in-process)",
        "config": config_of(args, nf, nb, world),
        "solver": {"jacobi_iterations_mean": round(st["jacobi_iterations"] / solves, 3),
                   "jacobi_capped_steps": int(st["jacobi_capped"]),
                   "max_relative_density_error": st["max_relative_aprde"],
                   "pcg_iterations_mean": round(st["pcg_iterations"] / max(st["pcg_solves"], 1.0), 3),
                   "wall_s": round(wall, 3)},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
        "tuning": tuning,
        "kernels": {k: {"launches": c, "ms": round(m, 3), "us_per_launch": round(1e3 * m / c, 2)}
                    for k, (c, m) in prof.items()},
        **extras,
    }
    if rank == 0:
        print(json.dumps(line))


def plain_roofline(d, prof, nf, nb, peak, peak_kind, timing, workload=None):
    """Roofline of the dominant kernel of a single-scene profile that has an
    algorithmic-byte formula (the grid update's kernels have none); the top
    kernel overall is named beside it where it is another."""
    if not prof:
        return None

    def has_formula(name):
        return name == "nhood_lists" or name in ALGO_BYTES

    ranked = sorted(prof.items(), key=lambda kv: -kv[1][1])
    cand = [(n, c, m) for n, (c, m) in ranked if has_formula(n)]
    if not cand:
        return {"kernel": ranked[0][0], "frac": None, "note": "no algorithmic-byte formula for any kernel"}
    name, cnt, ms = cand[0]
    total = kernel_bytes(name, cnt, nf, nb)
    if name == "nhood_lists":
        # per fluid query its position and count (16 B), per listed pair
        # (fluid and boundary neighbours) an index and a gradient factor
        # (8 B); the pairs of the lists as they stand after the pass
        d.update()
        pairs = d.nhood.query(d.model.get_group("f").index, count_pairs=True)
        total = cnt * (LIST_BYTES_PER_QUERY * nf + LIST_BYTES_PER_PAIR * pairs)
    roof = roofline_block(name, cnt, ms, total, peak, peak_kind, timing, workload)
    roof["share_of_kernel_time"] = round(ms / sum(m for _, m in prof.values()), 4)
    if ranked[0][0] != name:
        roof["top_kernel_without_formula"] = {"kernel": ranked[0][0], "ms": round(ranked[0][1][1], 3)}
    return roof


def run_e2e(args, sc, p, nf, dist, world, choice=None):
    """Same metric through the public API with host buffers, over the steps
    the device-timed value and the reference arm time: the scene is
    uploaded from pinned host memory and set up, and `warmup` steps run
    (untimed there too); then every one of the `steps` timed steps takes its
    input from the host (the current time) and brings its result (the fluid
    positions) back to pinned host memory inside the timed region.  The same
    run from the upload on (upload, set-up, warm-up and timed steps, all
    counted) is reported beside it."""
    from prtcl_gb300.core import DeviceScene

    def pinned_copy(a):
        try:
            import torch
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            return t.numpy(), t
        except Exception:
            return np.ascontiguousarray(a), None

    keep = []
    host = {}
    for k in ("fluid", "boundary"):
        arr, t = pinned_copy(sc[k])
        host[k] = arr
        keep.append(t)
    frame, t = pinned_copy(np.zeros((nf, 3), np.float32))
    keep.append(t)
    scene = dict(sc, fluid=host["fluid"], boundary=host["boundary"])
    barrier(dist)
    t0 = time.perf_counter()
    d = DeviceScene()
    if choice:
        tune.apply(d.model, choice)
    driver.setup_dam_break(d, scene, p)
    upload = sum(a.nbytes for a in host.values()) + nf * (12 + 12 + 4 + 4) + len(sc["boundary"]) * 4
    loop = driver.StepLoop(d, p, device_loop=True)
    posf = d.model.get_group("f").varying.get_field("position")
    for _ in range(args.warmup):
        loop.step(quiet=True)
        posf.download(out=frame)
    d.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        loop.step(quiet=True)  # the current time (4 bytes) goes to the device
        posf.download(out=frame)
    d.synchronize()
    t2 = time.perf_counter()
    secs = max_over_ranks(dist, t2 - t1)
    secs_all = max_over_ranks(dist, t2 - t0)
    total = args.warmup + args.steps
    return {"value": round(nf * args.steps * world / secs, 1), "unit": UNIT,
            "h2d_bytes_per_step": 4, "d2h_bytes_per_step": int(nf * 12),
            "includes": f"per step: the current time from the host, the step, the fluid positions back to pinned "
                        f"host memory; {args.steps} steps after {args.warmup} warm-up steps, as the device-timed "
                        f"value and the reference arm",
            "from_upload": {"value": round(nf * total * world / secs_all, 1), "unit": UNIT,
                            "h2d_bytes_per_step": int(upload / total + 4), "d2h_bytes_per_step": int(nf * 12),
                            "includes": f"scene upload from pinned host memory + set-up + all {total} steps "
                                        f"(warm-up included) with a position download per step"}}


def cpu_baseline(sc, p, nf, steps=2, threads=0):
    """The CPU oracle in reference mode on the host cores: a bounded sample of
    `steps` steps of the same scene after set-up."""
    from oracle import oracle as O
    O.build()
    th = O.set_threads(threads)
    o = O.Scene(np.float32, fp64_reductions=False)
    driver.setup_dam_break(o, sc, p)
    o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=p.get("viscosity", False))  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=p.get("viscosity", False))
    secs = time.perf_counter() - t0
    return {"value": round(nf * steps / secs, 1), "unit": UNIT, "cores": th, "kind": "port",
            "sample": f"{steps} steps of the same scene after set-up and one warm step ({secs:.1f} s)"}


def profile_pass(d, loop, steps):
    """{kernel: (launches, ms)} over `steps` more steps with CUDA events
    around every launch (device loops driven from the host)."""
    d.model.profile(True)
    d.model.profile_reset()
    for _ in range(steps):
        loop.step(quiet=True)
    d.synchronize()
    prof = d.model.profile_read()
    d.model.profile(False)
    return prof


def run_plain_27k(no_cpu=False, steps=1000, warmup=3, cpu_steps=10, peak=None, peak_kind=None):
    """The reference's plain configuration: the 27,000-particle dam break
    (spacing 0.025 m, 2 x 1 x 1 m box, dt 1e-3 s, IISPH to 0.1 % or 100
    iterations), all 1000 steps of the configuration timed on the device
    after `warmup` steps,
    the roofline of its dominant kernel, the same steps end to end through
    the public API (upload from pinned host memory, a position frame
    downloaded per step), beside the CPU oracle (reference mode, all host
    threads) on `cpu_steps` steps of the same scene."""
    from types import SimpleNamespace

    from prtcl_gb300.core import DeviceScene
    sc, p = scenes.dam_break(), dict(driver.DAM_BREAK_27K)
    nf, nb = len(sc["fluid"]), len(sc["boundary"])
    choice, tuning = tuned("plain", sc, p)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    tune.apply(d.model, choice)
    loop = driver.StepLoop(d, p, device_loop=True)
    for _ in range(warmup):
        loop.step(quiet=True)
    d.model.stats(reset=True)
    secs, wall, launches = timed_steps(d, loop, steps)
    st = d.model.stats(reset=True)
    out = {"workload": "dam break 27k fluid + %d boundary, IISPH, dt 1e-3 s" % nb,
           "steps": steps, "warmup": warmup, "value": round(nf * steps / secs, 1), "unit": UNIT,
           "ms_per_step": round(secs * 1e3 / steps, 4), "gpu_launches": int(launches),
           "jacobi_iterations_mean": round(st["jacobi_iterations"] / max(st["jacobi_solves"], 1.0), 3),
           "jacobi_capped_steps": int(st["jacobi_capped"]), "max_relative_density_error": st["max_relative_aprde"],
           "tuning": tuning}
    if peak is not None:
        prof = profile_pass(d, loop, 5)
        out["roofline"] = plain_roofline(d, prof, nf, nb, peak, peak_kind,
                                         "CUDA events around each launch over 5 extra steps")
    del loop, d
    out["e2e"] = run_e2e(SimpleNamespace(steps=steps, warmup=warmup), sc, p, nf, None, 1, choice)
    if not no_cpu:
        from oracle import oracle as O
        O.build()
        th = O.set_threads(0)
        o = O.Scene(np.float32, fp64_reductions=False)
        driver.setup_dam_break(o, sc, p)
        for _ in range(warmup):
            o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=False)
        t0 = time.perf_counter()
        for k in range(cpu_steps):
            o.step(permute=((k + 1) % p["permute_every"] == 0), max_iters=p["max_iters"], eta=p["eta"],
                   viscosity=False)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(nf * cpu_steps / cs, 1), "unit": UNIT, "cores": th, "kind": "port",
                               "sample": f"{cpu_steps} steps after {warmup} warm-up steps"}
    return out


def run_long(peak, steps=500, split=250):
    """Config 2 over its full 500 steps (the dam break develops, so the
    iteration counts change): particle-steps/s, mean Jacobi and PCG
    iterations over steps 1-250 and 251-500, each half timed with CUDA
    events on the model's stream."""
    from prtcl_gb300.core import DeviceScene
    sc, p = scenes.dam_break_1m(), driver.DAM_BREAK_1M
    nf = len(sc["fluid"])
    choice, tuning = tuned("plain", sc, p)
    d = DeviceScene()
    driver.setup_dam_break(d, sc, p)
    tune.apply(d.model, choice)
    loop = driver.StepLoop(d, p, device_loop=True)
    out = {"workload": "dam break 1M fluid, IISPH + WKBB18 PCG, dt 5e-4 s, steps 1-%d" % steps, "unit": UNIT,
           "tuning": tuning}
    for lo, hi in ((1, split), (split + 1, steps)):
        d.model.stats(reset=True)
        secs, _, _ = timed_steps(d, loop, hi - lo + 1)
        st = d.model.stats(reset=True)
        out[f"steps_{lo}_{hi}"] = {
            "value": round(nf * (hi - lo + 1) / secs, 1), "ms_per_step": round(secs * 1e3 / (hi - lo + 1), 3),
            "jacobi_iterations_mean": round(st["jacobi_iterations"] / max(st["jacobi_solves"], 1.0), 3),
            "jacobi_capped_steps": int(st["jacobi_capped"]),
            "max_relative_density_error": st["max_relative_aprde"],
            "pcg_iterations_mean": round(st["pcg_iterations"] / max(st["pcg_solves"], 1.0), 3)}
    x = d.get_varying("f", "position")
    out["final_state_finite"] = bool(np.isfinite(x).all())
    return out


def search_cpu_baseline(pts, r, n):
    """The oracle's grid update + the neighbour sets of every point (the
    reference's grid restated, OpenMP on all host threads), one full 4M
    search timed on the host."""
    from oracle import oracle as O
    O.build()
    th = O.set_threads(0)
    o = O.Scene(np.float32)
    o.add_group("p", "fluid")
    o.resize("p", n)
    o.set_varying("p", "position", pts)
    o.set_radius(r)
    t0 = time.perf_counter()
    o.update()
    offs, _ = o.neighbor_lists(0, 0, n, cap=n * 48)
    sec = time.perf_counter() - t0
    nbar = offs[-1] / n
    return {"value": round(n / sec, 1), "unit": "points/s", "cores": th, "kind": "port",
            "ms_per_search": round(sec * 1e3, 1), "achieved_GBps": round(float((32 + 4 * nbar) * n / sec / 1e9), 2),
            "sample": f"one full search (grid update + neighbour sets of all {n} points)"}


def run_search(peak, n=4_000_000, reps=5, target=40.0, no_cpu=False):
    """Neighbour search only (4M points in the unit cube, uniform and 64
    Gaussian blobs): grid update + the neighbour sets of every point, radius
    calibrated on the device to a mean of `target` neighbours (self
    included).  Algorithmic bytes per point: 32 + 4 n (positions in and
    sorted out, permutation, one 4-byte index per neighbour, CSR offset)."""
    import torch
    from prtcl_gb300.core import DeviceScene
    out = {}
    for dist, seed in (("uniform", 1), ("blobs", 2)):
        pts = scenes.search_points(n, dist, seed=seed)
        d = DeviceScene()
        d.add_group("p", "fluid")
        d.resize("p", n)
        d.set_varying("p", "position", pts)

        def mean_nbrs(r):
            d.set_radius(r)
            d.update()
            return d.nhood.query(0, count_pairs=True) / n

        r = scenes.calibrate_radius(mean_nbrs, n, target)
        nbar = mean_nbrs(r)
        s = torch.cuda.ExternalStream(d.model.stream_handle())
        for _ in range(2):
            d.update()
            d.nhood.query(0)
        d.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nvtx = nvtx_range(f"search_{dist}")
        e0.record(s)
        for _ in range(reps):
            d.update()
            d.nhood.query(0)
        e1.record(s)
        e1.synchronize()
        nvtx_end(nvtx)
        sec = e0.elapsed_time(e1) / 1e3 / reps
        algo = (32 + 4 * nbar) * n
        out[dist] = {"points": n, "radius": r, "mean_neighbours": round(nbar, 3),
                     "ms_per_search": round(sec * 1e3, 3), "points_per_s": round(n / sec, 1),
                     "achieved_GBps": round(algo / sec / 1e9, 1), "frac_of_hbm_peak": round(algo / sec / 1e9 / peak, 4),
                     "algorithmic_bytes": int(algo)}
        del d
        if not no_cpu:
            out[dist]["cpu_baseline"] = search_cpu_baseline(pts, r, n)
    return out


def batched_roofline(prof, sc, before, after, peak, peak_kind, timing):
    """Roofline of the dominant kernel of a batch profile.  A launch of a
    per-step procedure covers every scene; a relaxed-Jacobi sweep covers the
    scenes still iterating, so its items are the scenes' iteration counts
    over the profiled steps times their particle counts."""
    nf = sum(len(x["fluid"]) for x in sc)
    nb = sum(len(x["boundary"]) for x in sc)
    dit = [a["jacobi_iterations"] - b["jacobi_iterations"] for a, b in zip(after, before)]
    jf = sum(k * len(x["fluid"]) for k, x in zip(dit, sc))
    jb = sum(k * len(x["boundary"]) for k, x in zip(dit, sc))
    best = None
    for name, (cnt, ms) in prof.items():
        if name in ("iisph_accel", "iisph_pressure"):
            bf, bb = ALGO_BYTES[name]
            total = bf * jf + bb * jb
        else:
            total = kernel_bytes(name, cnt, nf, nb)
        if total is not None and (best is None or ms > best[2]):
            best = (name, cnt, ms, total)
    if best is None:
        return None
    roof = roofline_block(*best, peak, peak_kind, timing)
    top = max(prof.items(), key=lambda kv: kv[1][1])
    roof["share_of_kernel_time"] = round(best[2] / sum(m for _, m in prof.values()), 4)
    if top[0] != best[0]:
        roof["top_kernel_without_formula"] = {"kernel": top[0], "ms": round(top[1][1], 3)}
    return roof


def batched_cpu_baseline(sc, p, every=32, steps=3):
    """The oracle (reference mode, all host threads) on a fixed subset of the
    batch's scenes (every `every`-th), one after another, `steps` steps each
    after set-up and one warm step."""
    from oracle import oracle as O
    O.build()
    th = O.set_threads(0)
    sub = sc[::every]
    secs, work = 0.0, 0
    for x in sub:
        o = O.Scene(np.float32, fp64_reductions=False)
        driver.setup_dam_break(o, x, p)
        o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=False)
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=False)
        secs += time.perf_counter() - t0
        work += len(x["fluid"]) * steps
    return {"value": round(work / secs, 1), "unit": UNIT, "cores": th, "kind": "port",
            "sample": f"{len(sub)} of the {len(sc)} scenes (one in {every}, {sum(len(x['fluid']) for x in sub)} "
                      f"fluid particles), {steps} steps each after set-up and one warm step"}


def run_batched(count=256, steps=10, warmup=3, plain_steps=5, peak=None, peak_kind=None, no_cpu=False,
                profile_steps=3):
    """256 dam-break scenes, fluid counts log-uniform in 2,000-200,000,
    aspect ratios uniform in [0.5, 2], boxes 2x the fluid extent, parameters
    of the 27k dam break: all scenes stepped together by one batch, against
    the same scenes stepped one after another through the plain
    single-scene path.  Wall time with a device synchronise on both sides
    (the batch step includes its per-step host synchronisations)."""
    from prtcl_gb300.batch import Batch
    from prtcl_gb300.core import DeviceScene
    p = dict(driver.DAM_BREAK_27K)
    sc = scenes.mixed_batch(count=count)
    nf = sum(len(x["fluid"]) for x in sc)
    nb = sum(len(x["boundary"]) for x in sc)
    choice, tuning = tuned("batched", sc, p)
    bt = Batch(p)
    tune.apply(bt, choice)
    ids = [bt.add_scene(x["fluid"], x["boundary"]) for x in sc]
    bt.step(warmup)
    bt.synchronize()
    before = [bt.info(i) for i in ids]
    t0 = time.perf_counter()
    bt.step(steps)
    bt.synchronize()
    secs = time.perf_counter() - t0
    after = [bt.info(i) for i in ids]
    gb = bt.device_bytes() / 1e9
    solves = sum(a["jacobi_solves"] - b["jacobi_solves"] for a, b in zip(after, before))
    iters = sum(a["jacobi_iterations"] - b["jacobi_iterations"] for a, b in zip(after, before))
    capped = sum(a["jacobi_capped"] - b["jacobi_capped"] for a, b in zip(after, before))
    roof, kernels = None, None
    if peak is not None:
        bt.profile(True)
        bt.step(1)
        bt.synchronize()
        bt.profile_read()
        b0 = [bt.info(i) for i in ids]
        nvtx = nvtx_range("batched_profile_pass")
        bt.step(profile_steps)
        bt.synchronize()
        nvtx_end(nvtx)
        prof = bt.profile_read()
        b1 = [bt.info(i) for i in ids]
        bt.profile(False)
        roof = batched_roofline(prof, sc, b0, b1, peak, peak_kind,
                                f"CUDA events around each launch over {profile_steps} extra steps")
        kernels = {k: {"launches": c, "ms_per_step": round(m / profile_steps, 3)} for k, (c, m) in prof.items()}
    del bt
    tp, work = 0.0, 0
    for x in sc:
        cx, _ = tuned("plain", x, p)  # tuned per size class too, so the ratio compares tuned paths
        d = DeviceScene()
        driver.setup_dam_break(d, x, p)
        tune.apply(d.model, cx)
        loop = driver.StepLoop(d, p, device_loop=True)
        for _ in range(warmup):
            loop.step(quiet=True)
        d.synchronize()
        t1 = time.perf_counter()
        for _ in range(plain_steps):
            loop.step(quiet=True)
        d.synchronize()
        tp += time.perf_counter() - t1
        work += len(x["fluid"]) * plain_steps
        del loop, d
    v, vp = nf * steps / secs, work / tp
    return {"workload": f"{count} dam-break scenes, fluid log-uniform 2k-200k (seed 3), IISPH dt 1e-3 s",
            "fluid_particles": nf, "boundary_particles": nb, "steps": steps, "warmup": warmup,
            "value": round(v, 1), "unit": UNIT, "ms_per_step": round(secs * 1e3 / steps, 3),
            "plain_value": round(vp, 1), "plain_sample": f"{plain_steps} steps of each scene after {warmup} warm-up",
            "batched_over_plain": round(v / vp, 2), "jacobi_iterations_mean": round(iters / max(solves, 1), 3),
            "jacobi_capped_steps": int(capped), "device_GB": round(gb, 2), "roofline": roof, "kernels": kernels,
            "tuning": tuning,
            "cpu_baseline": None if no_cpu else batched_cpu_baseline(sc, p)}


def run_serving(count=48, rate=4.0):
    """Poisson arrivals (rate/s, seed 4) of dam-break requests, fluid
    log-uniform 5k-500k, steps uniform 100-1000, IISPH + WKBB18 viscosity;
    continuous batching under a 120 GB device budget."""
    from prtcl_gb300.batch import Batch
    from prtcl_gb300.serve import Server, poisson_requests, report
    p = dict(driver.DAM_BREAK_27K, viscosity=True)
    reqs = poisson_requests(count, rate, seed=4)
    for r in reqs:
        r.scene()  # requests arrive with their particles
    srv = Server(Batch, p, budget_bytes=120e9, keep_results=False)
    done = srv.run(reqs)
    rep = report(done, srv.makespan, srv.particle_steps, eta=p["eta"])
    rep.update({"workload": f"{count} requests, Poisson {rate}/s, fluid log-uniform 5k-500k, "
                            "steps uniform 100-1000, IISPH + WKBB18", "unit": UNIT, "batch_steps": srv.steps_run,
                "budget_GB": 120})
    return rep


def run_reference(args, rank, world, dist):
    """Reference arm: the CPU restatement of the reference's OpenMP path on
    all host threads (the reference itself does not build here: Eigen,
    Boost, Lua and its submodules are absent)."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    th = O.set_threads(0)
    sc, p = workload(args)
    nf = len(sc["fluid"])
    o = O.Scene(np.float32, fp64_reductions=False)
    driver.setup_dam_break(o, sc, p)
    visc = p.get("viscosity", False)
    for _ in range(args.warmup):
        o.step(permute=False, max_iters=p["max_iters"], eta=p["eta"], viscosity=visc)
    t0 = time.perf_counter()
    its = []
    for k in range(args.steps):
        st = o.step(permute=((k + 1) % p["permute_every"] == 0), max_iters=p["max_iters"], eta=p["eta"],
                    viscosity=visc)
        its.append(st["jacobi_iterations"])
    secs = time.perf_counter() - t0
    v = nf * args.steps / secs
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lattice dam break generated in-process)",
            "config": config_of(args, nf, len(sc["boundary"]), world),
            "solver": {"jacobi_iterations_mean": float(np.mean(its))},
            "cpu_baseline": {"value": round(v, 1), "unit": UNIT, "cores": th, "kind": "port",
                             "sample": f"{args.steps} full steps after {args.warmup} warm-up steps"},
            "e2e": {"value": round(v, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="prtcl_gb300", choices=["prtcl_gb300", "reference"])
    ap.add_argument("--config", default="1m", choices=["1m", "27k"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--profile-steps", type=int, default=3)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the neighbour-search, batched-scenes and serving measurements")
    ap.add_argument("--extras", type=lambda v: v.split(","), default=None, metavar="LEG,...",
                    help="run only these of the extra legs: long_run, plain_27k, search, batched, serving")
    ap.add_argument("--no-tune", action="store_true",
                    help="headline workload with the default knob values instead of the autotuner's choice")
    ap.add_argument("--knob", action="append", default=[], metavar="NAME=VALUE",
                    help="override one autotuner knob of the headline workload (repeatable), e.g. staging=1")
    args = ap.parse_args()
    knobs = {}
    for kv in args.knob:
        name, _, val = kv.partition("=")
        if name not in tune.VALUES or not val.lstrip("-").isdigit() or int(val) not in tune.VALUES[name]:
            ap.error(f"--knob {kv}: knobs are " + ", ".join(f"{k}={'/'.join(map(str, v))}"
                                                            for k, v in tune.VALUES.items()))
        knobs[name] = int(val)
    args.knob = knobs
    legs = ("long_run", "plain_27k", "search", "batched", "serving")
    if args.extras is not None and not set(args.extras) <= set(legs):
        ap.error("--extras: legs are " + ", ".join(legs))
    if args.warmup < 3 and args.impl != "reference":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, world, dist = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        from prtcl_gb300 import build
        build.build()
        run_ours(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
