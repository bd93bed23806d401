#!/usr/bin/env python3
"""PatchMatch MVS depth-map benchmark on one GPU per rank.

One step = one complete depth map (random init, initial costs, iterations x 4 sweeps) of the
1280x720 reference with 10 source views, 15x15 window, 5 iterations (box200_1280x720: a seeded
synthetic scene of 12 planes and 200 boxes standing in for the benchmark's data). The metric is
G cost-evals/s: NCC evaluations of one (pixel, hypothesis, source view) over the w x w window,
counted as the reference algorithm performs them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same algorithm (FP32, all host threads) on a
bounded sample of the same workload; the reference's own CUDA build does not compile with
CUDA 13 (texture references) and needs OpenCV and Boost.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="box200_1280x720")
    ap.add_argument("--precision", type=int, default=0, help="0 = FP32, 1 = FP16 texels (mixed)")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched (24 references) and full-scale (8 x 3072x2048) summaries")
    ap.add_argument("--profile", type=int, default=None, metavar="DIR",
                    help="run only the initial state and one sweep in direction DIR (for ncu)")
    ap.add_argument("--threads-per-line", type=int, default=0)
    ap.add_argument("--planes", type=int, default=0, help="--profile: slanted planes per pixel (1)")
    ap.add_argument("--learned", type=int, default=0, metavar="SWEEPS",
                    help="batched workloads: learned initialisation followed by SWEEPS sweeps")
    ap.add_argument("--profile-net", action="store_true",
                    help="run only the proposal network's forward pass on the workload (for ncu)")
    return ap.parse_args()


def run_profile(args):
    """Initial depth and costs, then one sweep: the launches an ncu capture looks at. A first
    engine tunes the warps per line (the choice is remembered per shape); the second one's
    sweep, inside the NVTX range "pm_profile", is the capture: its interior and edge launches
    (`ncu --nvtx --nvtx-include "pm_profile/" -k regex:sweep_kernel -c 2`)."""
    import torch
    from patchmatch_cuda_gb300 import Engine, scene
    wl = scene.WORKLOADS[args.workload]
    sv = scene.make_views(wl)
    params = wl.params(precision=args.precision, threads_per_line=args.threads_per_line, planes=args.planes)
    tune = Engine(sv.images, sv.ref_id, params)
    tune.init_depth()
    tune.compute_costs(1)
    tune.run_sweep(args.profile, 4 + args.profile, wl.num_samples)
    tune.close()
    eng = Engine(sv.images, sv.ref_id, params)
    eng.init_depth()
    eng.compute_costs(1)
    torch.cuda.nvtx.range_push("pm_profile")
    eng.run_sweep(args.profile, 4 + args.profile, wl.num_samples)
    torch.cuda.nvtx.range_pop()
    st = eng.stats()
    print(json.dumps({"sweep_ms": st.ms_sweeps, "cost_evals": st.cost_evals,
                      "threads_per_line": st.threads_per_line}))
    eng.close()
    return 0


def run_profile_net(args):
    """The proposal network's forward pass on the workload's plane-sweep input, 5 times."""
    import torch
    from patchmatch_cuda_gb300 import Engine, proposal, scene
    wl = scene.WORKLOADS[args.workload]
    sv = scene.make_views(wl)
    eng = Engine(sv.images, sv.ref_id, wl.params())
    net = proposal.for_engine(eng)
    hp, wp = eng.proposal_shape()
    x = torch.empty((hp, wp, 17), device="cuda")
    y = torch.empty((hp, wp, 2), device="cuda")
    eng.proposal_input(x.data_ptr())
    for _ in range(5):
        net.forward(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    print(json.dumps({"net_input": [hp, wp, 17], "gflop_per_forward": proposal.forward_flops(hp, wp) / 1e9}))
    net.close()
    eng.close()
    return 0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while active."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def dist_setup():
    """Ranks are independent replicas (one reference view each): the only exchange is the
    timing gather at the end, over gloo on the host -- no device collective."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def allreduce_max_sum(world: int, vmax: float, vsum: float):
    if world == 1:
        return vmax, vsum
    import torch
    import torch.distributed as dist
    t = torch.tensor([vmax], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    s = torch.tensor([vsum], dtype=torch.float64)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    return float(t.item()), float(s.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def profiled_traffic(workload: str):
    """DRAM bytes per sweep (its interior and edge launches together) from the committed ncu
    summary, if one exists."""
    f = ROOT / "profiles" / f"sweep_kernel_{workload}.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_sweep:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# The CPU legs (the GPU arm's cpu_baseline and --impl reference) time the same sample: one
# top-to-bottom sweep with numOfSamples views from the random initial state, over CPU_BLOCKS
# blocks of 32 columns spread evenly across the image, with the GPU arm's sampler.
CPU_BLOCKS = 4


def cpu_sample_blocks(width: int, n_blocks: int = CPU_BLOCKS) -> list[int]:
    total = (width + 31) // 32
    n = min(n_blocks, total)
    return sorted({int(round((i + 0.5) * total / n - 0.5)) for i in range(n)})


class CpuSweep:
    """The CPU baseline: the FP32 OpenMP restatement of the reference's per-pixel algorithm
    (pm_oracle.c compiled with real = float; lines of a sweep in parallel), the reported
    baseline the reference's missing CPU path calls for. (The reference's own kernels also run
    on the host, oracle/ref_host.cpp, but as a thread-per-lane emulation of GPU code: they pin
    parity, and timing them would flatter the GPU.) Initial state: the random initial depth and
    every view's cost on the sampled columns, set up outside the timed region."""

    def __init__(self, sv, wl, sampler: int):
        import numpy as np
        from oracle import pm_oracle
        self.wl = wl
        self.blocks = cpu_sample_blocks(wl.width)
        self.orc = pm_oracle.from_images(sv.images, sv.ref_id, wl.params(sampler=sampler), fp32=True)
        d0 = self.orc.init_depth()
        cols = np.concatenate([np.arange(32 * b, min(32 * b + 32, wl.width)) for b in self.blocks])
        c0 = np.full((wl.height, wl.width, len(sv.images) - 1), 2.0)
        xs, ys = np.meshgrid(cols, np.arange(wl.height))
        xs, ys = xs.ravel(), ys.ravel()
        for v in range(c0.shape[2]):
            c0[ys, xs, v] = self.orc.ncc_batch(xs, ys, np.full(xs.shape, v), d0[ys, xs], 1)
        self.d0, self.c0 = d0, c0
        self.sampler = sampler

    def step(self):
        """One timed sample: (cost-evals, seconds)."""
        d, c = self.d0.copy(), self.c0.copy()
        evals, elapsed = 0, 0.0
        for b in self.blocks:
            t = time.perf_counter()
            evals += self.orc.sweep(d, c, 1, 1, self.wl.num_samples, lines=(32 * b, 32 * b + 32))
            elapsed += time.perf_counter() - t
        return evals, elapsed

    def describe(self) -> dict:
        from oracle import pm_oracle
        return {"kind": "port", "cores": pm_oracle.num_threads(True),
                "sample": f"columns {', '.join(f'{32 * b}-{32 * b + 31}' for b in self.blocks)} of "
                          f"{self.wl.width} ({len(self.blocks)} blocks of 32 lines): one top-to-bottom sweep "
                          f"with S={self.wl.num_samples} from the random initial state, "
                          f"{'texture-unit' if self.sampler == 1 else 'exact'} bilinear weights",
                "code": "FP32 OpenMP restatement of the reference's kernels (oracle/pm_oracle.c, lines in parallel)"}


def cpu_baseline(sv, wl, sampler: int, seconds: float) -> dict:
    """The CPU leg of the GPU arm: CpuSweep's sample, repeated for about `seconds`."""
    cpu = CpuSweep(sv, wl, sampler)
    evals, elapsed, reps = 0, 0.0, 0
    while reps < 1 or elapsed < seconds:
        n, dt = cpu.step()
        evals += n
        elapsed += dt
        reps += 1
    out = {"value": evals / elapsed / 1e9, "unit": "G cost-evals/s", "seconds": round(elapsed, 3), "steps": reps}
    out.update(cpu.describe())
    return out


def run_reference(args):
    """The reference arm. The reference has no CPU path and its CUDA build does not compile with
    CUDA 13 (texture references), so this is the OpenMP FP32 restatement of its per-pixel
    algorithm on all host threads, each step the CPU legs' bounded sample of the workload, with
    the GPU arm's sampler. Rank 0 alone runs it."""
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    from patchmatch_cuda_gb300 import scene
    wl = scene.WORKLOADS[args.workload]
    sv = scene.make_views(wl)
    sampler = wl.params().sampler  # the GPU arm's (the default: texture-unit filtering)
    cpu = CpuSweep(sv, wl, sampler)
    times, evals = [], []
    for step in range(args.warmup + args.steps):
        n, dt = cpu.step()
        if step >= args.warmup:
            times.append(dt)
            evals.append(n)
    value = sum(evals) / sum(times) / 1e9
    desc = cpu.describe()
    print(json.dumps({
        "impl": "reference", "metric": "G cost-evals/s", "value": value, "unit": "G cost-evals/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": synthetic_data(wl),
        "config": static_config(args, wl, sampler),
        "cpu_baseline": dict(desc, value=value, unit="G cost-evals/s"),
        "e2e": {"value": value, "unit": "G cost-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)
    return 0


def synthetic_data(wl) -> str:
    return (f"synthetic (seeded scene: {wl.n_planes} planes + {wl.n_boxes} boxes, 1 ref + {wl.n_src} sources "
            f"on a 15 degree arc)")


def static_config(args, wl, sampler: int) -> dict:
    """The workload as both arms name it (nothing measured)."""
    return {"workload": args.workload, "width": wl.width, "height": wl.height, "n_src": wl.n_src,
            "window": 2 * wl.half_window + 1, "iterations": wl.iterations, "num_samples": wl.num_samples,
            "depth_range": [wl.depth_near, wl.depth_far], "prefilter": "none" if wl.prefilter == 0 else "box, sigma 1",
            "precision": "fp32" if args.precision == 0 else "mixed",
            "sampler": "texture-unit bilinear (the reference's fetch)" if sampler == 1 else "exact gather",
            "l2": "flushed before each depth map (256 MiB write, outside the timed events)"}


def _engine_available() -> bool:
    try:
        from patchmatch_cuda_gb300 import _native
        _native.load_engine()
        return True
    except Exception:
        return False


def run_ours(args):
    import numpy as np
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    from patchmatch_cuda_gb300 import Engine, _native, scene
    from patchmatch_cuda_gb300 import build as engine_build
    if not _native.ENGINE_PATH.exists():
        engine_build.build()
    wl = scene.WORKLOADS[args.workload]
    sv = scene.make_views(wl, seed=wl.seed + rank)  # each rank its own reference view (replicas)
    params = wl.params(precision=args.precision, gpu_id=local)
    eng = Engine(sv.images, sv.ref_id, params)
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    for _ in range(max(args.warmup, 0)):
        eng.run()
    evals_per_map = eng.stats().cost_evals
    evals_done_per_map = eng.stats().cost_evals_done
    # initial depth and costs, then each sweep: its interior lines and the lines within a
    # half-window of an image edge as two launches (one where every line is an edge line)
    sweep_launches = [2 if (wl.height if d % 2 == 0 else wl.width) > 2 * wl.half_window else 1 for d in range(4)]
    launches_per_map = 2 + wl.iterations * sum(sweep_launches)

    barrier(world)
    torch.cuda.synchronize()
    step_ms = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.run_async()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(world)
    total_ms, total_evals = allreduce_max_sum(world, sum(step_ms), float(evals_per_map * args.steps))
    depth = eng.depth()
    bad = scene.bad_pixel_rate(depth, sv.gt_depth)
    rel_err = np.abs(depth - sv.gt_depth) / sv.gt_depth
    rel_err = rel_err[np.isfinite(rel_err)]

    # dominant kernel: every sweep of one schedule timed on the engine's stream
    eng.init_depth()
    eng.compute_costs(1)
    sweep_ms, sweep_evals, sweep_done = [], [], []
    prev, prev_done = eng.stats().cost_evals, eng.stats().cost_evals_done
    for it in range(wl.iterations):
        for d in range(4):
            eng.run_sweep(d, 4 * it + d, 1 if it == 0 else wl.num_samples)
            st = eng.stats()
            sweep_ms.append(st.ms_sweeps)
            sweep_evals.append(st.cost_evals - prev)
            sweep_done.append(st.cost_evals_done - prev_done)
            prev, prev_done = st.cost_evals, st.cost_evals_done
    w = 2 * wl.half_window + 1
    flop_per_eval = 16 * w * w + 36
    launch_s = 1e-3 * sum(sweep_ms) / len(sweep_ms)
    flop_per_launch = flop_per_eval * sum(sweep_evals) / len(sweep_evals)
    props = torch.cuda.get_device_properties(local)
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = flop_per_launch / launch_s / 1e12
    flop_per_launch_done = flop_per_eval * sum(sweep_done) / len(sweep_done)
    achieved_done = flop_per_launch_done / launch_s / 1e12
    samples_per_s = (flop_per_launch / flop_per_eval) * w * w / launch_s
    samples_done_per_s = (flop_per_launch_done / flop_per_eval) * w * w / launch_s
    tex_peak_nominal = props.multi_processor_count * 4 * sm_max * 1e6
    tp = C.c_double(0.0)
    st_tp = _native.load_engine().pm_texture_peak(C.byref(tp))
    tex_peak = tp.value if st_tp == 0 and tp.value > 0 else tex_peak_nominal

    # end to end through the C ABI with host buffers: create (upload, prefilter, textures),
    # run, read the depth map back, destroy
    h2d = sum(im.image.nbytes for im in sv.images)
    d2h = wl.width * wl.height * 4
    e2e_times = []
    for i in range(1 + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = Engine(sv.images, sv.ref_id, params)
        e.run()
        _ = e.depth()
        e.close()
        torch.cuda.synchronize()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e_max, _ = allreduce_max_sum(world, sum(e2e_times), 0.0)
    e2e_value = total_evals / e2e_max / 1e9

    tpl = eng.stats().threads_per_line
    wpl = list(eng.stats().warps_per_line)
    # variants of the same workload, each one depth map timed once after a warm-up run
    variants = {}
    for name, over in [("f32_texels_box_prefilter", dict(prefilter=1)),
                       ("f16_texels_box_prefilter", dict(prefilter=1, precision=1)),
                       ("exact_sampler", dict(sampler=0)),
                       # slanted planes per pixel (no counterpart in the reference)
                       ("slanted_planes", dict(planes=1))]:
        ev = Engine(sv.images, sv.ref_id, wl.params(gpu_id=local, **over))
        ev.run()
        ev.run()
        st = ev.stats()
        dv = ev.depth()
        rel = np.abs(dv - sv.gt_depth) / sv.gt_depth
        variants[name] = {"ms_per_depth_map": st.ms_total, "g_cost_evals_per_s": st.cost_evals / st.ms_total / 1e6,
                          "bad_pixel_pct_1pct": round(100 * scene.bad_pixel_rate(dv, sv.gt_depth), 3),
                          "bad_pixel_pct_0p2pct": round(100 * float(np.mean(rel[np.isfinite(rel)] > 0.002)), 3),
                          "median_rel_err_pct": round(100 * float(np.median(rel[np.isfinite(rel)])), 4)}
        ev.close()
    learned = learned_vs_plain(sv, wl, local, flush, max(args.steps, 3))
    batched = None
    if not args.no_extras:
        eng.close()
        eng = None
        batched = {"batch24_mixed": measure_batch("batch24_mixed", local, rank, reps=2),
                   "full8_3072x2048": measure_batch("full8_3072x2048", local, rank, reps=1)}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sv, wl, params.sampler, args.cpu_seconds)
    if eng is not None:
        eng.close()

    if rank == 0:
        traffic = profiled_traffic(args.workload)
        out = {
            "metric": "G cost-evals/s", "value": total_evals / (total_ms * 1e-3) / 1e9, "unit": "G cost-evals/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("u8 texels, f32 arithmetic" if wl.prefilter == 0 else "f32") if args.precision == 0
            else "f16 texels, f32 arithmetic",
            "data": synthetic_data(wl),
            "config": static_config(args, wl, params.sampler),
            "depth_map": {
                "ms": total_ms / args.steps,
                "cost_evals": evals_per_map,
                "cost_evals_computed": evals_done_per_map,
                "cost_evals_note": "cost_evals counts the NCC evaluations the reference's algorithm performs "
                                   "(2 per view sample, every view on a refresh); cost_evals_computed those the "
                                   "engine evaluates (a view drawn twice or refreshed at a depth it was just "
                                   "evaluated at reuses the result)",
                "g_cost_evals_computed_per_s": evals_done_per_map / (total_ms / args.steps * 1e-3) / 1e9,
                "bad_pixel_pct_1pct": round(100 * bad, 3),
                "bad_pixel_pct_0p2pct": round(100 * float(np.mean(rel_err > 0.002)), 3),
                "median_rel_err_pct": round(100 * float(np.median(rel_err)), 4),
                "threads_per_line": tpl,
                "warps_per_line": {"vertical": {"interior": wpl[0], "edge_lines": wpl[1]},
                                   "horizontal": {"interior": wpl[2], "edge_lines": wpl[3]}},
            },
            "roofline": {
                "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": traffic,
                "kernel": "sweep_kernel", "launch_ms": 1e3 * launch_s,
                "flop_per_launch": flop_per_launch,
                "peak_source": "nominal FP32: SMs x 128 lanes x 2 x sm_max_mhz (MEASURED_PEAKS.json has no FP32 figure)",
                "achieved_computed": achieved_done, "frac_computed": achieved_done / fp32_peak,
                "flop_per_launch_computed": flop_per_launch_done,
                "tex_samples_per_s": samples_per_s, "tex_peak_samples_per_s": tex_peak,
                "tex_frac": samples_per_s / tex_peak,
                "tex_samples_computed_per_s": samples_done_per_s, "tex_frac_computed": samples_done_per_s / tex_peak,
                "tex_peak_source": "measured live by pm_texture_peak (layered u8 bilinear fetches in the NCC's "
                                   "access pattern, 64 warps per SM); nominal 4 per clock per SM = "
                                   f"{tex_peak_nominal / 1e9:.0f} G/s",
                "note": "achieved / tex_frac count the reference's algorithmic evaluations; the _computed "
                        "readings count the evaluations the kernel computes. A sweep is two concurrent launches "
                        "of sweep_kernel (interior lines, lines along the edges): launch_ms, flop_per_launch "
                        "and traffic are per sweep, both launches together",
            },
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "G cost-evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_max / args.steps},
            "variants": variants,
            "learned_vs_plain": learned,
            "batched": batched,
            "gpu_launches": launches_per_map * args.steps,
            "clocks": clocks.summary(),
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _timed_runs(eng, flush, reps):
    """Median ms of `reps` depth maps on the engine's stream (L2 flushed before each)."""
    import torch
    stream = torch.cuda.ExternalStream(eng.stream())
    eng.run()
    ms = []
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.run_async()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.median(ms)


def learned_vs_plain(sv, wl, device, flush, reps):
    """The learned proposal against plain PatchMatch on the same reference: ms per depth map
    (end of upload to depth ready, inputs resident) and bad-pixel rate against ground truth,
    plus the network's forward pass against the BF16 tensor peak (2 FLOP per MAC)."""
    import torch
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, Engine, proposal, scene
    if not proposal.WEIGHTS.exists():
        return None
    out = {}
    runs = [("plain_20_sweeps", dict()),
            ("learned_4_sweeps", dict(init_mode=INIT_PROPOSAL, num_sweeps=4, perturbation=0.05)),
            ("learned_8_sweeps", dict(init_mode=INIT_PROPOSAL, num_sweeps=8, perturbation=0.05)),
            # control: the learned schedule with every pixel from the random initialisation
            # (confidence threshold 1), i.e. what the network itself contributes
            ("control_random_init_4_sweeps", dict(init_mode=INIT_PROPOSAL, proposal_threshold=1.0, num_sweeps=4,
                                                  perturbation=0.05)),
            ("control_random_init_8_sweeps", dict(init_mode=INIT_PROPOSAL, proposal_threshold=1.0, num_sweeps=8,
                                                  perturbation=0.05)),
            # the refinement step after the last sweep (the reference's never-launched kernel's
            # 10 trials of sigma 0.05, and a finer 16 x 0.02)
            ("plain_20_sweeps_refine_10x0.05", dict(refine_trials=10, refine_sigma=0.05)),
            ("learned_4_sweeps_refine_10x0.05", dict(init_mode=INIT_PROPOSAL, num_sweeps=4, perturbation=0.05,
                                                     refine_trials=10, refine_sigma=0.05)),
            ("learned_4_sweeps_refine_16x0.02", dict(init_mode=INIT_PROPOSAL, num_sweeps=4, perturbation=0.05,
                                                     refine_trials=16, refine_sigma=0.02))]
    params = proposal.load_params()
    net_ms = gflop = None
    net_quality = None
    for name, over in runs:
        e = Engine(sv.images, sv.ref_id, wl.params(gpu_id=device, **over))
        learned = over.get("init_mode") == INIT_PROPOSAL
        net = proposal.for_engine(e, params) if learned else None
        ms = _timed_runs(e, flush, reps)
        out[name] = {"ms_per_depth_map": round(ms, 3),
                     "bad_pixel_pct_1pct": round(100 * scene.bad_pixel_rate(e.depth(), sv.gt_depth), 3),
                     "sweeps": over.get("num_sweeps", 4 * wl.iterations),
                     "refine": [over["refine_trials"], over["refine_sigma"]] if "refine_trials" in over else None,
                     "cost_evals": e.stats().cost_evals}
        if net is not None and net_ms is None:
            # the network alone: forward of the 17-channel plane-sweep input
            hp, wp = e.proposal_shape()
            x = torch.empty((hp, wp, 17), device="cuda")
            y = torch.empty((hp, wp, 2), device="cuda")
            e.proposal_input(x.data_ptr())
            for _ in range(3):
                net.forward(x.data_ptr(), y.data_ptr())
            t = []
            for _ in range(10):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                net.forward(x.data_ptr(), y.data_ptr(), torch.cuda.current_stream().cuda_stream)
                e1.record()
                e1.synchronize()
                t.append(e0.elapsed_time(e1))
            net_ms = statistics.median(t)
            gflop = proposal.forward_flops(hp, wp) / 1e9
            # the network's own prediction: confident fraction and its depth error there (4x4
            # blocks, harmonic mean of the ground truth)
            o = y.cpu().numpy().astype(np.float64)
            h4, w4 = e.height // 4, e.width // 4
            conf, s_ = o[:h4, :w4, 1], o[:h4, :w4, 0]
            thr = e.params.proposal_threshold
            inv_far, inv_range = 1.0 / wl.depth_far, 1.0 / wl.depth_near - 1.0 / wl.depth_far
            dn = 1.0 / (inv_far + s_ * inv_range)
            g4 = 1.0 / (1.0 / sv.gt_depth[:4 * h4, :4 * w4].reshape(h4, 4, w4, 4)).mean(axis=(1, 3))
            rel = np.abs(dn - g4) / g4
            net_quality = {"confident_fraction": round(float(np.mean(conf >= thr)), 4),
                           "median_rel_err_pct_confident": round(100 * float(np.median(rel[conf >= thr])), 2)
                           if np.any(conf >= thr) else None,
                           "median_rel_err_pct_all": round(100 * float(np.median(rel)), 2)}
        e.close()
        if net is not None:
            net.close()
    base = out["plain_20_sweeps"]["ms_per_depth_map"]
    for name, _ in runs[1:]:
        out[name]["speedup_vs_plain"] = round(base / out[name]["ms_per_depth_map"], 3)
    peak = float(measured_peaks().get("bf16_tflops", 1900.0))
    tflops = gflop / net_ms if net_ms else None
    out["network_forward"] = {"ms": round(net_ms, 4), "gflop": round(gflop, 3), "tflops": round(tflops, 3),
                              "peak_tflops": peak, "frac_of_bf16_peak": round(tflops / peak, 5),
                              "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"}
    out["network_prediction"] = net_quality
    return out


def measure_fusion(engines, refs, warmup: int, reps: int) -> dict:
    """Consistency filtering + fusion over the batch's depth maps, read in place (pm_fusion):
    device time of the three kernels by CUDA events, the HBM roofline of the algorithmic bytes
    (per pixel: its depth read once, fused depth and count written, 4 + 4 + 1 bytes; per kept
    pixel: fused depth read again and a 16-byte point written) and what the filter keeps."""
    from patchmatch_cuda_gb300 import Fusion, default_fuse_params, scene
    fus = Fusion(engines)
    params = default_fuse_params()
    for _ in range(warmup):
        fus.run(params)
    check, total = [], []
    for _ in range(reps):
        fus.run(params)
        inf = fus.info()
        check.append(inf["ms_check"])
        total.append(inf["ms_total"])
    launches = fus.info()["launches"]
    n_pts = fus.info()["points"]
    pix = sum(e.width * e.height for e in engines)
    checks = pix * (len(engines) - 1)
    kept_bad, kept_share, raw_bad = [], [], []
    for i, (e, sv) in enumerate(zip(engines, refs)):
        f, _ = fus.depth(i)
        gt = sv.gt_depth
        valid = gt > 0
        k = (f > 0) & valid
        kept_share.append(float(k.sum() / max(valid.sum(), 1)))
        kept_bad.append(float(np.mean(np.abs(f[k] - gt[k]) / gt[k] > 0.01)) if k.any() else 0.0)
        raw_bad.append(scene.bad_pixel_rate(e.depth(), gt))
    fus.close()
    ms_total = float(np.median(total))
    algo_bytes = pix * 9 + n_pts * 20
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    achieved = algo_bytes / (ms_total * 1e-3) / 1e9
    return {"params": {"max_reproj_px": params.max_reproj_px, "max_rel_depth": round(params.max_rel_depth, 6),
                       "min_consistent": params.min_consistent},
            "ms_check": round(float(np.median(check)), 4), "ms_total": round(ms_total, 4), "launches": launches,
            "pixel_checks_per_s_G": round(checks / (float(np.median(check)) * 1e-3) / 1e9, 2),
            "points": int(n_pts), "kept_share": round(float(np.mean(kept_share)), 4),
            "bad_pixel_pct_1pct_kept": round(100 * float(np.mean(kept_bad)), 3),
            "bad_pixel_pct_1pct_raw": round(100 * float(np.mean(raw_bad)), 3),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4) if hbm else None, "traffic": None,
                         "algorithmic_bytes": int(algo_bytes)}}


def measure_batch(workload: str, device: int, rank: int, reps: int, warmup: int = 1, learned: int = 0,
                  with_fusion: bool = True, clocks=None) -> dict:
    """A batched workload on one GPU, timed with CUDA events on the batch's stream:
      batch24_mixed     24 references of 640x480 / 1280x720 / 1920x1080 with 6-12 sources each
                        from one scene of 40 planes + 500 boxes;
      full8_3072x2048   8 references of 3072x2048 with 20 sources each, 19x19 window, depth
                        [0.5, 50], one scene of 60 planes + 2000 boxes.
    The whole schedule is one CUDA graph: one launch per sweep over all references of a group."""
    import torch
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, Batch, Engine, proposal, scene
    full = workload == "full8_3072x2048"
    refs = scene.make_full_batch() if full else scene.make_batch(seed=33 + rank)
    over = dict(init_mode=INIT_PROPOSAL, num_sweeps=learned, perturbation=0.05) if learned else {}
    engines = [Engine(sv.images, sv.ref_id, sv.workload.params(gpu_id=device, **over)) for sv in refs]
    nets = {}
    if learned:   # one network per reference size, shared (the batch runs them in turn)
        params = proposal.load_params()
        for e in engines:
            shape = e.proposal_shape()
            if shape not in nets:
                nets[shape] = proposal.ProposalNet(1, *shape)
                nets[shape].set_params(params)
            e.set_proposal(nets[shape])
    stream = torch.cuda.ExternalStream(engines[0].stream())
    batch = Batch(engines)                       # tunes warps per line, captures the graph
    info = batch.info()
    for _ in range(max(warmup, 1)):
        batch.run()
    evals = sum(e.stats().cost_evals for e in engines)
    evals_done = sum(e.stats().cost_evals_done for e in engines)
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    bad = [scene.bad_pixel_rate(e.depth(), sv.gt_depth) for e, sv in zip(engines, refs)]
    fusion = measure_fusion(engines, refs, 3, 5) if with_fusion else None
    out = {"workload": workload, "references": len(refs),
           "init": f"learned proposal + {learned} sweeps" if learned else "random (plain PatchMatch)",
           "sizes": sorted({f"{sv.workload.width}x{sv.workload.height}" for sv in refs}),
           "sources": [sv.workload.n_src for sv in refs], "window": 2 * refs[0].workload.half_window + 1,
           "iterations": refs[0].workload.iterations, "reps": reps,
           "ms_per_batch": sum(ms) / len(ms), "ms_per_batch_each": [round(x, 2) for x in ms],
           "cost_evals_per_batch": evals, "cost_evals_computed_per_batch": evals_done,
           "g_cost_evals_per_s": evals / (sum(ms) / len(ms) * 1e-3) / 1e9,
           "mean_bad_pixel_pct_1pct": round(100 * float(np.mean(bad)), 3),
           "launches": info["launches"], "warps_per_line": info["warps_per_line"],
           "texels": "u8 (the 8-bit inputs; half the bytes of FP16)",
           "schedule": "one CUDA graph per batch; one launch per sweep over all references of a group",
           "fusion": fusion}
    if clocks is not None:
        out["clocks"] = clocks.summary()
    batch.close()
    for e in engines:
        e.close()
    for n in nets.values():
        n.close()
    return out


def run_batched(args):
    """A batched workload (measure_batch) as the bench line."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    barrier(world)
    with ClockSampler(local) as clocks:
        res = measure_batch(args.workload, local, rank, args.steps, args.warmup, args.learned)
    barrier(world)
    total_ms, total_evals = allreduce_max_sum(world, res["ms_per_batch"] * args.steps,
                                              float(res["cost_evals_per_batch"] * args.steps))
    full = args.workload == "full8_3072x2048"
    if rank == 0:
        print(json.dumps({
            "metric": "G cost-evals/s", "value": total_evals / (total_ms * 1e-3) / 1e9, "unit": "G cost-evals/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8 texels, f32 arithmetic",
            "data": "synthetic (one scene of 60 planes + 2000 boxes)" if full else "synthetic (one scene of 40 planes + 500 boxes)",
            "config": {k: res[k] for k in ("workload", "references", "init", "sizes", "sources", "window", "iterations",
                                          "texels", "schedule")},
            "batch": {k: v for k, v in res.items() if k not in ("workload", "sizes", "sources")},
            "gpu_launches": res["launches"] * args.steps, "clocks": clocks.summary(),
        }), flush=True)
    return 0


def main():
    args = parse_args()
    if args.workload in ("batch24_mixed", "full8_3072x2048") and args.impl == "ours":
        import numpy as np  # noqa: F401
        return run_batched(args)
    if args.profile is not None:
        return run_profile(args)
    if args.profile_net:
        return run_profile_net(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
