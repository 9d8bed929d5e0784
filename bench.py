#!/usr/bin/env python
"""Frames/s of the image-formation path on the EPIFM-defocus workload.

Workload (one step = one camera frame): 20,000 emitters with x, y uniform over
a 512 x 512 field of 160 nm pixels (81.92 um) and z uniform in [-1, 1] um, half
diffusing at D = 0.01 um^2/s and half at 1.0 um^2/s; EPI illumination; 10 ms
exposure in 20 sub-steps; photobleaching with a 2 s mean lifetime; sCMOS camera
with per-pixel readout sigma ~ lognormal(ln 1.5 e-, 0.4) and per-pixel offset
~ N(100, 5); 12-bit ADC.  Synthetic, seeded inputs of these shapes.

``value``: frames/s with trajectories resident in HBM (sub-step records, tile
binning, splat, camera + ADC per frame; outputs stay on the device).
``e2e``: frames/s through ``scopyon_gb300.generate_images`` with host
trajectories (pinned H2D of each frame's sub-steps, D2H of the ADC frame).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_EMIT = 20000
IMAGE = 512
SUBSTEPS = 20
E2E_FRAMES = 20  # frames timed through the public API with host trajectories, per run
E2E_RUNS = 5  # sequences timed; the e2e value is their median
EXPOSURE = 0.010
PX = 16e-6 / 100
HALF = IMAGE * PX / 2
METRIC = "frames/s, 512^2 px 20k emitters (EPIFM defocus, sCMOS)"
WORKLOAD = "epifm_defocus_512px_20k_emitters_20substeps_scmos"


def workload_dict():
    """The ``config`` object of the JSON line (the same in both arms)."""
    return {"workload": WORKLOAD + ("_z0.1um_profiling" if Z_HALF < 1e-6 else ""),
            "n_emitters": N_EMIT, "image": [IMAGE, IMAGE], "substeps": SUBSTEPS,
            "exposure_s": EXPOSURE, "pixel_nm": PX * 1e9,
            "camera": "sCMOS per-pixel sigma, 12-bit", "psf": "Born-Wolf TRITC",
            "depth_range_um": [-Z_HALF * 1e6, Z_HALF * 1e6],
            "D_um2_per_s": [0.01, D_FAST * 1e12], "bleaching_mean_lifetime_s": 2.0,
            "l2": "inputs larger than L2 (PSF tables of every depth key, several GB)"}


def workload_config():
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "light_source": {"angle": 0.0},
        "detector": {"type": "CMOS", "image_size": [IMAGE, IMAGE], "exposure_time": EXPOSURE},
        "analog_to_digital_converter": {"bit": 12, "offset": 100, "type": "pixel", "count": 5.0,
                                        "fullwell": 30000},
        "effects": {"photo_bleaching": {"switch": True, "half_life": 2.0 * math.log(2.0)}},
        "gpu": {"cmos_noise": "scmos", "scmos_readout_median": 1.5, "scmos_readout_sigma": 0.4}}})
    return cfg


Z_HALF = 1e-6  # depth range [-Z_HALF, Z_HALF]; --small narrows it for profiling
D_FAST = 1.0e-12  # m^2/s of the faster half of the emitters


def trajectories(n_frames, seed=7):
    """Times and (n_frames*SUBSTEPS + 1, N, 3) Brownian positions (x, y, z)."""
    rng = numpy.random.RandomState(seed)
    steps = n_frames * SUBSTEPS
    dt = EXPOSURE / SUBSTEPS
    pos = numpy.empty((steps + 1, N_EMIT, 3))
    pos[0, :, 0] = rng.uniform(-HALF, HALF, N_EMIT)
    pos[0, :, 1] = rng.uniform(-HALF, HALF, N_EMIT)
    pos[0, :, 2] = rng.uniform(-Z_HALF, Z_HALF, N_EMIT)
    d = numpy.where(numpy.arange(N_EMIT) < N_EMIT // 2, 0.01e-12, D_FAST)
    scale = numpy.sqrt(2 * d * dt)[:, None]
    for t in range(steps):
        pos[t + 1] = pos[t] + scale * rng.standard_normal((N_EMIT, 3))
    times = numpy.arange(steps + 1) * dt
    return times, pos


def formatted(pos):
    out = numpy.empty(pos.shape[:2] + (5,))
    out[..., 0] = pos[..., 2]
    out[..., 1] = pos[..., 0]
    out[..., 2] = pos[..., 1]
    out[..., 3] = numpy.arange(pos.shape[1])
    out[..., 4] = 1.0
    return out


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.file,
                stderr=subprocess.DEVNULL)
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
        self.file.flush()
        rows = [r.split(",") for r in open(self.file.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def splat_algorithmic_bytes(n_rec, tile, halo):
    """Bytes one splat (the box kernel, which also adds the summed-area
    records) must move.

    Per emitter-step: its item index (4 B), the 32-byte record head, and the
    footprint's box-table block: (n_px)^2 FP32 pixel sums, n_px =
    1998 nm / px + 1 pixels per axis on average.  Per tile: the FP32
    (tile + halo)^2 buffer written (the merge that reads it back runs in the
    camera pass, sc_merge_camera).
    """
    n_px = 1998e-9 / PX + 1
    n_tiles = (IMAGE // tile) ** 2
    return n_rec * (4 + 32 + 4 * n_px * n_px) + n_tiles * (tile + halo) ** 2 * 4


# DRAM bytes (read + write) of the splat per splatted record, with the L2
# fetch granularity hint at 32 bytes: 328.25 MB over 368,363 records in one
# frame of `bench.py --small --tile 8 --warps 4` (dram__bytes_read.sum +
# dram__bytes_write.sum of splat_box_bulk_kernel under ncu --set full; the
# summed-area records it now adds itself moved 0.03 MB in their own pass).
SPLAT_TRAFFIC_PER_RECORD = 328.28e6 / 368363


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def replica_barrier(world):
    """All replicas reach this point (one process per GPU; no data exchange)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world, dev):
    """The largest of every replica's value (their timed regions' maximum)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gb300_arm(args, rank, world):
    import torch
    import scopyon_gb300 as sg
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import (TILE_CANDIDATES, EngineConfig, FrameGraph, FramePipeline,
                                     tune_tiles)

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    cfg = workload_config()
    rng = numpy.random.RandomState(11 + rank)
    eng = EngineConfig(cfg["default"], rng=rng)
    pipe = FramePipeline(eng, dev, psf=_psf_for(eng, dev))
    pipe.scmos_sigma_map(rng)
    t0 = time.time()
    if args.small:
        pipe.psf.ensure(list(range(0, int(Z_HALF / 1e-9) + 2)))
    else:
        pipe.psf.ensure_all()
    torch.cuda.synchronize()
    psf_build_s = time.time() - t0

    # trajectories on the device: two populations (D = 0.01 and 1 um^2/s), Philox normals
    n_timing = 16  # eager single frames timed kernel by kernel
    # several frames per graph replay, the records of the next frame running
    # beside the splat of this one: the most (up to 16) that divide the timed
    # frames.  Each replay fills and drains that pipeline once, so more
    # frames per replay hide more of it; every frame keeps its own outputs
    fps = max(k for k in range(1, 17) if args.steps % k == 0)
    n_frames = 4 * (args.warmup + args.steps + n_timing) + 8000 + 20 * len(TILE_CANDIDATES)
    dt = EXPOSURE / SUBSTEPS
    t = numpy.arange(n_frames * SUBSTEPS + 1) * dt
    # reflecting walls at the field's edges and at z = +-Z_HALF keep the
    # emitter density of the initial state (and, for --small, the depths
    # inside the keys built above)
    box = dict(lower=[-HALF, -HALF, -Z_HALF], upper=[HALF, HALF, Z_HALF], ndim=3, device=dev,
               boundary="reflecting")
    slow = sg.sample_inputs(t, N=N_EMIT // 2, D=0.01e-12, rng=rng, **box)
    fast = sg.sample_inputs(t, N=N_EMIT - N_EMIT // 2, D=D_FAST, rng=rng, start=N_EMIT // 2, **box)
    traj = sg.concatenate(slow, fast)
    pipe.ensure_slots(N_EMIT)
    beta = eng.half_life / math.log(2.0)
    pipe.budget[:N_EMIT].copy_(torch.from_numpy(rng.exponential(beta, N_EMIT) * eng.n_emit0))
    fg = FrameGraph(pipe, traj, SUBSTEPS, dt, seed=1234 + rank, frames_per_step=fps)
    if args.tile:  # a fixed tile shape (reproducible profiling), else the autotuner
        pipe.set_tiles(args.tile, args.warps, args.stages)
        tune = {}
    else:
        # every choice runs the same frames; the tuner restores the state after
        tune = tune_tiles(fg, frames=3)  # 5 steps per choice
    # the sequence's first frames are the ones timed, whatever the frames per
    # replay: its state at frame 0 (positions, budgets, frame counter) is
    # restored after the warm-up (emitters bleach as the sequence goes on, so
    # later frames hold fewer live emitters and less work)
    state0 = fg.state_dict()
    fg.capture()  # one eager step of fps frames, then the capture
    # at least W warm-up frames in all, and at least one replay of the graph
    # (its first launch uploads it)
    for _ in range(max(1, -(-args.warmup // fps) - 1)):
        fg.step()
    torch.cuda.synchronize()
    pipe.check_status()
    fg.load_state_dict(state0)
    replica_barrier(world)
    live0 = float((pipe.budget[:N_EMIT] > 0).float().mean())
    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.15)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    for _ in range(args.steps // fps):
        fg.step()
    end.record()
    torch.cuda.synchronize()
    replica_barrier(world)
    live1 = float((pipe.budget[:N_EMIT] > 0).float().mean())
    elapsed_ms = start.elapsed_time(end)
    # the splat's own duration: the same first frames again, launched eagerly
    # one at a time (no records kernel beside the splat) with events around
    # the splat and the stages
    fg.graph, fg.use_graph = None, False
    fg.load_state_dict(state0)
    per_replay, fg.frames_per_step = fg.frames_per_step, 1
    pipe.kernel_events = {}
    splat_recs = []
    for _ in range(n_timing):
        fg.step()
        # records binned this frame: the last bin offset
        splat_recs.append(int(pipe._cap["tile_start"][2 * pipe.tiles_x * pipe.tiles_y]))
    torch.cuda.synchronize()
    fg.frames_per_step = per_replay
    splat_ms = [a.elapsed_time(b) for a, b in pipe.kernel_events["splat"]]
    stage_ms = {k: sum(a.elapsed_time(b) for a, b in pipe.kernel_events[k]) /
                len(pipe.kernel_events[k]) for k in ("records", "camera")}
    pipe.kernel_events = None
    # keep the GPU busy with untimed graph frames so that nvidia-smi (100 ms
    # period) samples the clocks under this load for at least 1 s in all
    fg.use_graph = True
    pad_ms = 1000.0 - elapsed_ms
    t_pad = time.perf_counter()
    while (time.perf_counter() - t_pad) * 1e3 < pad_ms and fg.frames_done + 50 * fps < n_frames:
        for _ in range(50):
            fg.step()
        torch.cuda.synchronize()
    clk = clocks.stop()
    pipe.check_status()
    elapsed_ms = max_over_ranks(elapsed_ms, world, dev)
    ms_per_step = elapsed_ms / args.steps
    value = world * args.steps / (elapsed_ms / 1e3)

    cfg1 = None if args.small else config1_arm(args, dev)
    fwd_bwd = None if args.small else fwd_bwd_arm(args, dev)
    batched = None if args.small else batched_arm(args, dev)
    peak, peak_kind = load_peaks()
    large_stages = None if args.small else hbm_stages(dev, peak)
    # the host-bound leg last: right after a large process exits, the host's
    # memory reclaim slows pinned uploads for some seconds
    e2e = None if args.small else e2e_arm(args, cfg, dev, rank, world)

    splat_avg_ms = sum(splat_ms) / len(splat_ms)
    n_rec = sum(splat_recs) / len(splat_recs)
    alg = splat_algorithmic_bytes(n_rec, pipe.tile, pipe.halo)
    achieved = alg / (splat_avg_ms / 1e3) / 1e9
    tables_gb = (pipe.psf.tables.numel() + (pipe.psf.box.numel() if pipe.psf.box is not None
                                            else 0)) * 4 / 1e9
    result = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform initial positions, Philox Brownian steps on the GPU)",
        "config": workload_dict(),
        "run": {"depth_keys": len(pipe.psf.slot_of), "psf_tables_gb": round(tables_gb, 2),
                "tile": pipe.tile, "warps_per_tile": pipe.warps, "stages": pipe.stages,
                "box_kernel": "registers" if pipe.stages == 0 else "bulk-copy ring",
                "tile_autotune_ms_per_frame": {_tune_name(t, w, st): round(ms, 4)
                                               for (t, w, st), ms in tune.items()},
                "step": "one frame: Brownian sub-steps, physics, binning, splat, camera; "
                        "%d frame(s) per CUDA graph replay%s, each frame's expectation and "
                        "ADC counts in a buffer of its own" % (
                            fps, ", each frame's records kernel (side stream) overlapping "
                                 "the previous frame's binning, splat and camera"
                            if fps > 1 else ""),
                "frames_per_graph_replay": fps,
                "parallelism": "replicas" if world > 1 else "single",
                "boundary": "reflecting",
                "timed_frames": [0, args.steps],
                "warmup_frames": "the same frames, run before and rewound to frame 0",
                "live_emitters": [round(live0, 4), round(live1, 4)],
                "psf_build_s": round(psf_build_s, 3)},
        "e2e": e2e,
        "config1_plain_tirf": cfg1,
        "fwd_bwd": fwd_bwd,
        "batched": batched,
        "gpu_launches": fg.launches_per_frame * args.steps,
        "clocks": clk,
        "roofline": {"kernel": "splat_box_bulk_kernel (box and summed-area records)",
                     "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": SPLAT_TRAFFIC_PER_RECORD * n_rec,
                     "traffic_source": "DRAM bytes read + written per splat record in the ncu "
                                       "capture of the profiling case, times records",
                     "algorithmic_bytes": alg, "records": n_rec,
                     "avg_launch_ms": splat_avg_ms,
                     "timed_on": "%d eager single frames (the splat alone, no records kernel "
                                 "beside it) after the timed graph replays, the sequence's "
                                 "first frames again" % n_timing,
                     "stages": stage_rooflines(stage_ms, pipe, SUBSTEPS * N_EMIT, peak),
                     "stages_beyond_l2": large_stages},
    }
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"], result["rel_err"] = cpu_baseline_and_accuracy(dev)
    result["summary"] = summary(result)
    return result


def summary(r):
    """The headline figures in a few words (printed last, so they survive a
    truncated log)."""
    out = {"frames_per_s": round(r["value"], 1),
           "e2e_frames_per_s": round(r["e2e"]["value"], 1) if r.get("e2e") else None,
           "splat_frac": round(r["roofline"]["frac"], 3)}
    if r.get("rel_err"):
        out["rel_err_per_pixel"] = r["rel_err"]["per_pixel"]
        out["rel_err_norm"] = r["rel_err"]["norm"]
    c1 = r.get("config1_plain_tirf")
    if c1:
        out["config1_frames_per_s"] = round(c1["value"], 1)
        out["config1_e2e_frames_per_s"] = round(c1["e2e"]["value"], 1)
    fb = r.get("fwd_bwd")
    if fb:
        out["fwd_bwd_gaussian_model_512px_20k"] = {
            "frames_per_s": round(fb["value"], 1),
            "over_forward": round(fb["headline"]["fwd_bwd_over_forward"], 2)}
        out["dL_dD_100k_T100_over_forward"] = round(
            fb["diffusion_dD_100k_2048px_T100"]["fwd_bwd_over_forward"], 2)
        out["fwd_bwd_born_wolf_512px_20k"] = {
            "frames_per_s": round(fb["born_wolf_512px_20k"]["fwd_bwd_frames_per_s"], 1),
            "over_forward": round(fb["born_wolf_512px_20k"]["fwd_bwd_over_forward"], 2)}
    bt = r.get("batched")
    if bt:
        out["batched_over_per_field_loop"] = round(bt["batched_over_plain_loop"], 2)
        out["persistent_batched_over_per_field_loop"] = round(
            bt["persistent"]["over_plain_loop"], 2)
    st = r["roofline"].get("stages_beyond_l2")
    if st:
        out["diffusion_frac_beyond_l2"] = round(st["diffusion"]["frac"], 3)
        out["diffusion_frac_on_budget"] = round(st["diffusion"]["frac_on_budget"], 3)
        out["diffusion_fp64_rows_frac"] = round(st["diffusion"]["fp64_rows"]["frac"], 3)
        out["camera_frac_beyond_l2"] = round(st["camera"]["frac"], 3)
    return out


def e2e_arm(args, cfg, dev, rank, world):
    """Frames/s through the public API with host trajectories."""
    import torch
    import scopyon_gb300 as sg
    steps = min(args.steps, E2E_FRAMES)
    n_frames = args.warmup + steps
    times, pos = trajectories(n_frames, seed=21 + rank)
    ids = numpy.arange(N_EMIT, dtype=float)
    # host inputs exactly as scopyon.sample_inputs returns them: [(t, (N, 5) [x, y, z, id, 1])]
    inputs = [(float(t), numpy.hstack([pos[k], ids[:, None], numpy.ones((N_EMIT, 1))]))
              for k, t in enumerate(times)]
    # the leg is host-bound (Python per frame), and a window of a few
    # milliseconds on a shared host catches stalls: the median of E2E_RUNS
    # sequences, each through a new generator, and all of them reported
    runs = []
    for run in range(E2E_RUNS):
        gen = sg.generate_images(inputs, n_frames, config=cfg,
                                 rng=numpy.random.RandomState(3 + rank + 1000 * run), device=dev)
        for _ in range(args.warmup):
            next(gen)
        torch.cuda.synchronize()
        replica_barrier(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            img = next(gen)
            img.as_array()
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0, world, dev)
        runs.append(world * steps / dt)
        gen.close()
    return {"value": float(numpy.median(runs)), "unit": "frames/s", "frames": steps,
            "runs": [round(v, 1) for v in runs], "statistic": "median of the runs",
            # rows, then the unit times and the frame index
            "h2d_bytes_per_step": SUBSTEPS * N_EMIT * 5 * 8 + (SUBSTEPS + 1) * 8,
            "d2h_bytes_per_step": IMAGE * IMAGE * 4 + 16}


# ------------------------------------------------------- differentiable form
def _graph_time(fn, steps, warmup):
    """ms per call of fn replayed from a CUDA graph (warm-up calls run eagerly first)."""
    import torch
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):
            fn()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    for _ in range(warmup):
        g.replay()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(steps):
        g.replay()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def fwd_bwd_case(dev, frames, n_emit, image, sigma, penetration, z_half, steps, warmup, seed):
    """Forward and forward + Poisson NLL + adjoint of the differentiable image."""
    import torch
    from scopyon_gb300 import differentiable as dm
    rng = numpy.random.RandomState(seed)
    half = image * PX * 0.5
    e = numpy.zeros((frames, n_emit, 4), dtype=numpy.float32)
    e[..., 0] = rng.uniform(-half, half, (frames, n_emit))
    e[..., 1] = rng.uniform(-half, half, (frames, n_emit))
    e[..., 2] = rng.uniform(-z_half, z_half, (frames, n_emit))
    e[..., 3] = rng.lognormal(math.log(2000.0), 0.3, (frames, n_emit))
    model = dm.GaussianImageModel(image, image, PX, 1.5 * sigma, penetration=penetration,
                                  device=dev)
    emit = torch.tensor(e, device=dev).requires_grad_(True)
    bg = torch.full((frames,), 10.0, device=dev).requires_grad_(True)
    sig = torch.tensor(sigma, dtype=torch.float32, device=dev).requires_grad_(True)
    with torch.no_grad():
        counts = torch.poisson(dm.expected_image(emit, bg, sig, model).double(),
                               generator=torch.Generator(dev).manual_seed(seed)).float()

    def forward():
        with torch.no_grad():
            return dm.expected_image(emit, bg, sig, model)

    def step():
        loss = dm.poisson_nll(dm.expected_image(emit, bg, sig, model), counts)
        return torch.autograd.grad(loss, [emit, bg, sig])

    fwd_ms = _graph_time(forward, steps, warmup)
    fb_ms = _graph_time(step, steps, warmup)
    return {"frames": frames, "emitters_per_frame": n_emit, "image": [image, image],
            "sigma_nm": sigma * 1e9, "window_px": 2 * model.half_win + 1,
            "illumination": "EPI" if math.isinf(penetration) else
            "TIRF, %.0f nm penetration" % (penetration * 1e9),
            "forward_ms": fwd_ms, "fwd_bwd_ms": fb_ms, "fwd_bwd_over_forward": fb_ms / fwd_ms,
            "fwd_bwd_frames_per_s": frames / (fb_ms / 1e3)}


def diffusion_grad_case(dev, n_emit, image, T, steps, warmup, seed):
    """dL/dD through T Brownian sub-steps: forward (positions, summed frame,
    Gaussian-approximated sCMOS likelihood) and forward + backward (positions
    regenerated from their Philox counters, adjoint, reparameterised dL/dD)."""
    import torch
    from scopyon_gb300 import differentiable as dm
    rng = numpy.random.RandomState(seed)
    half = image * PX * 0.5
    e = numpy.zeros((n_emit, 4), dtype=numpy.float32)
    e[:, 0] = rng.uniform(-half, half, n_emit)
    e[:, 1] = rng.uniform(-half, half, n_emit)
    e[:, 3] = rng.lognormal(math.log(2000.0), 0.3, n_emit)
    sigma, dt, D_true = 120e-9, EXPOSURE / T, 0.05e-12
    model = dm.GaussianImageModel(image, image, PX, 1.5 * sigma, device=dev)
    emit = torch.tensor(e, device=dev)
    sig = torch.tensor(sigma, dtype=torch.float32, device=dev)
    # sCMOS read-noise variance per pixel: sigma ~ lognormal(ln 1.5, 0.4)
    var_map = torch.tensor(rng.lognormal(math.log(1.5), 0.4, (image, image)) ** 2,
                           dtype=torch.float32, device=dev)
    with torch.no_grad():
        pos = dm.diffusion_positions(torch.tensor(D_true, device=dev), emit, T, dt, seed=seed)
        mu = dm.expected_image(pos.reshape(1, -1, 4), torch.full((1,), 10.0, device=dev), sig,
                               model)[0]
        counts = mu + torch.sqrt(mu + var_map) * torch.randn(
            mu.shape, device=dev, generator=torch.Generator(dev).manual_seed(seed))
        del pos, mu
    D = torch.tensor(0.03e-12, dtype=torch.float32, device=dev).requires_grad_(True)

    def loss_fn(d):
        return dm.diffusion_loss(d, emit, counts, sig, model, T, dt, seed=seed + 1,
                                 background=10.0, readout_var=var_map)

    def forward():
        with torch.no_grad():
            return loss_fn(D)

    def step():
        return torch.autograd.grad(loss_fn(D), [D])

    fwd_ms = _graph_time(forward, steps, warmup)
    fb_ms = _graph_time(step, steps, warmup)
    return {"emitters": n_emit, "image": [image, image], "substeps": T,
            "D_um2_per_s": 0.05, "sigma_nm": sigma * 1e9,
            "loss": "Gaussian-approximated sCMOS NLL of the summed frame, FP64 reduction",
            "forward_ms": fwd_ms, "fwd_bwd_ms": fb_ms, "fwd_bwd_over_forward": fb_ms / fwd_ms,
            "emitter_steps_per_s_fwd_bwd": n_emit * T / (fb_ms / 1e3)}


def born_wolf_fwd_bwd_case(dev, steps, warmup, seed=15, n_emit=N_EMIT):
    """Forward and forward + Poisson NLL + adjoint of the differentiable
    Born-Wolf image on the workload's frame: 512^2 px of 160 nm, 20k emitters
    with z in +-1 um (about 1,000 depth keys), TRITC."""
    import torch
    from scopyon_gb300 import differentiable as dm
    rng = numpy.random.RandomState(seed)
    model = dm.BornWolfImageModel(workload_config(), device=dev)
    e = numpy.zeros((1, n_emit, 4), dtype=numpy.float32)
    e[..., 0] = rng.uniform(-HALF, HALF, (1, n_emit))
    e[..., 1] = rng.uniform(-HALF, HALF, (1, n_emit))
    e[..., 2] = rng.uniform(-Z_HALF, Z_HALF, (1, n_emit))
    e[..., 3] = rng.lognormal(math.log(2000.0), 0.3, (1, n_emit))
    emit = torch.tensor(e, device=dev).requires_grad_(True)
    bg = torch.full((1,), 10.0, device=dev).requires_grad_(True)
    model.ensure_keys(emit.detach())
    with torch.no_grad():
        counts = torch.poisson(dm.born_wolf_image(emit, bg, model).double(),
                               generator=torch.Generator(dev).manual_seed(seed)).float()

    def forward():
        with torch.no_grad():
            return dm.born_wolf_image(emit, bg, model)

    def step():
        loss = dm.poisson_nll(dm.born_wolf_image(emit, bg, model), counts)
        return torch.autograd.grad(loss, [emit, bg])

    # eager launches with a host check each: the median of three timings of
    # each, interleaved, so that a stall of the shared host skews neither
    fwd_runs, fb_runs = [], []
    for _ in range(3):
        fwd_runs.append(_event_ms(forward, steps, warmup))
        fb_runs.append(_event_ms(step, steps, warmup))
    fwd_ms, fb_ms = float(numpy.median(fwd_runs)), float(numpy.median(fb_runs))
    return {"model": "differentiable Born-Wolf image (cells integrated over each pixel, "
                     "adjacent depth keys blended)", "emitters": n_emit,
            "image": [IMAGE, IMAGE], "forward_ms": fwd_ms, "fwd_bwd_ms": fb_ms,
            "forward_runs_ms": [round(v, 3) for v in fwd_runs],
            "fwd_bwd_runs_ms": [round(v, 3) for v in fb_runs],
            "fwd_bwd_over_forward": fb_ms / fwd_ms,
            "fwd_bwd_frames_per_s": 1e3 / fb_ms,
            "timing": "eager launches with CUDA events (the forward checks the depth keys "
                      "on the host)"}


def fwd_bwd_arm(args, dev):
    """fwd+bwd frames/s of the differentiable image at 512^2 px, 20k emitters, and
    on a batch of 64 frames of 128^2 px with 200 emitters each."""
    steps = max(20, args.steps)
    headline = fwd_bwd_case(dev, 1, N_EMIT, IMAGE, 90e-9, math.inf, 1e-6, steps, args.warmup, 5)
    batch = fwd_bwd_case(dev, 64, 200, 128, 120e-9, 300e-9, 0.5e-6, steps, args.warmup, 6)
    dgrad = diffusion_grad_case(dev, 100000, 2048, 100, max(5, args.steps // 4), args.warmup, 9)
    bw = born_wolf_fwd_bwd_case(dev, max(10, args.steps), args.warmup)
    return {"value": headline["fwd_bwd_frames_per_s"], "unit": "frames/s",
            "model": "the differentiable Gaussian-PSF model (pixel-integrated Gaussians, "
                     "TIRF depth factor), not the Born-Wolf frame path",
            "workload": "differentiable Gaussian-PSF image, 512^2 px, 20k emitters: forward, "
                        "FP64 Poisson NLL, adjoint (dL/dx, dy, dz, dI, dbg, dsigma); one CUDA "
                        "graph replay per step",
            "dtype": "f32 (FP64 loss reduction)", "headline": headline,
            "batch_64x128px_200": batch, "diffusion_dD_100k_2048px_T100": dgrad,
            "born_wolf_512px_20k": bw}


# ------------------------------------------------------------- batched form
def config1(exposure=0.030):
    """Single-channel TIRF, EGFP, 160 nm pixels, EMCCD (QE 0.92, gain 300,
    readout 100 e-, offset 2000, 16-bit), 100 photons per emitter per ms."""
    import scopyon_gb300 as sg
    cfg = sg.DefaultConfiguration()
    cfg.update({"default": {
        "magnification": 100,
        "fluorophore": {"type": "EGFP"},
        "detector": {"type": "EMCCD", "exposure_time": exposure, "QE": 0.92, "emgain": 300,
                     "readout_noise": 100},
        "analog_to_digital_converter": {"bit": 16, "offset": 2000, "fullwell": 800000},
        "light_source": {"flux_density": 1.1745e7},
        "effects": {"photo_bleaching": {"switch": False}}}})
    return cfg


def config1_arm(args, dev, n_emit=1000, substeps=10, seed=17):
    """Frames/s of the plain TIRF workload the reference runs on the CPU: 1,000
    emitters over a 25.6 um field at z = 0, D = 0.1 um^2/s with no boundary
    (the reference's sample_inputs), 30 ms frames in 10 sub-steps, 160^2 px
    EMCCD, 100 photons per emitter per ms.  Device-resident frames replayed
    from CUDA graphs, and frames through ``generate_images`` with host
    trajectories (e2e)."""
    import torch
    import scopyon_gb300 as sg
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    cfg = config1()
    cfg.update({"default": {"detector": {"image_size": [160, 160]}}})
    rng = numpy.random.RandomState(seed)
    eng = EngineConfig(cfg["default"], rng=rng)
    pipe = FramePipeline(eng, dev, psf=_psf_for(eng, dev))
    pipe.psf.ensure([0])
    dt = eng.exposure_time / substeps
    steps = max(40, 4 * args.steps)
    n_frames = 4 * (args.warmup + steps) + 64
    half = 80 * PX
    traj = sg.sample_inputs(numpy.arange(n_frames * substeps + 1) * dt, N=n_emit, D=0.1e-12,
                            rng=rng, lower=-half, upper=half, ndim=2, device=dev)
    per = max(k for k in range(1, 17) if steps % k == 0)  # frames per replay, as above
    fg = FrameGraph(pipe, traj, substeps, dt, seed=seed, frames_per_step=per)
    fg.capture()
    for _ in range(-(-args.warmup // per)):
        fg.step()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(steps // per):
        fg.step()
    b.record()
    torch.cuda.synchronize()
    pipe.check_status()
    ms = a.elapsed_time(b) / steps
    # e2e: the public API on host trajectories (the reference's sample_inputs layout)
    e2e_frames = 20
    t_host = numpy.arange((args.warmup + e2e_frames) * substeps + 1) * dt
    hrng = numpy.random.RandomState(seed + 1)
    pts = numpy.zeros((n_emit, 4))
    pts[:, :2] = hrng.uniform(-half, half, (n_emit, 2))
    pts[:, 2] = numpy.arange(n_emit)
    pts[:, 3] = 1.0
    inputs = []
    for k, t in enumerate(t_host):
        if k:
            pts = pts.copy()
            pts[:, :2] += math.sqrt(2 * 0.1e-12 * dt) * hrng.standard_normal((n_emit, 2))
        inputs.append((float(t), pts))
    runs = []  # the median of E2E_RUNS sequences, as in the main e2e leg
    for run in range(E2E_RUNS):
        gen = sg.generate_images(inputs, args.warmup + e2e_frames, config=cfg,
                                 rng=numpy.random.RandomState(seed + 2 + 1000 * run), device=dev)
        for _ in range(args.warmup):
            next(gen).as_array()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_frames):
            next(gen).as_array()
        torch.cuda.synchronize()
        runs.append(e2e_frames / (time.perf_counter() - t0))
        gen.close()
    return {"workload": "plain TIRF: 1,000 emitters, 160^2 px EMCCD, 10 sub-steps of 3 ms, "
                        "100 photons/emitter/ms, D = 0.1 um^2/s",
            "value": 1e3 / ms, "unit": "frames/s", "ms_per_frame": ms, "frames": steps,
            "e2e": {"value": float(numpy.median(runs)), "unit": "frames/s", "frames": e2e_frames,
                    "runs": [round(v, 1) for v in runs], "statistic": "median of the runs",
                    "h2d_bytes_per_step": substeps * n_emit * 5 * 8 + (substeps + 1) * 8,
                    "d2h_bytes_per_step": 160 * 160 * 4 + 16}}


def stage_rooflines(stage_ms, pipe, n_rec, peak):
    # n_rec: records written per frame (every emitter at every sub-step)
    """HBM roofline of the two stages around the splat, from their CUDA-event
    durations on the same eager frames.  Algorithmic bytes: the records stage
    reads and writes each emitter's FP64 position (48 B), photon budget
    (16 B) and class (4 B) and writes each record (64 B) with its bin and rank
    (8 B); the camera pass (sc_merge_camera) reads the splat's tile buffers
    once (tiles x (tile + halo)^2 x 4 B), each pixel's offset and 1/gain
    (8 B, with fixed-pattern noise) and read-noise sigma (4 B, sCMOS), and
    writes the expectation (4 B) and the FP32 ADC count (4 B)."""
    n_px = pipe.nw * pipe.nh
    tiles = pipe.tiles_x * pipe.tiles_y * (pipe.tile + pipe.halo) ** 2 * 4
    out = {}
    for name, alg, bound in (
            ("records", N_EMIT * 68 + n_rec * 72,
             "latency of its phases (position chains, then the records of every sub-step) "
             "and footprint arithmetic, not HBM"),
            ("camera", tiles + n_px * (8 + (8 if pipe.pixel_maps else 0) +
                                       (4 if pipe.sigma is not None else 0)),
             "the tile-buffer sums and the per-pixel Poisson and normal draws (dependent "
             "table reads), not HBM")):
        ms = stage_ms[name]
        gbs = alg / (ms / 1e3) / 1e9
        out[name] = {"avg_launch_ms": ms, "algorithmic_bytes": alg, "achieved": gbs,
                     "unit": "GB/s", "frac": gbs / peak, "limited_by": bound}
    return out


def _event_ms(fn, steps, warmup):
    """Average CUDA-event time of fn() (launches on the current stream)."""
    import torch
    for _ in range(warmup):
        fn()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def hbm_stages(dev, peak, steps=20, warmup=3, n_emit=1 << 22, edge=8192, seed=5):
    """The diffusion kernel (sc_diffuse_steps) and the camera kernel (sc_camera)
    alone, each on a workload far larger than L2 (129 MB), so that their HBM
    rooflines mean something (a 512^2 frame moves only a few MB per stage).

    Diffusion: n_emit emitters, reflecting walls, SUBSTEPS Philox sub-steps per
    launch (FP32 moves); per emitter it reads and writes the position (48 B) and
    reads the class (4 B), per emitter-step it writes the 16-byte FP32 row
    [depth, x, y, 0] (layout 1, the rows device-trajectory frames read); the
    FP64 [depth, x, y, id, state] rows (40 B, layout 0) are timed beside it.
    Camera: the workload's sCMOS camera on an edge^2 frame;
    per pixel it reads photons, offset, 1/gain and readout sigma (16 B) and
    writes the expectation (4 B) and the FP32 ADC count (4 B)."""
    import torch
    import scopyon_gb300 as sg
    from scopyon_gb300 import _lib
    from scopyon_gb300._lib import call, ptr, stream_ptr
    gen = torch.Generator(dev).manual_seed(seed)
    out = {}

    # diffusion: uniform time grid, device frame counter advanced between launches
    rng = numpy.random.RandomState(seed)
    dt = EXPOSURE / SUBSTEPS
    t = numpy.arange(4 * SUBSTEPS + 1) * dt
    traj = sg.sample_inputs(t, N=n_emit, D=D_FAST, rng=rng, lower=[-HALF, -HALF, -Z_HALF],
                            upper=[HALF, HALF, Z_HALF], ndim=3, device=dev,
                            boundary="reflecting")
    traj.prepare_uniform(SUBSTEPS)
    frame = torch.zeros(1, dtype=torch.int64, device=dev)
    rows = torch.empty(SUBSTEPS * n_emit * 5, dtype=torch.float64, device=dev)
    layout = [1]

    def diffuse():
        traj.launch_frame(SUBSTEPS, rows, frame, layout=layout[0])
        call("sc_counter_add", ptr(frame), 1, stream_ptr())

    ms = _event_ms(diffuse, steps, warmup)
    alg = n_emit * (48 + 4) + n_emit * SUBSTEPS * 16
    # the budget of 16 B per record and 36 B of state per emitter
    budget = n_emit * 36 + n_emit * SUBSTEPS * 16
    gbs = alg / (ms / 1e3) / 1e9
    layout[0] = 0
    ms0 = _event_ms(diffuse, steps, warmup)
    alg0 = n_emit * (48 + 4) + n_emit * SUBSTEPS * 40
    out["diffusion"] = {"kernel": "diffuse_native_kernel (sc_diffuse_steps, FP32 rows)",
                        "emitters": n_emit,
                        "substeps": SUBSTEPS, "avg_launch_ms": ms, "algorithmic_bytes": alg,
                        "achieved": gbs, "unit": "GB/s", "frac": gbs / peak,
                        "budget_bytes": budget,
                        "frac_on_budget": budget / (ms / 1e3) / 1e9 / peak,
                        "fp64_rows": {"avg_launch_ms": ms0, "algorithmic_bytes": alg0,
                                      "achieved": alg0 / (ms0 / 1e3) / 1e9,
                                      "frac": alg0 / (ms0 / 1e3) / 1e9 / peak},
                        "timing": "includes one 1-thread frame-counter launch per step"}
    del rows, traj
    torch.cuda.empty_cache()

    # camera: the workload's sCMOS model on an edge x edge frame
    n = edge * edge
    photons = torch.rand(n, device=dev, generator=gen) * 200.0
    offset_f = torch.round(100.0 + 5.0 * torch.randn(n, device=dev, generator=gen))
    inv_gain_f = (4096.0 - offset_f) / 30000.0
    sigma = torch.exp(math.log(1.5) + 0.4 * torch.randn(n, device=dev, generator=gen))
    expect = torch.empty(n, dtype=torch.float32, device=dev)
    adc = torch.empty(n, dtype=torch.float32, device=dev)
    status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
    cp = _lib.CameraParams()
    cp.d_poisson_table = _lib.poisson_table(dev).data_ptr()
    cp.nw = cp.nh = edge
    cp.camera, cp.exact, cp.rounding, cp.bit = _lib.CAM_SCMOS, 0, 0, 12
    cp.qe, cp.background, cp.readout_noise, cp.emgain = 0.73, 0.0, 1.5, 1.0
    cp.fullwell, cp.offset0, cp.gain0 = 30000.0, 100.0, 30000.0 / 3996.0
    cp.seed = seed
    counter = [0]

    def camera():
        counter[0] += 1
        cp.counter = counter[0]
        call("sc_camera", cp, ptr(photons), None, None, ptr(offset_f), ptr(inv_gain_f),
             ptr(sigma), None, None, None, None, None, ptr(expect), None, ptr(adc), ptr(status),
             stream_ptr())

    ms = _event_ms(camera, steps, warmup)
    if int(status[0]):
        raise RuntimeError("camera status %d" % int(status[0]))
    alg = n * (16 + 4 + 4)
    gbs = alg / (ms / 1e3) / 1e9
    out["camera"] = {"kernel": "camera_native_kernel (sc_camera, sCMOS)", "image": [edge, edge],
                     "avg_launch_ms": ms, "algorithmic_bytes": alg, "achieved": gbs,
                     "unit": "GB/s", "frac": gbs / peak}
    return out


def _tune_name(t, w, st):
    """Label of a tile choice: edge, warps, and copies in flight or 'reg'."""
    return "%dx%d/%dw/%s" % (t, t, w, "reg" if st == 0 else "%ds" % st)


def _tune_names(tune):
    """Autotuner results keyed by readable names."""
    return {(_tune_name(*k) if len(k) == 3 else "%s=%s" % k): ms for k, ms in tune.items()}


def batched_arm(args, dev, n_fields=256, frames=50, substeps=10, seed=123, loop=True):
    """field-frames/s of 256 fields (edges 128/256/512 px, emitters log-uniform
    in [10, 50000], D log-uniform in [0.001, 1] um^2/s) batched in one canvas,
    next to the plain method's per-field frame loop (loop=False: the batch
    alone, for profiling; with --tile, a fixed tile shape instead of the
    autotuner)."""
    import torch
    from scopyon_gb300.base import _psf_for
    from scopyon_gb300.batch import BatchedFields
    from scopyon_gb300.epifm import EngineConfig, FrameGraph, FramePipeline
    from scopyon_gb300.sampling import DeviceTrajectories
    rng = numpy.random.RandomState(seed)
    sizes = rng.choice([128, 256, 512], n_fields)
    counts = numpy.exp(rng.uniform(math.log(10), math.log(50000), n_fields)).astype(int)
    D = numpy.exp(rng.uniform(math.log(1e-3), math.log(1.0), n_fields)) * 1e-12
    cfg = config1()
    per_step = 4  # four canvas frames per replay, each frame's records beside the previous splat
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def run(persistent):
        t0 = time.time()
        bf = BatchedFields(cfg, sizes, counts, D, frames, substeps, seed=seed, device=dev,
                           frames_per_step=per_step, persistent=persistent)
        if args.tile:
            bf.pipe.set_tiles(args.tile, args.warps, args.stages)
            tune = {}
        else:
            tune = bf.autotune(frames=1)
        bf.step()  # capture
        for _ in range(args.warmup):
            bf.step()
        steps = max(1, min(args.steps, frames - 2 - args.warmup) // per_step)
        torch.cuda.synchronize()
        a.record()
        for _ in range(steps):
            bf.step()
        b.record()
        torch.cuda.synchronize()
        bf.pipe.check_status()
        ms = a.elapsed_time(b) / (steps * per_step)
        setup = time.time() - t0
        del bf
        torch.cuda.empty_cache()
        return ms, tune, setup

    batch_ms, tune, setup_s = run(False)
    pers_ms, pers_tune, _ = run(True)
    if not loop:
        return {"value": n_fields / (batch_ms / 1e3), "unit": "field-frames/s",
                "batched_ms_per_frame_of_all_fields": batch_ms,
                "persistent_ms_per_frame_of_all_fields": pers_ms, "setup_s": setup_s}

    # the plain method, one field at a time: a pipeline, trajectories and frame per field
    fields = []
    for k in range(n_fields):
        fc = config1()
        fc.update({"default": {"detector": {"image_size": [int(sizes[k])] * 2}}})
        eng = EngineConfig(fc["default"], rng=numpy.random.RandomState(k))
        pipe = FramePipeline(eng, dev, psf=_psf_for(eng, dev))
        pipe.psf.ensure([0])
        half = sizes[k] * eng.px / 2
        pts = numpy.zeros((counts[k], 4))
        pts[:, :2] = rng.uniform(-half, half, (counts[k], 2))
        pts[:, 2] = numpy.arange(counts[k])
        pts[:, 3] = 1.0
        times = numpy.arange(8 * substeps + 1) * (eng.exposure_time / substeps)
        traj = DeviceTrajectories(times, pts, [[D[k], D[k]]], 2, k, boundary="reflecting",
                                  lower=[-half, -half, 0], upper=[half, half, 0], device=dev)
        pipe.ensure_slots(counts[k])
        fields.append(FrameGraph(pipe, traj, substeps, eng.exposure_time / substeps, seed=k,
                                 use_graph=False))

    def loop_ms(n):
        for fg in fields:
            fg.step()
        torch.cuda.synchronize()
        a.record()
        for _ in range(n):
            for fg in fields:
                fg.step()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    plain_eager_ms = loop_ms(2)
    for fg in fields:
        fg.use_graph = True
    plain_graph_ms = loop_ms(2)
    return {"value": n_fields / (batch_ms / 1e3), "unit": "field-frames/s",
            "workload": "%d fields of view, edges 128/256/512 px, %d emitters in all "
                        "(log-uniform 10..50000 per field), D log-uniform 0.001..1 um^2/s, "
                        "%d sub-steps per 30 ms frame, TIRF EGFP, EMCCD camera"
                        % (n_fields, int(counts.sum()), substeps),
            "batched_ms_per_frame_of_all_fields": batch_ms,
            "persistent": {
                "form": "one persistent launch per canvas frame (sc_batch_frame): resident "
                        "blocks take tiles and camera chunks from a work list, heaviest "
                        "fields first, each chunk waiting (bounded) for its field's tiles",
                "ms_per_frame_of_all_fields": pers_ms,
                "field_frames_per_s": n_fields / (pers_ms / 1e3),
                "over_plain_loop": plain_eager_ms / pers_ms,
                "autotune_ms_per_frame": _tune_names(pers_tune)},
            "plain_per_field_loop_ms": plain_eager_ms,
            "plain_per_field_graphs_ms": plain_graph_ms,
            "batched_over_plain_loop": plain_eager_ms / batch_ms,
            "batched_over_plain_graphs": plain_graph_ms / batch_ms,
            "autotune_ms_per_frame": _tune_names(tune),
            "setup_s": setup_s}


# ---------------------------------------------------------------- CPU baseline
def _cmos_table():
    """The reference's CMOS read-noise table (RNDist_F40), from the committed
    reference goldens."""
    g = numpy.load(os.path.join(ROOT, "tests", "golden", "reference_goldens.npz"))
    return numpy.asarray(g["cmos_table"])


def _oracle_params(cfg, rng):
    import oracle as O
    import scopyon_gb300 as sg
    from __graft_entry__ import _si_tree
    eng = sg.EPIFMSimulator(cfg, rng=numpy.random.RandomState(0)).base()
    return O.Params(_si_tree(cfg.yaml)["default"], float(eng.psf_wavelength),
                    eng.norm_coeff / eng.psf_normalization, rng=rng, na=eng.na,
                    cmos_table=_cmos_table())


def cpu_baseline_and_accuracy(dev, seed=61):
    """The CPU leg: the FP64 oracle forms one whole frame of the workload on
    the host cores (timed), and that frame checks the GPU's.

    Frame: the workload's first frame from host trajectories (20,000 emitters,
    20 sub-steps, depths in +-1 um), bleaching times drawn once and given to
    both sides.  GPU: ``generate_images`` with those inputs, native camera, so
    the expectation comes from the production FP32 path (records, box tables,
    tile bins, splat).  Oracle: the vectorised FP64 frame (a prefix sum per
    depth key, the keys spread over spawned processes) plus the reference's
    CMOS camera law vectorised (table read noise, Poisson signal).  Returns
    (cpu_baseline, rel_err)."""
    import multiprocessing as mp
    import torch
    import oracle as O
    from oracle import frames as F
    import scopyon_gb300 as sg
    times, pos = trajectories(1, seed=seed)
    ids = numpy.arange(N_EMIT, dtype=float)
    inputs = [(float(t), numpy.hstack([pos[k], ids[:, None], numpy.ones((N_EMIT, 1))]))
              for k, t in enumerate(times)]
    rng = numpy.random.RandomState(seed)
    bleach = dict(zip(range(N_EMIT), rng.exponential(2.0, N_EMIT)))
    cfg = workload_config()
    _, info = next(sg.generate_images(inputs, 1, config=cfg, rng=numpy.random.RandomState(seed),
                                      full_output=True, device=dev,
                                      draws=sg.InjectedDraws(bleach=bleach)))
    torch.cuda.synchronize()
    e_gpu = info["expectation"]
    workers = max(1, min(os.cpu_count() or 1, 64))
    params = _oracle_params(cfg, numpy.random.RandomState(seed))
    params.detector_type = "CMOS"
    data = [(t, O.format_data(p)) for t, p in inputs]
    with mp.get_context("spawn").Pool(workers) as pool:
        pool.map(abs, range(workers))  # workers started before the clock
        t0 = time.perf_counter()
        cam, _ = F.output_frame_fast(params, data, O.InjectedDraws(bleach, []), 0, states={},
                                     camera=False, pool=pool, workers=workers)
        t1 = time.perf_counter()
    e_ref = cam[:, :, 0]
    crng = numpy.random.RandomState(seed + 1)
    noise = O.cmos_table_draw(params.cmos_table, crng.random_sample(e_ref.shape))
    adc = O.adc_counts(crng.poisson(e_ref) + noise, params.fullwell, params.gain, params.offset,
                       params.bit)
    t2 = time.perf_counter()
    assert adc.shape == e_ref.shape
    big = e_ref > 1e-6 * e_ref.max()
    rel = {"per_pixel": float((numpy.abs(e_gpu - e_ref)[big] / e_ref[big]).max()),
           "norm": float(numpy.abs(e_gpu - e_ref).sum() / e_ref.sum()),
           "floor": "pixels above 1e-6 of the frame maximum (%d of %d)" % (int(big.sum()),
                                                                          big.size),
           "frame": "the workload's first frame: generate_images on host trajectories, "
                    "production FP32 path, against the FP64 oracle"}
    base = {"value": 1.0 / (t2 - t0), "unit": "frames/s", "cores": workers, "kind": "port",
            "sample": "one whole frame of the workload, not extrapolated: the FP64 oracle's "
                      "expectation (%d records over %d depth keys, %.2f s on %d processes) "
                      "and the CMOS camera (%.2f s)"
                      % (len(data[0][1]) * SUBSTEPS,
                         len(numpy.unique(F.depth_keys(pos[:-1, :, 2]))), t1 - t0, workers,
                         t2 - t1)}
    return base, rel


def _ref_worker(job):
    """One process's share of a reference-arm step: the reference's own
    per-element algorithms on a bounded sample, each timed per unit.

    * footprints: ``overlay_signal_`` slice sums of 1999^2 FP64 grids, one
      emitter-step at a time (``_epifm.py:224-282``), on depth keys built
      beforehand;
    * a depth key's grid: Born-Wolf radial table and ``radial_to_cartesian``
      (``_epifm.py:99-126``, ``:181-213``);
    * camera: the CMOS model pixel by pixel, a table draw then a Poisson draw
      (``_epifm.py:332-353``), with the RNDist_F40 table;
    * diffusion: ``move_points``' scalar normal per particle and axis
      (``sampling.py:115-119``)."""
    n_steps, n_keys, n_px, n_move, seed, table = job
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import oracle as O
    from scopyon_gb300._catalog import psf_wavelength_and_norm
    rng = numpy.random.RandomState(seed)
    wl, _ = psf_wavelength_and_norm("Tetramethylrhodamine(TRITC)")
    psf = O.PSFCache("Born-Wolf", wl)
    z = rng.uniform(-1e-6, 1e-6, size=n_keys)
    t0 = time.perf_counter()
    for d in z:
        psf.get(d)
    t_key = (time.perf_counter() - t0) / n_keys
    xy = rng.uniform(-HALF, HALF, size=(n_steps, 2))
    img = numpy.zeros((IMAGE, IMAGE))
    t0 = time.perf_counter()
    for k in range(n_steps):
        O.overlay_signal(img, psf.get(z[k % n_keys]), [0.0, xy[k, 0], xy[k, 1]], PX, 1.0)
    t_splat = (time.perf_counter() - t0) / n_steps

    class P:
        detector_type = "CMOS"
        cmos_table = table

    side = int(round(math.sqrt(n_px)))
    patch = rng.uniform(0, 20, size=(side, side))
    t0 = time.perf_counter()
    O.NumpyDraws(rng).camera(P, patch)
    t_px = (time.perf_counter() - t0) / patch.size
    pts = rng.uniform(-HALF, HALF, size=(n_move, 3))
    t0 = time.perf_counter()
    for i in range(n_move):
        for d in range(3):
            pts[i, d] += rng.normal(0.0, 1e-8)
    t_draw = (time.perf_counter() - t0) / (3 * n_move)
    return t_splat, t_px, t_draw, t_key


def reference_arm(args, rank, world):
    """The reference's own CPU algorithms (ported, per element, as the reference
    runs them) on all host cores.  Each step: every process times a bounded
    sample of footprint sums, camera pixels, diffusion draws and one depth-key
    grid.  ``value`` extrapolates the per-unit times to one frame of the
    workload (400k emitter-steps, 512^2 pixels, 1.2M diffusion draws) divided
    over the processes; ``ms_per_step`` is the wall time of the timed sample."""
    if rank != 0:
        return None
    import multiprocessing as mp
    threads = max(1, min(os.cpu_count() or 1, 64))
    table = _cmos_table()
    n_steps, n_keys, n_px, n_move = 40, 2, 1024, 2000
    res, walls = [], []
    with mp.get_context("spawn").Pool(threads) as pool:
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            out = pool.map(_ref_worker, [(n_steps, n_keys, n_px, n_move, 1000 * k + w, table)
                                         for w in range(threads)])
            if k >= args.warmup:
                res += out
                walls.append(time.perf_counter() - t0)
    t_splat, t_px, t_draw, t_key = (statistics.mean(r[i] for r in res) for i in range(4))
    parts = {"footprints_s": t_splat * SUBSTEPS * N_EMIT,
             "camera_s": t_px * IMAGE * IMAGE,
             "diffusion_s": t_draw * SUBSTEPS * N_EMIT * 3}
    sec_per_frame = sum(parts.values()) / threads
    value = 1.0 / sec_per_frame
    n_keys_frame = int(round(Z_HALF / 1e-9)) + 2  # keys 0..Z/1nm and the key past the cutoff
    sample = ("%d processes, each step per process: %d emitter-step footprint sums (1-nm slice "
              "sums of 1999^2 FP64 grids), %d CMOS camera pixels (RNDist_F40 table, Poisson), "
              "%d diffusion draws, %d depth-key grids; per unit %.2f ms / footprint, %.1f us / "
              "pixel, %.2f us / draw, %.0f ms / key" % (threads, n_steps, n_px, 3 * n_move,
                                                       n_keys, t_splat * 1e3, t_px * 1e6,
                                                       t_draw * 1e6, t_key * 1e3))
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(walls), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_dict(),
            "extrapolated": True,
            "extrapolation": "value = 1 / (per-frame work / processes): per-unit times of the "
                             "timed samples times one frame's units; ms_per_step is the wall "
                             "time of one timed sample step, not of a frame",
            "frame_seconds_one_process": {k: round(v, 2) for k, v in parts.items()},
            "psf_warmup_s_one_process": round(t_key * n_keys_frame, 1),
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tile", type=int, default=0,
                    help="splat tile edge (8 or 16); default: autotuned")
    ap.add_argument("--warps", type=int, default=4, help="warps per splat tile with --tile")
    ap.add_argument("--stages", type=int, default=4,
                    help="box-table block copies in flight per splat warp with --tile "
                         "(0: the register box kernel)")
    ap.add_argument("--case", choices=["dgrad", "batched", "fwdbwd", "stages", "bwdiff"],
                    default=None,
                    help="profiling: run one workload alone and print its result object "
                         "(dgrad: dL/dD at 100k emitters x 100 sub-steps on 2048^2 px; "
                         "batched: the 256-field canvas without the per-field loop; "
                         "fwdbwd: the differentiable image at 512^2 px, 20k emitters; "
                         "stages: the diffusion and camera kernels alone beyond L2; "
                         "bwdiff: the differentiable Born-Wolf image at 512^2 px, 20k emitters)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: depth range +-0.1 um between reflecting walls and "
                         "D = 0.01 um^2/s for all emitters (102 PSF keys, 2.9 GB of tables), "
                         "no e2e or CPU legs")
    args = ap.parse_args()
    if args.small:
        global Z_HALF, D_FAST
        Z_HALF, D_FAST = 0.1e-6, 0.01e-12
        args.no_cpu = True
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.case:
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        if args.case == "dgrad":
            res = diffusion_grad_case(dev, 100000, 2048, 100, args.steps, args.warmup, 9)
        elif args.case == "stages":
            # --small: 1M emitters and a 4096^2 frame (still beyond L2), for ncu
            res = hbm_stages(dev, load_peaks()[0], args.steps, args.warmup,
                             n_emit=1 << (20 if args.small else 22),
                             edge=4096 if args.small else 8192)
        elif args.case == "bwdiff":
            res = born_wolf_fwd_bwd_case(dev, args.steps, args.warmup)
        elif args.case == "fwdbwd":
            res = fwd_bwd_case(dev, 1, N_EMIT, IMAGE, 90e-9, math.inf, 1e-6, args.steps,
                               args.warmup, 5)
        else:
            res = batched_arm(args, dev, loop=False)
        print(json.dumps(res), flush=True)
        return
    if args.impl == "reference":
        res = reference_arm(args, rank, world)
        if res is not None:
            print(json.dumps(res), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    res = gb300_arm(args, rank, world)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
