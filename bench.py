"""Benchmark: SAR back-projection on the 4096-pulse x 8192-sample, 4096^2-pixel
scene (200 Rayleigh point targets, 20 dB clutter, 0.25 m pixels), split-precision
FP32 arithmetic, one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--mode split|fp16store|fp32|fp64]
  python bench.py --impl reference ...   # the CPU back-projection (FP64 oracle port) on host cores

Metric: Gpix*pulse/s = Nx*Ny*Np / back-projection time, with the range-compressed
data resident in HBM (range compression timed and reported separately).
`e2e` is the same metric through sarbp_image() with pinned host buffers: echo
upload, range compression, back-projection and image download every step.
Inputs (256 MB echo, 2 GB range-compressed data, 128 MB image) exceed the
129 MB L2, so no explicit flush is needed between steps.

Multi-GPU (torchrun): every rank images its own replica of the scene (weak
scaling; tiles/replicas need no exchange); time = max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic work of one pixel*pulse update (slant range, bin, linear
# interpolation, phase rotation, complex accumulate): 19 FP32-pipe operations
# and 3 MUFU operations (a square-root-class op, sin, cos).
FP32_OPS_PER_UPDATE = 19
MUFU_OPS_PER_UPDATE = 3
# DRAM bytes (read + write) and L2 bytes (lts__t_bytes.sum) per call, measured by
# ncu on GB300 for the default workload (4096 pulses x 8192 samples -> 4096^2,
# complex64 rows): profiles/traffic_bp_rc_config2.md (captured 2026-12-04, one-pass
# full-size captures of bp_kernel<2,0,3,0,8,0,16,0>, rc_forward_kernel<16384,512>
# and rc_inverse_kernel<16384,512,0>).  Back-projection: one launch; range
# compression: two batches of forward + inverse.
MEASURED_TRAFFIC = {
    ("full", "split"): {"bp": 234726656 + 115588864,
                        "rc": (134409984 + 209805824 + 268619008 + 1013745408) +
                              (134468864 + 207117824 + 268857344 + 1014054912)},
}
L2_TRAFFIC = {
    ("full", "split"): {"bp": 25964478848, "rc": 784757152 + 8282912800 + 791771840 + 8362595552},
}
# ncu's L2 peak for these launches: lts__t_bytes.sum / duration / pct_of_peak (same file)
L2_PEAK_GBS = 25964478848 / 53.124512e-3 / 0.0134 / 1e9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="split", choices=["split", "fp16store", "fp32", "fp64"])
    ap.add_argument("--size", default="full", choices=["full", "medium", "small"],
                    help="medium: 1024 pulses x 8192 samples, 2048^2 (profiling captures); small: config 1")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-probe", action="store_true", help="skip the issue-rate probe (profiling runs)")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the headline measurement: no FP16-storage, config-5 or serving keys")
    ap.add_argument("--c5", action="store_true",
                    help="config 5: 16384 x 16384 curved-track echo, 8192^2 image, FP16 storage, batched")
    ap.add_argument("--serve", action="store_true",
                    help="serving stream (config 4): Poisson arrivals at swept rates, p50/p99 latency")
    ap.add_argument("--wk", action="store_true",
                    help="omega-K imager on the reference's RADARSAT-1 configuration (3072 x 2048 -> 4096 x 3414)")
    ap.add_argument("--autofocus", action="store_true",
                    help="autofocus iterations and the projection kernel on a config-2 geometry")
    ap.add_argument("--ceos", action="store_true",
                    help="CEOS raw-data decode of the reference scene's size (3072 lines x 2048 cells)")
    ap.add_argument("--rates", default="10,20,30,40", help="arrival rates (jobs/s) for --serve")
    ap.add_argument("--jobs", type=int, default=60, help="jobs per rate for --serve")
    ap.add_argument("--step-updates", default="4294967296,0",
                    help="--serve schedules: comma list of step_updates (0: fixed 512 pulses per step)")
    return ap.parse_args()


def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    backend = "nccl"
    dist.init_process_group(backend)
    return dist.get_rank(), dist.get_world_size(), dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    from sar_cambrianaccelerationcard_gb300 import replicas
    return replicas.max_over_ranks(v, dist, device="cuda")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # return once nvidia-smi has written its first sample: its start-up
        # (NVML queries) then falls before the timed region, not inside it
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
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
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(size):
    from sar_cambrianaccelerationcard_gb300 import scenes
    if size == "small":
        return scenes.config1()
    if size == "medium":
        return scenes.config2(np_=1024, n_img=2048)
    return scenes.config2()


def cpu_tile_side(orc, scene, rc, seconds: float) -> int:
    """Side of the centred square tile whose FP64 oracle back-projection (all
    pulses) takes about `seconds` on this host, from a 64x64 probe; a
    multiple of 32, capped at the image."""
    g = scene.grid
    probe = min(64, g.nx, g.ny)
    t = time.perf_counter()
    orc.backproject(scene, rc, (g.nx // 2 - probe // 2, g.ny // 2 - probe // 2, probe, probe))
    rate = probe * probe * scene.np_ / max(time.perf_counter() - t, 1e-6)
    side = int(math.sqrt(seconds * rate / scene.np_)) // 32 * 32
    return max(32, min(side, g.nx, g.ny))


def host_threads() -> int:
    """Host threads this process may use (its CPU affinity).  The CPU arms run
    on rank 0 alone, so they take all of them rather than the OMP_NUM_THREADS=1
    that torchrun sets for every rank."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_sample(scene, threads=None, seconds: float = 12.0):
    """FP64 oracle back-projection of a centred square tile (all pulses) of the
    scene, sized for about `seconds` of host work, on range-compressed data
    computed by the oracle.  Returns (updates/s, cores, description, seconds)."""
    from oracle import oracle as orc
    orc.set_threads(threads or host_threads())
    cores = orc.threads()
    g = scene.grid
    # range-compress the pulses once (untimed setup): oracle FP64 chain
    echo = orc.echo(scene)
    rc = orc.range_compress(scene, echo)
    w = h = cpu_tile_side(orc, scene, rc, seconds)
    x0, y0 = g.nx // 2 - w // 2, g.ny // 2 - h // 2
    t = time.perf_counter()
    orc.backproject(scene, rc, (x0, y0, w, h))
    dt = time.perf_counter() - t
    upd = w * h * scene.np_
    desc = (f"FP64 oracle BP (restated BPA_SAR.m:177-197, linear interpolation) over a {w}x{h}-pixel tile "
            f"x all {scene.np_} pulses of the same scene ({upd:.3g} updates, {dt:.1f} s), {cores} OpenMP threads")
    return upd / dt, cores, desc, dt, rc, (x0, y0, w, h)


def run_reference(args):
    """CPU arm: the reference's back-projection algorithm on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.set_threads(host_threads())
    scene = workload(args.size)
    echo = orc.echo(scene)
    rc = orc.range_compress(scene, echo)
    g = scene.grid
    w = h = cpu_tile_side(orc, scene, rc, 5.0)  # ~5 s of host work per step
    region = (g.nx // 2 - w // 2, g.ny // 2 - h // 2, w, h)
    for _ in range(args.warmup):
        orc.backproject(scene, rc, region)
    t = time.perf_counter()
    for _ in range(args.steps):
        orc.backproject(scene, rc, region)
    dt = (time.perf_counter() - t) / max(1, args.steps)
    upd = w * h * scene.np_
    v = upd / dt / 1e9
    cores = orc.threads()
    line = {
        "impl": "reference", "metric": "BP Gpix*pulse/s", "value": v, "unit": "Gpix*pulse/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"stripmap BP {scene.np_} pulses x {scene.ns} samples -> {g.nx}x{g.ny} image",
                   "mode": "fp64-cpu", "sample_tile": [w, h]},
        "cpu_baseline": {"value": v, "unit": "Gpix*pulse/s", "cores": cores, "kind": "port",
                         "sample": f"{w}x{h} tile x {scene.np_} pulses per step ({upd:.3g} updates, "
                                   f"{dt:.1f} s; range compression untimed)"},
        "e2e": {"value": v, "unit": "Gpix*pulse/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0



def sub_grid(g, x0, y0, w, h):
    """Grid struct of the w x h pixels of grid struct g starting at pixel (x0, y0)."""
    from sar_cambrianaccelerationcard_gb300 import sarbp
    s = sarbp.Grid()
    for i in range(3):
        s.origin[i] = g.origin[i] + x0 * g.ux[i] + y0 * g.uy[i]
        s.ux[i], s.uy[i] = g.ux[i], g.uy[i]
    s.nx, s.ny = w, h
    return s


def isolated_target_pixels(scene, n=5, margin=48, radius_m=12.0):
    """Pixels (x, y) of up to n of the scene's brightest targets that have no
    other target within radius_m and lie at least `margin` pixels inside the
    image: their point responses can be measured without a neighbour's."""
    g = scene.grid
    M = np.column_stack([g.ux, g.uy])
    out = []
    for k in np.argsort(-scene.targets[:, 3]):
        t = scene.targets[k]
        if np.sum(np.linalg.norm(scene.targets[:, :3] - t[:3], axis=1) < radius_m) > 1:
            continue
        xy, *_ = np.linalg.lstsq(M, t[:3] - g.origin, rcond=None)
        x, y = int(round(xy[0])), int(round(xy[1]))
        if margin <= x < g.nx - margin and margin <= y < g.ny - margin:
            out.append((x, y))
        if len(out) == n:
            break
    return out


PATCH = 96  # pixels per side of the patch around a target (the metrics use 64)


def point_target_diffs(patches_gpu, patches_ref):
    """Largest peak shift (px) and PSLR / ISLR differences (dB) over target
    patches centred on their targets."""
    from sar_cambrianaccelerationcard_gb300 import metrics
    worst = {"targets": len(patches_ref), "peak_shift_px": 0.0, "pslr_diff_db": 0.0, "islr_diff_db": 0.0}
    for a, b in zip(patches_gpu, patches_ref):
        c = metrics.compare_point_targets(a, b, [(PATCH // 2, PATCH // 2)])
        for k in ("peak_shift_px", "pslr_diff_db", "islr_diff_db"):
            worst[k] = max(worst[k], c[k])
    return worst


def oracle_accuracy(orc, scene, rc_oracle, images, tile, targets):
    """FP64 oracle against the product on the same scene.  images maps a mode
    to a function (x0, y0, w, h) -> the product's pixels of that region
    (complex64).  Returns, per mode, the relative L2 error over `tile` and the
    point-target differences over patches around `targets`."""
    from sar_cambrianaccelerationcard_gb300 import metrics
    t = time.perf_counter()
    ref_tile = orc.backproject(scene, rc_oracle, tile)
    regions = [(x - PATCH // 2, y - PATCH // 2, PATCH, PATCH) for (x, y) in targets]
    ref_patches = [orc.backproject(scene, rc_oracle, r) for r in regions]
    out = {"tile": list(tile), "oracle_s": time.perf_counter() - t}
    for mode, get in images.items():
        d = {"rel_l2_db": metrics.rel_l2_db(get(*tile), ref_tile)}
        if targets:
            d.update(point_target_diffs([get(*r) for r in regions], ref_patches))
        out[mode] = d
    return out

def run_ours(args):
    import torch
    rank, world, dist = dist_init(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

    mode = sarbp.MODES[args.mode]
    scene = workload(args.size)
    scene.seed += rank  # every rank images its own independent scene (replicas, weak scaling)
    r, g, lay = sarbp.scene_args(scene)
    ctx = sarbp.Context(local)
    stream = torch.cuda.Stream()
    sptr = sarbp.ctypes.c_void_p(stream.cuda_stream)

    # --- inputs: GPU-synthesised echo (device), pinned host copy for e2e
    echo_d = torch.empty((scene.np_, scene.ns * 2), dtype=torch.float32, device="cuda")
    apc_d = torch.from_numpy(scene.apc).cuda()
    sarbp.synthesize(ctx, scene, out=echo_d)
    ctx.synchronize()
    storage = sarbp.STORE_C32H if mode == sarbp.MODE_FP16STORE else sarbp.STORE_C64
    esize = 8 if storage == sarbp.STORE_C64 else 4
    rc_d = torch.empty((scene.np_, lay.nbins * esize // 4), dtype=torch.float32, device="cuda")
    scale_d = torch.ones(scene.np_, dtype=torch.float32, device="cuda")
    img_d = torch.zeros((g.ny, g.nx * 2), dtype=torch.float32, device="cuda")

    def rc_step():
        ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo_d.data_ptr(), scene.np_, scene.ns,
                                               storage, rc_d.data_ptr(), scale_d.data_ptr(), sptr), "rc")

    view = sarbp.RcView()
    view.data, view.scale = rc_d.data_ptr(), scale_d.data_ptr() if storage == sarbp.STORE_C32H else None
    view.storage, view.np, view.nbins = storage, scene.np_, lay.nbins
    view.t0_bins, view.bin_rate = lay.t0_bins, lay.bin_rate

    def bp_step():
        ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(view), apc_d.data_ptr(),
                                            sarbp.ctypes.byref(g), mode, img_d.data_ptr(), 0, sptr), "bp")

    # range compression: warm-up calls, then the mean of timed calls (events on
    # the launching stream)
    for _ in range(max(1, args.warmup)):
        rc_step()
    stream.synchronize()
    ctx.synchronize()
    rc_ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    rc_reps = 5
    rc_ev[0].record(stream)
    for _ in range(rc_reps):
        rc_step()
    rc_ev[1].record(stream)
    stream.synchronize()
    ctx.synchronize()
    rc_ms = rc_ev[0].elapsed_time(rc_ev[1]) / rc_reps

    # --- device-resident timing of back-projection
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        bp_step()
    stream.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    n0 = ctx.launches()
    ev0.record(stream)
    bp_ms_each = []
    for _ in range(args.steps):
        bp_step()
    ev1.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    launches = ctx.launches() - n0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = max_over_ranks(dist, ms)
    ctx.synchronize()
    bp_ms_each = ctx.timings()[1]  # last launch, events on the launching stream
    updates = scene.updates
    value = updates * world / (ms * 1e-3) / 1e9

    img_split = img_d.cpu().numpy().view(np.complex64) if rank == 0 else None

    # --- end to end through sarbp_image with pinned host buffers
    e2e = None
    if not args.no_e2e:
        echo_h = torch.empty((scene.np_, scene.ns * 2), dtype=torch.float32, pin_memory=True)
        echo_h.copy_(echo_d.cpu())
        img_h = torch.empty((g.ny, g.nx * 2), dtype=torch.float32, pin_memory=True)
        apc_h = np.ascontiguousarray(scene.apc)

        def e2e_step():
            ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo_h.data_ptr(), scene.np_, scene.ns,
                                          apc_h.ctypes.data, sarbp.ctypes.byref(g), mode, img_h.data_ptr(), sptr),
                      "e2e")

        for _ in range(max(1, args.warmup)):
            e2e_step()
        barrier(dist)
        torch.cuda.synchronize()
        t = time.perf_counter()
        ksteps = max(1, min(args.steps, 5))
        for _ in range(ksteps):
            e2e_step()
        torch.cuda.synchronize()
        barrier(dist)
        e2e_s = max_over_ranks(dist, (time.perf_counter() - t) / ksteps)
        e2e = {"value": updates * world / e2e_s / 1e9, "unit": "Gpix*pulse/s",
               "h2d_bytes_per_step": scene.np_ * scene.ns * 8 + scene.np_ * 24,
               "d2h_bytes_per_step": g.nx * g.ny * 8, "ms_per_step": e2e_s * 1e3}

    # algorithmic BP bytes per launch: for every pulse the range bins between
    # the nearest and farthest pixel (9x9 lattice over the grid), read once,
    # plus the image written once
    fx, fy = np.meshgrid(np.linspace(0, g.nx - 1, 9), np.linspace(0, g.ny - 1, 9))
    pts = scene.grid.origin + fx.reshape(-1, 1) * scene.grid.ux + fy.reshape(-1, 1) * scene.grid.uy
    rng = np.linalg.norm(pts[None, :, :] - scene.apc[:, None, :], axis=2)
    span_bins = np.minimum(lay.nbins, (rng.max(axis=1) - rng.min(axis=1)) * 2.0 / scene.radar.c * lay.bin_rate)
    bp_alg_bytes = int(span_bins.sum() * esize + g.nx * g.ny * 8)

    # --- roofline: issue-rate ceiling from live microbenchmarks
    fp32_rate, mufu_rate, sms = (1.0, 1.0, 0) if args.no_probe else ctx.probe_issue_rates()
    peak = min(fp32_rate / FP32_OPS_PER_UPDATE, mufu_rate / MUFU_OPS_PER_UPDATE) / 1e9
    bp_rate = updates / (bp_ms_each * 1e-3) / 1e9 if bp_ms_each else None
    roofline = {
        "bound": "issue (FP32+MUFU)", "achieved": bp_rate, "peak": peak, "unit": "Gpix*pulse/s",
        "frac": (bp_rate / peak) if bp_rate else None,
        "traffic": MEASURED_TRAFFIC.get((args.size, args.mode), {}).get("bp"),
        "traffic_algorithmic": bp_alg_bytes,
        "peak_source": (f"measured live: FP32 FMA {fp32_rate / 1e12:.1f} T lanes/s, MUFU {mufu_rate / 1e12:.2f} T "
                        f"lanes/s on {sms} SMs; peak = min(FP32/{FP32_OPS_PER_UPDATE}, MUFU/{MUFU_OPS_PER_UPDATE})"),
        "kernel": "bp_kernel<SPLIT>",
    }
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm = None
    if os.path.exists(peaks_path):
        hbm = json.load(open(peaks_path)).get("hbm_gbs")
    l2 = L2_TRAFFIC.get((args.size, args.mode), {})
    if bp_ms_each and l2.get("bp"):
        # L2 bytes of the profiled launch over this run's launch time, against ncu's L2 peak
        bw = l2["bp"] / (bp_ms_each * 1e-3) / 1e9
        roofline["l2"] = {"achieved": bw, "peak": L2_PEAK_GBS, "unit": "GB/s", "frac": bw / L2_PEAK_GBS,
                          "traffic": l2["bp"], "source": "profiles/traffic_bp_rc_config2.md"}
    if bp_ms_each and hbm:
        # the same launch against HBM (of measured): algorithmic bytes / launch time
        bw = bp_alg_bytes / (bp_ms_each * 1e-3) / 1e9
        roofline["hbm"] = {"achieved": bw, "peak": hbm, "unit": "GB/s", "frac": bw / hbm,
                           "traffic_algorithmic": bp_alg_bytes}
    rc_bytes = scene.np_ * scene.ns * 8 + scene.np_ * lay.nbins * esize
    roofline_rc = {"bound": "hbm", "achieved": rc_bytes / (rc_ms * 1e-3) / 1e9 if rc_ms else None, "peak": hbm,
                   "unit": "GB/s", "frac": (rc_bytes / (rc_ms * 1e-3) / 1e9 / hbm) if (rc_ms and hbm) else None,
                   "traffic": MEASURED_TRAFFIC.get((args.size, args.mode), {}).get("rc"),
                   "kernel": "rc_forward_kernel<16384,512,false> + rc_inverse_kernel<16384,512,0>", "ms": rc_ms}
    if rc_ms and l2.get("rc"):
        bw = l2["rc"] / (rc_ms * 1e-3) / 1e9
        roofline_rc["l2"] = {"achieved": bw, "peak": L2_PEAK_GBS, "unit": "GB/s", "frac": bw / L2_PEAK_GBS,
                             "traffic": l2["rc"], "source": "profiles/traffic_bp_rc_config2.md"}
    # the transforms themselves: 1 forward + L inverse nfft-point FFTs per pulse at
    # 5 N log2 N flops each, against the live FP32 FMA rate (2 flops per lane)
    fft_flops = scene.np_ * (1 + scene.radar.upsample) * 5.0 * lay.nfft * math.log2(lay.nfft)
    if rc_ms:
        roofline_rc["fft_flops"] = fft_flops
        roofline_rc["fft_tflops"] = fft_flops / (rc_ms * 1e-3) / 1e12
        if not args.no_probe:
            roofline_rc["fft_frac_of_fp32"] = roofline_rc["fft_tflops"] * 1e12 / (2.0 * fp32_rate)

    cpu, rc_oracle = None, None
    if rank == 0 and not args.no_cpu:
        v, cores, desc, secs, rc_oracle, _ = cpu_sample(scene)
        cpu = {"value": v / 1e9, "unit": "Gpix*pulse/s", "cores": cores, "kind": "port", "sample": desc,
               "seconds": secs}

    # --- FP16 storage (config 3's mode at this size): range compression to
    # complex16 rows with per-pulse scales, then the same back-projection
    fp16 = None
    img_fp16 = None
    if not args.no_extras and args.mode == "split":
        h16 = torch.empty((scene.np_, lay.nbins), dtype=torch.float32, device="cuda")  # 4 bytes per bin
        sc16 = torch.empty(scene.np_, dtype=torch.float32, device="cuda")
        ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo_d.data_ptr(), scene.np_, scene.ns,
                                               sarbp.STORE_C32H, h16.data_ptr(), sc16.data_ptr(), sptr), "rc16")
        v16 = sarbp.RcView()
        v16.data, v16.scale, v16.storage, v16.np, v16.nbins = (h16.data_ptr(), sc16.data_ptr(), sarbp.STORE_C32H,
                                                               scene.np_, lay.nbins)
        v16.t0_bins, v16.bin_rate = lay.t0_bins, lay.bin_rate

        def bp16_step():
            ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(v16),
                                                apc_d.data_ptr(), sarbp.ctypes.byref(g), sarbp.MODE_FP16STORE,
                                                img_d.data_ptr(), 0, sptr), "bp16")

        for _ in range(2):
            bp16_step()
        stream.synchronize()
        e16 = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        k16 = max(2, min(args.steps, 5))
        e16[0].record(stream)
        for _ in range(k16):
            bp16_step()
        e16[1].record(stream)
        stream.synchronize()
        ctx.synchronize()
        ms16 = e16[0].elapsed_time(e16[1]) / k16
        fp16 = {"value": updates / (ms16 * 1e-3) / 1e9, "unit": "Gpix*pulse/s", "ms_per_step": ms16, "steps": k16,
                "rc_bytes": scene.np_ * lay.nbins * 4}
        if rank == 0:
            img_fp16 = img_d.cpu().numpy().view(np.complex64)
        del h16, sc16

    # --- the plain FP64 GPU mode (the comparator of the >= 5x target) against the
    # split mode on the same 1024^2 centre tile x all pulses of the same data
    fp64cmp = None
    if not args.no_extras and args.mode == "split" and args.size == "full":
        side = 1024
        x0, y0 = g.nx // 2 - side // 2, g.ny // 2 - side // 2
        gs = sub_grid(g, x0, y0, side, side)
        tile_img = torch.empty((side, 2 * side), dtype=torch.float32, device="cuda")

        def bp_tile(m):
            ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(view),
                                                apc_d.data_ptr(), sarbp.ctypes.byref(gs), m, tile_img.data_ptr(),
                                                0, sptr), "bp tile")

        tev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        tms = {}
        for m, reps in ((sarbp.MODE_FP64, 2), (sarbp.MODE_SPLIT, 10)):
            bp_tile(m)  # warm-up
            stream.synchronize()
            tev[0].record(stream)
            for _ in range(reps):
                bp_tile(m)
            tev[1].record(stream)
            stream.synchronize()
            tms[m] = tev[0].elapsed_time(tev[1]) / reps
        ctx.synchronize()
        upd = float(scene.np_) * side * side
        r64 = upd / (tms[sarbp.MODE_FP64] * 1e-3) / 1e9
        rsp = upd / (tms[sarbp.MODE_SPLIT] * 1e-3) / 1e9
        fp64cmp = {"tile": [x0, y0, side, side], "unit": "Gpix*pulse/s",
                   "fp64_gpu": {"value": r64, "ms": tms[sarbp.MODE_FP64]},
                   "split": {"value": rsp, "ms": tms[sarbp.MODE_SPLIT]},
                   "split_over_fp64": rsp / r64,
                   "fp16store_over_fp64": (fp16["value"] / r64) if fp16 else None}
        del tile_img

    # --- accuracy against the FP64 CPU oracle (BPA_SAR.m:177-197 restated):
    # the oracle's own range compression of its own echo, back-projected over
    # the 512^2 centre tile and over patches around the brightest isolated
    # targets; the product's split image is this run's timed image
    acc = {}
    if rank == 0 and rc_oracle is not None and args.size == "full":
        from oracle import oracle as orc
        tile = (g.nx // 2 - 256, g.ny // 2 - 256, 512, 512)
        targets = isolated_target_pixels(scene)

        def crop(img):
            return lambda x0, y0, w, h: img[y0:y0 + h, x0:x0 + w]

        def fp32_region(x0, y0, w, h):
            out = torch.zeros((h, 2 * w), dtype=torch.float32, device="cuda")
            ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(view),
                                                apc_d.data_ptr(), sarbp.ctypes.byref(sub_grid(g, x0, y0, w, h)),
                                                sarbp.MODE_FP32, out.data_ptr(), 0, sptr), "fp32")
            stream.synchronize()
            return out.cpu().numpy().view(np.complex64)

        images = {args.mode: crop(img_split)}
        if args.mode != "fp32":
            images["fp32"] = fp32_region
        if img_fp16 is not None:
            images["fp16store"] = crop(img_fp16)
        acc["vs_cpu_oracle"] = oracle_accuracy(orc, scene, rc_oracle, images, tile, targets)
        acc["vs_cpu_oracle"]["targets_px"] = [list(t) for t in targets]
    del rc_oracle

    extras = {}
    if not args.no_extras and args.size == "full" and world == 1:
        del echo_d, rc_d, img_d
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        ctx.trim()
        extras["c5"] = c5_measure(ctx, with_oracle=not args.no_cpu)
        torch.cuda.empty_cache()
        ctx.trim()
        extras["serve"] = serve_measure(rates=(20.0, 40.0), jobs=30, n_req=12)

    if rank == 0:
        line = {
            "metric": "BP Gpix*pulse/s", "value": value, "unit": "Gpix*pulse/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.mode != "fp64" else "f64",
            "data": "synthetic (GPU echo synthesiser, seeded)",
            "config": {"workload": (f"stripmap BP {scene.np_} pulses x {scene.ns} samples -> {g.nx}x{g.ny} image "
                                    f"at 0.25 m, {len(scene.targets)} targets, 20 dB clutter"),
                       "mode": args.mode, "upsample": scene.radar.upsample, "interp": "linear",
                       "l2": "inputs larger than L2 (2 GB range-compressed data, 128 MB image)"},
            "rc_ms": rc_ms,
            "accuracy": acc,
            "fp16store": fp16,
            "fp64_comparator": fp64cmp,
            **extras,
            "e2e": e2e,
            "roofline": roofline,
            "roofline_rc": roofline_rc,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def serve_requests(ctx, n_req, seed=4):
    """Config-4 request pool: aperture U[256, 8192] pulses x U[2048, 8192] samples,
    grid side log-uniform in [256, 4096], 9-200 targets, 20 dB SNR."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp, scenes
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_req):
        np_ = int(rng.integers(256, 8193)) // 16 * 16
        ns = int(rng.integers(2048, 8193)) // 4 * 4
        side = int(round(math.exp(rng.uniform(math.log(256), math.log(4096))))) // 32 * 32
        nt = int(rng.integers(9, 201))
        radar = scenes.Radar()
        grid = scenes.centred_grid(radar, side, side, 0.25)
        sc = scenes.Scene(name=f"req{i}", radar=radar, np_=np_, ns=ns, apc=scenes.straight_track(radar, np_),
                          grid=grid, targets=scenes.random_targets(grid, nt, seed + 1000 + i),
                          t_rec0=scenes.centred_record_start(radar, ns), snr_db=20.0, seed=seed + 1000 + i)
        dev = torch.empty((np_, ns * 2), dtype=torch.float32, device="cuda")
        sarbp.synthesize(ctx, sc, out=dev)
        ctx.synchronize()
        host = torch.empty((np_, ns * 2), dtype=torch.float32, pin_memory=True)
        host.copy_(dev)
        img = torch.empty((side, side * 2), dtype=torch.float32, pin_memory=True)
        reqs.append((sc, host, img))
        del dev
    return reqs


def serve_one_shot(reqs, reps=3):
    """Each request imaged alone through the one-shot calls with its echo
    already in HBM: device times (CUDA events on the launching stream, best of
    `reps` after one warm-up) of its range compression and its back-projection,
    the same kernels and plans the server runs.  Returns (updates, rc_ms, bp_ms)
    per request."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp
    ctx = sarbp.Context(0)
    stream = torch.cuda.Stream()
    sptr = sarbp.ctypes.c_void_p(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    out = []
    for sc, host, _ in reqs:
        r, g, lay = sarbp.scene_args(sc)
        echo = host.cuda()
        apc = torch.from_numpy(sc.apc).cuda()
        rc = torch.empty((sc.np_, lay.nbins * 2), dtype=torch.float32, device="cuda")
        img = torch.empty((g.ny, g.nx * 2), dtype=torch.float32, device="cuda")
        view = sarbp.RcView()
        view.data, view.scale = rc.data_ptr(), None
        view.storage, view.np, view.nbins = sarbp.STORE_C64, sc.np_, lay.nbins
        view.t0_bins, view.bin_rate = lay.t0_bins, lay.bin_rate
        best_rc = best_bp = float("inf")
        for k in range(reps + 1):
            ev[0].record(stream)
            ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), sc.np_, sc.ns,
                                                   sarbp.STORE_C64, rc.data_ptr(), None, sptr), "rc")
            ev[1].record(stream)
            ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(view),
                                                apc.data_ptr(), sarbp.ctypes.byref(g), sarbp.MODE_SPLIT,
                                                img.data_ptr(), 0, sptr), "bp")
            ev[2].record(stream)
            stream.synchronize()
            if k:
                best_rc = min(best_rc, ev[0].elapsed_time(ev[1]))
                best_bp = min(best_bp, ev[1].elapsed_time(ev[2]))
        out.append((float(sc.np_) * g.nx * g.ny, best_rc, best_bp))
        del echo, apc, rc, img
    ctx.close()
    torch.cuda.empty_cache()
    return out


def serve_sweep(reqs, rates, jobs, schedules, one_shot=None):
    """Poisson arrivals of the requests at each rate against one sarbp server
    per (schedule, rate); latency is submit entry -> image in host memory.
    With one_shot (serve_one_shot's figures) each run also reports the rates
    the same job draws reach imaged one at a time: back-projection alone (the
    reference for the steps' back-projection) and range compression plus
    back-projection (the reference for busy-time throughput)."""
    import threading
    from sar_cambrianaccelerationcard_gb300 import sarbp
    # rate-major, the schedules' order rotated per rate, so that a slow drift over
    # the sweep (power, clocks) does not favour the schedule that runs first
    runs = []
    for k, rate in enumerate(rates):
        for j in range(len(schedules)):
            runs.append((schedules[(j + k) % len(schedules)], rate))
    out = []
    for (sched, step_updates), rate in runs:
        clocks = ClockSampler(0)
        clocks.start()
        srv = sarbp.Server(0, max_jobs=16, hbm_budget_bytes=96 << 30, pulses_per_step=512,
                           step_updates=step_updates)
        # warm-up, untimed: a few requests through the same server back to back,
        # so that the timed stream does not start from an idle host and device
        # (after ten idle seconds the same stream ran with p50 55 ms against 38,
        # its admissions' device time 15% longer); the stats below are taken
        # from here on
        for k in range(SERVE_WARMUP_JOBS):
            sc, host, img = reqs[k % len(reqs)]
            r, g, _ = sarbp.scene_args(sc)
            srv.wait(srv.submit(r, g, host, sc.apc, sarbp.MODE_SPLIT, image=img), 600000)
        base = srv.stats()
        rng = np.random.default_rng(int(rate * 1000))
        order = rng.integers(0, len(reqs), jobs)
        gaps = rng.exponential(1.0 / rate, jobs)
        tickets = []
        t_first = time.perf_counter()

        def submitter():
            t_next = time.perf_counter()
            for k in range(jobs):
                t_next += gaps[k]
                d = t_next - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                sc, host, img = reqs[order[k]]
                r, g, _ = sarbp.scene_args(sc)
                tickets.append(srv.submit(r, g, host, sc.apc, sarbp.MODE_SPLIT, image=img))

        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        lat, upd = [], 0.0
        for t in tickets:
            st, js, _ = srv.wait(t, 600000)
            if st == sarbp.OK:
                lat.append(js.latency_ms)
                upd += js.updates
        t_last = time.perf_counter()
        stats = srv.stats()
        for f in ("updates", "busy_s", "step_device_s", "admit_device_s", "graph_launches"):
            setattr(stats, f, getattr(stats, f) - getattr(base, f))
        srv.close()
        clk = clocks.stop()
        lat.sort()
        pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))] if lat else None
        out.append({"schedule": sched, "rate_jobs_s": rate, "jobs": len(lat), "p50_ms": pct(0.50), "p99_ms": pct(0.99),
                    "mean_ms": sum(lat) / len(lat) if lat else None,
                    "gpix_pulse_s": upd / (t_last - t_first) / 1e9,
                    "busy_gpix_pulse_s": stats.updates / max(stats.busy_s, 1e-9) / 1e9,
                    # where the busy time went (device time from CUDA events): the steps'
                    # back-projection and the admissions' upload + range compression,
                    # which run beside the steps on their own stream
                    "busy_s": stats.busy_s, "step_device_s": stats.step_device_s,
                    "admit_device_s": stats.admit_device_s,
                    "bp_in_steps_gpix_pulse_s": stats.updates / max(stats.step_device_s, 1e-9) / 1e9,
                    "peak_active": stats.peak_active, "graph_launches": stats.graph_launches,
                    "peak_gb": stats.peak_bytes / 2**30, "clocks": clk})
        if one_shot is not None:
            u = sum(one_shot[i][0] for i in order)
            t_bp = sum(one_shot[i][2] for i in order) * 1e-3
            t_rc = sum(one_shot[i][1] for i in order) * 1e-3
            out[-1]["one_shot_same_jobs"] = {"bp_gpix_pulse_s": u / t_bp / 1e9,
                                             "rc_bp_gpix_pulse_s": u / (t_bp + t_rc) / 1e9}
    return out


SERVE_WARMUP_JOBS = 4  # untimed requests through each server before its timed stream

SERVE_WORKLOAD = ("config 4: Poisson arrivals, 256-8192 pulses x 2048-8192 samples, grids 256^2-4096^2 log-uniform "
                  "at 0.25 m, 9-200 targets, 20 dB SNR")


def schedule_names(step_updates):
    out = []
    for u in step_updates:
        name = (f"work-proportional steps (2^{u.bit_length() - 1} updates per job per step)" if u > 0
                else "fixed steps (512 pulses per job per step)")
        out.append((name, u))
    return out


def serve_measure(rates=(20.0, 40.0), jobs=30, n_req=12, step_updates=(1 << 32,)):
    """The serving key of the default run: a bounded sweep (n_req distinct
    requests drawn at random, `jobs` per rate, one schedule)."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp
    t0 = time.perf_counter()
    ctx = sarbp.Context(0)
    reqs = serve_requests(ctx, n_req)
    ctx.close()
    torch.cuda.empty_cache()
    one_shot = serve_one_shot(reqs)
    h2d = pinned_h2d_gbs()
    sweep = serve_sweep(reqs, list(rates), jobs, schedule_names(step_updates), one_shot)
    del reqs
    return {"metric": "serving p50/p99 latency (ms) and aggregate Gpix*pulse/s", "mode": "split",
            "workload": SERVE_WORKLOAD + f"; {n_req} distinct requests drawn at random, {jobs} jobs per rate",
            "server": {"max_jobs": 16, "hbm_budget_gb": 96, "graphs": True}, "sweep": sweep,
            "pinned_h2d_gbs": h2d, "seconds": time.perf_counter() - t0}


def pinned_h2d_gbs(nbytes=256 << 20, reps=10):
    """This host's pinned host-to-device copy rate (the path every served echo
    takes), one 256 MiB copy at a time after three warm-up copies."""
    import torch
    x = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        d.copy_(x, non_blocking=True)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(reps):
        d.copy_(x, non_blocking=True)
    torch.cuda.synchronize()
    return reps * nbytes / (time.perf_counter() - t) / 1e9


def run_serve(args):
    """Serving stream: a submitter thread draws Poisson arrivals and submits
    requests to one sarbp server; latency is submit -> image in host memory."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp
    torch.cuda.set_device(0)
    ctx = sarbp.Context(0)
    reqs = serve_requests(ctx, 24)
    ctx.close()
    torch.cuda.empty_cache()
    schedules = schedule_names(int(x) for x in args.step_updates.split(","))
    one_shot = serve_one_shot(reqs)
    out = serve_sweep(reqs, [float(r) for r in args.rates.split(",")], args.jobs, schedules, one_shot)
    line = {"metric": "serving p50/p99 latency and aggregate Gpix*pulse/s", "mode": "split",
            "workload": SERVE_WORKLOAD + "; 24 distinct requests drawn at random",
            "server": {"max_jobs": 16, "hbm_budget_gb": 96, "graphs": True,
                       "schedules": [{"name": n, "step_updates": u} for n, u in schedules]},
            "sweep": out}
    print(json.dumps(line))
    return 0


def c5_tile_window(sc, lay, x0, y0, w, h, margin=16):
    """Range bins [b0, b1) that back-projecting pixels [x0, x0 + w) x [y0, y0 + h)
    of config 5's grid can read over every pulse, with a margin."""
    g = sc.grid
    fx, fy = np.meshgrid(np.linspace(x0, x0 + w - 1, 9), np.linspace(y0, y0 + h - 1, 9))
    pts = g.origin + fx.reshape(-1, 1) * g.ux + fy.reshape(-1, 1) * g.uy
    rng = np.linalg.norm(pts[None, :, :] - sc.apc[:, None, :], axis=2)
    b = (2.0 * rng / sc.radar.c - lay.t0_bins) * lay.bin_rate
    return max(0, int(np.floor(b.min())) - margin), min(lay.nbins, int(np.ceil(b.max())) + margin)


def c5_measure(ctx, with_oracle=True):
    """Config 5: range compression (nfft 32768: two CTAs per forward transform,
    2-CTA clusters per inverse) to FP16 storage, then back-projection in
    sub-aperture (4096 pulses) x image-tile (4096^2) batches accumulated into
    the 8192^2 image.  Accuracy: the product's image over a 256^2 tile centred
    on the brightest isolated target against the FP64 oracle's back-projection
    of the product's complex64 range-compressed rows (the bins that tile
    reads), plus the product's range compression of a few whole pulses against
    the oracle's."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes
    t_all = time.perf_counter()
    sc = scenes.config5()
    r, g, lay = sarbp.scene_args(sc)
    echo = torch.empty((sc.np_, sc.ns * 2), dtype=torch.float32, device="cuda")
    sarbp.synthesize(ctx, sc, out=echo)
    ctx.synchronize()
    rc = torch.empty((sc.np_, lay.nbins), dtype=torch.float32, device="cuda")  # complex16 = 4 bytes/bin
    scale = torch.empty(sc.np_, dtype=torch.float32, device="cuda")
    apc = torch.from_numpy(sc.apc).cuda()
    img = torch.empty((g.ny, g.nx * 2), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sptr = sarbp.ctypes.c_void_p(stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    tile, sub = 4096, 4096
    row_bytes = lay.nbins * 4
    tile_buf = torch.empty((tile, tile * 2), dtype=torch.float32, device="cuda")

    def step():
        ev[0].record(stream)
        ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), sc.np_, sc.ns,
                                               sarbp.STORE_C32H, rc.data_ptr(), scale.data_ptr(), sptr), "rc")
        ev[1].record(stream)
        for ty in range(0, g.ny, tile):
            for tx in range(0, g.nx, tile):
                gs = sub_grid(g, tx, ty, min(tile, g.nx - tx), min(tile, g.ny - ty))
                for p0 in range(0, sc.np_, sub):
                    v = sarbp.RcView()
                    v.data = rc.data_ptr() + p0 * row_bytes
                    v.scale = scale.data_ptr() + p0 * 4
                    v.storage, v.np, v.nbins = sarbp.STORE_C32H, min(sub, sc.np_ - p0), lay.nbins
                    v.t0_bins, v.bin_rate = lay.t0_bins, lay.bin_rate
                    # the tile writes a strided sub-image: back-project into a contiguous tile buffer
                    ctx.check(ctx.lib.sarbp_backproject(ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(v),
                                                        apc.data_ptr() + p0 * 24, sarbp.ctypes.byref(gs),
                                                        sarbp.MODE_FP16STORE, tile_buf.data_ptr(), int(p0 > 0),
                                                        sptr), "bp")
                torch.cuda.current_stream().wait_stream(stream)
                with torch.cuda.stream(stream):
                    img.view(g.ny, g.nx, 2)[ty:ty + gs.ny, tx:tx + gs.nx].copy_(tile_buf.view(gs.ny, gs.nx, 2))
        ev[2].record(stream)

    step()  # warm-up
    stream.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    n0 = ctx.launches()
    step()
    stream.synchronize()
    clk = clocks.stop()
    ctx.synchronize()
    rc_ms = ev[0].elapsed_time(ev[1])
    bp_ms = ev[1].elapsed_time(ev[2])
    out = {"metric": "BP Gpix*pulse/s", "value": sc.updates / (bp_ms * 1e-3) / 1e9, "unit": "Gpix*pulse/s",
           "config": "config 5: 16384 pulses x 16384 samples (curved track: 0.5 m / 200 m sinusoid + 2 cm jitter) "
                     "-> 8192^2 at 0.25 m, 200 targets, 20 dB, FP16 storage + split precision, sub-apertures of "
                     "4096 pulses x 4096^2 tiles", "bp_ms": bp_ms, "rc_ms": rc_ms,
           "gpu_launches": ctx.launches() - n0, "rc_bytes_gib": sc.np_ * lay.nbins * 4 / 2**30, "clocks": clk}
    del tile_buf
    if with_oracle:
        from oracle import oracle as orc
        orc.set_threads(host_threads())
        rc64 = torch.empty((sc.np_, lay.nbins * 2), dtype=torch.float32, device="cuda")
        ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), sc.np_, sc.ns,
                                               sarbp.STORE_C64, rc64.data_ptr(), None, sptr), "rc64")
        stream.synchronize()
        ctx.synchronize()
        t = time.perf_counter()
        # range compression of whole pulses (32768-point split path) against the oracle's
        rows = [0, sc.np_ // 3, 2 * sc.np_ // 3, sc.np_ - 1]
        e_rows = echo[rows].cpu().numpy().view(np.complex64).astype(np.complex128)
        h = orc.chirp(lay.nc, 1.0 / sc.radar.fs, sc.radar.kr, sc.radar.tp, sc.radar.tp / 2.0, False)
        ref_rows = orc.range_compress_raw(e_rows, h, lay.nfft, lay.shift, sc.radar.upsample, 1.0 / lay.nfft,
                                          lay.nbins)
        rc_err = metrics.rel_l2_db(rc64[rows].cpu().numpy().view(np.complex64), ref_rows)
        # back-projection: a 256^2 tile centred on the brightest isolated target
        tx, ty = isolated_target_pixels(sc, n=1, margin=128)[0]
        x0, y0 = tx - 128, ty - 128
        b0, b1 = c5_tile_window(sc, lay, x0, y0, 256, 256)
        win = np.ascontiguousarray(rc64.view(sc.np_, lay.nbins, 2)[:, b0:b1].contiguous().cpu().numpy()
                                   .view(np.complex64)[..., 0])
        del rc64
        sg = sc.grid
        ref = orc.backproject_raw(win, sc.apc, sg.origin + x0 * sg.ux + y0 * sg.uy, sg.ux, sg.uy, (0, 0, 256, 256),
                                  sc.radar.fc, sc.radar.c, lay.t0_bins + b0 / lay.bin_rate, lay.bin_rate)
        mine = img.view(g.ny, g.nx, 2)[y0:y0 + 256, x0:x0 + 256].contiguous().cpu().numpy().view(np.complex64)[..., 0]
        c0, c1 = 128 - PATCH // 2, 128 + PATCH // 2
        pt = point_target_diffs([mine[c0:c1, c0:c1]], [ref[c0:c1, c0:c1]])
        out["accuracy"] = {"vs_cpu_oracle": {
            "fp16store": {"rel_l2_db": metrics.rel_l2_db(mine, ref), **pt},
            "tile": [x0, y0, 256, 256], "target_px": [tx, ty], "bins": [b0, b1],
            "oracle_input": "the product's complex64 range compression of the same echo (bins of the tile)",
            "rc_rel_l2_db_vs_oracle": rc_err, "rc_pulses_checked": rows,
            "oracle_s": time.perf_counter() - t}}
    del echo, rc, scale, apc, img
    out["seconds"] = time.perf_counter() - t_all
    return out


def run_c5(args):
    """Config 5 on its own line (see c5_measure)."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp
    torch.cuda.set_device(0)
    ctx = sarbp.Context(0)
    line = c5_measure(ctx, with_oracle=not args.no_cpu)
    print(json.dumps(line))
    ctx.close()
    return 0


def run_autofocus(args):
    """Autofocus on the APC track: sharpness iterations (back-projection with
    per-pulse phase corrections, sharpness weights, weighted projection) on a
    config-2 geometry with an injected phase error; the projection kernel timed
    alone against the same issue-rate roofline as back-projection."""
    import torch
    from sar_cambrianaccelerationcard_gb300 import sarbp, scenes
    torch.cuda.set_device(0)
    n_img = 2048 if args.size == "full" else (1024 if args.size == "medium" else 256)
    sc = scenes.config2(n_img=n_img)
    ctx = sarbp.Context(0)
    r, g, lay = sarbp.scene_args(sc)
    echo = torch.empty((sc.np_, sc.ns * 2), dtype=torch.float32, device="cuda")
    sarbp.synthesize(ctx, sc, out=echo)
    rc = torch.empty((sc.np_, lay.nbins), dtype=torch.complex64, device="cuda")
    ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), sc.np_, sc.ns,
                                           sarbp.STORE_C64, rc.data_ptr(), None, None), "rc")
    ctx.synchronize()
    del echo
    # phase error: 2 rad quadratic across the aperture + N(0, 0.4 rad), applied to the rows
    k = np.arange(sc.np_)
    eps = 8.0 * (k / (sc.np_ - 1) - 0.5) ** 2 + np.random.default_rng(3).normal(0, 0.4, sc.np_)
    rc *= torch.from_numpy(np.exp(1j * eps).astype(np.complex64)).cuda()[:, None]
    apc = torch.from_numpy(sc.apc).cuda()
    img = torch.empty((g.ny, g.nx), dtype=torch.complex64, device="cuda")
    iters = max(1, args.steps)
    upd = sc.np_ * g.nx * g.ny
    # warm-up, then the timed call (synchronous: host phase update per iteration)
    warm = max(3, args.warmup)
    ctx.autofocus(r, rc, apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, warm, image=img)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    n0 = ctx.launches()
    t = time.perf_counter()
    ph, sharp, _ = ctx.autofocus(r, rc, apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, iters, image=img)
    wall = time.perf_counter() - t
    launches = ctx.launches() - n0
    clk = clocks.stop()
    # `iters` iterations of one corrected back-projection and one projection,
    # then the final image's back-projection: 2 iters + 1 passes over the updates
    iter_ms = wall / iters * 1e3
    value = (2 * iters + 1) * upd / wall / 1e9
    res = ph + eps
    A = np.vstack([np.ones_like(k), k]).T.astype(np.float64)
    res = res - A @ np.linalg.lstsq(A, res, rcond=None)[0]
    # kernels alone, events on the launching stream
    stream = torch.cuda.Stream()
    sptr = sarbp.ctypes.c_void_p(stream.cuda_stream)
    w = torch.empty_like(img)
    w.copy_(img)
    out = torch.empty(sc.np_, dtype=torch.complex128, device="cuda")
    dph = torch.from_numpy(np.ascontiguousarray(ph)).cuda()
    v = sarbp.RcView()
    v.data, v.storage, v.np, v.nbins = rc.data_ptr(), sarbp.STORE_C64, sc.np_, lay.nbins
    v.t0_bins, v.bin_rate = lay.t0_bins, lay.bin_rate
    corr = sarbp.PulseCorr()
    corr.drange, corr.dphase = None, dph.data_ptr()

    def timed(fn, reps=5):
        for _ in range(2):
            fn()
        stream.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        for _ in range(reps):
            fn()
        ev[1].record(stream)
        stream.synchronize()
        return ev[0].elapsed_time(ev[1]) / reps

    proj_ms = timed(lambda: ctx.check(ctx.lib.sarbp_project_weighted(
        ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(v), apc.data_ptr(), sarbp.ctypes.byref(g),
        sarbp.MODE_SPLIT, sarbp.ctypes.byref(corr), w.data_ptr(), out.data_ptr(), sptr), "proj"))
    bpx_ms = timed(lambda: ctx.check(ctx.lib.sarbp_backproject_ex(
        ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(v), apc.data_ptr(), sarbp.ctypes.byref(g),
        sarbp.MODE_SPLIT, sarbp.ctypes.byref(corr), img.data_ptr(), 0, sptr), "bp_ex"))
    bp_ms = timed(lambda: ctx.check(ctx.lib.sarbp_backproject(
        ctx.h, sarbp.ctypes.byref(r), sarbp.ctypes.byref(v), apc.data_ptr(), sarbp.ctypes.byref(g),
        sarbp.MODE_SPLIT, img.data_ptr(), 0, sptr), "bp"))
    fp32_rate, mufu_rate, sms = ctx.probe_issue_rates()
    peak = min(fp32_rate / FP32_OPS_PER_UPDATE, mufu_rate / MUFU_OPS_PER_UPDATE) / 1e9
    proj_rate = upd / (proj_ms * 1e-3) / 1e9
    # CPU: one iteration's core (corrected BP + projection) of the FP64 oracle on a tile
    from oracle import oracle as orc
    orc.set_threads(host_threads())
    side = 512 if args.size == "full" else 128  # ~4 s of host work at full size
    cs = scenes.config2(n_img=side)
    crc = orc.range_compress(cs, orc.echo(cs)) * np.exp(1j * eps)[:, None]
    t = time.perf_counter()
    cimg = orc.backproject_corr(cs, crc, None, -eps)
    orc.project_weighted(cs, crc, np.abs(cimg) ** 2 * cimg, None, -eps)
    cpu_s = time.perf_counter() - t
    cpu_v = 2 * side * side * cs.np_ / cpu_s / 1e9
    line = {
        "metric": "autofocus Gpix*pulse/s (corrected back-projection + projection per iteration, final image "
                  "included)", "value": value,
        "unit": "Gpix*pulse/s", "n_gpus": 1, "steps": iters, "warmup": warm, "ms_per_step": iter_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (GPU echo synthesiser, seeded) with an injected per-pulse phase error",
        "config": {"workload": f"sharpness autofocus, {sc.np_} pulses x {sc.ns} samples -> {g.nx}x{g.ny} at 0.25 m, "
                               "phase error 2 rad quadratic + N(0, 0.4 rad)", "mode": "split",
                   "l2": "inputs larger than L2 (2 GB range-compressed data)"},
        "accuracy": {"phase_residual_rad_after_linear_fit": float(res.std()),
                     "sharpness_gain": float(sharp[-1] / sharp[0])},
        "kernels": {"projection_ms": proj_ms, "projection_gpix_pulse_s": proj_rate,
                    "corrected_bp_ms": bpx_ms, "plain_bp_ms": bp_ms},
        "roofline": {"bound": "issue (FP32+MUFU)", "achieved": proj_rate, "peak": peak, "unit": "Gpix*pulse/s",
                     "frac": proj_rate / peak, "traffic": None, "kernel": "bp_kernel<SPLIT, projection>"},
        "e2e": {"value": value, "unit": "Gpix*pulse/s", "h2d_bytes_per_step": 8 * sc.np_,
                "d2h_bytes_per_step": 16 * sc.np_ + 8, "ms_per_step": iter_ms,
                "note": "sarbp_autofocus itself: phases cross to the host every iteration"},
        "cpu_baseline": {"value": cpu_v, "unit": "Gpix*pulse/s", "cores": orc.threads(), "kind": "port",
                         "sample": f"FP64 oracle corrected BP + projection, {side}x{side} tile x {cs.np_} pulses "
                                   f"({cpu_s:.1f} s)"},
        "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


def wk_traffic_bytes(na: int, nr: int, NA: int, NR: int) -> int:
    """Algorithmic HBM bytes of one omega-K image: the first range DFT reads the
    echo and writes the padded array (padding rows cleared); the azimuth DFT,
    the Stolt pass, the range IDFT and the azimuth IDFT each read and write the
    NA x NR complex64 array once, and azimuth lengths outside 512..4096 (or not
    powers of two) add four transposes."""
    a = 8 * NA * NR
    cols = NA & (NA - 1) == 0 and 512 <= NA <= 4096
    return 8 * na * nr + a + 4 * 2 * a + (0 if cols else 4 * 2 * a)


def run_wk(args):
    """Omega-K imager on the reference's RADARSAT-1 configuration (wk.cc:76-96):
    3072 x 2048 echo padded to 4096 x 3414, seeded synthetic echo of that shape
    (the scene's data are not shipped to the GPU host); accuracy against the FP64
    restatement on the same input."""
    import torch
    from oracle import wk as wko
    from sar_cambrianaccelerationcard_gb300 import metrics, sarbp
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ctx = sarbp.Context(0)
    p = wko.radarsat1()
    w = sarbp.wk_params(p)
    na, nr = (3072, 2048) if args.size == "full" else ((768, 512) if args.size == "medium" else (192, 128))
    NA, NR, _ = ctx.wk_padded_size(na, nr)
    rng = np.random.default_rng(11 + rank)
    echo_h = (rng.standard_normal((na, nr)) + 1j * rng.standard_normal((na, nr))).astype(np.complex64)
    d_echo = torch.from_numpy(echo_h.view(np.float32)).cuda()
    d_img = torch.empty((NA, NR * 2), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sptr = sarbp.ctypes.c_void_p(stream.cuda_stream)

    def step():
        ctx.check(ctx.lib.sarbp_wk_image(ctx.h, sarbp.ctypes.byref(w), d_echo.data_ptr(), na, nr, d_img.data_ptr(),
                                         sptr), "wk")

    for _ in range(max(3, args.warmup)):
        step()
    stream.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    n0 = ctx.launches()
    # an image takes under 1 ms: at least 300 back to back (~0.25 s) so that the
    # clock sampler sees the timed region
    steps = max(args.steps, 300)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    stream.synchronize()
    clk = clocks.stop()
    launches = ctx.launches() - n0
    ms = ev0.elapsed_time(ev1) / steps
    npix = NA * NR
    # end to end: host echo in, host image out through the same call
    img_h = torch.empty((NA, NR * 2), dtype=torch.float32, pin_memory=True)
    echo_pin = torch.from_numpy(echo_h.view(np.float32)).pin_memory()
    t = time.perf_counter()
    ke = max(1, min(args.steps, 5))
    for _ in range(ke):
        ctx.check(ctx.lib.sarbp_wk_image(ctx.h, sarbp.ctypes.byref(w), echo_pin.data_ptr(), na, nr, img_h.data_ptr(),
                                         None), "wk e2e")
    e2e_s = (time.perf_counter() - t) / ke
    # accuracy and CPU time of the FP64 restatement on the same echo
    t = time.perf_counter()
    ref = wko.wk_image(echo_h.astype(np.complex128), p)
    cpu_s = time.perf_counter() - t
    err = metrics.rel_l2_db(d_img.cpu().numpy().view(np.complex64), ref)
    hbm = None
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        hbm = json.load(open(pk)).get("hbm_gbs")
    alg = wk_traffic_bytes(na, nr, NA, NR)
    line = {
        "metric": "omega-K image Mpix/s", "value": npix / (ms * 1e-3) / 1e6, "unit": "Mpix/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float phases)", "data": "synthetic (seeded)",
        "config": {"workload": f"omega-K RADARSAT-1 parameters, {na} x {nr} echo padded to {NA} x {NR}, Stolt "
                               f"{p.taps}-tap sinc", "l2": "working set 2 x 112 MB plus tables, larger than L2"},
        "accuracy": {"rel_l2_db_vs_fp64_restatement": err},
        "e2e": {"value": npix / e2e_s / 1e6, "unit": "Mpix/s", "h2d_bytes_per_step": 8 * na * nr,
                "d2h_bytes_per_step": 8 * npix, "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": (alg / (ms * 1e-3) / 1e9 / hbm) if hbm else None, "traffic": None,
                     "traffic_algorithmic": alg, "kernel": "whole omega-K pipeline"},
        "cpu_baseline": {"value": npix / cpu_s / 1e6, "unit": "Mpix/s", "cores": 1, "kind": "port",
                         "sample": f"FP64 numpy restatement of the same {na} x {nr} image ({cpu_s:.1f} s)"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    return 0


def run_ceos(args):
    """CEOS raw-data decode: the reference's extracted RADARSAT-1 scene size
    (3072 lines x 2048 cells from 9288-cell lines, code/data_process/CEOS/
    specify_parameters.m) out of a seeded synthetic CEOS file of 3072 lines."""
    import torch
    from oracle import ceos
    from sar_cambrianaccelerationcard_gb300 import sarbp
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    ctx = sarbp.Context(0)
    lay = ceos.CeosLayout()
    n, m, c0 = (3072, 2048, 1049) if args.size == "full" else (512, 2048, 1049)
    rng = np.random.default_rng(3)
    v = (2 * rng.integers(-8, 8, (n, m)) + 1) + 1j * (2 * rng.integers(-8, 8, (n, m)) + 1)
    raw = ceos.write(v, rng.integers(0, 32, n), lay, first_cell=c0, seed=4)
    d_raw = torch.from_numpy(raw).cuda()
    d_echo = torch.empty((n, 2 * m), dtype=torch.float32, device="cuda")
    d_agc = torch.empty(n, dtype=torch.int16, device="cuda")
    w = sarbp.ceos_layout()
    stream = torch.cuda.Stream()
    sp = sarbp.ctypes.c_void_p(stream.cuda_stream)

    def step(src, dst, agc, sptr):
        ctx.check(ctx.lib.sarbp_ceos_decode(ctx.h, src, raw.nbytes, sarbp.ctypes.byref(w), 0, n, c0, m, 1, dst,
                                            agc, sptr), "ceos")

    for _ in range(max(3, args.warmup)):
        step(d_raw.data_ptr(), d_echo.data_ptr(), d_agc.data_ptr(), sp)
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    # a decode takes under 20 us: at least 15000 back to back (~0.25 s) so that
    # the clock sampler sees the timed region and the host's enqueue rate (also
    # reported) runs ahead of the device
    steps = max(args.steps, 15000)
    src, dst, agc, t_host = d_raw.data_ptr(), d_echo.data_ptr(), d_agc.data_ptr(), time.perf_counter()
    e0.record(stream)
    for _ in range(steps):
        step(src, dst, agc, sp)
    e1.record(stream)
    t_host = time.perf_counter() - t_host
    stream.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / steps
    # bytes the decode must move: each line's sample window and AGC byte in, the echo out
    alg = n * (2 * m + 1) + 8 * n * m + 2 * n
    raw_pin = torch.from_numpy(raw).pin_memory()
    echo_h = torch.empty((n, 2 * m), dtype=torch.float32, pin_memory=True)
    agc_h = torch.empty(n, dtype=torch.int16, pin_memory=True)
    ke = max(1, min(args.steps, 5))
    t = time.perf_counter()
    for _ in range(ke):
        step(raw_pin.data_ptr(), echo_h.data_ptr(), agc_h.data_ptr(), None)
    e2e_s = (time.perf_counter() - t) / ke
    t = time.perf_counter()
    ref, _ = ceos.read(raw, lay, 0, n, c0, m)
    cpu_s = time.perf_counter() - t
    exact = bool(np.array_equal(d_echo.cpu().numpy().view(np.complex64), ref))
    hbm = None
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        hbm = json.load(open(pk)).get("hbm_gbs")
    line = {
        "metric": "CEOS decode range lines/s", "value": n / (ms * 1e-3), "unit": "lines/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
        "host_enqueue_us_per_call": 1e6 * t_host / steps,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8 -> f32", "data": "synthetic CEOS file (seeded)",
        "config": {"workload": f"RADARSAT-1 CEOS layout, {n} lines x {m} of 9288 cells from {raw.nbytes / 1e6:.0f} MB"},
        "accuracy": {"bit_exact_vs_reader_restatement": exact},
        "e2e": {"value": n / e2e_s, "unit": "lines/s", "h2d_bytes_per_step": raw.nbytes - lay.file_header,
                "d2h_bytes_per_step": 8 * n * m + 2 * n, "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": alg / (ms * 1e-3) / 1e9 / hbm if hbm else None, "traffic": None,
                     "traffic_algorithmic": alg, "kernel": "ceos_decode_kernel"},
        "cpu_baseline": {"value": n / cpu_s, "unit": "lines/s", "cores": 1, "kind": "port",
                         "sample": f"numpy restatement of the reader, same {n} lines ({cpu_s:.2f} s)"},
        "gpu_launches": args.steps, "clocks": clk,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.ceos:
        return run_ceos(args)
    if args.wk:
        return run_wk(args)
    if args.c5:
        return run_c5(args)
    if args.serve:
        return run_serve(args)
    if args.autofocus:
        return run_autofocus(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
