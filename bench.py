#!/usr/bin/env python
"""SVGF denoiser benchmark: 4K frames/s, HBM roofline fraction, end-to-end rate.

Workload (one "step" = one frame of the chain): the FULL SVGF (5 a-trous
levels, sigma_l 4 / sigma_n 128 / sigma_z 1, alpha 0.2) at 3840x2160 with
FP32 storage on a seeded synthetic 60-frame sequence (camera yaw 0.5 deg/frame
+ 0.05 m/frame, a plane appearing at frame 30), inputs RGBA32F radiance, R32F
depth, RGB32F normals, RG32F motion.  Steps cycle through the sequence; the
wrap from the last frame to the first is a camera cut (a full disocclusion).
Every frame's inputs (332 MB) and the state (664 MB) exceed the 126 MB L2, so
no explicit L2 flush is needed between steps.

  value : frames/s with inputs resident in HBM, device-timed with CUDA events
  e2e   : frames/s through the host-memory C-ABI call (tg_svgf_denoise_host):
          pinned host inputs copied in and the result copied out every step
  roofline : the dominant kernel family's compulsory bytes / its CUDA-event time
  cpu_baseline : the CPU oracle (float32 FULL port, OpenMP over rows) on the
          same frames, bounded to ~15 s

Multi-GPU: replicas only (every rank denoises its own stream; no collective on
the data path); value = frames of all ranks / max time over ranks.
"""
from __future__ import annotations

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

METRIC = "4K SVGF frames/s + % HBM roofline; batched p50/p99 ms vs plain at ≤1e-3 rel err"
KEYS = ("radiance", "depth", "normal", "motion")


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("tg", "reference"), default="tg")
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--mode", choices=("full", "ref"), default="full")
    ap.add_argument("--storage", choices=("fp32", "fp16"), default="fp32")
    ap.add_argument("--pool", type=int, default=60, help="distinct frames generated (the sequence length)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-profile", action="store_true", help="no per-kernel events in the timed region")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-extras", action="store_true", help="skip the FP16 / REF_EXACT / batched / accuracy lines")
    ap.add_argument("--batch-streams", type=int, default=64)
    ap.add_argument("--batch-frames", type=int, default=30)
    ap.add_argument("--serve-sessions", type=int, default=256)
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--serve-rate", type=float, default=4000.0)
    ap.add_argument("--serve-repeats", type=int, default=3, help="offered-load runs whose latencies are reported "
                                                                   "as the median")
    ap.add_argument("--only", choices=("fog", "post", "eye", "batched", "serving"), default=None,
                    help="run one line alone (froxel filter, bloom + post-process, eye readback for --steps timed "
                         "frames; the batched or the serving form) and print its JSON; one GPU")
    return ap.parse_args(argv)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        idx = {r[0] for r in rows}
        want = str(self.gpu_index) if str(self.gpu_index) in idx else rows[0][0]
        rows = [r for r in rows if r[0] == want]

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, world, device):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, world, device):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def workload(args):
    from tron_grid_gb300 import scene

    spec = scene.pan_with_disocclusion(args.width, args.height, seed=0)
    name = (f"{'FULL' if args.mode == 'full' else 'REF_EXACT'} SVGF {args.width}x{args.height}, "
            f"{args.storage.upper()} storage, {5 if args.mode == 'full' else 3} a-trous levels, "
            f"{args.pool}-frame synthetic sequence (yaw 0.5 deg + 0.05 m per frame, plane appears at frame 30)")
    return spec, name


def gen_frames(spec, n, dev, storage, mode):
    import torch

    from tron_grid_gb300 import scene

    sc = scene.PlaneScene(spec, device=dev)
    frames = []
    for t in range(n):
        fr = sc.frame(t)
        d = {k: fr[k] for k in KEYS}
        if storage == "fp16":
            d["radiance"] = d["radiance"].to(torch.float16)
            d["normal"] = scene.oct16_encode(d["normal"])
        if mode == "ref":
            d = {"radiance": d["radiance"]}
        frames.append(d)
    torch.cuda.synchronize()
    return frames


def algo_bytes_per_px(mode, storage):
    """Compulsory bytes per pixel of the whole chain: inputs once, state read + written once, output once."""
    if mode == "full":
        if storage == "fp32":
            inputs, state, out = 16 + 4 + 12 + 8, 16 + 16 + 8, 16
        else:
            inputs, state, out = 8 + 4 + 4 + 8, 8 + 8 + 4, 8
        return inputs + 2 * state + out
    if storage == "fp32":
        return 16 + 2 * 8 + 16
    return 8 + 2 * 4 + 8


def first_frames(steps, warmup, pool, event=30):
    """(w0, t0): the sequence index of the first warm-up frame and of the first timed frame.

    Steps walk the sequence in order (modulo its length).  When the timed steps cover less than the whole
    sequence, the window is placed so that it holds `event` (the frame where a plane appears: a forced
    disocclusion), and the warm-up frames are the ones just before it."""
    if pool > event and steps < pool:
        t0 = min(max(0, event - steps // 2), pool - steps)
    else:
        t0 = warmup % pool
    return (t0 - warmup) % pool, t0


def window_text(steps, t0, pool):
    last = t0 + steps - 1
    if steps >= pool:
        return f"{steps} frames from sequence frame {t0}, cycling the {pool}-frame sequence (every frame, cuts included)"
    return f"sequence frames {t0}..{last % pool}" + (" (wrapping: a camera cut)" if last >= pool else "")


def run_tg(args, rank, world, local):
    import torch

    import tron_grid_gb300 as tg

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    spec, name = workload(args)
    W, H = spec.width, spec.height
    mode = tg.MODE_FULL if args.mode == "full" else tg.MODE_REF_EXACT
    storage = tg.STORAGE_FP32 if args.storage == "fp32" else tg.STORAGE_FP16
    frames = gen_frames(spec, args.pool, dev, args.storage, args.mode)
    out_dt = torch.float32 if args.storage == "fp32" else torch.float16
    outs = [torch.empty((H, W, 4), dtype=out_dt, device=dev) for _ in range(2)]
    den = tg.Denoiser(W, H, mode=mode, storage=storage, device=local)
    kpf = den.info()["kernels_per_frame"]
    stream = torch.cuda.current_stream()

    w0, t0 = first_frames(args.steps, args.warmup, len(frames))

    def step(i):
        fr = frames[(w0 + i) % len(frames)]
        den.denoise(fr["radiance"], fr.get("depth"), fr.get("normal"), fr.get("motion"), out=outs[i & 1])

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = Clocks(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0] if world == 1 else local)
    clocks.start()
    if not args.no_profile:
        den.profile(True)
        den.profile_read(reset=True)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for i in range(args.steps):
        step(args.warmup + i)  # sequence frame (t0 + i) % pool
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = evs[0].elapsed_time(evs[-1])
    per = sorted(evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps))
    prof = den.profile_read(reset=True) if not args.no_profile else {}
    den.profile(False)
    t_max = max_over_ranks(total_ms, world, dev)
    frames_all = sum_over_ranks(float(args.steps), world, dev)
    value = frames_all / (t_max / 1000.0)
    px = W * H

    res = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": name, "width": W, "height": H, "mode": args.mode, "storage": args.storage,
                      "parallelism": f"replicas{world}" if world > 1 else "single",
                      "l2": "no flush: every frame's inputs (332 MB FP32) and state exceed the 126 MB L2",
                      "frames_in_pool": args.pool, "timed_frames": window_text(args.steps, t0, len(frames)),
                      "warmup_frames": f"the {args.warmup} sequence frames before the timed ones"},
           "mpx_per_s": value * px / 1e6,
           "p50_ms": per[len(per) // 2], "p99_ms": per[min(len(per) - 1, int(0.99 * len(per)))],
           "gpu_launches": kpf * args.steps}
    peak, peak_src = load_peaks()
    chain_bytes = algo_bytes_per_px(args.mode, args.storage) * px
    # The path's roofline: the compulsory bytes of the whole chain per frame (inputs once, state read and written
    # once, output once; a-trous scratch not counted) over the frame time.  `roofline` below is the dominant
    # kernel's own figure.
    res["chain_roofline"] = {"what": "the path's roofline: compulsory bytes of the whole chain per frame over the "
                                     "frame time",
                             "algo_bytes_per_px": algo_bytes_per_px(args.mode, args.storage),
                             "achieved": chain_bytes / (res["ms_per_step"] / 1e3) / 1e9, "peak": peak,
                             "unit": "GB/s", "peak_source": peak_src}
    res["chain_roofline"]["frac"] = res["chain_roofline"]["achieved"] / peak
    if prof:
        kern = {}
        for k, v in prof.items():
            ms = v["total_ms"] / max(v["launches"], 1)
            kern[k] = {"launches": v["launches"], "avg_ms": ms, "share": v["total_ms"] / max(total_ms, 1e-9),
                       "gbs": v["algo_bytes"] / max(v["total_ms"], 1e-12) / 1e6}
        dom = max(prof, key=lambda k: prof[k]["total_ms"])
        d = prof[dom]
        achieved = d["algo_bytes"] / (d["total_ms"] / 1e3) / 1e9
        traffic = load_traffic().get(f"{dom}:{args.mode}:{args.storage}")
        tr = None
        if traffic:
            tr = traffic["dram_bytes_per_px"] * px
        res["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "traffic": tr,
                           "algo_bytes_per_launch": d["algo_bytes"] / d["launches"], "peak_source": peak_src,
                           # the compute side of the same kernel: issue slots busy in the ncu capture of profiles/
                           "issue_active_pct": traffic.get("issue_active_pct") if traffic else None}
        res["kernels"] = kern
    res["clocks"] = clk
    den.close()
    del outs
    torch.cuda.synchronize()

    if not args.no_e2e:
        res["e2e"] = run_e2e(args, frames, dev, mode, storage, world, t0)
    else:
        res["e2e"] = None
    del frames
    torch.cuda.empty_cache()
    if not args.no_extras and args.mode == "full" and args.storage == "fp32":
        res["fp16_4k"] = run_single(args, dev, "full", "fp16", steps=min(args.steps, 120))
        res["ref_exact_4k"] = run_single(args, dev, "ref", "fp16", steps=min(args.steps, 120))
        # the reference's own published figure is ~0.71 ms for this chain at 1280x720 (debug build, RTX 4090 Laptop)
        res["ref_exact_720p"] = run_single(args, dev, "ref", "fp16", steps=min(args.steps, 200), size=(1280, 720))
        res["batched"] = run_batched(args, dev)
        res["serving"] = run_serving(args, dev)
        res["fog_filter"] = run_fog(args, dev, cpu=rank == 0 and world == 1 and not args.no_cpu)
        res["bloom_post"] = run_post(args, dev, cpu=rank == 0 and world == 1 and not args.no_cpu)
        res["eye_readback"] = run_eye(args, dev, cpu=rank == 0 and world == 1 and not args.no_cpu)
        if rank == 0:
            res["accuracy"] = run_accuracy(dev)
        torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_cpu:
        res["cpu_baseline"] = run_cpu_baseline(args, spec, seconds=args.cpu_seconds, start=t0)
    return res


def run_single(args, dev, mode_s, storage_s, steps, size=None):
    """Device-timed frames/s of one stream in another mode/storage on the same sequence (4K unless `size`)."""
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import scene

    spec, _ = workload(args)
    if size is not None:
        spec = scene.pan_with_disocclusion(size[0], size[1], seed=0)
    W, H = spec.width, spec.height
    frames = gen_frames(spec, min(args.pool, 30), dev, storage_s, mode_s)
    mode = tg.MODE_FULL if mode_s == "full" else tg.MODE_REF_EXACT
    storage = tg.STORAGE_FP32 if storage_s == "fp32" else tg.STORAGE_FP16
    dt = torch.float32 if storage_s == "fp32" else torch.float16
    out = torch.empty((H, W, 4), dtype=dt, device=dev)
    stream = torch.cuda.current_stream()

    def run(profile):
        """Frames 5 .. 5+steps-1 of the sequence after frames 0..4 on a fresh stream state: (ms per frame, the
        library's per-kernel profile or None)."""
        den = tg.Denoiser(W, H, mode=mode, storage=storage, device=dev.index)

        def step(i):
            fr = frames[i % len(frames)]
            den.denoise(fr["radiance"], fr.get("depth"), fr.get("normal"), fr.get("motion"), out=out)

        for i in range(5):
            step(i)
        torch.cuda.synchronize()
        if profile:
            den.profile(True)
            den.profile_read(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            step(5 + i)
        e1.record(stream)
        torch.cuda.synchronize()
        prof = den.profile_read(reset=True) if profile else None
        den.close()
        return e0.elapsed_time(e1) / steps, prof

    # frames/s from a run without the library's per-kernel events (on a chain of ~0.1 ms kernels their records
    # cost several percent), the per-kernel breakdown from a second, profiled run over the same frames
    ms, _ = run(False)
    _, prof = run(True)
    bpp = algo_bytes_per_px(mode_s, storage_s)
    peak, _ = load_peaks()
    return {"frames_per_s": 1e3 / ms, "ms_per_frame": ms, "mpx_per_s": W * H / ms / 1e3,
            "algo_bytes_per_px": bpp, "chain_hbm_frac": bpp * W * H / (ms / 1e3) / 1e9 / peak,
            "kernels": {k: {"launches": v["launches"], "avg_ms": v["total_ms"] / max(v["launches"], 1),
                            "gbs": v["algo_bytes"] / max(v["total_ms"], 1e-12) / 1e6} for k, v in prof.items()},
            "workload": f"{'FULL' if mode_s == 'full' else 'REF_EXACT'} {W}x{H} {storage_s.upper()} storage"}


def run_fog(args, dev, steps=200, cpu=True):
    """The volumetric-fog froxel filter (src/volumetric_filter.slang, tg_fog_filter) on rgba16f volumes: the
    reference's 320x180x64 grid and a 640x360x128 grid, one pass per frame of a 60-frame camera sequence with the
    (history, output) pair alternating.  Each pass is timed by its own CUDA events with L2 flushed (a 256 MB
    write) before it; the CPU baseline is the oracle on the host cores at the reference grid."""
    import numpy as np
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import fog_scene

    peak, src = load_peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    res = {"workload": "froxel filter, rgba16f inject/history/output, 60-frame camera sequence (yaw 0.5 deg + "
                       "0.05 m per frame), alpha 0.1, near 0.1 m, far 120 m",
           "algo_bytes_per_froxel": 24, "l2": "flushed (256 MB write) before every timed pass"}
    for name, kw in (("reference_grid", {}), ("grid_640x360x128", dict(width=640, height=360, depth=128))):
        spec = fog_scene.fog_config(**kw)
        sc = fog_scene.FogScene(spec, device=dev)
        pool = [sc.inject(t) for t in range(8)]
        params = [tg.fog_params(**sc.param_args(t)) for t in range(spec.frames)]
        ff = tg.FogFilter(spec.width, spec.height, spec.depth, device=dev)

        def step(i):
            t = 1 + i % (spec.frames - 1)
            ff.step(params[t], pool[t % len(pool)])

        for i in range(5):
            step(i)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        for i in range(steps):
            flush.fill_(i & 255)
            evs[i][0].record(stream)
            step(5 + i)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        ms = np.array([a.elapsed_time(b) for a, b in evs])
        n = spec.width * spec.height * spec.depth
        avg = float(ms.mean())
        gbs = 24 * n / (avg / 1e3) / 1e9
        res[name] = {"froxels": n, "ms_per_pass": avg, "p50_ms": float(np.median(ms)), "p99_ms": float(np.percentile(ms, 99)),
                     "gfroxels_per_s": n / avg / 1e6, "gpu_launches_per_pass": 1,
                     "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                  "peak_source": src}}
        del pool, ff
    del flush
    torch.cuda.empty_cache()
    if cpu:
        import oracle

        spec = fog_scene.fog_config()
        sc = fog_scene.FogScene(spec)
        hist = np.zeros((spec.depth, spec.height, spec.width, 4), np.float32)
        done, el = 0, 0.0
        while el < 5.0 and done < 59:
            t = 1 + done
            blk = oracle.fog_param_block(**sc.param_args(t))
            raw = sc.inject(t).float().numpy()
            t0 = time.perf_counter()
            hist = oracle.fog_filter(blk, raw, hist)
            el += time.perf_counter() - t0
            done += 1
        n = spec.width * spec.height * spec.depth
        res["cpu_baseline"] = {"value": done * n / el / 1e6, "unit": "Mfroxels/s", "ms_per_pass": el / done * 1e3,
                               "cores": oracle.num_threads(), "kind": "port",
                               "sample": f"{done} passes of the 320x180x64 sequence (float32, fp16 stores)"}
    return res


def run_post(args, dev, steps=200, cpu=True):
    """The bloom + post-process chain (src/bloom_downsample.slang, src/postprocess.slang; tg_post_process): rgba16f
    HDR in, B8G8R8A8 display image out, at 3840x2160 and at the reference's published 1280x720.  HDR frames are the
    4K sequence's noisy radiance (emitters up to 20 bloom); L2 is flushed (a 256 MB write) before every timed frame,
    each frame timed by its own CUDA events.  Compulsory bytes: HDR read 8 + display write 4 = 12 B/px (the bloom
    chain is scratch).  The CPU baseline is the oracle on the host cores at 4K."""
    import numpy as np
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import scene

    peak, src = load_peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    res = {"workload": "bloom extract + downsample + upsample mip chain (threshold 1.0, 6 mips) and post-process "
                       "(chromatic aberration, bloom 0.095, ACES, sRGB, grade, vignette), rgba16f HDR -> BGRA8",
           "algo_bytes_per_px": 12, "l2": "flushed (256 MB write) before every timed frame"}
    hdr4k = None
    for name, (W, H) in (("3840x2160", (3840, 2160)), ("1280x720", (1280, 720))):
        sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=0), device=dev)
        pool = [sc.frame(t)["radiance"].to(torch.float16).contiguous() for t in range(4)]
        if hdr4k is None:
            hdr4k = pool[0].float().cpu().numpy()
        pp = tg.PostProcessor(W, H, device=dev.index)
        out = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
        for i in range(5):
            pp.process(pool[i % 4], out)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        for i in range(steps):
            flush.fill_(i & 255)
            evs[i][0].record(stream)
            pp.process(pool[i % 4], out)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        ms = np.array([a.elapsed_time(b) for a, b in evs])
        avg = float(ms.mean())
        gbs = 12 * W * H / (avg / 1e3) / 1e9
        res[name] = {"ms_per_frame": avg, "p50_ms": float(np.median(ms)), "mpx_per_s": W * H / avg / 1e3,
                     "mip_count": pp.info()["mip_count"],
                     "gpu_launches_per_frame": 1 + max(0, pp.info()["mip_count"] - 6) + pp.info()["mip_count"],
                     "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                                  "peak_source": src}}
        pp.close()
        del pool
    res["1280x720"]["reference_published_ms"] = {"bloom_down": 0.025, "bloom_up": 0.020, "post": 0.029,
                                                 "note": "debug build, RTX 4090 Laptop (TODO.md:1483-1488)"}
    del flush
    torch.cuda.empty_cache()
    if cpu:
        import oracle

        done, el = 0, 0.0
        while el < 4.0 and done < 20:
            t0 = time.perf_counter()
            oracle.post_frame(hdr4k)
            el += time.perf_counter() - t0
            done += 1
        res["cpu_baseline"] = {"value": done / el, "unit": "frames/s", "ms_per_frame": el / done * 1e3,
                               "cores": oracle.num_threads(), "kind": "port",
                               "sample": f"{done} frames of 3840x2160 (float32 arithmetic, fp16 bloom, UNORM8 output)"}
    return res


def run_eye(args, dev, steps=200, cpu=True):
    """Eye-frame readback for AI entities (tg_eye_*; the reference's designed vision path, docs/AI_INTERFACE.md):
    every entity's BGRA8 display image + float32 depth packed as RGB888 + depth into a device slot, copied into a
    3-slot page-locked host ring, read two frames behind.  `gpu_ms_per_frame`: CUDA events around each frame's pack
    + copy; `frames_per_s`: the C API driven in a loop (image arrays built once), each submit followed by the
    acquire of frame t - 2, until the last frame lands in host memory.  Bytes to host = 7 per eye pixel."""
    import ctypes as C

    import numpy as np
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import _lib as L

    lib = L.load()
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    res = {"workload": "N eyes of BGRA8 colour + R32F depth -> RGB888 + float32 depth, 3-slot page-locked host ring"}
    for name, (n, w, h) in (("64x(64x64)", (64, 64, 64)), ("256x(128x128)", (256, 128, 128))):
        g = torch.Generator(device="cpu").manual_seed(n)
        cols = [torch.randint(0, 256, (h, w, 4), generator=g, dtype=torch.uint8).to(dev) for _ in range(n)]
        deps = [torch.rand((h, w), generator=g).to(dev) for _ in range(n)]
        er = tg.EyeReadback([(w, h)] * n, fovs=[1.57] * n, device=dev.index)
        ci = (L.Image * n)(*[L.Image(c.data_ptr(), w * 4, L.FMT_BGRA8, 0) for c in cols])
        di = (L.Image * n)(*[L.Image(d.data_ptr(), w * 4, L.FMT_R32F, 0) for d in deps])
        vis = (L.VisionData * n)()

        def step(t):
            L.check(lib.tg_eye_submit(er.handle, t, ci, di, sp))
            if t >= 2:
                L.check(lib.tg_eye_acquire(er.handle, t - 2, vis))

        for t in range(5):
            step(t)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            evs[i][0].record(stream)
            L.check(lib.tg_eye_submit(er.handle, 5 + i, ci, di, sp))
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        gpu_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        base = 5 + steps
        t0 = time.perf_counter()
        for i in range(steps):
            step(base + i)
        L.check(lib.tg_eye_acquire(er.handle, base + steps - 1, vis))
        el = time.perf_counter() - t0
        bytes_frame = n * w * h * 7
        res[name] = {"frames_per_s": steps / el, "ms_per_frame": el / steps * 1e3, "gpu_ms_per_frame": gpu_ms,
                     "host_gbs": bytes_frame / (gpu_ms / 1e3) / 1e9, "bytes_per_frame": bytes_frame,
                     "gpu_launches_per_frame": 1}
        if cpu:
            import oracle

            hc = [c.cpu().numpy() for c in cols]
            hd = [d.cpu().numpy() for d in deps]
            t0 = time.perf_counter()
            reps = 5
            for _ in range(reps):
                for c, d in zip(hc, hd):
                    oracle.eye_pack(c, d)
            res[name]["cpu_baseline"] = {"ms_per_frame": (time.perf_counter() - t0) / reps * 1e3, "cores": 1,
                                         "kind": "port", "sample": f"{reps} frames, numpy packing of host copies"}
        er.close()
    return res


def run_batched(args, dev):
    """Many-stream batch: N streams of seeded resolutions, FP16, one persistent launch per step (autotuned,
    graph-replayed), against the plain per-stream FP32 path on the same frames."""
    import numpy as np
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import scene
    from tron_grid_gb300.batch import Batch

    res_set = [(160, 90), (320, 180), (640, 360), (1280, 720)]
    specs = scene.stream_specs(args.batch_streams, res_set, seed=3, frames=args.batch_frames)
    sizes = [(s.width, s.height) for s in specs]
    F = args.batch_frames
    f32 = []
    f16 = []
    for sp in specs:
        sc = scene.PlaneScene(sp, device=dev)
        a32, a16 = [], []
        for t in range(F):
            fr = sc.frame(t)
            d = {k: fr[k] for k in KEYS}
            a32.append(d)
            a16.append({"radiance": d["radiance"].half(), "depth": d["depth"],
                        "normal": scene.oct16_encode(d["normal"]), "motion": d["motion"]})
        f32.append(a32)
        f16.append(a16)
    torch.cuda.synchronize()
    px = sum(w * h for w, h in sizes)
    ids = list(range(len(sizes)))
    warm = 3
    stream = torch.cuda.current_stream()

    # batched FP16
    b = Batch(sizes, storage=tg.STORAGE_FP16)
    outs16 = [torch.empty((h, w, 4), dtype=torch.float16, device=dev) for (w, h) in sizes]
    tune = b.autotune(ids, [f16[j][0] for j in ids], outs16, steps=3)
    for t in range(warm):
        b.denoise(ids, [f16[j][t] for j in ids], outs16)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(F - warm + 1)]
    torch.cuda.synchronize()
    evs[0].record(stream)
    for t in range(warm, F):
        b.denoise(ids, [f16[j][t] for j in ids], outs16)
        evs[t - warm + 1].record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    bt = sorted(evs[i].elapsed_time(evs[i + 1]) for i in range(F - warm))
    binfo = b.info()
    b.close()

    # plain per-stream FP32: one handle per stream, one call per stream per step
    dens = [tg.Denoiser(w, h, storage=tg.STORAGE_FP32, device=dev.index) for (w, h) in sizes]
    outs32 = [torch.empty((h, w, 4), device=dev) for (w, h) in sizes]
    for t in range(warm):
        for j in ids:
            fr = f32[j][t]
            dens[j].denoise(fr["radiance"], fr["depth"], fr["normal"], fr["motion"], out=outs32[j])
    pevs = [torch.cuda.Event(enable_timing=True) for _ in range(F - warm + 1)]
    torch.cuda.synchronize()
    pevs[0].record(stream)
    for t in range(warm, F):
        for j in ids:
            fr = f32[j][t]
            dens[j].denoise(fr["radiance"], fr["depth"], fr["normal"], fr["motion"], out=outs32[j])
        pevs[t - warm + 1].record(stream)
    torch.cuda.synchronize()
    pt = sorted(pevs[i].elapsed_time(pevs[i + 1]) for i in range(F - warm))
    for d in dens:
        d.close()
    # error of the batched FP16 result against the plain FP32 result (last frame, luminance)
    Y = torch.tensor([0.2126, 0.7152, 0.0722], device=dev)
    errs = []
    for j in ids:
        la = (outs16[j][..., :3].float() * Y).sum(-1)
        lb = (outs32[j][..., :3] * Y).sum(-1)
        errs.append(float(torch.sqrt(((la - lb) ** 2).sum() / (lb ** 2).sum().clamp_min(1e-30))))
    q = lambda v, f: v[min(len(v) - 1, int(f * len(v)))]
    b_mpx = px * len(bt) / (sum(bt) / 1e3) / 1e6
    p_mpx = px * len(pt) / (sum(pt) / 1e3) / 1e6
    return {"workload": f"{len(sizes)} streams from {res_set} (seeded), FULL, {F} frames, batched FP16 vs plain FP32",
            "total_px_per_step": px, "streams_by_size": {f"{w}x{h}": sizes.count((w, h)) for (w, h) in res_set},
            "batched": {"mpx_per_s": b_mpx, "p50_ms": q(bt, 0.5), "p99_ms": q(bt, 0.99),
                        "strategy": "persistent" if binfo["strategy"] == 1 else "stages",
                        "launches_per_step": 1 if binfo["strategy"] == 1 else 7,
                        "rows_per_thread": binfo["rows_per_thread"],
                        "ctas_per_sm": binfo["ctas_per_sm"], "graphs": binfo["graphs"],
                        "tuned_ms": tune["tuned_ms"], "barrier_timeouts": binfo["barrier_timeouts"]},
            "plain": {"mpx_per_s": p_mpx, "p50_ms": q(pt, 0.5), "p99_ms": q(pt, 0.99),
                      "launches_per_step": 7 * len(sizes)},
            "speedup_mpx": b_mpx / p_mpx, "rel_l2_vs_plain_max": max(errs)}


def run_serving(args, dev):
    """Serving: sessions of seeded resolutions submit frames as a Poisson process (aggregate rate),
    each session alternating exponential(2 s) idle and active periods; continuous batching (FP16 storage)
    against plain per-request launches (FP32 storage) on the same arrivals; 24 GB budget."""
    import numpy as np
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import scene
    from tron_grid_gb300.serve import Server

    res_set = [(160, 90), (320, 180), (640, 360), (1280, 720), (1920, 1080)]
    weights = [0.3, 0.3, 0.2, 0.15, 0.05]
    n = args.serve_sessions
    specs = scene.stream_specs(n, res_set, weights=weights, seed=7, frames=2)
    host = []
    for sp in specs:
        sc = scene.PlaneScene(sp, device=dev)
        fr2 = []
        for t in range(2):
            fr = sc.frame(t)
            d = {"radiance": fr["radiance"].half(), "depth": fr["depth"], "normal": scene.oct16_encode(fr["normal"]),
                 "motion": fr["motion"]}
            fr2.append({k: v.cpu().pin_memory() for k, v in d.items()})
        host.append(fr2)
    ring = 4
    outs = [[torch.empty((sp.height, sp.width, 4), dtype=torch.float16, pin_memory=True) for _ in range(ring)]
            for sp in specs]
    # arrivals: aggregate Poisson process over the sessions that are active at that moment
    rng = np.random.default_rng(11)
    T = args.serve_seconds
    switch = []
    for j in range(n):
        t, on, ev = 0.0, bool(rng.random() < 0.5), []
        while t < T:
            t += rng.exponential(2.0)
            ev.append(t)
        switch.append((on, np.array(ev)))

    def active(j, t):
        on, ev = switch[j]
        return on ^ bool(np.searchsorted(ev, t) % 2)

    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t >= T:
            break
        act = [j for j in range(n) if active(j, t)] or list(range(n))
        arrivals.append((t, int(rng.choice(act))))

    def run(server, paced):
        counts = [0] * n
        pending = {}
        lat = []
        t0 = time.perf_counter()
        for (ta, j) in arrivals:
            if paced:
                while time.perf_counter() - t0 < ta:
                    pass
            slot = counts[j] % ring
            key = (j, slot)
            if key in pending:  # the ring slot's previous frame must be done before its buffer is reused
                lat.append(server.wait(pending.pop(key)))
            pending[key] = server.submit(j, host[j][counts[j] % 2], outs[j][slot])
            counts[j] += 1
        for tk in list(pending.values()):
            lat.append(server.wait(tk))
        st = server.stats()
        ok = [x for x in lat if x["status"] == 0]
        q = np.sort([x["queue_ms"] for x in ok]) if ok else np.zeros(1)
        sv_ms = np.sort([x["latency_ms"] - x["queue_ms"] for x in ok]) if ok else np.zeros(1)
        st["queue_p50_ms"], st["queue_p99_ms"] = float(q[len(q) // 2]), float(q[min(len(q) - 1, int(0.99 * len(q)))])
        st["service_p50_ms"] = float(sv_ms[len(sv_ms) // 2])
        st["service_p99_ms"] = float(sv_ms[min(len(sv_ms) - 1, int(0.99 * len(sv_ms)))])
        st["mean_batch"] = float(np.mean([x["batch_size"] for x in ok])) if ok else 0.0
        return st

    out = {"workload": f"{n} sessions from {res_set} (weights {weights}), Poisson {args.serve_rate:.0f} frames/s for "
                       f"{T:.0f} s, exponential(2 s) idle/active periods, 24 GB budget, FP16 inputs",
           "requests": len(arrivals),
           "offered_mpx_per_s": sum(specs[j].width * specs[j].height for _, j in arrivals) / T / 1e6}
    for name, kw in (("batched", dict(batching=True, storage=tg.STORAGE_FP16, max_batch=min(n, 256))),
                     ("plain", dict(batching=False, storage=tg.STORAGE_FP32, max_batch=1))):
        sv = Server(24 << 30, max_sessions=n + 8, device=dev.index, **kw)
        # warm-up outside the timed runs: one frame of each resolution (loads the kernels, sizes the pools)
        seen = {}
        for j, sp in enumerate(specs):
            seen.setdefault((sp.width, sp.height), j)
        warm_ids = []
        for (wh, j) in seen.items():
            sid = 10_000_000 + j
            o = torch.empty_like(outs[j][0])
            for t in range(2):
                sv.wait(sv.submit(sid, host[j][t], o))
            warm_ids.append(sid)
        for sid in warm_ids:
            sv.end_session(sid)
        sv.stats(reset=True)
        res = {}
        # the offered-load run is repeated (the same arrivals each time) and its latencies reported as the median
        # over the repeats, with every repeat's p99 beside it: one run's tail moves with the shared host
        for mode, paced, reps in (("offered", True, args.serve_repeats), ("saturated", False, 1)):
            runs = []
            for _ in range(reps):
                st = run(sv, paced)
                runs.append({"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                             "mpx_per_s": st["mpx_per_s"], "completed": st["completed"], "failed": st["failed"],
                             "launches": st["launches"], "max_batch": st["max_batch_seen"],
                             "evictions": st["evictions"], "peak_resident_gb": st["peak_resident_bytes"] / 2 ** 30,
                             "queue_p50_ms": st["queue_p50_ms"], "queue_p99_ms": st["queue_p99_ms"],
                             "service_p50_ms": st["service_p50_ms"], "service_p99_ms": st["service_p99_ms"],
                             "mean_batch_of_a_request": st["mean_batch"]})
                sv.stats(reset=True)
            med = {k: (statistics.median(r[k] for r in runs) if isinstance(runs[0][k], float) else runs[0][k])
                   for k in runs[0]}
            if reps > 1:
                med["repeats"] = reps
                med["p99_ms_each"] = [round(r["p99_ms"], 3) for r in runs]
                med["p50_ms_each"] = [round(r["p50_ms"], 3) for r in runs]
            res[mode] = med
        sv.close()
        out[name] = res
    out["saturated_speedup_mpx"] = out["batched"]["saturated"]["mpx_per_s"] / max(out["plain"]["saturated"]["mpx_per_s"], 1e-9)
    return out


def run_accuracy(dev, W=3840, H=2160, frames=60):
    """The precision form's report: per-frame error of the FP32 and FP16-storage GPU paths against the float64
    oracle over the whole 60-frame sequence at 3840x2160 (frames generated on the GPU, the oracle on every host
    core).  Rows:
      fp32          FP32 storage vs float64 on the same (full-precision) inputs;
      fp16          FP16 storage (binary16 radiance, history, moments, octahedral normals) with an RGBA32F output
                    image vs float64 on the same binary16 radiance and octahedral normals: the error of the
                    FP16 state itself;
      fp16_inputs   the same FP16 result vs float64 on the full-precision inputs: adds the rounding of the
                    inputs to binary16 / octahedral codes;
      fp16_out16    the FP16 result as an RGBA16F output image would hold it (the kernel rounds its float32
                    output to nearest binary16 when it stores one) vs float64 on the same inputs.
    Metrics on luminance: max |d|, max |d| / max(|ref|, 1e-3), relative L2, PSNR with the reference frame's
    peak."""
    import numpy as np
    import torch

    import oracle
    import tron_grid_gb300 as tg
    from tron_grid_gb300 import scene

    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=0), device=dev)
    d32 = tg.Denoiser(W, H, storage=tg.STORAGE_FP32, device=dev.index)
    d16 = tg.Denoiser(W, H, storage=tg.STORAGE_FP16, device=dev.index)
    st = oracle.FullState(H, W, np.float64)
    stq = oracle.FullState(H, W, np.float64)
    P = oracle.full_params()
    Y = torch.tensor([0.2126, 0.7152, 0.0722], dtype=torch.float64, device=dev)
    o32 = torch.empty((H, W, 4), device=dev)
    o16 = torch.empty((H, W, 4), device=dev)
    names = ("fp32", "fp16", "fp16_inputs", "fp16_out16")
    rows = {k: [] for k in names}
    t_oracle = 0.0

    def lum_of(ref):
        return torch.from_numpy(ref[..., :3]).to(dev) @ Y

    for t in range(frames):
        fr = sc.frame(t)
        rad16, enc = fr["radiance"].half(), scene.oct16_encode(fr["normal"])
        d32.denoise(fr["radiance"], fr["depth"], fr["normal"], fr["motion"], out=o32)
        d16.denoise(rad16, fr["depth"], enc, fr["motion"], out=o16)
        dep, mot = fr["depth"].cpu().numpy(), fr["motion"].cpu().numpy()
        c0 = time.perf_counter()
        ref, _ = oracle.full_frame(P, st, fr["radiance"].cpu().numpy(), dep, fr["normal"].cpu().numpy(), mot)
        refq, _ = oracle.full_frame(P, stq, rad16.float().cpu().numpy(), dep, oracle.oct16_decode(enc.cpu().numpy()),
                                    mot)
        t_oracle += time.perf_counter() - c0
        lr, lq = lum_of(ref), lum_of(refq)
        for name, o, l in (("fp32", o32, lr), ("fp16", o16, lq), ("fp16_inputs", o16, lr),
                           ("fp16_out16", o16.half().float(), lq)):
            d = o[..., :3].double() @ Y - l
            mse = float((d * d).mean())
            peak = float(l.abs().max())
            rows[name].append({"max_abs": float(d.abs().max()),
                               "max_rel": float((d.abs() / l.abs().clamp_min(1e-3)).max()),
                               "rel_l2": float(torch.sqrt((d * d).sum() / (l * l).sum())),
                               "psnr_db": 10 * float(np.log10(peak * peak / mse)) if mse > 0 else None})
    d32.close()
    d16.close()
    out = {"workload": f"FULL {W}x{H}, {frames} frames (camera yaw 0.5 deg + 0.05 m per frame, plane appears at "
                       f"frame 30), GPU vs float64 oracle on {oracle.num_threads()} host threads "
                       f"({t_oracle / frames:.2f} s per frame for the two float64 runs)",
           "metric_floor": "relative errors divide by max(|reference luminance|, 1e-3)",
           "bytes_per_px": {"fp32_algo": algo_bytes_per_px("full", "fp32"), "fp16_algo": algo_bytes_per_px("full", "fp16")}}
    for name, r in rows.items():
        ps = [x["psnr_db"] for x in r if x["psnr_db"] is not None]
        worst = max(range(len(r)), key=lambda k: r[k]["max_rel"])
        out[name] = {"max_abs": max(x["max_abs"] for x in r), "max_rel": r[worst]["max_rel"], "max_rel_frame": worst,
                     "rel_l2_max": max(x["rel_l2"] for x in r), "psnr_db_min": min(ps) if ps else None,
                     "per_frame": {k: [float(f"{x[k]:.4g}") if x[k] is not None else None for x in r]
                                   for k in ("max_abs", "max_rel", "rel_l2", "psnr_db")}}
    return out


def run_e2e(args, frames, dev, mode, storage, world, t0=0):
    """Frames/s through tg_svgf_denoise_host with pinned host buffers (copies in the timed region); the host
    frames are the sequence's frames from t0 on, cycled."""
    import torch

    import tron_grid_gb300 as tg

    n_host = min(8, len(frames))
    host = [{k: v.cpu().pin_memory() for k, v in frames[(t0 + i) % len(frames)].items()} for i in range(n_host)]
    W, H = args.width, args.height
    out_dt = torch.float32 if args.storage == "fp32" else torch.float16
    houts = [torch.empty((H, W, 4), dtype=out_dt, pin_memory=True) for _ in range(3)]
    den = tg.Denoiser(W, H, mode=mode, storage=storage, device=dev.index)
    h2d = sum(v.numel() * v.element_size() for v in host[0].values())
    d2h = houts[0].numel() * houts[0].element_size()

    def step(i):
        fr = host[i % n_host]
        den.denoise_host(fr["radiance"], fr.get("depth"), fr.get("normal"), fr.get("motion"), out=houts[i % 3])

    for i in range(max(3, min(args.warmup, 8))):
        step(i)
    den.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    steps = args.steps
    c0 = time.perf_counter()
    for i in range(steps):
        step(i)
    den.synchronize()
    torch.cuda.synchronize()
    c1 = time.perf_counter()
    barrier(world)
    el = max_over_ranks(c1 - c0, world, dev)
    total = sum_over_ranks(float(steps), world, dev)
    den.close()
    link_ms = link_ms_per_step(host, houts, dev, steps)
    return {"value": total / el, "unit": "frames/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": el / steps * 1e3, "host_frames_cycled": n_host,
            "frames": f"sequence frames {t0}..{(t0 + n_host - 1) % len(frames)}, cycled",
            "api": "tg_svgf_denoise_host (pinned host buffers, a ring of three staging sets)",
            "copies_only_ms_per_step": link_ms, "link_bound_frames_per_s": 1e3 / link_ms,
            "frac_of_link_bound": (total / el) / (1e3 / link_ms),
            "link_bound": "the same copies with no compute: each step's inputs host->device on one stream and an "
                          "output device->host on another, concurrently (the host link's ceiling for this API)"}


def link_ms_per_step(host, houts, dev, steps):
    """Milliseconds per step of the end-to-end path's copies alone: the step's pinned inputs host->device on one
    stream while an output goes device->host on a second, as the denoiser's pipeline overlaps them."""
    import torch

    dbuf = {k: torch.empty(v.shape, dtype=v.dtype, device=dev) for k, v in host[0].items()}
    dout = torch.empty(houts[0].shape, dtype=houts[0].dtype, device=dev)
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def go(n):
        for i in range(n):
            with torch.cuda.stream(s_in):
                for k, v in host[i % len(host)].items():
                    dbuf[k].copy_(v, non_blocking=True)
            with torch.cuda.stream(s_out):
                houts[i % len(houts)].copy_(dout, non_blocking=True)

    go(3)
    torch.cuda.synchronize()
    c0 = time.perf_counter()
    go(steps)
    torch.cuda.synchronize()
    return (time.perf_counter() - c0) / steps * 1e3


def run_cpu_baseline(args, spec, seconds=15.0, frames=None, start=0, warm=3):
    """The float32 FULL oracle (a port of the path, OpenMP over rows, built for speed: oracle/build.py
    TIMING_CXXFLAGS) on the workload's own sequence: `warm` untimed frames before sequence frame `start`, then
    timed frames from `start` on, for `frames` frames or until `seconds` of CPU time."""
    import numpy as np

    import oracle
    from tron_grid_gb300 import scene

    sc = scene.PlaneScene(spec, device="cpu")
    W, H = spec.width, spec.height
    pool = spec.frames
    if args.mode == "full":
        P = oracle.full_params()
        st = oracle.FullState(H, W, np.float32)
    mom = np.zeros((H, W, 2), np.float32)
    f16 = args.storage == "fp16"

    def one(t):
        nonlocal mom
        fr = sc.frame(t % pool)
        arrs = [fr[k].numpy() for k in KEYS]
        if f16:
            arrs[0] = arrs[0].astype(np.float16).astype(np.float32)
        c0 = time.perf_counter()
        if args.mode == "full":
            oracle.full_frame(P, st, *arrs, fp16_store=oracle.fp16_storage_mask(True) if f16 else 0, timing=True)
        else:
            _, mom = oracle.ref_frame(arrs[0], mom, fp16_store=f16, timing=True)
        return time.perf_counter() - c0

    for t in range(start - warm, start):
        one(t)
    done, el = 0, 0.0
    while True:
        el += one(start + done)
        done += 1
        if (frames is not None and done >= frames) or (frames is None and el >= seconds):
            break
    last = (start + done - 1) % pool
    return {"value": done / el, "unit": "frames/s", "cores": oracle.num_threads(), "kind": "port",
            "flags": oracle.timing_flags(),
            "sample": f"sequence frames {start % pool}..{last} of the same {W}x{H} sequence after {warm} untimed "
                      f"frames ({el:.1f} s of CPU time, input generation excluded)"}


def run_reference(args, rank, world):
    """CPU arm: the oracle port of the path on the host cores (the reference's shader cannot run here), over the
    same warm-up and timed sequence frames as the GPU arm."""
    if rank != 0:
        return None
    spec, name = workload(args)
    import oracle

    # Each step is one frame on all host threads (about a second at 4K); steps and warm-up frames are those of
    # the GPU arm up to 120 and 20, so that the run ends within a few minutes.
    steps = max(1, min(args.steps, 120))
    warm = max(0, min(args.warmup, 20))
    w0, t0 = first_frames(steps, warm, spec.frames)
    base = run_cpu_baseline(args, spec, seconds=0.0, frames=steps, start=t0, warm=warm)
    v = base["value"]
    res = {"metric": METRIC, "impl": "reference", "value": v, "unit": "frames/s", "n_gpus": world, "steps": steps,
           "warmup": warm, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": name, "width": spec.width, "height": spec.height, "mode": args.mode,
                      "storage": args.storage},
           "cpu_baseline": base, "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    if args.mode == "full":
        res["note"] = ("the reference has no code for the FULL path (its shader stops before reprojection); the "
                       "timed CPU implementation is the oracle port of the FULL algorithm")
    if oracle.reference_available():
        import numpy as np

        from tron_grid_gb300 import scene

        sc = scene.PlaneScene(spec)
        raw = sc.frame(0)["radiance"].numpy().astype(np.float16).astype(np.float32)
        mom = np.zeros((spec.height, spec.width, 2), np.float32)
        t0 = time.perf_counter()
        n = 0
        while n < 2:
            _, mom = oracle.ref_frame_reference(raw, mom)
            n += 1
        dt = time.perf_counter() - t0
        res["reference_shader_exact"] = {"value": n / dt, "unit": "frames/s",
                                         "what": "src/svgf_denoise.slang compiled as C++ (reference constants, "
                                                 "fp16 images), same resolution"}
    return res


def main(argv=None):
    args = parse_args(argv)
    if args.only is not None:
        import torch

        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        if args.only in ("batched", "serving"):
            fn = run_batched if args.only == "batched" else run_serving
            print(json.dumps({args.only: fn(args, dev)}), flush=True)
            return
        fn = {"fog": run_fog, "post": run_post, "eye": run_eye}[args.only]
        print(json.dumps({args.only: fn(args, dev, steps=args.steps, cpu=not args.no_cpu)}), flush=True)
        return
    rank, world, local = dist_setup()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_tg(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
