"""Benchmark: batched AprilTag detection on one GB300 versus plain per-frame detect.

Workload: 4-camera batches of 1280x800 uint8 frames, both tag families per
frame, from 600 seeded synthetic frames (6 tag36h11 + 2 tag16h5
per frame, side 20-200 px, noise sigma 6, 3x3 blur on odd frames, two decoys
on every fourth frame, glyph clutter past the candidate cap on every eighth).
The 600 distinct frames (614 MB) are larger than L2, so no flush is needed.
One step is --batches-per-step (default 32) such batches issued round-robin
over the streams, so that even a 20-step run is long against the time it
takes to fill and drain the streams.

value     frames/s of the batched path with frames resident in HBM
          (bd_batch_submit_device), several batches in flight on S streams,
          timed with CUDA events; p50/p99 = per-batch latency, submit to
          results on the host.
e2e       the same through the host-input C ABI (bd_batch_submit_host) with
          frames in pinned host memory: H2D of the frames and D2H of the result
          records inside the timed region.
plain     the reference-style plain path: bd_detector_detect_host per frame
          and family (two detectors per frame, like two reference detectors).
roofline  the pipeline's algorithmic bytes (W*H per frame, the frame read
          once) / the timed wall, vs the measured HBM copy bandwidth; per
          kernel the same for the two stages that stream the frame (k_stats,
          k_binarize_runs), CUDA-event times for the latency-bound rest.
cpu_baseline  the CPU oracle (a restatement of the reference pipeline; the
          reference has no CPU detector) on the host cores, bounded sample.

--impl reference times the reference pipeline on the host CPU (the oracle
port, all host threads), same metric and workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

# Several batches run at once on separate streams; the default of 8 hardware
# work queues per context makes streams share queues and serialise.  Must be
# set before the CUDA context exists (the library reads nothing itself).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = Path(__file__).resolve().parent
sys.path[:0] = [str(REPO / "bd-cudatag_gb300"), str(REPO / "oracle")]

METRIC = "batched frames/s & p99 ms at 1280x800 vs plain per-frame detect, same GB300"
W, H = 1280, 800
POOL = 600
BATCH = 4
FAMILIES = 3  # both families
WORKLOAD = ("4-camera batches of 1280x800 uint8 frames, tag36h11+tag16h5 decoded per "
            "frame, 600 seeded frames (6 tag36h11 + 2 tag16h5, side 20-200 px, sigma 6, blur on "
            "odd frames, decoys on i%4==3, glyph clutter past the candidate cap on i%8==5)")


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def render_pool(count: int, offset: int = 0):
    import scenes

    frames, truth = scenes.render_many(scenes.MIXED_1280, [(W, H)] * count, threads=os.cpu_count() or 8,
                                       base=scenes.base_seed(scenes.MIXED_1280) + offset)
    return frames, truth


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        fd, name = tempfile.mkstemp(prefix="bd_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.fh.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            self.path.unlink(missing_ok=True)
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def aggregate_ranks(elapsed_ms: float, e2e_ms: float, steps: int, world: int, device="cuda",
                    batches_per_step: int = 1):
    """Whole-job throughput of `world` replicas: every rank processed
    steps * batches_per_step * BATCH frames, and the job lasts as long as the
    slowest rank (max over ranks of the device time).  Returns (elapsed_ms,
    e2e_ms, value, e2e_value) with the maxima."""
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([elapsed_ms, e2e_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms, e2e_ms = float(t[0]), float(t[1])
    frames_total = steps * batches_per_step * BATCH * world
    return elapsed_ms, e2e_ms, frames_total / (elapsed_ms * 1e-3), frames_total / (e2e_ms * 1e-3)


def pct(values, q):
    return float(np.percentile(np.asarray(values), q)) if len(values) else None


def run_batched(plans, streams, frame_sets, steps, warmup, device: bool, strides=None):
    """Round-robin batches over the plans in native code
    (bd_batch_pipeline); returns (elapsed ms by CUDA events, per-batch
    latencies in ms, submit to completion on the host)."""
    import torch

    import bdcudatag

    st = strides or [W] * BATCH
    if warmup:
        bdcudatag.pipeline(plans, frame_sets, st, warmup, device)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    main = torch.cuda.current_stream()
    start.record(main)
    for s in streams:
        s.wait_event(start)
    _, lat = bdcudatag.pipeline(plans, frame_sets, st, steps, device)
    for s in streams:
        main.wait_stream(s)
    stop.record(main)
    torch.cuda.synchronize()
    return start.elapsed_time(stop), list(lat)


def tune_throughput(plans, streams, frame_sets, steps=400, strides=None):
    """Autotuner for throughput: coordinate descent over the launch shapes,
    each candidate timed on the same multi-stream loop the benchmark reports
    (frames/s); keeps the fastest on every plan.  Launch shapes never change
    results."""
    grid = [("band_cap", [2048, 1024, 512]), ("quad_split", [32, 48, 64, 96, 0]),
            ("quad_warps", [2, 4, 8]), ("quad_ctas_per_sm", [2, 4, 8, 16]), ("stats_rows", [1, 2, 4]),
            ("fit_merged", [0, 1]), ("persistent", [0, 1]), ("persist_ctas", [0, 152, 76, 38])]
    best = dict(plans[0].launch())

    def score(cfg):
        for p in plans:
            p.set_launch(**cfg)
        ms, _ = run_batched(plans, streams, frame_sets, steps, 20, device=True, strides=strides)
        return steps / ms

    best_score = score(best)
    trials = [(dict(best), best_score)]
    for field, values in grid:
        for v in values:
            if v == best[field] or (field == "persist_ctas" and not best["persistent"]):
                continue
            cfg = dict(best, **{field: v})
            sc = score(cfg)
            trials.append((cfg, sc))
            if sc > best_score:
                best, best_score = cfg, sc
    for p in plans:
        p.set_launch(**best)
    return best, len(trials)


def launches_per_batch(launch: dict) -> int:
    if launch.get("persistent"):
        return 1
    return 8 if launch["quad_split"] > 0 and not launch.get("fit_merged") else 7


def measure_plain(frames, count):
    import bdcudatag

    dets = [bdcudatag.Detector(f, W, H) for f in (0, 1)]
    for k in range(5):
        for d in dets:
            d.detect(frames[k % len(frames)])
    lat = []
    t0 = time.perf_counter()
    for k in range(count):
        t = time.perf_counter()
        for d in dets:
            d.detect(frames[k % len(frames)])
        lat.append((time.perf_counter() - t) * 1e3)
    total = time.perf_counter() - t0
    gpu_ms = sum(d.stats().average_gpu_ms for d in dets)
    return {"value": count / total, "unit": "frames/s", "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "gpu_ms_per_frame": gpu_ms, "path": "bd_detector_detect_host, one tag36h11 and one "
            "tag16h5 detector per frame, pageable host frames, CUDA graph",
            "note": "this library's own single-frame path (the reference's C ABI call), not the "
                    "reference's GPU build: its sources cannot be built on the GPU host"}


def read_traffic():
    """Per-kernel DRAM bytes per launch (ncu dram__bytes_read.sum +
    dram__bytes_write.sum of the 4x1280x800 batch) from the committed
    summary, or {}."""
    traffic = {}
    tf = REPO / "profiles" / "dram_traffic.txt"
    if tf.exists():
        for line in tf.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#"):
                traffic[parts[0]] = int(parts[1])
    return traffic


def measure_roofline(plan, frame_sets, peaks, frames_per_s):
    """The pipeline's roofline figure, per-stage CUDA-event times and the
    GPU time of one batch as a graph replay.

    Pipeline: the algorithmic bytes are W*H per frame (the frame read once),
    so achieved = frames/s * W*H over the timed wall of the batched loop.
    Per stage: one un-graphed batch with events around every kernel
    (bd_batch_profile_device), mean over 14 batches after 2 warm-ups.  Only
    k_stats and k_binarize_runs stream the frame, so only they get an HBM
    fraction (their algorithmic bytes per launch / their mean duration); the
    other stages are gathers and union-find walks in L2, reported as time."""
    sums = None
    n = 0
    for k in range(min(16, len(frame_sets))):
        st = plan.profile_device(frame_sets[k], [W] * BATCH)
        if k < 2:
            continue  # warm-up
        sums = {s: sums.get(s, 0.0) + v for s, v in st.items()} if sums else dict(st)
        n += 1
    mean = {s: v / n for s, v in sums.items()}
    total = sum(mean.values())
    # One batch as the graph runs it (the two fit kernels side by side):
    # median GPU time of 50 replays after 10, CUDA events around the launch.
    single = []
    for k in range(60):
        plan.detect(frame_sets[k % len(frame_sets)], [W] * BATCH, device=True)
        if k >= 10:
            single.append(plan.last_gpu_ms())
    T = ((W + 7) // 8) * ((H + 7) // 8)
    per_frame = {
        "stats": W * H + 2 * T,                              # frame read once, tile min/max written
        "binarize_runs": W * H + ((W + 31) // 32) * 4 * H,   # frame rows read, bit rows written
    }
    traffic = read_traffic()
    peak = peaks.get("hbm_gbs")
    kernels = {}
    for stage, bpf in per_frame.items():
        if stage not in mean or mean[stage] <= 0:
            continue
        got = bpf * BATCH / (mean[stage] * 1e-3) / 1e9
        kernels[f"k_{stage}"] = {
            "bound": "hbm", "algorithmic_bytes": bpf * BATCH, "mean_launch_ms": round(mean[stage], 5),
            "achieved": round(got, 2), "frac": round(got / peak, 5) if peak else None,
            "traffic": traffic.get(f"k_{stage}")}
    achieved = frames_per_s * W * H / 1e9
    pipe_traffic = sum(traffic.values()) if traffic else None
    return {
        "bound": "hbm", "kernel": "pipeline (every stage of a 4x1280x800 batch, batches in flight)",
        "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 5) if peak else None,
        "frac_of": "measured copy bandwidth (MEASURED_PEAKS.json)",
        "bytes_per_batch": W * H * BATCH,
        "traffic": pipe_traffic,
        "traffic_source": "sum over the batch's kernels of ncu dram__bytes_read+write per launch "
                          "(profiles/dram_traffic.txt)",
        "kernels": kernels,
        "stage_ms": {k: round(v, 5) for k, v in mean.items()},
        "stage_ms_sum": round(total, 5),
        "stage_ms_note": "un-graphed, one kernel after another (the fit kernels too)",
        "single_batch_gpu_ms": round(float(np.median(single)), 5),
        "stage_share": {k: round(v / total, 4) for k, v in mean.items()},
        "latency_bound": "stages other than stats and binarize_runs: L2 gathers and union-find "
                         "walks, reported as time",
    }


SERVE_SIZES = [(640, 480), (1280, 720), (1280, 800), (1600, 1304), (1920, 1080), (2560, 1440),
               (3840, 2160)]


def serving_trace(seconds: float, seed: int = 6324 + 5000, scale: float = 1.0):
    """6 cameras: size drawn from 640x480..3840x2160, rate U(60, 120) fps
    (times `scale`), Poisson arrivals; returns (cameras, arrivals [(t,
    camera, k)]).  The cameras do not depend on `scale`."""
    rng = np.random.default_rng(seed)
    cams, arrivals = [], []
    for c in range(6):
        w, h = SERVE_SIZES[int(rng.integers(0, len(SERVE_SIZES)))]
        fps = float(rng.uniform(60.0, 120.0))
        cams.append((w, h, FAMILIES, fps))
    arr_rng = np.random.default_rng(seed + 1)
    for c, (_, _, _, fps) in enumerate(cams):
        rate = fps * scale
        t, k = float(arr_rng.exponential(1.0 / rate)), 0
        while t < seconds:
            arrivals.append((t, c, k))
            t += float(arr_rng.exponential(1.0 / rate))
            k += 1
    arrivals.sort()
    return cams, arrivals


MIXED_SIZES = [(640, 480), (1280, 800), (1600, 1304), (1920, 1080)] * 4


def measure_mixed_batches(steps: int, streams: int = 4, pool_batches: int = 8):
    """16-frame batches of uneven sizes (4 each of 640x480, 1280x800,
    1600x1304, 1920x1080), both families, autotuned launch shapes; frames/s
    with frames resident in HBM, and a bit-exact check of one batch against
    single-frame detection."""
    import torch

    import bdcudatag
    import scenes

    sizes = MIXED_SIZES * pool_batches
    frames, _ = scenes.render_many(scenes.MULTI_SIZE, sizes, threads=os.cpu_count() or 8)
    dev = [torch.from_numpy(f).cuda() for f in frames]
    nb = len(MIXED_SIZES)
    sets = [dev[k * nb:(k + 1) * nb] for k in range(pool_batches)]
    strides = [w for w, _ in MIXED_SIZES]
    cams = [(w, h, FAMILIES) for w, h in MIXED_SIZES]
    plans = [bdcudatag.Batch(cams) for _ in range(streams)]
    default_launch = plans[0].launch()
    latency_best, tuned_ms = plans[0].autotune(sets[0], strides, iterations=10)
    ts = [torch.cuda.Stream() for _ in range(streams)]
    for p, st in zip(plans, ts):
        p.set_stream(st)
    best, _ = tune_throughput(plans, ts, sets, steps=100, strides=strides)
    elapsed, lat = run_batched(plans, ts, sets, steps, 5, device=True, strides=strides)
    for p in plans:
        p.set_stream(None)
    found, out = plans[0].detect(sets[1], strides, device=True)
    exact = True
    for i in range(nb):
        w, h = MIXED_SIZES[i]
        for fam in (0, 1):
            n, d = bdcudatag.Detector(fam, w, h).detect(frames[nb + i])
            exact = exact and found[i, fam] == n and out[i, fam, :n].tobytes() == d.tobytes()
    batch_bytes = sum(w * h for w, h in MIXED_SIZES)
    return {"frames_per_s": round(steps * nb / (elapsed * 1e-3), 2), "batch_frames": nb,
            "batch_bytes": batch_bytes, "streams": streams, "steps": steps,
            "p50_ms": round(pct(lat, 50), 4), "p99_ms": round(pct(lat, 99), 4),
            "tuned_launch": best, "latency_tuned_launch": latency_best,
            "default_launch": default_launch,
            "tuned_batch_gpu_ms": round(tuned_ms, 4), "bit_exact_vs_single_frame": bool(exact)}


def serving_pools(cams, pool_per_cam: int = 12):
    """Seeded frames of every camera: (pageable list, pinned tensor)."""
    import torch

    import scenes

    pools = []
    for c, (w, h, _, _) in enumerate(cams):
        imgs, _ = scenes.render_many(scenes.SERVING, [(w, h)] * pool_per_cam, threads=os.cpu_count() or 8,
                                     base=scenes.base_seed(scenes.SERVING) + 1000 * c)
        pinned = torch.empty((pool_per_cam, h, w), dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = np.stack(imgs)
        pools.append((imgs, pinned))
    return pools


def run_server(cams, arrivals, pools, seconds: float, peaks=None, max_batches: int = 4,
               queue_depth: int = 16):
    """Feeds the arrivals to a bd_server in real time (frames from pinned
    pools), collects every result on a second thread; latency = the server's
    own arrival-to-completion time per frame."""
    import bdcudatag

    pool_per_cam = pools[0][1].shape[0]
    server = bdcudatag.Server([(w, h, f) for w, h, f, _ in cams], device_budget=24 << 30,
                              max_batches=max_batches, queue_depth=queue_depth)
    for c in range(len(cams)):  # warm-up: one frame per camera
        server.wait(server.submit(c, pools[c][1][0]))
    tickets: list = []
    lat: list[float] = []
    dropped = [0]
    accepted: list[int] = []  # camera of every admitted frame
    done = threading.Event()

    def collector():
        i = 0
        while True:
            while i >= len(tickets):
                if done.is_set() and i >= len(tickets):
                    return
                time.sleep(0.0002)
            rc, found, out, ms = server.wait(tickets[i])
            lat.append(ms)
            i += 1

    th = threading.Thread(target=collector)
    th.start()
    t0 = time.perf_counter()
    for t, c, k in arrivals:
        # Sleep (which lets the collector thread run) until just before the
        # arrival, then spin for the last fraction of a millisecond.
        while True:
            ahead = t - (time.perf_counter() - t0)
            if ahead <= 0:
                break
            if ahead > 5e-4:
                time.sleep(ahead - 3e-4)
        tk = server.submit(c, pools[c][1][k % pool_per_cam])
        if tk < 0:
            dropped[0] += 1
        else:
            tickets.append(tk)
            accepted.append(c)
    done.set()
    th.join()
    wall = time.perf_counter() - t0
    served_bytes = sum(cams[c][0] * cams[c][1] for c in accepted)
    st = server.stats()
    server.close()
    return {"frames_per_s": round(len(lat) / wall, 2), "p50_ms": round(pct(lat, 50), 4),
            "p99_ms": round(pct(lat, 99), 4), "completed": len(lat), "dropped": dropped[0],
            "offered_fps": round(len(arrivals) / seconds, 2), "seconds": seconds,
            "batches": int(st.batches), "mean_batch_frames": round(st.mean_batch_frames, 3),
            "plans": int(st.plans), "peak_inflight": int(st.peak_inflight),
            "device_bytes": int(st.device_bytes),
            # frame bytes served per second against the measured HBM copy peak
            "frame_gbs": round(served_bytes / wall / 1e9, 4),
            "hbm_frac": (round(served_bytes / wall / 1e9 / peaks["hbm_gbs"], 7)
                         if peaks and peaks.get("hbm_gbs") else None)}


def measure_serving(seconds: float, pool_per_cam: int = 12, peaks=None):
    """Six camera streams (Poisson arrivals at 60-120 fps each, sizes from
    640x480 to 3840x2160): continuous batching through bd_server versus a FIFO plain
    per-frame detector fed by the same arrivals."""
    import bdcudatag

    cams, arrivals = serving_trace(seconds)
    pools = serving_pools(cams, pool_per_cam)
    serve = run_server(cams, arrivals, pools, seconds, peaks)
    # Plain per-frame detect on the same arrivals: measured service time per
    # (camera, frame) -- both families -- fed through a FIFO queue.
    dets = [[bdcudatag.Detector(f, w, h) for f in (0, 1)] for w, h, _, _ in cams]
    service = {}
    for c in range(len(cams)):
        for k in range(pool_per_cam):
            img = pools[c][0][k]
            for d in dets[c]:
                d.detect(img)
            ts = []
            for _ in range(3):
                t = time.perf_counter()
                for d in dets[c]:
                    d.detect(img)
                ts.append(time.perf_counter() - t)
            service[(c, k)] = float(np.median(ts))
    free_at, plain_lat = 0.0, []
    for t, c, k in arrivals:
        start = max(t, free_at)
        free_at = start + service[(c, k % pool_per_cam)]
        plain_lat.append((free_at - t) * 1e3)
    mean_service = float(np.mean([service[(c, k % pool_per_cam)] for _, c, k in arrivals]))
    plain = {"p50_ms": round(pct(plain_lat, 50), 4), "p99_ms": round(pct(plain_lat, 99), 4),
             "capacity_fps": round(1.0 / mean_service, 2),
             "utilisation": round(len(arrivals) / seconds * mean_service, 3),
             "method": "bd_detector_detect_host (one detector per camera and family), measured "
                       "service time per frame, FIFO queue over the same arrival times"}
    return {"cameras": [{"width": w, "height": h, "fps": round(f, 1)} for w, h, _, f in cams],
            "server": serve, "plain": plain, "pressure": measure_serving_pressure(cams, pools, peaks)}


def measure_serving_pressure(cams, pools, peaks=None, scales=(4, 16, 64, 128, 256), seconds=4.0):
    """The same six cameras at arrival rates scaled up until the p99 latency
    passes 2 ms: how continuous batching behaves under load (frames per
    launch, refusals by the per-camera queue, p50/p99, frames/s)."""
    rows = []
    for scale in scales:
        _, arrivals = serving_trace(seconds, scale=scale)
        row = run_server(cams, arrivals, pools, seconds, peaks)
        row["scale"] = scale
        rows.append(row)
        if row["p99_ms"] is not None and row["p99_ms"] > 2.0:
            break
    return rows


def measure_refine(n_quads: int = 256, iterations: int = 5):
    """Corner refinement: photometric Gauss-Newton on detected quads of 1280x800
    frames, corners perturbed by U(-1.5, 1.5) px; corner error against ground
    truth before and after, and the kernel times (CUDA events)."""
    import itertools

    import torch

    import bdcudatag
    import scenes

    def matches(c, t):
        c = np.asarray(c, np.float64).reshape(4, 2)
        t = np.asarray(t, np.float64).reshape(4, 2)
        side = np.mean([np.hypot(*(t[(j + 1) % 4] - t[j])) for j in range(4)])
        return np.hypot(*(c.mean(0) - t.mean(0))) <= 0.75 * side

    def err(c, t):
        c = np.asarray(c, np.float64).reshape(4, 2)
        t = np.asarray(t, np.float64).reshape(4, 2)
        return min(np.mean([np.hypot(*(c[j] - t[p[j]])) for j in range(4)])
                   for p in itertools.permutations(range(4)))

    groups = {0: {"c": [], "t": [], "tm": [], "ix": []}, 1: {"c": [], "t": [], "tm": [], "ix": []}}
    frames = []
    dets = [bdcudatag.Detector(f, W, H) for f in (0, 1)]
    fi = 0
    while sum(len(g["c"]) for g in groups.values()) < n_quads and fi < 200:
        img, tags = scenes.render_scene(scenes.REFINE_1280, fi, W, H)
        for fam in (0, 1):
            n, d = dets[fam].detect(img)
            for k in range(n):
                for t in tags:
                    if t.family == fam and t.id == d["id"][k] and matches(d["corners"][k], t.corners):
                        g = groups[fam]
                        g["c"].append(d["corners"][k].astype(np.float32))
                        g["t"].append(t.corners.reshape(8))
                        g["tm"].append(bdcudatag.tag_template(fam, int(t.id)))
                        g["ix"].append(len(frames))
        frames.append(img)
        fi += 1
    rng = np.random.default_rng(6324 + 4000)
    images = torch.from_numpy(np.stack(frames)).cuda()
    before, after, gn_ms, fb_ms, count = [], [], 0.0, 0.0, 0
    for fam, g in groups.items():
        if not g["c"]:
            continue
        c0 = np.stack(g["c"])
        start = c0 + rng.uniform(-1.5, 1.5, c0.shape).astype(np.float32)
        co = torch.from_numpy(start.copy()).cuda()
        te = torch.from_numpy(np.stack(g["tm"])).cuda()
        ix = torch.from_numpy(np.array(g["ix"], np.int32)).cuda()
        args = bdcudatag.refine_args(images, co, te, ix, None, samples_per_cell=8)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        rc = bdcudatag.lib().bd_refine_gauss_newton(args, co.data_ptr(), iterations, None,
                                                     torch.cuda.current_stream().cuda_stream)
        e1.record()
        torch.cuda.synchronize()
        assert rc == 0, bdcudatag.last_error()
        gn_ms += e0.elapsed_time(e1)
        # forward + adjoint once, at the refined corners
        n = co.shape[0]
        cells = te.shape[-1]
        res = torch.empty((n, cells * cells * 64), device="cuda")
        gc = torch.empty_like(co)
        gi = torch.zeros(images.shape, device="cuda", dtype=torch.float32)
        args = bdcudatag.refine_args(images, co, te, ix, None, samples_per_cell=8)
        s = torch.cuda.current_stream().cuda_stream
        e0.record()
        bdcudatag.lib().bd_refine_forward(args, res.data_ptr(), None, s)
        bdcudatag.lib().bd_refine_backward(args, res.data_ptr(), gc.data_ptr(), gi.data_ptr(), s)
        e1.record()
        torch.cuda.synchronize()
        fb_ms += e0.elapsed_time(e1)
        refined = co.cpu().numpy()
        before += [err(a, t) for a, t in zip(start, g["t"])]
        after += [err(a, t) for a, t in zip(refined, g["t"])]
        count += n
    samples = sum(len(g["c"]) * (10 if f == 0 else 8) ** 2 * 64 for f, g in groups.items())
    return {"quads": count, "frames": len(frames), "iterations": iterations,
            "corner_err_before_px": {"mean": round(float(np.mean(before)), 4),
                                     "median": round(float(np.median(before)), 4)},
            "corner_err_after_px": {"mean": round(float(np.mean(after)), 4),
                                    "median": round(float(np.median(after)), 4),
                                    "p95": round(float(np.percentile(after, 95)), 4)},
            "gauss_newton_ms": round(gn_ms, 4), "forward_backward_ms": round(fb_ms, 4),
            "samples_per_pass": samples}


def measure_cpu_baseline(frames, seconds_budget=12.0):
    import oracle

    cores = os.cpu_count() or 1
    c0 = time.process_time()
    oracle.detect_many(frames[:2], [FAMILIES] * 2, threads=1)  # warm
    n1 = 8
    t = time.perf_counter()
    oracle.detect_many(frames[:n1], [FAMILIES] * n1, threads=1)
    single = n1 / (time.perf_counter() - t)
    # About seconds_budget of CPU time across all threads, cycling the pool.
    n = max(cores * 2, int(seconds_budget * single))
    sample = [frames[k % len(frames)] for k in range(n)]
    t = time.perf_counter()
    oracle.detect_many(sample, [FAMILIES] * n, threads=cores)
    multi = n / (time.perf_counter() - t)
    cpu_s = time.process_time() - c0
    return {"value": round(multi, 2), "unit": "frames/s", "cores": cores, "kind": "port",
            "single_thread": round(single, 2),
            "sample": f"{n} 1280x800 frames of the workload (cycling {len(frames)} seeded frames), both "
                      f"families, oracle on {cores} threads, plus {n1} frames on 1 thread; "
                      f"{cpu_s:.1f} s of CPU time"}


def bench_reference(args, rank):
    """The reference pipeline on the host CPU (oracle port, all threads)."""
    import oracle

    if rank != 0:
        return
    frames, _ = render_pool(64)
    cores = os.cpu_count() or 1
    # Throughput: the K steps' 4-camera batches as one stream of (frame,
    # family) tasks over every host thread (chunks of 1024 frames), so no
    # thread idles at the end of each small batch.  Latency: p50/p99 of
    # single 4-camera batches (8 tasks in parallel) on a bounded sample.
    for k in range(args.warmup):
        oracle.detect_many([frames[(k * BATCH + i) % 64] for i in range(BATCH)], [FAMILIES] * BATCH,
                           threads=cores)
    G = args.batches_per_step
    total_frames = args.steps * G * BATCH
    t0 = time.perf_counter()
    done = 0
    while done < total_frames:
        n = min(1024, total_frames - done)
        oracle.detect_many([frames[(done + i) % 64] for i in range(n)], [FAMILIES] * n, threads=cores)
        done += n
    total = time.perf_counter() - t0
    value = total_frames / total
    times = []
    for k in range(min(args.steps, 64)):
        sl = [frames[(k * BATCH + i) % 64] for i in range(BATCH)]
        t = time.perf_counter()
        oracle.detect_many(sl, [FAMILIES] * BATCH, threads=min(cores, 2 * BATCH))
        times.append((time.perf_counter() - t) * 1e3)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total * 1e3 / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "p50_ms": pct(times, 50), "p99_ms": pct(times, 99),
        "config": {"workload": WORKLOAD, "batch_frames": BATCH, "batches_per_step": G,
                   "step": f"{G} batches of {BATCH} frames", "frames_pool": 64},
        "cpu_baseline": {"value": round(value, 2), "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps * G} batches of {BATCH} 1280x800 workload frames (both "
                                   f"families) cycling 64 seeded frames, as (frame, family) tasks on "
                                   f"{cores} threads; p50/p99 over {len(times)} single batches"},
        "e2e": {"value": round(value, 2), "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU detector; this is the CPU restatement of its pipeline "
                "(oracle/), run on all host threads",
    }
    print(json.dumps(line), flush=True)


def bench_ours(args, rank, world, local_rank):
    import torch

    import bdcudatag

    torch.cuda.set_device(local_rank)
    peaks = {}
    pk = REPO / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    pool = 64 if args.quick else POOL
    frames, _ = render_pool(pool, offset=rank * POOL)
    pinned = torch.empty((pool, H, W), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = np.stack(frames)
    device = pinned.to(f"cuda:{local_rank}")
    torch.cuda.synchronize()
    sets_dev = [[device[(k * BATCH + i) % pool] for i in range(BATCH)] for k in range(pool // BATCH)]
    sets_host = [[pinned[(k * BATCH + i) % pool] for i in range(BATCH)] for k in range(pool // BATCH)]

    cams = [(W, H, FAMILIES)] * BATCH
    plans = [bdcudatag.Batch(cams) for _ in range(args.streams)]
    streams = [torch.cuda.Stream() for _ in range(args.streams)]
    for p, s in zip(plans, streams):
        p.set_stream(s)

    barrier(world)
    tuned, tune_trials = None, None
    if args.launch:
        fixed = {k: int(v) for k, v in (kv.split("=") for kv in args.launch.split(","))}
        for p in plans:
            p.set_launch(**fixed)
        tuned = plans[0].launch()
    elif args.tune or not args.quick:
        # Launch shapes scored on frames/s with all streams busy (untimed).
        tuned, tune_trials = tune_throughput(plans, streams, sets_dev)
    G = args.batches_per_step
    if args.quick:
        if tuned:
            print(json.dumps({"tuned": tuned}), flush=True)
        elapsed_ms, lat = run_batched(plans, streams, sets_dev, args.steps * G, args.warmup * G,
                                      device=True)
        # One batch alone: median GPU time (graph replay, CUDA events) of 50.
        plans[0].set_stream(None)
        single = []
        for k in range(60):
            plans[0].detect(sets_dev[k % len(sets_dev)], [W] * BATCH, device=True)
            if k >= 10:
                single.append(plans[0].last_gpu_ms())
        if rank == 0:
            print(json.dumps({"quick": True, "value": args.steps * G * BATCH / (elapsed_ms * 1e-3),
                              "unit": "frames/s", "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                              "streams": args.streams, "launch": plans[0].launch(),
                              "single_batch_gpu_ms": float(np.median(single))}), flush=True)
        return
    barrier(world)
    with ClockSampler(local_rank) as clocks:
        elapsed_ms, lat = run_batched(plans, streams, sets_dev, args.steps * G, args.warmup * G,
                                      device=True)
    barrier(world)
    e2e_ms, e2e_lat = run_batched(plans, streams, sets_host, args.steps * G, args.warmup * G,
                                  device=False)
    barrier(world)
    elapsed_ms, e2e_ms, value, e2e_value = aggregate_ranks(elapsed_ms, e2e_ms, args.steps, world,
                                                           batches_per_step=G)
    if rank != 0:
        return

    # Correctness spot check against the CPU oracle on one batch.
    import oracle

    found, out = plans[0].detect(sets_host[0], [W] * BATCH)
    for i in range(BATCH):
        for fam in (0, 1):
            n, want = oracle.Frame(frames[i], fam).detections()
            assert found[i, fam] == n and out[i, fam, :n].tobytes() == want.tobytes(), "parity"

    for p in plans:
        p.set_stream(None)
    roof = measure_roofline(plans[0], sets_dev, peaks, value / world)
    plain = measure_plain(frames, args.plain_frames)
    cpu = measure_cpu_baseline(frames)
    serving = measure_serving(args.serving_seconds, peaks=peaks) if args.serving_seconds > 0 else None
    refine = measure_refine()
    mixed = measure_mixed_batches(max(200, args.steps * G // 5), streams=min(args.streams, 8))
    result_bytes = BATCH * ((32 + 2 * plans[0].max_detections * 84 + 255) // 256 * 256)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(elapsed_ms / args.steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "p50_ms": round(pct(lat, 50), 4), "p99_ms": round(pct(lat, 99), 4),
        "config": {"workload": WORKLOAD, "batch_frames": BATCH, "batches_per_step": G,
                   "step": f"{G} batches of {BATCH} frames issued round-robin over {args.streams} "
                           f"streams", "streams": args.streams,
                   "launch": tuned, "tuning_trials": tune_trials,
                   "frames_pool": POOL, "families_per_frame": 2,
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                   "l2": "inputs larger than L2 (600 distinct 1 MB frames cycled)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e_value, 2), "unit": "frames/s",
                "p50_ms": round(pct(e2e_lat, 50), 4), "p99_ms": round(pct(e2e_lat, 99), 4),
                "h2d_bytes_per_step": G * BATCH * W * H, "d2h_bytes_per_step": G * result_bytes,
                "path": "bd_batch_submit_host/bd_batch_wait, frames in pinned host memory"},
        "plain": plain,
        "speedup_vs_plain": round(value / plain["value"], 2),
        "parity": {"vs_oracle": "bit-exact at every stage (bitmap, runs, labels, area/bbox, "
                                "candidates, quads, decodes, records); tests/",
                   "vs_reference_build": "not measured: the reference's GPU library cannot run "
                                         "on the GPU host; built the reference's way (nvcc "
                                         "contraction, CUDA libm) the same kernels move "
                                         "decoded corners by a median 3.4e-3 px and flip 2 of "
                                         "14,005 candidate decodes "
                                         "(tests/test_gpu_reference_arithmetic.py)"},
        "e2e_speedup_vs_plain": round(e2e_value / plain["value"], 2),
        "roofline": roof,
        "cpu_baseline": cpu,
        "serving": serving,
        "refine": refine,
        "mixed_size_batches": mixed,
        "clocks": clocks.summary(),
        # per batch: k_persistent alone, or k_stats, k_binarize_runs, k_merge,
        # k_region_stats, k_cand_count, k_fit_decode (+ k_fit_decode_big when
        # the split is on), k_finalize
        "gpu_launches": launches_per_batch(plans[0].launch()) * args.steps * G,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--batches-per-step", type=int, default=32,
                    help="4-camera batches per step, issued round-robin over the streams")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # 12 batches in flight: the GPU's saturated rate (12: 128k frames/s, p99
    # 0.45 ms; 8: 117k, 0.32 ms; 16-48 streams: 125-127k at higher p99).
    ap.add_argument("--streams", type=int, default=12)
    ap.add_argument("--plain-frames", type=int, default=300)
    ap.add_argument("--serving-seconds", type=float, default=60.0,
                    help="length of the six-camera serving run (0: skip)")
    ap.add_argument("--tune", action="store_true", help="tune launch shapes in --quick runs")
    ap.add_argument("--launch", default="",
                    help="fixed launch shapes instead of tuning, e.g. band_cap=1024,quad_split=48")
    ap.add_argument("--quick", action="store_true",
                    help="profiling run: 64-frame pool, batched device-input loop only")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local_rank = dist_info()
    if world > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "reference":
            if rank != 0:
                return
        else:
            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl")
    if args.impl == "reference":
        bench_reference(args, rank)
    else:
        bench_ours(args, rank, world, local_rank)
    if world > 1 and args.impl != "reference":
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
