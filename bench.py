"""Benchmark of the streaming-BASS (BIST) hot path on one node.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): the 30-frame 480x854 synthetic streaming video of the
streaming-propagation configuration (Voronoi frames with 400 seeds, per-region
affine motion, noise sigma 0.03, ground-truth forward flow), run through
frame 0 is plain BASS, frames 1..29 are flow propagation + hole fill + 20
boundary iterations with split/merge every 10, superpixel size 20.  Each GPU runs
--streams such videos (seeds rank*S..), advanced together: frame t of the streams
of one host lane is one batch of the batched engine (st_spix_gb300.batch), with
labels, parameters and previous frame resident on the device between batches.  A
step is the whole video of every stream.  Ranks are replicas (no collective on
the data path).  The plain per-frame path (bist_forward, one stream) is timed
beside it.  Prints ONE JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="bist_stream_480x854_T30", H=480, W=854, T=30, nseeds=400, sigma=0.03,
                sp_size=20, niters=20, prop_niters=20, sm_period=10, potts=0.5,
                sigma2_app=0.009 ** 2, alpha=math.log(0.5), split_alpha=0.0)
# Algorithmic bytes of one BASS pass (the scope's measurement rules): 4 sweeps x (label
# read 4 + image read 12 + label write 4) + the statistics of the new labels 16 = 96 B/px.
# The 4 sweep launches of an update do the whole pass: they keep the statistics current
# by moving those of every relabelled pixel (incremental statistics), so no separate
# statistics pass runs between two updates: 24 B/px per sweep launch on average.
SWEEP_BYTES_PER_PX = 24
# DRAM bytes (read + write) per sweep launch from one ncu capture of the same workload
# (a batch of 8 frames, mean of a full and an active-set sweep); a constant of that
# capture, re-taken whenever the sweep kernel changes, not a live measurement.
SWEEP_TRAFFIC_NCU = dict(bytes_per_launch=35589120,
                         source="ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                "profiles/kb_sweep_bist_stream_480x854_T30.md")
METRIC = "streamed frames/sec"
SERVE_LANES = 3          # host lanes of the serving legs in the default run


def gen_video(seed: int, T: int = None):
    from st_spix_gb300 import synth
    w = WORKLOAD
    vid, flows, _ = synth.voronoi_video(w["H"], w["W"], T or w["T"], w["nseeds"], w["sigma"],
                                        seed=seed)
    return vid, flows


# ---------------------------------------------------------------------------
# CPU leg: the oracle (CPU restatement of the reference path), one stream per
# worker process.  Each step runs the next `window` frames of every worker's stream
# (frame 0 plain BASS, frames 1..T-1 propagated; a stream restarts after its last
# frame), so consecutive steps walk the streaming workload's frame mix.
def workload_config() -> dict:
    """The `config` of both arms' bench lines: the streaming workload itself (the same
    dict on the GPU arm and the reference arm; run details go under "run")."""
    w = WORKLOAD
    return {"workload": w["name"], "H": w["H"], "W": w["W"], "T": w["T"],
            "nseeds": w["nseeds"], "sigma": w["sigma"], "sp_size": w["sp_size"],
            "niters": w["niters"], "prop_niters": w["prop_niters"], "sm_period": w["sm_period"],
            "frame_mix": "per stream: frame 0 plain BASS, frames 1-%d propagated" % (w["T"] - 1),
            "l2": "inputs larger than L2: a %dx%d frame and its flow take %.1f MB and a step "
                  "reads every frame of every stream it runs" %
                  (w["H"], w["W"], w["H"] * w["W"] * 20 / 1e6)}


def _cpu_config():
    from oracle import oracle as O
    w = WORKLOAD
    return O.default_config(niters=w["niters"], sp_size=w["sp_size"], prop_niters=w["prop_niters"],
                            sm_period=w["sm_period"], potts=w["potts"],
                            sigma2_app=w["sigma2_app"], alpha_hastings=w["alpha"])


def _cpu_stream_loop(seed, conn):
    """Worker process: owns one stream; each request runs its next `window` frames."""
    from oracle import oracle as O
    O.lib()
    vid, flows = gen_video(seed)
    cfg = _cpu_config()
    w = WORKLOAD
    t, prev = 0, None
    conn.send(("ready", 0, 0.0))
    while True:
        msg = conn.recv()
        if msg is None:
            break
        window = int(msg)
        t0 = time.perf_counter()
        for _ in range(window):
            if t == 0:
                rc, lab, params, n = O.run_bass(vid[0], cfg)
            else:
                lab_prev, params_prev, n_prev = prev
                rc, filled, shifted, pp = O.shift_and_fill(lab_prev, params_prev, n_prev,
                                                           flows[t - 1])
                if rc == 0:
                    rc, lab, params, n = O.run_prop(vid[t], cfg, w["prop_niters"], filled,
                                                    shifted, pp, n_prev)
            if rc != 0:
                conn.send(("error", rc, 0.0))
                return
            prev = (lab, params, n)
            t = (t + 1) % w["T"]
        conn.send(("ok", window, time.perf_counter() - t0))


class CpuBaseline:
    """One spawned process per host core, each owning one stream of the workload and
    running the oracle on the next `window` frames of it per step."""

    def __init__(self, window: int = 3):
        import multiprocessing as mp
        from oracle import oracle as O
        O.build()
        self.cores = os.cpu_count() or 1
        self.window = window
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for s in range(self.cores):
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_cpu_stream_loop, args=(s, b), daemon=True)
            pr.start()
            self.conns.append(a)
            self.procs.append(pr)
        for c in self.conns:
            c.recv()

    def step(self):
        t = time.perf_counter()
        for c in self.conns:
            c.send(self.window)
        frames = 0
        for c in self.conns:
            kind, n, _ = c.recv()
            if kind != "ok":
                raise RuntimeError("CPU baseline worker failed with status %d" % n)
            frames += n
        return frames, time.perf_counter() - t

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except (BrokenPipeError, OSError):
                pass
        for pr in self.procs:
            pr.join(timeout=30)

    def describe(self):
        w = WORKLOAD
        return (f"{self.cores} concurrent streams of the {w['H']}x{w['W']}x{w['T']} workload, "
                f"one process per core, each step the next {self.window} frames of every "
                f"stream (frame 0 plain BASS, frames 1-{w['T'] - 1} propagated, a stream "
                f"restarts after frame {w['T'] - 1}), oracle (CPU restatement)")


# ---------------------------------------------------------------------------
def sample_clocks(gpu_index: int, stop: threading.Event, out: list):
    q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={q}",
                              "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
        return
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append(line.strip())
    finally:
        p.terminate()
        try:
            p.wait(timeout=2)
        except Exception:
            p.kill()


def summarize_clocks(lines: list) -> dict:
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 8:
            continue
        try:
            sm.append(float(f[0]))
            mx = float(f[1])
        except ValueError:
            continue
        for n, v in zip(names, f[4:8]):
            if v.lower().startswith("active"):
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
            "reasons": sorted(reasons), "samples": len(sm)}


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"




def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over the ranks of the process group (x itself with one rank):
    the whole job's time is its slowest replica's."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seeds(rank: int, streams: int) -> list:
    """Video seeds of a replica's streams: disjoint across ranks (replicas only; no
    data is exchanged between GPUs)."""
    return [rank * streams + i for i in range(streams)]


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args, world, rank):
    """--impl reference: the reference path's CPU implementation (the oracle port; the
    reference itself has no CPU path) on all host cores, same metric and config."""
    if rank != 0:
        return
    base = CpuBaseline(window=3)
    try:
        for _ in range(args.warmup):
            base.step()
        frames, wall = 0, 0.0
        for _ in range(args.steps):
            f, w = base.step()
            frames += f
            wall += w
        v = frames / wall
        w = WORKLOAD
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * wall / max(args.steps, 1), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64+int64",
                "data": "synthetic",
                "config": workload_config(),
                "run": {"sample": base.describe(), "cores": base.cores},
                "cpu_baseline": {"value": v, "unit": "frames/s", "cores": base.cores,
                                 "kind": "port", "sample": base.describe()},
                "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
    finally:
        base.close()


SERVE = dict(name="serve_mixed_360p720p1080p_poisson30", mix=(0.4, 0.4, 0.2), T=30, fps=30.0,
             budget_gb=120, pool=3, streams=256)


def serve_leg(args, dev, rank, streams, frames, fps, lanes=None, max_batch=None,
              group_sizes=True, max_pixels=0):
    """The serving form on a mixed-resolution stream set (360p / 720p / 1080p at 0.4 /
    0.4 / 0.2, each stream a video generated as the streaming workload with its own
    Poisson `fps` arrivals), admitted under a 120 GB budget and served by continuous
    batching; the plain per-frame path (bist_forward, one frame at a time) is timed on
    one stream per resolution of the same set and weighted by the set's mix.  Returns
    the serving statistics, the plain figure and the clocks seen while serving."""
    import torch
    from st_spix_gb300 import bist_cuda, serve, synth

    w, sv = WORKLOAD, dict(SERVE, fps=fps, T=frames)
    res = synth.stream_resolution_mix(streams, seed=rank)
    cfg = dict(niters=w["niters"], sp_size=w["sp_size"], potts=w["potts"],
               sigma2_app=w["sigma2_app"], alpha=w["alpha"], split_alpha=w["split_alpha"],
               sm_period=w["sm_period"], prop_niters=w["prop_niters"])
    # a small pool of device-resident videos per resolution, shared by the streams
    pool = {}
    for hw in sorted(set(res)):
        pool[hw] = [synth.voronoi_video_device(hw[0], hw[1], sv["T"], w["nseeds"], w["sigma"],
                                               seed=1000 * hw[0] + j, device=dev)
                    for j in range(sv["pool"])]
    # plain per-frame path on a sample (one stream per resolution, all frames)
    plain_frames, plain_s = 0, 0.0
    for hw in sorted(pool):
        v, f = pool[hw][0]
        bist_cuda.bist_forward(v[:2].contiguous(), f[:1].contiguous(), w["niters"],
                               w["sp_size"], w["potts"], w["sigma2_app"], w["alpha"],
                               w["split_alpha"], True, False, sm_period=w["sm_period"],
                               prop_niters=w["prop_niters"])
        torch.cuda.synchronize()
        n_hw = sum(1 for r in res if r == hw)
        t0 = time.perf_counter()
        bist_cuda.bist_forward(v, f, w["niters"], w["sp_size"], w["potts"], w["sigma2_app"],
                               w["alpha"], w["split_alpha"], True, False,
                               sm_period=w["sm_period"], prop_niters=w["prop_niters"])
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # weight by the share of streams at this resolution
        plain_frames += n_hw * sv["T"]
        plain_s += n_hw * dt
    plain_fps = plain_frames / plain_s
    budget = int(sv["budget_gb"] * 2 ** 30)
    srv = serve.Server(budget, max_batch=max_batch or args.max_batch,
                       lanes=lanes or args.lanes, device=dev, seed=rank,
                       max_pixels=max_pixels, group_sizes=group_sizes, **cfg)
    # warm-up run (untimed): two short streams per resolution, so that the lanes'
    # engine contexts exist and the sweep tile classes are tuned
    for j, hw in enumerate(sorted(pool) * 2):
        v, f = pool[hw][0]
        srv.add(serve.StreamRequest(-1 - j, v[:4], f[:3], fps=1000.0))
    srv.run()
    torch.cuda.synchronize()
    for sid, hw in enumerate(res):
        v, f = pool[hw][sid % sv["pool"]]
        srv.add(serve.StreamRequest(sid, v, f, fps=sv["fps"]))
    clk_lines, stop = [], threading.Event()
    th = threading.Thread(target=sample_clocks, args=(args.local, stop, clk_lines), daemon=True)
    th.start()
    st = srv.run()
    stop.set()
    th.join(timeout=5)
    hist = {f"{h}p": sum(1 for r in res if r[0] == h) for h in sorted(set(r[0] for r in res))}
    return {"serving": st, "plain_per_frame_fps": plain_fps,
            "served_vs_plain": st["frames_per_s"] / plain_fps, "streams_by_height": hist,
            "offered_fps": streams * sv["fps"], "clocks": summarize_clocks(clk_lines)}


def run_serve(args, world, rank):
    """--mode serve: the serving form (serve_leg) on SERVE's stream set."""
    import torch

    torch.cuda.set_device(args.local)
    dev = torch.device("cuda", args.local)
    w, sv = WORKLOAD, dict(SERVE, fps=args.fps, T=args.frames)
    S = args.streams
    leg = serve_leg(args, dev, rank, S, sv["T"], sv["fps"],
                    group_sizes=not args.no_group_sizes, max_pixels=args.max_pixels)
    st = leg["serving"]
    if rank != 0:
        return
    line = {
        "metric": "served frames/sec (mixed 360p/720p/1080p streams)", "value": st["frames_per_s"],
        "unit": "frames/s", "n_gpus": world, "steps": 1, "warmup": 0,
        "ms_per_step": 1000 * st["wall_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64+int64", "data": "synthetic",
        "config": {"workload": sv["name"], "streams": S,
                   "streams_by_height": leg["streams_by_height"],
                   "frames_per_stream": sv["T"], "arrivals": "Poisson %.0f fps per stream" % sv["fps"],
                   "offered_fps": leg["offered_fps"], "budget_gb": sv["budget_gb"],
                   "max_batch": args.max_batch, "max_pixels": args.max_pixels,
                   "group_sizes": not args.no_group_sizes,
                   "lanes": args.lanes, "warmup": "2 streams x 4 frames per resolution, untimed",
                   "sp_size": w["sp_size"], "niters": w["niters"], "prop_niters": w["prop_niters"],
                   "sm_period": w["sm_period"]},
        "serving": st,
        "plain_per_frame_fps": leg["plain_per_frame_fps"],
        "served_vs_plain": leg["served_vs_plain"],
        "clocks": leg["clocks"],
    }
    print(json.dumps(line), flush=True)


def serving_summary(leg: dict, label: str) -> dict:
    """The serving figures the default bench line carries for one load."""
    st = leg["serving"]
    bh = st.get("by_height", {})
    return {"load": label, "streams_by_height": leg["streams_by_height"],
            "offered_fps": leg["offered_fps"], "served_fps": st.get("frames_per_s"),
            "frames": st.get("frames"), "plain_per_frame_fps": leg["plain_per_frame_fps"],
            "served_vs_plain": leg["served_vs_plain"],
            "p50_ms": st.get("p50_ms"), "p99_ms": st.get("p99_ms"),
            "p50_720p_ms": bh.get("720p", {}).get("p50_ms"),
            "p99_720p_ms": bh.get("720p", {}).get("p99_ms"),
            "by_height": bh, "mean_batch": st.get("mean_batch"),
            "clocks": leg["clocks"]}


BATCH = dict(name="batch64_uneven_240to1080", n=64, lo=240, hi=1080, seeds=(100, 800),
             sigma=(0.02, 0.08), sp=(12, 16, 20, 25), niters=20, sm_period=10)


def batch_frames(n: int, seed: int):
    """The uneven batch: H, W uniform in [240, 1080] rounded down to multiples of 8,
    a Voronoi frame with 100-800 seeds and noise sigma in [0.02, 0.08], superpixel
    size drawn from {12, 16, 20, 25}."""
    import numpy as np
    from st_spix_gb300 import synth
    b = BATCH
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        H = int(rng.integers(b["lo"], b["hi"] + 1)) // 8 * 8
        W = int(rng.integers(b["lo"], b["hi"] + 1)) // 8 * 8
        ns = int(rng.integers(b["seeds"][0], b["seeds"][1] + 1))
        sg = float(rng.uniform(*b["sigma"]))
        sp = int(rng.choice(b["sp"]))
        out.append((H, W, ns, sg, sp, 10_000 * seed + i))
    return out


def run_batch_mode(args, world, rank):
    """--mode batch: 64 independent frames of uneven size as ONE batch (every kernel
    of the path launched once for all frames), against the plain per-frame path
    (run_bass one frame at a time) on the same frames; labels must be identical."""
    import numpy as np
    import torch
    from st_spix_gb300 import batch, bist_cuda, synth

    torch.cuda.set_device(args.local)
    dev = torch.device("cuda", args.local)
    b, w = BATCH, WORKLOAD
    specs = batch_frames(b["n"], seed=rank)
    imgs = []
    for H, W, ns, sg, sp, sd in specs:
        v, _ = synth.voronoi_video_device(H, W, 1, ns, sg, seed=sd, device=dev)
        imgs.append((v[0].contiguous(), sp))
    cfg = dict(niters=b["niters"], potts=w["potts"], sigma2_app=w["sigma2_app"],
               alpha=w["alpha"], split_alpha=w["split_alpha"], sm_period=b["sm_period"])
    npix = sum(im.shape[0] * im.shape[1] for im, _ in imgs)

    def one_batch():
        fr = [batch.Frame(img=im, sp_size=sp) for im, sp in imgs]
        batch.process_batch(fr, **cfg)
        return fr

    for _ in range(args.warmup):
        one_batch()
    torch.cuda.synchronize()
    clk_lines, stop = [], threading.Event()
    th = threading.Thread(target=sample_clocks, args=(args.local, stop, clk_lines), daemon=True)
    th.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fr = one_batch()
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    stop.set()
    th.join(timeout=5)
    gpu_ms = bist_cuda._ctx(dev).last_batch_ms()
    # the same batch with the persistent work-queue sweep in place of one block per tile
    def one_batch_queue():
        fq = [batch.Frame(img=im, sp_size=sp) for im, sp in imgs]
        batch.process_batch(fq, sweep_queue=1, **cfg)
        return fq

    for _ in range(args.warmup):
        one_batch_queue()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fq = one_batch_queue()
    torch.cuda.synchronize()
    elapsed_q = time.perf_counter() - t0
    gpu_ms_q = bist_cuda._ctx(dev).last_batch_ms()
    same_q = sum(int(torch.equal(a.labels, b.labels)) for a, b in zip(fr, fq))
    # plain per-frame path on the same frames (one untimed pass first: workspace
    # growth and tile tuning for the single-frame sizes)
    for im, sp in imgs:
        bist_cuda.run_bass(im, sp_size=sp, **cfg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_labels = [bist_cuda.run_bass(im, sp_size=sp, **cfg)[0] for im, sp in imgs]
    torch.cuda.synchronize()
    plain = time.perf_counter() - t0
    same = sum(int(torch.equal(lab, f.labels)) for lab, f in zip(plain_labels, fr))
    if rank != 0:
        return
    value = b["n"] * args.steps / elapsed
    line = {
        "metric": "batched frames/sec (64 uneven frames per batch)", "value": value,
        "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64+int64", "data": "synthetic",
        "config": {"workload": b["name"], "frames": b["n"], "mpix_per_batch": npix / 1e6,
                   "niters": b["niters"], "sm_period": b["sm_period"],
                   "sp_sizes": b["sp"], "step": "one batch of all frames"},
        "batch_gpu_ms": gpu_ms,
        "mpix_per_s": npix * args.steps / elapsed / 1e6,
        "plain_per_frame_fps": b["n"] / plain,
        "batched_vs_plain": value / (b["n"] / plain),
        "frames_identical_to_plain": f"{same}/{b['n']}",
        "work_queue_sweep": {"value": b["n"] * args.steps / elapsed_q, "unit": "frames/s",
                             "batch_gpu_ms": gpu_ms_q,
                             "frames_identical": f"{same_q}/{b['n']}",
                             "note": "the same batch with the persistent work-queue sweep "
                                     "(stspix_config.sweep_queue = 1) in place of one block "
                                     "per tile"},
        "clocks": summarize_clocks(clk_lines),
    }
    print(json.dumps(line), flush=True)


IMAGE = dict(name="bass_image_240x320", H=240, W=320, nseeds=200, sigma=0.05, sp=15, niters=100,
             sm_period=20)


LATENCY = dict(name="latency_stream_480p_720p_1080p", sizes=((480, 854), (720, 1280), (1080, 1920)),
               frames=10, batches=(1, 8))


def frame_latencies(H, W, B, T, cfg, dev, nseeds, sigma):
    """Host wall ms of each propagated batch of B streams of H x W (frames 1..T-1), one
    frame per stream per batch, after one untimed pass over the same frames."""
    import torch
    from st_spix_gb300 import batch, synth
    vids = [synth.voronoi_video_device(H, W, T, nseeds, sigma, seed=i, device=dev)
            for i in range(B)]
    videos = [batch.Video(H, W, dev) for _ in range(B)]

    def run(times):
        for v in videos:
            v.reset()
        for t in range(T):
            fr = [batch.Frame(img=vids[i][0][t], flow=vids[i][1][t - 1] if t else None,
                              video=videos[i]) for i in range(B)]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            batch.process_batch(fr, **cfg)
            torch.cuda.synchronize()
            if t > 0:
                times.append(1000 * (time.perf_counter() - t0))
    run([])
    times = []
    run(times)
    for v in videos:
        v.close()
    return sorted(times)


def run_latency(args, world, rank):
    """--mode latency: per-frame latency of the streaming workload's propagated frames
    (400 seeds, sp 20, 20 iterations, split/merge every 10) with one frame per batch, and
    the per-frame cost at 8 frames per batch, at 480x854, 720p and 1080p; every stream
    runs its frames 0..frames-1 once untimed first."""
    import torch
    from st_spix_gb300 import batch, synth
    torch.cuda.set_device(args.local)
    dev = torch.device("cuda", args.local)
    w, lt = WORKLOAD, LATENCY
    cfg = dict(niters=w["niters"], sp_size=w["sp_size"], potts=w["potts"],
               sigma2_app=w["sigma2_app"], alpha=w["alpha"], split_alpha=w["split_alpha"],
               sm_period=w["sm_period"], prop_niters=w["prop_niters"])
    T = lt["frames"]
    res = {}
    for H, W in lt["sizes"]:
        for B in lt["batches"]:
            times = frame_latencies(H, W, B, T, cfg, dev, w["nseeds"], w["sigma"])
            res[f"{H}x{W}_batch{B}"] = {"batch_ms_p50": times[len(times) // 2],
                                        "batch_ms_max": times[-1],
                                        "ms_per_frame": sum(times) / len(times) / B}
    if rank != 0:
        return
    line = {"metric": "per-frame latency (propagated frames)",
            "value": res["720x1280_batch1"]["batch_ms_p50"], "unit": "ms",
            "n_gpus": world, "steps": T - 1, "warmup": 1, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64+int64",
            "data": "synthetic",
            "config": {"workload": lt["name"], "frames": T, "sp_size": w["sp_size"],
                       "niters": w["niters"], "sm_period": w["sm_period"],
                       "value": "720p, one frame per batch, median wall ms"},
            "by_size": res}
    print(json.dumps(line), flush=True)


def run_image(args, world, rank):
    """--mode image: plain BASS on one 240x320 Voronoi frame (200 seeds, noise 0.05,
    superpixel size 15, 100 iterations, split/merge every 20), one frame per call
    (run_bass), against the oracle on the same frame on one host core."""
    import numpy as np
    import torch
    from oracle import oracle as O
    from st_spix_gb300 import bist_cuda, synth

    torch.cuda.set_device(args.local)
    dev = torch.device("cuda", args.local)
    im = IMAGE
    img, _ = synth.voronoi_frame(im["H"], im["W"], im["nseeds"], im["sigma"], seed=rank)
    g = torch.from_numpy(img).to(dev)
    kw = dict(niters=im["niters"], sp_size=im["sp"], sm_period=im["sm_period"])
    for _ in range(args.warmup):
        lab, _ = bist_cuda.run_bass(g, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lab, params = bist_cuda.run_bass(g, **kw)
    torch.cuda.synchronize()
    el = (time.perf_counter() - t0) / args.steps
    O.build()
    t0 = time.perf_counter()
    st, olab, _, n = O.run_bass(img, O.default_config(**kw))
    cpu = time.perf_counter() - t0
    same = bool(np.array_equal(olab, lab.cpu().numpy()))
    if rank != 0:
        return
    line = {"metric": "frames/sec (plain BASS, one 240x320 frame per call)", "value": 1.0 / el,
            "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * el, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64+int64", "data": "synthetic",
            "config": {"workload": im["name"], **{k: im[k] for k in ("H", "W", "nseeds", "sigma", "sp", "niters", "sm_period")}},
            "nspix": int(params.n), "labels_identical_to_oracle": same,
            "cpu_baseline": {"value": 1.0 / cpu, "unit": "frames/s", "cores": 1, "kind": "port",
                             "sample": "the same frame, oracle (CPU restatement), one core"}}
    print(json.dumps(line), flush=True)


PRECISION = dict(name="precision_4k_2160x3840", H=2160, W=3840, nseeds=2000, sp=25, niters=20,
                 sm_period=10, frames=3)


def total_marginal_np(n, s, q, b0, log_01_b0):
    """The split/merge marginal of one superpixel over three channels (the engine's
    total_marginal, FP64), vectorised: n [m], s and q [m,3]."""
    import numpy as np
    a_n = 1e4 + n / 2.0
    d = 0.5 * (q - s * s / n[:, None])
    lr = np.where(b0 + d < 0, log_01_b0, np.log1p(d / b0))
    return (-a_n[:, None] * lr).sum(1) + 3 * (-0.5 * np.log(n) - n * (0.5 * np.log(np.pi) + np.log(2.0)))


def run_precision(args, world, rank):
    """--mode precision: accumulator precision study on a 4K video (2160x3840, 2000
    Voronoi seeds, superpixel size 25): the colour sums of the statistics as int64
    fixed point (this engine), FP32 atomics (the reference's choice) and FP64 atomics
    (the oracle).  Same labels: per-superpixel mean and colour-scatter errors against
    FP64 and merge Hastings accept/reject flips over all adjacent pairs; full runs:
    label agreement of FP32 / FP64 runs with the int64 run; per-kernel GB/s at 4K."""
    import numpy as np
    import torch
    from st_spix_gb300 import batch, bist_cuda, synth, _lib

    torch.cuda.set_device(args.local)
    dev = torch.device("cuda", args.local)
    pc, w = PRECISION, WORKLOAD
    T = pc["frames"]
    vid, flo = synth.voronoi_video_device(pc["H"], pc["W"], T, pc["nseeds"], w["sigma"],
                                          seed=rank, device=dev)
    base = dict(niters=pc["niters"], sp_size=pc["sp"], potts=w["potts"], sigma2_app=w["sigma2_app"],
                alpha=w["alpha"], split_alpha=w["split_alpha"], sm_period=pc["sm_period"],
                prop_niters=pc["niters"])
    ctx = bist_cuda._ctx(dev)
    labels, secs, logs = {}, {}, {}
    for acc in (0, 1, 2):
        v = batch.Video(pc["H"], pc["W"], dev)
        outs = []
        if acc == 0:
            ctx.profile(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for t in range(T):
            f = batch.Frame(img=vid[t], flow=flo[t - 1] if t else None, video=v)
            batch.process_batch([f], accumulator=acc, **base)
            outs.append(f.labels.clone())
        torch.cuda.synchronize()
        secs[acc] = time.perf_counter() - t0
        if acc == 0:
            kern = ctx.profile_kernels()
            ctx.profile(False)
        labels[acc] = outs
        v.close()
    npix = pc["H"] * pc["W"]
    def matched(a, b):
        """Fraction of pixels whose label in a maps to their label in b when every
        label of a is matched to the label of b it overlaps most."""
        a = a.reshape(-1).long()
        b = b.reshape(-1).long()
        nb = int(b.max().item()) + 2
        key = (a + 1) * nb + (b + 1)
        uk, cnt = torch.unique(key, return_counts=True)
        ua = uk // nb
        best = torch.zeros(int(ua.max().item()) + 1, dtype=cnt.dtype, device=cnt.device)
        best.scatter_reduce_(0, ua, cnt, reduce="amax")
        return float(best.sum().item()) / a.numel()
    agree = {name: [float((labels[a][t] == labels[0][t]).float().mean().item()) for t in range(T)]
             for name, a in (("fp32", 1), ("fp64", 2))}
    agree_m = {name: [matched(labels[a][t], labels[0][t]) for t in range(T)]
               for name, a in (("fp32", 1), ("fp64", 2))}
    # same labels, three accumulators
    cfg0 = _lib.default_config(sigma2_app=w["sigma2_app"])
    b0 = float(np.float32(np.float32(np.sqrt(cfg0.sigma2_app) * 2) * np.float32(1e4)))
    log_01_b0 = np.log(0.1) - np.log(b0)
    log_alpha = float(np.log(np.float32(np.exp(w["alpha"]))))
    per_frame = []
    import ctypes as C
    for t in range(T):
        lab = labels[0][t]
        n = int(lab.max().item()) + 1
        st = {}
        for acc in (0, 1, 2):
            out = torch.empty(7 * n, dtype=torch.float64, device=dev)
            ctx.check(ctx.lib.stspix_label_stats(ctx.handle, bist_cuda._stream(dev), vid[t].data_ptr(),
                                                 lab.data_ptr(), pc["H"], pc["W"], n, acc,
                                                 out.data_ptr()))
            st[acc] = out.view(n, 7).cpu().numpy()
        live = st[2][:, 0] > 0
        cnt = st[2][live, 0]
        res = {}
        for name, a in (("int64", 0), ("fp32", 1)):
            mu_a = st[a][live, 1:4] / cnt[:, None]
            mu_r = st[2][live, 1:4] / cnt[:, None]
            scat_a = st[a][live, 4:7] - st[a][live, 1:4] ** 2 / cnt[:, None]
            scat_r = st[2][live, 4:7] - st[2][live, 1:4] ** 2 / cnt[:, None]
            rel_mu = np.abs(mu_a - mu_r) / np.maximum(np.abs(mu_r), 1e-12)
            rel_sc = np.abs(scat_a - scat_r) / np.maximum(np.abs(scat_r), 1e-12)
            res[name] = {"mean_rel_err_max": float(rel_mu.max()),
                         "mean_rel_err_median": float(np.median(rel_mu)),
                         "scatter_rel_err_max": float(rel_sc.max()),
                         "scatter_rel_err_median": float(np.median(rel_sc))}
        # merge Hastings decisions over all adjacent pairs
        L = lab.cpu().numpy()
        pr = np.concatenate([np.stack([L[:, :-1].ravel(), L[:, 1:].ravel()], 1),
                             np.stack([L[:-1, :].ravel(), L[1:, :].ravel()], 1)])
        pr = pr[(pr[:, 0] != pr[:, 1]) & (pr[:, 0] >= 0) & (pr[:, 1] >= 0)]
        pr = np.unique(np.sort(pr, 1), axis=0)
        dec = {}
        for a in (0, 1, 2):
            S = st[a]
            na, nb_ = S[pr[:, 0], 0], S[pr[:, 1], 0]
            ma = total_marginal_np(na, S[pr[:, 0], 1:4], S[pr[:, 0], 4:7], b0, log_01_b0)
            mb = total_marginal_np(nb_, S[pr[:, 1], 1:4], S[pr[:, 1], 4:7], b0, log_01_b0)
            mf = total_marginal_np(na + nb_, S[pr[:, 0], 1:4] + S[pr[:, 1], 1:4],
                                   S[pr[:, 0], 4:7] + S[pr[:, 1], 4:7], b0, log_01_b0)
            h = mf - (log_alpha + ma + mb)
            dec[a] = (h > -2, h)
        for name, a in (("int64", 0), ("fp32", 1)):
            res[name]["merge_flips_vs_fp64"] = int((dec[a][0] != dec[2][0]).sum())
            res[name]["hastings_abs_err_max"] = float(np.abs(dec[a][1] - dec[2][1]).max())
        res["pairs"] = int(len(pr))
        res["superpixels"] = int(live.sum())
        per_frame.append(res)
    # per-kernel bandwidth of the int64 run at 4K (CUDA events)
    bytes_per_px = {"kb_sweep_t32": 20, "kb_sweep_t64": 20, "kb_accumulate": 16}
    gbs = {}
    for k, (nl, ms) in kern.items():
        if k in bytes_per_px and ms > 0:
            gbs[k] = {"launches": nl, "avg_us": 1000 * ms / nl,
                      "achieved_gbs": bytes_per_px[k] * npix * nl / (ms / 1000) / 1e9}
    peak, peak_kind = read_peaks()
    if rank != 0:
        return
    line = {
        "metric": "accumulator precision study (4K)", "value": agree_m["fp32"][-1],
        "unit": "matched label agreement of the FP32-accumulator run with the int64 run, last frame",
        "n_gpus": world, "steps": 1, "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64+int64", "data": "synthetic",
        "config": {"workload": pc["name"], "H": pc["H"], "W": pc["W"], "frames": T,
                   "nseeds": pc["nseeds"], "sp_size": pc["sp"], "niters": pc["niters"],
                   "sm_period": pc["sm_period"],
                   "sample": "first %d frames of the 60-frame configuration" % T},
        "label_agreement_vs_int64": {"raw": agree, "matched": agree_m},
        "same_labels": per_frame,
        "seconds_per_run": secs,
        "kernel_gbs_int64_run": gbs, "hbm_peak_gbs": peak, "peak_source": peak_kind,
    }
    print(json.dumps(line), flush=True)


def main():
    faulthandler.enable(all_threads=True)
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--streams", type=int, default=None,
                    help="video streams per GPU (default 32; serve: 256); stream mode: frame "
                         "t of every stream of a lane runs as one batch")
    ap.add_argument("--lanes", type=int, default=None,
                    help="host threads per GPU, each with its own CUDA stream, engine "
                         "context and share of the streams (default 4 in stream mode, "
                         "else 3)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="stream",
                    choices=["stream", "serve", "batch", "precision", "image", "latency"],
                    help="stream: the 480x854 streaming workload (default); serve: the "
                         "serving form on mixed-resolution Poisson streams; batch: 64 "
                         "independent frames of uneven size as one batch; precision: the "
                         "accumulator precision study at 4K; image: plain BASS on one "
                         "240x320 frame; latency: per-frame latency at 480p/720p/1080p")
    ap.add_argument("--max-batch", type=int, default=8, help="serve: frames per batch")
    ap.add_argument("--max-pixels", type=int, default=0,
                    help="serve: pixels per batch (0: no cap); bounds a batch's GPU time")
    ap.add_argument("--fps", type=float, default=30.0, help="serve: mean frame rate per stream")
    ap.add_argument("--frames", type=int, default=30, help="serve: frames per stream")
    ap.add_argument("--sweep-schedule", type=int, default=0, choices=[0, 1, 2],
                    help="stream: boundary sweeps per launch (0 autotuned, 1 one, 2 two); "
                         "the labels are the same")
    ap.add_argument("--sweep-tile", type=int, default=0, choices=[0, 16, 32, 64],
                    help="stream: single-sweep tile width (0 autotuned); profiler runs pin "
                         "the width the autotuner picks without the profiler")
    ap.add_argument("--sweep-queue", type=int, default=0, choices=[0, 1],
                    help="stream: 1 runs single sweeps as the persistent work-queue kernel")
    ap.add_argument("--no-group-sizes", action="store_true",
                    help="serve: batches take frames oldest first across sizes (default: the "
                         "oldest frame's size first)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true",
                    help="stream: skip the serving figures (config-3 load and the sustained load)")
    ap.add_argument("--serve-frames", type=int, default=10,
                    help="stream: frames per stream of the config-3 serving leg (bounds its time)")
    ap.add_argument("--no-batch-graphs", action="store_true",
                    help="stream: launch every batch step's kernels one by one (ncu lists no "
                         "kernel of a graph that holds conditional nodes)")
    args = ap.parse_args()
    if args.streams is None:
        args.streams = SERVE["streams"] if args.mode == "serve" else 32
    if args.lanes is None:
        # stream mode: 4 host lanes of 8 streams (24 on 3: 2377 frames/s, 32 on 4: 2471,
        # 40 on 5: 2465); the serving form keeps 3
        args.lanes = 4 if args.mode == "stream" else 3
    world, rank, local = dist_setup()
    args.local = local
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.mode == "serve":
        return run_serve(args, world, rank)
    if args.mode == "batch":
        return run_batch_mode(args, world, rank)
    if args.mode == "precision":
        return run_precision(args, world, rank)
    if args.mode == "image":
        return run_image(args, world, rank)
    if args.mode == "latency":
        return run_latency(args, world, rank)
    args.warmup = max(args.warmup, 3)

    import numpy as np
    import torch
    from st_spix_gb300 import batch, bist_cuda

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    w = WORKLOAD
    S = max(1, args.streams)
    NL = max(1, min(args.lanes, S))
    T = w["T"]
    cfg = dict(niters=w["niters"], sp_size=w["sp_size"], potts=w["potts"],
               sigma2_app=w["sigma2_app"], alpha=w["alpha"], split_alpha=w["split_alpha"],
               sm_period=w["sm_period"], prop_niters=w["prop_niters"],
               sweep_schedule=args.sweep_schedule, sweep_tile=args.sweep_tile,
               sweep_queue=args.sweep_queue)

    # one video per stream (seed = rank * S + i), generated on the device; the host
    # copies feed the end-to-end leg
    from st_spix_gb300 import synth
    dvid, dflo = [], []
    for i, sd in enumerate(replica_seeds(rank, S)):
        out = synth.voronoi_video_device(w["H"], w["W"], T, w["nseeds"], w["sigma"],
                                         seed=sd, device=dev, regions=i == 0)
        dvid.append(out[0])
        dflo.append(out[1])
        if i == 0:
            regions0 = out[2]      # ground truth of stream 0 for the quality scores
    host = [(v.cpu().numpy(), f.cpu().numpy()) for v, f in zip(dvid, dflo)]
    dout = [torch.empty((T, w["H"], w["W"]), dtype=torch.int32, device=dev) for _ in range(S)]
    lanes = [list(range(j, S, NL)) for j in range(NL)]
    cstreams = [torch.cuda.Stream(dev) for _ in range(NL)]
    videos, ctxs = [], []
    for j in range(NL):
        with torch.cuda.stream(cstreams[j]):
            videos.append([batch.Video(w["H"], w["W"], dev) for _ in lanes[j]])
            ctxs.append(bist_cuda._ctx(dev))
            ctxs[-1].set_batch_graphs(not args.no_batch_graphs)
    batch_ms = [[] for _ in range(NL)]

    def video_pass(j, vid, flo, out, record, before=None, after=None):
        """All T frames of lane j's streams: frame t of every stream in one batch
        (before(t) / after(t): hooks around batch t)."""
        for v in videos[j]:
            v.reset()
        for t in range(T):
            if before:
                before(t)
            fr = [batch.Frame(img=vid[i][t], flow=flo[i][t - 1] if t > 0 else None,
                              video=videos[j][k], labels=out[i][t])
                  for k, i in enumerate(lanes[j])]
            batch.process_batch(fr, **cfg)
            if after:
                after(t)
            if record:
                batch_ms[j].append(ctxs[j].last_batch_ms())

    def run_lanes(fn, nsteps):
        gate = threading.Barrier(NL)
        errs = []

        def body(j):
            try:
                torch.cuda.set_device(dev)
                with torch.cuda.stream(cstreams[j]):
                    gate.wait()
                    for st in range(nsteps):
                        fn(j, st)
                    cstreams[j].synchronize()
            except Exception as e:  # surfaced below
                errs.append(repr(e))
        th = [threading.Thread(target=body, args=(j,)) for j in range(NL)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errs:
            raise RuntimeError("; ".join(errs))

    run_lanes(lambda j, st: video_pass(j, dvid, dflo, dout, False), args.warmup)
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs, larger than L2) -----------------
    clk_lines, stop = [], threading.Event()
    th = threading.Thread(target=sample_clocks, args=(local, stop, clk_lines), daemon=True)
    th.start()
    l0 = [c.launches() for c in ctxs]
    g0 = [c.graph_replays() for c in ctxs]
    barrier()
    torch.cuda.synchronize()
    # device time: one start event, every lane's stream waits on it and records its own
    # end event after its last batch; the step time is the latest end
    ev0 = torch.cuda.Event(enable_timing=True)
    ev_end = [torch.cuda.Event(enable_timing=True) for _ in range(NL)]
    ev0.record()
    for cs in cstreams:
        cs.wait_event(ev0)
    t0 = time.perf_counter()

    lane_done = [0.0] * NL

    def timed(j, st):
        video_pass(j, dvid, dflo, dout, True)
        if st == args.steps - 1:
            ev_end[j].record(cstreams[j])
            lane_done[j] = time.perf_counter() - t0
    run_lanes(timed, args.steps)
    t_joined = time.perf_counter() - t0
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    elapsed = max(ev0.elapsed_time(e) for e in ev_end) / 1000.0
    barrier()
    total_launches = sum(c.launches() - a for c, a in zip(ctxs, l0))
    replays = sum(c.graph_replays() - a for c, a in zip(ctxs, g0))
    stop.set()
    th.join(timeout=5)
    elapsed = max_over_ranks(elapsed, world, dev)
    frames_total = world * S * T * args.steps
    value = frames_total / elapsed

    # ---- plain per-frame path: one stream, frame by frame (bist_forward) -------
    def plain_call():
        return bist_cuda.bist_forward(dvid[0], dflo[0], w["niters"], w["sp_size"], w["potts"],
                                      w["sigma2_app"], w["alpha"], w["split_alpha"], True, False,
                                      sm_period=w["sm_period"], prop_niters=w["prop_niters"])
    pstream = torch.cuda.Stream(dev)
    with torch.cuda.stream(pstream):
        plain_call()
        pstream.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plain_out = plain_call()
        pstream.synchronize()
        plain_fps = T * args.steps / (time.perf_counter() - t0)
    agree = float((plain_out == dout[0]).float().mean().item())

    # ---- quality scores of stream 0 against its generator's regions (GPU) --------
    from st_spix_gb300 import metrics
    metrics.evaluate(dvid[0][:2], dout[0][:2], regions0[:2])       # first-use warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qual = metrics.computeSummary(dvid[0], regions0, dout[0])
    torch.cuda.synchronize()
    qual_ms = 1000 * (time.perf_counter() - t0)

    # ---- 720p frame latency: one stream alone, one frame per batch -------------------
    lat = frame_latencies(720, 1280, 1, T, cfg, dev, w["nseeds"], w["sigma"])
    lat720 = {"frames": len(lat), "p50_ms": lat[len(lat) // 2],
              "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
              "note": "one 720p stream of the same video model alone, one frame per batch, host "
                      "wall per propagated frame (frames 1..%d, after one untimed pass)" % (T - 1)}

    # ---- per-family device time of lane 0's batches (CUDA events on its stream) --
    with torch.cuda.stream(cstreams[0]):
        ctxs[0].profile(True)
        video_pass(0, dvid, dflo, dout, False)
        cstreams[0].synchronize()
        prof = ctxs[0].profile_get()
        sweep_kernels = {k: v[0] for k, v in ctxs[0].profile_kernels().items()
                         if k.startswith("kb_sweep")}
        ctxs[0].profile(False)

    # ---- e2e through the public API with host buffers --------------------------
    h_vid = [torch.from_numpy(v).pin_memory() for v, _ in host]
    h_flo = [torch.from_numpy(f).pin_memory() for _, f in host]
    h_out = [torch.empty((T, w["H"], w["W"]), dtype=torch.int32).pin_memory() for _ in range(S)]
    e_vid = [torch.empty_like(v) for v in dvid]
    e_flo = [torch.empty_like(f) for f in dflo]

    # Frames stream in: each lane keeps the host->device copies of its next LOOKAHEAD
    # frames queued on its copy-in stream (the steps form one continuous sequence of
    # frames), so the copy engines serve the lanes' frames in step with the batches
    # instead of one lane's whole step ahead of the others; batch t waits for frame t
    # only, a frame buffer is refilled once the previous step's batches that read it are
    # done, and frame t's labels go back on the copy-out stream while later batches run.
    # The streams are synchronised once, after the last step.
    LOOKAHEAD = 3
    in_streams = [torch.cuda.Stream(dev) for _ in range(NL)]
    out_streams = [torch.cuda.Stream(dev) for _ in range(NL)]
    in_ev = [dict() for _ in range(NL)]          # (step, t) -> copy-in done
    read_ev = [dict() for _ in range(NL)]        # t -> previous use of frame buffer t done

    def enqueue(j, st, t):
        with torch.cuda.stream(in_streams[j]):
            # frame t is read by batch t, its flow by batch t + 1
            dep = read_ev[j].get(min(t + 1, T - 1))
            if dep is not None:
                in_streams[j].wait_event(dep)
            for i in lanes[j]:
                e_vid[i][t].copy_(h_vid[i][t], non_blocking=True)
                if t < T - 1:
                    e_flo[i][t].copy_(h_flo[i][t], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(in_streams[j])
            in_ev[j][(st, t)] = ev

    def e2e(j, st):
        if st == 0:
            for t in range(min(LOOKAHEAD, T)):
                enqueue(j, 0, t)

        def before(t):
            g = st * T + t + LOOKAHEAD
            if g < args.steps * T:
                enqueue(j, g // T, g % T)
            cstreams[j].wait_event(in_ev[j].pop((st, t)))

        def after(t):
            ev = torch.cuda.Event()
            ev.record(cstreams[j])
            read_ev[j][t] = ev
            out_streams[j].wait_event(ev)
            with torch.cuda.stream(out_streams[j]):
                for i in lanes[j]:
                    h_out[i][t].copy_(dout[i][t], non_blocking=True)
        video_pass(j, e_vid, e_flo, dout, False, before, after)
        if st == args.steps - 1:
            out_streams[j].synchronize()
            cstreams[j].synchronize()

    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_lanes(e2e, args.steps)
    e2e_elapsed = time.perf_counter() - t0
    barrier()
    e2e_elapsed = max_over_ranks(e2e_elapsed, world, dev)
    e2e_value = frames_total / e2e_elapsed

    # ---- serving form on the mixed-resolution set: config-3 load (256 streams, Poisson
    # 30 fps, frames per stream bounded) and the largest load it sustains (streams at
    # 30 fps offering 85 % of the rate served under the config-3 backlog) -------------
    serving = None
    if not args.no_serve and world == 1:
        full = serve_leg(args, dev, rank, SERVE["streams"], args.serve_frames, SERVE["fps"],
                         lanes=SERVE_LANES)
        served = full["serving"].get("frames_per_s") or 0.0
        # the largest load served as offered: start at 85 % of the config-3 served rate and
        # shrink until the served rate is within 5 % of the offered one (3 tries at most)
        n_sus, tries = max(1, int(0.85 * served / SERVE["fps"])), []
        for _ in range(3):
            sus = serve_leg(args, dev, rank, n_sus, WORKLOAD["T"], SERVE["fps"],
                            lanes=SERVE_LANES)
            got = sus["serving"].get("frames_per_s") or 0.0
            tries.append({"streams": n_sus, "offered_fps": sus["offered_fps"], "served_fps": got})
            if got >= 0.95 * sus["offered_fps"] or n_sus == 1:
                break
            n_sus = max(1, int(0.9 * n_sus * got / sus["offered_fps"]))
        light = serve_leg(args, dev, rank, 4, WORKLOAD["T"], SERVE["fps"], lanes=SERVE_LANES)
        serving = {"config3": serving_summary(full, "256 streams, Poisson 30 fps each, %d frames "
                                               "per stream" % args.serve_frames),
                   "sustained": dict(serving_summary(sus, "%d streams, Poisson 30 fps each, %d "
                                                     "frames per stream" % (n_sus, WORKLOAD["T"])),
                                     search=tries),
                   "light": serving_summary(light, "4 streams, Poisson 30 fps each, %d frames per "
                                            "stream" % WORKLOAD["T"]),
                   "target": "served / plain >= 5 and 720p p99 < 10 ms"}

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel ---------------------------------------
    npix = w["H"] * w["W"]
    B0 = len(lanes[0])
    fam = max(prof, key=lambda k: prof[k][1])
    nsweep = prof["sweep"][0]       # one fused launch per sweep, over the lane's batch
    sweep_ms = prof["sweep"][1]
    peak, peak_kind = read_peaks()
    per_launch = SWEEP_BYTES_PER_PX * npix * B0
    achieved = per_launch * nsweep / (sweep_ms / 1000.0) / 1e9 if sweep_ms else 0
    passes_per_video = w["niters"] + (T - 1) * w["prop_niters"]
    mpix_pass = world * S * args.steps * passes_per_video * npix / elapsed / 1e6

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        base = CpuBaseline(window=3)
        try:
            cpu_frames, cpu_wall = base.step()
            cpu = {"value": cpu_frames / cpu_wall, "unit": "frames/s", "cores": base.cores,
                   "kind": "port", "sample": base.describe()}
        finally:
            base.close()

    bms = sorted(x for lst in batch_ms for x in lst)
    pct = lambda q: bms[min(len(bms) - 1, int(q * len(bms)))] if bms else None
    h_bytes = sum(v.nbytes + f.nbytes for v, f in host)
    line = {
        "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/f64+int64", "data": "synthetic",
        "config": workload_config(),
        "run": {"streams_per_gpu": S, "lanes": NL, "batch_per_lane": B0,
                   "sweep_schedule": args.sweep_schedule, "sweep_tile": args.sweep_tile,
                   "sweep_queue": args.sweep_queue,
                   "batch_graphs": not args.no_batch_graphs,
                   "step": "all %d frames of every stream; frame t of a lane's streams is "
                           "one batch" % T,
                   "parallelism": f"replicas{world}",
                   "inputs_mb_per_step": h_bytes // 2 ** 20},
        "p50_frame_ms": pct(0.50), "p99_frame_ms": pct(0.99),
        "latency_720p": lat720,
        "latency_note": "frame latency = GPU time of the batch the frame ran in",
        "plain_per_frame_fps": plain_fps,
        "plain_vs_batched_label_agreement": agree,
        "mpix_per_s_per_pass": mpix_pass,
        "roofline": {"bound": "hbm", "kernel": "kb_sweep (border + 4 parity phases, batched; statistics fused into the last sweep of each update)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": SWEEP_TRAFFIC_NCU["bytes_per_launch"],
                     "traffic_source": SWEEP_TRAFFIC_NCU["source"],
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": per_launch,
                     "dominant_family": fam,
                     "family_ms": {k: round(v[1], 3) for k, v in prof.items()},
                     "family_launches": {k: v[0] for k, v in prof.items()},
                     "sweep_kernels_lane0": sweep_kernels},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "frames/s",
                "h2d_bytes_per_step": int(h_bytes),
                "d2h_bytes_per_step": int(sum(o.numel() * 4 for o in h_out))},
        "gpu_launches": int(total_launches),
        "graph_replays": int(replays),
        "sweep_choices": [c.sweep_choices() for c in ctxs],
        "timing": "CUDA events (start on the default stream, every lane's stream waits on it; "
                  "step time = latest lane end); host wall %.1f ms per step (last lane "
                  "done %.1f ms, threads joined %.1f ms after the start, %d steps)" %
                  (1000 * wall / args.steps, 1000 * max(lane_done), 1000 * t_joined, args.steps),
        "clocks": summarize_clocks(clk_lines),
        "serving": serving,
        "quality": dict({k: qual[k] for k in ("tex", "szv", "ev", "ev3d", "pooling", "ue2d",
                                              "sa2d", "ue3d", "sa3d", "spnum", "ave_nsp")},
                        stream=0, ground_truth="generator regions (%d)" % w["nseeds"],
                        evaluate_ms=qual_ms),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
