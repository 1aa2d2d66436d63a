"""Serving form of the streaming-BASS path: many concurrent video streams, admitted
under a device-memory budget, served by continuous batching.

The reference processes one video per call, one frame after another
(st_spix/csrc/bist/pyapi.cu:46 main_loop); a serving deployment has many streams
whose frames arrive over time.  Here

  * every admitted stream keeps its labels, superpixel parameters and superpixel
    count resident on the device between frames (st_spix_gb300.batch.Video);
  * streams are admitted while their resident bytes fit the budget next to the
    working buffers of the batches in flight; a stream that does not fit waits
    until one that finished releases its memory;
  * host lanes (each a thread with its own CUDA stream and engine context) take the
    frames that have arrived -- at most one per stream, oldest first, up to
    max_batch -- as one batch whenever they are free, so frames that arrive while
    other batches are on the GPU join the next batch and batches overlap on the
    device.

A frame's result does not depend on the batch it ran in (every kernel is
slot-local), so each stream's labels equal those of bist_forward on that stream
alone.  Scheduler is the host logic alone (no GPU), Server drives it on a GPU.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np


# ---------------------------------------------------------------------------
# Host logic: admission and batch selection.
@dataclass
class _StreamState:
    sid: int
    nbytes: int
    rel_arrivals: np.ndarray          # arrival times relative to admission (s)
    kind: object = None               # streams of one kind can reuse each other's state
    npix: int = 0                     # pixels per frame (batch pixel cap)
    arrivals: Optional[np.ndarray] = None
    admitted_at: Optional[float] = None
    next: int = 0                     # next frame index to serve
    in_flight: bool = False
    finished: bool = False

    @property
    def nframes(self) -> int:
        return len(self.rel_arrivals)


class Scheduler:
    """Admission under a byte budget and continuous-batching frame selection.

    budget: device bytes available; reserve: bytes held by the working buffers of
    the batches in flight (taken off the budget up front).  Streams are offered
    with their resident bytes, a kind (streams of one kind have the same state
    size) and frame arrival times (relative to admission), and admitted in offer
    order while they fit.  The state of a finished stream stays allocated as a spare
    of its kind (still counted as used) until a new stream of that kind takes it
    over; when a stream needs fresh bytes that do not fit, spares of other kinds
    are evicted first (their kinds are appended to `evicted` for the caller to
    free).  A batch holds at most max_batch frames and, when max_pixels is set, at most
    that many pixels (but always at least one frame): the cap bounds a batch's GPU
    time and so the latency of the frames in it.  Not thread-safe; Server serialises
    calls with a lock."""

    def __init__(self, budget: int, reserve: int, max_batch: int, max_pixels: int = 0,
                 group_sizes: bool = True):
        if reserve > budget:
            raise ValueError(f"working buffers ({reserve} B) exceed the budget ({budget} B)")
        self.budget, self.reserve, self.max_batch = int(budget), int(reserve), int(max_batch)
        self.max_pixels = int(max_pixels)
        self.group_sizes = bool(group_sizes)
        self.used = self.reserve
        self.streams: Dict[int, _StreamState] = {}
        self.queue: List[int] = []        # offered, not yet admitted (FIFO)
        self.active: List[int] = []       # admitted, not finished
        self.latency: List[Tuple[int, int, float, float]] = []  # (sid, frame, arrival, done)
        self.peak_used = self.used
        self.spare: Dict[object, List[int]] = {}   # kind -> bytes of spare states
        self.evicted: List[object] = []
        self.reused = 0

    def offer(self, sid: int, nbytes: int, rel_arrivals, now: float = 0.0, kind=None,
              npix: int = 0) -> bool:
        """Offer a stream; returns True if it was admitted at once."""
        if sid in self.streams:
            raise ValueError(f"stream {sid} offered twice")
        if self.reserve + nbytes > self.budget:
            raise ValueError(f"stream {sid} needs {nbytes} B: never fits the budget")
        self.streams[sid] = _StreamState(sid, int(nbytes), np.asarray(rel_arrivals, float),
                                         kind if kind is not None else ("bytes", int(nbytes)),
                                         int(npix))
        self.queue.append(sid)
        self.admit(now)
        return self.streams[sid].admitted_at is not None

    def admit(self, now: float) -> List[int]:
        """Admit queued streams in order while they fit; returns the admitted ids."""
        out = []
        while self.queue:
            st = self.streams[self.queue[0]]
            mine = self.spare.get(st.kind)
            if mine:
                self.used -= mine.pop()          # take over a spare state of this kind
                self.reused += 1
            else:
                while self.used + st.nbytes > self.budget and self._evict(st.kind):
                    pass
                if self.used + st.nbytes > self.budget:
                    break
            self.queue.pop(0)
            self.used += st.nbytes
            self.peak_used = max(self.peak_used, self.used)
            st.admitted_at = now
            st.arrivals = now + st.rel_arrivals
            self.active.append(st.sid)
            out.append(st.sid)
        return out

    def next_batch(self, now: float) -> List[Tuple[int, int, float]]:
        """Frames that have arrived, one per idle stream, at most max_batch (and
        max_pixels); they are marked in flight.  Items: (sid, frame, arrival).  The
        oldest frame goes first, then (group_sizes) the other frames of its size, then
        the rest, each oldest first: batches of one frame size waste no grid blocks on
        smaller frames and repeat their launch sequence (which the engine replays as a
        CUDA graph)."""
        ready = []
        for sid in self.active:
            st = self.streams[sid]
            if st.in_flight or st.next >= st.nframes:
                continue
            a = st.arrivals[st.next]
            if a <= now:
                ready.append((a, sid))
        ready.sort()
        if self.group_sizes and ready:
            n0 = self.streams[ready[0][1]].npix
            ready = ([r for r in ready if self.streams[r[1]].npix == n0] +
                     [r for r in ready if self.streams[r[1]].npix != n0])
        items, pix = [], 0
        for a, sid in ready:
            if len(items) >= self.max_batch:
                break
            st = self.streams[sid]
            if self.max_pixels and items and pix + st.npix > self.max_pixels:
                break          # oldest first: a later, smaller frame does not jump the queue
            pix += st.npix
            st.in_flight = True
            items.append((sid, st.next, float(a)))
        return items

    def complete(self, items, done: float) -> List[int]:
        """Record a finished batch; returns the ids of streams that finished (their
        memory is released and queued streams are admitted)."""
        finished = []
        for sid, fi, a in items:
            st = self.streams[sid]
            if not st.in_flight or fi != st.next:
                raise RuntimeError(f"stream {sid}: frame {fi} completed out of order")
            self.latency.append((sid, fi, a, done))
            st.next += 1
            st.in_flight = False
            if st.next >= st.nframes:
                st.finished = True
                self.active.remove(sid)
                self.spare.setdefault(st.kind, []).append(st.nbytes)   # still allocated
                finished.append(sid)
        if finished:
            self.admit(done)
        return finished

    def _evict(self, keep_kind) -> bool:
        for kind, lst in self.spare.items():
            if kind != keep_kind and lst:
                self.used -= lst.pop()
                self.evicted.append(kind)
                return True
        return False

    def next_arrival(self) -> Optional[float]:
        """Earliest arrival of a frame that could be batched next (None if none)."""
        t = None
        for sid in self.active:
            st = self.streams[sid]
            if st.in_flight or st.next >= st.nframes:
                continue
            a = st.arrivals[st.next]
            t = a if t is None else min(t, a)
        return t

    def done(self) -> bool:
        return not self.queue and not self.active


def poisson_arrivals(nframes: int, fps: float, rng: np.random.Generator) -> np.ndarray:
    """Arrival times (s) of a Poisson process of rate fps, first frame at 0."""
    gaps = rng.exponential(1.0 / fps, size=max(nframes - 1, 0))
    return np.concatenate([[0.0], np.cumsum(gaps)])


def percentile(xs, q):
    if not len(xs):
        return None
    return float(np.percentile(np.asarray(xs, float), q))


# ---------------------------------------------------------------------------
# GPU server.
@dataclass
class StreamRequest:
    """A video stream: frames vid f32 [T,H,W,3] and forward flows f32 [T-1,H,W,2]
    on the device (views into shared inputs are fine), frame rate of the arrivals,
    superpixel size (0: the config's)."""
    sid: int
    vid: "object"
    flows: "object"
    fps: float = 30.0
    sp_size: int = 0
    keep_labels: bool = False       # keep every frame's labels (else only the last)


class Server:
    """Continuous-batching server on one GPU (see the module docstring)."""

    def __init__(self, budget_bytes: int, max_batch: int = 8, lanes: int = 2, device=None,
                 seed: int = 0, max_pixels: int = 0, group_sizes: bool = True, **cfg):
        import torch
        from . import batch, bist_cuda, _lib
        self._torch, self._batch, self._bist, self._lib = torch, batch, bist_cuda, _lib
        idx = None if device is None else torch.device(device).index
        self.device = torch.device("cuda", torch.cuda.current_device() if idx is None else idx)
        self.budget = int(budget_bytes)
        self.max_batch = int(max_batch)
        self.max_pixels = int(max_pixels)
        self.group_sizes = bool(group_sizes)
        self.lanes = int(lanes)
        self.cfg = cfg
        self.sp_default = int(cfg.get("sp_size", 15))
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self.requests: Dict[int, StreamRequest] = {}      # added, not yet served
        self.served: Dict[int, StreamRequest] = {}
        self.labels: Dict[int, object] = {}
        self.videos: Dict[int, object] = {}
        self.batch_sizes: List[int] = []
        self.batch_ms: List[float] = []
        self._spare: Dict[Tuple[int, int], list] = {}
        self._spare_lock = threading.Lock()
        self._streams = []    # one CUDA stream per lane, kept across runs (warm contexts)

    def add(self, req: StreamRequest):
        if req.sid in self.requests or req.sid in self.served:
            raise ValueError(f"stream {req.sid} added twice")
        self.requests[req.sid] = req

    def stream_bytes(self, req: StreamRequest) -> int:
        T, H, W = req.vid.shape[0], req.vid.shape[1], req.vid.shape[2]
        vb, _ = self._lib.footprint(H, W, req.sp_size or self.sp_default)
        return vb + 4 * H * W * (T if req.keep_labels else 1)

    def run(self) -> dict:
        """Serve every stream added since the last run; returns its statistics.  The
        lanes' CUDA streams (and so their engine contexts and tuned tile shapes) are
        kept for later runs."""
        torch = self._torch
        reqs = list(self.requests.values())
        if not reqs:
            return {}
        while len(self._streams) < self.lanes:
            self._streams.append(torch.cuda.Stream(self.device))
        self.batch_sizes, self.batch_ms = [], []
        # the largest frame's working buffers for every batch position of every lane
        slot_b = max(self._lib.footprint(r.vid.shape[1], r.vid.shape[2],
                                         r.sp_size or self.sp_default)[1] for r in reqs)
        sched = Scheduler(self.budget, self.lanes * self.max_batch * slot_b, self.max_batch,
                          self.max_pixels, self.group_sizes)
        lock = threading.Lock()
        wake = threading.Condition(lock)
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0
        for r in reqs:
            T, H, W = r.vid.shape[0], r.vid.shape[1], r.vid.shape[2]
            sched.offer(r.sid, self.stream_bytes(r), poisson_arrivals(T, r.fps, self.rng), 0.0,
                        kind=(H, W, T if r.keep_labels else 1), npix=H * W)
        dev = self.device
        errors = []
        replays = [0] * self.lanes

        def lane(j):
            try:
                torch.cuda.set_device(dev)
                with torch.cuda.stream(self._streams[j]):
                    ctx = self._bist._ctx(dev)
                    r0 = ctx.graph_replays()
                    while True:
                        with lock:
                            replays[j] = ctx.graph_replays() - r0
                            if sched.done() or errors:
                                wake.notify_all()
                                return
                            now = clock()
                            items = sched.next_batch(now)
                            if not items:
                                t = sched.next_arrival()
                                wait = 0.05 if t is None else max(0.0, min(0.05, t - now))
                                wake.wait(timeout=wait)
                                continue
                        frames = []
                        for sid, fi, _ in items:
                            r = self.requests[sid]
                            v = self.videos.get(sid)
                            if v is None:
                                v, lab = self._state_for(r)
                                self.videos[sid] = v
                                self.labels[sid] = lab
                            out = self.labels[sid][fi if r.keep_labels else 0]
                            frames.append(self._batch.Frame(
                                img=r.vid[fi], flow=r.flows[fi - 1] if fi > 0 else None,
                                video=v, sp_size=r.sp_size, labels=out))
                        self._batch.process_batch(frames, **self.cfg)
                        done = clock()
                        ms = self._bist._ctx(dev).last_batch_ms()
                        with lock:
                            self.batch_sizes.append(len(items))
                            self.batch_ms.append(ms)
                            for sid in sched.complete(items, done):
                                r = self.requests[sid]
                                self._release(r, self.videos.pop(sid), self.labels[sid])
                            evicted, sched.evicted = sched.evicted, []
                        for kind in evicted:
                            self._evict(kind)
                        with lock:
                            wake.notify_all()
            except Exception as e:  # surfaced by run()
                with lock:
                    errors.append(repr(e))
                    wake.notify_all()

        th = [threading.Thread(target=lane, args=(j,)) for j in range(self.lanes)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for vs in self._spare.values():
            for v, _ in vs:
                v.close()
        self._spare.clear()
        if errors:
            raise RuntimeError("; ".join(errors))
        out = self.stats(sched)
        out["graph_replays"] = int(sum(replays))
        self.served.update(self.requests)
        self.requests = {}
        return out

    # The state (video + label buffer) of a finished stream is kept and handed to the
    # next stream of the same kind (reset first), as the scheduler's accounting
    # assumes; it is freed only when the scheduler evicts it.
    def _state_for(self, r):
        kind = (r.vid.shape[1], r.vid.shape[2], r.vid.shape[0] if r.keep_labels else 1)
        v = lab = None
        with self._spare_lock:
            spare = self._spare.get(kind)
            if spare:
                v, lab = spare.pop()
        if v is not None:
            v.reset()
        else:
            v = self._batch.Video(kind[0], kind[1], self.device)
        if lab is None:
            lab = self._torch.empty((kind[2], kind[0], kind[1]), dtype=self._torch.int32,
                                    device=self.device)
        return v, lab

    def _release(self, r, v, lab):
        # kept labels are the stream's result and go to the caller, not to reuse
        kind = (r.vid.shape[1], r.vid.shape[2], r.vid.shape[0] if r.keep_labels else 1)
        with self._spare_lock:
            self._spare.setdefault(kind, []).append((v, None if r.keep_labels else lab))

    def _evict(self, kind):
        with self._spare_lock:
            lst = self._spare.get(kind)
            item = lst.pop() if lst else None
        if item is not None:
            item[0].close()

    def stats(self, sched: Scheduler) -> dict:
        lat = sched.latency
        if not lat:
            return {"frames": 0}
        first = min(a for _, _, a, _ in lat)
        last = max(d for _, _, _, d in lat)
        res = {}
        for sid, fi, a, d in lat:
            r = self.requests[sid]
            key = f"{r.vid.shape[1]}p"
            res.setdefault(key, []).append(1000 * (d - a))
        all_ms = [1000 * (d - a) for _, _, a, d in lat]
        return {
            "frames": len(lat),
            "wall_s": last - first,
            "frames_per_s": len(lat) / max(last - first, 1e-9),
            "p50_ms": percentile(all_ms, 50), "p99_ms": percentile(all_ms, 99),
            "by_height": {k: {"frames": len(v), "p50_ms": percentile(v, 50),
                              "p99_ms": percentile(v, 99)} for k, v in sorted(res.items())},
            "mean_batch": float(np.mean(self.batch_sizes)) if self.batch_sizes else 0.0,
            "batches": len(self.batch_sizes),
            "batch_gpu_ms_p50": percentile(self.batch_ms, 50),
            "peak_bytes": sched.peak_used, "budget_bytes": sched.budget,
            "reserve_bytes": sched.reserve,
        }
