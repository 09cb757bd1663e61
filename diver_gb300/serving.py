"""Multi-scene render serving with continuous batching.

Several scenes stay resident on the device (feature grid, occupancy, decoder
weights).  Render requests (scene id, camera, resolution) arrive over time;
the server admits a request when its scene is resident (loading it if the
HBM budget allows, evicting idle scenes least-recently-used first) and when
ray slots are free, splits it into ray chunks, and at every step batches the
pending chunks of all admitted requests: one batch per scene, launched on that
scene's stream, so batches of different scenes overlap on the device.  A
request that arrives while others are in flight joins at the next step.

Each ray's result depends only on that ray's own segments (per-segment decode,
per-ray compositing), so a request renders to the same values alone or in any
mix of other requests.

The scheduler (`Scheduler`) is plain Python and independent of the renderer;
`GpuRenderer` runs the CUDA path (traversal, tensor-core or FP32 decoder,
compositing).
"""
from __future__ import annotations

import heapq
import itertools
import time
from collections import OrderedDict, deque
from dataclasses import dataclass, field

import torch

from .ray_voxel_intersection import PendingSegments


@dataclass
class Request:
    rid: int
    scene: str
    c2w: torch.Tensor          # 3x4 camera-to-world
    height: int
    width: int
    focal: float
    arrival: float = 0.0       # seconds (relative to the run's start)
    # filled by the server
    admitted: float | None = None
    done: float | None = None
    rgb: torch.Tensor | None = None
    next_ray: int = 0
    pending_chunks: int = 0

    @property
    def rays(self) -> int:
        return self.height * self.width

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


@dataclass
class SceneEntry:
    name: str
    nbytes: int
    loader: object               # callable() -> resident scene object
    resident: object | None = None
    active: int = 0              # admitted requests using it


class Residency:
    """HBM-budgeted scene residency with LRU eviction of idle scenes.
    `reserved_bytes` of the budget are set aside for the working memory of
    the batches in flight (segment lists, decoder outputs); scenes are charged
    the bytes given at registration (their grids, any 16-bit copy of the grid
    the renderer makes, occupancy and weights) against the rest."""

    def __init__(self, budget_bytes: int, reserved_bytes: int = 0):
        self.budget = int(budget_bytes)
        self.reserved = int(reserved_bytes)
        if self.reserved >= self.budget:
            raise ValueError("the reserved working memory leaves no HBM budget for scenes")
        self.scenes: dict[str, SceneEntry] = {}
        self.lru: OrderedDict[str, None] = OrderedDict()
        self.used = 0

    @property
    def scene_budget(self) -> int:
        return self.budget - self.reserved

    def register(self, name: str, nbytes: int, loader) -> None:
        if nbytes > self.scene_budget:
            raise ValueError(f"scene {name} ({nbytes} B) exceeds the HBM budget for scenes ({self.scene_budget} B)")
        self.scenes[name] = SceneEntry(name, int(nbytes), loader)

    def acquire(self, name: str) -> bool:
        """Makes `name` resident (evicting idle scenes if needed); False if it cannot fit now."""
        e = self.scenes[name]
        if e.resident is None:
            need = self.used + e.nbytes - self.scene_budget
            if need > 0:
                victims = [n for n in self.lru if self.scenes[n].active == 0 and self.scenes[n].resident is not None]
                freed = 0
                chosen = []
                for n in victims:
                    if freed >= need:
                        break
                    chosen.append(n)
                    freed += self.scenes[n].nbytes
                if freed < need:
                    return False
                for n in chosen:
                    self.evict(n)
            e.resident = e.loader()
            self.used += e.nbytes
        e.active += 1
        self.lru.pop(name, None)
        self.lru[name] = None
        return True

    def release(self, name: str) -> None:
        self.scenes[name].active -= 1

    def evict(self, name: str) -> None:
        e = self.scenes[name]
        if e.resident is not None:
            e.resident = None
            self.used -= e.nbytes
            self.lru.pop(name, None)


@dataclass(order=True)
class _Arrival:
    t: float
    seq: int
    req: Request = field(compare=False)


class Scheduler:
    """Continuous batching: admission by ray slots and scene residency,
    chunked work, one batch per scene per step."""

    def __init__(self, residency: Residency, max_rays_in_flight: int = 1 << 22, chunk_rays: int = 1 << 18):
        self.res = residency
        self.max_rays = int(max_rays_in_flight)
        self.chunk = int(chunk_rays)
        self.arrivals: list[_Arrival] = []
        self.waiting: deque[Request] = deque()
        self.active: list[Request] = []
        self.finished: list[Request] = []
        self._seq = itertools.count()

    def submit(self, req: Request) -> None:
        heapq.heappush(self.arrivals, _Arrival(req.arrival, next(self._seq), req))

    def _in_flight(self) -> int:
        return sum(r.rays for r in self.active)

    def admit(self, now: float) -> None:
        while self.arrivals and self.arrivals[0].t <= now:
            self.waiting.append(heapq.heappop(self.arrivals).req)
        still = deque()
        while self.waiting:
            r = self.waiting.popleft()
            if self._in_flight() + r.rays > self.max_rays and self.active:
                still.append(r)
                continue
            if not self.res.acquire(r.scene):
                still.append(r)
                continue
            r.admitted = now
            self.active.append(r)
        self.waiting = still

    def next_batches(self) -> dict[str, list[tuple[Request, int, int]]]:
        """{scene: [(request, first ray, ray count), ...]}: one chunk of every active request."""
        out: dict[str, list] = {}
        for r in self.active:
            if r.next_ray < r.rays:
                n = min(self.chunk, r.rays - r.next_ray)
                out.setdefault(r.scene, []).append((r, r.next_ray, n))
                r.next_ray += n
                r.pending_chunks += 1
        return out

    def chunk_done(self, r: Request, now: float) -> None:
        r.pending_chunks -= 1
        if r.next_ray >= r.rays and r.pending_chunks == 0 and r.done is None:
            r.done = now
            self.active.remove(r)
            self.finished.append(r)
            self.res.release(r.scene)

    def idle(self) -> bool:
        return not (self.arrivals or self.waiting or self.active)

    def next_arrival(self) -> float | None:
        return self.arrivals[0].t if self.arrivals else None


class GpuRenderer:
    """Renders batches of rays of one resident scene on that scene's stream."""

    def __init__(self, form: str = "bf16"):
        self.form = form
        self.streams: dict[str, torch.cuda.Stream] = {}

    def stream(self, scene: str) -> torch.cuda.Stream:
        if scene not in self.streams:
            self.streams[scene] = torch.cuda.Stream()
        return self.streams[scene]

    @staticmethod
    def rays_for(req: Request, first: int, count: int, device):
        """The chunk's camera rays, generated on the device for its pixels only."""
        from .scenes import camera_rays_device

        return camera_rays_device(req.c2w, req.height, req.width, req.focal, device, first, count)

    def render(self, field_model, work: list[tuple[Request, int, int]]):
        """Launches one batch for all chunks in `work` on the scene's stream; returns
        (event, [(request, first, count)])."""
        return self.render_many([(field_model, work)])[0]

    def render_many(self, batches) -> list:
        """Launches one batch per scene ([(model, work), ...]), each on its scene's
        stream, in two passes: first every batch's rays and traversal count walk,
        then, scene by scene, the total's host read, the emission walk, decode and
        compositing.  The count walks (one warp per SM each) of all scenes run
        together, and the host reads a total only once its walk has had the time
        of the others' launches.  Returns [(event, [(request, first, count)])]."""
        began = []
        for field_model, work in batches:
            dev = field_model.voxels.device
            st = self.stream(work[0][0].scene)
            with torch.cuda.stream(st):
                os_, ds_ = zip(*(self.rays_for(r, a, n, dev) for r, a, n in work))
                o = torch.cat(os_)
                d = torch.cat(ds_)
                began.append((field_model, work, st, o, d, field_model.begin_segments(o, d)))
        out = []
        for field_model, work, st, o, d, pending in began:
            dev = field_model.voxels.device
            with torch.cuda.stream(st):
                seg = pending.finish() if isinstance(pending, PendingSegments) else pending
                with torch.no_grad():
                    rgb, _ = field_model(o, d, form=self.form, segments=seg)
                done = []
                k = 0
                for r, a, n in work:
                    if r.rgb is None:
                        r.rgb = torch.empty(r.rays, 3, device=dev)
                    r.rgb[a:a + n].copy_(rgb[k:k + n])
                    done.append((r, a, n))
                    k += n
                ev = torch.cuda.Event()
                ev.record(st)
            out.append((ev, done))
        return out


def serve(requests: list[Request], residency: Residency, renderer: GpuRenderer, realtime: bool = True,
          max_rays_in_flight: int = 1 << 22, chunk_rays: int = 1 << 18) -> list[Request]:
    """Runs the request stream to completion.  With `realtime`, arrival times are
    honoured against the wall clock; otherwise all requests are available at once
    (in arrival order).  Returns the finished requests with their latencies."""
    sch = Scheduler(residency, max_rays_in_flight, chunk_rays)
    for r in requests:
        sch.submit(r)
    t0 = time.perf_counter()
    inflight: list[tuple[torch.cuda.Event, list]] = []
    while not sch.idle():
        now = time.perf_counter() - t0 if realtime else float("inf")
        sch.admit(now)
        if not sch.active and sch.waiting and not inflight:
            # with nothing running, admission only fails when the scene cannot fit the budget
            raise RuntimeError("requests cannot be admitted: scene larger than the free HBM budget")
        batches = sch.next_batches()
        if batches:
            items = [(residency.scenes[scene].resident, work) for scene, work in batches.items()]
            many = getattr(renderer, "render_many", None)  # one pass over all scenes when the renderer has it
            inflight.extend(many(items) if many else [renderer.render(m, w) for m, w in items])
        # retire finished batches (poll; block only if nothing else can progress)
        if not batches and inflight:
            inflight[0][0].synchronize()
        still = []
        for ev, out in inflight:
            if ev.query():
                t = time.perf_counter() - t0
                for r, a, n in out:
                    sch.chunk_done(r, t)
            else:
                still.append((ev, out))
        inflight = still
        if realtime and not batches and not inflight:
            nxt = sch.next_arrival()
            if nxt is not None:
                time.sleep(max(0.0, min(nxt - (time.perf_counter() - t0), 0.01)))
    return sch.finished


def latency_summary(done: list[Request]) -> dict:
    lat = sorted(r.latency for r in done if r.latency is not None)
    if not lat:
        return {"requests": 0}

    def pct(p):
        return lat[min(len(lat) - 1, int(round(p * (len(lat) - 1))))] * 1e3

    rays = sum(r.rays for r in done)
    span = max(r.done for r in done) - min(r.arrival for r in done)
    return {"requests": len(lat), "p50_ms": pct(0.5), "p99_ms": pct(0.99), "rays": rays,
            "Mrays_per_s": rays / span / 1e6 if span > 0 else None}
