"""Continuous-batching render server for resident Universal Beta Splatting scenes.

Several scenes stay resident in HBM as their raw parameters.  Render
requests (scene, camera) arrive over time; the loop admits them as batch
slots and intersection-buffer memory free up, batches the waiting requests of
one scene into one fused multi-view launch (views of any mix of
resolutions), runs up to `max_slots` batches at once on separate CUDA streams
so their work overlaps on the device, and releases each request when its
batch's completion event has fired and its image has been copied to pinned
host memory.  Latency is measured from a request's arrival to that point.

The reference renders one view per call (`BetaModel.render`,
scene/beta_model.py:660-722, used by view.py / render.py); `run_plain` serves
the same requests that way -- one request per launch, in arrival order -- as
the comparison form.

Admission needs each batch's intersection count before it runs; it is
estimated from the scene's intersections per pixel seen so far (seeded by one
calibration render per scene) with a safety margin.  A batch whose
intersections exceed its buffer is detected from the device-side count when
it completes and re-run with the measured size before any of its results are
released, so estimates affect memory use and latency, never results.
"""
import time
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib as L
from .render import PARAM_ORDER, STATUS_NEG_DEPTH, Views
from .scene import Camera, orbit_view


@dataclass
class Request:
    rid: int
    scene: str
    camera: Camera
    arrival: float  # seconds from the start of the run


@dataclass
class Done:
    rid: int
    scene: str
    arrival: float
    finish: float
    batch_size: int
    image: Optional[torch.Tensor] = None  # [H, W, 3] pinned host tensor when kept

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


@dataclass
class ServeConfig:
    max_slots: int = 4            # batches in flight at once (one CUDA stream each)
    max_batch_views: int = 8      # views per fused launch
    mem_budget: int = 16 << 30    # bytes of intersection buffers + images in flight
    margin: float = 1.25          # intersection estimate safety factor
    # upper bound on a batch's estimated intersections (None: no bound): a
    # batch's device time grows with its intersections, so under a latency
    # target this keeps one large batch from holding its requests (and those
    # queued behind it) past the target; the first request always goes
    max_batch_isects: Optional[int] = None
    tile_size: int = 16
    keep_images: bool = False     # keep every image (tests); else only latency


def poisson_trace(rate: float, duration: float, scenes: Sequence[str],
                  resolutions: Sequence[tuple], seed: int = 0, radius: float = 4.0,
                  focal_per_width: float = 1500.0 / 1920.0, device="cuda") -> List[Request]:
    """Seeded Poisson arrivals at `rate` per second over `duration` seconds;
    each request picks a scene and a resolution uniformly and a random orbit
    camera looking at the origin (focal length proportional to width)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        sc = scenes[int(rng.integers(len(scenes)))]
        w, h = resolutions[int(rng.integers(len(resolutions)))]
        f = focal_per_width * w
        cam = orbit_view(int(rng.integers(1 << 30)), radius, w, h, f, f, device=device)
        out.append(Request(len(out), sc, cam, t))


# ------------------------------------------------------------------ policy
class Scheduler:
    """Admission and batching policy (host logic only, no device calls).

    `estimate(scene, cams)` returns the expected intersections of a batch;
    `cost(scene, cams, isects)` its device bytes.  Waiting requests are served
    first come first served: the oldest waiting request's scene forms the next
    batch, which takes that scene's waiting requests in arrival order up to
    max_batch_views, max_batch_isects (estimated) and the memory left."""

    def __init__(self, cfg: ServeConfig, estimate: Callable, cost: Callable):
        self.cfg = cfg
        self.estimate = estimate
        self.cost = cost
        self.waiting: List[Request] = []
        self.in_flight_bytes = 0
        self.slots_busy = 0

    def arrive(self, reqs: Sequence[Request]):
        self.waiting.extend(reqs)

    def next_batch(self):
        """A (scene, requests, isect capacity, bytes) batch to launch now, or None."""
        if not self.waiting or self.slots_busy >= self.cfg.max_slots:
            return None
        scene = self.waiting[0].scene
        chosen, cams = [], []
        for r in self.waiting:
            if r.scene != scene:
                continue
            trial = cams + [r.camera]
            est = self.estimate(scene, trial)
            if chosen and self.cfg.max_batch_isects is not None and \
                    est > self.cfg.max_batch_isects:
                break
            cap = int(est * self.cfg.margin) + 4096
            need = self.cost(scene, trial, cap)
            if chosen and self.in_flight_bytes + need > self.cfg.mem_budget:
                break
            if not chosen and self.in_flight_bytes + need > self.cfg.mem_budget and \
                    self.in_flight_bytes > 0:
                return None  # wait for memory to free up
            chosen.append(r)
            cams = trial
            if len(chosen) >= self.cfg.max_batch_views:
                break
        cap = int(self.estimate(scene, cams) * self.cfg.margin) + 4096
        need = self.cost(scene, cams, cap)
        ids = {r.rid for r in chosen}
        self.waiting = [r for r in self.waiting if r.rid not in ids]
        self.in_flight_bytes += need
        self.slots_busy += 1
        return scene, chosen, cap, need

    def release(self, nbytes: int):
        self.in_flight_bytes -= nbytes
        self.slots_busy -= 1


# ------------------------------------------------------------------- device
@dataclass
class _Batch:
    scene: str
    reqs: List[Request]
    cap: int
    nbytes: int
    stream: torch.cuda.Stream
    views: Views = None
    colors: torch.Tensor = None
    host: torch.Tensor = None
    stats: torch.Tensor = None
    ws: torch.Tensor = None
    event: torch.cuda.Event = None
    tries: int = 0


class Server:
    """Continuous-batching server over resident scenes (see module docstring)."""

    def __init__(self, scenes: Dict[str, Dict[str, torch.Tensor]], cfg: ServeConfig = None,
                 device="cuda", eps2d=0.3, near_plane=0.01, far_plane=1e10):
        self.cfg = cfg or ServeConfig()
        self.device = torch.device(device)
        self.scenes = {}
        self.ipp = {}  # intersections per pixel, per scene
        for name, p in scenes.items():
            self.add_scene(name, p)
        self.eps2d, self.near, self.far = eps2d, near_plane, far_plane
        self.streams = [torch.cuda.Stream(self.device) for _ in range(self.cfg.max_slots)]
        self.free_streams = list(range(self.cfg.max_slots))
        self.bg = torch.zeros(self.cfg.max_batch_views, 3, device=self.device)
        self.reruns = 0

    # scenes -------------------------------------------------------------
    def add_scene(self, name: str, params: Dict[str, torch.Tensor]):
        """Make a scene resident: raw parameter tensors under the reference's
        names (xyz, mean, scale, l_triangle, opacity, beta, rgb)."""
        q = {k: params[k].detach().to(self.device, torch.float32).contiguous()
             for k in PARAM_ORDER}
        q["opacity"] = q["opacity"].reshape(-1)
        self.scenes[name] = q
        self.ipp.pop(name, None)  # a new scene is calibrated afresh

    def load_scene(self, name: str, path: str):
        """Make the scene of a reference PLY file resident (scene/beta_model.py:
        322-404's format; the vertex records go to the device as they are and
        are unpacked there, ubs.ply.load_ply)."""
        from .ply import load_ply
        self.add_scene(name, load_ply(path, self.device))

    # sizes --------------------------------------------------------------
    def _dim(self, scene):
        return self.scenes[scene]["scale"].shape[1]

    def estimate(self, scene, cams):
        return self.ipp.get(scene, 8.0) * sum(c.width * c.height for c in cams)

    def _n_buckets(self, cams):
        ts = self.cfg.tile_size
        return sum(((c.width + ts - 1) // ts) * ((c.height + ts - 1) // ts) for c in cams)

    def cost(self, scene, cams, cap):
        N = self.scenes[scene]["xyz"].shape[0]
        ws = L.query("ubs_scene_workspace_bytes", len(cams), N, self._n_buckets(cams), cap)
        return int(ws) + sum(c.width * c.height for c in cams) * 20

    # launching ------------------------------------------------------------
    def _launch(self, b: _Batch):
        p = self.scenes[b.scene]
        cams = [r.camera for r in b.reqs]
        C = len(cams)
        with torch.cuda.stream(b.stream):
            b.views = Views(cams, tile_size=self.cfg.tile_size, device=self.device,
                            stream=b.stream)
            P = b.views.n_pixels
            N = p["xyz"].shape[0]
            b.ws = L.workspace(L.query("ubs_scene_workspace_bytes", C, N, b.views.n_buckets,
                                       b.cap), self.device)
            b.colors = torch.empty(P, 3, device=self.device)
            alphas = torch.empty(P, device=self.device)
            last = torch.empty(P, dtype=torch.int32, device=self.device)
            bg = self.bg[:C]
            L.call("ubs_scene_forward", self._dim(b.scene), N, *[L.ptr(p[k]) for k in PARAM_ORDER],
                   C, L.ptr(b.views.viewmats), L.ptr(b.views.intr), L.ptr(b.views.centers),
                   L.ptr(b.views.times), L.ptr(b.views.dims), L.ptr(b.views.tile_base),
                   L.ptr(b.views.pix_base), b.views.n_buckets, self.cfg.tile_size,
                   float(self.eps2d), float(self.near), float(self.far), 0.0, L.ptr(bg),
                   L.ptr(b.colors), L.ptr(alphas), L.ptr(last), b.cap, L.ptr(b.ws),
                   b.ws.numel(), L.stream_ptr(b.stream))
            b.stats = torch.empty(2, dtype=torch.int64, pin_memory=True)
            b.stats.copy_(b.ws[:16].view(torch.int64), non_blocking=True)
            b.host = torch.empty(P, 3, pin_memory=True)
            b.host.copy_(b.colors, non_blocking=True)
            b.event = torch.cuda.Event()
            b.event.record(b.stream)
        b.tries += 1

    def _finish(self, b: _Batch, now: float, out: List[Done]):
        T, status = int(b.stats[0]), int(b.stats[1]) & 0xffffffff
        if status & STATUS_NEG_DEPTH:
            raise RuntimeError("serve: a visible primitive has a negative depth")
        pixels = sum(r.camera.width * r.camera.height for r in b.reqs)
        # running maximum: views of one scene differ a lot in intersections per
        # pixel, and an underestimate costs a re-run
        self.ipp[b.scene] = max(self.ipp.get(b.scene, 0.0), T / pixels)
        if T > b.cap:  # overflow: re-run with the measured size before releasing anything
            self.reruns += 1
            b.cap = int(T * 1.1) + 4096
            self._launch(b)
            return False
        imgs = b.views.split(b.host) if self.cfg.keep_images else [None] * len(b.reqs)
        for r, im in zip(b.reqs, imgs):
            out.append(Done(r.rid, r.scene, r.arrival, now, len(b.reqs), im))
        return True

    def calibrate(self, cams_per_scene: Dict[str, Camera]):
        """One render per scene to seed its intersections-per-pixel estimate."""
        for name, cam in cams_per_scene.items():
            b = _Batch(name, [Request(-1, name, cam, 0.0)], int(64 * cam.width * cam.height), 0,
                       self.streams[0])
            self._launch(b)
            b.event.synchronize()
            self._finish(b, 0.0, [])

    # the loop ---------------------------------------------------------------
    def run(self, trace: Sequence[Request], realtime: bool = True) -> List[Done]:
        """Serve `trace`; with realtime=False every request is available at
        time 0 (saturation throughput).  Returns completions in finish order."""
        sched = Scheduler(self.cfg, self.estimate, self.cost)
        pending = sorted(trace, key=lambda r: r.arrival)
        i = 0
        running: List[_Batch] = []
        done: List[Done] = []
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        while i < len(pending) or sched.waiting or running:
            now = time.perf_counter() - t0
            new = []
            while i < len(pending) and (not realtime or pending[i].arrival <= now):
                r = pending[i]
                new.append(r if realtime else Request(r.rid, r.scene, r.camera, 0.0))
                i += 1
            sched.arrive(new)
            # completions
            still = []
            for b in running:
                if b.event.query():
                    if self._finish(b, time.perf_counter() - t0, done):
                        sched.release(b.nbytes)
                        self.free_streams.append(self.streams.index(b.stream))
                        b.ws = b.colors = None
                        continue
                still.append(b)
            running = still
            # admissions
            while True:
                nb = sched.next_batch()
                if nb is None:
                    break
                scene, reqs, cap, nbytes = nb
                st = self.streams[self.free_streams.pop()]
                b = _Batch(scene, reqs, cap, nbytes, st)
                self._launch(b)
                running.append(b)
            if not running and not sched.waiting and i < len(pending) and realtime:
                # idle until the next arrival
                wait = pending[i].arrival - (time.perf_counter() - t0)
                if wait > 2e-4:
                    time.sleep(wait - 1e-4)
        return done


def run_plain(render_one: Callable[[Request], torch.Tensor], trace: Sequence[Request],
              realtime: bool = True) -> List[Done]:
    """One request per launch in arrival order: wait for the request, render
    it with `render_one` (returns the device image), copy the image to pinned
    host memory and synchronise before taking the next one."""
    pending = sorted(trace, key=lambda r: r.arrival)
    done = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in pending:
        arrival = r.arrival if realtime else 0.0
        now = time.perf_counter() - t0
        if realtime and arrival > now:
            time.sleep(arrival - now)
        img = render_one(r)
        host = torch.empty(img.shape, pin_memory=True)
        host.copy_(img, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        done.append(Done(r.rid, r.scene, arrival, time.perf_counter() - t0, 1))
    return done


def latency_stats(done: Sequence[Done], makespan: Optional[float] = None) -> dict:
    lat = np.array([d.latency for d in done]) * 1e3
    span = makespan if makespan is not None else max(d.finish for d in done)
    return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "frames_per_s": len(done) / span if span > 0 else None,
            "mean_batch": float(np.mean([d.batch_size for d in done]))}
