"""Render serving with continuous batching.

Scenes stay resident on the device.  Render requests (scene, camera, image
size) arrive at any time.  The server keeps up to ``slots`` batches in flight,
each on its own CUDA stream; whenever a slot is free it admits the oldest
waiting requests -- as many as fit under ``max_views`` and under the part of
the device-memory budget that the resident scenes and the batches in flight
leave -- plans them as ONE batch (one launch per stage over all their views,
any mix of scenes and image sizes, see ``batch.BatchPipeline``) and enqueues it
without waiting.  ``poll()`` retires the batches whose completion event has
fired: their memory reservation is released, their requests get their images
and latencies, and new requests are admitted into the freed slot.  Batches on
different streams overlap on the device.

Each batch's key buffer is sized from running estimates of keys per Gaussian,
one per (scene, image size), with a safety margin; every retired batch scales
the estimates of its views by its actual key total over the estimated one.
The binning's 16-byte status block is copied back asynchronously
with the batch and decoded when the batch retires; a batch whose keys did not
fit is re-run with the exact capacity before any of its images is published.

A served image is the same as rendering that request alone with the same tile
shape: the batch renders every view from the per-view tile lists with the
per-view arithmetic, so neither batch composition nor overlap changes a bit.

Memory accounting: a batch reserves its per-item buffers (projection outputs,
rectangles, counts: 52 bytes per (view, Gaussian) item), the binning
workspace and key list for its key capacity, its start/end arrays and its
images, until it retires.  Images handed to requests are the caller's.
"""
from __future__ import annotations

import collections
import ctypes
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._torch import ptr
from .batch import BatchPipeline, Scene, ViewSpec
from .camera import CameraInfo, look_at_c2w
from .renderer import RasterSettings

ITEM_BYTES = 8 + 16 + 4 + 4 + 16 + 4  # mean2d, cov2d, depth, alpha, rect, counts
MIN_KEYS = 1 << 16


@dataclass(eq=False)
class Request:
    scene: int
    c2w: np.ndarray
    cam: CameraInfo
    t_arrival: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    state: str = "new"      # waiting | running | done | cancelled | rejected
    image: torch.Tensor | None = None  # [h, w, 3] on the device once done
    rid: int = -1
    batch_id: int = -1
    error: str = ""

    @property
    def latency_ms(self) -> float:
        return (self.t_done - self.t_arrival) * 1e3


@dataclass(eq=False)
class _Batch:
    bid: int
    requests: list
    pipe: BatchPipeline
    stream: torch.cuda.Stream
    event: torch.cuda.Event
    status: torch.Tensor   # pinned 16-byte status block of the binning
    reserved: int
    t_launch: float


def select_batch(waiting, sh_order_of, max_views: int, avail_bytes: int, batch_bytes) -> list[int]:
    """Indices (into `waiting`, oldest first) of the next batch: requests in
    arrival order that share the oldest request's SH order, at most
    `max_views` of them, stopping at the first one that would take the batch
    over `avail_bytes` (so no request is overtaken by a later one of the same
    SH order).  Empty when even the oldest request does not fit."""
    if not waiting:
        return []
    C = sh_order_of(waiting[0])
    batch, taken = [], []
    for i, r in enumerate(waiting):
        if len(taken) == max_views:
            break
        if sh_order_of(r) != C:  # one SH order per batch; the others wait their turn
            continue
        if batch_bytes(batch + [r]) > avail_bytes:
            break
        batch.append(r)
        taken.append(i)
    return taken


class RenderServer:
    """Continuous-batching render loop over resident scenes (forward only)."""

    def __init__(self, scenes: list[Scene], device=None, budget_bytes: float = 150e9, max_views: int = 16,
                 slots: int = 2, settings: RasterSettings | None = None, keys_per_gaussian: float = 4.0,
                 retain_images: bool = True):
        if slots < 1 or max_views < 1:
            raise ValueError("slots and max_views must be positive")
        self.device = torch.device(device or "cuda")
        self.scenes = list(scenes)
        self.settings = settings or RasterSettings()
        self.budget = int(budget_bytes)
        self.resident = sum(self._scene_bytes(s) for s in self.scenes)
        if self.resident > self.budget:
            raise ValueError(f"the resident scenes ({self.resident} bytes) exceed the memory budget")
        self.sh_orders = [int(round(s.sh.shape[-1] ** 0.5)) if self.settings.sh_order is None
                          else self.settings.sh_order for s in self.scenes]
        self.max_views = max_views
        self.slots = slots
        self.retain_images = retain_images
        self.default_kpg = float(keys_per_gaussian)
        self.keys_per_gaussian: dict[tuple, float] = {}  # (scene, w, h) -> keys per Gaussian
        self.margin = 1.5
        self.waiting: collections.deque[Request] = collections.deque()
        self.in_flight: list[_Batch] = []
        self.reserved = 0
        self.peak_reserved = 0
        self.completed: list[Request] = []
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.n_batches = 0
        self.n_reruns = 0
        self.host_launch_s = 0.0  # host time spent planning and enqueueing batches
        self.batch_sizes: list[int] = []
        self._next_rid = 0
        self._lib = _lib.load()

    # ---------------------------------------------------------------- scenes
    @staticmethod
    def _scene_bytes(s: Scene) -> int:
        return sum(t.numel() * t.element_size() for t in (s.mean, s.qvec, s.log_scale, s.sh, s.alpha_logit))

    def add_scene(self, scene: Scene | str) -> int:
        """Make a scene resident (a Scene or the path of an SHRenderer
        checkpoint); returns its index.  Refused when it does not fit the
        memory budget next to the resident scenes and the batches in flight."""
        if not isinstance(scene, Scene):
            scene = Scene.from_checkpoint(scene, self.device)
        need = self._scene_bytes(scene)
        if self.resident + self.reserved + need > self.budget:
            raise MemoryError(f"scene of {need} bytes does not fit the memory budget")
        self.resident += need
        C = int(round(scene.sh.shape[-1] ** 0.5)) if self.settings.sh_order is None else self.settings.sh_order
        for i, s in enumerate(self.scenes):  # reuse a freed slot
            if s is None:
                self.scenes[i] = scene
                self.sh_orders[i] = C
                return i
        self.scenes.append(scene)
        self.sh_orders.append(C)
        return len(self.scenes) - 1

    def remove_scene(self, index: int) -> None:
        """Release a resident scene that no waiting or running request uses."""
        s = self.scenes[index]
        if s is None:
            raise IndexError(f"scene {index} is not resident")
        busy = any(r.scene == index for r in self.waiting) or any(
            r.scene == index for b in self.in_flight for r in b.requests)
        if busy:
            raise RuntimeError(f"scene {index} has requests waiting or in flight")
        self.resident -= self._scene_bytes(s)
        self.scenes[index] = None
        for key in [k for k in self.keys_per_gaussian if k[0] == index]:
            del self.keys_per_gaussian[key]

    # -------------------------------------------------------------- requests
    def submit(self, scene: int, c2w, cam: CameraInfo, t_arrival: float | None = None) -> Request:
        if not 0 <= scene < len(self.scenes) or self.scenes[scene] is None:
            raise IndexError(f"scene {scene} is not resident")
        req = Request(scene, np.asarray(c2w, np.float32), cam)
        req.rid = self._next_rid
        self._next_rid += 1
        req.t_arrival = time.perf_counter() if t_arrival is None else t_arrival
        if self._batch_bytes([req]) + self.resident > self.budget:
            req.state, req.error = "rejected", "request alone exceeds the memory budget"
            return req
        req.state = "waiting"
        self.waiting.append(req)
        return req

    def cancel(self, req: Request) -> bool:
        """Withdraw a request that has not been admitted yet."""
        if req.state != "waiting":
            return False
        self.waiting.remove(req)
        req.state = "cancelled"
        return True

    # ------------------------------------------------------------- admission
    def _tiles(self, cam: CameraInfo) -> int:
        ntw, nth = self.settings.tiles(cam)
        return ntw * nth

    def _kpg(self, r: Request) -> float:
        return self.keys_per_gaussian.get((r.scene, r.cam.w, r.cam.h), self.default_kpg)

    def _estimated_keys(self, reqs) -> float:
        return sum(self.scenes[r.scene].n * self._kpg(r) for r in reqs)

    def _key_capacity(self, reqs) -> int:
        return max(int(self._estimated_keys(reqs) * self.margin) + 4096, MIN_KEYS)

    def _correct_estimates(self, reqs, total: int, exact: bool):
        """Scale the views' estimates by actual/estimated keys of their batch
        (fully after an overflow, a quarter of the way otherwise)."""
        est = self._estimated_keys(reqs)
        ratio = total / max(est, 1.0)
        f = ratio if exact else 0.75 + 0.25 * ratio
        for key in {(r.scene, r.cam.w, r.cam.h) for r in reqs}:
            self.keys_per_gaussian[key] = self.keys_per_gaussian.get(key, self.default_kpg) * f

    def _batch_bytes(self, reqs, cap: int | None = None) -> int:
        items = sum(self.scenes[r.scene].n for r in reqs)
        tiles = sum(self._tiles(r.cam) for r in reqs)
        pixels = sum(r.cam.w * r.cam.h for r in reqs)
        cap = self._key_capacity(reqs) if cap is None else cap
        ws = int(self._lib.gsx_binning_workspace_bytes(items, cap, tiles))
        return items * ITEM_BYTES + ws + 4 * cap + 8 * tiles + 12 * pixels + 512 * len(reqs)

    def _free_stream(self):
        busy = {id(b.stream) for b in self.in_flight}
        return next(s for s in self.streams if id(s) not in busy)

    def _admit(self):
        while len(self.in_flight) < self.slots and self.waiting:
            taken = select_batch(self.waiting, lambda r: self.sh_orders[r.scene], self.max_views,
                                 self.budget - self.resident - self.reserved, self._batch_bytes)
            if not taken:
                return  # memory frees up when a batch retires
            batch = [self.waiting[i] for i in taken]
            for i in reversed(taken):
                del self.waiting[i]
            self._launch(batch)

    def _launch(self, reqs, cap: int | None = None):
        cap = self._key_capacity(reqs) if cap is None else cap
        need = self._batch_bytes(reqs, cap)
        stream = self._free_stream()
        now = time.perf_counter()
        for r in reqs:
            r.state, r.t_admit, r.batch_id = "running", now, self.n_batches
        pipe = BatchPipeline(self.device, self.settings)
        pipe.key_capacity = cap
        status = torch.zeros(16, dtype=torch.uint8, pin_memory=True)
        with torch.cuda.stream(stream):
            pipe.plan(self.scenes, [ViewSpec(r.scene, r.c2w, r.cam) for r in reqs], backward=False,
                      sh_order=self.sh_orders[reqs[0].scene])
            pipe.forward_async()
            _lib.check(self._lib.gsx_binning_status_copy_async(ptr(pipe.ws), pipe.n_items, pipe.key_capacity,
                                                               status.data_ptr(), stream.cuda_stream),
                       "gsx_binning_status_copy_async")
            event = torch.cuda.Event()
            event.record(stream)
        self.reserved += need
        self.peak_reserved = max(self.peak_reserved, self.reserved)
        self.in_flight.append(_Batch(self.n_batches, reqs, pipe, stream, event, status, need, now))
        self.host_launch_s += time.perf_counter() - now
        self.n_batches += 1
        self.batch_sizes.append(len(reqs))

    # ----------------------------------------------------------- retirement
    def _retire(self) -> list[Request]:
        done, rerun, still = [], [], []
        for b in self.in_flight:
            if not b.event.query():
                still.append(b)
                continue
            self.reserved -= b.reserved
            k = ctypes.c_int64(0)
            st = self._lib.gsx_binning_status_decode(b.status.data_ptr(), b.pipe.key_capacity, 0, 0,
                                                     ctypes.byref(k))
            total = int(k.value)
            if st == _lib.GSX_ERR_CAPACITY:
                self._correct_estimates(b.requests, total, exact=True)
                rerun.append((b.requests, total + total // 8 + 4096))
                continue
            _lib.check(st, "batched binning")
            self._correct_estimates(b.requests, total, exact=False)
            now = time.perf_counter()
            for r, img in zip(b.requests, b.pipe.images):
                r.image = img if self.retain_images else None
                r.t_done = now
                r.state = "done"
                done.append(r)
        self.in_flight = still
        for reqs, cap in rerun:
            self.n_reruns += 1
            self._launch(reqs, cap)
        self.completed.extend(done)
        return done

    def poll(self) -> list[Request]:
        """Retire finished batches, admit waiting requests; returns the
        requests completed by this call."""
        done = self._retire()
        self._admit()
        return done

    def drain(self):
        while self.waiting or self.in_flight:
            self.poll()

    @property
    def idle(self) -> bool:
        return not self.waiting and not self.in_flight


# ------------------------------------------------------------------ workload
def serving_scenes(device, n_scenes: int = 8, lo: int = 100_000, hi: int = 2_000_000,
                   sh_degree: int = 0) -> list[Scene]:
    """Resident scenes of the serving workload: Gaussian counts log-uniform in
    [lo, hi] (seeded), scene i drawn as in the small workload with seed i."""
    from . import scene as S

    u = S.uniform(1234, 0, n_scenes)
    counts = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo))).astype(np.int64)
    out = []
    for i, n in enumerate(counts):
        sc = S.make_scene(int(n), i, mean_dist="uniform", log_scale_mu=-3.0, log_scale_sigma=0.5,
                          alpha_sigma=1.0, sh_degree=sh_degree, dc_from_rgb=True)
        out.append(Scene.from_arrays(sc, device))
    return out


def poisson_requests(n_scenes: int, rate: float, duration: float, seed: int = 0,
                     sizes=((512, 512), (1280, 720), (1920, 1080)), fov: float = 60.0):
    """(arrival offset in s, scene, c2w, camera) of a Poisson stream: uniform
    scene, camera uniform on the sphere of radius U[5, 10] looking at the
    origin, image size uniform over `sizes`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cams = [CameraInfo.from_vertical_fov(fov, w, h) for w, h in sizes]
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = rng.uniform(5.0, 10.0)
        out.append((t, int(rng.integers(n_scenes)), look_at_c2w(r * d), cams[int(rng.integers(len(cams)))]))
    return out


def run_stream(server: RenderServer, arrivals, realtime: bool = True, on_done=None):
    """Submit (offset, scene, c2w, cam) arrivals at their times (or all at
    once when realtime is False) and serve until every request is done.
    Returns (requests, wall seconds from the first arrival to the last
    completion)."""
    t0 = time.perf_counter()
    reqs = []
    i, n = 0, len(arrivals)
    while i < n or not server.idle:
        now = time.perf_counter()
        while i < n and (not realtime or t0 + arrivals[i][0] <= now):
            off, scene, c2w, cam = arrivals[i]
            reqs.append(server.submit(scene, c2w, cam, t_arrival=(t0 + off) if realtime else now))
            i += 1
        done = server.poll()
        if on_done is not None:
            for r in done:
                on_done(r)
    torch.cuda.synchronize(server.device)
    t_first = min(r.t_arrival for r in reqs) if reqs else t0
    t_last = max((r.t_done for r in reqs if r.state == "done"), default=t0)
    return reqs, t_last - t_first


def latency_stats(reqs) -> dict:
    lat = np.array([r.latency_ms for r in reqs if r.state == "done"])
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None, "max_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max())}
