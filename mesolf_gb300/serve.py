"""Serving loop for streams of light-field frames (patches of a carpet arriving at a frame
rate), on top of the batched tensor-core solve.

A request is one patch of one frame.  The server keeps, resident in HBM, the phase-space
PSF (its taps and tensor-core tables), one work set per lane sized once for ALL patches of
the carpet (every patch owns fixed lenslet positions -- a slot -- in it), and one volume per
patch: the previous frame's reconstruction, which warm-starts the next frame of that patch
(the reference's ``Xguess`` initial value, ``recon_theory_phase_space_LFM_with_filter.m:72-73``,
replaced by the last result).  Everything is allocated when the server starts; nothing is
allocated on the request path.

* Continuous batching.  ``lanes`` worker threads each own a CUDA stream and a work set.
  Whenever a lane is free it takes every patch whose oldest pending frame is ready (the
  patch is not on the GPU in another lane), oldest arrival first, up to ``max_batch``
  patches, and runs them as one batch: the lane's work set with the other patches left out
  (``BatchSolver.run`` with ``None`` images: their weights are 0 for the run, so their tiles
  are skipped).  Requests that arrive while other batches are on the GPU join the next batch
  a lane forms, so the lanes' batches overlap on the device.
* Admission by free HBM, once: the server starts only if one work set plus the per-patch
  volumes fit in the free device memory minus ``reserve_bytes``, and opens as many of the
  requested lanes as fit.
* ``drop_stale``: when a patch has several frames waiting, a lane takes the newest and
  completes the older ones with :class:`FrameDropped` (a live display wants the latest
  volume; an overloaded stream then stays bounded instead of queueing without end).
* Cancellation: :meth:`SolveServer.cancel` withdraws a queued request at once; a request
  already on the GPU is withdrawn when its batch ends, and if every request of that batch
  is withdrawn the batch itself is stopped between view steps (``BatchSolver.cancel``),
  leaving each patch's warm-start volume at the previous frame.
* Latency is measured from the request's arrival time to the moment its volume is in host
  memory; :meth:`SolveServer.report` gives p50 / p99 and the deconvolved voxels/s.

The result of a request is identical whether it is solved alone or in a mix: each patch
occupies its own lenslet positions of the work set, its view weights, plane range and
filter are its own, and a view that is active only for other patches leaves it unchanged
(weight 0 keeps ``X`` bit for bit).
"""
from __future__ import annotations

import collections
import concurrent.futures
import dataclasses
import threading
import time

import numpy as np

__all__ = ["Request", "Scheduler", "SolveServer", "FrameDropped"]


class FrameDropped(Exception):
    """A frame superseded by a newer frame of the same patch before it was solved
    (``SolveServer(drop_stale=True)``)."""


@dataclasses.dataclass
class Request:
    patch: int
    frame: int
    lf: object                     # host (Xr, Xc) float32 image
    t_arrival: float               # time.perf_counter() seconds
    future: concurrent.futures.Future = dataclasses.field(default_factory=concurrent.futures.Future)
    t_done: float = 0.0
    withdrawn: bool = False        # cancelled while on the GPU


class Scheduler:
    """Batching and admission decisions; no device work (unit-testable on the CPU).

    ``plan_bytes(patches)`` gives the device bytes a new work set for that composition
    needs; ``free_bytes()`` the device memory free now; ``evict()`` frees one idle cached
    work set and returns True, or returns False when there is none.  (The slot-based
    SolveServer allocates its work sets up front and passes hooks under which every batch
    fits.)  ``drop_stale``: a picked patch with several pending frames takes its newest;
    the older ones are moved to ``dropped`` for the caller to complete.
    """

    def __init__(self, n_patches, max_batch, plan_bytes, free_bytes, evict, reserve_bytes=0, drop_stale=False):
        self.queues = [collections.deque() for _ in range(n_patches)]
        self.last_frame = [None] * n_patches
        self.busy = set()
        self.max_batch = max(1, int(max_batch))
        self.plan_bytes = plan_bytes
        self.free_bytes = free_bytes
        self.evict = evict
        self.reserve = int(reserve_bytes)
        self.drop_stale = drop_stale
        self.dropped = []

    def add(self, req: Request):
        last = self.last_frame[req.patch]
        if last is not None and last >= req.frame:
            raise ValueError(f"patch {req.patch}: frame {req.frame} after frame {last}")
        self.last_frame[req.patch] = req.frame
        self.queues[req.patch].append(req)

    def remove(self, patch, frame):
        """Take a pending request out of its queue; returns it, or None if not queued."""
        q = self.queues[patch]
        for r in q:
            if r.frame == frame:
                q.remove(r)
                return r
        return None

    def pending(self):
        return sum(len(q) for q in self.queues)

    def ready(self):
        """Patches with a pending frame and not on the GPU, oldest head first."""
        r = [p for p, q in enumerate(self.queues) if q and p not in self.busy]
        r.sort(key=lambda p: (self.queues[p][0].t_arrival, p))
        return r

    def pick(self, cached):
        """Requests of the next batch (removed from the queues, patches marked busy), or
        [] if nothing is ready or nothing fits.  ``cached(key)`` tells whether the work
        set of a composition (sorted tuple of patch ids) already exists."""
        chosen = self.ready()[: self.max_batch]
        while chosen:
            key = tuple(sorted(chosen))
            if cached(key):
                break
            need = self.plan_bytes(key)
            if need <= self.free_bytes() - self.reserve:
                break
            if self.evict():
                continue
            chosen = chosen[:-1]
        if not chosen:
            return []
        reqs = []
        for p in sorted(chosen):
            q = self.queues[p]
            while self.drop_stale and len(q) > 1:
                self.dropped.append(q.popleft())
            reqs.append(q.popleft())
        self.busy.update(chosen)
        return reqs

    def done(self, patches):
        self.busy.difference_update(patches)


class SolveServer:
    """Continuous-batching RL server over one phase-space PSF.

    ``patches``: list of ((Xr, Xc), (z0, nz)) -- the carpet's patch geometries (the same
    for every frame).  ``submit(patch, frame, lf)`` returns a Future whose result is the
    (Xr, Xc, nz) float32 volume as a host array of its own (copied out of the patch's
    pinned staging buffer before the patch's next frame can run).  A withdrawn request's
    future is cancelled; a dropped one raises :class:`FrameDropped`.
    """

    def __init__(self, psf, patches, iters=3, precision="bf16x2", lanes=2, max_batch=None,
                 reserve_bytes=2 << 30, warm_start=True, drop_stale=False):
        import torch
        from .api import BatchSolver
        self.torch = torch
        self.psf = psf
        self.geo = [((int(s[0]), int(s[1])), (int(z[0]), int(z[1]))) for s, z in patches]
        self.iters = int(iters)
        self.precision = precision
        self.warm_start = warm_start
        P = len(self.geo)
        shapes = [g[0] for g in self.geo]
        planes = [g[1] for g in self.geo]
        # admission, once: per-patch volumes and images (shared by the lanes) plus one work
        # set per lane, within the free device memory minus the reserve
        per_patch = sum(4 * xr * xc * (nz + 1) for (xr, xc), (_, nz) in self.geo)
        plan = BatchSolver.plan_bytes(psf, shapes, planes)
        free = int(torch.cuda.mem_get_info()[0]) - int(reserve_bytes) - per_patch
        if plan > free:
            raise MemoryError(f"serving work set needs {plan + per_patch} bytes; "
                              f"{free + per_patch} free beyond the reserve")
        lanes = max(1, min(int(lanes), free // plan))
        if max_batch is None:
            max_batch = -(-P // lanes)
        self.lanes = lanes
        self._works = [BatchSolver(psf, shapes, planes) for _ in range(lanes)]
        self._state, self._lf_dev, self._pinned_in, self._pinned_out = [], [], [], []
        for (xr, xc), (_, nz) in self.geo:
            self._state.append(torch.empty((nz, xc, xr), dtype=torch.float32, device="cuda").permute(2, 1, 0))
            self._lf_dev.append(torch.empty((xc, xr), dtype=torch.float32, device="cuda").t())
            self._pinned_in.append(torch.empty((xc, xr), dtype=torch.float32, pin_memory=True).t())
            self._pinned_out.append(torch.empty((nz, xc, xr), dtype=torch.float32, pin_memory=True).permute(2, 1, 0))
        self._have_state = [False] * P
        self._lock = threading.Condition()
        # the first run of a work set captures its CUDA graphs: never while the other lane
        # runs its own first run (the library serialises captures against its allocations)
        self._device_lock = threading.RLock()
        self._captured = set()
        self.sched = Scheduler(P, max_batch, lambda key: 0, lambda: 1, lambda: False, 0, drop_stale=drop_stale)
        self._running = {}            # lane -> its requests on the GPU
        self._lat = []
        self._voxels = 0
        self._dropped = 0
        self._withdrawn = 0
        self._t_first = None
        self._t_last = 0.0
        self._batches = []
        self._closing = False
        self._error = None
        self._lanes = []
        for k in range(lanes):
            th = threading.Thread(target=self._lane, args=(k,), name=f"mlf-lane{k}", daemon=True)
            th.start()
            self._lanes.append(th)

    # ---------------------------------------------------------------- client side
    def submit(self, patch, frame, lf, t_arrival=None):
        req = Request(int(patch), int(frame), lf, time.perf_counter() if t_arrival is None else t_arrival)
        with self._lock:
            if self._error is not None:
                raise RuntimeError("server failed") from self._error
            if self._t_first is None or req.t_arrival < self._t_first:
                self._t_first = req.t_arrival
            self.sched.add(req)
            self._lock.notify_all()
        return req.future

    def cancel(self, patch, frame):
        """Withdraw a request.  Queued: removed and its future cancelled at once.  On the
        GPU: its future is cancelled when its batch ends, and when every request of that
        batch has been withdrawn the batch is stopped between view steps (its patches keep
        the previous frame as warm start).  Returns False if the request is unknown or
        already done."""
        with self._lock:
            r = self.sched.remove(int(patch), int(frame))
            if r is not None:
                r.future.cancel()
                self._withdrawn += 1
                self._lock.notify_all()
                return True
            for lane, reqs in self._running.items():
                for r in reqs:
                    if r.patch == patch and r.frame == frame and not r.withdrawn:
                        r.withdrawn = True
                        if all(x.withdrawn for x in reqs):
                            self._works[lane].cancel()
                        return True
        return False

    def drain(self, timeout=None):
        """Wait until every submitted request is done."""
        t_end = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while self.sched.pending() or self.sched.busy:
                if self._error is not None:
                    raise RuntimeError("server failed") from self._error
                left = None if t_end is None else t_end - time.perf_counter()
                if left is not None and left <= 0:
                    raise TimeoutError("requests still pending")
                self._lock.wait(timeout=0.05 if left is None else min(0.05, left))

    def report(self):
        lat = np.array(self._lat) * 1e3
        wall = max(1e-9, self._t_last - (self._t_first or 0.0))
        return {
            "requests": int(lat.size),
            "dropped": int(self._dropped),
            "withdrawn": int(self._withdrawn),
            "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
            "max_ms": float(lat.max()) if lat.size else None,
            "voxels": int(self._voxels),
            "wall_s": wall,
            "voxels_per_s": self._voxels / wall,
            "batches": len(self._batches),
            "mean_batch": float(np.mean([len(b) for b in self._batches])) if self._batches else 0.0,
            "lanes": self.lanes,
        }

    def latencies_ms(self):
        """Latencies (ms) of the requests served since the last reset, in completion order."""
        with self._lock:
            return [1e3 * x for x in self._lat]

    def reset_stats(self):
        """Forget the latencies and throughput recorded so far (e.g. after a warm-up)."""
        with self._lock:
            self._lat.clear()
            self._voxels = 0
            self._dropped = 0
            self._withdrawn = 0
            self._batches.clear()
            self._t_first = None
            self._t_last = 0.0

    def close(self):
        with self._lock:
            self._closing = True
            self._lock.notify_all()
        for th in self._lanes:
            th.join()
        for w in self._works:
            w.close()
        self._works = []

    # ---------------------------------------------------------------- lanes
    def _lane(self, lane):
        torch = self.torch
        stream = torch.cuda.Stream()
        work = self._works[lane]
        while True:
            with self._lock:
                reqs = []
                while not reqs:
                    if self._closing:
                        return
                    reqs = self.sched.pick(lambda key: True)
                    for d in self.sched.dropped:
                        d.future.set_exception(FrameDropped(f"patch {d.patch}: frame {d.frame} superseded"))
                        self._dropped += 1
                    self.sched.dropped.clear()
                    if not reqs:
                        self._lock.wait(timeout=0.05)
                key = tuple(r.patch for r in reqs)
                self._running[lane] = reqs
            try:
                if lane in self._captured:
                    outs, stopped = self._run(work, reqs, stream)
                else:
                    with self._device_lock:
                        outs, stopped = self._run(work, reqs, stream)
                    self._captured.add(lane)
                err = None
            except Exception as e:  # noqa: BLE001 - reported through the futures
                err, outs, stopped = e, None, False
            t_done = time.perf_counter()
            with self._lock:
                self._running.pop(lane, None)
                self.sched.done(key)
                if err is None and not stopped:
                    self._batches.append(key)
                    for r, o in zip(reqs, outs):
                        self._have_state[r.patch] = True
                        if r.withdrawn:
                            continue
                        r.t_done = t_done
                        self._lat.append(t_done - r.t_arrival)
                        self._voxels += int(np.prod(o.shape))
                    self._t_last = max(self._t_last, t_done)
                self._withdrawn += sum(1 for r in reqs if r.withdrawn)
                self._lock.notify_all()
            for k, r in enumerate(reqs):
                if r.withdrawn or (stopped and err is None):
                    r.future.cancel()
                elif err is None:
                    r.future.set_result(outs[k])
                else:
                    r.future.set_exception(err)

    def _run(self, work, reqs, stream):
        """One batch on the lane's work set (the other patches left out).  Returns the
        results and whether the run was stopped by a cancellation."""
        torch = self.torch
        P = len(self.geo)
        lfs, warm, outs = [None] * P, [None] * P, [None] * P
        with torch.cuda.stream(stream):
            for r in reqs:
                p = r.patch
                src = r.lf if torch.is_tensor(r.lf) else torch.from_numpy(np.asarray(r.lf, dtype=np.float32))
                self._pinned_in[p].copy_(src)
                self._lf_dev[p].copy_(self._pinned_in[p], non_blocking=True)
                lfs[p] = self._lf_dev[p]
                warm[p] = self._state[p] if (self.warm_start and self._have_state[p]) else None
                outs[p] = self._state[p]
            work.run(lfs, self.iters, precision=self.precision, warm=warm, outs=outs,
                     stream=stream.cuda_stream, want_stats=False)
            for r in reqs:
                self._pinned_out[r.patch].copy_(self._state[r.patch], non_blocking=True)
            stream.synchronize()
        if work.cancelled:
            return None, True
        # column-major (Xr, Xc, nz) copies, as MATLAB would hold them
        return [np.array(self._pinned_out[r.patch].numpy(), order="F", copy=True) for r in reqs], False
