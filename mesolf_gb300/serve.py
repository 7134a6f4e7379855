"""Serving loop for streams of light-field frames (patches of a carpet arriving at a frame
rate), on top of the batched tensor-core solve.

A request is one patch of one frame.  The server keeps, resident in HBM, the phase-space
PSF (its taps and spectra-free tensor-core tables), one batch work set per patch
composition in use, and one volume per patch: the previous frame's reconstruction, which
warm-starts the next frame of that patch (the reference's ``Xguess`` initial value,
``recon_theory_phase_space_LFM_with_filter.m:72-73``, replaced by the last result).

* Continuous batching.  ``lanes`` worker threads each own a CUDA stream.  Whenever a lane
  is free it takes every patch whose oldest pending frame is ready (the patch is not on
  the GPU in another lane), oldest arrival first, up to ``max_batch`` patches, and runs
  them as one batch (one launch per view step for all of them).  Requests that arrive
  while other batches are on the GPU are admitted into the next batch a lane forms, so
  two batches overlap on the device (copies of one with kernels of the other).
* Admission by free HBM.  A batch whose work set is not yet allocated is admitted only if
  its planned bytes (``BatchSolver.plan_bytes``) plus its new per-patch volumes fit in the
  free device memory minus ``reserve_bytes``; otherwise idle work sets are evicted (least
  recently used first), and if that is not enough the batch is shrunk (youngest requests
  first).  A batch of one patch that cannot fit while nothing else runs fails its request.
* Latency is measured from the request's arrival time to the moment its volume is in host
  memory; :meth:`SolveServer.report` gives p50 / p99 and the deconvolved voxels/s.

The result of a request is identical whether it is solved alone or in a mix: each patch
occupies its own lenslet positions of the batch, its view weights, plane range and
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

__all__ = ["Request", "Scheduler", "SolveServer"]


@dataclasses.dataclass
class Request:
    patch: int
    frame: int
    lf: object                     # host (Xr, Xc) float32 image
    t_arrival: float               # time.perf_counter() seconds
    future: concurrent.futures.Future = dataclasses.field(default_factory=concurrent.futures.Future)
    t_done: float = 0.0


class Scheduler:
    """Batching and admission decisions; no device work (unit-testable on the CPU).

    ``plan_bytes(patches)`` gives the device bytes a new work set for that composition
    needs; ``free_bytes()`` the device memory free now; ``evict()`` frees one idle cached
    work set and returns True, or returns False when there is none.
    """

    def __init__(self, n_patches, max_batch, plan_bytes, free_bytes, evict, reserve_bytes=0):
        self.queues = [collections.deque() for _ in range(n_patches)]
        self.last_frame = [None] * n_patches
        self.busy = set()
        self.max_batch = max(1, int(max_batch))
        self.plan_bytes = plan_bytes
        self.free_bytes = free_bytes
        self.evict = evict
        self.reserve = int(reserve_bytes)

    def add(self, req: Request):
        last = self.last_frame[req.patch]
        if last is not None and last >= req.frame:
            raise ValueError(f"patch {req.patch}: frame {req.frame} after frame {last}")
        self.last_frame[req.patch] = req.frame
        self.queues[req.patch].append(req)

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
        reqs = [self.queues[p].popleft() for p in sorted(chosen)]
        self.busy.update(chosen)
        return reqs

    def done(self, patches):
        self.busy.difference_update(patches)


class SolveServer:
    """Continuous-batching RL server over one phase-space PSF.

    ``patches``: list of ((Xr, Xc), (z0, nz)) -- the carpet's patch geometries (the same
    for every frame).  ``submit(patch, frame, lf)`` returns a Future whose result is the
    (Xr, Xc, nz) float32 volume as a host array of its own (copied out of the patch's
    pinned staging buffer before the patch's next frame can run).
    """

    def __init__(self, psf, patches, iters=3, precision="bf16x2", lanes=2, max_batch=None,
                 reserve_bytes=2 << 30, warm_start=True, cache_limit=8):
        import torch
        from .api import BatchSolver
        self.torch = torch
        self.psf = psf
        self.geo = [((int(s[0]), int(s[1])), (int(z[0]), int(z[1]))) for s, z in patches]
        self.iters = int(iters)
        self.precision = precision
        self.warm_start = warm_start
        P = len(self.geo)
        if max_batch is None:
            max_batch = -(-P // max(1, lanes))
        self._BatchSolver = BatchSolver
        self._works = collections.OrderedDict()   # composition -> BatchSolver (LRU order)
        self._in_use = set()
        self._cache_limit = cache_limit
        self._lock = threading.Condition()
        # allocations, releases and the first run of a work set (which captures its CUDA
        # graph) never overlap: a release synchronises the device and would invalidate a
        # capture running on the other lane
        self._device_lock = threading.RLock()
        self._captured = set()
        self.sched = Scheduler(P, max_batch, self._plan_bytes, self._free_bytes, self._evict_one, reserve_bytes)
        self._state = [None] * P                  # resident per-patch volume (device)
        self._have_state = [False] * P
        self._lf_dev = [None] * P
        self._pinned_in = [None] * P
        self._pinned_out = [None] * P
        self._lat = []
        self._voxels = 0
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

    # ---------------------------------------------------------------- admission hooks
    def _plan_bytes(self, key):
        shapes = [self.geo[p][0] for p in key]
        planes = [self.geo[p][1] for p in key]
        b = self._BatchSolver.plan_bytes(self.psf, shapes, planes)
        for p in key:   # per-patch volume and image, allocated on first use
            if self._state[p] is None:
                (xr, xc), (_, nz) = self.geo[p]
                b += 4 * xr * xc * (nz + 1)
        return b

    def _free_bytes(self):
        free, _ = self.torch.cuda.mem_get_info()
        return int(free)

    def _evict_one(self):
        for key in list(self._works):
            if key not in self._in_use:
                w = self._works.pop(key)
                self._captured.discard(key)
                with self._device_lock:
                    w.close()
                return True
        return False

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
            "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
            "max_ms": float(lat.max()) if lat.size else None,
            "voxels": int(self._voxels),
            "wall_s": wall,
            "voxels_per_s": self._voxels / wall,
            "batches": len(self._batches),
            "mean_batch": float(np.mean([len(b) for b in self._batches])) if self._batches else 0.0,
        }

    def reset_stats(self):
        """Forget the latencies and throughput recorded so far (e.g. after a warm-up)."""
        with self._lock:
            self._lat.clear()
            self._voxels = 0
            self._batches.clear()
            self._t_first = None
            self._t_last = 0.0

    def close(self):
        with self._lock:
            self._closing = True
            self._lock.notify_all()
        for th in self._lanes:
            th.join()
        for w in self._works.values():
            w.close()
        self._works.clear()

    # ---------------------------------------------------------------- lanes
    def _buffers(self, p):
        torch = self.torch
        (xr, xc), (_, nz) = self.geo[p]
        if self._state[p] is None:
            self._state[p] = torch.empty((nz, xc, xr), dtype=torch.float32, device="cuda").permute(2, 1, 0)
            self._lf_dev[p] = torch.empty((xc, xr), dtype=torch.float32, device="cuda").t()
            self._pinned_in[p] = torch.empty((xc, xr), dtype=torch.float32, pin_memory=True).t()
            self._pinned_out[p] = torch.empty((nz, xc, xr), dtype=torch.float32,
                                              pin_memory=True).permute(2, 1, 0)

    def _work(self, key):
        w = self._works.get(key)
        if w is None:
            w = self._BatchSolver(self.psf, [self.geo[p][0] for p in key], [self.geo[p][1] for p in key])
            self._works[key] = w
            while len(self._works) > self._cache_limit and self._evict_one():
                pass
        self._works.move_to_end(key)
        return w

    def _lane(self, lane):
        torch = self.torch
        stream = torch.cuda.Stream()
        while True:
            with self._lock:
                reqs = []
                while not reqs:
                    if self._closing:
                        return
                    reqs = self.sched.pick(lambda key: key in self._works)
                    if not reqs:
                        if self.sched.ready() and not self.sched.busy:
                            # nothing running and the oldest single patch does not fit
                            p = self.sched.ready()[0]
                            r = self.sched.queues[p].popleft()
                            r.future.set_exception(MemoryError(
                                f"patch {p}: work set does not fit in free device memory"))
                            self._lock.notify_all()
                            continue
                        self._lock.wait(timeout=0.05)
                key = tuple(r.patch for r in reqs)
                try:
                    with self._device_lock:
                        for p in key:
                            self._buffers(p)
                        work = self._work(key)
                except Exception as e:  # allocation failure: fail this batch's requests
                    self.sched.done(key)
                    for r in reqs:
                        r.future.set_exception(e)
                    self._lock.notify_all()
                    continue
                self._in_use.add(key)
            try:
                if key in self._captured:
                    outs = self._run(work, key, reqs, stream)
                else:
                    with self._device_lock:
                        outs = self._run(work, key, reqs, stream)
                    self._captured.add(key)
                err = None
            except Exception as e:  # noqa: BLE001 - reported through the futures
                err = e
            t_done = time.perf_counter()
            with self._lock:
                self._in_use.discard(key)
                self.sched.done(key)
                if err is None:
                    self._batches.append(key)
                    for r, o in zip(reqs, outs):
                        r.t_done = t_done
                        self._lat.append(t_done - r.t_arrival)
                        self._voxels += int(np.prod(o.shape))
                        self._have_state[r.patch] = True
                    self._t_last = max(self._t_last, t_done)
                self._lock.notify_all()
            for k, r in enumerate(reqs):
                if err is None:
                    r.future.set_result(outs[k])
                else:
                    r.future.set_exception(err)

    def _run(self, work, key, reqs, stream):
        torch = self.torch
        with torch.cuda.stream(stream):
            lfs, warm, outs, host = [], [], [], []
            for r in reqs:
                p = r.patch
                src = r.lf if torch.is_tensor(r.lf) else torch.from_numpy(np.asarray(r.lf, dtype=np.float32))
                self._pinned_in[p].copy_(src)
                self._lf_dev[p].copy_(self._pinned_in[p], non_blocking=True)
                lfs.append(self._lf_dev[p])
                warm.append(self._state[p] if (self.warm_start and self._have_state[p]) else None)
                outs.append(self._state[p])
            work.run(lfs, self.iters, precision=self.precision, warm=warm, outs=outs,
                     stream=stream.cuda_stream, want_stats=False)
            for r in reqs:
                p = r.patch
                self._pinned_out[p].copy_(self._state[p], non_blocking=True)
                host.append(self._pinned_out[p])
            stream.synchronize()
        # column-major (Xr, Xc, nz) copies, as MATLAB would hold them
        return [np.array(h.numpy(), order="F", copy=True) for h in host]
