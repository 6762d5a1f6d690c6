"""Render serving: a request loop with continuous batching over resident
resources.

A job (``scenes.Job``) asks for one image: a mesh of the resident pool under
its own camera, at its own resolution.  The server keeps the pool (meshes,
mip-mapped textures, the programme) resident in every batch slot, and
renders jobs in *batches*: a slot is one pipeline whose colour and depth
buffers form an atlas; a batch packs the queued jobs into the atlas (shelf
packing, arrival order), records each job as a viewport rectangle
(``ps3d_set_viewport_rect``) plus a read-out of its rectangle into the job's
result buffer (``ps3d_copy_colour_rect``, pinned host memory), and launches
the whole batch as one device pass.  While a slot's batch runs, new arrivals
queue; as soon as any slot is free, the next batch is formed from everything
queued that fits ("continuous batching").  With two or more slots, batches
overlap on the device (each slot has its own stream).

Admission is by memory: a job enters a batch only if (a) its rectangle fits
the atlas next to the batch's other jobs, (b) the batch's per-triangle device
scratch stays within the slot's share of the HBM budget (by default a
fraction of the free device memory measured when the server starts), and (c)
its result fits the pinned result arena; otherwise it waits for the next
batch.  A job that could never fit (larger than the atlas or the budget) is
refused at submission.

The images are bit-identical to rendering each job alone in a pipeline of its
own size: a viewport rectangle only offsets the pixel grid, and every job's
pixels are produced by its own triangles only.

``PlainLoop`` is the baseline: one job at a time, in arrival order, each in a
pipeline of its size (one pipeline per resolution), waiting for each result.
"""
from __future__ import annotations

import collections
import dataclasses
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import scenes as S

# device scratch per triangle of a pass (triangle record 64 B, varyings
# 3 x 9 floats) and per (bin, triangle) pair (4 sort arrays x 4 B), with ~2
# pairs per triangle, plus margin
SCRATCH_BYTES_PER_TRIANGLE = 64 + 108 + 2 * 16 + 24


class ShelfPacker:
    """Places rectangles left to right on shelves, in the order given; a
    shelf's height is that of its first rectangle."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.shelves: List[List[int]] = []   # [y, height, x_used]
        self.top = 0

    def place(self, w: int, h: int) -> Optional[Tuple[int, int]]:
        if w > self.width or h > self.height:
            return None
        for sh in self.shelves:
            if h <= sh[1] and sh[2] + w <= self.width:
                x = sh[2]
                sh[2] += w
                return x, sh[0]
        if self.top + h > self.height:
            return None
        self.shelves.append([self.top, h, w])
        self.top += h
        return 0, self.shelves[-1][0]

    def used_height(self) -> int:
        return self.top


class ResultArena:
    """First-fit allocator over one pinned host buffer for job results."""

    def __init__(self, nbytes: int, pinned: bool = True):
        self.nbytes = nbytes
        if pinned:
            import torch
            self._t = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
            self.buf = self._t.numpy()
        else:
            self.buf = np.empty(nbytes, dtype=np.uint8)
        self.base = self.buf.ctypes.data
        self.free: List[Tuple[int, int]] = [(0, nbytes)]   # (offset, size), sorted by offset

    def alloc(self, n: int) -> Optional[int]:
        n = (n + 255) // 256 * 256
        for i, (off, size) in enumerate(self.free):
            if size >= n:
                if size == n:
                    del self.free[i]
                else:
                    self.free[i] = (off + n, size - n)
                return off
        return None

    def release(self, off: int, n: int) -> None:
        n = (n + 255) // 256 * 256
        self.free.append((off, n))
        self.free.sort()
        merged: List[Tuple[int, int]] = []
        for o, s in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + s)
            else:
                merged.append((o, s))
        self.free = merged

    def view(self, off: int, w: int, h: int) -> np.ndarray:
        return self.buf[off:off + w * h * 4].reshape(h, w, 4)


@dataclasses.dataclass
class Done:
    job: S.Job
    t_start: float      # when its batch was launched (s after the stream start)
    t_done: float       # when the host saw it complete
    image: Optional[np.ndarray]
    batch: int


@dataclasses.dataclass
class _Batch:
    seq: int
    jobs: List[Tuple[S.Job, int, int, int]]   # job, x, y, arena offset
    t_launch: float
    triangles: int


def _clear_ops():
    return [("clearDepth", 1.0), ("clearColour", 0xFF000000)]


def job_ops(pool: S.Scene, job: S.Job) -> list:
    """The calls that render `job` alone in a pipeline of its own size (with
    `pool`'s resources): clears, the pool's common state, the job's draws."""
    return _clear_ops() + pool.info["common"] + job.ops


class RenderServer:
    def __init__(self, pool: S.Scene, atlas: Tuple[int, int] = (4096, 4096), slots: int = 2,
                 hbm_budget: Optional[int] = None, arena_bytes: int = 1 << 30, bin_width: Optional[int] = None,
                 pinned: bool = True):
        from .pipeline import PuresoftPipeline
        self.pool = pool
        self.atlas = atlas
        self.pipes = []
        for _ in range(slots):
            p = PuresoftPipeline(*atlas)
            S.replay_setup(pool, p)
            if bin_width:
                p.setBinWidth(bin_width)
            self.pipes.append(p)
        for p in self.pipes:
            p.finish()
        if hbm_budget is None:
            hbm_budget = self.free_device_memory() // 2
        self.hbm_budget = hbm_budget
        self.slot_budget = hbm_budget // max(1, slots)
        self.max_batch_triangles = max(1, self.slot_budget // SCRATCH_BYTES_PER_TRIANGLE)
        self.arena = ResultArena(arena_bytes, pinned=pinned)
        self.batches = 0

    @staticmethod
    def free_device_memory() -> int:
        try:
            import torch
            return int(torch.cuda.mem_get_info()[0])
        except Exception:
            return 8 << 30

    def admissible(self, job: S.Job) -> bool:
        return (job.width <= self.atlas[0] and job.height <= self.atlas[1] and
                job.triangles <= self.max_batch_triangles and job.width * job.height * 4 <= self.arena.nbytes)

    def close(self):
        for p in self.pipes:
            p.close()
        self.pipes = []

    # -- one batch
    def _form(self, queue: collections.deque) -> List[Tuple[S.Job, int, int, int]]:
        packer = ShelfPacker(*self.atlas)
        placed = []
        tris = 0
        while queue:
            job = queue[0]
            if placed and tris + job.triangles > self.max_batch_triangles:
                break
            xy = packer.place(job.width, job.height)
            if xy is None:
                break
            off = self.arena.alloc(job.width * job.height * 4)
            if off is None:
                break
            queue.popleft()
            tris += job.triangles
            placed.append((job, xy[0], xy[1], off))
        return placed

    def _launch(self, pipe, placed):
        S.replay_ops(_clear_ops() + self.pool.info["common"], pipe)
        for job, x, y, off in placed:
            pipe.setViewportRect(x, y, job.width, job.height)
            S.replay_ops(job.ops, pipe)
            pipe.copyColourRect(x, y, job.width, job.height, self.arena.base + off, job.width * 4)
        pipe.flush()

    def serve(self, jobs: Sequence[S.Job], keep_images: bool = False, realtime: bool = True,
              poll_s: float = 20e-6) -> List[Done]:
        """Serves `jobs` (sorted by arrival) as they arrive; returns one
        record per job in completion order.  With realtime=False every job
        is present at time 0 (a closed-loop capacity run)."""
        for j in jobs:
            if not self.admissible(j):
                raise ValueError("job %d (%dx%d, %d triangles) can never be admitted" % (
                    j.id, j.width, j.height, j.triangles))
        n = len(jobs)
        queue: collections.deque = collections.deque()
        busy: Dict[int, _Batch] = {}
        done: List[Done] = []
        nxt = 0
        t0 = time.perf_counter()
        while len(done) < n:
            now = time.perf_counter() - t0
            while nxt < n and (not realtime or jobs[nxt].arrival <= now):
                queue.append(jobs[nxt])
                nxt += 1
            progressed = False
            for slot in list(busy):
                pipe = self.pipes[slot]
                if pipe.query():
                    pipe.finish()          # verifies the pass (and re-runs it after a bin-list overflow)
                    t = time.perf_counter() - t0
                    b = busy.pop(slot)
                    for job, x, y, off in b.jobs:
                        img = self.arena.view(off, job.width, job.height).copy() if keep_images else None
                        self.arena.release(off, job.width * job.height * 4)
                        done.append(Done(job, b.t_launch, t, img, b.seq))
                    progressed = True
            for slot in range(len(self.pipes)):
                if slot in busy or not queue:
                    continue
                placed = self._form(queue)
                if not placed:
                    break
                t = time.perf_counter() - t0
                self._launch(self.pipes[slot], placed)
                busy[slot] = _Batch(self.batches, placed, t, sum(j.triangles for j, *_ in placed))
                self.batches += 1
                progressed = True
            if not progressed:
                if busy:
                    time.sleep(poll_s)
                elif nxt < n and realtime:
                    wait = jobs[nxt].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 1e-3))
        return done


class PlainLoop:
    """One job at a time, in arrival order, each rendered alone in a pipeline
    of its own size and waited for."""

    def __init__(self, pool: S.Scene, resolutions: Sequence[Tuple[int, int]] = S.C5_RESOLUTIONS,
                 bin_width: Optional[int] = None, arena_bytes: int = 64 << 20, pinned: bool = True):
        from .pipeline import PuresoftPipeline
        self.pool = pool
        self.pipes = {}
        for wh in resolutions:
            p = PuresoftPipeline(*wh)
            S.replay_setup(pool, p)
            if bin_width:
                p.setBinWidth(bin_width)
            p.finish()
            self.pipes[wh] = p
        self.arena = ResultArena(arena_bytes, pinned=pinned)

    def close(self):
        for p in self.pipes.values():
            p.close()
        self.pipes = {}

    def render(self, job: S.Job, out_off: int = 0) -> None:
        p = self.pipes[(job.width, job.height)]
        S.replay_ops(job_ops(self.pool, job), p)
        p.copyColourRect(0, 0, job.width, job.height, self.arena.base + out_off, job.width * 4)
        p.finish()

    def serve(self, jobs: Sequence[S.Job], keep_images: bool = False, realtime: bool = True) -> List[Done]:
        done = []
        t0 = time.perf_counter()
        for job in jobs:
            if realtime:
                while time.perf_counter() - t0 < job.arrival:
                    time.sleep(min(1e-3, max(0.0, job.arrival - (time.perf_counter() - t0))))
            t_start = time.perf_counter() - t0
            self.render(job)
            t = time.perf_counter() - t0
            img = self.arena.view(0, job.width, job.height).copy() if keep_images else None
            done.append(Done(job, t_start, t, img, len(done)))
        return done


def summarize(done: Sequence[Done], realtime: bool = True) -> Dict[str, float]:
    """images/s over the whole stream and arrival-to-completion latency
    percentiles (ms)."""
    lat = np.array([d.t_done - (d.job.arrival if realtime else 0.0) for d in done]) * 1e3
    first = min(d.job.arrival for d in done) if realtime else 0.0
    span = max(d.t_done for d in done) - first
    return {"images": len(done), "images_per_s": len(done) / span if span > 0 else float("inf"),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "makespan_s": span,
            "batches": len({d.batch for d in done})}
