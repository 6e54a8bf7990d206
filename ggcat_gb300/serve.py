"""Continuous-batching query serving over the device-resident graph index.

Requests (query sequences of mixed lengths) arrive over time.  The server keeps up to
``slots`` batches in flight on the GPU (each slot has its own stream and buffers, see
``ggcat_gpu_query_submit``); whenever a slot is free it admits every queued request that
fits the batch budget (k-mer positions, bounded by free device memory) and submits them as
one lookup launch, so requests that arrive while others run are folded into the next batch
and their work overlaps on the device.  Latency of a request = completion time − arrival.

``one_per_launch=True`` gives the baseline: every request is its own batch.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class ServeResult:
    matched: list  # per request: matched k-mer occurrences
    latency_s: np.ndarray  # per request
    wall_s: float
    kmers: int
    batches: int
    batch_sizes: list = field(default_factory=list)

    @property
    def kmers_per_s(self) -> float:
        return self.kmers / self.wall_s if self.wall_s > 0 else 0.0

    def pct_ms(self, q: float) -> float:
        return float(np.percentile(self.latency_s, q) * 1e3) if len(self.latency_s) else 0.0


def _pack(queries: list) -> tuple:
    lens = np.array([len(q) for q in queries], np.uint64)
    off = np.zeros(len(queries), np.uint64)
    if len(queries) > 1:
        off[1:] = np.cumsum(lens[:-1] + 1)
    text = np.empty(int(lens.sum()) + len(queries), np.uint8)
    for o, q in zip(off.tolist(), queries):
        text[o:o + len(q)] = np.frombuffer(q, np.uint8) if isinstance(q, (bytes, bytearray)) else q
        text[o + len(q)] = 10
    return text, off, lens


def serve(ctx, k: int, queries: list, arrivals: np.ndarray, slots: int = 4, max_batch_kmers: int | None = None,
          one_per_launch: bool = False, free_bytes: int | None = None) -> ServeResult:
    """Replays `queries` arriving at `arrivals` (seconds from start) through the server."""
    n = len(queries)
    order = np.argsort(arrivals, kind="stable")
    if max_batch_kmers is None:
        # budget by free device memory: ~1 byte of text + 16 bytes of work items per 2K k-mers
        fb = free_bytes if free_bytes is not None else (8 << 30)
        max_batch_kmers = int(max(1 << 20, min(fb // 8, 512 << 20)))
    nk = np.array([max(len(q) - k + 1, 0) for q in queries], np.int64)
    matched = [None] * n
    done_t = np.zeros(n)
    queue: list[int] = []
    inflight: dict[int, tuple] = {}
    nxt = 0
    batches = 0
    sizes = []
    t0 = time.perf_counter()
    while nxt < n or queue or inflight:
        now = time.perf_counter() - t0
        while nxt < n and arrivals[order[nxt]] <= now:
            queue.append(int(order[nxt]))
            nxt += 1
        # completions
        for s in list(inflight):
            if ctx.query_poll(s):
                ids, _ = inflight.pop(s)
                res = ctx.query_wait(s)
                tdone = time.perf_counter() - t0
                for i, r in zip(ids, res.tolist()):
                    matched[i] = r
                    done_t[i] = tdone
        # admissions
        free_slots = [s for s in range(slots) if s not in inflight]
        while queue and free_slots:
            s = free_slots.pop(0)
            take, budget = [], 0
            while queue and (not take or (not one_per_launch and budget + nk[queue[0]] <= max_batch_kmers)):
                i = queue.pop(0)
                take.append(i)
                budget += int(nk[i])
                if one_per_launch:
                    break
            text, off, ln = _pack([queries[i] for i in take])
            ctx.query_submit(s, text, off, ln)
            inflight[s] = (take, time.perf_counter() - t0)
            batches += 1
            sizes.append(len(take))
        if not inflight and not queue and nxt < n:
            # idle until the next arrival
            wait = arrivals[order[nxt]] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.001))
    wall = time.perf_counter() - t0
    lat = done_t - arrivals
    return ServeResult(matched, lat, wall, int(nk.sum()), batches, sizes)
