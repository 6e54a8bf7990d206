"""Continuous-batching query serving over the device-resident graph index.

Requests (query sequences of mixed lengths) arrive over time.  The server keeps up to
``slots`` batches in flight on the GPU (each slot has its own stream and buffers, see
``ggcat_gpu_query_submit``); whenever a slot is free it admits the queued requests that fit
the batch budget (k-mer positions, bounded by free device memory) and submits them as one
lookup launch, so requests that arrive while others run are folded into the next batch and
their work overlaps on the device.  Latency of a request = completion time - arrival time.

``one_per_launch=True`` gives the baseline: every request is its own batch.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class ServeResult:
    matched: np.ndarray  # per request: matched k-mer occurrences
    latency_s: np.ndarray  # per request
    wall_s: float
    kmers: int
    batches: int
    batch_sizes: list = field(default_factory=list)
    color_totals: np.ndarray | None = None  # coloured index: per request, sum of its per-colour counts

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
    text = np.full(int(lens.sum()) + len(queries), 10, np.uint8)
    for o, q in zip(off.tolist(), queries):
        text[o:o + len(q)] = np.frombuffer(q, np.uint8) if isinstance(q, (bytes, bytearray)) else q
    return text, off, lens


def serve(ctx, k: int, text: np.ndarray, off: np.ndarray, lens: np.ndarray, arrivals: np.ndarray, slots: int = 4,
          max_batch_kmers: int = 64 << 20, one_per_launch: bool = False, colored: bool = False,
          free_bytes=None, bytes_per_kmer: float = 2.0) -> ServeResult:
    """Replays the queries (text layout: query i = text[off[i] : off[i] + lens[i]], arrivals
    non-decreasing, in seconds from the start) through the server.  With a coloured index,
    ``colored=True`` also reads every batch's per-colour counts back.  ``free_bytes`` (a
    callable returning the device's free memory) is asked at every admission: a batch admits
    at most half of the free memory's worth of k-mer positions (``bytes_per_kmer`` device bytes
    each) and never more than ``max_batch_kmers``; at least one request is always admitted."""
    n = len(off)
    off = np.asarray(off, np.uint64)
    lens = np.asarray(lens, np.uint64)
    nk = np.maximum(lens.astype(np.int64) - (k - 1), 0)
    cum = np.concatenate([[0], np.cumsum(nk)])
    matched = np.zeros(n, np.uint64)
    ctot = np.zeros(n, np.uint64) if colored else None
    done_t = np.zeros(n)
    inflight: dict[int, tuple] = {}
    head = 0  # next request not yet submitted (arrival order = index order)
    batches = 0
    sizes = []
    t0 = time.perf_counter()
    while head < n or inflight:
        for s in list(inflight):
            if ctx.query_poll(s):
                a, b = inflight.pop(s)
                res = ctx.query_wait(s)
                matched[a:b] = res
                if colored:
                    ctot[a:b] = ctx.query_color_counts(s).sum(axis=1)
                done_t[a:b] = time.perf_counter() - t0
        now = time.perf_counter() - t0
        arrived = int(np.searchsorted(arrivals, now, side="right"))
        free = [s for s in range(slots) if s not in inflight]
        while free and head < arrived:
            s = free.pop(0)
            if one_per_launch:
                b = head + 1
            else:
                # admit every arrived request that fits the k-mer budget (at least one); the
                # budget shrinks with the device's free memory
                budget = max_batch_kmers
                if free_bytes is not None:
                    budget = max(1, min(budget, int(free_bytes() / (2.0 * bytes_per_kmer))))
                lim = cum[head] + budget
                b = max(head + 1, min(arrived, int(np.searchsorted(cum, lim, side="right")) - 1))
            lo = int(off[head])
            hi = int(off[b - 1] + lens[b - 1])
            ctx.query_submit(s, text[lo:hi], off[head:b] - np.uint64(lo), lens[head:b])
            inflight[s] = (head, b)
            batches += 1
            sizes.append(b - head)
            head = b
        if not inflight and head < n:
            wait = arrivals[head] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.0005))
    wall = time.perf_counter() - t0
    return ServeResult(matched, done_t - arrivals, wall, int(nk.sum()), batches, sizes, ctot)
