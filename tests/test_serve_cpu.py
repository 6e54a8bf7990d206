"""Continuous-batching serving logic (ggcat_gb300/serve.py) on the CPU: a fake device context
answers each submitted batch through the oracle's query and completes it after a random
number of polls, so batches overlap and finish out of order.  Every request's result must
equal its result alone; batches are contiguous runs of arrived requests within the k-mer
budget; no slot is reused while its batch is in flight."""
import numpy as np
import pytest

import oracle
from ggcat_gb300 import serve, synth

K = 31


class FakeDevice:
    def __init__(self, lo, hi, rng, gc_off=None, gc_colors=None, ncolors=0):
        self.lo, self.hi, self.rng = lo, hi, rng
        self.gc_off, self.gc_colors, self.ncolors = gc_off, gc_colors, ncolors
        self.busy, self.last = {}, {}
        self.submitted = []  # (slot, n requests, k-mer positions)

    def query_submit(self, s, text, off, lens):
        assert s not in self.busy, "slot reused while in flight"
        off = np.asarray(off, np.uint64)
        lens = np.asarray(lens, np.uint64)
        assert len(off) >= 1 and int(off[0]) == 0
        m, _, pc = oracle.query(self.lo, self.hi, text, off, lens, K, gc_off=self.gc_off, gc_colors=self.gc_colors,
                                ncolors=self.ncolors)
        self.busy[s] = [int(self.rng.integers(0, 4)), m, pc]
        nk = int(np.maximum(lens.astype(np.int64) - (K - 1), 0).sum())
        self.submitted.append((s, len(off), nk))

    def query_poll(self, s):
        st = self.busy[s]
        if st[0] == 0:
            return True
        st[0] -= 1
        return False

    def query_wait(self, s):
        st = self.busy.pop(s)
        self.last[s] = st
        return st[1]

    def query_color_counts(self, s):
        # like the C API: a slot's results stay readable after the wait, until its next submit
        return self.last[s][2]


@pytest.fixture(scope="module")
def graph():
    rng = np.random.default_rng(11)
    anc = synth.random_genome(30_000, rng)
    gs = [synth.substitute(anc, r, rng) for r in (0.002, 0.01, 0.02)]
    text, off, ln, col = synth.pack_sequences(gs, [0, 1, 2])
    r = oracle.build_graph(text, off, ln, oracle.params(k=K, m=10, bucket_bits=4, second_bits=2, threads=2,
                                                         colors=True), seq_colors=col)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    queries, arrivals = synth.query_stream(gs, 120, rng, min_len=20, max_len=3000, rate_per_s=200_000.0)
    qt, qo, ql = serve._pack(queries)
    alone, _, pc = oracle.query(lo, hi, qt, qo, ql, K, gc_off=coff, gc_colors=ccol, ncolors=3)
    return lo, hi, coff, ccol, qt, qo, ql, arrivals, alone, pc


@pytest.mark.parametrize("slots,budget,spread", [(1, 1 << 20, False), (3, 500, False), (4, 2000, True),
                                                 (2, 1, True)])
def test_batched_results_equal_alone(graph, slots, budget, spread):
    lo, hi, coff, ccol, qt, qo, ql, arrivals, alone, pc = graph
    arr = arrivals if spread else np.zeros_like(arrivals)
    dev = FakeDevice(lo, hi, np.random.default_rng(slots))
    res = serve.serve(dev, K, qt, qo, ql, arr, slots=slots, max_batch_kmers=budget)
    assert (res.matched == alone).all()
    assert sum(n for _, n, _ in dev.submitted) == len(qo) == sum(res.batch_sizes)
    assert res.batches == len(dev.submitted)
    # a batch holds more than one request only if it stays within the budget
    assert all(n == 1 or nk <= budget for _, n, nk in dev.submitted)
    assert (res.latency_s >= 0).all()
    if not spread and budget >= 1 << 20:
        assert res.batches == 1  # everything waiting at t = 0 fits one batch


def test_one_per_launch(graph):
    lo, hi, coff, ccol, qt, qo, ql, arrivals, alone, pc = graph
    dev = FakeDevice(lo, hi, np.random.default_rng(5))
    res = serve.serve(dev, K, qt, qo, ql, np.zeros_like(arrivals), slots=3, one_per_launch=True)
    assert res.batches == len(qo) and set(res.batch_sizes) == {1}
    assert (res.matched == alone).all()


def test_colored_totals(graph):
    lo, hi, coff, ccol, qt, qo, ql, arrivals, alone, pc = graph
    dev = FakeDevice(lo, hi, np.random.default_rng(9), gc_off=coff, gc_colors=ccol, ncolors=3)
    res = serve.serve(dev, K, qt, qo, ql, arrivals, slots=2, max_batch_kmers=4000, colored=True)
    assert (res.matched == alone).all()
    assert (res.color_totals == pc.sum(axis=1)).all()


def test_admission_follows_free_memory(graph):
    """The batch budget is recomputed from the device's free memory at every admission: with
    free memory shrinking over time, every multi-request batch fits the budget its admission
    saw, and results still equal each request's result alone."""
    lo, hi, coff, ccol, qt, qo, ql, arrivals, alone, pc = graph
    dev = FakeDevice(lo, hi, np.random.default_rng(13))
    seen = []

    def free_bytes():
        # 40 KB free at first, 400 bytes less at every admission (never below 2 KB)
        f = max(2048, 40_000 - 400 * len(seen))
        seen.append(f)
        return f

    res = serve.serve(dev, K, qt, qo, ql, np.zeros_like(arrivals), slots=2, max_batch_kmers=1 << 20,
                      free_bytes=free_bytes, bytes_per_kmer=2.0)
    assert (res.matched == alone).all()
    assert len(seen) == res.batches
    for (_, n, nk), f in zip(dev.submitted, seen):
        assert n == 1 or nk <= f / 4.0
