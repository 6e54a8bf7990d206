"""The allocation-free bucket histogram entry point against the regular bucketize.

Callers that cannot allocate device memory (their memory is owned by another allocator,
or allocation is not allowed where they run) use ggcat_gpu_bucket_histogram_noalloc with
their own input/output buffers; its only scratch is a static device array.  Its per-bucket
superkmer counts, k-mer counts and offsets must equal those derived from the records of
ggcat_gpu_bucketize, on two calls in a row (the second must not see the first's scratch)."""
import ctypes as C

import numpy as np
import pytest

from ggcat_gb300 import _native, synth

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(31)
    g = synth.random_genome(120_000, rng)
    g = synth.add_repeats(g, 0.03, 400, 5, 30, rng)
    reads = synth.sample_reads(g, 6000, 150, 0.005, 0.001, rng)
    a = synth.pack_reads(reads)[0]
    gs = [g] + [synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng)]
    gs += [np.frombuffer(b"A" * 200 + b"N" + b"ACGT" * 40, np.uint8)]
    b = synth.pack_sequences(gs)[0]
    return [(a, 31, 10, 10), (b, 31, 10, 6), (a, 63, 12, 8)]


def _edge_text(k, m, seed=5):
    """Pieces of length k - 1, k and k + 1, then a long sequence whose N runs and record
    boundaries sit just before, on and just after multiples of the histogram kernel's
    per-thread chunk (the pending-first, continued and piece-end paths)."""
    rng = np.random.default_rng(seed)
    wn = k - m
    chunk = ((512 + wn - 1) // wn) * wn
    pieces = []
    for ln in (k - 1, k, k + 1) * 6:
        pieces.append(synth.random_genome(ln, rng))
    g = synth.random_genome(40 * chunk, rng).copy()
    offs = (-k, -2, -1, 0, 1, k - 1)
    for c in range(1, 38):
        p = c * chunk + offs[c % len(offs)]
        if c % 3 == 0:
            g[p:p + 3] = ord("N")
        else:
            g[p] = ord("N")
    pieces.append(g)
    text = synth.pack_sequences(pieces)[0]
    # separators on chunk multiples of the whole text too
    for c in range(3, text.size // chunk, 7):
        text[c * chunk + offs[c % len(offs)]] = 10
    return text


EDGE_CASES = [(31, 10, 6), (12, 10, 5), (64, 32, 8)]


def _expected(ctx, torch, text, k, m, bbits):
    d = torch.from_numpy(text).cuda()
    p = _native.make_params(k=k, m=m, bucket_bits=bbits, second_bits=2)
    ctx.bucketize(d.data_ptr(), d.numel(), p, torch.cuda.current_stream().cuda_stream)
    sk = ctx.superkmers()
    nb = (1 << bbits) + 1
    cnt = np.bincount(sk["bucket"].astype(np.int64), minlength=nb).astype(np.uint64)
    kms = np.bincount(sk["bucket"].astype(np.int64), weights=(sk["len"].astype(np.int64) - k + 1),
                      minlength=nb).astype(np.uint64)
    off = np.zeros(nb + 1, np.uint64)
    off[1:] = np.cumsum(cnt)
    return cnt, kms, off


def test_noalloc_histogram_matches_bucketize_twice_in_a_row():
    torch = pytest.importorskip("torch")
    L = _native.load()
    ctx = _native.GpuContext(0)
    try:
        cases = _inputs()
        for text, k, m, bbits in cases[:2] + [cases[0], cases[2]]:
            nb = (1 << bbits) + 1
            exp = _expected(ctx, torch, text, k, m, bbits)
            d_text = torch.from_numpy(text).cuda()
            outs = [torch.full((n,), 0xDEAD, dtype=torch.int64, device="cuda") for n in (nb, nb, nb + 1)]
            stream = torch.cuda.current_stream()
            rc = L.ggcat_gpu_bucket_histogram_noalloc(C.c_void_p(d_text.data_ptr()), d_text.numel(), k, m, bbits,
                                                      C.c_void_p(outs[0].data_ptr()), C.c_void_p(outs[1].data_ptr()),
                                                      C.c_void_p(outs[2].data_ptr()), C.c_void_p(stream.cuda_stream))
            assert rc == 0
            torch.cuda.synchronize()
            got = [o.cpu().numpy().astype(np.uint64) for o in outs]
            for g_, e_ in zip(got, exp):
                assert (g_ == e_).all()
    finally:
        ctx.close()


def test_noalloc_rejects_too_many_buckets():
    torch = pytest.importorskip("torch")
    L = _native.load()
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    o = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = L.ggcat_gpu_bucket_histogram_noalloc(C.c_void_p(d.data_ptr()), 64, 31, 10, 14, C.c_void_p(o.data_ptr()),
                                              C.c_void_p(o.data_ptr()), C.c_void_p(o.data_ptr()), None)
    assert rc == -7  # GGCAT_GPU_ETOOLARGE: more buckets than the static scratch holds


def test_noalloc_edge_pieces_and_chunk_boundaries():
    """Pieces shorter than, equal to and one longer than k, N runs and separators next to the
    per-thread chunk boundaries, k - m = 2 and k = 64 with m = 32: equal to ggcat_gpu_bucketize."""
    torch = pytest.importorskip("torch")
    L = _native.load()
    ctx = _native.GpuContext(0)
    try:
        for k, m, bbits in EDGE_CASES:
            text = _edge_text(k, m)
            nb = (1 << bbits) + 1
            exp = _expected(ctx, torch, text, k, m, bbits)
            assert exp[0].sum() > 0
            d_text = torch.from_numpy(text).cuda()
            outs = [torch.full((n,), 0xDEAD, dtype=torch.int64, device="cuda") for n in (nb, nb, nb + 1)]
            rc = L.ggcat_gpu_bucket_histogram_noalloc(C.c_void_p(d_text.data_ptr()), d_text.numel(), k, m, bbits,
                                                      C.c_void_p(outs[0].data_ptr()), C.c_void_p(outs[1].data_ptr()),
                                                      C.c_void_p(outs[2].data_ptr()),
                                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
            assert rc == 0
            torch.cuda.synchronize()
            for g_, e_ in zip([o.cpu().numpy().astype(np.uint64) for o in outs], exp):
                assert (g_ == e_).all(), (k, m)
    finally:
        ctx.close()
