"""GPU colour-subset dedup against the oracle's MultipleColorsManager restatement: every
surviving k-mer's decoded colour set, subset uniqueness, and per-colour query counts."""
import numpy as np
import pytest

import oracle
from ggcat_gb300 import _native, serve, synth

pytestmark = pytest.mark.gpu


def _colored_input(seed=21, n_genomes=12, L=60_000):
    rng = np.random.default_rng(seed)
    anc = synth.random_genome(L, rng)
    gs = [synth.indels(synth.substitute(anc, float(rng.uniform(0.001, 0.03)), rng), 0.001, 20, rng)
          for _ in range(n_genomes)]
    # two sequences per colour for some colours (a colour is a file, not a sequence)
    seqs, cols = [], []
    for c, g in enumerate(gs):
        if c % 3 == 0:
            half = len(g) // 2
            seqs += [g[:half], g[half:]]
            cols += [c, c]
        else:
            seqs.append(g)
            cols.append(c)
    text, off, ln, col = synth.pack_sequences(seqs, cols)
    return text, off, ln, col, gs, n_genomes


@pytest.fixture(scope="module")
def built():
    text, off, ln, col, gs, nc = _colored_input()
    ctx = _native.GpuContext(0)
    p = _native.make_params(k=31, m=10, bucket_bits=6, second_bits=2, min_multiplicity=1, keep_kmers=True)
    ctx.build_text(text, p)
    ctx.colors(off, col, nc)
    r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=6, second_bits=2, threads=4,
                                                         colors=True), seq_colors=col)
    yield ctx, r, text, off, ln, col, gs, nc
    ctx.close()


def _decode(bm_row):
    cols = []
    for w, word in enumerate(bm_row.tolist()):
        for b in range(32):
            if (word >> b) & 1:
                cols.append(w * 32 + b)
    return tuple(cols)


def test_kmer_color_sets_match_oracle(built):
    ctx, r, *_ = built
    keys, mult = ctx.kmers()
    subs = ctx.kmer_subsets()
    bitmaps = ctx.subsets()
    decoded = [_decode(row) for row in bitmaps]
    assert len(set(decoded)) == len(decoded)  # every subset appears once
    got = {}
    for kk, sid in zip(keys.tolist(), subs.tolist()):
        cs = decoded[sid]
        assert got.get(kk, cs) == cs
        got[kk] = cs
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    exp = {int(lo[i]): tuple(int(c) for c in ccol[coff[i]:coff[i + 1]]) for i in range(len(lo))}
    assert got == exp


def test_colored_query_counts_match_oracle(built):
    ctx, r, text, off, ln, col, gs, nc = built
    ctx.query_index_colored()
    rng = np.random.default_rng(5)
    queries, _ = synth.query_stream(gs, 60, rng, min_len=20, max_len=8000)
    qt, qo, ql = serve._pack(queries)
    ctx.query_submit(1, qt, qo, ql)
    matched = ctx.query_wait(1)
    counts = ctx.query_color_counts(1)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    em, _, epc = oracle.query(lo, hi, qt, qo, ql, 31, gc_off=coff, gc_colors=ccol, ncolors=nc)
    assert (matched == em).all()
    assert (counts == epc).all()
    assert epc.sum() > 0


def test_colored_serving_matches_direct_batch(built):
    """The continuous-batching loop over a coloured index returns, per query, the same
    per-colour totals as one direct batch (and as the oracle)."""
    ctx, r, text, off, ln, col, gs, nc = built
    ctx.query_index_colored()
    rng = np.random.default_rng(9)
    queries, arrivals = synth.query_stream(gs, 40, rng, min_len=40, max_len=5000, rate_per_s=5000.0)
    qt, qo, ql = serve._pack(queries)
    res = serve.serve(ctx, 31, qt, qo, ql, arrivals, slots=3, max_batch_kmers=3000, colored=True)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    em, _, epc = oracle.query(lo, hi, qt, qo, ql, 31, gc_off=coff, gc_colors=ccol, ncolors=nc)
    assert (res.matched == em).all()
    assert (res.color_totals == epc.sum(axis=1)).all()
    assert res.batches > 1


def _check_color_sets(ctx, r):
    keys, _ = ctx.kmers()
    subs = ctx.kmer_subsets()
    decoded = [_decode(row) for row in ctx.subsets()]
    assert len(set(decoded)) == len(decoded)
    got = {}
    for kk, sid in zip(keys.tolist(), subs.tolist()):
        assert got.get(kk, decoded[sid]) == decoded[sid]
        got[kk] = decoded[sid]
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    assert got == {int(lo[i]): tuple(int(c) for c in ccol[coff[i]:coff[i + 1]]) for i in range(len(lo))}


@pytest.mark.parametrize("n_reads,read_len,colors", [(300, 150, 5), (70_000, 60, 4)])
def test_color_sets_mixed_lengths_and_read_sets(n_reads, read_len, colors):
    """The occurrence pass's other chunk orders: a genome beside short reads (rows are equal
    slices of the text) and more sequences than it keeps rows for (text order)."""
    rng = np.random.default_rng(n_reads)
    g = synth.random_genome(200_000, rng)
    reads = synth.sample_reads(g, n_reads, read_len, 0.002, 0.0, rng)
    seqs = [g] + list(reads)
    cols = [0] + [1 + i % (colors - 1) for i in range(n_reads)]
    text, off, ln, col = synth.pack_sequences(seqs, cols)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=31, m=10, bucket_bits=6, second_bits=2, min_multiplicity=1, keep_kmers=True)
        ctx.build_text(text, p)
        ctx.colors(off, col, colors)
        r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=6, second_bits=2, threads=4,
                                                             colors=True), seq_colors=col)
        _check_color_sets(ctx, r)
    finally:
        ctx.close()


def test_color_sets_and_query_k63_match_oracle():
    """Colours for k > 32: u128 keys in 32-byte table slots (key claimed by a 128-bit
    compare-and-swap, id stored after it), 128-bit rolling in the occurrence pass, and the
    coloured query over a u128 index."""
    text, off, ln, col, gs, nc = _colored_input(seed=33, n_genomes=10, L=50_000)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=63, m=12, bucket_bits=6, second_bits=2, min_multiplicity=1, keep_kmers=True)
        ctx.build_text(text, p)
        ctx.colors(off, col, nc)
        keys, _ = ctx.kmers()
        subs = ctx.kmer_subsets()
        decoded = [_decode(row) for row in ctx.subsets()]
        assert len(set(decoded)) == len(decoded)
        got = {}
        for (lo_w, hi_w), sid in zip(keys.tolist(), subs.tolist()):
            assert got.get((lo_w, hi_w), decoded[sid]) == decoded[sid]
            got[(lo_w, hi_w)] = decoded[sid]
        r = oracle.build_graph(text, off, ln, oracle.params(k=63, m=12, bucket_bits=6, second_bits=2, threads=4,
                                                             colors=True), seq_colors=col)
        lo, hi, _ = r.kmers()
        coff, ccol = r.kmer_colors()
        exp = {(int(lo[i]), int(hi[i])): tuple(int(c) for c in ccol[coff[i]:coff[i + 1]]) for i in range(len(lo))}
        assert got == exp and len(exp) > 0
        ctx.query_index_colored()
        rng = np.random.default_rng(8)
        queries, _ = synth.query_stream(gs, 40, rng, min_len=70, max_len=6000)
        qt, qo, ql = serve._pack(queries)
        ctx.query_submit(1, qt, qo, ql)
        matched = ctx.query_wait(1)
        counts = ctx.query_color_counts(1)
        em, _, epc = oracle.query(lo, hi, qt, qo, ql, 63, gc_off=coff, gc_colors=ccol, ncolors=nc)
        assert (matched == em).all() and em.sum() > 0
        assert (counts == epc).all()
    finally:
        ctx.close()


@pytest.mark.parametrize("k,m,bbits", [(31, 10, 6), (31, 10, 3), (45, 12, 5)])
def test_colors_collected_by_the_merge(k, m, bbits):
    """Colours announced before the build (ggcat_gpu_colors_prepare) are collected by the merge
    units; ggcat_gpu_colors then merges the dumped copies of a k-mer (a copy in a neighbouring
    sub-bucket sees only its boundary occurrences) instead of reading the text.  The per-k-mer
    colour sets equal the oracle's and the text pass's, and each set is one subset."""
    from oracle import parity

    text, off, ln, col, gs, nc = _colored_input(seed=31 + k + bbits)
    p = _native.make_params(k=k, m=m, bucket_bits=bbits, second_bits=2, min_multiplicity=1, keep_kmers=True)
    r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=m, bucket_bits=bbits, second_bits=2, threads=4,
                                                         colors=True), seq_colors=col)
    digests = []
    for prepare in (True, False):
        ctx = _native.GpuContext(0)
        try:
            if prepare:
                ctx.colors_prepare(off, col, nc)
            ctx.build_text(text, p)
            ctx.colors(off, col, nc)
            assert ctx.stats()["colors_collected"] == (1 if prepare else 0)
            keys, _ = ctx.kmers()
            res = parity.compare_color_sets(keys, ctx.kmer_subsets(), ctx.subsets(), r)
            assert res["equal"], res
            digests.append(res["digest_gpu"])
        finally:
            ctx.close()
    assert digests[0] == digests[1]


@pytest.mark.parametrize("n_genomes,max_rate", [(40, 0.03), (70, 0.0005), (200, 0.03), (300, 0.002)])
def test_colored_query_counts_many_colours(n_genomes, max_rate):
    """Subset bitmaps of 2, 3, 7 and 10 words: the warp-per-run lookup (up to 8 words; 70 and
    200 colours end in a partial word) and the per-query CTA lookup (above 8 words).  Queries
    are longer than one work item (4096 k-mer positions) and some hold N runs; the low
    divergence cases give long runs of one subset (multiplicities above 1)."""
    rng = np.random.default_rng(1000 + n_genomes)
    anc = synth.random_genome(12_000, rng)
    gs = [synth.indels(synth.substitute(anc, float(rng.uniform(0.0, max_rate)), rng), 0.0005, 10, rng)
          for _ in range(n_genomes)]
    text, off, ln, col = synth.pack_sequences(gs, list(range(n_genomes)))
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=31, m=10, bucket_bits=6, second_bits=2, min_multiplicity=1, keep_kmers=True)
        ctx.build_text(text, p)
        ctx.colors(off, col, n_genomes)
        r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=6, second_bits=2, threads=8,
                                                             colors=True), seq_colors=col)
        ctx.query_index_colored()
        queries, _ = synth.query_stream(gs, 50, rng, min_len=20, max_len=12_000)
        qt, qo, ql = serve._pack(queries)
        for i in range(0, len(qo), 3):  # N runs inside every third query
            if ql[i] > 100:
                at = int(qo[i]) + int(rng.integers(0, int(ql[i]) - 10))
                qt[at:at + int(rng.integers(1, 6))] = ord("N")
        ctx.query_submit(2, qt, qo, ql)
        matched = ctx.query_wait(2)
        counts = ctx.query_color_counts(2)
        lo, hi, _ = r.kmers()
        coff, ccol = r.kmer_colors()
        em, _, epc = oracle.query(lo, hi, qt, qo, ql, 31, gc_off=coff, gc_colors=ccol, ncolors=n_genomes)
        assert counts.shape == (len(qo), n_genomes)
        assert (matched == em).all()
        assert (counts == epc).all()
        assert epc[:, -1].sum() > 0 and epc.sum() > 0
    finally:
        ctx.close()
