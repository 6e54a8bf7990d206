"""Bucket-store spill: with a small spill budget (spill_mb) the text is bucketized in pieces
whose records go to pinned host memory and the merge runs bucket range by bucket range; the
superkmer records, surviving k-mers, unitigs and colour sets are bit-identical to the resident
path's and to the oracle's."""
import numpy as np
import pytest

import oracle
from oracle import parity
from ggcat_gb300 import _native, synth

pytestmark = pytest.mark.gpu


def _reads(seed=41, genome=150_000, n_reads=14_000):
    rng = np.random.default_rng(seed)
    g = synth.add_repeats(synth.random_genome(genome, rng), 0.02, 500, 20, 60, rng)
    return synth.pack_reads(synth.sample_reads(g, n_reads, 150, 0.005, 0.0005, rng))


def _outputs(ctx, text, p):
    ctx.build_text(text, p)
    st = ctx.stats()
    sk = ctx.superkmers()
    keys, mult = ctx.kmers()
    ctx.link(p.k)
    bases, uo, ul, uf = ctx.unitigs()
    lines = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, p.k)
    return st, sk, keys, mult, lines


def _sk_sorted(a):
    cols = ["start", "len", "bucket", "second_bucket", "minimizer_pos", "rc", "flags"]
    arr = np.stack([a[c].astype(np.uint64) for c in cols], axis=1)
    return arr[np.lexsort(arr.T[::-1])]


@pytest.mark.parametrize("k,m,hk", [(31, 10, _native.GGCAT_HASH_SEQHASH), (63, 12, _native.GGCAT_HASH_RABIN_KARP128)])
def test_spilled_build_equals_resident(k, m, hk):
    text, off, ln, _ = _reads()
    ctx = _native.GpuContext(0)
    try:
        base = dict(k=k, m=m, bucket_bits=6, second_bits=2, min_multiplicity=2, hash_kind=hk, keep_kmers=True)
        st0, sk0, k0, m0, l0 = _outputs(ctx, text, _native.make_params(**base))
        assert st0["spill_pieces"] == 0
        st1, sk1, k1, m1, l1 = _outputs(ctx, text, _native.make_params(**base, spill_mb=1))
        assert st1["spill_pieces"] > 1 and st1["spill_ranges"] > 1
        assert st1["superkmers"] == st0["superkmers"] and st1["kmer_instances"] == st0["kmer_instances"]
        assert (_sk_sorted(sk1) == _sk_sorted(sk0)).all()
        a = parity.device_kmers(k0, m0)
        b = parity.device_kmers(k1, m1)
        assert all((x == y).all() for x, y in zip(a[:3], b[:3])) and a[3] and b[3]
        assert l1 == l0
        r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=m, bucket_bits=6, second_bits=2,
                                                             min_multiplicity=2, threads=8,
                                                             hash_kind=oracle.H_CN_RK128 if k > 32 else None))
        assert parity.compare_kmers(k1, m1, r)["equal"]
        assert parity.compare_unitigs(l1, r)["equal"]
    finally:
        ctx.close()


def test_spilled_colored_build():
    rng = np.random.default_rng(5)
    anc = synth.random_genome(80_000, rng)
    gs = [synth.indels(synth.substitute(anc, float(rng.uniform(0.002, 0.02)), rng), 0.001, 20, rng) for _ in range(6)]
    text, off, ln, col = synth.pack_sequences(gs, list(range(6)))
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=31, m=10, bucket_bits=6, second_bits=1, min_multiplicity=1, keep_kmers=True,
                                spill_mb=1)
        ctx.build_text(text, p)
        assert ctx.stats()["spill_ranges"] > 1
        ctx.colors(off, col, 6)
        keys, _ = ctx.kmers()
        r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=6, second_bits=1, threads=8,
                                                             colors=True), seq_colors=col)
        assert parity.compare_color_sets(keys, ctx.kmer_subsets(), ctx.subsets(), r)["equal"]
    finally:
        ctx.close()
