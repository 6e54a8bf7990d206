"""GPU builds of the benchmark configurations' inputs, at their stated sizes or large
slices of them, against the oracle's builds of the same inputs (order-free comparisons of
oracle/parity.py): the 3 x 5 Mbp genomes in full, a 100 Mbp read set of the skewed-read
shape, a 50 Mbp long-k read set (k=63, Rabin-Karp u128), the first 32 genomes of the
coloured workload (colour sets) with 2,000 coloured queries of the query workload."""
import os

import numpy as np
import pytest

import oracle
from oracle import parity
from ggcat_gb300 import _native, synth

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def ctx():
    c = _native.GpuContext(0)
    yield c
    c.close()


def _build_parity(ctx, w, hash_kind=None):
    hk = _native.GGCAT_HASH_RABIN_KARP128 if hash_kind == "rk128" else _native.GGCAT_HASH_SEQHASH
    p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6,
                            min_multiplicity=w.min_multiplicity, hash_kind=hk, keep_kmers=True)
    ctx.build_text(w.text, p)
    keys, mult = ctx.kmers()
    ctx.link(w.k)
    bases, uo, ul, uf = ctx.unitigs()
    lines = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, w.k)
    op = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6, min_multiplicity=w.min_multiplicity,
                       threads=THREADS, hash_kind=oracle.H_CN_RK128 if hash_kind == "rk128" else None)
    r = oracle.build_graph(w.text, w.seq_off, w.seq_len, op)
    km = parity.compare_kmers(keys, mult, r)
    un = parity.compare_unitigs(lines, r)
    assert km["kmers_oracle"] > 0 and un["unitigs_oracle"] > 0
    assert km["equal"], km
    assert un["equal"], un


def test_genomes_3x5Mbp_full(ctx):
    _build_parity(ctx, synth.config_genomes())


def test_skewed_reads_100Mbp(ctx):
    # the skewed-read shape (2% of the genome in 500-bp repeats copied 20-200 times, 20x
    # 150-bp reads, 0.5% substitutions, 0.01% N, min multiplicity 2) on a 5 Mbp genome
    _build_parity(ctx, synth.config_skewed_reads(genome_len=5_000_000))


def test_longk_reads_50Mbp(ctx):
    _build_parity(ctx, synth.config_long_k(genome_len=2_500_000), hash_kind="rk128")


def test_colored_32_genomes_and_2000_queries(ctx):
    w = synth.config_colored(n_genomes=32)
    p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=1, min_multiplicity=1,
                            keep_kmers=True)
    ctx.build_text(w.text, p)
    ctx.colors(w.seq_off, w.seq_color, 32)
    keys, _ = ctx.kmers()
    op = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=1, min_multiplicity=1, threads=THREADS,
                       colors=True)
    r = oracle.build_graph(w.text, w.seq_off, w.seq_len, op, seq_colors=w.seq_color)
    cs = parity.compare_color_sets(keys, ctx.kmer_subsets(), ctx.subsets(), r)
    assert cs["equal"], cs
    ctx.query_index_colored()
    genomes = [w.text[int(o):int(o) + int(n)] for o, n in zip(w.seq_off.tolist(), w.seq_len.tolist())]
    qt, qo, ql, _ = synth.query_workload(genomes, 2000)
    ctx.query_submit(0, qt, qo, ql)
    matched = ctx.query_wait(0)
    counts = ctx.query_color_counts(0)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    em, _, epc = oracle.query(lo, hi, qt, qo, ql, w.k, gc_off=coff, gc_colors=ccol, ncolors=32)
    q = parity.compare_query_counts(matched, counts, em, epc)
    assert q["equal"] and q["matched_kmers"] > 0, q
