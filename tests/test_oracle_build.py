"""The oracle's build (bucketing -> per-sub-bucket merge -> link) against an
independent naive global restatement: same surviving canonical k-mers with the same
multiplicities, same canonical maximal-unitig set."""
import numpy as np
import pytest

import oracle
from ggcat_gb300 import synth
from tests import naive


def _kmers_to_strings(lo, hi, k):
    dec = b"ACTG"
    out = []
    for a, b in zip(lo.tolist(), hi.tolist()):
        v = a | (b << 64)
        out.append(naive.canon(bytes(dec[(v >> (2 * i)) & 3] for i in range(k))))
    return out


def _run(seqs, k=31, m=10, bucket_bits=4, second_bits=2, min_mult=1, threads=2, hash_kind=None):
    text, off, ln, col = synth.pack_sequences([np.frombuffer(s, np.uint8) for s in seqs])
    p = oracle.params(k=k, m=m, bucket_bits=bucket_bits, second_bits=second_bits, min_multiplicity=min_mult,
                      threads=threads, hash_kind=hash_kind)
    r = oracle.build_graph(text, off, ln, p)
    lo, hi, mult = r.kmers()
    got_k = dict(zip(_kmers_to_strings(lo, hi, k), mult.tolist()))
    exp_all = naive.kmer_counts(seqs, k)
    exp_k = {x: c for x, c in exp_all.items() if c >= min_mult}
    assert got_k == exp_k
    exp_u = naive.canonical_set(naive.maximal_unitigs(set(exp_k), k), k)
    assert r.unitigs() == exp_u
    return r


def _genome_mix(seed, L=6000, copies=3, sub=0.01, reads=0):
    rng = np.random.default_rng(seed)
    g = synth.random_genome(L, rng)
    g = synth.add_repeats(g, 0.05, 80, 2, 6, rng)
    seqs = [g.tobytes()]
    for _ in range(copies - 1):
        seqs.append(synth.indels(synth.substitute(g, sub, rng), 0.002, 5, rng).tobytes())
    if reads:
        rr = synth.sample_reads(g, reads, 100, 0.01, 0.002, rng)
        seqs.extend(r.tobytes() for r in rr)
    return seqs


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_build_genomes_min1(seed):
    _run(_genome_mix(seed))


@pytest.mark.parametrize("seed", [4, 5])
def test_build_reads_min2(seed):
    _run(_genome_mix(seed, L=3000, copies=1, reads=400), min_mult=2)


def test_build_low_complexity_and_n():
    seqs = [b"A" * 200 + b"N" + b"ACGT" * 50 + b"nnn" + b"acgtacgatcgatcgatcagctagcatcgactagcatcgac" * 3,
            b"AC" * 100, b"GATTACA" * 40 + b"N" * 5 + b"TTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTT"]
    _run(seqs, bucket_bits=3, second_bits=1)


def test_build_rk128_matches_seqhash():
    seqs = _genome_mix(7, L=2500, copies=2)
    a = _run(seqs, hash_kind=oracle.H_CN_SEQ64)
    b = _run(seqs, hash_kind=oracle.H_CN_RK128)
    assert a.unitigs() == b.unitigs()


def test_build_k63_seq128():
    seqs = _genome_mix(8, L=2500, copies=2)
    _run(seqs, k=63, m=12, hash_kind=oracle.H_CN_SEQ128)


def test_rabin_karp_selects_the_same_kmers_as_seqhash():
    """The device keys its tables by the canonical packed k-mer for every hash kind; the
    reference's Rabin-Karp u128 keys give the same multiplicities and unitigs (k = 63)."""
    rng = np.random.default_rng(3)
    g = synth.random_genome(40_000, rng)
    gs = [g, synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng)]
    text, off, ln, _ = synth.pack_sequences(gs)
    res = []
    for kind in (oracle.H_CN_SEQ128, oracle.H_CN_RK128):
        r = oracle.build_graph(text, off, ln, oracle.params(k=63, m=12, bucket_bits=6, second_bits=2,
                                                            hash_kind=kind, threads=4))
        lo, hi, mult = r.kmers()
        res.append((sorted(zip(lo.tolist(), hi.tolist(), mult.tolist())), r.unitigs()))
    assert res[0] == res[1]


def test_build_colors_match_naive():
    """Per-k-mer colour sets (MultipleColorsManager semantics: sorted distinct colours of all
    occurrences), on inputs whose k-mer maps grow while they fill."""
    rng = np.random.default_rng(8)
    seqs, cols = [], []
    for c in range(5):
        g = synth.random_genome(3000, rng)
        seqs += [g.tobytes(), synth.substitute(g, 0.02, rng).tobytes()]
        cols += [c, (c + 1) % 5]
    text, off, ln, _ = synth.pack_sequences([np.frombuffer(s, np.uint8) for s in seqs])
    col = np.asarray(cols, np.uint32)
    r = oracle.build_graph(text, off, ln, oracle.params(k=31, m=10, bucket_bits=3, second_bits=1, threads=2,
                                                        colors=True), seq_colors=col)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    names = _kmers_to_strings(lo, hi, 31)
    got = {names[i]: tuple(int(c) for c in ccol[coff[i]:coff[i + 1]]) for i in range(len(names))}
    assert got == naive.kmer_colors(seqs, cols, 31)


@pytest.mark.parametrize("k,m", [(20, 8), (32, 10), (48, 12), (64, 14)])
def test_build_even_k_palindromes(k, m):
    """Even k: hairpins s + revcomp(s) and short palindromes pasted into a genome give k-mers
    equal to their reverse complement; the oracle's walk must stop on them as the naive
    global walk does (a path that enters one ends there), so the k-mer sets and the unitig
    sets are equal.  Multiplicities are equal except at some palindromic k-mers: the two
    m-mers that tie for such a k-mer's minimum are each other's mirror, the reference's
    splitter cuts there (same value at a new position, batch_minqueue.rs:150-156) into two
    records of the same bucket that both hold the k-mer, one of them with a single ignored
    flag, so MapEntry::get_kmer_multiplicity (map_entry.rs:79-84) does not halve the count
    and the k-mer reads twice per occurrence.  The oracle restates that."""
    rng = np.random.default_rng(k)
    seqs = []
    for _ in range(40):
        s = synth.random_genome(int(rng.integers(k // 2, 3 * k)), rng)
        seqs.append(np.concatenate([s, synth.revcomp(s)]).tobytes())
    g = synth.random_genome(3000, rng).copy()
    for _ in range(30):
        half = synth.random_genome(k // 2, rng)
        pal = np.concatenate([half, synth.revcomp(half)])
        for p in rng.integers(0, len(g) - k, size=int(rng.integers(1, 4))).tolist():
            g[p:p + k] = pal
    seqs.append(g.tobytes())
    seqs += [r.tobytes() for r in synth.sample_reads(g, 150, 120, 0.003, 0.0, rng)]
    text, off, ln, _ = synth.pack_sequences([np.frombuffer(s, np.uint8) for s in seqs])
    r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=m, bucket_bits=4, second_bits=2, threads=2))
    lo, hi, mult = r.kmers()
    got = dict(zip(_kmers_to_strings(lo, hi, k), mult.tolist()))
    exp = naive.kmer_counts(seqs, k)
    assert set(got) == set(exp)
    pals = {x for x in exp if x == naive.rc(x)}
    assert len(pals) > 20
    for x, c in exp.items():
        if x in pals:
            assert c <= got[x] <= 2 * c, (x, got[x], c)
        else:
            assert got[x] == c, (x, got[x], c)
    assert r.unitigs() == naive.canonical_set(naive.maximal_unitigs(set(exp), k), k)


def _wide_kmers_to_strings(words, k):
    dec = b"ACTG"
    out = []
    for w in words.tolist():
        v = w[0] | (w[1] << 64) | (w[2] << 128) | (w[3] << 192)
        out.append(naive.canon(bytes(dec[(v >> (2 * i)) & 3] for i in range(k))))
    return out


@pytest.mark.parametrize("k,m,min_mult", [(65, 14, 1), (75, 16, 2), (101, 25, 1), (128, 32, 1), (96, 20, 1)])
def test_build_long_k_rabin_karp(k, m, min_mult):
    """k > 64: the reference keys k-mers by the canonical Rabin-Karp u128 hash
    (crates/api/src/utils.rs:10-69); the oracle counts and extends by that hash and reports
    the packed k-mers in 4 words.  Against the naive global computation: same k-mers with the
    same multiplicities, same maximal unitigs (genome copies with variants, read sets, and for
    even k hairpins whose centre k-mer is its own reverse complement)."""
    rng = np.random.default_rng(k)
    seqs = [x.tobytes() for x in synth.sample_reads(synth.random_genome(4000, rng), 200, 300, 0.004, 0.0, rng)]
    seqs += _genome_mix(k, L=3000, copies=2)
    if k % 2 == 0:
        for _ in range(20):
            s = synth.random_genome(int(rng.integers(k // 2, 2 * k)), rng)
            seqs.append(np.concatenate([s, synth.revcomp(s)]).tobytes())
    text, off, ln, _ = synth.pack_sequences([np.frombuffer(s, np.uint8) for s in seqs])
    p = oracle.params(k=k, m=m, bucket_bits=4, second_bits=2, min_multiplicity=min_mult, threads=2,
                      hash_kind=oracle.H_CN_RK128)
    r = oracle.build_graph(text, off, ln, p)
    words, mult = r.kmers_wide()
    got = dict(zip(_wide_kmers_to_strings(words, k), mult.tolist()))
    exp_all = naive.kmer_counts(seqs, k)
    exp = {x: c for x, c in exp_all.items() if c >= min_mult}
    assert set(got) == set(exp)
    for x, c in exp.items():
        if x == naive.rc(x):  # the splitter's double count at rc-symmetric k-mers (even k)
            assert c <= got[x] <= 2 * c
        else:
            assert got[x] == c
    assert r.unitigs() == naive.canonical_set(naive.maximal_unitigs(set(exp), k), k)


def test_seq_hash_rejects_k_above_64():
    text, off, ln, _ = synth.pack_sequences([np.frombuffer(b"ACGT" * 40, np.uint8)])
    with pytest.raises(ValueError):
        oracle.build_graph(text, off, ln, oracle.params(k=65, m=14, hash_kind=oracle.H_CN_SEQ128))
