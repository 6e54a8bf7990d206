"""The order-free parity checks (oracle/parity.py) on oracle outputs: a build compared with
itself in device form is equal, and a planted difference (one multiplicity, one k-mer, one
colour, one unitig base, one query count) is caught.  CPU only."""
import numpy as np

import oracle
from oracle import parity
from ggcat_gb300 import synth


def _genomes_build(colors=False, k=31):
    rng = np.random.default_rng(77)
    anc = synth.random_genome(20_000, rng)
    gs = [synth.indels(synth.substitute(anc, 0.01, rng), 0.001, 10, rng) for _ in range(4)]
    text, off, ln, col = synth.pack_sequences(gs, list(range(4)))
    p = oracle.params(k=k, m=10 if k <= 32 else 12, bucket_bits=4, second_bits=2, threads=2, colors=colors)
    return oracle.build_graph(text, off, ln, p, seq_colors=col if colors else None), text, off, ln


def _device_form(r, k):
    """The oracle's k-mers as the device dumps them: every k-mer reported by some copies (as
    if from several sub-buckets), shuffled."""
    lo, hi, mult = r.kmers()
    rng = np.random.default_rng(1)
    reps = rng.integers(1, 3, size=lo.size)
    idx = rng.permutation(np.repeat(np.arange(lo.size), reps))
    keys = lo[idx] if k <= 32 else np.stack([lo[idx], hi[idx]], axis=1)
    return keys, mult[idx], idx


def test_kmers_equal_and_planted_differences():
    r, *_ = _genomes_build()
    keys, mult, idx = _device_form(r, 31)
    assert parity.compare_kmers(keys, mult, r)["equal"]
    bad = mult.copy()
    bad[5] += 1
    assert not parity.compare_kmers(keys, bad, r)["equal"]
    keep = idx != idx[0]  # one k-mer missing entirely
    assert not parity.compare_kmers(keys[keep], mult[keep], r)["equal"]


def test_kmers_equal_k63():
    r, *_ = _genomes_build(k=63)
    keys, mult, _ = _device_form(r, 63)
    assert keys.ndim == 2
    assert parity.compare_kmers(keys, mult, r)["equal"]
    bad = keys.copy()
    bad[3, 1] ^= 1
    assert not parity.compare_kmers(bad, mult, r)["equal"]


def test_unitigs_equal_and_planted_difference():
    r, *_ = _genomes_build()
    lines = r.unitigs()
    assert parity.compare_unitigs(lines, r)["equal"]
    b = bytearray(lines)
    b[10] = ord("A") if b[10] != ord("A") else ord("C")
    assert not parity.compare_unitigs(bytes(b), r)["equal"]


def test_color_sets_equal_and_planted_difference():
    r, *_ = _genomes_build(colors=True)
    lo, hi, _ = r.kmers()
    olo, ohi, obm = parity.oracle_color_bitmaps(r, 1)
    subsets, sid = np.unique(obm, axis=0, return_inverse=True)
    sid = sid.reshape(-1)
    rng = np.random.default_rng(3)
    reps = rng.integers(1, 3, size=olo.size)
    idx = rng.permutation(np.repeat(np.arange(olo.size), reps))
    assert parity.compare_color_sets(olo[idx], sid[idx], subsets, r)["equal"]
    # one copy of a k-mer resolving to another subset
    bad = sid[idx].copy()
    bad[0] = (bad[0] + 1) % subsets.shape[0]
    assert not parity.compare_color_sets(olo[idx], bad, subsets, r)["equal"]
    # a duplicated subset row
    dup = np.concatenate([subsets, subsets[:1]])
    assert not parity.compare_color_sets(olo[idx], sid[idx], dup, r)["equal"]


def test_query_counts():
    m = np.array([3, 0, 5], np.uint64)
    c = np.array([[1, 2], [0, 0], [5, 5]], np.uint64)
    assert parity.compare_query_counts(m, c, m.copy(), c.copy())["equal"]
    c2 = c.copy()
    c2[2, 1] = 4
    assert not parity.compare_query_counts(m, c2, m, c)["equal"]
    assert not parity.compare_query_counts(m, None, m + 1, None)["equal"]
