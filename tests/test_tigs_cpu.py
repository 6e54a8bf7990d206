"""Greedy matchtigs, eulertigs and pathtigs of maximal unitigs (ggcat_gpu_compute_tigs, host
code): the k-mer spectrum is kept, eulertigs and pathtigs hold every k-mer once, the eulertig
count is the minimum (per connected component of the unitig graph max(1, sum of binode
imbalances / 2), computed here independently), and greedy matchtigs are never longer in total
than eulertigs.  The unitigs come from tests/naive.py's compaction of small k-mer sets built to
have tips, bubbles, cycles and (k-1)-mers or k-mers that are their own reverse complement."""
import random

import numpy as np
import pytest

import naive
from ggcat_gb300 import _native


def _arrays(unitigs):
    seqs = [s for s, _ in unitigs]
    lens = np.array([len(s) for s in seqs], np.uint64)
    off = np.zeros(len(seqs), np.uint64)
    if len(seqs) > 1:
        off[1:] = np.cumsum(lens[:-1])
    return np.frombuffer(b"".join(seqs), np.uint8).copy() if seqs else np.zeros(0, np.uint8), off, lens


def _strings(b, o, l):
    return [bytes(b[int(x):int(x) + int(y)]) for x, y in zip(o, l)]


def _kmers(strings, k):
    out = []
    for s in strings:
        out += [naive.canon(s[i:i + k]) for i in range(len(s) - k + 1)]
    return out


def _kmer_set(rng, k, n_seqs, length, mutate):
    base = bytes(rng.choice(b"ACGT") for _ in range(length))
    seqs = [base]
    for _ in range(n_seqs - 1):
        s = bytearray(base)
        for _ in range(mutate):
            s[rng.randrange(length)] = rng.choice(b"ACGT")
        a = rng.randrange(length // 2)
        seqs.append(bytes(s[a:a + rng.randrange(length // 4, length - a + 1)]))
    kmers = set()
    for s in seqs:
        for i in range(len(s) - k + 1):
            kmers.add(naive.canon(s[i:i + k]))
    return kmers


CASES = [
    # (k, sequences, length, substitutions per copy, seed)
    (5, 6, 60, 3, 1),       # dense: palindromic 4-mers, many junctions
    (6, 5, 80, 4, 2),       # even k: palindromic k-mers
    (7, 8, 120, 5, 3),
    (11, 10, 400, 6, 4),
    (31, 12, 2000, 10, 5),
    (32, 6, 1500, 8, 6),
    (65, 5, 1200, 6, 7),    # (k-1)-mers over 128 bits
]


@pytest.mark.parametrize("k,n_seqs,length,mutate,seed", CASES)
def test_tigs_keep_the_spectrum_and_eulertigs_are_minimal(k, n_seqs, length, mutate, seed):
    rng = random.Random(seed)
    kmers = _kmer_set(rng, k, n_seqs, length, mutate)
    unitigs = naive.maximal_unitigs(kmers, k)
    b, o, l = _arrays(unitigs)
    seqs = [s for s, _ in unitigs]
    total_kmers = sum(len(s) - k + 1 for s in seqs)
    assert total_kmers == len(kmers)
    res = {}
    for mode in (_native.TIGS_EULERTIGS, _native.TIGS_PATHTIGS, _native.TIGS_GREEDY_MATCHTIGS):
        tb, to, tl = _native.compute_tigs(b, o, l, k, mode)
        tigs = _strings(tb, to, tl)
        assert all(len(t) >= k for t in tigs)
        got = _kmers(tigs, k)
        assert set(got) == kmers
        if mode != _native.TIGS_GREEDY_MATCHTIGS:
            assert len(got) == len(kmers)  # every k-mer once
            assert int(tl.sum()) == total_kmers + len(tigs) * (k - 1)
        res[mode] = tigs
    lb = naive.tig_lower_bound(seqs, k)
    assert len(res[_native.TIGS_EULERTIGS]) == lb
    assert len(res[_native.TIGS_PATHTIGS]) >= lb
    eul_chars = sum(len(t) for t in res[_native.TIGS_EULERTIGS])
    mt_chars = sum(len(t) for t in res[_native.TIGS_GREEDY_MATCHTIGS])
    assert mt_chars <= eul_chars
    assert len(res[_native.TIGS_GREEDY_MATCHTIGS]) <= lb


def test_greedy_matchtigs_join_through_a_short_bridge():
    """Two Y junctions joined by a short unitig M of three k-mers (A1, A2 -> M -> B1, B2):
    eulertigs need three strings (A1 M B1, A2, B2); greedy matchtigs join A2's end to B2's
    start through M (three repeated k-mers, three characters instead of the k-1 of a new
    string), two strings and k-4 characters fewer."""
    k = 11
    rng = random.Random(9)

    def rnd(n):
        return bytes(rng.choice(b"ACGT") for _ in range(n))

    core = rnd(k - 1 + 3)
    a1, b1 = rnd(30) + b"A", b"C" + rnd(30)
    a2, b2 = rnd(30) + b"G", b"T" + rnd(30)
    kmers = {naive.canon(s[i:i + k]) for s in (a1 + core + b1, a2 + core + b2) for i in range(len(s) - k + 1)}
    unitigs = naive.maximal_unitigs(kmers, k)
    assert len(unitigs) == 5
    b, o, l = _arrays(unitigs)
    eul = _strings(*_native.compute_tigs(b, o, l, k, _native.TIGS_EULERTIGS))
    mt = _strings(*_native.compute_tigs(b, o, l, k, _native.TIGS_GREEDY_MATCHTIGS))
    assert set(_kmers(mt, k)) == kmers and len(_kmers(mt, k)) == len(kmers) + 3
    assert len(eul) == naive.tig_lower_bound([s for s, _ in unitigs], k) == 3
    assert len(mt) == 2
    assert sum(map(len, mt)) == sum(map(len, eul)) - (k - 1) + 3


def test_tigs_of_a_cycle_and_of_nothing():
    k = 9
    rng = random.Random(4)
    ring = bytes(rng.choice(b"ACGT") for _ in range(50))
    circ = ring + ring[:k - 1]
    kmers = {naive.canon(circ[i:i + k]) for i in range(len(circ) - k + 1)}
    unitigs = naive.maximal_unitigs(kmers, k)
    b, o, l = _arrays(unitigs)
    for mode in (2, 3, 4):
        tigs = _strings(*_native.compute_tigs(b, o, l, k, mode))
        assert len(tigs) == 1 and set(_kmers(tigs, k)) == kmers
        assert len(_kmers(tigs, k)) == len(kmers)
        tb, to, tl = _native.compute_tigs(np.zeros(0, np.uint8), np.zeros(0, np.uint64), np.zeros(0, np.uint64), k,
                                          mode)
        assert len(to) == 0 and len(tb) == 0


def test_tigs_reject_bad_input():
    b, o, l = _arrays([(b"ACGTACG", False)])
    with pytest.raises(_native.GgcatGpuError):
        _native.compute_tigs(b, o, l, 9, _native.TIGS_EULERTIGS)  # shorter than k
    with pytest.raises(_native.GgcatGpuError):
        _native.compute_tigs(b, o, l, 5, 7)  # unknown mode
    b2, o2, l2 = _arrays([(b"ACGTNCGTA", False)])
    with pytest.raises(_native.GgcatGpuError):
        _native.compute_tigs(b2, o2, l2, 5, _native.TIGS_PATHTIGS)


def test_compute_tigs_c_abi_size_query_and_capacity():
    """NULL outputs return the sizes; a buffer smaller than the strings is refused (not
    overrun); Σ len bytes and n entries hold any mode's output."""
    import ctypes as C

    k = 7
    rng = random.Random(11)
    kmers = _kmer_set(rng, k, 6, 120, 5)
    unitigs = naive.maximal_unitigs(kmers, k)
    b, o, l = _arrays(unitigs)
    L = _native.load()
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    for mode in (2, 3, 4):
        n_out, b_out = C.c_uint64(), C.c_uint64()
        rc = L.ggcat_gpu_compute_tigs(P(b), P(o), P(l), len(o), k, mode, None, 0, None, None, 0, C.byref(n_out),
                                      C.byref(b_out))
        assert rc == 0 and 0 < n_out.value <= len(o) and 0 < b_out.value <= int(l.sum())
        ob = np.zeros(b_out.value, np.uint8)
        oo = np.zeros(n_out.value, np.uint64)
        ol = np.zeros(n_out.value, np.uint64)
        small = np.zeros(b_out.value - 1, np.uint8)
        rc = L.ggcat_gpu_compute_tigs(P(b), P(o), P(l), len(o), k, mode, P(small), small.size, P(oo), P(ol), oo.size,
                                      C.byref(n_out), C.byref(b_out))
        assert rc == -1  # GGCAT_GPU_EINVAL
        rc = L.ggcat_gpu_compute_tigs(P(b), P(o), P(l), len(o), k, mode, P(ob), ob.size, P(oo), P(ol), oo.size,
                                      C.byref(n_out), C.byref(b_out))
        assert rc == 0 and int(ol.sum()) == ob.size
        tb, to, tl = _native.compute_tigs(b, o, l, k, mode)
        assert bytes(tb) == bytes(ob) and (to == oo).all() and (tl == ol).all()
