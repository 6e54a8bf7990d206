"""Port of the reference's hash property harness (crates/hashes/src/lib.rs:265-454)
applied to the oracle's hash families, plus the reference's known-answer packing
vector (crates/io/src/compressed_read.rs:1011-1023).  These pin the oracle."""
import numpy as np
import pytest

import oracle

DEC = np.frombuffer(b"ACTG", np.uint8)


def gen_bases(n, seed):
    # crates/hashes/src/lib.rs:226-234 draws uniform 2-bit codes from a seeded PCG32;
    # the properties checked below hold for any input, so any seeded generator serves.
    rng = np.random.default_rng(seed)
    return DEC[rng.integers(0, 4, size=n)]


def key(row, canonical):
    fw = int(row[0]) | (int(row[1]) << 64)
    rc = int(row[2]) | (int(row[3]) << 64)
    return min(fw, rc) if canonical else fw


KINDS = [
    # (kind, ks, canonical, invertible, bits)
    (oracle.H_CN_SEQ64, list(range(2, 32)), True, True, 64),
    (oracle.H_FW_SEQ64, list(range(2, 32)), False, True, 64),
    (oracle.H_CN_SEQ128, list(range(2, 64, 3)), True, True, 128),
    (oracle.H_FW_SEQ128, list(range(2, 64, 5)), False, True, 128),
    (oracle.H_CN_RK64, [2, 3, 5, 8, 15, 31, 32, 33, 63, 64, 65, 100, 257], True, False, 64),
    (oracle.H_FW_RK64, [2, 3, 15, 31, 63, 100], False, False, 64),
    (oracle.H_CN_RK128, [2, 3, 5, 8, 15, 31, 32, 33, 63, 64, 65, 100, 257, 1000], True, False, 128),
    (oracle.H_FW_RK128, [2, 15, 31, 63, 129], False, False, 128),
]


@pytest.mark.parametrize("kind,ks,canonical,invertible,bits", KINDS)
def test_hash_function_properties(kind, ks, canonical, invertible, bits):
    for k in ks:
        bases = gen_bases(k * 10, 773 + k)
        cb = oracle.compress(bases)
        hashes = oracle.hash_iter(kind, cb, k)
        keys = [key(r, canonical) for r in hashes]
        # distribution test: no collisions between different k-mers for >= 64-bit hashes
        seen = {}
        for i, h in enumerate(keys):
            s = bases[i : i + k].tobytes()
            if h in seen:
                assert seen[h] == s or (canonical and seen[h] == _rc(s)), f"collision k={k}"
            seen[h] = s
        # double hash test
        d = oracle.hash_iter(kind, np.concatenate([cb, cb]), k)
        n = len(bases) - k + 1
        assert (d[:n] == d[n + k - 1 :]).all()
        # canonical test
        if canonical:
            rcb = oracle.compress(np.frombuffer(_rc(bases.tobytes()), np.uint8))
            rh = oracle.hash_iter(kind, rcb, k)
            assert keys == [key(r, True) for r in rh][::-1]
        # manual forward + reverse roll test
        for i in range(len(hashes) - 1):
            assert oracle.roll_fw(kind, hashes[i], k, cb[i], cb[i + k]) == tuple(int(x) for x in hashes[i + 1])
        for i in range(len(hashes) - 1, 0, -1):
            assert oracle.roll_bw(kind, hashes[i], k, cb[i + k - 1], cb[i - 1]) == tuple(int(x) for x in hashes[i - 1])
        # manual remove tests (k-1 hashes)
        lh = oracle.hash_iter(kind, cb, k - 1) if k > 1 else None
        if k > 2 or not (kind in (oracle.H_CN_RK64, oracle.H_CN_RK128, oracle.H_FW_RK64, oracle.H_FW_RK128)):
            for i in range(len(hashes)):
                assert oracle.remove_fw(kind, hashes[i], k, cb[i]) == tuple(int(x) for x in lh[i + 1])
                assert oracle.remove_bw(kind, hashes[i], k, cb[i + k - 1]) == tuple(int(x) for x in lh[i])
        # invertibility test: the seq-hash value is the 2-bit packed k-mer (LE)
        if invertible:
            for i in range(0, len(bases) - k, max(1, k // 3)):
                h = keys[i]
                dec = bytes(DEC[(h >> (2 * j)) & 3] for j in range(k))
                s = bases[i : i + k].tobytes()
                assert dec == s or dec == _rc(s)


def _rc(s: bytes) -> bytes:
    return s.translate(bytes.maketrans(b"ACGT", b"TGCA"))[::-1]


def test_nthash_matches_definition():
    """nt-hash rolling values equal the per-m-mer definition XOR rotl(h(c_i), m-1-i)."""
    M = 0x397F178C6AE330F9
    mask = (1 << 64) - 1

    def rotl(x, r):
        r %= 64
        return ((x << r) | (x >> (64 - r))) & mask if r else x

    bases = gen_bases(300, 11)
    cb = oracle.compress(bases)
    for m in (1, 2, 5, 10, 12, 21, 64, 65):
        fw, rc = oracle.nthash(cb, m)
        for i in range(0, len(fw), 7):
            f = 0
            r = 0
            for j in range(m):
                c = int(cb[i + j])
                f ^= rotl(((2 * c + 1) * M) & mask, m - 1 - j)
                r ^= rotl(((((2 * c) ^ 4) + 1) * M) & mask, j)
            assert int(fw[i]) == f and int(rc[i]) == r


@pytest.mark.parametrize("m", [10, 11, 12])
def test_nthash_canonical_minimizer_values_collision_free(m):
    """Two m-mers that are neither equal nor reverse complements never share the
    canonical minimizer value min(fw,rc)<<1: the sliding-window minimum can then be
    computed from (value, count) alone, exactly as the batched queue reports it."""
    n = 4**m
    codes = np.arange(n, dtype=np.uint64)
    # all m-mers as 2-bit sequences (A0 C1 T2 G3 code order), first base = high digit
    seqs = np.zeros((n, m), np.uint8)
    x = codes.copy()
    for j in range(m - 1, -1, -1):
        seqs[:, j] = (x & 3).astype(np.uint8)
        x >>= np.uint64(2)
    M = np.uint64(0x397F178C6AE330F9)
    fw = np.zeros(n, np.uint64)
    rc = np.zeros(n, np.uint64)
    for j in range(m):
        c = seqs[:, j].astype(np.uint64)
        hf = (np.uint64(2) * c + np.uint64(1)) * M
        hr = (((np.uint64(2) * c) ^ np.uint64(4)) + np.uint64(1)) * M
        rf = np.uint64((m - 1 - j) % 64)
        rr = np.uint64(j % 64)
        fw ^= (hf << rf) | (hf >> ((np.uint64(64) - rf) % np.uint64(64))) if rf else hf
        rc ^= (hr << rr) | (hr >> ((np.uint64(64) - rr) % np.uint64(64))) if rr else hr
    val = np.minimum(fw, rc) << np.uint64(1)
    # canonical identity of the m-mer: min(code, rc code)
    rcodes = np.zeros(n, np.uint64)
    for j in range(m):
        rcodes = (rcodes << np.uint64(2)) | (seqs[:, m - 1 - j].astype(np.uint64) ^ np.uint64(2))
    ident = np.minimum(codes, rcodes)
    order = np.lexsort((ident, val))
    v = val[order]
    idn = ident[order]
    same_val = v[1:] == v[:-1]
    assert not (same_val & (idn[1:] != idn[:-1])).any()


def test_known_answer_rc_packing():
    """compressed_read.rs:1011-1023: packing the reverse complement of a read."""
    bases = b"ACGTACGCGGTAGCTAAGCATCGATGCCGATCGTGTTTAACCATG"
    expected_rc = b"CATGGTTAAACACGATCGGCATCGATGCTTAGCTACCGCGTACGT"
    assert _rc(bases) == expected_rc
    cb = oracle.compress(bases)
    # 2-bit code A0 C1 T2 G3, complement = code ^ 2
    rc_codes = (cb[::-1] ^ 2)
    assert bytes(DEC[rc_codes]) == expected_rc
