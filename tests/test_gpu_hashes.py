"""Device hash families against the oracle's restatement of crates/hashes, bit for bit."""
import numpy as np
import pytest

import oracle
from ggcat_gb300 import _native

pytestmark = pytest.mark.gpu

# device kind -> oracle kind
KINDS = {0: oracle.H_CN_SEQ64, 1: oracle.H_FW_SEQ64, 2: oracle.H_CN_SEQ128, 3: oracle.H_FW_SEQ128,
         4: oracle.H_CN_RK128, 5: oracle.H_FW_RK128}


@pytest.fixture(scope="module")
def ctx():
    c = _native.GpuContext(0)
    yield c
    c.close()


def _text(seed, n=5000):
    rng = np.random.default_rng(seed)
    t = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, size=n)].copy()
    t[rng.integers(0, n, size=20)] = ord("N")
    return t


def _device_hashes(ctx, torch, text, k, kind):
    d = torch.from_numpy(text).cuda()
    out = torch.empty(2 * len(text), dtype=torch.int64, device="cuda")
    ctx.kmer_hashes(d.data_ptr(), d.numel(), k, kind, out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint64).reshape(-1, 2)


def _expected(text, k, okind):
    """oracle hashes per valid window (runs split at N)."""
    exp = np.full((len(text), 2), np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    cb = oracle.compress(text)
    valid = np.isin(text, np.frombuffer(b"ACGT", np.uint8))
    i = 0
    while i < len(text):
        if not valid[i]:
            i += 1
            continue
        j = i
        while j < len(text) and valid[j]:
            j += 1
        if j - i >= k:
            h = oracle.hash_iter(okind, cb[i:j], k)
            canon = okind in (oracle.H_CN_SEQ64, oracle.H_CN_SEQ128, oracle.H_CN_RK128)
            for t, row in enumerate(h):
                fw = int(row[0]) | (int(row[1]) << 64)
                rc = int(row[2]) | (int(row[3]) << 64)
                v = min(fw, rc) if canon else fw
                exp[i + t] = (v & ((1 << 64) - 1), v >> 64)
        i = j
    return exp


@pytest.mark.parametrize("kind,k", [(0, 31), (0, 32), (1, 21), (2, 63), (2, 33), (3, 64), (4, 63), (4, 101), (5, 31)])
def test_kmer_hashes_match_oracle(ctx, kind, k):
    torch = pytest.importorskip("torch")
    text = _text(kind * 100 + k)
    got = _device_hashes(ctx, torch, text, k, kind)
    exp = _expected(text, k, KINDS[kind])
    assert (got == exp).all()


@pytest.mark.parametrize("m", [10, 12])
def test_nthash_minimizer_values_match_oracle(ctx, m):
    torch = pytest.importorskip("torch")
    text = _text(m, 3000)
    got = _device_hashes(ctx, torch, text, m, 6)
    cb = oracle.compress(text)
    valid = np.isin(text, np.frombuffer(b"ACGT", np.uint8))
    for i in range(len(text) - m + 1):
        if not valid[i:i + m].all():
            assert got[i, 0] == np.uint64(0xFFFFFFFFFFFFFFFF)
            continue
        fw, rc = oracle.nthash(cb[i:i + m], m)
        v = (min(int(fw[0]), int(rc[0])) << 1 & ((1 << 64) - 1)) | int(int(fw[0]) != int(rc[0]))
        assert int(got[i, 0]) == v and int(got[i, 1]) == 0
