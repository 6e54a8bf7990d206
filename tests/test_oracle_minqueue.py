"""The oracle's BatchMinQueue restatement against the window-minimum specification
of crates/hashes/src/rolling/minqueue_testing.rs:335-370: each reported minimum equals
the window's minimum (unique flag masked), and its unique flag (bit 0) is cleared
exactly when the minimum occurs more than once in the window (or its m-mer is
rc-symmetric, whose flag bit was never set)."""
import numpy as np
import pytest

import oracle


def spec_window(vals, w):
    out = []
    for j in range(len(vals) - w + 1):
        win = vals[j : j + w]
        masked = [v & ~1 for v in win]
        mv = min(masked)
        occ = [v for v in win if v & ~1 == mv]
        flag = 1 if (len(occ) == 1 and occ[0] & 1) else 0
        out.append(mv | flag)
    return out


@pytest.mark.parametrize("w", [2, 3, 5, 13, 21, 51])
@pytest.mark.parametrize("spread", [8, 1000, 1 << 62])
def test_minimizers_match_spec(w, spread):
    rng = np.random.default_rng(w * 7 + spread % 97)
    n = 600
    vals = (rng.integers(0, spread, size=n, dtype=np.uint64) << np.uint64(1)) | (rng.random(n) < 0.9).astype(np.uint64)
    got = oracle.minqueue_minimizers(w, vals)
    assert [int(x) for x in got["v"]] == spec_window([int(v) for v in vals], w)


def test_splits_positions():
    """Splits are reported where the minimum value changes, or where a unique minimum
    moves to another position; the final record is at n - size (batch_minqueue.rs:131)."""
    rng = np.random.default_rng(5)
    w = 21
    n = 500
    vals = (rng.integers(0, 300, size=n, dtype=np.uint64) << np.uint64(1)) | np.uint64(1)
    pos, val, last = oracle.minqueue_splits(w, vals)
    mins = oracle.minqueue_minimizers(w, vals)
    exp = []
    for j in range(1, len(mins)):
        a, b = mins[j - 1], mins[j]
        if a["v"] != b["v"] or (a["index"] != b["index"] and b["v"] & 1):
            exp.append(j)
    exp.append(n - w)
    assert [int(p) for p in pos] == exp
    assert last[-1] == 1 and last[:-1].sum() == 0
