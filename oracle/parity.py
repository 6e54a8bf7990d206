"""Order-free parity checks of device outputs against the oracle (test infrastructure only).

Used by ``tests/`` and by ``bench.py``'s CPU-baseline leg, whose oracle run doubles as the
checker of the GPU's output on the same input.  Everything here is vectorised numpy so
that full-size workloads (10^8 k-mers) compare in seconds.

Compared objects, each reduced to a canonical sorted form:
- surviving k-mers with multiplicities (the device reports a k-mer once per sub-bucket it
  occurs in; the copies must agree and are collapsed);
- the canonical maximal-unitig set (lines canonicalised by the oracle's own routine);
- per-k-mer colour sets (device subset ids resolved to bitmaps, oracle colour lists
  turned into bitmaps);
- per-query matched counts and per-colour counts.
"""
from __future__ import annotations

import hashlib

import numpy as np


def _digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def device_kmers(keys: np.ndarray, mult: np.ndarray):
    """Sorted unique (lo, hi, mult) of the device k-mer dump.  ``keys`` is (n,) u64 for
    k <= 32 or (n, 2) u64 (lo, hi) above (see ``compare_kmers_wide`` for k > 64).  Returns
    also whether every copy of a k-mer (one per sub-bucket) carries the same multiplicity."""
    keys = np.asarray(keys)
    mult = np.asarray(mult).astype(np.uint64)
    if keys.ndim == 1:
        lo = keys.astype(np.uint64)
        hi = np.zeros_like(lo)
    else:
        lo = keys[:, 0].astype(np.uint64)
        hi = keys[:, 1].astype(np.uint64)
    order = np.lexsort((mult, lo, hi))
    lo, hi, mult = lo[order], hi[order], mult[order]
    if lo.size == 0:
        return lo, hi, mult, True
    new_key = np.ones(lo.size, bool)
    new_key[1:] = (lo[1:] != lo[:-1]) | (hi[1:] != hi[:-1])
    # copies of one key must have equal multiplicities: after sorting by (hi, lo, mult) a
    # differing copy shows as a change of mult without a change of key
    consistent = bool(((mult[1:] == mult[:-1]) | new_key[1:]).all())
    return lo[new_key], hi[new_key], mult[new_key], consistent


def compare_kmers(keys, mult, oracle_result) -> dict:
    """Surviving k-mers and multiplicities of the device against the oracle's."""
    glo, ghi, gm, consistent = device_kmers(keys, mult)
    olo, ohi, om = oracle_result.kmers()
    order = np.lexsort((olo, ohi))
    olo, ohi, om = olo[order], ohi[order], om[order].astype(np.uint64)
    equal = consistent and glo.size == olo.size and bool(
        (glo == olo).all() and (ghi == ohi).all() and (gm == om).all())
    return {"equal": bool(equal), "kmers_gpu": int(glo.size), "kmers_oracle": int(olo.size),
            "digest_gpu": _digest(glo, ghi, gm), "digest_oracle": _digest(olo, ohi, om)}


def compare_kmers_wide(keys, mult, oracle_result) -> dict:
    """k > 64: the device dump ((n, 4) words) against the oracle's wide k-mers, both reduced
    to sorted unique rows of (w3, w2, w1, w0, mult); every copy of a k-mer must agree."""
    keys = np.asarray(keys, np.uint64).reshape(-1, 4)
    mult = np.asarray(mult).astype(np.uint64)
    rows = np.column_stack([keys[:, 3], keys[:, 2], keys[:, 1], keys[:, 0], mult])
    rows = np.unique(rows, axis=0)
    keys_only = rows[:, :4]
    consistent = keys_only.shape[0] == 0 or bool((keys_only[1:] != keys_only[:-1]).any(axis=1).all())
    ow, om = oracle_result.kmers_wide()
    orows = np.unique(np.column_stack([ow[:, 3], ow[:, 2], ow[:, 1], ow[:, 0], om.astype(np.uint64)]), axis=0)
    equal = consistent and rows.shape == orows.shape and bool((rows == orows).all())
    return {"equal": bool(equal), "kmers_gpu": int(rows.shape[0]), "kmers_oracle": int(orows.shape[0]),
            "digest_gpu": _digest(rows), "digest_oracle": _digest(orows)}


def compare_unitigs(canonical_gpu_lines: bytes, oracle_result) -> dict:
    """Canonical sorted maximal-unitig sets (bytes, one unitig per line)."""
    exp = oracle_result.unitigs()
    return {"equal": canonical_gpu_lines == exp, "unitigs_gpu": canonical_gpu_lines.count(b"\n"),
            "unitigs_oracle": exp.count(b"\n"), "digest_gpu": hashlib.sha256(canonical_gpu_lines).hexdigest()[:16],
            "digest_oracle": hashlib.sha256(exp).hexdigest()[:16]}


def oracle_color_bitmaps(oracle_result, words: int):
    """(lo, hi, bitmaps[n, words]) of the oracle's per-k-mer colour lists, sorted by (hi, lo)."""
    lo, hi, _ = oracle_result.kmers()
    off, cols = oracle_result.kmer_colors()
    n = lo.size
    bm = np.zeros((n, words), np.uint32)
    if cols.size:
        owner = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        np.bitwise_or.at(bm, (owner, (cols // 32).astype(np.int64)), (np.uint32(1) << (cols % 32)).astype(np.uint32))
    order = np.lexsort((lo, hi))
    return lo[order], hi[order], bm[order]


def compare_color_sets(keys, subset_ids, subset_bitmaps, oracle_result) -> dict:
    """Per-k-mer colour sets: device subset ids resolved to their bitmaps (every copy of a
    k-mer must resolve to the same set; every subset must be distinct) against the
    oracle's colour lists."""
    keys = np.asarray(keys)
    bm = np.asarray(subset_bitmaps, np.uint32)
    words = bm.shape[1] if bm.ndim == 2 else 1
    bm = bm.reshape(-1, words)
    distinct_subsets = np.unique(bm, axis=0).shape[0] == bm.shape[0]
    if keys.ndim == 1:
        lo = keys.astype(np.uint64)
        hi = np.zeros_like(lo)
    else:
        lo, hi = keys[:, 0].astype(np.uint64), keys[:, 1].astype(np.uint64)
    sid = np.asarray(subset_ids).astype(np.int64)
    rows = bm[sid]
    # sort by key, then by the set, so that differing copies of a key are adjacent
    order = np.lexsort(tuple(rows[:, w] for w in range(words - 1, -1, -1)) + (lo, hi))
    lo, hi, rows = lo[order], hi[order], rows[order]
    new_key = np.ones(lo.size, bool)
    if lo.size:
        new_key[1:] = (lo[1:] != lo[:-1]) | (hi[1:] != hi[:-1])
        same_row = (rows[1:] == rows[:-1]).all(axis=1)
        consistent = bool((same_row | new_key[1:]).all())
    else:
        consistent = True
    glo, ghi, grows = lo[new_key], hi[new_key], rows[new_key]
    olo, ohi, orows = oracle_color_bitmaps(oracle_result, words)
    equal = consistent and distinct_subsets and glo.size == olo.size and bool(
        (glo == olo).all() and (ghi == ohi).all() and (grows == orows).all())
    return {"equal": bool(equal), "kmers_gpu": int(glo.size), "kmers_oracle": int(olo.size),
            "subsets": int(bm.shape[0]), "digest_gpu": _digest(glo, ghi, grows),
            "digest_oracle": _digest(olo, ohi, orows)}


def compare_query_counts(matched, color_counts, exp_matched, exp_counts) -> dict:
    """Per-query matched k-mer counts and per-(query, colour) counts."""
    matched = np.asarray(matched, np.uint64)
    exp_matched = np.asarray(exp_matched, np.uint64)
    eq = matched.shape == exp_matched.shape and bool((matched == exp_matched).all())
    if color_counts is not None:
        cc = np.asarray(color_counts, np.uint64)
        ec = np.asarray(exp_counts, np.uint64)
        eq = eq and cc.shape == ec.shape and bool((cc == ec).all())
    return {"equal": bool(eq), "queries": int(matched.size), "matched_kmers": int(exp_matched.sum()),
            "digest_gpu": _digest(matched, color_counts if color_counts is not None else np.zeros(0)),
            "digest_oracle": _digest(exp_matched, exp_counts if exp_counts is not None else np.zeros(0))}
