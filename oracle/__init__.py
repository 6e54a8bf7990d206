"""Oracle (test infrastructure only).

ctypes front-end over ``oracle/_build/libggcat_oracle.so``, the C restatement of the
reference's build hot path and query lookup.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this module,
and only as the checker or as the timed CPU baseline; the ``ggcat_gb300`` package
never imports it.

Parity status: hashes and the sliding-window minimum are pinned by a port of the
reference's own property tests; end-to-end outputs are unpinned because the
reference (Rust) cannot be compiled here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libggcat_oracle.so")
_lib = None

# hash kinds, mirror of oracle_hashes.h
H_CN_SEQ64, H_FW_SEQ64, H_CN_SEQ128, H_FW_SEQ128, H_CN_RK128, H_FW_RK128, H_CN_RK64, H_FW_RK64 = range(8)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc only, seconds)."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    for f in ("oracle.c", "oracle.h", "oracle_hashes.c", "oracle_hashes.h"):
        if os.path.getmtime(os.path.join(_HERE, f)) > t:
            return True
    return False


class Params(C.Structure):
    _fields_ = [
        ("k", C.c_int),
        ("m", C.c_int),
        ("bucket_bits", C.c_int),
        ("second_bits", C.c_int),
        ("canonical", C.c_int),
        ("hash_kind", C.c_int),
        ("min_multiplicity", C.c_int),
        ("threads", C.c_int),
        ("colors", C.c_int),
    ]


class ExtHash(C.Structure):
    _fields_ = [("fw_lo", C.c_uint64), ("fw_hi", C.c_uint64), ("rc_lo", C.c_uint64), ("rc_hi", C.c_uint64)]


MQ_ITEM = np.dtype([("v", "<u8"), ("index", "<u4"), ("is_forward", "u1"), ("pad", "u1", 3)])
SUPERKMER = np.dtype(
    [
        ("start", "<u8"),
        ("len", "<u4"),
        ("bucket", "<u2"),
        ("second_bucket", "<u2"),
        ("minimizer_pos", "<u2"),
        ("rc", "u1"),
        ("flags", "u1"),
        ("seq_index", "<u4"),
        ("minimizer", "<u8"),
    ],
    align=True,
)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P = C.c_void_p
        sz = C.c_size_t
        L.orc_nthash_iter.restype = sz
        L.orc_nthash_iter.argtypes = [P, sz, C.c_int, P, P]
        L.orc_hash_iter.restype = sz
        L.orc_hash_iter.argtypes = [C.c_int, P, sz, C.c_int, P]
        L.orc_hash_roll_fw.restype = ExtHash
        L.orc_hash_roll_fw.argtypes = [C.c_int, ExtHash, C.c_int, C.c_uint8, C.c_uint8]
        L.orc_hash_roll_bw.restype = ExtHash
        L.orc_hash_roll_bw.argtypes = [C.c_int, ExtHash, C.c_int, C.c_uint8, C.c_uint8]
        L.orc_hash_remove_fw.restype = ExtHash
        L.orc_hash_remove_fw.argtypes = [C.c_int, ExtHash, C.c_int, C.c_uint8]
        L.orc_hash_remove_bw.restype = ExtHash
        L.orc_hash_remove_bw.argtypes = [C.c_int, ExtHash, C.c_int, C.c_uint8]
        L.orc_minqueue_splits.restype = sz
        L.orc_minqueue_splits.argtypes = [sz, P, sz, sz, sz, C.c_int, P, P, P, sz]
        L.orc_minqueue_minimizers.restype = sz
        L.orc_minqueue_minimizers.argtypes = [sz, P, sz, sz, C.c_int, P, sz]
        L.orc_bucketize.restype = sz
        L.orc_bucketize.argtypes = [P, P, P, sz, C.POINTER(Params), P, sz]
        L.orc_fasta_parse.restype = sz
        L.orc_fasta_parse.argtypes = [P, sz, C.c_long, P, sz, P, P, sz, C.POINTER(sz)]
        L.orc_build.restype = P
        L.orc_build.argtypes = [P, P, P, P, sz, C.POINTER(Params)]
        L.orc_build_free.argtypes = [P]
        L.orc_build_kmers.restype = sz
        L.orc_build_kmers.argtypes = [P, P, P, P, sz]
        L.orc_build_kmers_wide.restype = sz
        L.orc_build_kmers_wide.argtypes = [P, P, P, sz]
        L.orc_build_kmer_colors.restype = sz
        L.orc_build_kmer_colors.argtypes = [P, P, P, sz]
        L.orc_build_unitigs.restype = sz
        L.orc_build_unitigs.argtypes = [P, P, sz]
        L.orc_build_partial_count.restype = sz
        L.orc_build_partial_count.argtypes = [P]
        L.orc_canonicalize_unitigs.restype = sz
        L.orc_canonicalize_unitigs.argtypes = [P, sz, P, sz, C.c_int, P, sz]
        L.orc_query.restype = C.c_int
        L.orc_query.argtypes = [P, P, sz, P, P, C.c_uint32, P, P, P, sz, C.c_int, C.c_int, P, P, P]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def compress(seq: bytes | np.ndarray) -> np.ndarray:
    a = np.frombuffer(seq, dtype=np.uint8) if isinstance(seq, (bytes, bytearray)) else seq
    return ((a >> 1) & 3).astype(np.uint8)


def nthash(cbases: np.ndarray, m: int):
    cb = np.ascontiguousarray(cbases, dtype=np.uint8)
    n = max(len(cb) - m + 1, 0)
    fw = np.zeros(n, np.uint64)
    rc = np.zeros(n, np.uint64)
    lib().orc_nthash_iter(_ptr(cb), len(cb), m, _ptr(fw), _ptr(rc))
    return fw, rc


def hash_iter(kind: int, cbases: np.ndarray, k: int) -> np.ndarray:
    """Returns array (n, 4) of uint64: fw_lo, fw_hi, rc_lo, rc_hi."""
    cb = np.ascontiguousarray(cbases, dtype=np.uint8)
    n = max(len(cb) - k + 1, 0)
    out = np.zeros((n, 4), np.uint64)
    lib().orc_hash_iter(kind, _ptr(cb), len(cb), k, _ptr(out))
    return out


def _eh(row) -> ExtHash:
    return ExtHash(int(row[0]), int(row[1]), int(row[2]), int(row[3]))


def _row(h: ExtHash):
    return (h.fw_lo, h.fw_hi, h.rc_lo, h.rc_hi)


def roll_fw(kind, row, k, out_b, in_b):
    return _row(lib().orc_hash_roll_fw(kind, _eh(row), k, out_b, in_b))


def roll_bw(kind, row, k, out_b, in_b):
    return _row(lib().orc_hash_roll_bw(kind, _eh(row), k, out_b, in_b))


def remove_fw(kind, row, k, out_b):
    return _row(lib().orc_hash_remove_fw(kind, _eh(row), k, out_b))


def remove_bw(kind, row, k, out_b):
    return _row(lib().orc_hash_remove_bw(kind, _eh(row), k, out_b))


def minqueue_splits(size: int, values: np.ndarray, index=None, is_forward=None, skip_b=0, skip_e=0, dup=True):
    n = len(values)
    items = np.zeros(n, MQ_ITEM)
    items["v"] = values
    items["index"] = np.arange(n) if index is None else index
    if is_forward is not None:
        items["is_forward"] = is_forward
    cap = n + 4
    pos = np.zeros(cap, np.uint64)
    val = np.zeros(cap, MQ_ITEM)
    last = np.zeros(cap, np.uint8)
    cnt = lib().orc_minqueue_splits(size, _ptr(items), n, skip_b, skip_e, int(dup), _ptr(pos), _ptr(val), _ptr(last), cap)
    return pos[:cnt], val[:cnt], last[:cnt]


def minqueue_minimizers(size: int, values: np.ndarray, dup=True, skip_e=0):
    n = len(values)
    items = np.zeros(n, MQ_ITEM)
    items["v"] = values
    items["index"] = np.arange(n)
    out = np.zeros(n + 1, MQ_ITEM)
    cnt = lib().orc_minqueue_minimizers(size, _ptr(items), n, skip_e, int(dup), _ptr(out), n + 1)
    return out[:cnt]


def params(k=31, m=10, bucket_bits=10, second_bits=3, canonical=True, hash_kind=None, min_multiplicity=1, threads=1,
           colors=False) -> Params:
    if hash_kind is None:
        hash_kind = H_CN_SEQ64 if k <= 32 else H_CN_SEQ128
    return Params(k, m, bucket_bits, second_bits, int(canonical), hash_kind, min_multiplicity, threads, int(colors))


def bucketize(text: np.ndarray, seq_off: np.ndarray, seq_len: np.ndarray, p: Params) -> np.ndarray:
    text = np.ascontiguousarray(text, dtype=np.uint8)
    off = np.ascontiguousarray(seq_off, dtype=np.uint64)
    ln = np.ascontiguousarray(seq_len, dtype=np.uint64)
    n = lib().orc_bucketize(_ptr(text), _ptr(off), _ptr(ln), len(off), C.byref(p), None, 0)
    out = np.zeros(n, SUPERKMER)
    lib().orc_bucketize(_ptr(text), _ptr(off), _ptr(ln), len(off), C.byref(p), _ptr(out), n)
    return out


def fasta_parse(data: bytes, copyback: int):
    buf = np.frombuffer(data, dtype=np.uint8)
    text = np.zeros(len(buf) + 1024 + 4 * max(copyback, 0) * (len(buf) // (4 << 20) + 2), np.uint8)
    cap = len(buf) // 2 + 16
    off = np.zeros(cap, np.uint64)
    ln = np.zeros(cap, np.uint64)
    used = C.c_size_t(0)
    n = lib().orc_fasta_parse(_ptr(buf), len(buf), copyback, _ptr(text), len(text), _ptr(off), _ptr(ln), cap,
                              C.byref(used))
    assert used.value <= len(text) and n <= cap
    return text[: used.value], off[:n], ln[:n]


class BuildResult:
    def __init__(self, handle, k):
        self.h = handle
        self.k = k

    def __del__(self):
        if self.h:
            lib().orc_build_free(self.h)
            self.h = None

    def kmers(self):
        n = lib().orc_build_kmers(self.h, None, None, None, 0)
        lo = np.zeros(n, np.uint64)
        hi = np.zeros(n, np.uint64)
        mult = np.zeros(n, np.uint64)
        lib().orc_build_kmers(self.h, _ptr(lo), _ptr(hi), _ptr(mult), n)
        return lo, hi, mult

    def kmers_wide(self):
        """Surviving k-mers as (n, 4) u64 words (bases 0-31, 32-63, 64-95, 96-127; k <= 128)
        with their multiplicities."""
        n = lib().orc_build_kmers_wide(self.h, None, None, 0)
        words = np.zeros((n, 4), np.uint64)
        mult = np.zeros(n, np.uint64)
        lib().orc_build_kmers_wide(self.h, _ptr(words), _ptr(mult), n)
        return words, mult

    def kmer_colors(self):
        n = lib().orc_build_kmers(self.h, None, None, None, 0)
        tot = lib().orc_build_kmer_colors(self.h, None, None, 0)
        off = np.zeros(n + 1, np.uint64)
        col = np.zeros(max(tot, 1), np.uint32)
        lib().orc_build_kmer_colors(self.h, _ptr(off), _ptr(col), tot)
        return off, col[:tot]

    def unitigs(self) -> bytes:
        n = lib().orc_build_unitigs(self.h, None, 0)
        buf = np.zeros(n + 1, np.uint8)
        lib().orc_build_unitigs(self.h, _ptr(buf), n + 1)
        return buf[:n].tobytes()

    def partial_count(self) -> int:
        return lib().orc_build_partial_count(self.h)


def build_graph(text, seq_off, seq_len, p: Params, seq_colors=None) -> BuildResult:
    text = np.ascontiguousarray(text, dtype=np.uint8)
    off = np.ascontiguousarray(seq_off, dtype=np.uint64)
    ln = np.ascontiguousarray(seq_len, dtype=np.uint64)
    col = None if seq_colors is None else np.ascontiguousarray(seq_colors, dtype=np.uint32)
    h = lib().orc_build(_ptr(text), _ptr(off), _ptr(ln), _ptr(col), len(off), C.byref(p))
    if not h:
        raise ValueError("oracle: unsupported parameters")
    r = BuildResult(h, p.k)
    r._keep = (text, off, ln, col)
    return r


def canonicalize_unitigs(lines: bytes, circular: np.ndarray, k: int) -> bytes:
    buf = np.frombuffer(lines, dtype=np.uint8)
    circ = np.ascontiguousarray(circular, dtype=np.uint8)
    n = lib().orc_canonicalize_unitigs(_ptr(buf), len(buf), _ptr(circ), len(circ), k, None, 0)
    out = np.zeros(n + 1, np.uint8)
    lib().orc_canonicalize_unitigs(_ptr(buf), len(buf), _ptr(circ), len(circ), k, _ptr(out), n + 1)
    return out[:n].tobytes()


def query(graph_lo, graph_hi, qtext, q_off, q_len, k, gc_off=None, gc_colors=None, ncolors=0):
    glo = np.ascontiguousarray(graph_lo, np.uint64)
    ghi = np.ascontiguousarray(graph_hi, np.uint64)
    qt = np.ascontiguousarray(qtext, np.uint8)
    qo = np.ascontiguousarray(q_off, np.uint64)
    ql = np.ascontiguousarray(q_len, np.uint64)
    nq = len(qo)
    matched = np.zeros(nq, np.uint64)
    qk = np.zeros(nq, np.uint64)
    pc = np.zeros(nq * ncolors, np.uint64) if ncolors else None
    go = None if gc_off is None else np.ascontiguousarray(gc_off, np.uint64)
    gcc = None if gc_colors is None else np.ascontiguousarray(gc_colors, np.uint32)
    lib().orc_query(_ptr(glo), _ptr(ghi), len(glo), _ptr(go), _ptr(gcc), ncolors, _ptr(qt), _ptr(qo), _ptr(ql), nq, k,
                    0, _ptr(matched), _ptr(qk), _ptr(pc))
    return matched, qk, (pc.reshape(nq, ncolors) if ncolors else None)
