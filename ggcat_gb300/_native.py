"""ctypes binding of the C ABI declared in include/ggcat_gb300.h.

The CUDA library is the only compute path: if it cannot be built or loaded this module
raises, there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

GGCAT_GPU_OK = 0
GGCAT_HASH_SEQHASH = 1
GGCAT_HASH_RABIN_KARP128 = 4
GGCAT_MERGE_BATCHED = 0
GGCAT_MERGE_PER_BUCKET = 1

_ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "EDEVICE", -5: "EUNSUPPORTED", -6: "EIO", -7: "ETOOLARGE"}


class GgcatGpuError(RuntimeError):
    pass


class Params(C.Structure):
    _fields_ = [
        ("k", C.c_int32),
        ("m", C.c_int32),
        ("bucket_bits", C.c_int32),
        ("second_bits", C.c_int32),
        ("min_multiplicity", C.c_int32),
        ("hash_kind", C.c_int32),
        ("forward_only", C.c_int32),
        ("merge_mode", C.c_int32),
        ("unit_target", C.c_int32),
        ("keep_kmers", C.c_int32),
        ("subbin_bytes", C.c_int32),
        ("table_load_pct", C.c_int32),
        ("small_limit", C.c_int32),
        ("copy_pieces", C.c_int32),
        ("spill_mb", C.c_int32),
        ("small_batch", C.c_int32),
        ("wide_batch", C.c_int32),
        ("wide_limit", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("text_bytes", C.c_uint64),
        ("superkmers", C.c_uint64),
        ("kmer_instances", C.c_uint64),
        ("merge_units_small", C.c_uint64),
        ("merge_units_large", C.c_uint64),
        ("partial_unitigs", C.c_uint64),
        ("partial_bases", C.c_uint64),
        ("surviving_kmers", C.c_uint64),
        ("final_unitigs", C.c_uint64),
        ("ms_pack", C.c_double),
        ("ms_bucketize", C.c_double),
        ("ms_merge", C.c_double),
        ("ms_link", C.c_double),
        ("distinct_kmers", C.c_uint64),
        ("merge_units_spilled", C.c_uint64),
        ("merge_units_ext_global", C.c_uint64),
        ("merge_units_walk", C.c_uint64),
        ("merge_graph_captures", C.c_uint64),
        ("merge_graph_replays", C.c_uint64),
        ("spill_pieces", C.c_uint64),
        ("spill_ranges", C.c_uint64),
        ("spill_bytes", C.c_uint64),
        ("ms_tier", C.c_double * 4),
        ("colors_collected", C.c_uint64),
    ]


SUPERKMER = np.dtype(
    [
        ("start", "<u8"),
        ("len", "<u4"),
        ("bucket", "<u2"),
        ("second_bucket", "<u2"),
        ("minimizer_pos", "<u2"),
        ("rc", "u1"),
        ("flags", "u1"),
    ],
    align=True,
)

# every symbol include/ggcat_gb300.h declares
EXPORTED = [
    "ggcat_gpu_create",
    "ggcat_gpu_destroy",
    "ggcat_gpu_last_error",
    "ggcat_gpu_kernel_launches",
    "ggcat_gpu_bucketize",
    "ggcat_gpu_superkmers_copy",
    "ggcat_gpu_merge",
    "ggcat_gpu_autotune",
    "ggcat_gpu_partial_unitigs_copy",
    "ggcat_gpu_kmers_copy",
    "ggcat_gpu_link",
    "ggcat_gpu_unitigs_copy",
    "ggcat_gpu_get_stats",
    "ggcat_gpu_build_text",
    "ggcat_gpu_fasta_parse",
    "ggcat_gpu_fastq_parse",
    "ggcat_gpu_read_sequences_file",
    "ggcat_gpu_read_sequences_files",
    "ggcat_gpu_unitig_links",
    "ggcat_gpu_compute_tigs",
    "ggcat_gpu_write_graph",
    "ggcat_gpu_dump_unitigs",
    "ggcat_gpu_collect_streams",
    "ggcat_gpu_build_from_streams",
    "ggcat_gpu_build_from_files",
    "ggcat_gpu_build_from_files_ex",
    "ggcat_gpu_colors",
    "ggcat_gpu_colors_prepare",
    "ggcat_gpu_kmer_subsets_copy",
    "ggcat_gpu_subsets_copy",
    "ggcat_gpu_query_index",
    "ggcat_gpu_query_index_colored",
    "ggcat_gpu_query_from_files",
    "ggcat_gpu_query_graph",
    "ggcat_gpu_query_submit",
    "ggcat_gpu_query_poll",
    "ggcat_gpu_query_wait",
    "ggcat_gpu_query_color_counts",
    "ggcat_gpu_kmer_hashes",
    "ggcat_gpu_colormap_file",
    "ggcat_gpu_write_colormap",
    "ggcat_gpu_dump_colors",
    "ggcat_gpu_query_colormap",
    "ggcat_gpu_bucket_histogram_noalloc",
]

QUERY_SLOTS = 4

_lib = None


def library_path() -> str:
    return _build.LIB


# ggcat_gpu_dump_fn: (fn_ctx, seq, len, colors, n_colors, same_colors)
DUMP_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int)
COLORMAP_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint64)
# ggcat_gpu_seq_fn and ggcat_gpu_stream
SEQ_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_uint64)
READ_BLOCK_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int64, SEQ_FN, C.c_void_p)


class Stream(C.Structure):
    _fields_ = [("stream_ctx", C.c_void_p), ("read_block", READ_BLOCK_FN)]


def load(build: bool = True):
    """Loads (building first if needed) libggcat_gb300.so and declares the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise GgcatGpuError(f"CUDA library missing: {path}")
    L = C.CDLL(path)
    P, u64, sz = C.c_void_p, C.c_uint64, C.c_size_t
    pu64 = C.POINTER(C.c_uint64)
    L.ggcat_gpu_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    L.ggcat_gpu_destroy.argtypes = [P]
    L.ggcat_gpu_destroy.restype = None
    L.ggcat_gpu_last_error.argtypes = [P]
    L.ggcat_gpu_last_error.restype = C.c_char_p
    L.ggcat_gpu_kernel_launches.argtypes = [P]
    L.ggcat_gpu_kernel_launches.restype = u64
    L.ggcat_gpu_bucketize.argtypes = [P, P, u64, C.POINTER(Params), P, pu64]
    L.ggcat_gpu_superkmers_copy.argtypes = [P, P, u64, pu64]
    L.ggcat_gpu_merge.argtypes = [P, C.POINTER(Params), P]
    L.ggcat_gpu_query_graph.argtypes = [P, C.c_char_p, C.c_char_p, C.c_char_p, sz, sz, C.c_int, sz, C.c_int, sz,
                                        C.c_char_p, u64]
    L.ggcat_gpu_query_from_files.argtypes = [P, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_char_p,
                                             u64]
    L.ggcat_gpu_autotune.argtypes = [P, P, u64, C.POINTER(Params), u64, P, C.POINTER(Params),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ggcat_gpu_partial_unitigs_copy.argtypes = [P, P, u64, P, P, P, u64, pu64, pu64]
    L.ggcat_gpu_kmers_copy.argtypes = [P, P, P, u64, pu64]
    L.ggcat_gpu_link.argtypes = [P, C.c_int]
    L.ggcat_gpu_unitigs_copy.argtypes = [P, P, u64, P, P, P, u64, pu64, pu64]
    L.ggcat_gpu_get_stats.argtypes = [P, C.POINTER(Stats)]
    L.ggcat_gpu_build_text.argtypes = [P, P, u64, C.POINTER(Params), P]
    L.ggcat_gpu_fasta_parse.argtypes = [P, u64, C.c_int64, P, u64, pu64, pu64]
    L.ggcat_gpu_fastq_parse.argtypes = [P, u64, P, u64, pu64, pu64]
    L.ggcat_gpu_read_sequences_file.argtypes = [C.c_char_p, C.c_int64, P, u64, pu64, pu64, C.c_char_p, u64]
    L.ggcat_gpu_read_sequences_files.argtypes = [C.POINTER(C.c_char_p), u64, C.c_int64, C.c_int, P, u64, pu64,
                                                 C.c_char_p, u64]
    L.ggcat_gpu_unitig_links.argtypes = [P, P, P, u64, C.c_int, P, P, P, P, u64, pu64]
    L.ggcat_gpu_compute_tigs.argtypes = [P, P, P, u64, C.c_int, C.c_int, P, u64, P, P, u64, pu64, pu64]
    L.ggcat_gpu_write_graph.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_char_p, u64]
    L.ggcat_gpu_dump_unitigs.argtypes = [C.c_char_p, C.c_int, C.c_int, DUMP_FN, C.c_void_p]
    L.ggcat_gpu_colormap_file.argtypes = [C.c_char_p, C.c_char_p, u64]
    L.ggcat_gpu_write_colormap.argtypes = [C.c_char_p, C.POINTER(C.c_char_p), u64, P, P, u64]
    L.ggcat_gpu_dump_colors.argtypes = [C.c_char_p, P, u64, pu64, pu64]
    L.ggcat_gpu_query_colormap.argtypes = [C.c_char_p, P, u64, C.c_int, COLORMAP_FN, C.c_void_p]
    L.ggcat_gpu_collect_streams.argtypes = [C.POINTER(Stream), u64, C.c_int64, P, u64, pu64]
    L.ggcat_gpu_build_from_streams.argtypes = [P, C.POINTER(Stream), sz, C.c_char_p, sz, sz, C.c_int, sz, sz]
    L.ggcat_gpu_build_from_files.argtypes = [P, C.POINTER(C.c_char_p), sz, C.c_char_p, sz, sz, C.c_int, sz, sz]
    L.ggcat_gpu_build_from_files_ex.argtypes = [P, C.POINTER(C.c_char_p), sz, C.c_char_p, C.POINTER(C.c_char_p), sz,
                                                sz, sz, C.c_int, sz, C.c_int, sz, C.c_int, C.c_int]
    L.ggcat_gpu_bucket_histogram_noalloc.argtypes = [P, u64, C.c_int32, C.c_int32, C.c_int32, P, P, P, P]
    L.ggcat_gpu_kmer_hashes.argtypes = [P, P, u64, C.c_int, C.c_int, P, P]
    L.ggcat_gpu_colors.argtypes = [P, P, P, u64, C.c_uint32, P]
    L.ggcat_gpu_colors_prepare.argtypes = [P, P, P, u64, C.c_uint32]
    L.ggcat_gpu_kmer_subsets_copy.argtypes = [P, P, u64, pu64]
    L.ggcat_gpu_subsets_copy.argtypes = [P, P, u64, pu64, C.POINTER(C.c_uint32)]
    L.ggcat_gpu_query_index.argtypes = [P, P, u64, C.c_int, P]
    L.ggcat_gpu_query_index_colored.argtypes = [P, P]
    L.ggcat_gpu_query_submit.argtypes = [P, C.c_int, P, u64, P, P, u64]
    L.ggcat_gpu_query_poll.argtypes = [P, C.c_int]
    L.ggcat_gpu_query_wait.argtypes = [P, C.c_int, P, u64, pu64]
    L.ggcat_gpu_query_color_counts.argtypes = [P, C.c_int, P, u64, C.POINTER(C.c_uint32)]
    for name in EXPORTED:
        if name not in ("ggcat_gpu_destroy", "ggcat_gpu_last_error", "ggcat_gpu_kernel_launches"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    return a.ctypes.data_as(C.c_void_p)


def make_params(k=31, m=None, bucket_bits=10, second_bits=3, min_multiplicity=1, hash_kind=GGCAT_HASH_SEQHASH,
                forward_only=False, merge_mode=GGCAT_MERGE_BATCHED, unit_target=0, keep_kmers=False,
                subbin_bytes=0, table_load_pct=0, small_limit=0, copy_pieces=0, spill_mb=0, small_batch=0,
                wide_batch=0, wide_limit=0) -> Params:
    if m is None:
        m = compute_best_m(k)
    return Params(k, m, bucket_bits, second_bits, min_multiplicity, hash_kind, int(forward_only), merge_mode,
                  unit_target, int(keep_kmers), subbin_bytes, table_load_pct, small_limit, copy_pieces, spill_mb,
                  small_batch, wide_batch, wide_limit)


def compute_best_m(k: int) -> int:
    """crates/utils/src/lib.rs:29-40."""
    if k <= 13:
        return max(k // 2, k - 4)
    if k <= 15:
        return 9
    if k <= 21:
        return 10
    if k <= 30:
        return 11
    if k <= 37:
        return 12
    if k <= 42:
        return 13
    if k <= 64:
        return 14
    return (k + 2) // 4  # f64::round: halves away from zero


class GpuContext:
    """One device context of the library (all device buffers are owned by it)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.ggcat_gpu_create(device, C.byref(h))
        if rc != 0:
            raise GgcatGpuError(f"ggcat_gpu_create failed ({_ERRORS.get(rc, rc)}): is a CUDA device available?")
        self.h = h
        self.k = 0  # k of the last bucketize / build

    def close(self):
        if getattr(self, "h", None):
            self.L.ggcat_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.L.ggcat_gpu_last_error(self.h)
            raise GgcatGpuError(f"{what}: {_ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")

    @property
    def kernel_launches(self) -> int:
        return int(self.L.ggcat_gpu_kernel_launches(self.h))

    def bucketize(self, d_text_ptr: int, text_len: int, p: Params, stream: int = 0) -> int:
        n = C.c_uint64()
        self._check(self.L.ggcat_gpu_bucketize(self.h, C.c_void_p(d_text_ptr), text_len, C.byref(p),
                                               C.c_void_p(stream), C.byref(n)), "bucketize")
        self.k = p.k
        return n.value

    def superkmers(self) -> np.ndarray:
        n = C.c_uint64()
        self._check(self.L.ggcat_gpu_superkmers_copy(self.h, None, 0, C.byref(n)), "superkmers_copy")
        out = np.zeros(n.value, SUPERKMER)
        self._check(self.L.ggcat_gpu_superkmers_copy(self.h, _ptr(out), n.value, C.byref(n)), "superkmers_copy")
        return out

    def merge(self, p: Params, stream: int = 0):
        self._check(self.L.ggcat_gpu_merge(self.h, C.byref(p), C.c_void_p(stream)), "merge")

    def build_text(self, text: np.ndarray, p: Params, stream: int = 0):
        t = np.ascontiguousarray(text, dtype=np.uint8)
        self._check(self.L.ggcat_gpu_build_text(self.h, _ptr(t), len(t), C.byref(p), C.c_void_p(stream)), "build_text")
        self.k = p.k

    def _unitigs(self, fn, what):
        nu, nb = C.c_uint64(), C.c_uint64()
        self._check(fn(self.h, None, 0, None, None, None, 0, C.byref(nu), C.byref(nb)), what)
        bases = np.zeros(nb.value, np.uint8)
        off = np.zeros(nu.value, np.uint64)
        ln = np.zeros(nu.value, np.uint32)
        fl = np.zeros(nu.value, np.uint8)
        self._check(fn(self.h, _ptr(bases), nb.value, _ptr(off), _ptr(ln), _ptr(fl), nu.value, C.byref(nu),
                       C.byref(nb)), what)
        return bases, off, ln, fl

    def partial_unitigs(self):
        return self._unitigs(self.L.ggcat_gpu_partial_unitigs_copy, "partial_unitigs_copy")

    def kmers(self):
        """Surviving canonical k-mers and multiplicities.  keys: u64 array for k <= 32, an
        (n, 2) array of (lo, hi) words for 32 < k <= 64, an (n, 4) array of words (bases 0-31,
        32-63, 64-95, 96-126) above."""
        n = C.c_uint64()
        self._check(self.L.ggcat_gpu_kmers_copy(self.h, None, None, 0, C.byref(n)), "kmers_copy")
        words = 4 if self.k > 64 else 2 if self.k > 32 else 1
        keys = np.zeros((n.value, words) if words > 1 else n.value, np.uint64)
        mult = np.zeros(n.value, np.uint64)
        self._check(self.L.ggcat_gpu_kmers_copy(self.h, _ptr(keys), _ptr(mult), n.value, C.byref(n)), "kmers_copy")
        return keys, mult

    def link(self, k: int):
        self._check(self.L.ggcat_gpu_link(self.h, k), "link")

    def unitigs(self):
        return self._unitigs(self.L.ggcat_gpu_unitigs_copy, "unitigs_copy")

    def kmer_hashes(self, d_text_ptr: int, length: int, k: int, kind: int, d_out_ptr: int, stream: int = 0):
        self._check(self.L.ggcat_gpu_kmer_hashes(self.h, C.c_void_p(d_text_ptr), length, k, kind,
                                                 C.c_void_p(d_out_ptr), C.c_void_p(stream)), "kmer_hashes")

    # ---- colours ----
    def colors_prepare(self, seq_off, seq_color, n_colors: int):
        """Announces the colour table of the next build, so that its merge collects the colours."""
        off = np.ascontiguousarray(seq_off, np.uint64)
        col = np.ascontiguousarray(seq_color, np.uint32)
        self._check(self.L.ggcat_gpu_colors_prepare(self.h, _ptr(off), _ptr(col), off.size, n_colors),
                    "colors_prepare")

    def colors(self, seq_off, seq_color, n_colors: int, stream: int = 0):
        so = np.ascontiguousarray(seq_off, np.uint64)
        sc = np.ascontiguousarray(seq_color, np.uint32)
        self._check(self.L.ggcat_gpu_colors(self.h, _ptr(so), _ptr(sc), len(so), n_colors, C.c_void_p(stream)),
                    "colors")

    def kmer_subsets(self) -> np.ndarray:
        n = C.c_uint64()
        self._check(self.L.ggcat_gpu_kmer_subsets_copy(self.h, None, 0, C.byref(n)), "kmer_subsets_copy")
        out = np.zeros(n.value, np.uint32)
        self._check(self.L.ggcat_gpu_kmer_subsets_copy(self.h, _ptr(out), n.value, C.byref(n)), "kmer_subsets_copy")
        return out

    def subsets(self) -> np.ndarray:
        """(n_subsets, words) uint32 colour bitmaps."""
        n, w = C.c_uint64(), C.c_uint32()
        self._check(self.L.ggcat_gpu_subsets_copy(self.h, None, 0, C.byref(n), C.byref(w)), "subsets_copy")
        out = np.zeros(n.value * w.value, np.uint32)
        self._check(self.L.ggcat_gpu_subsets_copy(self.h, _ptr(out), out.size, C.byref(n), C.byref(w)), "subsets_copy")
        return out.reshape(n.value, w.value)

    # ---- query ----
    def query_index(self, d_graph_ptr: int, length: int, k: int, stream: int = 0):
        self._check(self.L.ggcat_gpu_query_index(self.h, C.c_void_p(d_graph_ptr), length, k, C.c_void_p(stream)),
                    "query_index")

    def query_index_colored(self, stream: int = 0):
        self._check(self.L.ggcat_gpu_query_index_colored(self.h, C.c_void_p(stream)), "query_index_colored")

    def query_submit(self, slot: int, text: np.ndarray, off: np.ndarray, ln: np.ndarray):
        t = np.ascontiguousarray(text, np.uint8)
        o = np.ascontiguousarray(off, np.uint64)
        l_ = np.ascontiguousarray(ln, np.uint64)
        self._check(self.L.ggcat_gpu_query_submit(self.h, slot, _ptr(t), len(t), _ptr(o), _ptr(l_), len(o)),
                    "query_submit")
        if not hasattr(self, "_slot_nq"):
            self._slot_nq = {}
        self._slot_nq[slot] = len(o)

    def query_poll(self, slot: int) -> bool:
        rc = self.L.ggcat_gpu_query_poll(self.h, slot)
        if rc < 0:
            self._check(rc, "query_poll")
        return rc == 1

    def query_wait(self, slot: int) -> np.ndarray:
        """Waits for the slot's batch and returns the matched k-mer count of each query."""
        nq = self._slot_nq.get(slot, 0)
        out = np.zeros(nq, np.uint64)
        got = C.c_uint64()
        self._check(self.L.ggcat_gpu_query_wait(self.h, slot, _ptr(out), nq, C.byref(got)), "query_wait")
        return out

    def query_color_counts(self, slot: int) -> np.ndarray:
        """(nq, n_colors) per-colour counts of the slot's last (waited) coloured batch."""
        nq = self._slot_nq.get(slot, 0)
        nc = C.c_uint32()
        self._check(self.L.ggcat_gpu_query_color_counts(self.h, slot, None, 0, C.byref(nc)), "query_color_counts")
        out = np.zeros(nq * nc.value, np.uint64)
        self._check(self.L.ggcat_gpu_query_color_counts(self.h, slot, _ptr(out), out.size, C.byref(nc)),
                    "query_color_counts")
        return out.reshape(nq, nc.value)

    def autotune(self, d_text: int, n: int, p: Params, sample_bytes: int = 0, stream: int = 0):
        """Tuned copy of p (device text at d_text), with the device times of p and of the
        tuned params: (params, default_ms, tuned_ms)."""
        best = Params()
        dm, bm = C.c_double(), C.c_double()
        self._check(self.L.ggcat_gpu_autotune(self.h, C.c_void_p(d_text), n, C.byref(p), sample_bytes,
                                              C.c_void_p(stream), C.byref(best), C.byref(dm), C.byref(bm)),
                    "autotune")
        return best, dm.value, bm.value

    def stats(self) -> dict:
        s = Stats()
        self._check(self.L.ggcat_gpu_get_stats(self.h, C.byref(s)), "get_stats")
        out = {f: getattr(s, f) for f, _ in Stats._fields_}
        out["ms_tier"] = list(s.ms_tier)
        return out


def fasta_parse(data: bytes, copyback: int):
    """FASTA -> device text layout, with the reference's 4 MiB + copyback chunking."""
    L = load()
    buf = np.frombuffer(data, dtype=np.uint8)
    need, pieces = C.c_uint64(), C.c_uint64()
    rc = L.ggcat_gpu_fasta_parse(_ptr(buf), len(buf), copyback, None, 0, C.byref(need), C.byref(pieces))
    if rc:
        raise GgcatGpuError("fasta_parse failed")
    text = np.zeros(need.value, np.uint8)
    rc = L.ggcat_gpu_fasta_parse(_ptr(buf), len(buf), copyback, _ptr(text), need.value, C.byref(need), C.byref(pieces))
    if rc:
        raise GgcatGpuError("fasta_parse failed")
    return text


def fastq_parse(data: bytes):
    """FASTQ -> device text layout, one piece per record."""
    L = load()
    buf = np.frombuffer(data, dtype=np.uint8)
    need, n = C.c_uint64(), C.c_uint64()
    if L.ggcat_gpu_fastq_parse(_ptr(buf), len(buf), None, 0, C.byref(need), C.byref(n)):
        raise GgcatGpuError("fastq_parse failed")
    text = np.zeros(need.value, np.uint8)
    if L.ggcat_gpu_fastq_parse(_ptr(buf), len(buf), _ptr(text), need.value, C.byref(need), C.byref(n)):
        raise GgcatGpuError("fastq_parse failed")
    return text


def read_sequences_file(path: str, copyback: int = -1):
    """One FASTA / FASTQ file (plain or gz, lz4, bz2, xz, zst) -> device text layout."""
    L = load()
    need, n = C.c_uint64(), C.c_uint64()
    err = C.create_string_buffer(512)
    rc = L.ggcat_gpu_read_sequences_file(os.fsencode(path), copyback, None, 0, C.byref(need), C.byref(n), err, 512)
    if rc:
        raise GgcatGpuError(f"read_sequences_file failed ({_ERRORS.get(rc, rc)}): {err.value.decode()}")
    text = np.zeros(need.value, np.uint8)
    rc = L.ggcat_gpu_read_sequences_file(os.fsencode(path), copyback, _ptr(text), need.value, C.byref(need),
                                         C.byref(n), err, 512)
    if rc:
        raise GgcatGpuError(f"read_sequences_file failed ({_ERRORS.get(rc, rc)}): {err.value.decode()}")
    return text


def read_sequences_files(paths, copyback: int = -1, threads: int = 4):
    """Several files read on `threads` host threads, concatenated in input order."""
    L = load()
    arr = (C.c_char_p * len(paths))(*[os.fsencode(p) for p in paths])
    need = C.c_uint64()
    err = C.create_string_buffer(512)
    rc = L.ggcat_gpu_read_sequences_files(arr, len(paths), copyback, threads, None, 0, C.byref(need), err, 512)
    if rc:
        raise GgcatGpuError(f"read_sequences_files failed ({_ERRORS.get(rc, rc)}): {err.value.decode()}")
    text = np.zeros(need.value, np.uint8)
    rc = L.ggcat_gpu_read_sequences_files(arr, len(paths), copyback, threads, _ptr(text), need.value, C.byref(need),
                                          err, 512)
    if rc:
        raise GgcatGpuError(f"read_sequences_files failed ({_ERRORS.get(rc, rc)}): {err.value.decode()}")
    return text


def unitig_links(bases: np.ndarray, off: np.ndarray, ln: np.ndarray, k: int):
    """Maximal-unitig links: (list_off, other, overlap, flags); list 2i = links from unitig
    i's end, 2i + 1 = from its beginning; flags bit 0 flip_current, bit 1 flip_other."""
    L = load()
    b = np.ascontiguousarray(bases, np.uint8)
    o = np.ascontiguousarray(off, np.uint64)
    n_ = np.ascontiguousarray(ln, np.uint64)
    n = len(o)
    lo = np.zeros(2 * n + 1, np.uint64)
    cnt = C.c_uint64()
    rc = L.ggcat_gpu_unitig_links(_ptr(b), _ptr(o), _ptr(n_), n, k, _ptr(lo), None, None, None, 0, C.byref(cnt))
    if rc:
        raise GgcatGpuError(f"unitig_links failed ({_ERRORS.get(rc, rc)})")
    other = np.zeros(cnt.value, np.uint64)
    overlap = np.zeros(cnt.value, np.uint64)
    flags = np.zeros(cnt.value, np.uint8)
    rc = L.ggcat_gpu_unitig_links(_ptr(b), _ptr(o), _ptr(n_), n, k, _ptr(lo), _ptr(other), _ptr(overlap),
                                  _ptr(flags), cnt.value, C.byref(cnt))
    if rc:
        raise GgcatGpuError(f"unitig_links failed ({_ERRORS.get(rc, rc)})")
    return lo, other, overlap, flags


TIGS_GREEDY_MATCHTIGS, TIGS_EULERTIGS, TIGS_PATHTIGS = 2, 3, 4


def compute_tigs(bases: np.ndarray, off: np.ndarray, ln: np.ndarray, k: int, mode: int):
    """Greedy matchtigs / eulertigs / pathtigs (mode 2 / 3 / 4) of the unitigs
    bases[off[i]:off[i] + ln[i]]: (bases, off, len) of the strings."""
    L = load()
    b = np.ascontiguousarray(bases, np.uint8)
    o = np.ascontiguousarray(off, np.uint64)
    n_ = np.ascontiguousarray(ln, np.uint64)
    n = len(o)
    cap_b = int(n_.sum()) if n else 0
    ob = np.zeros(max(cap_b, 1), np.uint8)
    oo = np.zeros(max(n, 1), np.uint64)
    ol = np.zeros(max(n, 1), np.uint64)
    cnt, nb = C.c_uint64(), C.c_uint64()
    rc = L.ggcat_gpu_compute_tigs(_ptr(b), _ptr(o), _ptr(n_), n, k, mode, _ptr(ob), ob.size, _ptr(oo), _ptr(ol),
                                  oo.size, C.byref(cnt), C.byref(nb))
    if rc:
        raise GgcatGpuError(f"compute_tigs failed ({_ERRORS.get(rc, rc)})")
    return ob[:nb.value].copy(), oo[:cnt.value].copy(), ol[:cnt.value].copy()


def dump_unitigs(graph_input: str, k: int, colors: bool = False) -> list:
    """ggcat_dump_unitigs: the pieces of the graph FASTA as bytes; with colors, tuples
    (bases, colours, same_colors) of the single-subset pieces."""
    L = load()
    out = []

    def cb(_ctx, seq, n, cols, nc, same):
        b = C.string_at(seq, n)
        if colors:
            cp = C.cast(cols, C.POINTER(C.c_uint32))
            out.append((b, [int(cp[i]) for i in range(nc)], bool(same)))
        else:
            out.append(b)

    fn = DUMP_FN(cb)
    rc = L.ggcat_gpu_dump_unitigs(os.fsencode(graph_input), k, int(bool(colors)), fn, None)
    if rc:
        raise GgcatGpuError(f"dump_unitigs failed ({_ERRORS.get(rc, rc)})")
    return out


def make_streams(sources: list, seen_copyback: list | None = None):
    """ggcat_gpu_stream array over Python sources (each a list of byte strings, emitted in
    order); keep the returned tuple alive while the library uses it."""
    keep = []
    arr = (Stream * len(sources))()
    for i, seqs in enumerate(sources):
        def read_block(_ctx, copyback, emit, emit_ctx, seqs=seqs):
            if seen_copyback is not None:
                seen_copyback.append(copyback)
            for s in seqs:
                buf = C.create_string_buffer(bytes(s), len(s))
                emit(emit_ctx, C.cast(buf, C.c_void_p), len(s))
        fn = READ_BLOCK_FN(read_block)
        keep.append(fn)
        arr[i].stream_ctx = None
        arr[i].read_block = fn
    return arr, keep


def collect_streams(sources: list, copyback: int, seen_copyback: list | None = None) -> np.ndarray:
    L = load()
    arr, keep = make_streams(sources, seen_copyback)
    need = C.c_uint64()
    if L.ggcat_gpu_collect_streams(arr, len(sources), copyback, None, 0, C.byref(need)):
        raise GgcatGpuError("collect_streams failed")
    text = np.zeros(need.value, np.uint8)
    if L.ggcat_gpu_collect_streams(arr, len(sources), copyback, _ptr(text), need.value, C.byref(need)):
        raise GgcatGpuError("collect_streams failed")
    del keep
    return text


def write_graph(unitigs_fasta: str, output_file: str, k: int, unitig_links: bool = False, gfa_version: int = 0):
    """A FASTA of unitigs rewritten as FASTA with link annotations or as GFA v1 / v2."""
    L = load()
    err = C.create_string_buffer(512)
    rc = L.ggcat_gpu_write_graph(os.fsencode(unitigs_fasta), os.fsencode(output_file), k, int(unitig_links),
                                 gfa_version, err, 512)
    if rc:
        raise GgcatGpuError(f"write_graph failed ({_ERRORS.get(rc, rc)}): {err.value.decode()}")


def unitig_lines(bases: np.ndarray, off: np.ndarray, ln: np.ndarray) -> bytes:
    """'\\n'-terminated unitig lines from (bases, offsets, lengths), gathered in one pass."""
    ln64 = np.asarray(ln).astype(np.int64)
    n = ln64.size
    if n == 0:
        return b""
    if bases.size == 0:
        return b"\n" * n
    out_start = np.zeros(n, np.int64)
    out_start[1:] = np.cumsum(ln64[:-1] + 1)
    total = int(ln64.sum()) + n
    src = np.arange(total, dtype=np.int64) + np.repeat(np.asarray(off).astype(np.int64) - out_start, ln64 + 1)
    out = bases[np.minimum(src, bases.size - 1)]  # the newline slots are overwritten below
    out[out_start + ln64] = 10
    return out.tobytes()


# ---- colormap file ----
def colormap_file(graph_file: str) -> str:
    """The colormap path of a graph file (the graph path with its extension replaced by
    "colors.dat")."""
    L = load()
    out = C.create_string_buffer(len(os.fsencode(graph_file)) + 64)
    rc = L.ggcat_gpu_colormap_file(os.fsencode(graph_file), out, len(out))
    if rc:
        raise GgcatGpuError(f"colormap_file failed ({_ERRORS.get(rc, rc)})")
    return os.fsdecode(out.value)


def write_colormap(path: str, color_names: list, subsets: list):
    """Writes a colormap file: colour names and subsets (each a sorted list of colour indices)."""
    L = load()
    names = (C.c_char_p * max(1, len(color_names)))(*[n.encode() for n in color_names])
    off = np.zeros(len(subsets) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in subsets])
    cols = np.ascontiguousarray(np.concatenate([np.asarray(x, np.uint32) for x in subsets]) if subsets
                                else np.zeros(1, np.uint32), np.uint32)
    rc = L.ggcat_gpu_write_colormap(os.fsencode(path), names, len(color_names), _ptr(off), _ptr(cols), len(subsets))
    if rc:
        raise GgcatGpuError(f"write_colormap failed ({_ERRORS.get(rc, rc)})")


def dump_colors(colormap: str) -> list:
    """Colour names of a colormap, in colour index order (ggcat_dump_colors)."""
    L = load()
    nb, nc = C.c_uint64(), C.c_uint64()
    rc = L.ggcat_gpu_dump_colors(os.fsencode(colormap), None, 0, C.byref(nb), C.byref(nc))
    if rc:
        raise GgcatGpuError(f"dump_colors failed ({_ERRORS.get(rc, rc)})")
    buf = C.create_string_buffer(max(1, nb.value))
    rc = L.ggcat_gpu_dump_colors(os.fsencode(colormap), buf, nb.value, C.byref(nb), C.byref(nc))
    if rc:
        raise GgcatGpuError(f"dump_colors failed ({_ERRORS.get(rc, rc)})")
    return [x.decode() for x in buf.raw[:nb.value].split(b"\0")[:nc.value]]


def query_colormap(colormap: str, subsets) -> dict:
    """Colours of the given subsets: {subset: [colours]} (ggcat_query_colormap)."""
    L = load()
    out = {}

    def cb(_ctx, subset, cols, n):
        out[int(subset)] = [int(cols[i]) for i in range(n)]

    fn = COLORMAP_FN(cb)
    q = np.ascontiguousarray(np.asarray(subsets, np.uint32))
    rc = L.ggcat_gpu_query_colormap(os.fsencode(colormap), _ptr(q), len(q), 1, fn, None)
    if rc:
        raise GgcatGpuError(f"query_colormap failed ({_ERRORS.get(rc, rc)})")
    return out
