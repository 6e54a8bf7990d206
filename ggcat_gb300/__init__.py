"""ggcat_gb300 — GB300-native (sm_103a) build hot path and query lookup of GGCAT.

The host interface mirrors GGCAT's ``GGCATInstance`` (crates/api/src/lib.rs:118-478):
``GGCATInstance.create(config)`` returns a process-wide singleton, and
``build_graph(...)`` builds the compacted de Bruijn graph of FASTA inputs.  The compute
runs in hand-written CUDA kernels behind the C ABI in ``include/ggcat_gb300.h``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass
from typing import Callable, Optional, Sequence

from ._native import (GGCAT_HASH_RABIN_KARP128, GGCAT_HASH_SEQHASH, GGCAT_MERGE_BATCHED, GGCAT_MERGE_PER_BUCKET,
                      GgcatGpuError, GpuContext, Params, compute_best_m, fasta_parse, load, make_params)

__all__ = [
    "GGCATConfig",
    "GGCATInstance",
    "ExtraElaboration",
    "GfaVersion",
    "GpuContext",
    "GgcatGpuError",
    "Params",
    "make_params",
    "compute_best_m",
    "fasta_parse",
    "GGCAT_MERGE_BATCHED",
    "GGCAT_MERGE_PER_BUCKET",
    "GGCAT_HASH_SEQHASH",
    "GGCAT_HASH_RABIN_KARP128",
]


class ExtraElaboration:
    """crates/api/src/lib.rs:99-116, numbered as the C API numbers the first five
    (capi/src/lib.rs:115-121).  The matchtig family (2-4) is computed over the final unitigs
    (greedy matchtigs of an uncoloured graph only).  FAST_SIMPLITIGS and FAST_EULERTIGS (Rust
    API only; GGCAT builds them inside its merge, eulertigs.rs) are served by the same host
    pathtigs and eulertigs: a simplitig set and the minimum eulertig set, every k-mer once,
    not GGCAT's own strings."""

    NONE = 0
    UNITIG_LINKS = 1
    GREEDY_MATCHTIGS = 2
    EULERTIGS = 3
    PATHTIGS = 4
    FAST_SIMPLITIGS = 5
    FAST_EULERTIGS = 6

    # the C ABI's extra_elab for each value
    _C = {0: 0, 1: 1, 2: 2, 3: 3, 4: 4, 5: 4, 6: 3}


class GfaVersion:
    """crates/api/src/lib.rs:69-72 (as the C API's gfa_output_version: 1, 2)."""

    V1 = 1
    V2 = 2


@dataclass
class GGCATConfig:
    """crates/api/src/lib.rs:75-99."""

    temp_dir: Optional[str] = None
    memory: float = 2.0
    prefer_memory: bool = True
    total_threads_count: int = os.cpu_count() or 1
    intermediate_compression_level: Optional[int] = None
    stats_file: Optional[str] = None
    messages_callback: Optional[Callable[[int, str], None]] = None
    device: int = 0


class GGCATInstance:
    """Process-wide singleton: a second ``create`` returns the first instance and ignores
    its config, as the reference does (crates/api/src/lib.rs:141-214)."""

    _instance: Optional["GGCATInstance"] = None
    _lock = threading.Lock()

    def __init__(self, config: GGCATConfig):
        self.config = config
        self.ctx = GpuContext(config.device)

    @classmethod
    def create(cls, config: GGCATConfig | None = None) -> "GGCATInstance":
        with cls._lock:
            if cls._instance is None:
                cls._instance = GGCATInstance(config or GGCATConfig())
            return cls._instance

    def build_graph(
        self,
        input_streams: Sequence[str],
        output_file: str,
        color_names: Optional[Sequence[str]] = None,
        kmer_length: int = 31,
        threads_count: int = 1,
        forward_only: bool = False,
        minimizer_length: Optional[int] = None,
        colors: bool = False,
        min_multiplicity: int = 2,
        extra_elab: int = ExtraElaboration.NONE,
        gfa_output_version: Optional[int] = None,
    ) -> str:
        """crates/api/src/lib.rs:217-322 — returns the output path ("" on failure, like
        the C API's ``unwrap_or_default``).  With ``colors`` every input is one colour and the
        colormap is written beside the graph (``get_colormap_file``)."""
        if extra_elab not in ExtraElaboration._C:
            raise GgcatGpuError(f"extra_elab {extra_elab} is not an ExtraElaboration")
        if colors and extra_elab == ExtraElaboration.GREEDY_MATCHTIGS:
            raise GgcatGpuError("greedy matchtigs of a coloured graph are not built")
        gfa = int(gfa_output_version or 0)
        if gfa not in (0, GfaVersion.V1, GfaVersion.V2):
            raise GgcatGpuError(f"gfa_output_version {gfa_output_version} is not 1 or 2")
        L = load()
        arr = (C.c_char_p * len(input_streams))(*[os.fsencode(p) for p in input_streams])
        m = (1 << 64) - 1 if minimizer_length is None else minimizer_length
        names = list(color_names or [])
        carr = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
        rc = L.ggcat_gpu_build_from_files_ex(self.ctx.h, arr, len(input_streams), os.fsencode(output_file), carr,
                                             len(names), kmer_length, threads_count, int(forward_only), m,
                                             int(bool(colors)), min_multiplicity, ExtraElaboration._C[extra_elab], gfa)
        if rc != 0:
            msg = L.ggcat_gpu_last_error(self.ctx.h)
            if self.config.messages_callback:
                self.config.messages_callback(2, msg.decode() if msg else "")
            return ""
        return output_file

    def query_graph(
        self,
        input_graph: str,
        input_query: str,
        output_file_prefix: str,
        kmer_length: int = 31,
        threads_count: int = 1,
        forward_only: bool = False,
        minimizer_length: Optional[int] = None,
        colors: bool = False,
        color_output_format: int = 0,
    ) -> str:
        """crates/api/src/lib.rs:325-382: the querier's CSV (query_index,matched_kmers,
        query_kmers,match_percentage), or with ``colors`` the JSON lines of per-colour match
        fractions (``color_output_format`` 0: colour indices, 1: colour names); returns the
        output path ("" on failure, like the C API)."""
        L = load()
        out = C.create_string_buffer(4096)
        m = (1 << 64) - 1 if minimizer_length is None else minimizer_length
        rc = L.ggcat_gpu_query_graph(self.ctx.h, os.fsencode(input_graph), os.fsencode(input_query),
                                     os.fsencode(output_file_prefix), kmer_length, threads_count, int(forward_only), m,
                                     int(bool(colors)), int(color_output_format), out, len(out))
        if rc != 0:
            msg = L.ggcat_gpu_last_error(self.ctx.h)
            if self.config.messages_callback:
                self.config.messages_callback(2, msg.decode() if msg else "")
            return ""
        return out.value.decode()

    @staticmethod
    def get_colormap_file(graph_file: str) -> str:
        """crates/api/src/lib.rs:385-387."""
        from . import _native

        return _native.colormap_file(graph_file)

    @staticmethod
    def dump_colors(input_colormap: str) -> list:
        """crates/api/src/lib.rs:392-408: the colour names, by colour index."""
        from . import _native

        return _native.dump_colors(input_colormap)

    def query_colormap(self, colormap_file: str, subsets, single_thread_output_function: bool,
                       output_function: Callable[[int, list], None]) -> None:
        """crates/api/src/lib.rs:412-429: output_function(subset, colours) per distinct subset."""
        from . import _native

        for sub, cols in sorted(_native.query_colormap(colormap_file, subsets).items()):
            output_function(sub, cols)

    def dump_unitigs(self, graph_input: str, kmer_length: int, minimizer_length: Optional[int], colors: bool,
                     threads_count: int, single_thread_output_function: bool,
                     output_function: Callable[[bytes, list, bool], None]) -> None:
        """crates/api/src/lib.rs:434-477."""
        from . import _native

        for item in _native.dump_unitigs(graph_input, kmer_length, colors):
            if colors:
                output_function(*item)
            else:
                output_function(item, [], False)
