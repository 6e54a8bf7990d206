"""Benchmark of the GB300 build hot path (minimizer bucketing + per-bucket k-mer merge).

One "step" = one pass of the hot path (pack, bucketize, partition, merge with unitig
extension) over the skewed read workload: a 50 Mbp genome with 2% of its length in
500-bp repeats copied 20-200 times, sampled at 20x with 150-bp reads from both strands,
0.5% substitutions, 0.01% N; k=31, m=10, 1024 buckets, min multiplicity 2.  Inputs are
seeded synthetic data of that shape (the reference names no dataset).

Prints one JSON line (rank 0).  ``value`` is Gbases/s with the input resident in HBM;
``e2e`` is the same metric through the C ABI call with host buffers (pinned H2D copy of
the text and D2H of the partial unitigs inside the timed region).

``--impl reference`` times the CPU implementation of the same path on the host cores
(the oracle restatement with all threads: the Rust reference cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "build Gbases/s bit-exact (batched vs per-bucket launch)"

# DRAM bytes (read + write) of the merge-phase kernels per k-mer instance: ncu
# dram__bytes_read.sum + dram__bytes_write.sum of the S, W and M merge_unit_kernel launches on
# the 80 Mbp case of this workload (154.8 MB over 69.47 M instances); scaled by instances.
MERGE_DRAM_BYTES_PER_INSTANCE = 2.23


# the knobs ggcat_gpu_autotune chooses (the sub-bin digit width and the per-class knobs)
TUNED_KNOBS = ("subbin_bytes", "unit_target", "small_limit", "small_batch", "wide_batch", "wide_limit",
               "table_load_pct")


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="skewed", choices=["skewed", "longk"],
                    help="skewed: 150-bp reads of a repeat-rich 50 Mbp genome, k=31 (the headline); "
                         "longk: 250-bp reads of a 100 Mbp GC-0.4 genome, k=63, Rabin-Karp 128-bit hash")
    ap.add_argument("--genome", type=int, default=0, help="genome length (0 = the workload's own)")
    ap.add_argument("--coverage", type=float, default=20.0)
    ap.add_argument("--no-per-bucket", action="store_true", help="skip timing the per-bucket launch form")
    ap.add_argument("--cpu-sample-bases", type=int, default=0,
                    help="reads prefix (bases) the CPU baseline builds; 0 = the whole input")
    ap.add_argument("--ref-budget-s", type=float, default=420.0,
                    help="--impl reference: stop timing steps once this many seconds are spent")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity checks of the GPU outputs against the oracle")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--verify", action="store_true", help="check batched == per-bucket unitig sets (slow)")
    ap.add_argument("--no-query", action="store_true", help="skip the query-serving measurement")
    ap.add_argument("--no-colored", action="store_true", help="skip the coloured build + query measurement")
    ap.add_argument("--colors", type=int, default=256, help="genomes (colours) of the coloured workload")
    ap.add_argument("--query-genomes", type=int, default=16, help="member genomes of the queried graph")
    ap.add_argument("--queries", type=int, default=20000, help="queries of the uncoloured serving measurement")
    ap.add_argument("--colored-queries", type=int, default=100000,
                    help="queries of the coloured serving measurement (against the 256-genome coloured graph)")
    ap.add_argument("--no-autotune", action="store_true", help="skip the autotuned-knobs measurement")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 3-genome and long-k build measurements")
    ap.add_argument("--query-rate", type=float, default=20000.0, help="Poisson arrival rate (queries/s)")
    ap.add_argument("--colored-only", action="store_true",
                    help="run only the coloured build + query section and print its JSON object "
                         "(a small case for profiling the colour kernels: --colors 64 --colored-queries 1000)")
    return ap.parse_args()


def max_over_ranks(value: float, dist, device) -> float:
    """The slowest rank's time (replicas: every rank builds its own copy of the workload)."""
    if not dist:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gbases_per_s(bases_per_rank: int, world_size: int, ms: float) -> float:
    """Whole-job throughput of N replicas: all ranks' bases over the slowest rank's time."""
    return bases_per_rank * world_size / (ms * 1e-3) / 1e9


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _workload(args):
    from ggcat_gb300 import synth

    if args.workload == "longk":
        return synth.config_long_k(genome_len=args.genome or 100_000_000, coverage=args.coverage)
    return synth.config_skewed_reads(genome_len=args.genome or 50_000_000, coverage=args.coverage)


def _hash_kind(w):
    from ggcat_gb300 import _native

    return _native.GGCAT_HASH_RABIN_KARP128 if getattr(w, "hash_kind", "") == "rk128" else _native.GGCAT_HASH_SEQHASH


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.f:
            return None
        try:
            self.f.flush()
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
            os.unlink(self.f.name)
        except Exception:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(w, sample_bases: int, threads: int, keep: bool = False):
    """Times the oracle (CPU restatement, all threads) on the whole input (sample_bases = 0)
    or on a bounded prefix of the reads.  With keep, also returns the oracle's build, which
    then checks the GPU's output on the same input."""
    import oracle

    n_seq = len(w.seq_off)
    per = float(w.seq_len.mean()) if n_seq else 1.0
    take = n_seq if sample_bases <= 0 else max(1, min(n_seq, int(sample_bases / per)))
    end = int(w.seq_off[take - 1] + w.seq_len[take - 1] + 1)
    text = w.text[:end]
    p = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6, min_multiplicity=w.min_multiplicity,
                      threads=threads, hash_kind=oracle.H_CN_RK128 if getattr(w, "hash_kind", "") == "rk128" else None)
    t0 = time.perf_counter()
    r = oracle.build_graph(text, w.seq_off[:take], w.seq_len[:take], p)
    dt = time.perf_counter() - t0
    bases = int(w.seq_len[:take].sum())
    if not keep:
        del r
        r = None
    return bases / dt / 1e9, bases, dt, take, r


def gpu_build_outputs(ctx, text, p, stream=0):
    """Surviving k-mers (with multiplicities) and the canonical final-unitig set of one GPU
    build of host `text` through the C ABI (ggcat_gpu_build_text with keep_kmers, then the
    device link stage)."""
    import oracle
    from ggcat_gb300 import _native

    pk = _native.Params.from_buffer_copy(p)
    pk.keep_kmers = 1
    ctx.build_text(text, pk, stream)
    keys, mult = ctx.kmers()
    ctx.link(p.k)
    bases, uo, ul, uf = ctx.unitigs()
    lines = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, p.k)
    return keys, mult, lines


def build_parity(ctx, text, p, oracle_result, stream=0) -> dict:
    """GPU build of `text` against the oracle's build of the same input: k-mers with
    multiplicities and the final unitig set, both order-free."""
    from oracle import parity

    keys, mult, lines = gpu_build_outputs(ctx, text, p, stream)
    km = parity.compare_kmers(keys, mult, oracle_result)
    un = parity.compare_unitigs(lines, oracle_result)
    return {"equal": bool(km["equal"] and un["equal"]), "kmers": km, "unitigs": un}


def longk_slice_parity(w, n_reads: int, threads: int, dev) -> dict:
    """The first n_reads reads of the long-k workload (k=63, m=12, Rabin-Karp u128, 4096
    buckets, min multiplicity 2): GPU build against the oracle's."""
    import oracle
    from ggcat_gb300 import _native

    take = min(n_reads, len(w.seq_off))
    end = int(w.seq_off[take - 1] + w.seq_len[take - 1] + 1)
    text = w.text[:end]
    op = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6, min_multiplicity=w.min_multiplicity,
                       threads=threads, hash_kind=oracle.H_CN_RK128)
    r = oracle.build_graph(text, w.seq_off[:take], w.seq_len[:take], op)
    ctx = _native.GpuContext(dev)
    try:
        p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6,
                                min_multiplicity=w.min_multiplicity, hash_kind=_native.GGCAT_HASH_RABIN_KARP128)
        out = build_parity(ctx, text, p, r)
    finally:
        ctx.close()
    out["input"] = f"first {take} reads ({int(w.seq_len[:take].sum())} bases) of {w.name}"
    return out


def colored_parity(n_genomes: int, n_queries: int, threads: int, dev) -> dict:
    """The first n_genomes genomes of the coloured workload (one colour each, k=31, m=10,
    4096 buckets): per-k-mer colour sets against the oracle's, then the first n_queries
    queries of the coloured query workload (lengths log-uniform 100 bp - 100 kbp, 80%
    substrings of member genomes) looked up on the GPU's coloured index against the oracle's
    per-query matched and per-colour counts."""
    import oracle
    from oracle import parity
    from ggcat_gb300 import _native, synth

    w = synth.config_colored(n_genomes=n_genomes)
    op = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=1, min_multiplicity=1, threads=threads,
                       colors=True)
    r = oracle.build_graph(w.text, w.seq_off, w.seq_len, op, seq_colors=w.seq_color)
    ctx = _native.GpuContext(dev)
    try:
        p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=1, min_multiplicity=1,
                                keep_kmers=True)
        ctx.colors_prepare(w.seq_off, w.seq_color, n_genomes)  # colours collected by the merge
        ctx.build_text(w.text, p)
        ctx.colors(w.seq_off, w.seq_color, n_genomes)
        collected = bool(ctx.stats()["colors_collected"])
        keys, _ = ctx.kmers()
        cs = parity.compare_color_sets(keys, ctx.kmer_subsets(), ctx.subsets(), r)
        cs["collected_by_merge"] = collected
        ctx.query_index_colored()
        genomes = [w.text[int(o):int(o) + int(ln)] for o, ln in zip(w.seq_off.tolist(), w.seq_len.tolist())]
        qt, qo, ql, _ = synth.query_workload(genomes, n_queries)
        ctx.query_submit(0, qt, qo, ql)
        matched = ctx.query_wait(0)
        counts = ctx.query_color_counts(0)
    finally:
        ctx.close()
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    em, _, epc = oracle.query(lo, hi, qt, qo, ql, w.k, gc_off=coff, gc_colors=ccol, ncolors=n_genomes)
    q = parity.compare_query_counts(matched, counts, em, epc)
    return {"colors": {**cs, "input": f"first {n_genomes} genomes of the coloured workload ({w.name})"},
            "query": {**q, "input": f"first {n_queries} queries of the coloured query workload"}}


def query_bench(args, ctx, torch, dev):
    """Query serving: graph of member genomes built on the GPU (bucketize + merge + link),
    resident index, Poisson arrivals of mixed-length queries, continuous batching vs one
    query per launch.  Returns the JSON object of the query measurement."""
    from ggcat_gb300 import _native, serve, synth

    rng = np.random.default_rng(0x67636174 + 3)
    anc = synth.random_genome(4_000_000, rng)
    genomes = [synth.indels(synth.substitute(anc, float(rng.uniform(0.001, 0.02)), rng), 0.0005, 50, rng)
               for _ in range(args.query_genomes)]
    text, off, ln, _ = synth.pack_sequences(genomes)
    p = _native.make_params(k=31, m=10, bucket_bits=12, second_bits=4, min_multiplicity=1)
    ctx.build_text(text, p)
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    graph = np.frombuffer(_native.unitig_lines(bases, uo, ul), np.uint8)
    d_graph = torch.from_numpy(graph.copy()).to(f"cuda:{dev}")
    t0 = time.perf_counter()
    ctx.query_index(d_graph.data_ptr(), d_graph.numel(), 31)
    index_s = time.perf_counter() - t0
    qt, qo, ql, arr = synth.query_workload(genomes, args.queries, rate_per_s=args.query_rate)
    # warm-up
    serve.serve(ctx, 31, qt, qo[:200], ql[:200], np.zeros(200), slots=4)
    budget = 256 << 20
    free_fn = lambda: torch.cuda.mem_get_info(dev)[0]  # noqa: E731  (asked at every admission)
    rb = serve.serve(ctx, 31, qt, qo, ql, arr, slots=4, max_batch_kmers=budget, free_bytes=free_fn)
    n1 = min(len(qo), max(1000, args.queries // 10))
    r1 = serve.serve(ctx, 31, qt, qo[:n1], ql[:n1], arr[:n1], slots=4, one_per_launch=True)
    rb1 = serve.serve(ctx, 31, qt, qo[:n1], ql[:n1], arr[:n1], slots=4, max_batch_kmers=budget, free_bytes=free_fn)
    same = bool((rb.matched[:n1] == r1.matched).all() and (rb1.matched == r1.matched).all())
    return {
        "metric": "query kmers/s + p50/p99 ms",
        "graph": f"{args.query_genomes} genomes x 4 Mbp (ancestor + 0.1-2% substitutions, 0.05% indels), "
                 f"{len(uo)} unitigs, uncoloured",
        "queries": int(len(qo)),
        "query_kmers": int(rb.kmers),
        "arrival_rate_per_s": args.query_rate,
        "batched": {"kmers_per_s": round(rb.kmers_per_s, 1), "p50_ms": round(rb.pct_ms(50), 3),
                    "p99_ms": round(rb.pct_ms(99), 3), "batches": rb.batches, "wall_s": round(rb.wall_s, 3),
                    "max_batch_kmers": budget},
        "one_per_launch": {"queries": int(n1), "kmers_per_s": round(r1.kmers_per_s, 1),
                           "p50_ms": round(r1.pct_ms(50), 3), "p99_ms": round(r1.pct_ms(99), 3),
                           "wall_s": round(r1.wall_s, 3)},
        "like_for_like": {"queries": int(n1), "batched": {"kmers_per_s": round(rb1.kmers_per_s, 1),
                                                          "p50_ms": round(rb1.pct_ms(50), 3),
                                                          "p99_ms": round(rb1.pct_ms(99), 3)},
                          "one_per_launch": {"kmers_per_s": round(r1.kmers_per_s, 1),
                                             "p50_ms": round(r1.pct_ms(50), 3), "p99_ms": round(r1.pct_ms(99), 3)}},
        "results_identical_alone_vs_batched": same,
        "index_build_s": round(index_s, 3),
    }


def colored_bench(args, ctx, torch, dev):
    """Coloured build (256 genomes x 4 Mbp from one ancestor, one colour each, k=31, 4096
    buckets): device build, colour-subset dedup, then coloured query serving (per query and
    colour, the number of query k-mers present in that colour)."""
    from ggcat_gb300 import _native, serve, synth

    w = synth.config_colored(n_genomes=args.colors)
    p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=1, min_multiplicity=1,
                            keep_kmers=True)
    stream = torch.cuda.current_stream(dev).cuda_stream
    res = {}
    for rep_i in range(2):  # the first pass warms up (allocations)
        # the colour table announced before the build: the merge collects the colours and the
        # colour phase merges the dumped copies instead of reading the text again
        ctx.colors_prepare(w.seq_off, w.seq_color, args.colors)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.build_text(w.text, p, stream)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ctx.colors(w.seq_off, w.seq_color, args.colors, stream)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        st = ctx.stats()
        res = {"build_e2e_ms": round((t1 - t0) * 1e3, 3), "ms_bucketize": round(st["ms_bucketize"], 3),
               "ms_merge": round(st["ms_merge"], 3), "colors_ms": round((t2 - t1) * 1e3, 3),
               "colors_collected_by_merge": bool(st["colors_collected"]),
               "merge_class_ms": [round(x, 3) for x in st["ms_tier"]]}
    n_sub = int(ctx.subsets().shape[0])
    st = ctx.stats()
    ctx.query_index_colored()
    genomes = [w.text[int(o):int(o) + int(ln)] for o, ln in zip(w.seq_off.tolist(), w.seq_len.tolist())]
    qt, qo, ql, arr = synth.query_workload(genomes, args.colored_queries, rate_per_s=args.query_rate)
    serve.serve(ctx, 31, qt, qo[:200], ql[:200], np.zeros(200), slots=4, colored=True)
    budget = 256 << 20
    free_fn = lambda: torch.cuda.mem_get_info(dev)[0]  # noqa: E731  (asked at every admission)
    rb = serve.serve(ctx, 31, qt, qo, ql, arr, slots=4, max_batch_kmers=budget, colored=True, free_bytes=free_fn)
    n1 = min(len(qo), 10000)
    r1 = serve.serve(ctx, 31, qt, qo[:n1], ql[:n1], arr[:n1], slots=4, one_per_launch=True, colored=True)
    rb1 = serve.serve(ctx, 31, qt, qo[:n1], ql[:n1], arr[:n1], slots=4, max_batch_kmers=budget, colored=True,
                      free_bytes=free_fn)
    same = bool((rb.matched[:n1] == r1.matched).all() and (rb.color_totals[:n1] == r1.color_totals).all()
                and (rb1.matched == r1.matched).all())
    # arrival-rate sweep (the knee): the same queries with the Poisson gaps scaled; "inf" = all
    # queries waiting at t = 0
    sweep = []
    # untimed pass with every query waiting at t = 0: the slots' pinned staging buffers grow to
    # the largest batch here, not inside the measured runs
    serve.serve(ctx, 31, qt, qo, ql, np.zeros_like(arr), slots=4, max_batch_kmers=budget, colored=True,
                free_bytes=free_fn)
    for rate in (80_000.0, 320_000.0, float("inf")):
        a2 = np.zeros_like(arr) if rate == float("inf") else arr * (args.query_rate / rate)
        r2 = serve.serve(ctx, 31, qt, qo, ql, a2, slots=4, max_batch_kmers=budget, colored=True, free_bytes=free_fn)
        sweep.append({"arrival_rate_per_s": rate if rate != float("inf") else "all at t=0",
                      "kmers_per_s": round(r2.kmers_per_s, 1), "p50_ms": round(r2.pct_ms(50), 3),
                      "p99_ms": round(r2.pct_ms(99), 3), "batches": r2.batches})
    return {
        "workload": w.name, "bases": int(w.bases), "colors": args.colors,
        "build": {**res, "device_gbases_per_s": round(w.bases / ((res["ms_bucketize"] + res["ms_merge"]) * 1e-3) / 1e9, 3),
                  "distinct_kmers": int(st["distinct_kmers"]), "surviving_kmers": int(st["surviving_kmers"]),
                  "color_subsets": n_sub},
        "query": {"queries": int(len(qo)), "query_kmers": int(rb.kmers), "arrival_rate_per_s": args.query_rate,
                  "kmers_per_s": round(rb.kmers_per_s, 1), "p50_ms": round(rb.pct_ms(50), 3),
                  "p99_ms": round(rb.pct_ms(99), 3), "batches": rb.batches, "max_batch_kmers": budget,
                  "color_hits_total": int(rb.color_totals.sum()),
                  "one_per_launch": {"queries": int(n1), "kmers_per_s": round(r1.kmers_per_s, 1),
                                     "p50_ms": round(r1.pct_ms(50), 3), "p99_ms": round(r1.pct_ms(99), 3)},
                  "like_for_like": {"queries": int(n1),
                                    "batched": {"kmers_per_s": round(rb1.kmers_per_s, 1),
                                                "p50_ms": round(rb1.pct_ms(50), 3), "p99_ms": round(rb1.pct_ms(99), 3)},
                                    "one_per_launch": {"kmers_per_s": round(r1.kmers_per_s, 1),
                                                       "p50_ms": round(r1.pct_ms(50), 3),
                                                       "p99_ms": round(r1.pct_ms(99), 3)}},
                  "results_identical_alone_vs_batched": same, "rate_sweep": sweep},
    }


def build_config_bench(w, torch, dev, steps=3, cpu_threads=0, tune=False):
    """One build workload on a fresh context: device Gbases/s (bucketize + merge, input in
    HBM, median of `steps` after one warm-up) and end-to-end Gbases/s through the C ABI from
    pinned host memory (text copy in, partial unitigs out), plus the host link stage time.
    With cpu_threads > 0 the oracle (CPU restatement) builds the whole input too."""
    from ggcat_gb300 import _native

    ctx = _native.GpuContext(dev)
    try:
        hk = _native.GGCAT_HASH_RABIN_KARP128 if getattr(w, "hash_kind", "") == "rk128" else _native.GGCAT_HASH_SEQHASH
        p = _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6,
                                min_multiplicity=w.min_multiplicity, hash_kind=hk)
        d = torch.from_numpy(w.text).to(f"cuda:{dev}")
        ms = []
        for i in range(steps + 1):
            ctx.bucketize(d.data_ptr(), d.numel(), p, 0)
            ctx.merge(p, 0)
            torch.cuda.synchronize()
            st = ctx.stats()
            if i:
                ms.append(st["ms_pack"] + st["ms_bucketize"] + st["ms_merge"])
        tuned = None
        if tune:
            t0 = time.perf_counter()
            best, d_ms, b_ms = ctx.autotune(d.data_ptr(), d.numel(), p)
            tune_s = time.perf_counter() - t0
            ms_t = []
            for i in range(steps + 1):
                ctx.bucketize(d.data_ptr(), d.numel(), best, 0)
                ctx.merge(best, 0)
                torch.cuda.synchronize()
                st = ctx.stats()
                if i:
                    ms_t.append(st["ms_pack"] + st["ms_bucketize"] + st["ms_merge"])
            tuned = {"device_gbases_per_s": round(w.bases / (statistics.median(ms_t) * 1e-3) / 1e9, 3),
                     "device_ms": round(statistics.median(ms_t), 3), "tuning_s": round(tune_s, 2),
                     "knobs": {f: int(getattr(best, f)) for f in TUNED_KNOBS}}
        del d
        dev_ms = statistics.median(ms)
        h = torch.from_numpy(w.text).pin_memory()
        ctx.build_text(h.numpy(), p)
        torch.cuda.synchronize()
        e2e_runs = []
        for _ in range(3):  # median of three host-memory builds (one is noisy on the host side)
            t0 = time.perf_counter()
            ctx.build_text(h.numpy(), p)
            e2e_runs.append(time.perf_counter() - t0)
        e2e_s = statistics.median(e2e_runs)
        ctx.link(w.k)
        st = ctx.stats()
        link_ms = st["ms_link"]
        out = {"workload": w.name, "bases": int(w.bases), "k": w.k, "m": w.m, "buckets": 1 << w.bucket_bits,
               "min_multiplicity": w.min_multiplicity, "hash": getattr(w, "hash_kind", "seq-hash"),
               "device_gbases_per_s": round(w.bases / (dev_ms * 1e-3) / 1e9, 3), "device_ms": round(dev_ms, 3),
               "e2e_gbases_per_s": round(w.bases / e2e_s / 1e9, 3), "link_ms": round(link_ms, 1),
               "e2e_final_unitigs_gbases_per_s": round(w.bases / (e2e_s + link_ms * 1e-3) / 1e9, 3),
               "autotuned": tuned,
               "superkmers": int(st["superkmers"]), "kmer_instances": int(st["kmer_instances"]),
               "final_unitigs": int(st["final_unitigs"])}
        if cpu_threads > 0:
            # the oracle builds the whole input (timed), then checks the GPU's k-mers and unitigs
            import oracle

            op = oracle.params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6,
                               min_multiplicity=w.min_multiplicity, threads=cpu_threads,
                               hash_kind=oracle.H_CN_RK128 if getattr(w, "hash_kind", "") == "rk128" else None)
            t0 = time.perf_counter()
            r = oracle.build_graph(w.text, w.seq_off, w.seq_len, op)
            dt = time.perf_counter() - t0
            out["cpu_oracle"] = {"gbases_per_s": round(w.bases / dt / 1e9, 5), "seconds": round(dt, 2),
                                 "cores": cpu_threads, "kind": "port"}
            out["parity"] = build_parity(ctx, w.text, p, r)
            out["surviving_kmers"] = out["parity"]["kmers"]["kmers_gpu"]
            del r
    finally:
        ctx.close()
    return out


def run_reference(args):
    """The CPU arm: the oracle restatement (C, all host threads) builds the whole input of the
    GPU arm's workload in every timed step (the Rust reference cannot be compiled here).
    Warm-up steps build a 30 Mbp prefix.  A full-input step takes tens of seconds, so timed
    steps stop once --ref-budget-s is spent; the line reports the steps actually timed."""
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    w = _workload(args)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(w, 30_000_000, threads)
    vals, t_start = [], time.perf_counter()
    bases = take = 0
    for i in range(args.steps):
        v, bases, dt, take, _ = cpu_baseline(w, args.cpu_sample_bases, threads)
        vals.append(v)
        spent = time.perf_counter() - t_start
        if spent + dt > args.ref_budget_s:
            break
    value = statistics.median(vals)
    whole = take == len(w.seq_off)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 6),
        "unit": "Gbases/s",
        "n_gpus": args.gpus,
        "steps": len(vals),
        "steps_requested": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(bases / value / 1e6, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64" if w.k <= 32 else "u128",
        "data": "synthetic (seeded)",
        "config": _config(w, ws) if whole else {**_config(w, ws), "workload": w.name + f" (first {take} reads)"},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gbases/s", "cores": threads, "kind": "port",
                         "sample": (f"whole input ({take} reads, {bases} bases) per step" if whole else
                                    f"first {take} reads ({bases} bases) per step") +
                                   "; the Rust reference cannot be compiled here, so the oracle restatement "
                                   "(C, pthreads) is timed; warm-up steps on a 30 Mbp prefix"},
        "e2e": {"value": round(value, 6), "unit": "Gbases/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _config(w, ws):
    return {"workload": w.name, "k": w.k, "m": w.m, "buckets": 1 << w.bucket_bits,
            "min_multiplicity": w.min_multiplicity, "bases_per_gpu": int(w.bases),
            "hash": getattr(w, "hash_kind", "seq-hash"),
            "l2": (f"input ({w.text.size / 1e9:.2f} GB) larger than L2 (129 MB); no flush" if w.text.size > 129e6
                   else f"input ({w.text.size / 1e6:.1f} MB) fits in L2; no flush"),
            "parallelism": f"replicas x{ws}"}


def run_gpu(args):
    import torch

    from ggcat_gb300 import _native

    ws, rank, local = _dist()
    dev = local
    torch.cuda.set_device(dev)
    dist = None
    if ws > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=torch.device("cuda", dev))
        dist = tdist
    w = _workload(args)
    bases = w.bases
    ctx = _native.GpuContext(dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    d_text = torch.from_numpy(w.text).to(f"cuda:{dev}")
    torch.cuda.synchronize()

    def params(mode):
        return _native.make_params(k=w.k, m=w.m, bucket_bits=w.bucket_bits, second_bits=6,
                                   min_multiplicity=w.min_multiplicity, merge_mode=mode, hash_kind=_hash_kind(w))

    def step(p):
        ctx.bucketize(d_text.data_ptr(), d_text.numel(), p, sptr)
        ctx.merge(p, sptr)

    def timed(p, steps, warmup):
        for _ in range(warmup):
            step(p)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = ctx.kernel_launches
        e0.record(stream)
        ph = {"ms_pack": 0.0, "ms_bucketize": 0.0, "ms_merge": 0.0}
        for _ in range(steps):
            step(p)
            st = ctx.stats()
            for key in ph:
                ph[key] += st[key]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, dist, f"cuda:{dev}")
        return ms, (ctx.kernel_launches - l0) // steps, {k2: v / steps for k2, v in ph.items()}, st

    pb = params(_native.GGCAT_MERGE_BATCHED)
    with ClockSampler(dev) as clk:
        ms, launches, phases, st = timed(pb, args.steps, args.warmup)
    clocks = clk.summary()
    value = job_gbases_per_s(bases, ws, ms)

    # autotuned knobs (sub-bin digit width, then per bucket-size class: S-unit packing, size
    # limit and insert batch, W insert batch and size limit, global-table load) on the same
    # input, timed like the headline
    autotuned = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        best, d_ms, b_ms = ctx.autotune(d_text.data_ptr(), d_text.numel(), pb, 0, sptr)
        tune_s = time.perf_counter() - t0
        ms_t, _, phases_t, _ = timed(best, max(1, min(args.steps, 3)), 1)
        autotuned = {"value": round(bases * ws / (ms_t * 1e-3) / 1e9, 4), "ms_per_step": round(ms_t, 3),
                     "phases_ms": {k2: round(v, 3) for k2, v in phases_t.items()},
                     "class_ms_default": [round(x, 3) for x in st["ms_tier"]],
                     "class_ms_tuned": [round(x, 3) for x in ctx.stats()["ms_tier"]],
                     "knobs": {f: int(getattr(best, f)) for f in TUNED_KNOBS},
                     "tuning_s": round(tune_s, 2), "trial_ms_default": round(d_ms, 3), "trial_ms_tuned": round(b_ms, 3)}

    per_bucket = None
    if not args.no_per_bucket:
        pp = params(_native.GGCAT_MERGE_PER_BUCKET)
        ms_pb, launches_pb, phases_pb, _ = timed(pp, max(1, min(args.steps, 3)), 1)
        per_bucket = {"value": round(bases * ws / (ms_pb * 1e-3) / 1e9, 4), "ms_per_step": round(ms_pb, 3),
                      "ms_merge": round(phases_pb["ms_merge"], 3), "gpu_launches": launches_pb,
                      "merge_speedup_batched": round(phases_pb["ms_merge"] / max(phases["ms_merge"], 1e-9), 2)}

    # e2e through the C ABI with host buffers (pinned input; partial unitigs read back)
    h_text = torch.from_numpy(w.text).pin_memory()
    hp = h_text.numpy()
    for _ in range(max(1, args.warmup)):
        ctx.build_text(hp, pb, sptr)
    torch.cuda.synchronize()
    e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e_steps):
        ctx.build_text(hp, pb, sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / e_steps
    st2 = ctx.stats()
    d2h = int(st2["partial_bases"] + st2["partial_unitigs"] * (8 + 4 + 1))
    e2e_value = bases * ws / wall / 1e9
    # the whole build to final unitigs: the same call, then the device link stage (pairing of
    # sub-bucket boundary ends, chains and cycles) with the unitigs copied to the host; one
    # untimed round first (the link stage's buffers are allocated on its first call), then the
    # median of three timed rounds
    ctx.build_text(hp, pb, sptr)
    ctx.link(w.k)
    full, links = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        ctx.build_text(hp, pb, sptr)
        ctx.link(w.k)
        full.append(time.perf_counter() - t0)
        links.append(ctx.stats()["ms_link"])
    full_s = statistics.median(full)
    st3 = ctx.stats()
    e2e_final = {"value": round(bases * ws / full_s / 1e9, 4), "unit": "Gbases/s",
                 "link_ms": round(statistics.median(links), 3), "final_unitigs": int(st3["final_unitigs"])}

    # roofline of the dominant phase, the merge (merge_unit_kernel S and M tiers + L kernels,
    # about 3/4 of the step).  Algorithmic bytes per step: every superkmer read once in 2-bit
    # form with an 8-byte header (ceil(L/4) + 8), every k-mer instance's key written and read
    # once (8 + 8 bytes), every distinct k-mer of a unit written with its count (8 + 4).
    peak, peak_kind = _peaks()
    n = w.text.size
    S, I, D = st["superkmers"], st["kmer_instances"], st["distinct_kmers"]
    merge_bytes = (I + S * (w.k - 1)) / 4 + S * 8.375 + 16 * I + 12 * D
    merge_ms = phases["ms_merge"]
    achieved = merge_bytes / (merge_ms * 1e-3) / 1e9 if merge_ms > 0 else 0.0
    # DRAM bytes of the merge kernels per k-mer instance, from one ncu capture of the 4 Mbp-genome
    # (80 Mbp of reads) case of this workload, scaled by the instances of this step
    traffic = round(MERGE_DRAM_BYTES_PER_INSTANCE * I) if MERGE_DRAM_BYTES_PER_INSTANCE else None
    roofline = {"bound": "hbm", "kernel": "merge phase: merge_unit_kernel S/W/M tiers + large_* (one CUDA graph)",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_step": int(merge_bytes), "phase_ms": round(merge_ms, 3)}
    # the bucketing phase (pack + bucketize + partition), algorithmic bytes per step: the ASCII
    # text read once and every superkmer written once in 2-bit form with an 8-byte header,
    # N + sum(ceil(L/4) + 8) (the bucket store's record payload)
    bucket_bytes = n + (I + S * (w.k - 1)) / 4 + S * 8.375
    bucket_ms = phases["ms_pack"] + phases["ms_bucketize"]
    b_ach = bucket_bytes / (bucket_ms * 1e-3) / 1e9 if bucket_ms > 0 else 0.0
    roofline_bucketing = {"bound": "hbm", "kernel": "pack_kernel + bucketize_kernel + partition_kernel",
                          "achieved": round(b_ach, 1),
                          "peak": peak, "unit": "GB/s", "frac": round(b_ach / peak, 4), "peak_kind": peak_kind,
                          "algorithmic_bytes_per_step": int(bucket_bytes), "phase_ms": round(bucket_ms, 3)}

    # CPU baseline: the oracle builds the whole input once (timed); its output then checks the
    # GPU's build of the same input (k-mers with multiplicities, final unitigs), outside every
    # timed region
    cpu, parity = None, {}
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, cb, dt, take, r = cpu_baseline(w, args.cpu_sample_bases, threads, keep=not args.no_parity)
        whole = take == len(w.seq_off)
        cpu = {"value": round(v, 6), "unit": "Gbases/s", "cores": threads, "kind": "port",
               "sample": (f"whole input ({take} reads, {cb} bases)" if whole else f"first {take} reads ({cb} bases)")
                         + f", oracle restatement (C, pthreads), one run of {dt:.1f} s"}
        if r is not None:
            end = int(w.seq_off[take - 1] + w.seq_len[take - 1] + 1)
            parity["C2_" + ("whole_input" if whole else "prefix")] = build_parity(ctx, w.text[:end], pb, r, sptr)
            del r

    query = None
    if rank == 0 and not args.no_query:
        query = query_bench(args, ctx, torch, dev)
    colored = None
    if rank == 0 and not args.no_colored:
        colored = colored_bench(args, ctx, torch, dev)
    ctx.close()
    del d_text
    torch.cuda.empty_cache()

    configs = None
    if rank == 0 and not args.no_configs:
        from ggcat_gb300 import synth

        configs = {"genomes_3x5Mbp": build_config_bench(synth.config_genomes(), torch, dev, steps=5,
                                                        cpu_threads=0 if args.no_cpu_baseline else
                                                        os.cpu_count() or 1)}
        w_longk = synth.config_long_k()
        configs["longk_2Gbp"] = build_config_bench(w_longk, torch, dev, steps=3, tune=True)

    if configs is not None and not args.no_parity:
        parity.update({"C1_" + k2: v2["parity"] for k2, v2 in configs.items() if "parity" in v2})
    if rank == 0 and not args.no_parity and not args.no_configs and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        parity["C4_longk_slice"] = longk_slice_parity(w_longk, 400_000, threads, dev)
        parity["C3_C5_colored_32"] = colored_parity(32, 2000, threads, dev)
    if parity:
        flags = [v.get("equal", all(x.get("equal") for x in v.values() if isinstance(x, dict)))
                 for v in parity.values()]
        parity["all_equal"] = bool(all(flags))

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 4),
            "unit": "Gbases/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms, 3),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "u64" if w.k <= 32 else "u128",
            "data": "synthetic (seeded)",
            "config": _config(w, ws),
            "merge": "batched persistent",
            "phases_ms": {k2: round(v, 3) for k2, v in phases.items()},
            "stats": {"superkmers": int(st["superkmers"]), "kmer_instances": int(st["kmer_instances"]),
                      "distinct_kmers": int(D), "partial_unitigs": int(st["partial_unitigs"]),
                      "small_units": int(st["merge_units_small"]), "large_units": int(st["merge_units_large"]),
                      "spilled_units": int(st["merge_units_spilled"])},
            "per_bucket": per_bucket,
            "autotuned": autotuned,
            "e2e": {"value": round(e2e_value, 4), "unit": "Gbases/s", "h2d_bytes_per_step": int(n),
                    "d2h_bytes_per_step": d2h},
            "e2e_final_unitigs": e2e_final,
            "gpu_launches": int(launches),
            "roofline": roofline,
            "roofline_bucketing": roofline_bucketing,
            "cpu_baseline": cpu,
            "parity": parity or None,
            "query": query,
            "colored": colored,
            "configs": configs,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_colored_only(args):
    import torch

    from ggcat_gb300 import _native

    torch.cuda.set_device(0)
    ctx = _native.GpuContext(0)
    try:
        print(json.dumps({"section": "colored", **colored_bench(args, ctx, torch, 0)}), flush=True)
    finally:
        ctx.close()
    return 0


def main():
    args = _args()
    if args.colored_only:
        return run_colored_only(args)
    if args.workload != "skewed":
        args.no_query = True  # the query and coloured sections use k=31 graphs
        args.no_colored = True
        args.no_configs = True
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
