"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference publishes no dataset for this path, so every workload is generated
from a seed: i.i.d. genomes (optionally GC-biased), mutated copies with
substitutions and indels, repeat families, and reads sampled from both strands
with substitution errors and ``N`` calls.

Inputs are returned in the device "text" layout used by the library: all sequences
concatenated, each followed by one ``\\n`` separator byte (a non-ACGT byte, so it
splits k-mers exactly like an ``N``), plus ``(offset, length)`` per sequence.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
_COMP = np.zeros(256, dtype=np.uint8)
for a, b in zip(b"ACGTNacgtn\n", b"TGCANtgcan\n"):
    _COMP[a] = b


def revcomp(seq: np.ndarray) -> np.ndarray:
    return _COMP[seq[::-1]]


def random_genome(n: int, rng: np.random.Generator, gc: float = 0.5) -> np.ndarray:
    """i.i.d. genome; P(C)=P(G)=gc/2, P(A)=P(T)=(1-gc)/2."""
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    return BASES[rng.choice(4, size=n, p=p).astype(np.uint8)]


def substitute(seq: np.ndarray, rate: float, rng: np.random.Generator) -> np.ndarray:
    out = seq.copy()
    if rate <= 0 or len(seq) == 0:
        return out
    idx = np.nonzero(rng.random(len(seq)) < rate)[0]
    code = np.searchsorted(BASES, out[idx])  # A0 C1 G2 T3 in BASES order
    code = (code + rng.integers(1, 4, size=len(idx))) % 4
    out[idx] = BASES[code]
    return out


def indels(seq: np.ndarray, rate: float, max_len: int, rng: np.random.Generator) -> np.ndarray:
    """Random insertions/deletions of length U[1, max_len] at per-base rate ``rate``."""
    if rate <= 0:
        return seq.copy()
    n_ev = rng.binomial(len(seq), rate)
    pos = np.sort(rng.integers(0, len(seq), size=n_ev))
    lens = rng.integers(1, max_len + 1, size=n_ev)
    is_ins = rng.random(n_ev) < 0.5
    pieces = []
    last = 0
    for p, ln, ins in zip(pos.tolist(), lens.tolist(), is_ins.tolist()):
        if p < last:
            continue
        pieces.append(seq[last:p])
        if ins:
            pieces.append(BASES[rng.integers(0, 4, size=ln)])
            last = p
        else:
            last = min(len(seq), p + ln)
    pieces.append(seq[last:])
    return np.concatenate(pieces)


def add_repeats(seq: np.ndarray, frac: float, rep_len: int, cmin: int, cmax: int, rng: np.random.Generator):
    """Overwrite ``frac`` of the genome with copies of ``rep_len``-bp repeat families,
    each family copied U[cmin, cmax] times at random positions."""
    out = seq.copy()
    target = int(frac * len(seq))
    done = 0
    while done < target:
        fam = BASES[rng.integers(0, 4, size=rep_len)]
        copies = int(rng.integers(cmin, cmax + 1))
        for p in rng.integers(0, len(seq) - rep_len, size=copies).tolist():
            out[p : p + rep_len] = fam
        done += copies * rep_len
    return out


def sample_reads(genome: np.ndarray, n_reads: int, read_len: int, sub_rate: float, n_rate: float,
                 rng: np.random.Generator, chunk: int = 1 << 20) -> np.ndarray:
    """Reads from uniform positions on both strands; returns an (n_reads, read_len) array."""
    out = np.empty((n_reads, read_len), dtype=np.uint8)
    ar = np.arange(read_len)
    for s in range(0, n_reads, chunk):
        e = min(n_reads, s + chunk)
        starts = rng.integers(0, len(genome) - read_len + 1, size=e - s)
        r = genome[starts[:, None] + ar[None, :]]
        rc = rng.random(e - s) < 0.5
        r[rc] = _COMP[r[rc][:, ::-1]]
        if sub_rate > 0:
            m = rng.random(r.shape) < sub_rate
            code = np.searchsorted(BASES, r[m])
            r[m] = BASES[(code + rng.integers(1, 4, size=code.shape)) % 4]
        if n_rate > 0:
            r[rng.random(r.shape) < n_rate] = ord("N")
        out[s:e] = r
    return out


@dataclass
class Workload:
    """Sequences in text layout plus per-sequence colour (file index)."""

    name: str
    text: np.ndarray  # uint8, sequences each followed by b"\n"
    seq_off: np.ndarray  # uint64
    seq_len: np.ndarray  # uint64
    seq_color: np.ndarray  # uint32, colour (input file index) of each sequence
    k: int
    m: int
    bucket_bits: int
    min_multiplicity: int
    hash_kind: str = "seqhash"
    colors: bool = False

    @property
    def bases(self) -> int:
        return int(self.seq_len.sum())


def pack_sequences(seqs: list[np.ndarray], colors: list[int] | None = None) -> tuple:
    lens = np.array([len(s) for s in seqs], dtype=np.uint64)
    off = np.zeros(len(seqs), dtype=np.uint64)
    if len(seqs) > 1:
        off[1:] = np.cumsum(lens[:-1] + 1)
    text = np.empty(int(lens.sum()) + len(seqs), dtype=np.uint8)
    for o, s in zip(off.tolist(), seqs):
        text[o : o + len(s)] = s
        text[o + len(s)] = 10
    col = np.zeros(len(seqs), np.uint32) if colors is None else np.asarray(colors, np.uint32)
    return text, off, lens, col


def pack_reads(reads: np.ndarray) -> tuple:
    n, L = reads.shape
    text = np.empty((n, L + 1), dtype=np.uint8)
    text[:, :L] = reads
    text[:, L] = 10
    off = np.arange(n, dtype=np.uint64) * np.uint64(L + 1)
    lens = np.full(n, L, dtype=np.uint64)
    return text.reshape(-1), off, lens, np.zeros(n, np.uint32)


def config_genomes(seed: int = 0x67636174 + 1, genome_len: int = 5_000_000, n_genomes: int = 3) -> Workload:
    """Plain uncoloured build: genome 1 i.i.d.; the others copy it with 1% substitutions
    and 0.1% indels of 1-10 bp.  k=31, m=10, 1024 buckets, min multiplicity 1."""
    rng = np.random.default_rng(seed)
    g1 = random_genome(genome_len, rng)
    gs = [g1] + [indels(substitute(g1, 0.01, rng), 0.001, 10, rng) for _ in range(n_genomes - 1)]
    text, off, ln, col = pack_sequences(gs)
    return Workload("genomes-3x5Mbp", text, off, ln, col, k=31, m=10, bucket_bits=10, min_multiplicity=1)


def config_skewed_reads(seed: int = 0x67636174 + 2, genome_len: int = 50_000_000, coverage: float = 20.0,
                        read_len: int = 150) -> Workload:
    """Skewed read set: genome with 2% of its length in 500-bp repeats copied 20-200
    times; reads at ``coverage`` from both strands, 0.5% substitutions, 0.01% N.
    k=31, m=10, 1024 buckets, min multiplicity 2."""
    rng = np.random.default_rng(seed)
    g = random_genome(genome_len, rng)
    g = add_repeats(g, 0.02, 500, 20, 200, rng)
    n_reads = int(genome_len * coverage / read_len)
    reads = sample_reads(g, n_reads, read_len, 0.005, 0.0001, rng)
    text, off, ln, col = pack_reads(reads)
    return Workload(f"skewed-reads-{n_reads}x{read_len}bp", text, off, ln, col, k=31, m=10, bucket_bits=10,
                    min_multiplicity=2)


def config_colored(seed: int = 0x67636174 + 3, genome_len: int = 4_000_000, n_genomes: int = 256) -> Workload:
    """Coloured build: genomes derived from one ancestor with per-genome substitution
    rate U[0.1%, 2%] and 0.05% indels of 1-50 bp; one colour per genome.  k=31, m=10,
    4096 buckets, min multiplicity 1."""
    rng = np.random.default_rng(seed)
    anc = random_genome(genome_len, rng)
    gs = []
    for _ in range(n_genomes):
        rate = float(rng.uniform(0.001, 0.02))
        gs.append(indels(substitute(anc, rate, rng), 0.0005, 50, rng))
    text, off, ln, col = pack_sequences(gs, list(range(n_genomes)))
    return Workload(f"colored-{n_genomes}x{genome_len // 1_000_000}Mbp", text, off, ln, col, k=31, m=10,
                    bucket_bits=12, min_multiplicity=1, colors=True)


def config_long_k(seed: int = 0x67636174 + 4, genome_len: int = 100_000_000, coverage: float = 20.0,
                  read_len: int = 250) -> Workload:
    """Long-k reads: GC 0.4 genome, 250-bp reads at 20x, 1% substitutions.  k=63, m=12,
    Rabin-Karp 128-bit merging hash, 4096 buckets, min multiplicity 2."""
    rng = np.random.default_rng(seed)
    g = random_genome(genome_len, rng, gc=0.4)
    n_reads = int(genome_len * coverage / read_len)
    reads = sample_reads(g, n_reads, read_len, 0.01, 0.0, rng)
    text, off, ln, col = pack_reads(reads)
    return Workload(f"longk-reads-{n_reads}x{read_len}bp", text, off, ln, col, k=63, m=12, bucket_bits=12,
                    min_multiplicity=2, hash_kind="rk128")


def to_fasta(w: Workload, line_width: int = 0) -> bytes:
    """FASTA bytes of a workload (one record per sequence)."""
    parts = []
    for i, (o, l) in enumerate(zip(w.seq_off.tolist(), w.seq_len.tolist())):
        s = w.text[o : o + l].tobytes()
        parts.append(b">seq%d\n" % i)
        if line_width and line_width > 0:
            parts.extend(s[j : j + line_width] + b"\n" for j in range(0, len(s), line_width))
        else:
            parts.append(s + b"\n")
    return b"".join(parts)


def query_stream(genomes: list, n_queries: int, rng: np.random.Generator, min_len: int = 100,
                 max_len: int = 100_000, member_frac: float = 0.8, sub_rate: float = 0.01,
                 rate_per_s: float = 1000.0):
    """Queries with log-uniform lengths in [min_len, max_len]: a fraction `member_frac` are
    substrings of random member genomes with `sub_rate` substitutions, the rest fresh i.i.d.
    sequence.  Returns (list of uint8 arrays, Poisson arrival times in seconds)."""
    lens = np.exp(rng.uniform(np.log(min_len), np.log(max_len), size=n_queries)).astype(np.int64)
    out = []
    for L in lens.tolist():
        if rng.random() < member_frac:
            g = genomes[int(rng.integers(0, len(genomes)))]
            L = min(L, len(g))
            s = int(rng.integers(0, len(g) - L + 1))
            q = substitute(g[s:s + L], sub_rate, rng)
            if rng.random() < 0.5:
                q = revcomp(q)
        else:
            q = random_genome(L, rng)
        out.append(q)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=n_queries))
    return out, arrivals


def query_workload(genomes: list, n_queries: int, seed: int = 0x67636174 + 5, min_len: int = 100,
                   max_len: int = 100_000, member_frac: float = 0.8, sub_rate: float = 0.01,
                   rate_per_s: float = 50_000.0):
    """Vectorised query set of the serving workload: lengths log-uniform in
    [min_len, max_len], `member_frac` substrings of random member genomes (either strand)
    with `sub_rate` substitutions, the rest fresh i.i.d. sequence; Poisson arrivals.
    Returns (text, offsets, lengths, arrivals) in the text layout."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.uniform(np.log(min_len), np.log(max_len), size=n_queries)).astype(np.int64)
    member = rng.random(n_queries) < member_frac
    off = np.zeros(n_queries, np.uint64)
    off[1:] = np.cumsum(lens[:-1] + 1).astype(np.uint64)
    text = np.full(int(lens.sum()) + n_queries, 10, np.uint8)
    which = rng.integers(0, len(genomes), size=n_queries)
    strand = rng.random(n_queries) < 0.5
    for i in range(n_queries):
        L = int(lens[i])
        o = int(off[i])
        if member[i]:
            g = genomes[int(which[i])]
            L = min(L, len(g))
            s = int(rng.integers(0, len(g) - L + 1))
            q = g[s:s + L]
            if strand[i]:
                q = revcomp(q)
            text[o:o + L] = q
        else:
            text[o:o + L] = BASES[rng.integers(0, 4, size=L)]
        lens[i] = L
        text[o + L] = 10
    # substitutions on member queries (vectorised over the whole text)
    m = rng.random(text.size) < sub_rate
    m &= text != 10
    code = np.searchsorted(BASES, text[m])
    text[m] = BASES[(code + rng.integers(1, 4, size=code.shape)) % 4]
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=n_queries))
    return text, off, lens.astype(np.uint64), arrivals
