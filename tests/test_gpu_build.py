"""GPU parity of the build hot path against the oracle: superkmer records, surviving
k-mers with multiplicities, and the canonical maximal-unitig set (bit-exact)."""
import os

import numpy as np
import pytest

import oracle
from ggcat_gb300 import _native, synth
from ggcat_gb300._native import GpuContext, make_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = GpuContext(0)
    yield c
    c.close()


def _workload(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "genomes":
        g = synth.random_genome(200_000, rng)
        g = synth.add_repeats(g, 0.03, 300, 3, 12, rng)
        gs = [g] + [synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng) for _ in range(2)]
        return synth.pack_sequences(gs)
    if kind == "reads":
        g = synth.random_genome(100_000, rng)
        g = synth.add_repeats(g, 0.02, 500, 20, 60, rng)
        reads = synth.sample_reads(g, 15_000, 150, 0.005, 0.0005, rng)
        return synth.pack_reads(reads)
    if kind == "lowcomplexity":
        seqs = [np.frombuffer(s, np.uint8) for s in (
            b"A" * 300, b"AC" * 200 + b"N" + b"ACGT" * 80, b"GATTACA" * 60, b"acgtnNACGTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTTT" * 5,
            b"CCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCCGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGGG")]
        seqs += [synth.random_genome(int(n), rng) for n in rng.integers(25, 120, size=200)]
        return synth.pack_sequences(seqs)
    if kind.startswith("planted"):
        # a random sequence with the m-mer of smallest canonical nt-hash planted every k - m
        # bases: every (k-1)-mer window holds exactly one copy, so all its k-mers (all
        # distinct) fall into one sub-bucket ("planted31:2500" sets the sequence length)
        # ("planted31:2500:only" leaves out the second, random sequence)
        name, _, rest = kind.partition(":")
        ln_s, _, only = rest.partition(":")
        k, m, mm, n = (31, 10, b"CAGAGCTTGC", 12000) if name == "planted31" else (63, 12, b"CAGACTATCGCG", 8000)
        n = int(ln_s) if ln_s else n
        g = synth.random_genome(n, rng).copy()
        pat = np.frombuffer(mm, np.uint8)
        for p in range(0, n - len(pat), k - m):
            g[p:p + len(pat)] = pat
        return synth.pack_sequences([g] if only else [g, synth.random_genome(3000, rng)])
    raise ValueError(kind)


def _oracle_params(p, threads=8):
    return oracle.params(k=p.k, m=p.m, bucket_bits=p.bucket_bits, second_bits=p.second_bits,
                         min_multiplicity=p.min_multiplicity, threads=threads)


def _sorted_sk(a):
    a = np.asarray(a)
    cols = ["start", "len", "bucket", "second_bucket", "minimizer_pos", "rc", "flags"]
    arr = np.stack([a[c].astype(np.uint64) for c in cols], axis=1)
    order = np.lexsort(arr.T[::-1])
    return arr[order]


CASES = [("genomes", 1, 10, 1), ("reads", 2, 10, 2), ("lowcomplexity", 3, 4, 1), ("reads", 4, 6, 1)]


@pytest.mark.parametrize("kind,seed,bbits,minm", CASES)
def test_bucketize_matches_oracle(ctx, kind, seed, bbits, minm):
    text, off, ln, _ = _workload(kind, seed)
    p = make_params(k=31, m=10, bucket_bits=bbits, second_bits=3, min_multiplicity=minm, keep_kmers=True)
    ctx.build_text(text, p)
    got = ctx.superkmers()
    exp = oracle.bucketize(text, off, ln, _oracle_params(p))
    assert len(got) == len(exp)
    assert (_sorted_sk(got) == _sorted_sk(exp)).all()


def _kmer_dict(keys, mult):
    d = {}
    keys = keys.tolist() if isinstance(keys, np.ndarray) else keys
    for kk, mm in zip(keys, mult.tolist()):
        if kk in d:
            assert d[kk] == mm, "k-mer multiplicity differs between sub-buckets"
        d[kk] = mm
    return d


@pytest.mark.parametrize("mode", [_native.GGCAT_MERGE_BATCHED, _native.GGCAT_MERGE_PER_BUCKET])
@pytest.mark.parametrize("kind,seed,bbits,minm", CASES)
def test_merge_matches_oracle(ctx, kind, seed, bbits, minm, mode):
    text, off, ln, _ = _workload(kind, seed)
    p = make_params(k=31, m=10, bucket_bits=bbits, second_bits=3, min_multiplicity=minm, keep_kmers=True,
                    merge_mode=mode)
    ctx.build_text(text, p)
    keys, mult = ctx.kmers()
    r = oracle.build_graph(text, off, ln, _oracle_params(p))
    lo, hi, emult = r.kmers()
    assert (hi == 0).all()
    assert _kmer_dict(keys, mult) == dict(zip(lo.tolist(), emult.tolist()))
    ctx.link(p.k)
    bases, uo, ul, uf = ctx.unitigs()
    lines = _native.unitig_lines(bases, uo, ul)
    got = oracle.canonicalize_unitigs(lines, (uf >> 2) & 1, p.k)
    assert got == r.unitigs()


def test_small_unit_target_changes_nothing(ctx):
    """Any packing of sub-bins into merge units gives the same unitigs."""
    text, off, ln, _ = _workload("reads", 7)
    outs = []
    for target in (64, 900, 0, -1):
        p = make_params(k=31, m=10, bucket_bits=8, second_bits=2, min_multiplicity=2, unit_target=target)
        ctx.build_text(text, p)
        ctx.link(31)
        bases, uo, ul, uf = ctx.unitigs()
        outs.append(oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31))
    assert outs[0] == outs[1] == outs[2] == outs[3]


@pytest.mark.parametrize("kind,bbits,minm,k,m", [("planted31", 1, 1, 31, 10), ("planted63", 1, 1, 63, 12),
                                                 ("reads", 2, 2, 31, 10), ("genomes", 1, 1, 31, 10)])
def test_shared_memory_attempt_and_spill(ctx, kind, bbits, minm, k, m):
    """Sub-buckets of several thousand k-mer instances try the shared-memory table first and
    move to the global-memory tier when their distinct k-mers do not fit (planted: one
    sub-bucket of all-distinct k-mers).  Same result as the oracle either way."""
    text, off, ln, _ = _workload(kind, 21)
    p = make_params(k=k, m=m, bucket_bits=bbits, second_bits=1, min_multiplicity=minm, keep_kmers=True)
    ctx.build_text(text, p)
    st = ctx.stats()
    if kind.startswith("planted"):
        assert st["merge_units_spilled"] > 0
    assert st["distinct_kmers"] >= st["surviving_kmers"] > 0
    keys, mult = ctx.kmers()
    if k > 32:
        keys = [int(a) | (int(b) << 64) for a, b in keys.tolist()]
    got = _kmer_dict(keys, mult)
    op = oracle.params(k=k, m=m, bucket_bits=bbits, second_bits=1, min_multiplicity=minm, threads=8)
    r = oracle.build_graph(text, off, ln, op)
    lo, hi, emult = r.kmers()
    assert got == {int(a) | (int(b) << 64): int(c) for a, b, c in zip(lo.tolist(), hi.tolist(), emult.tolist())}
    ctx.link(k)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k) == r.unitigs()


@pytest.mark.parametrize("kind,k,m", [("planted31:2500:only", 31, 10), ("planted31:5000:only", 31, 10),
                                      ("planted31:8000:only", 31, 10), ("planted31:9000:only", 31, 10),
                                      ("planted63:1300:only", 63, 12),
                                      ("planted63:2500:only", 63, 12), ("planted63:5000:only", 63, 12),
                                      ("planted31:8000", 31, 10), ("planted63:5000", 63, 12)])
def test_many_survivors_rank_in_global_scratch(ctx, kind, k, m):
    """A unit with more surviving k-mers than its tier's shared-memory ranking arrays hold
    (S, W and M tiers by the planted length) is ranked in the CTA's global scratch: same
    k-mers and unitigs as the oracle, and no unit falls back to per-thread walks."""
    text, off, ln, _ = _workload(kind, 23)
    p = make_params(k=k, m=m, bucket_bits=1, second_bits=1, min_multiplicity=1, keep_kmers=True)
    ctx.build_text(text, p)
    st = ctx.stats()
    assert st["merge_units_ext_global"] > 0
    assert st["merge_units_walk"] == 0
    keys, mult = ctx.kmers()
    if k > 32:
        keys = [int(a) | (int(b) << 64) for a, b in keys.tolist()]
    got = _kmer_dict(keys, mult)
    op = oracle.params(k=k, m=m, bucket_bits=1, second_bits=1, min_multiplicity=1, threads=8)
    r = oracle.build_graph(text, off, ln, op)
    lo, hi, emult = r.kmers()
    assert got == {int(a) | (int(b) << 64): int(c) for a, b, c in zip(lo.tolist(), hi.tolist(), emult.tolist())}
    ctx.link(k)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k) == r.unitigs()


def test_genome_family_min_multiplicity_one(ctx):
    """Many related genomes (one ancestor, per-genome substitutions and indels) with
    min multiplicity 1, the shape of a coloured build: big minimizer groups whose k-mers
    nearly all survive.  Bit-exact against the oracle, no walk fallback."""
    rng = np.random.default_rng(31)
    anc = synth.random_genome(60_000, rng)
    gs = [synth.indels(synth.substitute(anc, float(rng.uniform(0.001, 0.02)), rng), 0.0005, 50, rng)
          for _ in range(48)]
    text, off, ln, _ = synth.pack_sequences(gs)
    p = make_params(k=31, m=10, bucket_bits=6, second_bits=1, min_multiplicity=1, keep_kmers=True)
    ctx.build_text(text, p)
    st = ctx.stats()
    assert st["merge_units_walk"] == 0
    keys, mult = ctx.kmers()
    r = oracle.build_graph(text, off, ln, _oracle_params(p))
    lo, hi, emult = r.kmers()
    assert _kmer_dict(keys, mult) == dict(zip(lo.tolist(), emult.tolist()))
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31) == r.unitigs()


def test_merge_phase_replays_as_cuda_graph():
    """The batched merge phase is captured as a CUDA graph once per buffer layout and then
    replayed: a second build of the same input replays without a new capture and gives the
    same unitigs (both equal to the oracle's)."""
    c = GpuContext(0)
    try:
        text, off, ln, _ = _workload("reads", 11)
        p = make_params(k=31, m=10, bucket_bits=8, second_bits=2, min_multiplicity=2)
        outs, st = [], []
        for _ in range(2):
            c.build_text(text, p)
            st.append(c.stats())
            c.link(31)
            bases, uo, ul, uf = c.unitigs()
            outs.append(oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31))
        assert st[0]["merge_graph_captures"] >= 1
        assert st[1]["merge_graph_captures"] == st[0]["merge_graph_captures"]
        assert st[1]["merge_graph_replays"] == st[0]["merge_graph_replays"] + 1
        r = oracle.build_graph(text, off, ln, _oracle_params(p))
        assert outs[0] == outs[1] == r.unitigs()
    finally:
        c.close()


@pytest.mark.parametrize("knobs", [dict(subbin_bytes=256), dict(subbin_bytes=4096), dict(table_load_pct=50),
                                   dict(table_load_pct=90), dict(small_limit=800),
                                   dict(unit_target=-1, small_limit=1600, table_load_pct=65),
                                   dict(small_batch=1, wide_batch=32), dict(small_batch=7, wide_batch=3),
                                   dict(wide_limit=4096, wide_batch=8), dict(wide_limit=100, small_batch=32)])
def test_tuning_knobs_change_nothing(ctx, knobs):
    """Sub-bin digit width, S-unit size limit, packing target, global-table load and the
    per-class knobs (S / W insert batches, W sub-bin limit) change only the speed: k-mers and
    unitigs stay equal to the oracle's."""
    text, off, ln, _ = _workload("reads", 13)
    p = make_params(k=31, m=10, bucket_bits=6, second_bits=2, min_multiplicity=2, keep_kmers=True, **knobs)
    ctx.build_text(text, p)
    keys, mult = ctx.kmers()
    r = oracle.build_graph(text, off, ln, _oracle_params(p))
    lo, hi, emult = r.kmers()
    assert _kmer_dict(keys, mult) == dict(zip(lo.tolist(), emult.tolist()))
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31) == r.unitigs()


def test_autotune_params_build_the_same_graph(ctx):
    """The autotuner measures candidates on the device (the digit width by the whole step, each
    bucket-size class's knobs by the device time of the classes they move work between) and
    returns knobs from its candidate sets; a build with them equals the oracle."""
    torch = pytest.importorskip("torch")
    text, off, ln, _ = _workload("reads", 17)
    p = make_params(k=31, m=10, bucket_bits=8, second_bits=2, min_multiplicity=2)
    d = torch.from_numpy(text).cuda()
    best, default_ms, best_ms = ctx.autotune(d.data_ptr(), d.numel(), p)
    assert 0 < best_ms
    assert best.subbin_bytes in (0, 256, 512, 1024, 2048, 4096)
    assert best.unit_target in (0, -1, 1024, 2048)
    assert best.small_limit in (0, 2400, 1600)
    assert best.small_batch in (0, 8, 16, 32)
    assert best.wide_batch in (0, 8, 12, 16, 24, 32)
    assert best.wide_limit in (0, 32768, 16384)
    assert best.table_load_pct in (0, 50, 65, 90)
    # per-class device times of the tuned build, one per bucket-size class
    ctx.build_text(text, best)
    assert len(ctx.stats()["ms_tier"]) == 4 and ctx.stats()["ms_tier"][0] >= 0
    assert (best.k, best.m, best.min_multiplicity) == (p.k, p.m, p.min_multiplicity)
    ctx.build_text(text, best)
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    r = oracle.build_graph(text, off, ln, _oracle_params(p))
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31) == r.unitigs()


@pytest.mark.parametrize("k,m,n,extra", [(31, 10, 20_000, False), (31, 10, 3_000, True), (63, 12, 12_000, False)])
def test_link_joins_cycles_across_buckets(ctx, k, m, n, extra):
    """A circular genome (its first k-1 bases appended) makes one k-mer cycle that crosses
    many buckets: the device link stage cuts it once, drops its mirror copy and emits one
    circular unitig; with a second, linear genome the chains and the cycle coexist."""
    rng = np.random.default_rng(n + k)
    g = synth.random_genome(n, rng)
    seqs = [np.concatenate([g, g[:k - 1]])]
    if extra:
        seqs.append(synth.random_genome(5_000, rng))
    text, off, ln, _ = synth.pack_sequences(seqs)
    p = make_params(k=k, m=m, bucket_bits=4, second_bits=1, min_multiplicity=1)
    ctx.build_text(text, p)
    ctx.link(k)
    bases, uo, ul, uf = ctx.unitigs()
    got = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k)
    op = oracle.params(k=k, m=m, bucket_bits=4, second_bits=1, min_multiplicity=1, threads=8)
    assert got == oracle.build_graph(text, off, ln, op).unitigs()
    assert int(((uf >> 2) & 1).sum()) >= 1


@pytest.mark.parametrize("case", ["empty", "short", "all_n", "one_kmer", "separators"])
def test_edge_case_inputs_match_oracle(ctx, case):
    """Inputs without k-mers or with a single one: empty text, sequences shorter than k, only
    N, exactly k bases, and a text of separators with k-mers split by them."""
    rng = np.random.default_rng(5)
    g = synth.random_genome(31, rng)
    seqs = {"empty": [],
            "short": [synth.random_genome(int(n), rng) for n in (1, 5, 29, 30)],
            "all_n": [np.frombuffer(b"N" * 200, np.uint8), np.frombuffer(b"n" * 40, np.uint8)],
            "one_kmer": [g],
            "separators": [synth.random_genome(35, rng), np.frombuffer(b"ACGT" * 20, np.uint8)]}[case]
    text, off, ln, _ = synth.pack_sequences(seqs) if seqs else (np.zeros(0, np.uint8), np.zeros(0, np.uint64),
                                                                 np.zeros(0, np.uint64), None)
    p = make_params(k=31, m=10, bucket_bits=4, second_bits=1, min_multiplicity=1, keep_kmers=True)
    ctx.build_text(text, p)
    keys, mult = ctx.kmers()
    r = oracle.build_graph(text, off, ln, _oracle_params(p))
    lo, hi, emult = r.kmers()
    assert _kmer_dict(keys, mult) == dict(zip(lo.tolist(), emult.tolist()))
    ctx.link(31)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, 31) == r.unitigs()


@pytest.mark.parametrize("mode", [_native.GGCAT_MERGE_BATCHED, _native.GGCAT_MERGE_PER_BUCKET])
@pytest.mark.parametrize("kind,k,m,okind", [("genomes", 31, 10, oracle.H_FW_SEQ64), ("reads", 31, 10, oracle.H_FW_SEQ64),
                                            ("reads", 63, 12, oracle.H_FW_SEQ128)])
def test_forward_only_matches_oracle(ctx, kind, k, m, okind, mode):
    """Forward-only builds (forward seq-hash): records stay in text orientation, k-mers are
    keyed and extended as read (successors forward, predecessors backward) and only forward
    paths are emitted; k-mers and unitigs equal the oracle's forward-hash build."""
    text, off, ln, _ = _workload(kind, 41)
    p = make_params(k=k, m=m, bucket_bits=6, second_bits=2, min_multiplicity=1, keep_kmers=True, forward_only=True,
                    merge_mode=mode)
    ctx.build_text(text, p)
    keys, mult = ctx.kmers()
    if k > 32:
        keys = [int(a) | (int(b) << 64) for a, b in keys.tolist()]
    op = oracle.params(k=k, m=m, bucket_bits=6, second_bits=2, canonical=False, hash_kind=okind, min_multiplicity=1,
                       threads=8)
    r = oracle.build_graph(text, off, ln, op)
    lo, hi, emult = r.kmers()
    assert _kmer_dict(keys, mult) == {int(a) | (int(b) << 64): int(c)
                                      for a, b, c in zip(lo.tolist(), hi.tolist(), emult.tolist())}
    ctx.link(k)
    bases, uo, ul, uf = ctx.unitigs()
    assert oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k) == r.unitigs()


def test_build_graph_from_fasta_files_matches_oracle(tmp_path):
    """GGCATInstance.build_graph on FASTA files (FASTA reader, device build, device link,
    FASTA writer): the unitigs of the written file equal the oracle's for the same reads."""
    import ggcat_gb300

    rng = np.random.default_rng(9)
    g = synth.random_genome(60_000, rng)
    files = []
    for i in range(2):
        reads = synth.sample_reads(g, 3000, 150, 0.003, 0.0, rng)
        path = tmp_path / f"r{i}.fa"
        with open(path, "wb") as f:
            for j, rd in enumerate(reads):
                f.write(b">r%d_%d\n" % (i, j) + rd.tobytes() + b"\n")
        files.append(str(path))
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = tmp_path / "out.fa"
    assert inst.build_graph(files, str(out), kmer_length=31, minimizer_length=10, min_multiplicity=2) == str(out)
    lines = open(out, "rb").read().split(b"\n")
    assert all(h.startswith(b">") and b" LN:i:" in h for h in lines[0:-1:2])
    seqs = [x for x in lines[1::2] if x]
    got = oracle.canonicalize_unitigs(b"".join(x + b"\n" for x in seqs), np.zeros(len(seqs), np.uint8), 31)
    # the unitig set does not depend on the bucket counts the file path picks
    ftext, foff, fln = oracle.fasta_parse(b"".join(open(f, "rb").read() for f in files), 30)
    r = oracle.build_graph(ftext, foff, fln, oracle.params(k=31, m=10, bucket_bits=10, second_bits=3,
                                                          min_multiplicity=2, threads=8))
    assert got == r.unitigs()


def test_device_pointer_bucketize(ctx):
    """bucketize on a caller-owned device buffer and stream (torch only as plumbing)."""
    torch = pytest.importorskip("torch")
    text, off, ln, _ = _workload("genomes", 9)
    d = torch.from_numpy(text).cuda()
    s = torch.cuda.current_stream()
    p = make_params(k=31, m=10, bucket_bits=10, second_bits=3)
    n = ctx.bucketize(d.data_ptr(), d.numel(), p, s.cuda_stream)
    got = ctx.superkmers()
    exp = oracle.bucketize(text, off, ln, _oracle_params(p))
    assert n == len(exp)
    assert (_sorted_sk(got) == _sorted_sk(exp)).all()


# k > 32: 128-bit table keys (seq-hash u128, and Rabin-Karp u128 which selects the same
# k-mer identities); the oracle follows the reference hash of each case.
WIDE = [("reads", 11, 63, 12, oracle.H_CN_SEQ128, _native.GGCAT_HASH_SEQHASH, 2),
        ("genomes", 12, 63, 12, oracle.H_CN_RK128, _native.GGCAT_HASH_RABIN_KARP128, 1),
        ("genomes", 13, 33, 11, oracle.H_CN_SEQ128, _native.GGCAT_HASH_SEQHASH, 1),
        ("lowcomplexity", 14, 45, 9, oracle.H_CN_SEQ128, _native.GGCAT_HASH_SEQHASH, 1)]


@pytest.mark.parametrize("mode", [_native.GGCAT_MERGE_BATCHED, _native.GGCAT_MERGE_PER_BUCKET])
@pytest.mark.parametrize("kind,seed,k,m,okind,hkind,minm", WIDE)
def test_wide_k_matches_oracle(ctx, kind, seed, k, m, okind, hkind, minm, mode):
    text, off, ln, _ = _workload(kind, seed)
    p = make_params(k=k, m=m, bucket_bits=8, second_bits=2, min_multiplicity=minm, hash_kind=hkind,
                    keep_kmers=True, merge_mode=mode)
    ctx.build_text(text, p)
    op = oracle.params(k=k, m=m, bucket_bits=8, second_bits=2, min_multiplicity=minm, hash_kind=okind, threads=8)
    assert (_sorted_sk(ctx.superkmers()) == _sorted_sk(oracle.bucketize(text, off, ln, op))).all()
    keys, mult = ctx.kmers()
    assert keys.ndim == 2
    got = _kmer_dict([int(a) | (int(b) << 64) for a, b in keys.tolist()], mult)
    r = oracle.build_graph(text, off, ln, op)
    lo, hi, emult = r.kmers()
    assert got == {int(a) | (int(b) << 64): int(c) for a, b, c in zip(lo.tolist(), hi.tolist(), emult.tolist())}
    ctx.link(k)
    bases, uo, ul, uf = ctx.unitigs()
    got_u = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k)
    assert got_u == r.unitigs()


_RC = bytes.maketrans(b"ACGT", b"TGCA")


def _unitig_multiset(ctx):
    """Partial unitigs up to orientation: which end a path is written from depends on the
    table slots its k-mers landed in, so each is taken as min(s, revcomp(s)) with its link
    flags (bit 0 backward, bit 1 forward) swapped when reversed.  Circular ones (bit 2) start
    anywhere and are left to the final-unitig comparison."""
    bases, off, ln, fl = ctx.partial_unitigs()
    out = []
    for o, n, f in zip(off.tolist(), ln.tolist(), fl.tolist()):
        if f & 4:
            continue
        s = bases[o:o + n].tobytes()
        r = s.translate(_RC)[::-1]
        if r < s:
            s, f = r, (f & ~3) | ((f & 1) << 1) | ((f >> 1) & 1)
        out.append((s, f))
    return sorted(out)


@pytest.mark.parametrize("pieces", [4, 16])
@pytest.mark.parametrize("k,m,read_len", [(31, 10, 150), (63, 12, 250)])
def test_pinned_text_pipelined_equals_pageable(ctx, k, m, read_len, pieces):
    """build_text from pinned host memory copies the text in pieces on its own stream and
    packs / bucketizes each piece on a stream of its own while the next ones are in flight (16
    pieces: one or two bucketize blocks each, their kernels overlapping); the records, k-mers
    and partial unitigs equal those of the one-copy (pageable) path."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(k)
    g = synth.random_genome(300_000, rng)
    reads = synth.sample_reads(g, 6_000_000 // read_len, read_len, 0.005, 0.0002, rng)
    text, _, _, _ = synth.pack_reads(reads)
    assert len(text) > 8 * 262144  # several bucketize blocks per piece
    p = make_params(k=k, m=m, bucket_bits=8, second_bits=3, min_multiplicity=2, keep_kmers=True,
                    copy_pieces=pieces)

    def run(t):
        ctx.build_text(t, p)
        sk, (keys, mult), parts = _sorted_sk(ctx.superkmers()), ctx.kmers(), _unitig_multiset(ctx)
        ctx.link(k)
        bases, uo, ul, uf = ctx.unitigs()
        final = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k)
        kk = sorted(zip(map(tuple, keys.reshape(len(mult), -1).tolist()), mult.tolist()))
        return sk, kk, parts, final

    sk_a, k_a, u_a, f_a = run(text)
    sk_b, k_b, u_b, f_b = run(torch.from_numpy(text).pin_memory().numpy())
    assert len(sk_a) > 0 and (sk_a == sk_b).all()
    assert k_a == k_b
    assert u_a == u_b
    assert f_a == f_b and len(f_a) > 0


def test_build_from_streams_matches_files(tmp_path):
    """ggcat_gpu_build_from_streams (crates/capi/src/lib.rs:226-292): two streams emitting the
    reads of two FASTA files, in pieces of varying size, build the same graph file as
    ggcat_gpu_build_from_files on those files, and its unitigs equal the oracle's."""
    import ctypes as C

    rng = np.random.default_rng(21)
    g = synth.random_genome(50_000, rng)
    files, sources = [], []
    for i in range(2):
        reads = synth.sample_reads(g, 2500, 150, 0.003, 0.0, rng)
        path = tmp_path / f"s{i}.fa"
        with open(path, "wb") as f:
            for j, rd in enumerate(reads):
                f.write(b">s%d_%d\n" % (i, j) + rd.tobytes() + b"\n")
        files.append(str(path))
        sources.append([rd.tobytes() for rd in reads])
    L = _native.load()
    out_s, out_f = tmp_path / "streams.fa", tmp_path / "files.fa"
    arr, keep = _native.make_streams(sources)
    c = _native.GpuContext(0)
    try:
        assert L.ggcat_gpu_build_from_streams(c.h, arr, 2, os.fsencode(str(out_s)), 31, 4, 0, 10, 2) == 0
        names = (C.c_char_p * 2)(*[os.fsencode(f) for f in files])
        assert L.ggcat_gpu_build_from_files(c.h, names, 2, os.fsencode(str(out_f)), 31, 4, 0, 10, 2) == 0
    finally:
        c.close()
    del keep

    def unitig_set(path):
        lines = open(path, "rb").read().split(b"\n")
        seqs = [x for x in lines[1::2] if x]
        return oracle.canonicalize_unitigs(b"".join(x + b"\n" for x in seqs), np.zeros(len(seqs), np.uint8), 31)

    got = unitig_set(out_s)
    assert got == unitig_set(out_f)
    ftext, foff, fln = oracle.fasta_parse(b"".join(open(f, "rb").read() for f in files), 30)
    r = oracle.build_graph(ftext, foff, fln, oracle.params(k=31, m=10, bucket_bits=10, second_bits=3,
                                                          min_multiplicity=2, threads=8))
    assert got == r.unitigs()
