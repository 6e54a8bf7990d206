"""k > 64 on the device against the oracle.  The reference keys such k-mers by the canonical
Rabin-Karp u128 hash (crates/api/src/utils.rs:10-69); the device keys its global-memory merge
tables by the canonical packed k-mer in four words (u256), which selects the same k-mer
identities short of a 128-bit hash collision.  Surviving k-mers with multiplicities and the
final unitigs must equal the oracle's, batched and per-bucket; the file path picks the
Rabin-Karp hash and m = round(k / 4) by itself."""
import numpy as np
import pytest

import oracle
from oracle import parity
from ggcat_gb300 import _native, synth

pytestmark = pytest.mark.gpu


def _long_k_input(k, seed):
    rng = np.random.default_rng(seed)
    g = synth.random_genome(30_000, rng)
    g = synth.add_repeats(g, 0.05, 3 * k, 2, 5, rng)
    seqs = [g, synth.indels(synth.substitute(g, 0.01, rng), 0.002, 5, rng)]
    seqs += list(synth.sample_reads(g, 1500, 300, 0.004, 0.0, rng))
    if k % 2 == 0:  # hairpins: the centre k-mer is its own reverse complement
        for _ in range(40):
            s = synth.random_genome(int(rng.integers(k // 2, 2 * k)), rng)
            seqs.append(np.concatenate([s, synth.revcomp(s)]))
    return synth.pack_sequences(seqs)


@pytest.mark.parametrize("mode", [_native.GGCAT_MERGE_BATCHED, _native.GGCAT_MERGE_PER_BUCKET])
@pytest.mark.parametrize("k,m,minm", [(65, 16, 1), (75, 19, 2), (96, 24, 1), (101, 25, 1), (127, 32, 2)])
def test_long_k_matches_oracle(k, m, minm, mode):
    text, off, ln, _ = _long_k_input(k, k)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=k, m=m, bucket_bits=6, second_bits=2, min_multiplicity=minm, keep_kmers=True,
                                merge_mode=mode, hash_kind=_native.GGCAT_HASH_RABIN_KARP128)
        ctx.build_text(text, p)
        keys, mult = ctx.kmers()
        assert keys.shape[1] == 4
        ctx.link(k)
        bases, uo, ul, uf = ctx.unitigs()
        lines = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k)
        r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=m, bucket_bits=6, second_bits=2,
                                                             min_multiplicity=minm, threads=8,
                                                             hash_kind=oracle.H_CN_RK128))
        km = parity.compare_kmers_wide(keys, mult, r)
        assert km["equal"] and km["kmers_oracle"] > 0, km
        un = parity.compare_unitigs(lines, r)
        assert un["equal"], un
    finally:
        ctx.close()


def test_long_k_rejects_sequence_hash_and_k_above_127():
    text, _, _, _ = _long_k_input(65, 1)
    ctx = _native.GpuContext(0)
    try:
        with pytest.raises(_native.GgcatGpuError, match="EINVAL"):
            ctx.build_text(text, _native.make_params(k=65, m=16, hash_kind=_native.GGCAT_HASH_SEQHASH))
        with pytest.raises(_native.GgcatGpuError, match="EUNSUPPORTED"):
            ctx.build_text(text, _native.make_params(k=128, m=32, hash_kind=_native.GGCAT_HASH_RABIN_KARP128))
    finally:
        ctx.close()


def test_long_k_graph_from_files(tmp_path):
    """GGCATInstance.build_graph at k = 101: the Rabin-Karp hash and m = 25 chosen like the
    reference's HashType::Auto and compute_best_m; the written unitigs equal the oracle's."""
    import ggcat_gb300

    rng = np.random.default_rng(5)
    g = synth.random_genome(40_000, rng)
    path = tmp_path / "r.fa"
    with open(path, "wb") as f:
        for j, rd in enumerate(synth.sample_reads(g, 2500, 250, 0.003, 0.0, rng)):
            f.write(b">r%d\n" % j + rd.tobytes() + b"\n")
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = tmp_path / "out.fa"
    inst.build_graph([str(path)], str(out), kmer_length=101, min_multiplicity=2)
    lines = open(out, "rb").read().split(b"\n")
    seqs = [x for x in lines[1::2] if x]
    got = oracle.canonicalize_unitigs(b"".join(x + b"\n" for x in seqs), np.zeros(len(seqs), np.uint8), 101)
    ftext, foff, fln = oracle.fasta_parse(open(path, "rb").read(), 100)
    r = oracle.build_graph(ftext, foff, fln, oracle.params(k=101, m=25, bucket_bits=8, second_bits=2,
                                                          min_multiplicity=2, threads=8, hash_kind=oracle.H_CN_RK128))
    assert got == r.unitigs()
