"""Even k on the device against the oracle: k-mers equal to their reverse complement exist
only for even k, and the hash-map walk treats them as path ends (a walk that enters one stops,
its successor being the mirror of where it came from).  Inputs rich in them: hairpin sequences
(s + revcomp(s)), repeats of short palindromes, and ordinary reads; k = 20, 32 (u64 keys), 48
and 64 (u128 keys); batched and per-bucket merges; the canonical unitig set and the surviving
k-mers with multiplicities must equal the oracle's."""
import numpy as np
import pytest

import oracle
from oracle import parity
from ggcat_gb300 import _native, synth

pytestmark = pytest.mark.gpu


def _palindromic_input(k, seed):
    rng = np.random.default_rng(seed)
    seqs = []
    for _ in range(300):  # hairpins: s + revcomp(s), |s| from k/2 to 3k
        s = synth.random_genome(int(rng.integers(k // 2, 3 * k)), rng)
        seqs.append(np.concatenate([s, synth.revcomp(s)]))
    g = synth.random_genome(40_000, rng).copy()
    for _ in range(200):  # short palindromes pasted into a genome, several copies each
        half = synth.random_genome(k // 2, rng)
        pal = np.concatenate([half, synth.revcomp(half)])
        for p in rng.integers(0, len(g) - k, size=int(rng.integers(1, 4))).tolist():
            g[p:p + k] = pal
    seqs.append(g)
    seqs += list(synth.sample_reads(g, 3000, 150, 0.003, 0.0, rng))
    return synth.pack_sequences(seqs)


@pytest.mark.parametrize("mode", [_native.GGCAT_MERGE_BATCHED, _native.GGCAT_MERGE_PER_BUCKET])
@pytest.mark.parametrize("k,m,minm", [(20, 8, 1), (32, 10, 1), (32, 10, 2), (48, 12, 1), (64, 14, 1)])
def test_even_k_matches_oracle(k, m, minm, mode):
    text, off, ln, _ = _palindromic_input(k, 100 + k)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=k, m=m, bucket_bits=5, second_bits=2, min_multiplicity=minm, keep_kmers=True,
                                merge_mode=mode)
        ctx.build_text(text, p)
        keys, mult = ctx.kmers()
        ctx.link(k)
        bases, uo, ul, uf = ctx.unitigs()
        lines = oracle.canonicalize_unitigs(_native.unitig_lines(bases, uo, ul), (uf >> 2) & 1, k)
        r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=m, bucket_bits=5, second_bits=2,
                                                             min_multiplicity=minm, threads=8))
        km = parity.compare_kmers(keys, mult, r)
        assert km["equal"] and km["kmers_oracle"] > 0, km
        un = parity.compare_unitigs(lines, r)
        assert un["equal"], un
    finally:
        ctx.close()


def test_forward_only_k32_rejected():
    text, _, _, _ = _palindromic_input(32, 1)
    ctx = _native.GpuContext(0)
    try:
        p = _native.make_params(k=32, m=10, bucket_bits=5, second_bits=2, forward_only=True)
        with pytest.raises(_native.GgcatGpuError, match="EUNSUPPORTED"):
            ctx.build_text(text, p)
    finally:
        ctx.close()
