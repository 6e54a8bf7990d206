"""GGCATInstance.build_graph with extra_elab greedy matchtigs / eulertigs / pathtigs: the
unitigs are built on the GPU, the strings on the host (ggcat_gpu_compute_tigs).  Each output
keeps the k-mer spectrum of the unitig output of the same input (every k-mer once for
eulertigs and pathtigs), the eulertig count is the minimum for those unitigs, and the GFA form
holds the same strings as segments."""
import numpy as np
import pytest

import naive
from ggcat_gb300 import synth

pytestmark = pytest.mark.gpu

K = 31


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    rng = np.random.default_rng(83)
    g = synth.random_genome(150_000, rng)
    gs = [g] + [synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng) for _ in range(2)]
    d = tmp_path_factory.mktemp("tigs")
    files = []
    for i, s in enumerate(gs):
        p = d / f"g{i}.fa"
        p.write_bytes(b">g%d\n%s\n" % (i, s.tobytes()))
        files.append(str(p))
    return d, files


def _records(data: bytes):
    heads, seqs = [], []
    for block in data.split(b">")[1:]:
        h, _, rest = block.partition(b"\n")
        heads.append(h)
        seqs.append(rest.replace(b"\n", b""))
    return heads, seqs


def _kmers(seqs):
    out = []
    for s in seqs:
        out += [naive.canon(s[i:i + K]) for i in range(len(s) - K + 1)]
    return out


def test_tigs_through_build_graph(inputs):
    import ggcat_gb300
    from ggcat_gb300 import ExtraElaboration as E

    d, files = inputs
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out_u = str(d / "unitigs.fa")
    assert inst.build_graph(files, out_u, kmer_length=K, min_multiplicity=1) == out_u
    _, useqs = _records(open(out_u, "rb").read())
    kmers = _kmers(useqs)
    assert len(kmers) == len(set(kmers)) > 0
    kset = set(kmers)
    lb = naive.tig_lower_bound(useqs, K)
    got = {}
    for mode in (E.EULERTIGS, E.PATHTIGS, E.GREEDY_MATCHTIGS, E.FAST_SIMPLITIGS, E.FAST_EULERTIGS):
        out = str(d / f"tigs{mode}.fa")
        assert inst.build_graph(files, out, kmer_length=K, min_multiplicity=1, extra_elab=mode) == out
        heads, seqs = _records(open(out, "rb").read())
        for i, (h, s) in enumerate(zip(heads, seqs)):
            assert h == b"%d LN:i:%d" % (i, len(s)) and len(s) >= K
        tk = _kmers(seqs)
        assert set(tk) == kset
        if mode != E.GREEDY_MATCHTIGS:
            assert len(tk) == len(kset)
        got[mode] = seqs
    # the eulertigs of this run's unitigs are minimal; a rebuild may number the unitigs
    # differently but not change the graph
    assert len(got[E.EULERTIGS]) == len(got[E.FAST_EULERTIGS]) == lb
    assert len(got[E.FAST_SIMPLITIGS]) >= lb
    assert len(got[E.PATHTIGS]) >= lb
    assert len(got[E.GREEDY_MATCHTIGS]) <= lb
    assert sum(map(len, got[E.GREEDY_MATCHTIGS])) <= sum(map(len, got[E.EULERTIGS]))
    # GFA v1: the same strings as segments, no links
    out_g = str(d / "eul.gfa")
    assert inst.build_graph(files, out_g, kmer_length=K, min_multiplicity=1, extra_elab=E.EULERTIGS,
                            gfa_output_version=ggcat_gb300.GfaVersion.V1) == out_g
    lines = [l for l in open(out_g, "rb").read().split(b"\n") if l]
    segs = [l.split(b"\t")[2] for l in lines if l.startswith(b"S\t")]
    assert not any(l.startswith(b"L\t") for l in lines)
    assert set(_kmers(segs)) == kset and len(segs) == lb


def test_greedy_matchtigs_of_a_coloured_graph_are_refused(inputs):
    """A join repeats k-mers whose colours the strings would have to carry twice; the
    reference's writer stops there too (compute_matchtigs.rs:496-503)."""
    import ggcat_gb300

    d, files = inputs
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    with pytest.raises(ggcat_gb300.GgcatGpuError):
        inst.build_graph(files, str(d / "c.fa"), kmer_length=K, min_multiplicity=1, colors=True,
                         extra_elab=ggcat_gb300.ExtraElaboration.GREEDY_MATCHTIGS)
