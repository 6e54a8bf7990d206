"""GGCATInstance.build_graph with unitig links and GFA output: the unitigs built on the GPU,
then the host links / GFA writer; the links equal the restatement's over the written
unitigs, the unitig set equals the oracle's."""
import numpy as np
import pytest

import naive
import oracle
from ggcat_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    rng = np.random.default_rng(71)
    g = synth.random_genome(120_000, rng)  # no repeats: no circular unitigs
    gs = [g, synth.indels(synth.substitute(g, 0.01, rng), 0.001, 10, rng)]
    d = tmp_path_factory.mktemp("graph_out")
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


def test_unitig_links_fasta(inputs):
    import ggcat_gb300

    d, files = inputs
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = str(d / "links.fa")
    assert inst.build_graph(files, out, kmer_length=31, min_multiplicity=1,
                            extra_elab=ggcat_gb300.ExtraElaboration.UNITIG_LINKS) == out
    heads, seqs = _records(open(out, "rb").read())
    exp = naive.unitig_links(seqs, 31)
    n_links = 0
    for i, (h, (end, beg)) in enumerate(zip(heads, exp)):
        parts = h.split(b" ")
        assert parts[0] == b"%d" % i and parts[1] == b"LN:i:%d" % len(seqs[i])
        got = sorted(parts[2:])
        want = sorted(b"L:%s:%d:%s" % (b"-" if fc else b"+", j, b"-" if fo else b"+") for j, _, fc, fo in end + beg)
        assert got == want
        n_links += len(want)
    assert n_links > 0
    # the unitigs themselves are the oracle's (read from the same files)
    ftext, foff, fln = oracle.fasta_parse(b"".join(open(f, "rb").read() for f in files), 30)
    r = oracle.build_graph(ftext, foff, fln, oracle.params(k=31, m=10, bucket_bits=6, second_bits=2, threads=4,
                                                          min_multiplicity=1))
    got = oracle.canonicalize_unitigs(b"".join(s + b"\n" for s in seqs), np.zeros(len(seqs), np.uint8), 31)
    assert got == r.unitigs()


@pytest.mark.parametrize("version", [1, 2])
def test_gfa(inputs, version):
    import ggcat_gb300

    d, files = inputs
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = str(d / f"graph{version}.gfa")
    assert inst.build_graph(files, out, kmer_length=31, min_multiplicity=1, gfa_output_version=version,
                            extra_elab=ggcat_gb300.ExtraElaboration.UNITIG_LINKS) == out
    lines = open(out, "rb").read().split(b"\n")[:-1]
    s_lines = [x.split(b"\t") for x in lines if x.startswith(b"S\t")]
    seqs = [f[2] if version == 1 else f[3] for f in s_lines]
    assert [int(f[1]) for f in s_lines] == list(range(len(seqs)))
    exp = naive.unitig_links(seqs, 31)
    tag = b"L\t" if version == 1 else b"E\t"
    assert sum(x.startswith(tag) for x in lines) == sum(len(a) + len(b) for a, b in exp) > 0
