"""The coloured drop-in path end to end through GGCATInstance (the C ABI's
ggcat_gpu_build_from_files_ex / ggcat_gpu_query_graph / ggcat_gpu_dump_unitigs and the colormap
entries): a coloured build from one FASTA file per colour (one of them gzip-compressed) writes
the unitigs with C: runs and the colormap beside them; decoding both gives every k-mer's colour
set, compared with the oracle's; the coloured query writes the JSON lines of per-colour match
fractions, compared with the oracle's counts; the coloured dump gives every k-mer once with its
colours."""
import gzip
import json

import numpy as np
import pytest

import oracle
from ggcat_gb300 import serve, synth

pytestmark = pytest.mark.gpu

K = 31


def _files(tmp_path, n=6, L=60_000, seed=12):
    rng = np.random.default_rng(seed)
    anc = synth.random_genome(L, rng)
    genomes, paths = [], []
    for i in range(n):
        g = synth.indels(synth.substitute(anc, float(rng.uniform(0.002, 0.02)), rng), 0.001, 20, rng)
        genomes.append(g)
        body = b">g%d part1\n" % i + g[: len(g) // 2].tobytes() + b"\n>g%d part2\n" % i + g[len(g) // 2:].tobytes() + b"\n"
        if i == 2:
            p = tmp_path / f"genome{i}.fa.gz"
            p.write_bytes(gzip.compress(body))
        else:
            p = tmp_path / f"genome{i}.fa"
            p.write_bytes(body)
        paths.append(str(p))
    return genomes, paths


def _oracle(genomes):
    seqs, cols = [], []
    for i, g in enumerate(genomes):
        seqs += [g[: len(g) // 2], g[len(g) // 2:]]
        cols += [i, i]
    text, off, ln, col = synth.pack_sequences(seqs, cols)
    return oracle.build_graph(text, off, ln, oracle.params(k=K, m=10, bucket_bits=6, second_bits=2, threads=8,
                                                            colors=True), seq_colors=col)


def _read_graph(path):
    recs = []
    hdr = None
    for line in open(path, "rb").read().split(b"\n"):
        if line.startswith(b">"):
            hdr = line
        elif line and hdr is not None:
            runs = [(int(t.split(b":")[1], 16), int(t.split(b":")[2])) for t in hdr.split() if t.startswith(b"C:")]
            recs.append((line, runs))
            hdr = None
    return recs


@pytest.fixture(scope="module")
def colored_graph(tmp_path_factory):
    import ggcat_gb300

    tmp = tmp_path_factory.mktemp("colored")
    genomes, paths = _files(tmp)
    names = [f"genome_{i}" for i in range(len(paths))]
    inst = ggcat_gb300.GGCATInstance.create(ggcat_gb300.GGCATConfig())
    out = str(tmp / "graph.fa")
    assert inst.build_graph(paths, out, color_names=names, kmer_length=K, colors=True, min_multiplicity=1) == out
    return inst, out, genomes, names, _oracle(genomes), tmp


def _canon(s):
    rc = bytes(synth.revcomp(np.frombuffer(s, np.uint8)))
    return min(s, rc)


_CODE = {0: b"A", 1: b"C", 2: b"T", 3: b"G"}


def _unpack(v):
    """an oracle key (2-bit packed, base i at bits 2i, A0 C1 T2 G3) as bases"""
    return b"".join(_CODE[(int(v) >> (2 * j)) & 3] for j in range(K))


def test_colored_build_colour_sets_and_unitigs(colored_graph):
    inst, out, genomes, names, r, _ = colored_graph
    cmap = inst.get_colormap_file(out)
    assert cmap.endswith("graph.colors.dat")
    assert inst.dump_colors(cmap) == names
    recs = _read_graph(out)
    subs = sorted({s for _, runs in recs for s, _ in runs})
    colours = {}
    inst.query_colormap(cmap, subs, True, lambda s, c: colours.__setitem__(s, tuple(c)))
    assert sorted(colours) == subs
    got = {}
    for seq, runs in recs:
        assert sum(c for _, c in runs) == len(seq) - K + 1
        j = 0
        for s, c in runs:
            for t in range(c):
                km = _canon(seq[j + t:j + t + K])
                assert km not in got
                got[km] = colours[s]
            j += c
    # the unitig set equals the oracle's
    seqs = [s for s, _ in recs]
    canon = oracle.canonicalize_unitigs(b"".join(x + b"\n" for x in seqs), np.zeros(len(seqs), np.uint8), K)
    assert canon == r.unitigs()
    # every oracle k-mer's colour set (keyed by the lexicographically smaller orientation, like `got`)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    exp = {_canon(_unpack(lo[i])): tuple(int(c) for c in ccol[coff[i]:coff[i + 1]]) for i in range(len(lo))}
    assert got == exp


@pytest.mark.parametrize("fmt", [0, 1])
def test_colored_query_jsonl(colored_graph, fmt):
    inst, out, genomes, names, r, tmp = colored_graph
    rng = np.random.default_rng(77)
    queries, _ = synth.query_stream(genomes, 40, rng, min_len=40, max_len=4000)
    queries.append(synth.random_genome(500, rng))  # almost surely no match: no line
    qpath = tmp / f"q{fmt}.fa"
    qpath.write_bytes(b"".join(b">q%d\n" % i + q.tobytes() + b"\n" for i, q in enumerate(queries)))
    res = inst.query_graph(out, str(qpath), str(tmp / f"res{fmt}"), kmer_length=K, colors=True,
                           color_output_format=fmt)
    assert res.endswith(".jsonl")
    lines = [json.loads(x) for x in open(res).read().splitlines()]
    qt, qo, ql = serve._pack(queries)
    lo, hi, _ = r.kmers()
    coff, ccol = r.kmer_colors()
    em, qk, epc = oracle.query(lo, hi, qt, qo, ql, K, gc_off=coff, gc_colors=ccol, ncolors=len(genomes))
    exp = []
    for i in range(len(queries)):
        if epc[i].sum() == 0:
            continue
        m = {}
        for c in range(len(genomes)):
            if epc[i, c]:
                key = names[c] if fmt == 1 else str(c)
                m[key] = float("%.2f" % (epc[i, c] / (int(ql[i]) - K + 1)))
        exp.append({"query_index": i, "matches": m})
    assert lines == exp and len(exp) >= 30


def test_colored_dump_unitigs(colored_graph):
    inst, out, genomes, names, r, _ = colored_graph
    got = {}
    last = [None]

    def fn(seq, cols, same):
        assert same == (last[0] == tuple(cols))
        last[0] = tuple(cols)
        for j in range(len(seq) - K + 1):
            km = _canon(seq[j:j + K])
            assert km not in got
            got[km] = tuple(cols)

    inst.dump_unitigs(out, K, None, True, 1, True, fn)
    lo, _, _ = r.kmers()
    assert len(got) == len(lo)


def _kmer_colours(inst, path):
    """k-mer -> colour tuple from a coloured graph FASTA (C: runs) and its colormap; also the
    number of records.  Every k-mer must appear once."""
    cmap = inst.get_colormap_file(path)
    recs = _read_graph(path)
    subs = sorted({s for _, runs in recs for s, _ in runs})
    colours = {}
    inst.query_colormap(cmap, subs, True, lambda s, c: colours.__setitem__(s, tuple(c)))
    got = {}
    for seq, runs in recs:
        assert sum(c for _, c in runs) == len(seq) - K + 1
        j = 0
        for s, c in runs:
            for t in range(c):
                km = _canon(seq[j + t:j + t + K])
                assert km not in got
                got[km] = colours[s]
            j += c
    return got, len(recs)


@pytest.mark.parametrize("mode", [3, 4])
def test_colored_eulertigs_and_pathtigs_keep_every_kmer_colour(colored_graph, mode):
    """Eulertigs (3) and pathtigs (4) of a coloured graph: every k-mer once, with the colour set
    it has in the unitig graph (the C: runs follow each string, reversed through unitigs it
    reads reverse complemented), in fewer records than the unitigs."""
    import ggcat_gb300

    inst, out, genomes, names, r, tmp = colored_graph
    paths = [str(tmp / (f"genome{i}.fa.gz" if i == 2 else f"genome{i}.fa")) for i in range(len(names))]
    exp, n_unitigs = _kmer_colours(inst, out)
    tout = str(tmp / f"tigs{mode}.fa")
    assert inst.build_graph(paths, tout, color_names=names, kmer_length=K, colors=True, min_multiplicity=1,
                            extra_elab=mode) == tout
    got, n_tigs = _kmer_colours(inst, tout)
    assert got == exp
    assert n_tigs < n_unitigs
    with pytest.raises(ggcat_gb300.GgcatGpuError):
        inst.build_graph(paths, str(tmp / "mt.fa"), kmer_length=K, colors=True, min_multiplicity=1,
                         extra_elab=ggcat_gb300.ExtraElaboration.GREEDY_MATCHTIGS)
