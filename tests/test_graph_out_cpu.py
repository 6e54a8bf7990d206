"""Maximal-unitig links and the FASTA / GFA writers (host code, no GPU) against a string
restatement of build_maximal_unitigs_links and of the reference's writers."""
import numpy as np
import pytest

import naive
import oracle
from ggcat_gb300 import _native, synth


def _arrays(unitigs):
    bases = np.frombuffer(b"".join(unitigs), np.uint8)
    ln = np.array([len(u) for u in unitigs], np.uint64)
    off = np.zeros(len(unitigs), np.uint64)
    if len(unitigs) > 1:
        off[1:] = np.cumsum(ln[:-1])
    return bases, off, ln


def _native_links(unitigs, k):
    bases, off, ln = _arrays(unitigs)
    lo, other, overlap, flags = _native.unitig_links(bases, off, ln, k)
    out = []
    for i in range(len(unitigs)):
        lists = []
        for s in (2 * i, 2 * i + 1):
            lists.append([(int(other[j]), int(overlap[j]), bool(flags[j] & 1), bool(flags[j] & 2))
                          for j in range(int(lo[s]), int(lo[s + 1]))])
        out.append(tuple(lists))
    return out


def _key(lst):
    # the reference orders a list by the other index only; ties may come in any order
    return [sorted(v for v in lst if v[0] == j) for j in sorted({v[0] for v in lst})]


def _same(got, exp):
    assert len(got) == len(exp)
    for g, e in zip(got, exp):
        assert [_key(x) for x in g] == [_key(x) for x in e]
        for x in g:
            assert [v[0] for v in x] == sorted(v[0] for v in x)


@pytest.mark.parametrize("seed", range(6))
def test_links_random_short_strings(seed):
    """Short strings over a small k: many shared (k-1)-mers, and (k-1)-mers equal to their
    own reverse complement (e.g. ACGT for k = 5)."""
    rng = np.random.default_rng(seed)
    k = 5
    unitigs = [synth.random_genome(int(rng.integers(k, 9)), rng).tobytes() for _ in range(300)]
    unitigs += [b"ACGTA", b"TACGT", b"AATTC", b"GAATT", b"ACGTACGT"]
    _same(_native_links(unitigs, k), naive.unitig_links(unitigs, k))


@pytest.mark.parametrize("k", [31, 63, 65, 101, 127])
def test_links_of_built_unitigs(k):
    """Links of built unitigs against the string restatement; above k = 64 the (k-1)-mers take
    up to 126 bases (the oracle builds those graphs with the Rabin-Karp u128 hash)."""
    rng = np.random.default_rng(k)
    g = synth.add_repeats(synth.random_genome(60_000, rng), 0.05, 3 * k, 3, 10, rng)
    text, off, ln, _ = synth.pack_sequences([g, synth.substitute(g, 0.01, rng)])
    r = oracle.build_graph(text, off, ln, oracle.params(k=k, m=12 if k > 32 else 10, bucket_bits=4, second_bits=2,
                                                         threads=4,
                                                         hash_kind=oracle.H_CN_RK128 if k > 64 else None))
    unitigs = [line for line in r.unitigs().split(b"\n") if line]
    got, exp = _native_links(unitigs, k), naive.unitig_links(unitigs, k)
    _same(got, exp)
    assert sum(len(a) + len(b) for a, b in got) > 0


def _fasta(unitigs):
    return b"".join(b">%d LN:i:%d\n%s\n" % (i, len(u), u) for i, u in enumerate(unitigs))


def _expected_output(unitigs, k, links, gfa):
    lines = []
    nl = naive.unitig_links(unitigs, k) if links else [([], [])] * len(unitigs)
    for i, u in enumerate(unitigs):
        ls = nl[i][0] + nl[i][1]
        if gfa == 0:
            h = b">%d LN:i:%d" % (i, len(u)) + b"".join(
                b" L:%s:%d:%s" % (b"-" if fc else b"+", j, b"-" if fo else b"+") for j, _, fc, fo in ls)
            lines += [h, u]
        elif gfa == 1:
            lines.append(b"S\t%d\t%s\tLN:i:%d" % (i, u, len(u)))
            lines += [b"L\t%d\t%s\t%d\t%s\t%dM" % (i, b"-" if fc else b"+", j, b"-" if fo else b"+", k - 1)
                      for j, _, fc, fo in ls]
        else:
            lines.append(b"S\t%d\t%d\t%s" % (i, len(u), u))
            for j, ov, fc, fo in ls:
                b1, e1 = (0, k - 1) if fc else (len(u) - k + 1, len(u))
                lines.append(b"E\t*\t%d%s\t%d%s\t%d\t%d%s\t%d\t%d%s" % (
                    i, b"-" if fc else b"+", j, b"-" if fo else b"+", b1, e1, b"" if fc else b"$", ov, ov + k - 1,
                    b"$" if ov > 0 else b""))
    return lines


@pytest.mark.parametrize("gfa", [0, 1, 2])
@pytest.mark.parametrize("links", [False, True])
def test_write_graph(tmp_path, gfa, links):
    rng = np.random.default_rng(7)
    k = 7
    # distinct unitigs with distinct ends, so every list order is fixed
    unitigs, seen = [], set()
    while len(unitigs) < 120:
        u = synth.random_genome(int(rng.integers(k, 20)), rng).tobytes()
        ends = {u[:k - 1], u[len(u) - k + 1:]}
        if ends & seen or naive.rc(u[:k - 1]) in seen:
            continue
        unitigs.append(u)
        seen |= ends
    # and chained ones: 120 -> 121 -> 122, and 123 reverse-complement joined to 121
    base = synth.random_genome(40, rng).tobytes()
    unitigs += [base[:16], base[10:28], base[22:40], naive.rc(base[14:22] + b"A")]
    src = tmp_path / "unitigs.fa"
    src.write_bytes(_fasta(unitigs))
    out = tmp_path / ("graph.gfa" if gfa else "graph.fa")
    _native.write_graph(str(src), str(out), k, links, gfa)
    got = out.read_bytes().split(b"\n")
    assert got[-1] == b""
    exp = _expected_output(unitigs, k, links, gfa)
    if links:
        # lists may order ties differently: compare per unitig as sorted line groups
        assert sorted(got[:-1]) == sorted(exp)
    else:
        assert got[:-1] == exp


def test_errors(tmp_path):
    bases, off, ln = _arrays([b"ACGTACGT", b"ACG"])
    with pytest.raises(_native.GgcatGpuError, match="EINVAL"):
        _native.unitig_links(bases, off, ln, 5)  # a unitig shorter than k
    bases, off, ln = _arrays([b"ACGTNCGT"])
    with pytest.raises(_native.GgcatGpuError, match="EINVAL"):
        _native.unitig_links(bases, off, ln, 5)
    src = tmp_path / "u.fa"
    src.write_bytes(b">0 LN:i:8\nACGTACGT\n")
    with pytest.raises(_native.GgcatGpuError, match="EINVAL"):
        _native.write_graph(str(src), str(tmp_path / "o.gfa"), 5, True, 3)


def test_dump_unitigs(tmp_path):
    """ggcat_dump_unitigs on an uncoloured graph: one call per piece of the graph FASTA (records
    cut with the k - 1 copyback), the piece's bases."""
    rng = np.random.default_rng(3)
    unitigs = [synth.random_genome(int(rng.integers(31, 400)), rng).tobytes() for _ in range(50)]
    src = tmp_path / "graph.fa"
    src.write_bytes(_fasta(unitigs))
    assert _native.dump_unitigs(str(src), 31) == unitigs
    L = _native.load()
    fn = _native.DUMP_FN(lambda *a: None)
    assert L.ggcat_gpu_dump_unitigs(str(src).encode(), 31, 1, fn, None) == -6  # colours, no colormap: EIO


def test_dump_unitigs_colored(tmp_path):
    """The coloured branch of ggcat_dump_unitigs on a hand-made coloured graph (C: runs in the
    headers, a colormap beside it): every k-mer once, in single-subset pieces grouped by subset
    in ascending order, with the subset's colours and same_colors on all but the first piece of
    a group."""
    rng = np.random.default_rng(8)
    k = 11
    subsets = [[0], [1, 3], [0, 1, 2, 3], [2]]
    recs, truth = [], []
    for u in range(20):
        seq = synth.random_genome(int(rng.integers(k, 120)), rng).tobytes()
        nk = len(seq) - k + 1
        runs, left, pos = [], nk, 0
        while left:
            c = int(rng.integers(1, left + 1))
            sub = int(rng.integers(0, len(subsets)))
            if runs and runs[-1][0] == sub:
                runs[-1][1] += c
            else:
                runs.append([sub, c])
            for j in range(c):
                truth.append((seq[pos + j:pos + j + k], sub))
            pos += c
            left -= c
        hdr = f">{u} LN:i:{len(seq)}" + "".join(f" C:{a:x}:{b}" for a, b in runs)
        recs.append(hdr.encode() + b"\n" + seq + b"\n")
    g = tmp_path / "cg.fa"
    g.write_bytes(b"".join(recs))
    _native.write_colormap(str(tmp_path / "cg.colors.dat"), ["a", "b", "c", "d"], subsets)
    out = _native.dump_unitigs(str(g), k, colors=True)
    got, last = [], None
    for bases, cols, same in out:
        sub = subsets.index(cols)
        assert same == (last == sub)
        assert last is None or sub >= last
        last = sub
        for j in range(len(bases) - k + 1):
            got.append((bases[j:j + k], sub))
    assert sorted(got) == sorted(truth)

