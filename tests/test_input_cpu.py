"""Host input readers (no GPU): FASTQ parsing against a restatement of the reference's
state machine, and whole files read like the reference's SequencesReader -- FASTA / FASTQ by
the extension chain, decompressed by the last extension (gz, bz2, xz from the standard
library; zst and lz4 compressed through the system libraries) -- equal to the parse of the
plain bytes."""
import bz2
import ctypes as C
import gzip
import lzma

import numpy as np
import pytest

import naive
import oracle
from ggcat_gb300 import _native, synth

FASTQ_CASES = {
    "plain": b"@r1\nACGTACGTTT\n+\nIIIIIIIIII\n@r2\nggcaNNtt\n+r2\nIIIIIIII\n",
    "crlf": b"@r1\r\nACGTAC\r\n+\r\nIIIIII\r\n@r2\r\nTTGG\r\n+\r\nIIII\r\n",
    "no_final_newline": b"@r1\nACGT\n+\nIIII\n@r2\nGGCC\n+\nIIII",
    "empty_sequence": b"@r1\n\n+\n\n@r2\nACG\n+\nIII\n",
    "ends_after_sequence": b"@r1\nACGT\n+\nIIII\n@r2\nGATTACA\n",
    "ends_after_plus": b"@r1\nACGT\n+\nIIII\n@r2\nGATTACA\n+\n",
    "iupac": b"@r1\nACGTRYKMSWBDHVN-.acgtx\n+\nIIIIIIIIIIIIIIIIIIIIII\n",
    "empty_file": b"",
}


@pytest.mark.parametrize("name", sorted(FASTQ_CASES))
def test_fastq_parse_matches_restatement(name):
    data = FASTQ_CASES[name]
    got = _native.fastq_parse(data).tobytes()
    exp = b"".join(r + b"\n" for r in naive.fastq_records(data))
    assert got == exp


def _fasta_bytes(seed=3, n=40):
    rng = np.random.default_rng(seed)
    recs = []
    for i in range(n):
        g = synth.random_genome(int(rng.integers(1, 3000)), rng).tobytes().decode()
        lines = "\n".join(g[j:j + 61] for j in range(0, len(g), 61))
        recs.append(f">seq{i} some description\n{lines.lower() if i % 7 == 0 else lines}\n")
    # (no ';' comment line: after one the reference skips every following full line)
    return ("".join(recs) + ">empty\n").encode()


def _fastq_bytes(seed=4, n=300):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = synth.random_genome(int(rng.integers(0, 200)), rng).tobytes()
        out.append(b"@read%d\n%s\n+\n%s\n" % (i, s, b"I" * len(s)))
    return b"".join(out)


def _zstd(data: bytes) -> bytes:
    try:
        lib = C.CDLL("libzstd.so.1")
    except OSError:
        pytest.skip("libzstd.so.1 not installed")
    lib.ZSTD_compressBound.restype = C.c_size_t
    lib.ZSTD_compressBound.argtypes = [C.c_size_t]
    lib.ZSTD_compress.restype = C.c_size_t
    lib.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
    cap = lib.ZSTD_compressBound(len(data))
    dst = C.create_string_buffer(cap)
    n = lib.ZSTD_compress(dst, cap, data, len(data), 3)
    assert n <= cap
    return dst.raw[:n]


def _lz4(data: bytes) -> bytes:
    try:
        lib = C.CDLL("liblz4.so.1")
    except OSError:
        pytest.skip("liblz4.so.1 not installed")
    lib.LZ4F_compressFrameBound.restype = C.c_size_t
    lib.LZ4F_compressFrameBound.argtypes = [C.c_size_t, C.c_void_p]
    lib.LZ4F_compressFrame.restype = C.c_size_t
    lib.LZ4F_compressFrame.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]
    cap = lib.LZ4F_compressFrameBound(len(data), None)
    dst = C.create_string_buffer(cap)
    n = lib.LZ4F_compressFrame(dst, cap, data, len(data), None)
    assert n <= cap
    return dst.raw[:n]


COMPRESSORS = {
    "": lambda b: b,
    ".gz": gzip.compress,
    ".bz2": bz2.compress,
    ".xz": lzma.compress,
    ".zst": _zstd,
    ".lz4": _lz4,
}


@pytest.mark.parametrize("ext", sorted(COMPRESSORS))
@pytest.mark.parametrize("kind,name", [("fasta", "genome.fa"), ("fasta", "genome.fna"), ("fastq", "reads.fq"),
                                       ("fastq", "reads.fastq")])
def test_read_sequences_file(tmp_path, kind, name, ext):
    data = _fasta_bytes() if kind == "fasta" else _fastq_bytes()
    path = tmp_path / (name + ext)
    path.write_bytes(COMPRESSORS[ext](data))
    got = _native.read_sequences_file(str(path), 30).tobytes()
    exp = _native.fasta_parse(data, 30).tobytes() if kind == "fasta" else _native.fastq_parse(data).tobytes()
    assert got == exp and len(exp) > 0


def test_fasta_file_matches_oracle_parse(tmp_path):
    data = _fasta_bytes(seed=9)
    path = tmp_path / "g.fasta.gz"
    path.write_bytes(gzip.compress(data))
    got = _native.read_sequences_file(str(path), 30)
    text, off, ln = oracle.fasta_parse(data, 30)
    exp = b"".join(text[o:o + n].tobytes() + b"\n" for o, n in zip(off.tolist(), ln.tolist()))
    assert got.tobytes() == exp and len(exp) > 0


def test_concatenated_members_and_frames(tmp_path):
    a, b = _fastq_bytes(seed=1, n=50), _fastq_bytes(seed=2, n=70)
    exp = _native.fastq_parse(a + b).tobytes()
    for ext, comp in ((".gz", gzip.compress), (".bz2", bz2.compress), (".xz", lzma.compress), (".zst", _zstd),
                      (".lz4", _lz4)):
        path = tmp_path / ("two.fq" + ext)
        path.write_bytes(comp(a) + comp(b))
        assert _native.read_sequences_file(str(path)).tobytes() == exp, ext


def test_unknown_type_and_bad_files(tmp_path):
    plain = tmp_path / "reads.txt"
    plain.write_bytes(_fastq_bytes(n=3))
    with pytest.raises(_native.GgcatGpuError, match="EUNSUPPORTED"):
        _native.read_sequences_file(str(plain))
    with pytest.raises(_native.GgcatGpuError, match="EIO"):
        _native.read_sequences_file(str(tmp_path / "missing.fa"))
    corrupt = tmp_path / "reads.fq.gz"
    corrupt.write_bytes(_fastq_bytes(n=3))  # not gzip data
    with pytest.raises(_native.GgcatGpuError, match="EIO"):
        _native.read_sequences_file(str(corrupt))
    whole = gzip.compress(_fastq_bytes(n=200))
    truncated = tmp_path / "cut.fq.gz"
    truncated.write_bytes(whole[: len(whole) // 2])
    with pytest.raises(_native.GgcatGpuError, match="EIO"):
        _native.read_sequences_file(str(truncated))
    for ext, comp in ((".bz2", bz2.compress), (".xz", lzma.compress), (".zst", _zstd), (".lz4", _lz4)):
        whole = comp(_fastq_bytes(n=200))
        cut = tmp_path / ("cut.fq" + ext)
        cut.write_bytes(whole[: len(whole) // 2])
        with pytest.raises(_native.GgcatGpuError, match="EIO"):
            _native.read_sequences_file(str(cut))


def test_extension_chain(tmp_path):
    """The type is the first known extension from the end: 'x.fa.backup.gz' is FASTA."""
    data = _fasta_bytes(seed=5, n=5)
    path = tmp_path / "x.fa.backup.gz"
    path.write_bytes(gzip.compress(data))
    assert _native.read_sequences_file(str(path), 30).tobytes() == _native.fasta_parse(data, 30).tobytes()


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_many_files_in_input_order(tmp_path, threads):
    """Files read on several threads are concatenated in input order, like one after another."""
    paths, exp = [], b""
    for i in range(11):
        kind = i % 3
        data = _fasta_bytes(seed=100 + i, n=5) if kind else _fastq_bytes(seed=200 + i, n=20)
        name = f"f{i}." + ("fa" if kind else "fq") + (".gz" if i % 2 else "")
        p = tmp_path / name
        p.write_bytes(gzip.compress(data) if i % 2 else data)
        paths.append(str(p))
        exp += _native.read_sequences_file(str(p), 30).tobytes()
    assert _native.read_sequences_files(paths, 30, threads).tobytes() == exp
    bad = paths[:4] + [str(tmp_path / "missing.fa")] + paths[4:]
    with pytest.raises(_native.GgcatGpuError, match="EIO"):
        _native.read_sequences_files(bad, 30, threads)



def _big_fasta(seed, crlf=False, comment=False):
    rng = np.random.default_rng(seed)
    parts = []
    total = 0
    i = 0
    while total < 20 << 20:
        n = int(rng.choice([200, 5_000, 300_000, 5_000_000]))  # some records above the 4 MiB buffer
        s = synth.random_genome(n, rng).tobytes()
        eol = b"\r\n" if crlf else b"\n"
        width = int(rng.choice([60, 80, 1 << 30]))
        body = eol.join(s[j:j + width] for j in range(0, len(s), width))
        parts.append(b">rec%d len=%d" % (i, n) + eol + body + eol)
        if comment and i == 3:
            parts.append(b";a comment" + eol)
        total += len(parts[-1])
        i += 1
    return b"".join(parts)


@pytest.mark.parametrize("crlf,comment", [(False, False), (True, False), (False, True)])
@pytest.mark.parametrize("threads", [2, 5, 16])
def test_large_fasta_parsed_on_threads_equals_whole_file_parse(tmp_path, crlf, comment, threads):
    """A FASTA file of 16 MiB or more is parsed in record-aligned ranges on threads; the text
    (pieces cut with the copyback across the 4 MiB buffers) equals the whole-file parse.  A
    file with a ';' comment line is parsed whole."""
    data = _big_fasta(crlf * 2 + comment, crlf, comment)
    p = tmp_path / "big.fa"
    p.write_bytes(data)
    got = _native.read_sequences_files([str(p)], 30, threads).tobytes()
    assert got == _native.fasta_parse(data, 30).tobytes()


def test_collect_streams():
    """ggcat_gpu_collect_streams (the text of ggcat_gpu_build_from_streams): every emitted
    sequence normalised like the reader and followed by a newline, streams in order, the
    copyback handed to each stream."""
    srcs = [[b"ACGTacgtNx", b"", b"GATTACA"], [b"ccccRYTT", b"A" * 100]]
    seen = []
    got = _native.collect_streams(srcs, 30, seen).tobytes()
    exp = b"".join(naive.normalize(s) + b"\n" for src in srcs for s in src)
    assert got == exp
    assert seen == [30] * (2 * len(srcs))  # the wrapper reads every stream twice: size, then text

