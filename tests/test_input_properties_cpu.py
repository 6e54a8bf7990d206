"""Property tests of the host parsers (no GPU): arbitrary FASTQ / FASTA byte streams built from
the formats' pieces -- CR/LF mixes, lowercase and other letters, missing final newlines, empty
records, comment lines -- parse like the restatement of the reference's FASTQ reader and like
the oracle's FASTA reader."""
import pytest

hypothesis = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")

import naive  # noqa: E402
import oracle  # noqa: E402
from ggcat_gb300 import _native  # noqa: E402

settings = hypothesis.settings(max_examples=300, deadline=None,
                               suppress_health_check=[hypothesis.HealthCheck.too_slow])

bases = st.text(alphabet="ACGTacgtNnRYK-", max_size=40).map(str.encode)
eol = st.sampled_from([b"\n", b"\r\n"])


@st.composite
def fastq_files(draw):
    out = b""
    for _ in range(draw(st.integers(0, 6))):
        s = draw(bases)
        e = draw(eol)
        out += b"@r" + str(draw(st.integers(0, 99))).encode() + e + s + e + b"+" + e + b"I" * len(s) + e
    if draw(st.booleans()):  # a truncated last record
        parts = [b"@t", draw(bases), b"+", b"II"]
        out += b"\n".join(parts[:draw(st.integers(1, 4))])
    elif out and draw(st.booleans()):
        out = out.rstrip(b"\r\n")
    return out


@st.composite
def fasta_files(draw):
    out = b""
    for _ in range(draw(st.integers(0, 6))):
        e = draw(eol)
        out += b">h" + str(draw(st.integers(0, 99))).encode() + draw(st.sampled_from([b"", b" desc"])) + e
        for _ in range(draw(st.integers(0, 3))):
            out += draw(bases) + e
    if draw(st.booleans()):
        out += b";c" + draw(eol) + b">x" + draw(eol) + draw(bases)
    return out


@settings
@hypothesis.given(fastq_files())
def test_fastq_matches_restatement(data):
    got = _native.fastq_parse(data).tobytes()
    assert got == b"".join(r + b"\n" for r in naive.fastq_records(data))


@settings
@hypothesis.given(fasta_files(), st.sampled_from([-1, 4, 30]))
def test_fasta_matches_oracle(data, copyback):
    got = _native.fasta_parse(data, copyback).tobytes()
    text, off, ln = oracle.fasta_parse(data, copyback)
    assert got == b"".join(text[o:o + n].tobytes() + b"\n" for o, n in zip(off.tolist(), ln.tolist()))


def test_fasta_record_across_buffer_boundary():
    """A sequence line crossing the 4 MiB line buffer (a partial line) with the copyback cut."""
    seq = (b"ACGT" * (1 << 20)) + b"GATTACA" * 100
    data = b">long\n" + seq + b"\n>short\nACGTACGT\n"
    got = _native.fasta_parse(data, 30).tobytes()
    text, off, ln = oracle.fasta_parse(data, 30)
    assert got == b"".join(text[o:o + n].tobytes() + b"\n" for o, n in zip(off.tolist(), ln.tolist()))
