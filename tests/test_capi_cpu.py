"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, exports every
symbol include/ggcat_gb300.h declares, and its host FASTA reader cuts records exactly
like the oracle's restatement of SequencesReader::process_fasta."""
import os
import re

import numpy as np
import pytest

import oracle
from ggcat_gb300 import _native, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_header_symbols():
    L = _native.load()
    hdr = open(os.path.join(ROOT, "include", "ggcat_gb300.h")).read()
    declared = set(re.findall(r"\b(ggcat_gpu_\w+)\s*\(", hdr))
    assert declared, "no declarations parsed"
    assert declared == set(_native.EXPORTED)
    for name in declared:
        assert hasattr(L, name), name


def _fasta_cases():
    rng = np.random.default_rng(3)
    big = synth.random_genome(9_500_000, rng).tobytes()
    small = [synth.random_genome(int(n), rng).tobytes() for n in rng.integers(50, 400, size=30)]
    cases = []
    # long record, 60-column lines: two 4 MiB cuts with k-1 copyback
    cases.append(b">big one\n" + b"\n".join(big[i:i + 60] for i in range(0, len(big), 60)) + b"\n")
    # unwrapped long record (one line longer than the 4 MiB read buffer), no trailing newline
    cases.append(b">x\n" + big[:5_000_000])
    # many short records, CRLF line ends, comments, lowercase and IUPAC letters
    parts = []
    for i, s in enumerate(small):
        s = s[:10] + b"nRyk" + s[10:].lower() if i % 3 == 0 else s
        if i % 5 == 0:
            parts.append(b";comment line\r\n")
        parts.append(b">r%d desc\r\n" % i + b"\r\n".join(s[j:j + 70] for j in range(0, len(s), 70)) + b"\r\n")
    cases.append(b"".join(parts))
    return cases


@pytest.mark.parametrize("case", range(3))
@pytest.mark.parametrize("k", [31, 63])
def test_fasta_parse_matches_oracle(case, k):
    data = _fasta_cases()[case]
    got = _native.fasta_parse(data, k - 1)
    text, off, ln = oracle.fasta_parse(data, k - 1)
    exp = b"".join(text[o:o + l].tobytes() + b"\n" for o, l in zip(off.tolist(), ln.tolist()))
    assert got.tobytes() == exp
