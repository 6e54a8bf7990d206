"""Small, slow, independent Python restatements used to cross-check the oracle:
global canonical k-mer counting and maximal-unitig construction over the
bidirected de Bruijn graph of surviving canonical k-mers."""
from __future__ import annotations

COMP = bytes.maketrans(b"ACGT", b"TGCA")


def rc(s: bytes) -> bytes:
    return s.translate(COMP)[::-1]


def canon(s: bytes) -> bytes:
    r = rc(s)
    return s if s <= r else r


def pieces(seq: bytes, k: int):
    """Split at every non-ACGT byte (after upper-casing acgt), keep runs >= k."""
    norm = bytes(c if c in b"ACGT" else (c - 32 if c in b"acgt" else ord("N")) for c in seq)
    for part in norm.split(b"N"):
        if len(part) >= k:
            yield part


def kmer_counts(seqs, k: int) -> dict:
    cnt = {}
    for s in seqs:
        for p in pieces(s, k):
            for i in range(len(p) - k + 1):
                c = canon(p[i : i + k])
                cnt[c] = cnt.get(c, 0) + 1
    return cnt


def kmer_colors(seqs, colors, k: int) -> dict:
    """canonical k-mer -> sorted tuple of the colours of the sequences that contain it."""
    out = {}
    for s, c in zip(seqs, colors):
        for p in pieces(s, k):
            for i in range(len(p) - k + 1):
                out.setdefault(canon(p[i : i + k]), set()).add(int(c))
    return {x: tuple(sorted(v)) for x, v in out.items()}


def maximal_unitigs(kmers: set, k: int):
    """Returns list of (sequence, circular) for the maximal unitigs of a canonical k-mer set."""

    def succ(s):
        return [s[1:] + b for b in (b"A", b"C", b"G", b"T") if canon(s[1:] + b) in kmers]

    def pred(s):
        return [b + s[:-1] for b in (b"A", b"C", b"G", b"T") if canon(b + s[:-1]) in kmers]

    def step(s):
        nx = succ(s)
        if len(nx) != 1:
            return None
        t = nx[0]
        if len(pred(t)) != 1:
            return None
        return t

    used = set()
    out = []

    def extend(start_oriented, seq, origin):
        """Extend to the right of start_oriented, appending to seq; stop at branches or
        at an already used k-mer (as the reference's hash-map extender does)."""
        cur = start_oriented
        while True:
            t = step(cur)
            if t is None:
                return False
            if canon(t) in used:
                return t == origin
            used.add(canon(t))
            seq += t[-1:]
            cur = t

    for x in sorted(kmers):
        if x in used:
            continue
        used.add(x)
        fwd = bytearray(x)
        circ = extend(x, fwd, x)
        bwd = bytearray(rc(x))
        extend(rc(x), bwd, rc(x))
        full = rc(bytes(bwd)) + bytes(fwd[k:])
        out.append((full, circ and len(bwd) == k))
    return out


def canonical_unitig(seq: bytes, circular: bool, k: int) -> bytes:
    r = rc(seq)
    if not circular:
        return min(seq, r)
    n = len(seq) - k + 1
    best = None
    for src in (seq, r):
        cyc = src[:n]
        for rot in range(n):
            cand = bytes(cyc[(rot + i) % n] for i in range(len(seq)))
            if best is None or cand < best:
                best = cand
    return best


def canonical_set(unitigs, k: int) -> bytes:
    lines = sorted(canonical_unitig(s, c, k) for s, c in unitigs)
    return b"".join(l + b"\n" for l in lines)


def _lines(data: bytes):
    """LinesReader::process_lines over one buffer (crates/io/src/lines_reader.rs:147-213):
    (line, partial) per line, '\\r' before the line end dropped; a last line without a
    newline is partial."""
    p = 0
    while True:
        e = data.find(b"\n", p)
        if e < 0:
            last = data[p:]
            if last.endswith(b"\r"):
                last = last[:-1]
            if last:
                yield last, True
            return
        line = data[p:e]
        if line.endswith(b"\r") and e != p:
            line = line[:-1]
        yield line, False
        p = e + 1


def normalize(seq: bytes) -> bytes:
    return bytes(c if c in b"ACGT" else (c - 32 if c in b"acgt" else ord("N")) for c in seq)


def fastq_records(data: bytes) -> list[bytes]:
    """SequencesReader::process_fastq (crates/io/src/sequences_reader.rs:183-241) for inputs
    below the 4 MiB line buffer: the state cycles ident -> sequence -> quality; in the quality
    state the first full line (the '+' line) is skipped without advancing, the next full line
    emits the record (even with an empty sequence); at the end a non-empty sequence read so
    far is emitted."""
    out, state, skipped_plus, seq = [], 0, False, b""
    for line, partial in _lines(data):
        if state == 2:
            if not skipped_plus:
                if not partial:
                    skipped_plus = True
                continue
            if not partial:
                out.append(normalize(seq))
                seq = b""
                skipped_plus = False
        elif state == 1:
            seq += line
        if not partial:
            state = (state + 1) % 3
    if seq:
        out.append(normalize(seq))
    return out


def unitig_links(unitigs: list[bytes], k: int):
    """build_maximal_unitigs_links (crates/assembler_pipeline/src/maximal_unitig_links.rs:55-417)
    restated over strings: per unitig (links from its end, links from its beginning), each a
    list of (other, overlap start, flip_current, flip_other) ordered by the other index.
    is_forward of a (k-1)-mer = it is below its reverse complement; for one equal to its
    reverse complement the is_forward entry's list is kept when it is not empty."""
    w = k - 1
    groups = {}
    for i, u in enumerate(unitigs):
        first, last = u[:w], u[len(u) - w:]
        for pos, x, ov in ((0, first, 0), (1, last, len(u) - w)):
            r = rc(x)
            fwd = x < r
            d = fwd if pos == 0 else (not fwd)
            key = min(x, r)
            groups.setdefault(key, []).append((i, pos, ov, d, True))
            if x == r:
                groups[key].append((i, pos, ov, not d, False))
    slots = [[None, None] for _ in unitigs]  # [end, beginning]
    for ents in groups.values():
        if len(ents) < 2:
            continue
        ents.sort(key=lambda e: (e[0], e[1], not e[4]))
        for i, pos, ov, d, primary in ents:
            lst = [(j, jov, pos == 0, jpos == 1) for j, jpos, jov, jd, _ in ents if jd != d]
            if not lst:
                continue
            s = 1 if pos == 0 else 0
            cur = slots[i][s]
            if cur is None or (primary and not cur[1]):
                slots[i][s] = (lst, primary)
    return [tuple(s[0] if s else [] for s in sl) for sl in slots]


def tig_lower_bound(seqs, k: int) -> int:
    """The fewest strings that hold every k-mer of the unitigs `seqs` once (eulertigs): per
    connected component of the unitig graph max(1, sum of binode imbalances / 2), a binode
    being a canonical (k-1)-mer, its imbalance |#ends read into a unitig as the canonical
    (k-1)-mer - #ends read as its reverse complement| (the parity of its ends when it is its
    own reverse complement)."""
    binode = {}
    counts = {}
    parent = list(range(len(seqs)))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for u, s in enumerate(seqs):
        for into in (s[:k - 1], rc(s[len(s) - k + 1:])):
            c = canon(into)
            pal = into == rc(into)
            t = 0 if (pal or into == c) else 1
            if c in binode:
                parent[find(u)] = find(binode[c])
            else:
                binode[c] = u
            cnt = counts.setdefault(c, [0, 0, pal])
            cnt[t] += 1
    comp_imb = {}
    for c, (n0, n1, pal) in counts.items():
        imb = (n0 + n1) % 2 if pal else abs(n0 - n1)
        r = find(binode[c])
        comp_imb[r] = comp_imb.get(r, 0) + imb
    roots = {find(u) for u in range(len(seqs))}
    return sum(max(1, comp_imb.get(r, 0) // 2) for r in roots)
