"""The colormap file (colour subsets of a coloured graph) against a Python restatement of the
reference's run-length colormap layout (crates/colors/src/storage/{serializer,run_length,
deserializer}.rs): subset encoding known answers, the reference's own subset round-trip vectors,
the file layout read independently, frames compressed by liblz4 (as the reference writes
them) read back, and the colormap path rule.  CPU only."""
import ctypes as C
import ctypes.util
import struct

import numpy as np
import pytest

from ggcat_gb300 import _native

# ColorIndexSerializer round-trip vectors (run_length.rs:312-333)
REF_VECTORS = [[0, 1, 2, 3, 4, 5, 6, 7], [0], [1], [1, 2, 5, 10, 15, 30, 45], [1, 100, 200, 300, 400, 800],
               [3, 6, 9, 12, 70, 71, 72, 73, 74, 88, 95, 100, 105, 110, 198, 384]]


def _varint(v):
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        out.append(b | (0x80 if v else 0))
        if not v:
            return bytes(out)


def _encode(c):
    """ColorIndexSerializer::serialize_colors, restated."""
    out = bytearray(_varint(c[0] + 2))
    so, so_val, so_cnt = False, 0, 0
    for i in range(1, len(c)):
        d = c[i] - c[i - 1]
        flush = False
        if i + 1 < len(c):
            nd = c[i + 1] - c[i]
            if d == nd:
                if not so:
                    if i + 2 < len(c) and c[i + 2] - c[i + 1] == d:
                        out += _varint(1)
                        so, so_val, so_cnt = True, d, 2
                else:
                    so_cnt += 1
            elif so:
                flush = True
        elif so:
            flush = True
        if flush:
            out += _varint(so_val) + _varint(so_cnt)
            so = False
        elif not so:
            out += _varint(d + 1)
    return bytes(out + _varint(0))


def _read_varint(b, p):
    r = s = 0
    while True:
        x = b[p]
        p += 1
        r |= (x & 0x7F) << s
        s += 7
        if not x & 0x80:
            return r, p


def _decode(b, p):
    v, p = _read_varint(b, p)
    cur = v - 2
    out = [cur]
    while True:
        v, p = _read_varint(b, p)
        if v == 0:
            return out, p
        if v == 1:
            val, p = _read_varint(b, p)
            cnt, p = _read_varint(b, p)
            for _ in range(cnt):
                cur += val
                out.append(cur)
        else:
            cur += v - 1
            out.append(cur)


def _frame_payload_uncompressed(b, p):
    """An LZ4 frame with stored blocks: returns (payload, end)."""
    assert struct.unpack_from("<I", b, p)[0] == 0x184D2204
    flg = b[p + 4]
    p += 7 + (8 if flg & 8 else 0) + (4 if flg & 1 else 0)
    data = bytearray()
    while True:
        bs = struct.unpack_from("<I", b, p)[0]
        p += 4
        if bs == 0:
            break
        assert bs & 0x80000000, "stored block expected"
        n = bs & 0x7FFFFFFF
        data += b[p:p + n]
        p += n + (4 if flg & 0x10 else 0)
    return bytes(data), p + (4 if flg & 4 else 0)


def test_subset_encoding_known_answers():
    assert _encode([0]) == b"\x02\x00"
    assert _encode([0, 1, 2, 3, 4, 5, 6, 7]) == b"\x02\x01\x01\x07\x00"
    assert _encode([1, 2, 5, 10, 15, 30, 45]) == bytes([3, 2, 4, 6, 6, 16, 16, 0])
    for v in REF_VECTORS:
        assert _decode(_encode(v), 0)[0] == v


def test_colormap_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    subsets = list(REF_VECTORS)
    for _ in range(45_000):  # three chunks of 20000 subsets
        n = int(rng.integers(1, 12))
        subsets.append(sorted(set(rng.integers(0, 300, size=n).tolist())))
    names = [f"genome_{i}.fa" for i in range(300)]
    path = str(tmp_path / "g.colors.dat")
    _native.write_colormap(path, names, subsets)
    b = open(path, "rb").read()
    magic, version, index_off, ncol, nsub, total, unc = struct.unpack_from("<16s6Q", b, 0)
    assert magic == b"GGCAT_CMAP_RNLEN" and version == 1 and ncol == 300 and nsub == len(subsets)
    assert total == len(b)
    raw, p = _frame_payload_uncompressed(b, 64)
    (cnt,) = struct.unpack_from("<Q", raw, 0)
    q, got_names = 8, []
    for _ in range(cnt):
        (ln,) = struct.unpack_from("<Q", raw, q)
        got_names.append(raw[q + 8:q + 8 + ln].decode())
        q += 8 + ln
    assert got_names == names
    (npairs,) = struct.unpack_from("<Q", b, index_off)
    pairs = [struct.unpack_from("<IQ", b, index_off + 8 + 12 * i) for i in range(npairs)]
    assert [s for s, _ in pairs] == [0, 20000, 40000]
    assert struct.unpack_from("<Q", b, index_off + 8 + 12 * npairs)[0] == len(subsets)
    decoded, uncompressed = [], 0
    for start, off in pairs:
        payload, _ = _frame_payload_uncompressed(b, off)
        uncompressed += len(payload)
        q = 0
        while q < len(payload):
            s, q = _decode(payload, q)
            decoded.append(s)
    assert decoded == subsets and uncompressed == unc
    # the library's own reader
    assert _native.dump_colors(path) == names
    want = [0, 5, 19999, 20000, 44999, 3, 3, len(subsets) - 1]
    got = _native.query_colormap(path, want)
    assert sorted(got) == sorted(set(want))
    for s in set(want):
        assert got[s] == subsets[s]
    with pytest.raises(_native.GgcatGpuError):
        _native.query_colormap(path, [len(subsets)])


def _lz4():
    name = ctypes.util.find_library("lz4") or "liblz4.so.1"
    try:
        return C.CDLL(name)
    except OSError:
        return None


class _FrameInfo(C.Structure):
    _fields_ = [("blockSizeID", C.c_int), ("blockMode", C.c_int), ("contentChecksumFlag", C.c_int),
                ("frameType", C.c_int), ("contentSize", C.c_ulonglong), ("dictID", C.c_uint),
                ("blockChecksumFlag", C.c_int)]


class _Prefs(C.Structure):
    _fields_ = [("frameInfo", _FrameInfo), ("compressionLevel", C.c_int), ("autoFlush", C.c_uint),
                ("favorDecSpeed", C.c_uint), ("reserved", C.c_uint * 3)]


def _compress(L, data, linked, content_ck, block_ck):
    pr = _Prefs()
    pr.frameInfo.blockSizeID = 4  # 64 KB blocks
    pr.frameInfo.blockMode = 0 if linked else 1
    pr.frameInfo.contentChecksumFlag = int(content_ck)
    pr.frameInfo.blockChecksumFlag = int(block_ck)
    pr.frameInfo.contentSize = len(data)
    pr.compressionLevel = 4
    L.LZ4F_compressFrameBound.restype = C.c_size_t
    L.LZ4F_compressFrameBound.argtypes = [C.c_size_t, C.c_void_p]
    L.LZ4F_compressFrame.restype = C.c_size_t
    L.LZ4F_compressFrame.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]
    cap = L.LZ4F_compressFrameBound(len(data), C.byref(pr))
    dst = C.create_string_buffer(cap)
    n = L.LZ4F_compressFrame(dst, cap, data, len(data), C.byref(pr))
    assert n < (1 << 62)
    return dst.raw[:n]


@pytest.mark.parametrize("linked,content_ck,block_ck", [(True, True, False), (False, False, True),
                                                        (True, False, False)])
def test_reads_compressed_frames(tmp_path, linked, content_ck, block_ck):
    """Colormaps whose frames are LZ4-compressed (the reference's lz4 encoder) load too."""
    L = _lz4()
    if L is None:
        pytest.skip("liblz4 not available")
    rng = np.random.default_rng(9)
    # repetitive subsets, so that matches reach back across 64 KB blocks
    base = [sorted(set(rng.integers(0, 50, size=int(rng.integers(1, 6))).tolist())) for _ in range(300)]
    subsets = [base[i % 300] for i in range(30000)]
    names = ["a", "b\"c", "d\\e"] + [f"n{i}" for i in range(47)]
    names_raw = struct.pack("<Q", len(names)) + b"".join(struct.pack("<Q", len(n.encode())) + n.encode()
                                                          for n in names)
    body = bytearray(64)
    body += _compress(L, names_raw, linked, content_ck, block_ck)
    pairs, unc = [], 0
    for s0 in range(0, len(subsets), 20000):
        payload = b"".join(_encode(s) for s in subsets[s0:s0 + 20000])
        unc += len(payload)
        pairs.append((s0, len(body)))
        body += _compress(L, payload, linked, content_ck, block_ck)
    index_off = len(body)
    body += struct.pack("<Q", len(pairs)) + b"".join(struct.pack("<IQ", s, o) for s, o in pairs)
    body += struct.pack("<Q", len(subsets))
    body[0:64] = struct.pack("<16s6Q", b"GGCAT_CMAP_RNLEN", 1, index_off, len(names), len(subsets), len(body), unc)
    path = str(tmp_path / "ref.colors.dat")
    open(path, "wb").write(bytes(body))
    assert _native.dump_colors(path) == names
    want = list(range(0, 30000, 997)) + [19999, 20000, 29999]
    got = _native.query_colormap(path, want)
    for s in want:
        assert got[s] == subsets[s]


@pytest.mark.parametrize("graph,cmap", [("out.fa", "out.colors.dat"), ("dir.x/out", "dir.x/out.colors.dat"),
                                        ("out.fasta.lz4", "out.fasta.colors.dat"), ("/a/b/graph", "/a/b/graph.colors.dat"),
                                        (".hidden", ".hidden.colors.dat")])
def test_colormap_path(graph, cmap):
    assert _native.colormap_file(graph) == cmap
