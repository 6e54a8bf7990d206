// Host input readers of the build and query paths: a whole file, decompressed by its last
// extension and parsed as FASTA or FASTQ by its extension chain, into the device text layout
// (normalised pieces, each followed by '\n').
//   LinesReader::read_binary_file (crates/io/src/lines_reader.rs:60-143): gz, lz4, bz2, xz,
//     zst/zstd, anything else read as is;
//   SequencesReader::process_file_extended (crates/io/src/sequences_reader.rs:56-104): the
//     type is the first known extension walking from the end (fq/fastq; fa/fasta/fna/ffn),
//     any other name is rejected;
//   process_fasta (:106-182) with the 4 MiB line buffers of LinesReader::process_lines
//     (lines_reader.rs:147-213) and an optional copyback that cuts long records into
//     overlapping pieces; process_fastq (:183-241).
// The decompressors are the system's shared libraries, opened at run time (libz, liblz4,
// libbz2, liblzma, libzstd): nothing is needed to build, and a missing library is an error
// only for the files that need it.
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ggcat_gb300.h"
#include "input.h"

namespace ggcat {
namespace {

// ACGTacgt -> upper case, anything else -> N (SEQ_LETTERS_MAPPING, sequences_reader.rs:26-37)
struct Normaliser {
    uint8_t t[256];
    Normaliser() {
        for (int i = 0; i < 256; i++) t[i] = 'N';
        for (const char c : {'A', 'C', 'G', 'T'}) t[(uint8_t)c] = t[(uint8_t)(c | 0x20)] = (uint8_t)c;
    }
};
const Normaliser kNorm;

// Output of the parsers: the text plus, per piece, its offset and length.
struct Sink {
    uint8_t *out;  // null: count only
    uint64_t cap, used = 0, pieces = 0;
    std::vector<uint64_t> *off = nullptr, *len = nullptr;
    void emit(const uint8_t *s, size_t n) {
        if (off) off->push_back(used);
        if (len) len->push_back(n);
        if (out && used + n + 1 <= cap) {
            for (size_t i = 0; i < n; i++) out[used + i] = kNorm.t[s[i]];
            out[used + n] = '\n';
        }
        used += n + 1;
        pieces++;
    }
};

// The line splitter of LinesReader over 4 MiB buffers: a line that crosses a buffer end is
// delivered in parts (partial = true), '\r' before '\n' and at a buffer end is dropped.
// [s, e) of the file is split into the buffers the whole file would be read in (file
// positions that are multiples of 4 MiB), so a range that starts at a line start gives the
// same callbacks as the whole-file pass; the final (finished) callback closes the range.
template <typename F>
void for_each_line(const uint8_t *file, uint64_t s, uint64_t e, F &&line) {
    constexpr uint64_t kBuf = 4u << 20;
    for (uint64_t base = s; base < e;) {
        const uint64_t bend = std::min<uint64_t>(e, (base / kBuf + 1) * kBuf);
        const uint64_t blen = bend - base;
        const uint8_t *buf = file + base;
        uint64_t p = 0;
        for (;;) {
            const uint8_t *nl = (const uint8_t *)memchr(buf + p, '\n', blen - p);
            if (nl) {
                const uint64_t pos = (uint64_t)(nl - buf);
                uint64_t bpos = pos;
                if (bpos != p && buf[bpos - 1] == '\r') bpos--;
                line(buf + p, bpos - p, false, false);
                p = pos + 1;
            } else {
                uint64_t l = blen - p;
                if (l > 0 && buf[blen - 1] == '\r') l--;
                if (l > 0) line(buf + p, l, true, false);
                break;
            }
        }
        base = bend;
    }
    line(nullptr, 0, false, true);
}
template <typename F>
void for_each_line(const uint8_t *file, uint64_t n, F &&line) {
    for_each_line(file, 0, n, line);
}

// process_fasta: records from '>' lines, ';' comment lines skipped, empty records dropped;
// with copyback >= 0 a record reaching max(4 MiB, 2 copyback) bases is emitted and restarted
// from its last copyback bases.
void parse_fasta(const uint8_t *file, uint64_t s, uint64_t e, int64_t copyback, Sink &sink) {
    const size_t flush = std::max<size_t>(4u << 20, copyback > 0 ? (size_t)copyback * 2 : 0);
    std::vector<uint8_t> seq;
    bool on_comment = false, new_line = true, ident = false;
    for_each_line(file, s, e, [&](const uint8_t *l, size_t len, bool partial, bool finished) {
        if (on_comment) {
            on_comment = !partial;
        } else if (finished || (new_line && len > 0 && l[0] == '>')) {
            if (!seq.empty()) sink.emit(seq.data(), seq.size());
            seq.clear();
            ident = partial;
        } else if (new_line && len > 0 && l[0] == ';') {
            on_comment = true;
        } else if (ident) {
            if (!partial) ident = false;
        } else {
            seq.insert(seq.end(), l, l + len);
        }
        if (copyback >= 0 && seq.size() >= flush) {
            sink.emit(seq.data(), seq.size());
            std::vector<uint8_t> tail(seq.end() - (long)copyback, seq.end());
            seq.swap(tail);
        }
        new_line = !partial;
    });
}

// process_fastq: four-line records (ident, sequence, '+' line, quality); a record is emitted
// when its quality line ends, even with an empty sequence; a file ending inside a record
// emits the sequence read so far if it is not empty.  Records are never cut.
void parse_fastq(const uint8_t *file, uint64_t n, Sink &sink) {
    enum { kIdent = 0, kSeq = 1, kQual = 2 };
    int state = kIdent;
    bool skipped_plus = false;
    std::vector<uint8_t> seq;
    for_each_line(file, n, [&](const uint8_t *l, size_t len, bool partial, bool finished) {
        if (finished) {
            if (!seq.empty()) sink.emit(seq.data(), seq.size());
            return;
        }
        if (state == kQual) {
            if (!skipped_plus) {
                if (!partial) skipped_plus = true;
                return;  // the '+' line does not advance the state
            }
            if (!partial) {
                sink.emit(seq.data(), seq.size());
                seq.clear();
                skipped_plus = false;
            }
        } else if (state == kSeq) {
            seq.insert(seq.end(), l, l + len);
        }
        if (!partial) state = (state + 1) % 3;
    });
}

// ---- decompression through the system libraries ----

// the first of the names that loads; each decompressor keeps its handle in a function-local
// static, so a library is opened once per process
void *open_first(std::initializer_list<const char *> names) {
    for (const char *nm : names)
        if (void *h = dlopen(nm, RTLD_NOW | RTLD_LOCAL)) return h;
    return nullptr;
}

template <typename F>
bool bind(void *h, const char *name, F &fn) {
    fn = reinterpret_cast<F>(dlsym(h, name));
    return fn != nullptr;
}

constexpr size_t kOutChunk = 4u << 20;

// zlib (z_stream of zlib.h), gzip or zlib streams, concatenated gzip members
struct ZStream {
    const uint8_t *next_in;
    unsigned avail_in;
    unsigned long total_in;
    uint8_t *next_out;
    unsigned avail_out;
    unsigned long total_out;
    const char *msg;
    void *state;
    void *zalloc, *zfree, *opaque;
    int data_type;
    unsigned long adler, reserved;
};
int inflate_gz(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    static void *const h = open_first({"libz.so.1", "libz.so"});
    if (!h) return err = "gz input needs libz.so.1", GGCAT_GPU_EUNSUPPORTED;
    const char *(*version)() = nullptr;
    int (*init2)(ZStream *, int, const char *, int) = nullptr;
    int (*inflate)(ZStream *, int) = nullptr;
    int (*reset)(ZStream *) = nullptr;
    int (*end)(ZStream *) = nullptr;
    if (!bind(h, "zlibVersion", version) || !bind(h, "inflateInit2_", init2) || !bind(h, "inflate", inflate) ||
        !bind(h, "inflateReset", reset) || !bind(h, "inflateEnd", end))
        return err = "libz.so.1 lacks the inflate entry points", GGCAT_GPU_EUNSUPPORTED;
    ZStream z{};
    if (init2(&z, 15 + 32, version(), (int)sizeof(ZStream)) != 0) return err = "inflateInit2 failed", GGCAT_GPU_EIO;
    // the input is handed over in windows of at most 1 GiB (avail_in is 32 bits)
    z.next_in = in.data();
    z.avail_in = (unsigned)std::min<size_t>(in.size(), 1u << 30);
    int rc = GGCAT_GPU_OK;
    for (;;) {
        const size_t o = out.size();
        out.resize(o + kOutChunk);
        z.next_out = out.data() + o;
        z.avail_out = (unsigned)kOutChunk;
        const int r = inflate(&z, 0);
        out.resize(o + (kOutChunk - z.avail_out));
        const size_t pos = (size_t)(z.next_in - in.data());
        if (z.avail_in == 0 && pos < in.size()) z.avail_in = (unsigned)std::min<size_t>(in.size() - pos, 1u << 30);
        if (r == 1) {  // end of a member: another may follow
            if (pos >= in.size()) break;
            if (reset(&z) != 0) {
                rc = GGCAT_GPU_EIO;
                err = "inflateReset failed";
                break;
            }
            continue;
        }
        if (r == -5 && z.avail_in == 0 && pos >= in.size()) {  // input ended inside a member
            rc = GGCAT_GPU_EIO;
            err = "truncated gz input";
            break;
        }
        if (r != 0 && r != -5) {
            rc = GGCAT_GPU_EIO;
            err = std::string("corrupt gz input") + (z.msg ? std::string(": ") + z.msg : std::string());
            break;
        }
    }
    end(&z);
    return rc;
}

// bzip2 (bz_stream of bzlib.h), concatenated streams
struct BzStream {
    const char *next_in;
    unsigned avail_in, total_in_lo32, total_in_hi32;
    char *next_out;
    unsigned avail_out, total_out_lo32, total_out_hi32;
    void *state;
    void *bzalloc, *bzfree, *opaque;
};
int inflate_bz2(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    static void *const h = open_first({"libbz2.so.1.0", "libbz2.so.1", "libbz2.so"});
    if (!h) return err = "bz2 input needs libbz2.so.1.0", GGCAT_GPU_EUNSUPPORTED;
    int (*init)(BzStream *, int, int) = nullptr;
    int (*dec)(BzStream *) = nullptr;
    int (*end)(BzStream *) = nullptr;
    if (!bind(h, "BZ2_bzDecompressInit", init) || !bind(h, "BZ2_bzDecompress", dec) ||
        !bind(h, "BZ2_bzDecompressEnd", end))
        return err = "libbz2 lacks the decompression entry points", GGCAT_GPU_EUNSUPPORTED;
    size_t pos = 0;
    while (pos < in.size()) {
        BzStream s{};
        if (init(&s, 0, 0) != 0) return err = "BZ2_bzDecompressInit failed", GGCAT_GPU_EIO;
        int r = 0;
        for (;;) {
            const size_t window = std::min<size_t>(in.size() - pos, 1u << 30);
            s.next_in = reinterpret_cast<const char *>(in.data() + pos);
            s.avail_in = (unsigned)window;
            const size_t o = out.size();
            out.resize(o + kOutChunk);
            s.next_out = reinterpret_cast<char *>(out.data() + o);
            s.avail_out = (unsigned)kOutChunk;
            r = dec(&s);
            out.resize(o + (kOutChunk - s.avail_out));
            pos += window - s.avail_in;
            if (r == 4) break;  // end of this stream
            if (r != 0) break;
            if (pos >= in.size() && s.avail_out != 0) {
                r = -7;  // input ended inside a stream
                break;
            }
        }
        end(&s);
        if (r != 4) return err = r == -7 ? "truncated bz2 input" : "corrupt bz2 input", GGCAT_GPU_EIO;
    }
    return GGCAT_GPU_OK;
}

// xz (lzma_stream of lzma.h), concatenated streams
struct LzmaStream {
    const uint8_t *next_in;
    size_t avail_in;
    uint64_t total_in;
    uint8_t *next_out;
    size_t avail_out;
    uint64_t total_out;
    const void *allocator;
    void *internal;
    void *reserved_ptr[4];
    uint64_t reserved_u64[2];
    size_t reserved_size[2];
    int reserved_enum[2];
};
int inflate_xz(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    static void *const h = open_first({"liblzma.so.5", "liblzma.so"});
    if (!h) return err = "xz input needs liblzma.so.5", GGCAT_GPU_EUNSUPPORTED;
    int (*decoder)(LzmaStream *, uint64_t, uint32_t) = nullptr;
    int (*code)(LzmaStream *, int) = nullptr;
    void (*end)(LzmaStream *) = nullptr;
    if (!bind(h, "lzma_stream_decoder", decoder) || !bind(h, "lzma_code", code) || !bind(h, "lzma_end", end))
        return err = "liblzma lacks the decoder entry points", GGCAT_GPU_EUNSUPPORTED;
    LzmaStream s{};
    const uint32_t kConcatenated = 0x08;
    if (decoder(&s, ~0ull, kConcatenated) != 0) return err = "lzma_stream_decoder failed", GGCAT_GPU_EIO;
    s.next_in = in.data();
    s.avail_in = in.size();
    int rc = GGCAT_GPU_OK;
    for (;;) {
        const size_t o = out.size();
        out.resize(o + kOutChunk);
        s.next_out = out.data() + o;
        s.avail_out = kOutChunk;
        const int r = code(&s, s.avail_in ? 0 : 3);  // LZMA_RUN, then LZMA_FINISH
        out.resize(o + (kOutChunk - s.avail_out));
        if (r == 1) break;  // LZMA_STREAM_END
        if (r != 0) {
            rc = GGCAT_GPU_EIO;
            err = r == 10 ? "truncated xz input" : "corrupt xz input";
            break;
        }
    }
    end(&s);
    return rc;
}

// zstd streaming decompression (ZSTD_inBuffer / ZSTD_outBuffer of zstd.h), concatenated frames
struct ZstdIn {
    const void *src;
    size_t size, pos;
};
struct ZstdOut {
    void *dst;
    size_t size, pos;
};
int inflate_zstd(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    static void *const h = open_first({"libzstd.so.1", "libzstd.so"});
    if (!h) return err = "zst input needs libzstd.so.1", GGCAT_GPU_EUNSUPPORTED;
    void *(*create)() = nullptr;
    size_t (*init)(void *) = nullptr;
    size_t (*dec)(void *, ZstdOut *, ZstdIn *) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    size_t (*free_fn)(void *) = nullptr;
    if (!bind(h, "ZSTD_createDStream", create) || !bind(h, "ZSTD_initDStream", init) ||
        !bind(h, "ZSTD_decompressStream", dec) || !bind(h, "ZSTD_isError", is_error) ||
        !bind(h, "ZSTD_freeDStream", free_fn))
        return err = "libzstd lacks the streaming entry points", GGCAT_GPU_EUNSUPPORTED;
    void *ds = create();
    if (!ds || is_error(init(ds))) return err = "ZSTD_initDStream failed", GGCAT_GPU_EIO;
    ZstdIn zi{in.data(), in.size(), 0};
    size_t last = 0;
    int rc = GGCAT_GPU_OK;
    while (zi.pos < zi.size || last != 0) {
        const size_t o = out.size();
        out.resize(o + kOutChunk);
        ZstdOut zo{out.data() + o, kOutChunk, 0};
        const size_t before = zi.pos;
        last = dec(ds, &zo, &zi);
        out.resize(o + zo.pos);
        if (is_error(last)) {
            rc = GGCAT_GPU_EIO;
            err = "corrupt zst input";
            break;
        }
        if (zi.pos == before && zo.pos == 0 && zi.pos >= zi.size) {  // wants input that is not there
            rc = GGCAT_GPU_EIO;
            err = "truncated zst input";
            break;
        }
    }
    free_fn(ds);
    return rc;
}

// lz4 frame format (LZ4F_* of lz4frame.h), concatenated frames
int inflate_lz4(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err) {
    static void *const h = open_first({"liblz4.so.1", "liblz4.so"});
    if (!h) return err = "lz4 input needs liblz4.so.1", GGCAT_GPU_EUNSUPPORTED;
    size_t (*create)(void **, unsigned) = nullptr;
    size_t (*dec)(void *, void *, size_t *, const void *, size_t *, const void *) = nullptr;
    unsigned (*is_error)(size_t) = nullptr;
    size_t (*free_fn)(void *) = nullptr;
    if (!bind(h, "LZ4F_createDecompressionContext", create) || !bind(h, "LZ4F_decompress", dec) ||
        !bind(h, "LZ4F_isError", is_error) || !bind(h, "LZ4F_freeDecompressionContext", free_fn))
        return err = "liblz4 lacks the frame entry points", GGCAT_GPU_EUNSUPPORTED;
    void *dc = nullptr;
    if (is_error(create(&dc, 100u /* LZ4F_VERSION */))) return err = "LZ4F context failed", GGCAT_GPU_EIO;
    size_t pos = 0, hint = 1;
    int rc = GGCAT_GPU_OK;
    for (;;) {
        const size_t o = out.size();
        out.resize(o + kOutChunk);
        size_t dst = kOutChunk, src = in.size() - pos;
        hint = dec(dc, out.data() + o, &dst, in.data() + pos, &src, nullptr);
        out.resize(o + dst);
        pos += src;
        if (is_error(hint)) {
            rc = GGCAT_GPU_EIO;
            err = "corrupt lz4 input";
            break;
        }
        // done (all input read and the last frame complete), or no progress possible
        if (pos >= in.size() && (hint == 0 || dst == 0)) break;
        if (src == 0 && dst == 0) break;
    }
    if (rc == GGCAT_GPU_OK && hint != 0) {  // input ended inside a frame
        rc = GGCAT_GPU_EIO;
        err = "truncated lz4 input";
    }
    free_fn(dc);
    return rc;
}

bool has_ext(const std::string &name, const char *ext) {
    const size_t n = strlen(ext);
    return name.size() > n + 1 && name[name.size() - n - 1] == '.' && name.compare(name.size() - n, n, ext) == 0;
}

std::string base_name(const char *path) {
    std::string p(path);
    const size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

}  // namespace

int sequence_format(const char *path) {
    // process_file_extended: strip extensions from the end until a known one is found
    std::string name = base_name(path);
    for (;;) {
        const size_t dot = name.find_last_of('.');
        if (dot == std::string::npos || dot == 0) return kFormatUnknown;
        const std::string ext = name.substr(dot + 1);
        if (ext == "fq" || ext == "fastq") return kFormatFastq;
        if (ext == "fa" || ext == "fasta" || ext == "fna" || ext == "ffn") return kFormatFasta;
        name.resize(dot);
    }
}

int read_input_file(const char *path, std::vector<uint8_t> &out, std::string &err) {
    out.clear();
    FILE *f = fopen(path, "rb");
    if (!f) return err = std::string("cannot read ") + path, GGCAT_GPU_EIO;
    std::vector<uint8_t> raw;
    // one read of the whole file when its size is known (a regular file), else in pieces
    if (fseek(f, 0, SEEK_END) == 0) {
        const long sz = ftell(f);
        if (sz > 0 && fseek(f, 0, SEEK_SET) == 0) {
            raw.resize((size_t)sz);
            raw.resize(fread(raw.data(), 1, raw.size(), f));
        }
    }
    uint8_t buf[1 << 16];
    size_t r;
    while ((r = fread(buf, 1, sizeof buf, f)) > 0) raw.insert(raw.end(), buf, buf + r);  // the rest, if any
    const bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) return err = std::string("cannot read ") + path, GGCAT_GPU_EIO;
    const std::string name = base_name(path);
    int rc = GGCAT_GPU_OK;
    if (has_ext(name, "gz")) rc = inflate_gz(raw, out, err);
    else if (has_ext(name, "lz4")) rc = inflate_lz4(raw, out, err);
    else if (has_ext(name, "bz2")) rc = inflate_bz2(raw, out, err);
    else if (has_ext(name, "xz")) rc = inflate_xz(raw, out, err);
    else if (has_ext(name, "zst") || has_ext(name, "zstd")) rc = inflate_zstd(raw, out, err);
    else out.swap(raw);
    if (rc) err += std::string(" (") + path + ")";
    return rc;
}

int parse_sequences(const uint8_t *data, uint64_t n, int format, int64_t copyback, uint8_t *h_text, uint64_t cap,
                    uint64_t *text_len, uint64_t *n_pieces, std::vector<uint64_t> *off, std::vector<uint64_t> *len) {
    if (!data && n) return GGCAT_GPU_EINVAL;
    Sink sink{h_text, h_text ? cap : 0};
    sink.off = off;
    sink.len = len;
    if (format == kFormatFastq) parse_fastq(data, n, sink);
    else if (format == kFormatFasta) parse_fasta(data, 0, n, copyback, sink);
    else return GGCAT_GPU_EINVAL;
    if (text_len) *text_len = sink.used;
    if (n_pieces) *n_pieces = sink.pieces;
    if (h_text && sink.used > cap) return GGCAT_GPU_EINVAL;
    return GGCAT_GPU_OK;
}

namespace {

bool has_comment_line(const uint8_t *data, uint64_t n) {
    if (n && data[0] == ';') return true;
    for (const uint8_t *p = data; (p = (const uint8_t *)memchr(p, ';', (size_t)(data + n - p))) != nullptr; p++)
        if (p > data && p[-1] == '\n') return true;
    return false;
}

// FASTA parsed in ranges on threads, appended to text: the ranges start at record starts
// ('>' after '\n') near equal shares of the file and keep the whole-file line buffers, so the
// output is the whole-file parse's byte for byte.  Not used when the file has a ';' comment
// line: after one the reference skips lines across records.
void parse_fasta_threads(const uint8_t *data, uint64_t n, int64_t copyback, int threads, std::vector<uint8_t> &text,
                         std::vector<uint64_t> *off, std::vector<uint64_t> *len) {
    std::vector<uint64_t> cuts{0};
    for (int t = 1; t < threads; t++) {
        uint64_t q = std::max<uint64_t>(cuts.back() + 1, n * (uint64_t)t / (uint64_t)threads);
        for (; q < n; q++) {
            const uint8_t *gt = (const uint8_t *)memchr(data + q, '>', (size_t)(n - q));
            if (!gt) {
                q = n;
                break;
            }
            q = (uint64_t)(gt - data);
            if (q > 0 && data[q - 1] == '\n') break;
        }
        if (q >= n) break;
        cuts.push_back(q);
    }
    cuts.push_back(n);
    const size_t nc = cuts.size() - 1;
    // sizes of every range, then each range parsed straight into its place in text
    std::vector<uint64_t> at(nc + 1, 0);
    std::vector<std::vector<uint64_t>> offs(nc), lens(nc);
    const uint64_t base = text.size();
    auto run = [&](auto &&body) {
        std::atomic<size_t> next{0};
        auto work = [&]() {
            for (size_t c = next++; c < nc; c = next++) body(c);
        };
        std::vector<std::thread> pool;
        for (size_t t = 1; t < std::min<size_t>(nc, (size_t)threads); t++) pool.emplace_back(work);
        work();
        for (auto &th : pool) th.join();
    };
    run([&](size_t c) {
        Sink count{nullptr, 0};
        parse_fasta(data, cuts[c], cuts[c + 1], copyback, count);
        at[c + 1] = count.used;
    });
    for (size_t c = 0; c < nc; c++) at[c + 1] += at[c];
    text.resize(base + at[nc]);
    run([&](size_t c) {
        Sink fill{text.data() + base + at[c], at[c + 1] - at[c]};
        fill.off = off ? &offs[c] : nullptr;
        fill.len = len ? &lens[c] : nullptr;
        parse_fasta(data, cuts[c], cuts[c + 1], copyback, fill);
    });
    for (size_t c = 0; c < nc; c++) {
        if (off)
            for (uint64_t v : offs[c]) off->push_back(base + at[c] + v);
        if (len) len->insert(len->end(), lens[c].begin(), lens[c].end());
    }
}

}  // namespace

int read_sequences(const char *path, int64_t copyback, std::vector<uint8_t> &text, std::vector<uint64_t> *off,
                   std::vector<uint64_t> *len, std::string &err, int threads) {
    const int format = sequence_format(path);
    if (format == kFormatUnknown)
        return err = std::string("cannot recognize the file type of ") + path, GGCAT_GPU_EUNSUPPORTED;
    std::vector<uint8_t> data;
    int rc = read_input_file(path, data, err);
    if (rc) return rc;
    if (format == kFormatFasta && threads > 1 && data.size() >= (16u << 20) &&
        !has_comment_line(data.data(), data.size())) {
        parse_fasta_threads(data.data(), data.size(), copyback, threads, text, off, len);
        return GGCAT_GPU_OK;
    }
    uint64_t need = 0, pieces = 0;
    parse_sequences(data.data(), data.size(), format, copyback, nullptr, 0, &need, &pieces, nullptr, nullptr);
    const size_t o = text.size();
    text.resize(o + need);
    std::vector<uint64_t> loff;
    rc = parse_sequences(data.data(), data.size(), format, copyback, text.data() + o, need, &need, &pieces,
                         off ? &loff : nullptr, len);
    if (off)
        for (uint64_t v : loff) off->push_back(v + o);
    return rc;
}

int read_sequences_files(const char *const *paths, size_t n, int64_t copyback, int threads, std::vector<uint8_t> &text,
                         std::string &err, std::vector<uint64_t> *file_off) {
    // each file into its own buffer on a pool of threads (files are claimed in order), then
    // concatenated in input order: the same text as reading them one after another
    std::vector<std::vector<uint8_t>> parts(n);
    std::vector<std::string> errs(n);
    std::vector<int> rcs(n, GGCAT_GPU_OK);
    std::atomic<size_t> next{0};
    // threads left over by fewer files than threads parse inside the files
    const int per_file = std::max(1, (threads > 0 ? threads : 1) / (int)std::max<size_t>(1, n));
    auto work = [&]() {
        for (size_t i = next++; i < n; i = next++)
            rcs[i] = read_sequences(paths[i], copyback, parts[i], nullptr, nullptr, errs[i], per_file);
    };
    const size_t nt = std::max<size_t>(1, std::min<size_t>(n, threads > 0 ? (size_t)threads : 1));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    size_t total = 0;
    for (size_t i = 0; i < n; i++) {
        if (rcs[i]) return err = errs[i], rcs[i];
        total += parts[i].size();
    }
    text.clear();
    text.reserve(total);
    if (file_off) file_off->clear();
    for (auto &p : parts) {
        if (file_off) file_off->push_back(text.size());
        text.insert(text.end(), p.begin(), p.end());
        std::vector<uint8_t>().swap(p);
    }
    return GGCAT_GPU_OK;
}

int collect_streams(const ggcat_gpu_stream *streams, size_t n, int64_t copyback, std::vector<uint8_t> &text) {
    for (size_t i = 0; i < n; i++)
        if (!streams[i].read_block) return GGCAT_GPU_EINVAL;
    auto emit = [](void *c, const uint8_t *seq, uint64_t len) {
        auto &t = *static_cast<std::vector<uint8_t> *>(c);
        const size_t o = t.size();
        t.resize(o + len + 1);
        for (uint64_t j = 0; j < len; j++) t[o + j] = kNorm.t[seq[j]];
        t[o + len] = '\n';
    };
    for (size_t i = 0; i < n; i++) streams[i].read_block(streams[i].stream_ctx, copyback, emit, &text);
    return GGCAT_GPU_OK;
}

}  // namespace ggcat

extern "C" int ggcat_gpu_collect_streams(const ggcat_gpu_stream *streams, uint64_t n, int64_t copyback, uint8_t *h_text,
                                         uint64_t text_cap, uint64_t *text_len) {
    if (n && !streams) return GGCAT_GPU_EINVAL;
    std::vector<uint8_t> text;
    const int rc = ggcat::collect_streams(streams, (size_t)n, copyback, text);
    if (rc) return rc;
    if (text_len) *text_len = text.size();
    if (h_text) {
        if (text.size() > text_cap) return GGCAT_GPU_EINVAL;
        memcpy(h_text, text.data(), text.size());
    }
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_read_sequences_files(const char *const *paths, uint64_t n, int64_t copyback, int threads,
                                              uint8_t *h_text, uint64_t text_cap, uint64_t *text_len, char *err,
                                              uint64_t err_cap) {
    if (n && !paths) return GGCAT_GPU_EINVAL;
    std::string e;
    std::vector<uint8_t> text;
    const int rc = ggcat::read_sequences_files(paths, (size_t)n, copyback, threads, text, e);
    if (err && err_cap) {
        const size_t m = std::min<size_t>(e.size(), err_cap - 1);
        memcpy(err, e.data(), m);
        err[m] = 0;
    }
    if (rc) return rc;
    if (text_len) *text_len = text.size();
    if (h_text) {
        if (text.size() > text_cap) return GGCAT_GPU_EINVAL;
        memcpy(h_text, text.data(), text.size());
    }
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_fasta_parse(const uint8_t *h_file, uint64_t file_len, int64_t copyback, uint8_t *h_text,
                                     uint64_t text_cap, uint64_t *text_len, uint64_t *n_pieces) {
    return ggcat::parse_sequences(h_file, file_len, ggcat::kFormatFasta, copyback, h_text, text_cap, text_len,
                                  n_pieces, nullptr, nullptr);
}

extern "C" int ggcat_gpu_fastq_parse(const uint8_t *h_file, uint64_t file_len, uint8_t *h_text, uint64_t text_cap,
                                     uint64_t *text_len, uint64_t *n_records) {
    return ggcat::parse_sequences(h_file, file_len, ggcat::kFormatFastq, -1, h_text, text_cap, text_len, n_records,
                                  nullptr, nullptr);
}

extern "C" int ggcat_gpu_read_sequences_file(const char *path, int64_t copyback, uint8_t *h_text, uint64_t text_cap,
                                             uint64_t *text_len, uint64_t *n_pieces, char *err, uint64_t err_cap) {
    if (!path) return GGCAT_GPU_EINVAL;
    std::string e;
    std::vector<uint8_t> text;
    const int rc = ggcat::read_sequences(path, copyback, text, nullptr, nullptr, e);
    if (err && err_cap) {
        const size_t n = std::min<size_t>(e.size(), err_cap - 1);
        memcpy(err, e.data(), n);
        err[n] = 0;
    }
    if (rc) return rc;
    if (text_len) *text_len = text.size();
    if (n_pieces) *n_pieces = (uint64_t)std::count(text.begin(), text.end(), (uint8_t)'\n');
    if (h_text) {
        if (text.size() > text_cap) return GGCAT_GPU_EINVAL;
        memcpy(h_text, text.data(), text.size());
    }
    return GGCAT_GPU_OK;
}
