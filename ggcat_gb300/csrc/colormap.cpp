// Colour-subset map file of a coloured graph ("<graph>.colors.dat"), in the layout of the
// reference's run-length colormap (crates/colors/src/storage/{serializer,run_length,
// deserializer}.rs), so that a graph built here can be read by GGCAT's tools and the other
// way round:
//
//   header (64 bytes, ColorsFileHeader): magic "GGCAT_CMAP_RNLEN", version 1, index offset,
//          colour count, subset count, total size, total uncompressed size (u64 LE each)
//   LZ4 frame: bincode Vec<String> of the colour names (u64 count, u64 length + bytes each)
//   per chunk of 20000 subsets (COLORS_SINGLE_BATCH_SIZE): one LZ4 frame of the subsets'
//          encodings, one after another
//   index: bincode ColorsIndexMap { pairs: Vec<(start_index u32, file_offset u64)>,
//          subsets_count u64 }
//
// A subset (sorted colour indices) is encoded as in ColorIndexSerializer::serialize_colors
// (run_length.rs:24-80): varint(first + 2), then per following colour varint(diff + 1), where
// three or more equal consecutive differences are written as varint(1), varint(diff),
// varint(count), and a final varint(0).  Varints are LEB128 (io/src/varint.rs:8-24).
//
// Frames are written with uncompressed blocks (a valid LZ4 frame that any LZ4 decoder reads;
// no compression library is needed); the reader decodes compressed blocks too, linked or
// independent, with or without checksums, so files written by the reference load as well.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ggcat_gb300.h"
#include "colormap.h"

namespace ggcat {
namespace cmap {

static const char kMagic[16] = {'G', 'G', 'C', 'A', 'T', '_', 'C', 'M', 'A', 'P', '_', 'R', 'N', 'L', 'E', 'N'};
constexpr uint64_t kVersion = 1;
constexpr uint64_t kHeaderSize = 64;
constexpr uint64_t kBatch = 20000;           // COLORS_SINGLE_BATCH_SIZE (crates/config/src/lib.rs:97)
constexpr uint32_t kLz4Magic = 0x184D2204u;
constexpr uint32_t kLz4MaxBlock = 4u << 20;  // block maximum size of the frames written (BD = 7)

static void put_u32(std::vector<uint8_t> &o, uint32_t v) {
    for (int i = 0; i < 4; i++) o.push_back((uint8_t)(v >> (8 * i)));
}
static void put_u64(std::vector<uint8_t> &o, uint64_t v) {
    for (int i = 0; i < 8; i++) o.push_back((uint8_t)(v >> (8 * i)));
}
static uint32_t get_u32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
static uint64_t get_u64(const uint8_t *p) { return (uint64_t)get_u32(p) | ((uint64_t)get_u32(p + 4) << 32); }

// xxHash32 of fewer than 16 bytes (the LZ4 frame header checksum), from the published
// xxHash specification.
static uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
static uint32_t xxh32_short(const uint8_t *p, size_t len, uint32_t seed) {
    const uint32_t P1 = 2654435761u, P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;
    uint32_t h = seed + P5 + (uint32_t)len;
    size_t i = 0;
    for (; i + 4 <= len; i += 4) {
        h += get_u32(p + i) * P3;
        h = rotl32(h, 17) * P4;
    }
    for (; i < len; i++) {
        h += (uint32_t)p[i] * P5;
        h = rotl32(h, 11) * P1;
    }
    h ^= h >> 15;
    h *= P2;
    h ^= h >> 13;
    h *= P3;
    h ^= h >> 16;
    return h;
}

// One LZ4 frame holding `data` in uncompressed blocks (LZ4 frame format: magic, FLG = version
// 1 + independent blocks, BD = 4 MB blocks, header checksum, blocks with the uncompressed bit,
// end mark).
void lz4_frame_store(std::vector<uint8_t> &out, const uint8_t *data, size_t n) {
    put_u32(out, kLz4Magic);
    const uint8_t desc[2] = {0x60, 0x70};
    out.push_back(desc[0]);
    out.push_back(desc[1]);
    out.push_back((uint8_t)((xxh32_short(desc, 2, 0) >> 8) & 0xFF));
    for (size_t o = 0; o < n; o += kLz4MaxBlock) {
        const uint32_t b = (uint32_t)std::min<size_t>(kLz4MaxBlock, n - o);
        put_u32(out, b | 0x80000000u);
        out.insert(out.end(), data + o, data + o + b);
    }
    put_u32(out, 0);
}

// LZ4 block (compressed) into out, appended; matches may reach into earlier output (linked
// blocks).  Returns false on malformed input.
static bool lz4_block_decode(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t out_limit) {
    size_t i = 0;
    while (i < n) {
        const uint32_t token = in[i++];
        size_t lit = token >> 4;
        if (lit == 15) {
            uint8_t b;
            do {
                if (i >= n) return false;
                b = in[i++];
                lit += b;
            } while (b == 255);
        }
        if (lit > n - i || out.size() + lit > out_limit) return false;
        out.insert(out.end(), in + i, in + i + lit);
        i += lit;
        if (i == n) break;  // the last sequence has literals only
        if (i + 2 > n) return false;
        const size_t off = (size_t)in[i] | ((size_t)in[i + 1] << 8);
        i += 2;
        if (off == 0 || off > out.size()) return false;
        size_t ml = (token & 15) + 4;
        if ((token & 15) == 15) {
            uint8_t b;
            do {
                if (i >= n) return false;
                b = in[i++];
                ml += b;
            } while (b == 255);
        }
        if (out.size() + ml > out_limit) return false;
        const size_t from = out.size() - off;
        for (size_t j = 0; j < ml; j++) out.push_back(out[from + j]);  // may overlap itself
    }
    return true;
}

// Decodes one LZ4 frame starting at in[0]; *used receives the frame's size in bytes.
bool lz4_frame_decode(const uint8_t *in, size_t n, size_t *used, std::vector<uint8_t> &out) {
    out.clear();
    if (n < 7 || get_u32(in) != kLz4Magic) return false;
    const uint8_t flg = in[4];
    if ((flg >> 6) != 1) return false;
    const bool block_ck = (flg >> 4) & 1, content_size = (flg >> 3) & 1, content_ck = (flg >> 2) & 1,
               dict = flg & 1;
    size_t i = 6 + (content_size ? 8 : 0) + (dict ? 4 : 0) + 1;  // FLG, BD, options, HC
    if (i > n) return false;
    const size_t limit = (size_t)1 << 40;
    for (;;) {
        if (i + 4 > n) return false;
        const uint32_t bs = get_u32(in + i);
        i += 4;
        if (bs == 0) break;
        const uint32_t sz = bs & 0x7fffffffu;
        if (sz > n - i) return false;
        if (bs & 0x80000000u) {
            out.insert(out.end(), in + i, in + i + sz);
        } else if (!lz4_block_decode(in + i, sz, out, limit)) {
            return false;
        }
        i += sz + (block_ck ? 4 : 0);
    }
    if (content_ck) i += 4;
    if (i > n) return false;
    *used = i;
    return true;
}

void varint_put(std::vector<uint8_t> &o, uint64_t v) {
    do {
        const uint8_t b = (uint8_t)(v & 0x7f);
        v >>= 7;
        o.push_back(b | (v ? 0x80 : 0));
    } while (v);
}

bool varint_get(const uint8_t *&p, const uint8_t *end, uint64_t *v) {
    uint64_t r = 0;
    for (int s = 0; s < 64; s += 7) {
        if (p >= end) return false;
        const uint8_t b = *p++;
        r |= (uint64_t)(b & 0x7f) << s;
        if (!(b & 0x80)) {
            *v = r;
            return true;
        }
    }
    return false;
}

// ColorIndexSerializer::serialize_colors (run_length.rs:25-80); colors sorted ascending, n >= 1
void subset_encode(std::vector<uint8_t> &o, const uint32_t *c, size_t n) {
    varint_put(o, (uint64_t)c[0] + 2);
    uint32_t last = c[0];
    bool second_order = false;
    uint64_t so_value = 0, so_count = 0;
    for (size_t i = 1; i < n; i++) {
        const uint32_t diff = c[i] - last;
        bool flush = false;
        if (i + 1 < n) {
            const uint32_t next = c[i + 1] - c[i];
            if (diff == next) {
                if (!second_order) {
                    // at least three equal differences in a row before the second-order form pays
                    if (i + 2 < n && c[i + 2] - c[i + 1] == diff) {
                        varint_put(o, 1);
                        so_count = 2;
                        second_order = true;
                        so_value = diff;
                    }
                } else {
                    so_count++;
                }
            } else if (second_order) {
                flush = true;
            }
        } else if (second_order) {
            flush = true;
        }
        if (flush) {
            varint_put(o, so_value);
            varint_put(o, so_count);
            second_order = false;
        } else if (!second_order) {
            varint_put(o, (uint64_t)diff + 1);
        }
        last = c[i];
    }
    varint_put(o, 0);
}

// ColorIndexSerializer::deserialize_colors (run_length.rs:82-119)
bool subset_decode(const uint8_t *&p, const uint8_t *end, std::vector<uint32_t> &out) {
    out.clear();
    uint64_t v;
    if (!varint_get(p, end, &v) || v < 2) return false;
    uint64_t cur = v - 2;
    out.push_back((uint32_t)cur);
    for (;;) {
        if (!varint_get(p, end, &v)) return false;
        if (v == 0) break;
        if (v == 1) {
            uint64_t val, cnt;
            if (!varint_get(p, end, &val) || !varint_get(p, end, &cnt)) return false;
            if (cnt > (1u << 24)) return false;
            for (uint64_t j = 0; j < cnt; j++) {
                cur += val;
                out.push_back((uint32_t)cur);
            }
        } else {
            cur += v - 1;
            out.push_back((uint32_t)cur);
        }
    }
    return true;
}

static void put_string_vec(std::vector<uint8_t> &o, const std::vector<std::string> &names) {
    put_u64(o, names.size());
    for (const auto &s : names) {
        put_u64(o, s.size());
        o.insert(o.end(), s.begin(), s.end());
    }
}

int write(const char *path, const std::vector<std::string> &names, uint64_t n_subsets,
          const std::function<void(uint64_t, std::vector<uint32_t> &)> &subset) {
    FILE *f = fopen(path, "wb");
    if (!f) return GGCAT_GPU_EIO;
    std::vector<uint8_t> buf(kHeaderSize, 0), raw, frame;
    put_string_vec(raw, names);
    lz4_frame_store(buf, raw.data(), raw.size());
    uint64_t offset = buf.size(), uncompressed = 0;
    bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    std::vector<std::pair<uint32_t, uint64_t>> index;
    std::vector<uint32_t> cols;
    for (uint64_t s0 = 0; s0 < n_subsets && ok; s0 += kBatch) {
        raw.clear();
        const uint64_t s1 = std::min<uint64_t>(n_subsets, s0 + kBatch);
        for (uint64_t s = s0; s < s1; s++) {
            subset(s, cols);
            if (cols.empty()) {
                fclose(f);
                return GGCAT_GPU_EINVAL;
            }
            subset_encode(raw, cols.data(), cols.size());
        }
        frame.clear();
        lz4_frame_store(frame, raw.data(), raw.size());
        index.emplace_back((uint32_t)s0, offset);
        ok = fwrite(frame.data(), 1, frame.size(), f) == frame.size();
        offset += frame.size();
        uncompressed += raw.size();
    }
    // index (ColorsIndexMap, bincode), then the header in place
    const uint64_t index_offset = offset;
    buf.clear();
    put_u64(buf, index.size());
    for (const auto &e : index) {
        put_u32(buf, e.first);
        put_u64(buf, e.second);
    }
    put_u64(buf, n_subsets);
    if (ok) ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    const uint64_t total = offset + buf.size();
    std::vector<uint8_t> hdr(kMagic, kMagic + 16);
    put_u64(hdr, kVersion);
    put_u64(hdr, index_offset);
    put_u64(hdr, names.size());
    put_u64(hdr, n_subsets);
    put_u64(hdr, total);
    put_u64(hdr, uncompressed);
    if (ok) ok = fseek(f, 0, SEEK_SET) == 0 && fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
    if (ok) ok = ferror(f) == 0;
    if (fclose(f) != 0) ok = false;
    return ok ? GGCAT_GPU_OK : GGCAT_GPU_EIO;
}

int Reader::open(const char *path, std::string *err) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        if (err) *err = std::string("cannot open ") + path;
        return GGCAT_GPU_EIO;
    }
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    data.resize(sz > 0 ? (size_t)sz : 0);
    const bool rd = data.empty() || fread(data.data(), 1, data.size(), f) == data.size();
    fclose(f);
    auto bad = [&](const char *why) {
        if (err) *err = std::string(path) + ": " + why;
        return GGCAT_GPU_EIO;
    };
    if (!rd || data.size() < kHeaderSize) return bad("short colormap file");
    if (memcmp(data.data(), kMagic, 16) != 0) return bad("not a run-length colormap (magic)");
    index_offset = get_u64(&data[24]);
    colors_count = get_u64(&data[32]);
    subsets_count = get_u64(&data[40]);
    // colour names
    size_t used = 0;
    std::vector<uint8_t> raw;
    if (!lz4_frame_decode(data.data() + kHeaderSize, data.size() - kHeaderSize, &used, raw))
        return bad("bad colour-name frame");
    if (raw.size() < 8) return bad("bad colour-name list");
    const uint64_t nn = get_u64(raw.data());
    size_t p = 8;
    names.clear();
    for (uint64_t i = 0; i < nn; i++) {
        if (p + 8 > raw.size()) return bad("bad colour-name list");
        const uint64_t ln = get_u64(&raw[p]);
        p += 8;
        if (ln > raw.size() - p) return bad("bad colour-name list");
        names.emplace_back(reinterpret_cast<const char *>(&raw[p]), (size_t)ln);
        p += ln;
    }
    // chunk index
    if (index_offset + 8 > data.size()) return bad("bad index offset");
    const uint8_t *q = &data[index_offset];
    const uint64_t np = get_u64(q);
    if (np > (data.size() - index_offset) / 12) return bad("bad index");
    chunks.clear();
    for (uint64_t i = 0; i < np; i++) chunks.emplace_back(get_u32(q + 8 + 12 * i), get_u64(q + 12 + 12 * i));
    std::sort(chunks.begin(), chunks.end());
    cur_chunk = (size_t)-1;
    return GGCAT_GPU_OK;
}

bool Reader::get(uint32_t subset, std::vector<uint32_t> &out) {
    if (subset >= subsets_count || chunks.empty()) return false;
    size_t c = (size_t)(std::upper_bound(chunks.begin(), chunks.end(), std::make_pair(subset, UINT64_MAX)) -
                        chunks.begin());
    if (c == 0) return false;
    c--;
    if (c != cur_chunk || subset < cur_index) {
        size_t used = 0;
        const uint64_t off = chunks[c].second;
        if (off >= data.size() || !lz4_frame_decode(data.data() + off, data.size() - off, &used, chunk_raw))
            return false;
        cur_chunk = c;
        cur_index = chunks[c].first;
        cur_pos = 0;
    }
    const uint8_t *p = chunk_raw.data() + cur_pos, *end = chunk_raw.data() + chunk_raw.size();
    while (cur_index < subset) {
        if (!subset_decode(p, end, out)) return false;
        cur_index++;
    }
    if (!subset_decode(p, end, out)) return false;
    cur_index++;
    cur_pos = (size_t)(p - chunk_raw.data());
    return true;
}

}  // namespace cmap
}  // namespace ggcat

using namespace ggcat;

// GGCATInstance::get_colormap_file (crates/api/src/lib.rs:385-387): the graph path with its
// last extension replaced by "colors.dat" (Path::with_extension)
std::string ggcat_colormap_path(const std::string &graph) {
    const size_t slash = graph.find_last_of('/');
    const size_t name = slash == std::string::npos ? 0 : slash + 1;
    const size_t dot = graph.find_last_of('.');
    if (dot == std::string::npos || dot < name || dot == name) return graph + ".colors.dat";
    return graph.substr(0, dot) + ".colors.dat";
}

extern "C" int ggcat_gpu_colormap_file(const char *graph_file, char *out, uint64_t out_cap) {
    if (!graph_file || !out || out_cap == 0) return GGCAT_GPU_EINVAL;
    const std::string p = ggcat_colormap_path(graph_file);
    if (p.size() + 1 > out_cap) return GGCAT_GPU_ETOOLARGE;
    memcpy(out, p.c_str(), p.size() + 1);
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_write_colormap(const char *path, const char *const *color_names, uint64_t n_colors,
                                        const uint64_t *subset_off, const uint32_t *subset_colors,
                                        uint64_t n_subsets) {
    if (!path || (n_colors && !color_names) || (n_subsets && (!subset_off || !subset_colors)))
        return GGCAT_GPU_EINVAL;
    std::vector<std::string> names;
    for (uint64_t i = 0; i < n_colors; i++) names.emplace_back(color_names[i] ? color_names[i] : "");
    for (uint64_t s = 0; s < n_subsets; s++) {
        if (subset_off[s + 1] <= subset_off[s]) return GGCAT_GPU_EINVAL;  // empty subset
        for (uint64_t j = subset_off[s] + 1; j < subset_off[s + 1]; j++)
            if (subset_colors[j] <= subset_colors[j - 1]) return GGCAT_GPU_EINVAL;  // not strictly ascending
    }
    return cmap::write(path, names, n_subsets, [&](uint64_t s, std::vector<uint32_t> &out) {
        out.assign(subset_colors + subset_off[s], subset_colors + subset_off[s + 1]);
    });
}

extern "C" int ggcat_gpu_dump_colors(const char *colormap, char *h_names, uint64_t cap, uint64_t *names_bytes,
                                     uint64_t *n_colors) {
    if (!colormap) return GGCAT_GPU_EINVAL;
    cmap::Reader r;
    int rc = r.open(colormap, nullptr);
    if (rc) return rc;
    uint64_t need = 0;
    for (const auto &s : r.names) need += s.size() + 1;
    if (names_bytes) *names_bytes = need;
    if (n_colors) *n_colors = r.names.size();
    if (!h_names) return GGCAT_GPU_OK;
    if (cap < need) return GGCAT_GPU_ETOOLARGE;
    uint64_t o = 0;
    for (const auto &s : r.names) {
        memcpy(h_names + o, s.data(), s.size());
        h_names[o + s.size()] = '\0';
        o += s.size() + 1;
    }
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_colormap(const char *colormap, const uint32_t *subsets, uint64_t n_subsets,
                                        int single_thread_output_function, ggcat_gpu_colormap_fn fn, void *fn_ctx) {
    (void)single_thread_output_function;  // the subsets are decoded and reported on the calling thread
    if (!colormap || !fn || (n_subsets && !subsets)) return GGCAT_GPU_EINVAL;
    cmap::Reader r;
    int rc = r.open(colormap, nullptr);
    if (rc) return rc;
    std::vector<uint32_t> q(subsets, subsets + n_subsets), cols;
    std::sort(q.begin(), q.end());
    q.erase(std::unique(q.begin(), q.end()), q.end());
    for (uint32_t s : q) {
        if (!r.get(s, cols)) return GGCAT_GPU_EINVAL;  // not a subset of this colormap
        fn(fn_ctx, s, cols.data(), cols.size());
    }
    return GGCAT_GPU_OK;
}
