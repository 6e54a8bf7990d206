// Graph output on the host (graph_out.cpp): maximal-unitig links and the FASTA / GFA writers.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace ggcat {

// a (k-1)-mer of up to 126 bases as a 256-bit integer hi * 2^128 + lo
struct Key256 {
    unsigned __int128 hi = 0, lo = 0;
};
inline bool operator<(const Key256 &a, const Key256 &b) { return a.hi != b.hi ? a.hi < b.hi : a.lo < b.lo; }
inline bool operator==(const Key256 &a, const Key256 &b) { return a.hi == b.hi && a.lo == b.lo; }
inline bool operator!=(const Key256 &a, const Key256 &b) { return !(a == b); }

inline int base_code(uint8_t c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

// forward and reverse-complement packing of s[0, n), n <= 126, base i at bits 2(n-1-i)
// (lexicographic order of the integers = order of the strings); false on a non-ACGT byte
inline bool pack_bases(const uint8_t *s, int n, Key256 &fw, Key256 &rc) {
    using u128 = unsigned __int128;
    fw = rc = Key256{};
    for (int i = 0; i < n; i++) {
        const int c = base_code(s[i]);
        if (c < 0) return false;
        fw.hi = (fw.hi << 2) | (fw.lo >> 126);
        fw.lo = (fw.lo << 2) | (u128)c;
        if (2 * i < 128)
            rc.lo |= (u128)(3 - c) << (2 * i);
        else
            rc.hi |= (u128)(3 - c) << (2 * i - 128);
    }
    return true;
}

struct UnitigLink {
    uint64_t other;    // index of the linked unitig
    uint64_t overlap;  // start of the shared (k-1)-mer in the other unitig
    uint8_t flags;     // bit 0 flip_current (link from this unitig's beginning), bit 1 flip_other
};

// links of n unitigs (bases[off[i], off[i] + len[i]), ACGT only, len >= k): list 2i holds the
// links from unitig i's end, list 2i + 1 those from its beginning, as
// links[list_off[l], list_off[l + 1])
int unitig_links(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                 std::vector<UnitigLink> &links, std::vector<uint64_t> &list_off, std::string &err);

// rewrites a FASTA of unitigs (">i ..." records in index order) as FASTA with link
// annotations (gfa_version 0, with_links 1) or as GFA v1 / v2 (links when with_links)
int write_graph(const char *unitigs_fasta, const char *output_file, int k, int with_links, int gfa_version,
                std::string &err);

// appends header content of unitig i after ">i LN:i:len" (the colour runs of a coloured graph)
typedef std::function<void(uint64_t, std::string &)> HeaderExtra;

// the same from unitigs in memory (bases[off[i], off[i] + len[i]), index order)
int write_graph_arrays(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                       int with_links, int gfa_version, const HeaderExtra *extra, const char *output_file,
                       std::string &err);

// tigs.cpp: eulertigs / pathtigs / greedy matchtigs of the unitigs (mode = GGCAT_GPU_TIGS_*);
// with walk / walk_end, string i's unitigs in order as the ends they are entered through
// (2u: unitig u forwards, 2u + 1: reverse complemented), walk[walk_end[i - 1], walk_end[i])
int compute_tigs(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k, int mode,
                 std::vector<uint8_t> &out_bases, std::vector<uint64_t> &out_off, std::vector<uint64_t> &out_len,
                 std::string &err, std::vector<uint64_t> *walk = nullptr, std::vector<uint64_t> *walk_end = nullptr);

}  // namespace ggcat
