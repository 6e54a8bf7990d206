// Graph output on the host (graph_out.cpp): maximal-unitig links and the FASTA / GFA writers.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace ggcat {

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

}  // namespace ggcat
