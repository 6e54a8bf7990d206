// Graph output on the host: the maximal-unitig links and the FASTA / GFA writers.
//   build_maximal_unitigs_links (crates/assembler_pipeline/src/maximal_unitig_links.rs:55-417):
//     every unitig gives an entry for its first (k-1)-mer (Beginning, direction = is_forward)
//     and its last (k-1)-mer (Ending, direction = !is_forward, overlap start = len - k + 1),
//     plus the opposite direction when that (k-1)-mer is its own reverse complement; entries
//     with the same canonical (k-1)-mer and different directions link, with flags
//     flip_current = (this entry is a Beginning), flip_other = (the other is an Ending); the
//     links of an entry are ordered by the other unitig's index.  A unitig keeps one link list
//     per end (mappings_loader.rs:56-72: the list's flip_current picks the slot).  Grouping
//     by the exact canonical (k-1)-mer gives the links of every hash family the reference
//     uses (the direction of a (k-1)-mer and of its reverse complement are always opposite).
//   FASTA (sequence_output/src/structured_sequences/fasta.rs:153-200): ">{i} LN:i:{len}",
//     then " L:{+|-}:{j}:{+|-}" per link, end list first (maximal_unitig_index.rs:301-321).
//   GFA (gfa.rs:167-252, maximal_unitig_index.rs:323-372): v1 "S\t{i}\t{seq}\tLN:i:{len}" and
//     "L\t{i}\t{+|-}\t{j}\t{+|-}\t{k-1}M"; v2 "S\t{i}\t{len}\t{seq}" and
//     "E\t*\t{i}{+|-}\t{j}{+|-}\t{b1}\t{e1}[$]\t{b2}\t{e2}[$]".
// One choice is ours: for a (k-1)-mer that is its own reverse complement the reference
// writes two link lists for the same end and keeps whichever is read last (thread order);
// this keeps the list of the is_forward entry when it is not empty.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "graph_out.h"
#include "ggcat_gb300.h"
#include "input.h"

namespace ggcat {
namespace {

struct EndEntry {
    Key256 key;        // canonical (k-1)-mer, 2 bits per base
    uint64_t unitig;
    uint64_t overlap;  // start of the (k-1)-mer in the unitig
    uint8_t ending;    // 0 Beginning, 1 Ending
    uint8_t dir;
    uint8_t primary;   // 0 for the extra entry of a self-reverse-complement (k-1)-mer
};

}  // namespace

int unitig_links(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                 std::vector<UnitigLink> &links, std::vector<uint64_t> &list_off, std::string &err) {
    links.clear();
    list_off.assign(2 * n + 1, 0);
    if (k < 2 || k > 127) return err = "unitig links support 2 <= k <= 127", GGCAT_GPU_EUNSUPPORTED;
    const int w = k - 1;
    std::vector<EndEntry> ent;
    ent.reserve(4 * n);
    for (uint64_t i = 0; i < n; i++) {
        if (len[i] < (uint64_t)k) return err = "unitig shorter than k", GGCAT_GPU_EINVAL;
        const uint8_t *s = bases + off[i];
        Key256 f, r;
        if (!pack_bases(s, w, f, r)) return err = "unitig with a non-ACGT base", GGCAT_GPU_EINVAL;
        const Key256 kb = f < r ? f : r;
        const uint8_t fwd_b = f < r;
        ent.push_back({kb, i, 0, 0, fwd_b, 1});
        if (f == r) ent.push_back({kb, i, 0, 0, (uint8_t)!fwd_b, 0});
        const uint64_t ov = len[i] - (uint64_t)w;
        if (!pack_bases(s + ov, w, f, r)) return err = "unitig with a non-ACGT base", GGCAT_GPU_EINVAL;
        const Key256 ke = f < r ? f : r;
        const uint8_t fwd_e = f < r;
        ent.push_back({ke, i, ov, 1, (uint8_t)!fwd_e, 1});
        if (f == r) ent.push_back({ke, i, ov, 1, fwd_e, 0});
    }
    std::sort(ent.begin(), ent.end(), [](const EndEntry &a, const EndEntry &b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.unitig != b.unitig) return a.unitig < b.unitig;
        if (a.ending != b.ending) return a.ending < b.ending;
        return a.primary > b.primary;
    });
    // per (unitig, end): the chosen list as a range of `tmp`
    std::vector<UnitigLink> tmp;
    std::vector<std::pair<uint64_t, uint64_t>> slot(2 * n, {0, 0});
    std::vector<uint8_t> slot_primary(2 * n, 0);
    for (size_t a = 0; a < ent.size();) {
        size_t b = a + 1;
        while (b < ent.size() && ent[b].key == ent[a].key) b++;
        if (b - a > 1) {
            for (size_t x = a; x < b; x++) {
                const EndEntry &val = ent[x];
                const uint64_t start = tmp.size();
                for (size_t y = a; y < b; y++) {
                    const EndEntry &v = ent[y];
                    if (v.dir == val.dir) continue;
                    tmp.push_back({v.unitig, v.overlap, (uint8_t)((val.ending ? 0 : 1) | (v.ending ? 2 : 0))});
                }
                const uint64_t cnt = tmp.size() - start;
                if (!cnt) continue;
                // slot 2i: links from the end (flip_current = 0), 2i + 1: from the beginning
                const uint64_t sl = 2 * val.unitig + (val.ending ? 0 : 1);
                if (slot[sl].second == 0 || (val.primary && !slot_primary[sl])) {
                    slot[sl] = {start, cnt};
                    slot_primary[sl] = val.primary;
                }
            }
        }
        a = b;
    }
    for (uint64_t s = 0; s < 2 * n; s++) {
        list_off[s] = links.size();
        links.insert(links.end(), tmp.begin() + (long)slot[s].first, tmp.begin() + (long)(slot[s].first + slot[s].second));
    }
    list_off[2 * n] = links.size();
    return GGCAT_GPU_OK;
}

int write_graph(const char *unitigs_fasta, const char *output_file, int k, int with_links, int gfa_version,
                std::string &err) {
    if (gfa_version != 0 && gfa_version != 1 && gfa_version != 2)
        return err = "gfa_version must be 0 (FASTA), 1 or 2", GGCAT_GPU_EINVAL;
    std::vector<uint8_t> text;
    std::vector<uint64_t> off, len;
    int rc = read_sequences(unitigs_fasta, -1, text, &off, &len, err);
    if (rc) return rc;
    return write_graph_arrays(text.data(), off.data(), len.data(), off.size(), k, with_links, gfa_version, nullptr,
                              output_file, err);
}

int write_graph_arrays(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                       int with_links, int gfa_version, const HeaderExtra *extra, const char *output_file,
                       std::string &err) {
    if (gfa_version != 0 && gfa_version != 1 && gfa_version != 2)
        return err = "gfa_version must be 0 (FASTA), 1 or 2", GGCAT_GPU_EINVAL;
    std::vector<UnitigLink> links;
    std::vector<uint64_t> lo;
    if (with_links) {
        const int rc = unitig_links(bases, off, len, n, k, links, lo, err);
        if (rc) return rc;
    }
    FILE *f = fopen(output_file, "wb");
    if (!f) return err = std::string("cannot write ") + output_file, GGCAT_GPU_EIO;
    std::string line;
    for (uint64_t i = 0; i < n; i++) {
        const char *seq = reinterpret_cast<const char *>(bases + off[i]);
        const unsigned long long L = len[i];
        char buf[128];
        if (gfa_version == 0) {
            // ">id LN:i:len", then the colour runs, then the links (fasta.rs:183-211)
            snprintf(buf, sizeof buf, ">%llu LN:i:%llu", (unsigned long long)i, L);
            line = buf;
            if (extra) (*extra)(i, line);
            if (with_links)
                for (uint64_t j = lo[2 * i]; j < lo[2 * i + 2]; j++) {
                    snprintf(buf, sizeof buf, " L:%c:%llu:%c", (links[j].flags & 1) ? '-' : '+',
                             (unsigned long long)links[j].other, (links[j].flags & 2) ? '-' : '+');
                    line += buf;
                }
            line += '\n';
            line.append(seq, (size_t)L);
            line += '\n';
        } else {
            if (gfa_version == 1) {
                snprintf(buf, sizeof buf, "S\t%llu\t", (unsigned long long)i);
                line = buf;
                line.append(seq, (size_t)L);
                snprintf(buf, sizeof buf, "\tLN:i:%llu\n", L);
                line += buf;
            } else {
                snprintf(buf, sizeof buf, "S\t%llu\t%llu\t", (unsigned long long)i, L);
                line = buf;
                line.append(seq, (size_t)L);
                line += '\n';
            }
            if (with_links)
                for (uint64_t j = lo[2 * i]; j < lo[2 * i + 2]; j++) {
                    const UnitigLink &e = links[j];
                    const char c1 = (e.flags & 1) ? '-' : '+', c2 = (e.flags & 2) ? '-' : '+';
                    if (gfa_version == 1) {
                        snprintf(buf, sizeof buf, "L\t%llu\t%c\t%llu\t%c\t%dM\n", (unsigned long long)i, c1,
                                 (unsigned long long)e.other, c2, k - 1);
                    } else {
                        const bool cur_begin = e.flags & 1;
                        const unsigned long long b1 = cur_begin ? 0 : L - (unsigned long long)k + 1;
                        const unsigned long long e1 = cur_begin ? (unsigned long long)k - 1 : L;
                        const unsigned long long b2 = e.overlap, e2 = e.overlap + (unsigned long long)k - 1;
                        snprintf(buf, sizeof buf, "E\t*\t%llu%c\t%llu%c\t%llu\t%llu%s\t%llu\t%llu%s\n",
                                 (unsigned long long)i, c1, (unsigned long long)e.other, c2, b1, e1,
                                 cur_begin ? "" : "$", b2, e2, e.overlap > 0 ? "$" : "");
                    }
                    line += buf;
                }
        }
        if (fwrite(line.data(), 1, line.size(), f) != line.size()) {
            fclose(f);
            return err = std::string("cannot write ") + output_file, GGCAT_GPU_EIO;
        }
    }
    if (fclose(f) != 0) return err = std::string("cannot write ") + output_file, GGCAT_GPU_EIO;
    return GGCAT_GPU_OK;
}

}  // namespace ggcat

extern "C" int ggcat_gpu_unitig_links(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n,
                                      int k, uint64_t *list_off, uint64_t *other, uint64_t *overlap, uint8_t *flags,
                                      uint64_t cap, uint64_t *n_links) {
    if (n && (!bases || !off || !len)) return GGCAT_GPU_EINVAL;
    std::vector<ggcat::UnitigLink> links;
    std::vector<uint64_t> lo;
    std::string err;
    const int rc = ggcat::unitig_links(bases, off, len, n, k, links, lo, err);
    if (rc) return rc;
    if (n_links) *n_links = links.size();
    if (list_off) memcpy(list_off, lo.data(), lo.size() * sizeof(uint64_t));
    const uint64_t m = std::min<uint64_t>(cap, links.size());
    for (uint64_t i = 0; i < m; i++) {
        if (other) other[i] = links[i].other;
        if (overlap) overlap[i] = links[i].overlap;
        if (flags) flags[i] = links[i].flags;
    }
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_write_graph(const char *unitigs_fasta, const char *output_file, int k, int unitig_links,
                                     int gfa_version, char *err, uint64_t err_cap) {
    if (!unitigs_fasta || !output_file) return GGCAT_GPU_EINVAL;
    std::string e;
    const int rc = ggcat::write_graph(unitigs_fasta, output_file, k, unitig_links, gfa_version, e);
    if (err && err_cap) {
        const size_t m = std::min<size_t>(e.size(), err_cap - 1);
        memcpy(err, e.data(), m);
        err[m] = 0;
    }
    return rc;
}

int dump_colored_unitigs(const char *graph_input, int k, ggcat_gpu_dump_fn fn, void *fn_ctx);  // capi.cu

extern "C" int ggcat_gpu_dump_unitigs(const char *graph_input, int k, int colors, ggcat_gpu_dump_fn fn, void *fn_ctx) {
    if (!graph_input || !fn || k < 2) return GGCAT_GPU_EINVAL;
    if (colors) return dump_colored_unitigs(graph_input, k, fn, fn_ctx);
    std::vector<uint8_t> text;
    std::vector<uint64_t> off, len;
    std::string err;
    const int rc = ggcat::read_sequences(graph_input, k - 1, text, &off, &len, err);
    if (rc) return rc;
    for (size_t i = 0; i < off.size(); i++) fn(fn_ctx, text.data() + off[i], len[i], nullptr, 0, 0);
    return GGCAT_GPU_OK;
}

