// Spectrum-preserving string sets over the final unitigs, on the host: eulertigs, pathtigs and
// greedy matchtigs (ExtraElaboration::{Eulertigs, Pathtigs, GreedyMatchtigs},
// crates/api/src/lib.rs:101-116; compute_matchtigs_thread,
// crates/assembler_pipeline/src/compute_matchtigs.rs:380-537, which hands the unitig graph to
// the matchtigs crate 2.1.x: EulertigAlgorithm, PathtigAlgorithm, GreedytigAlgorithm).  The
// crate is a third-party dependency; this file restates the published algorithms (Schmidt and
// Alanko, "Eulertigs: minimum plain text representation of k-mer sets without repetitions in
// linear time", 2023; Schmidt, Khan, Alanko, Pibiri, Tomescu, "Matchtigs: minimum plain text
// representation of k-mer sets", 2023) on our own graph structures.
//
// Graph.  A binode is a canonical (k-1)-mer; every unitig joins the binodes of its first and
// last (k-1)-mer.  A unitig end has a type: 0 when its (k-1)-mer, read into the unitig, is the
// canonical one, 1 otherwise.  A walk passing a binode leaves a unitig through one end and
// enters the next through another end of the other type (same (k-1)-mer, same orientation);
// at a binode whose (k-1)-mer is its own reverse complement any two ends pair.  A string is a
// walk: its first unitig in full, every later one from offset k-1.
//
// Eulertigs: every binode is balanced with dummy edges to a virtual binode (|#type 0 - #type 1|
// of them, one for an odd palindromic binode), Hierholzer's algorithm runs with the type
// constraint, and the circuits are cut at the dummy edges: max(1, sum of imbalances / 2)
// strings per connected component, each k-mer once — the minimum.
// Pathtigs: a greedy walk cover (each unused unitig extended forwards, then backwards, along
// unused unitigs), each k-mer once.
// Greedy matchtigs: the eulertig construction where two surplus ends are first joined, cheapest
// first, by a shortest walk of at most k-2 k-mers (Dijkstra over (binode, type) states); a join
// of w k-mers repeats them and costs w characters instead of the k-1 of a new string, and is
// written by appending the next unitig from offset k-1-w (compute_matchtigs.rs:490-515).
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <queue>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "ggcat_gb300.h"
#include "graph_out.h"

namespace ggcat {
namespace {

constexpr uint8_t kAny = 2;  // the "need" of a palindromic binode (and of the virtual one)

// Host threads: the output does not depend on their number (fixed partitions, candidates and
// strings ordered before use).
int tig_threads() { return (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency())); }

// f(begin, end, thread) over [0, n) in at most T contiguous ranges of at least `grain` items
template <class F>
void par_for(uint64_t n, int T, uint64_t grain, F f) {
    const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)T, n / std::max<uint64_t>(grain, 1)));
    if (parts <= 1) {
        if (n) f(0, n, 0);
        return;
    }
    const uint64_t per = (n + parts - 1) / parts;
    std::vector<std::thread> th;
    for (uint64_t t = 0; t < parts; t++) {
        const uint64_t a = std::min(n, per * t), b = std::min(n, a + per);
        if (a < b) th.emplace_back(f, a, b, (int)t);
    }
    for (auto &x : th) x.join();
}

struct TigGraph {
    uint64_t n = 0;              // real unitigs; edges >= n are dummies
    uint32_t n_bins = 0;         // real binodes; the virtual binode is n_bins
    std::vector<uint32_t> bin;   // per end (2e start, 2e + 1 end of edge e)
    std::vector<uint8_t> type;   // per end
    std::vector<uint8_t> pal;    // per binode (+ virtual)
    std::vector<int64_t> weight;  // per dummy edge: -1 virtual, else the join's k-mers
    std::vector<uint64_t> kmers;  // per real unitig
    // unused ends by (binode, type) (palindromic binodes: type 0 only), popped from the back
    std::vector<uint64_t> pool_off, pool_top, pool;
    std::vector<uint8_t> used;   // per edge
    // per end, packed by build_pools for the walks (one random access per step): its binode,
    // the need after leaving a unitig through it and the need it departs with
    struct EndInfo {
        uint32_t bin;
        uint8_t exit_need, dep_need;
    };
    std::vector<EndInfo> info;

    uint64_t edges() const { return bin.size() / 2; }
    uint8_t need_after_exit(uint64_t e) const { return info[e].exit_need; }
    uint8_t need_of_departure(uint64_t f) const { return info[f].dep_need; }

    void add_dummy(uint32_t b1, uint8_t t1, uint32_t b2, uint8_t t2, int64_t w) {
        bin.push_back(b1);
        type.push_back(t1);
        bin.push_back(b2);
        type.push_back(t2);
        weight.push_back(w);
    }

    void build_pools() {
        const uint64_t ne = bin.size();
        const uint64_t slots = 2ull * (n_bins + 1);
        pool_off.assign(slots + 1, 0);
        for (uint64_t e = 0; e < ne; e++) pool_off[2ull * bin[e] + (pal[bin[e]] ? 0 : type[e]) + 1]++;
        for (uint64_t s = 0; s < slots; s++) pool_off[s + 1] += pool_off[s];
        pool.assign(ne, 0);
        pool_top.assign(slots, 0);
        std::vector<uint64_t> cur(pool_off.begin(), pool_off.end() - 1);
        // ends pushed in decreasing order so that pops come out in increasing order
        for (uint64_t e = ne; e-- > 0;) pool[cur[2ull * bin[e] + (pal[bin[e]] ? 0 : type[e])]++] = e;
        for (uint64_t s = 0; s < slots; s++) pool_top[s] = pool_off[s + 1];
        used.assign(edges(), 0);
        info.resize(ne);
        for (uint64_t e = 0; e < ne; e++) {
            const bool p = pal[bin[e]];
            info[e] = {bin[e], p ? kAny : (uint8_t)(1u - type[e]), p ? kAny : type[e]};
        }
    }

    // an unused end at binode b of type `need` (any type at a palindromic binode), or -1
    int64_t take(uint32_t b, uint8_t need) {
        const uint64_t s = 2ull * b + (need == kAny ? 0 : need);
        uint64_t &top = pool_top[s];
        while (top > pool_off[s]) {
            const uint64_t f = pool[top - 1];
            if (!used[f >> 1]) return (int64_t)f;
            top--;
        }
        return -1;
    }
};

// binodes and end types of the unitigs; false on a unitig shorter than k or a non-ACGT base.
// Ends are packed on threads, split into kParts partitions by a hash of their (k-1)-mer and
// numbered partition by partition (each sorted on its own thread).
bool build_graph(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k, TigGraph &g,
                 std::string &err) {
    constexpr uint32_t kParts = 64;
    const int w = k - 1;
    const int T = tig_threads();
    g.n = n;
    g.bin.assign(2 * n, 0);
    g.type.assign(2 * n, 0);
    g.kmers.assign(n, 0);
    std::vector<Key256> key(2 * n);
    std::vector<uint8_t> end_pal(2 * n, 0), part(2 * n, 0);
    std::atomic<int> bad{0};  // 1 short, 2 non-ACGT
    par_for(n, T, 4096, [&](uint64_t u0, uint64_t u1, int) {
        for (uint64_t u = u0; u < u1; u++) {
            if (len[u] < (uint64_t)k) {
                bad.store(1);
                return;
            }
            g.kmers[u] = len[u] - (uint64_t)k + 1;
            const uint8_t *s = bases + off[u];
            for (uint64_t i = 0; i < len[u]; i++)
                if (base_code(s[i]) < 0) {
                    bad.store(2);
                    return;
                }
            Key256 f, r;
            pack_bases(s, w, f, r);
            // start end: read into the unitig as its first (k-1)-mer
            key[2 * u] = f < r ? f : r;
            g.type[2 * u] = f < r || f == r ? 0 : 1;
            end_pal[2 * u] = f == r;
            pack_bases(s + len[u] - (uint64_t)w, w, f, r);
            // end end: read into the unitig as the reverse complement of its last (k-1)-mer
            key[2 * u + 1] = f < r ? f : r;
            g.type[2 * u + 1] = r < f || f == r ? 0 : 1;
            end_pal[2 * u + 1] = f == r;
            for (uint64_t e = 2 * u; e < 2 * u + 2; e++) {
                const uint64_t h = (uint64_t)key[e].lo ^ (uint64_t)(key[e].lo >> 64) * 0x9E3779B97F4A7C15ull ^
                                   (uint64_t)key[e].hi * 0xC2B2AE3D27D4EB4Full;
                part[e] = (uint8_t)((h * 0xD6E8FEB86659FD93ull) >> 58);  // top 6 bits: kParts = 64
            }
        }
    });
    if (bad.load()) return err = bad.load() == 1 ? "unitig shorter than k" : "unitig with a non-ACGT base", false;
    // ends grouped by partition, in increasing end order within each
    std::vector<uint64_t> pstart(kParts + 1, 0);
    for (uint64_t e = 0; e < 2 * n; e++) pstart[part[e] + 1]++;
    for (uint32_t p = 0; p < kParts; p++) pstart[p + 1] += pstart[p];
    std::vector<uint64_t> order(2 * n);
    {
        std::vector<uint64_t> cur(pstart.begin(), pstart.end() - 1);
        for (uint64_t e = 0; e < 2 * n; e++) order[cur[part[e]]++] = e;
    }
    std::vector<uint32_t> local(2 * n, 0), pbins(kParts, 0);
    std::atomic<uint32_t> next{0};
    auto number = [&](uint64_t, uint64_t, int) {
        for (uint32_t p; (p = next.fetch_add(1)) < kParts;) {
            auto *first = order.data() + pstart[p], *last = order.data() + pstart[p + 1];
            std::sort(first, last, [&](uint64_t x, uint64_t y) { return key[x] != key[y] ? key[x] < key[y] : x < y; });
            uint32_t nb = 0;
            for (auto *q = first; q < last; q++) {
                if (q > first && key[*q] != key[*(q - 1)]) nb++;
                local[*q] = nb;
            }
            pbins[p] = first < last ? nb + 1 : 0;
        }
    };
    par_for((uint64_t)T, T, 1, number);
    std::vector<uint64_t> pbase(kParts + 1, 0);
    for (uint32_t p = 0; p < kParts; p++) pbase[p + 1] = pbase[p] + pbins[p];
    if (pbase[kParts] >= 0xffffffffull) return err = "too many distinct (k-1)-mers", false;
    g.n_bins = (uint32_t)pbase[kParts];
    g.pal.assign(g.n_bins + 1, 0);
    par_for(2 * n, T, 1 << 16, [&](uint64_t e0, uint64_t e1, int) {
        for (uint64_t e = e0; e < e1; e++) g.bin[e] = (uint32_t)pbase[part[e]] + local[e];
    });
    for (uint64_t e = 0; e < 2 * n; e++) g.pal[g.bin[e]] = end_pal[e];
    g.pal[g.n_bins] = 1;  // the virtual binode pairs any two dummy ends
    return true;
}

// per binode: surplus ends (unmatched in any walk cover) and their type (kAny when palindromic)
void surplus(const TigGraph &g, std::vector<uint64_t> &cnt, std::vector<uint8_t> &ty) {
    std::vector<uint64_t> c0(g.n_bins, 0), c1(g.n_bins, 0);
    for (uint64_t e = 0; e < 2 * g.n; e++) (g.type[e] ? c1 : c0)[g.bin[e]]++;
    cnt.assign(g.n_bins, 0);
    ty.assign(g.n_bins, 0);
    for (uint32_t b = 0; b < g.n_bins; b++) {
        if (g.pal[b]) {
            cnt[b] = (c0[b] + c1[b]) & 1;
            ty[b] = kAny;
        } else if (c0[b] != c1[b]) {
            cnt[b] = c0[b] > c1[b] ? c0[b] - c1[b] : c1[b] - c0[b];
            ty[b] = c0[b] > c1[b] ? 0 : 1;
        }
    }
}

// the end type a dummy needs at binode b to pair with a surplus end of type t there
inline uint8_t dummy_type(uint8_t t) { return t == kAny ? 0 : (uint8_t)(1u - t); }

// Hierholzer with the type constraint from state (b, need); appends the circuit's entered ends
void circuit(TigGraph &g, uint32_t b0, uint8_t need0, std::vector<uint64_t> &out) {
    std::vector<uint64_t> stack, rev;
    uint32_t b = b0;
    uint8_t need = need0;
    for (;;) {
        const int64_t f = g.take(b, need);
        if (f >= 0) {
            g.used[(uint64_t)f >> 1] = 1;
            stack.push_back((uint64_t)f);
            const auto &xi = g.info[(uint64_t)f ^ 1u];
            b = xi.bin;
            need = xi.exit_need;
            continue;
        }
        if (stack.empty()) break;
        const uint64_t top = stack.back();
        stack.pop_back();
        rev.push_back(top);
        b = g.info[top].bin;
        need = g.info[top].dep_need;
    }
    out.insert(out.end(), rev.rbegin(), rev.rend());
}

// the strings, as walks: entered ends of real unitigs and of joins, walk w in
// ends[end[w - 1], end[w])
struct Walks {
    std::vector<uint64_t> ends, end;
    void add(const uint64_t *f, size_t n) {
        if (!n) return;
        ends.insert(ends.end(), f, f + n);
        end.push_back(ends.size());
    }
};

struct TigOut {
    std::vector<uint8_t> bases;
    std::vector<uint64_t> off, len;
    std::vector<uint64_t> walk, walk_off;  // per string: the entered ends of its real unitigs
};

// every walk spelled (first unitig in full, later ones from offset k-1, or k-1-w after a join
// of w k-mers), sizes first, then the strings on threads
void materialize(const TigGraph &g, const uint8_t *bases, const uint64_t *off, const uint64_t *len, int k,
                 const Walks &W, TigOut &o) {
    const uint64_t nw = W.end.size();
    const int T = tig_threads();
    std::vector<uint64_t> size(nw, 0), reals(nw, 0);
    auto range = [&](uint64_t w) { return std::make_pair(w ? W.end[w - 1] : 0, W.end[w]); };
    par_for(nw, T, 1024, [&](uint64_t w0, uint64_t w1, int) {
        for (uint64_t w = w0; w < w1; w++) {
            const auto [a, b] = range(w);
            int64_t join = 0;
            bool first = true;
            for (uint64_t i = a; i < b; i++) {
                const uint64_t e = W.ends[i] >> 1;
                if (e >= g.n) {
                    join = g.weight[e - g.n];
                    continue;
                }
                size[w] += len[e] - (first ? 0 : (uint64_t)(k - 1 - join));
                reals[w]++;
                first = false;
                join = 0;
            }
        }
    });
    o.off.assign(nw, 0);
    o.len.assign(size.begin(), size.end());
    o.walk_off.assign(nw, 0);
    uint64_t total = 0, treal = 0;
    for (uint64_t w = 0; w < nw; w++) {
        o.off[w] = total;
        total += size[w];
        treal += reals[w];
        o.walk_off[w] = treal;
    }
    o.bases.resize(total);
    o.walk.resize(treal);
    par_for(nw, T, 1024, [&](uint64_t w0, uint64_t w1, int) {
        for (uint64_t w = w0; w < w1; w++) {
            const auto [a, b] = range(w);
            uint8_t *dst = o.bases.data() + o.off[w];
            uint64_t *rw = o.walk.data() + (o.walk_off[w] - reals[w]);
            int64_t join = 0;
            bool first = true;
            for (uint64_t i = a; i < b; i++) {
                const uint64_t f = W.ends[i], e = f >> 1;
                if (e >= g.n) {
                    join = g.weight[e - g.n];
                    continue;
                }
                const uint8_t *src = bases + off[e];
                const uint64_t L = len[e];
                const uint64_t from = first ? 0 : (uint64_t)(k - 1 - join);
                *rw++ = f;
                if (!(f & 1)) {
                    memcpy(dst, src + from, L - from);
                    dst += L - from;
                } else {
                    for (uint64_t j = from; j < L; j++) {
                        const uint8_t c = src[L - 1 - j];
                        *dst++ = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
                    }
                }
                first = false;
                join = 0;
            }
        }
    });
}

// circuits of the balanced graph cut at the virtual dummies; a closed circuit without them is
// one string, opened after a join when it holds one (that join's k-mers are then not repeated)
void emit_circuits(TigGraph &g, Walks &W) {
    g.build_pools();
    std::vector<uint64_t> c;
    auto is_virtual = [&](uint64_t f) { return (f >> 1) >= g.n && g.weight[(f >> 1) - g.n] < 0; };
    auto is_join = [&](uint64_t f) { return (f >> 1) >= g.n && g.weight[(f >> 1) - g.n] >= 0; };
    if (g.edges() > g.n) {
        c.clear();
        circuit(g, g.n_bins, kAny, c);
        size_t a = 0;
        for (size_t i = 0; i <= c.size(); i++) {
            if (i == c.size() || is_virtual(c[i])) {
                W.add(c.data() + a, i - a);
                a = i + 1;
            }
        }
    }
    for (uint64_t u = 0; u < g.n; u++) {
        if (g.used[u]) continue;
        c.clear();
        circuit(g, g.bin[2 * u], g.need_of_departure(2 * u), c);
        size_t j = 0;
        while (j < c.size() && !is_join(c[j])) j++;
        if (j < c.size()) std::rotate(c.begin(), c.begin() + (long)j + 1, c.end());  // the join now ends it
        if (!c.empty() && is_join(c.back())) c.pop_back();
        W.add(c.data(), c.size());
    }
}

void eulertigs(TigGraph &g, Walks &W) {
    std::vector<uint64_t> cnt;
    std::vector<uint8_t> ty;
    surplus(g, cnt, ty);
    for (uint32_t b = 0; b < g.n_bins; b++)
        for (uint64_t i = 0; i < cnt[b]; i++) g.add_dummy(b, dummy_type(ty[b]), g.n_bins, 0, -1);
    emit_circuits(g, W);
}

void pathtigs(TigGraph &g, Walks &W) {
    g.build_pools();
    std::vector<uint64_t> fwd, bwd, walk;
    for (uint64_t u = 0; u < g.n; u++) {
        if (g.used[u]) continue;
        g.used[u] = 1;
        // a unitig that leaves through end x is followed by one entered through an unused end of
        // the other type at x's binode; extending backwards is the same step from the start end
        auto extend = [&](uint64_t x, std::vector<uint64_t> &chain) {
            chain.clear();
            for (;;) {
                const int64_t f = g.take(g.info[x].bin, g.info[x].exit_need);
                if (f < 0) break;
                g.used[(uint64_t)f >> 1] = 1;
                chain.push_back((uint64_t)f);
                x = (uint64_t)f ^ 1u;
            }
        };
        extend(2 * u + 1, fwd);
        extend(2 * u, bwd);
        walk.clear();
        for (size_t i = bwd.size(); i-- > 0;) walk.push_back(bwd[i] ^ 1u);  // entered through the other end
        walk.push_back(2 * u);
        walk.insert(walk.end(), fwd.begin(), fwd.end());
        W.add(walk.data(), walk.size());
    }
}

void greedy_matchtigs(TigGraph &g, int k, Walks &W) {
    std::vector<uint64_t> cnt;
    std::vector<uint8_t> ty;
    surplus(g, cnt, ty);
    g.build_pools();  // adjacency for the searches (nothing is used yet)
    const int64_t max_cost = k - 2;
    // states (binode, need): 2b + need, a palindromic binode only 2b
    auto sid = [&](uint32_t b, uint8_t need) { return 2ull * b + (need == kAny ? 0 : need); };
    struct Cand {
        int64_t cost;
        uint32_t b1, b2;
    };
    // one bounded search per surplus binode, on threads (16-bit distances: costs stay below
    // k - 1 <= 126; at most 2 GB of distance arrays in all), candidates merged then sorted
    std::vector<uint32_t> sources;
    for (uint32_t b1 = 0; b1 < g.n_bins && max_cost > 0; b1++)
        if (cnt[b1]) sources.push_back(b1);
    const uint64_t dist_bytes = 4ull * (g.n_bins + 1);
    const int T = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)tig_threads(), (2ull << 30) / dist_bytes));
    std::vector<std::vector<Cand>> tcand(T);
    std::atomic<uint64_t> next{0};
    // costs are whole k-mer counts >= 1 per unitig and at most max_cost: a bucket queue (Dial)
    auto search = [&](uint64_t, uint64_t, int t) {
        std::vector<int16_t> dist(2ull * (g.n_bins + 1), -1);
        std::vector<uint64_t> touched;
        std::vector<std::vector<uint64_t>> bq((size_t)max_cost + 1);
        std::vector<Cand> &cand = tcand[t];
        for (uint64_t i0; (i0 = next.fetch_add(64)) < sources.size();) {
            for (uint64_t i = i0; i < std::min<uint64_t>(sources.size(), i0 + 64); i++) {
                const uint32_t b1 = sources[i];
                // leave b1 as the walk ending at one of its surplus ends would: through an end of
                // the other type (any type at a palindromic binode)
                const uint8_t n0 = ty[b1] == kAny ? kAny : (uint8_t)(1u - ty[b1]);
                const uint64_t s0 = sid(b1, n0);
                dist[s0] = 0;
                touched.push_back(s0);
                bq[0].push_back(s0);
                for (int64_t d = 0; d <= max_cost; d++) {
                    // a bucket only receives states of larger cost while it is read (every
                    // step adds at least one k-mer), so it is read by index
                    for (size_t qi = 0; qi < bq[(size_t)d].size(); qi++) {
                        const uint64_t st = bq[(size_t)d][qi];
                        if (dist[st] != d) continue;
                        const uint32_t b = (uint32_t)(st >> 1);
                        // a surplus end at b can start the next walk when the state's need is its type
                        if (d > 0 && cnt[b] && (ty[b] == kAny || (uint8_t)(st & 1) == ty[b]))
                            cand.push_back({d, b1, b});
                        for (uint64_t p = g.pool_off[st]; p < g.pool_off[st + 1]; p++) {
                            const uint64_t f = g.pool[p];
                            const uint64_t x = f ^ 1u;
                            const int64_t nd = d + (int64_t)g.kmers[f >> 1];
                            if (nd > max_cost) continue;
                            const uint64_t tt = sid(g.info[x].bin, g.info[x].exit_need);
                            if (dist[tt] < 0 || nd < dist[tt]) {
                                if (dist[tt] < 0) touched.push_back(tt);
                                dist[tt] = (int16_t)nd;
                                bq[(size_t)nd].push_back(tt);
                            }
                        }
                    }
                    bq[(size_t)d].clear();
                }
                for (const uint64_t tt : touched) dist[tt] = -1;
                touched.clear();
            }
        }
    };
    par_for((uint64_t)T, T, 1, search);
    std::vector<Cand> cand;
    for (auto &v : tcand) cand.insert(cand.end(), v.begin(), v.end());
    std::sort(cand.begin(), cand.end(), [](const Cand &a, const Cand &b) {
        if (a.cost != b.cost) return a.cost < b.cost;
        if (a.b1 != b.b1) return a.b1 < b.b1;
        return a.b2 < b.b2;
    });
    std::vector<uint64_t> rem = cnt;
    for (const Cand &c : cand) {
        if (c.b1 == c.b2 ? rem[c.b1] < 2 : (!rem[c.b1] || !rem[c.b2])) continue;
        rem[c.b1]--;
        rem[c.b2]--;
        g.add_dummy(c.b1, dummy_type(ty[c.b1]), c.b2, dummy_type(ty[c.b2]), c.cost);
    }
    for (uint32_t b = 0; b < g.n_bins; b++)
        for (uint64_t i = 0; i < rem[b]; i++) g.add_dummy(b, dummy_type(ty[b]), g.n_bins, 0, -1);
    emit_circuits(g, W);
}

}  // namespace

// mode: GGCAT_GPU_TIGS_GREEDY_MATCHTIGS / _EULERTIGS / _PATHTIGS (the extra_elab numbers)
int compute_tigs(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k, int mode,
                 std::vector<uint8_t> &out_bases, std::vector<uint64_t> &out_off, std::vector<uint64_t> &out_len,
                 std::string &err, std::vector<uint64_t> *walk, std::vector<uint64_t> *walk_end) {
    out_bases.clear();
    out_off.clear();
    out_len.clear();
    if (k < 3 || k > 127) return err = "tigs support 3 <= k <= 127", GGCAT_GPU_EUNSUPPORTED;
    if (mode != GGCAT_GPU_TIGS_GREEDY_MATCHTIGS && mode != GGCAT_GPU_TIGS_EULERTIGS && mode != GGCAT_GPU_TIGS_PATHTIGS)
        return err = "unknown tig mode", GGCAT_GPU_EINVAL;
    TigGraph g;
    if (!build_graph(bases, off, len, n, k, g, err)) return GGCAT_GPU_EINVAL;
    Walks W;
    if (mode == GGCAT_GPU_TIGS_EULERTIGS)
        eulertigs(g, W);
    else if (mode == GGCAT_GPU_TIGS_PATHTIGS)
        pathtigs(g, W);
    else
        greedy_matchtigs(g, k, W);
    TigOut o;
    materialize(g, bases, off, len, k, W, o);
    out_bases.swap(o.bases);
    out_off.swap(o.off);
    out_len.swap(o.len);
    if (walk) walk->swap(o.walk);
    if (walk_end) walk_end->swap(o.walk_off);
    return GGCAT_GPU_OK;
}

}  // namespace ggcat

extern "C" int ggcat_gpu_compute_tigs(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                                      int mode, uint8_t *out_bases, uint64_t bases_cap, uint64_t *out_off,
                                      uint64_t *out_len, uint64_t n_cap, uint64_t *n_out, uint64_t *bases_out) {
    if ((n && (!bases || !off || !len)) || !n_out || !bases_out) return GGCAT_GPU_EINVAL;
    std::vector<uint8_t> b;
    std::vector<uint64_t> o, l;
    std::string err;
    const int rc = ggcat::compute_tigs(bases, off, len, n, k, mode, b, o, l, err);
    if (rc) return rc;
    *n_out = o.size();
    *bases_out = b.size();
    if (!out_bases || !out_off || !out_len) return GGCAT_GPU_OK;  // sizes only
    if (bases_cap < b.size() || n_cap < o.size()) return GGCAT_GPU_EINVAL;
    if (!b.empty()) memcpy(out_bases, b.data(), b.size());
    if (!o.empty()) {
        memcpy(out_off, o.data(), o.size() * sizeof(uint64_t));
        memcpy(out_len, l.data(), l.size() * sizeof(uint64_t));
    }
    return GGCAT_GPU_OK;
}
