// Per-sub-bucket k-mer merge on sm_103a.
//
// Replaces assembler_kmers_merge's per-bucket work (ParallelKmersMergeFinalExecutor::process_map,
// crates/assembler_kmers_merge/src/final_executor.rs:277-509, with the unitig extenders of
// crates/assembler_kmers_merge/src/unitigs_extender/{sorting,hashmap}.rs).  A merge unit is a
// run of sub-bins of one bucket, i.e. a union of whole minimizer groups, so the k-mer
// multiplicities (MapEntry counting with the both-ends halving rule,
// crates/structs/src/map_entry.rs:79-84) and the within-unit unitig extension follow the
// hash-map extender exactly (hashmap.rs:162-297, 361-601).
//
// Small units (<= kSmallSlots table slots) are processed one per CTA by a persistent kernel
// that keeps the unit's hash table in shared memory; large units use a global-memory table
// processed grid-wide by three kernels (insert, extend, cycles).
#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace ggcat {

template <typename KT>
struct Table {
    KT *keys;
    uint32_t *vals;  // count (30 bits) | flags << 30 (bit30: begin ignored, bit31: end ignored)
    uint8_t *vis;
    uint32_t cap;    // power of two
};

constexpr uint32_t kCountMask = (1u << 30) - 1;

// Multiplicative range reduction of the 32-bit hash onto [0, cap): any capacity (the W tier's
// shared table is not a power of two); for a power of two these are the top log2(cap) bits
template <typename KT>
__device__ __forceinline__ uint32_t slot_of(KT key, uint32_t cap) {
    return (uint32_t)(((uint64_t)KeyOps<KT>::hash(key) * cap) >> 32);
}

// next slot of a linear probe
__device__ __forceinline__ uint32_t next_slot(uint32_t s, uint32_t cap) { return s + 1 == cap ? 0u : s + 1; }

template <typename KT>
__device__ __forceinline__ int64_t tfind(const Table<KT> &t, KT key) {
    uint32_t s = slot_of(key, t.cap);
    for (uint32_t probe = 0; probe < t.cap; probe++) {
        const KT kk = t.keys[s];
        if (kk == key) return s;
        if (kk == KeyOps<KT>::empty()) return -1;
        s = next_slot(s, t.cap);
    }
    return -1;
}

// find-or-insert; created reports whether this call made the entry
template <typename KT>
__device__ __forceinline__ int64_t tinsert_created(const Table<KT> &t, KT key, unsigned *status, bool &created) {
    uint32_t s = slot_of(key, t.cap);
    created = false;
    for (uint32_t probe = 0; probe < t.cap; probe++) {
        const int r = slot_claim(&t.keys[s], key, created);
        if (r > 0) return s;
        if (r < 0) {
            atomicOr(status, kStatusWaitLimit);
            return -1;
        }
        s = next_slot(s, t.cap);
    }
    atomicOr(status, kStatusTableFull);
    return -1;
}

template <typename KT>
__device__ __forceinline__ int64_t tinsert(const Table<KT> &t, KT key, unsigned *status) {
    bool created;
    return tinsert_created(t, key, status, created);
}

// Shared-memory forms of the table operations (explicit state space: the table pointers reach
// the helpers through a struct, so the shared window is stated rather than inferred).
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t lds_u64(uint32_t a) {
    uint64_t v;
    asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t cas_shared_u64(uint32_t a, uint64_t cmp, uint64_t val) {
    uint64_t o;
    asm volatile("atom.shared.cas.b64 %0, [%1], %2, %3;" : "=l"(o) : "r"(a), "l"(cmp), "l"(val) : "memory");
    return o;
}
__device__ __forceinline__ uint32_t cas_shared_u32(uint32_t a, uint32_t cmp, uint32_t val) {
    uint32_t o;
    asm volatile("atom.shared.cas.b32 %0, [%1], %2, %3;" : "=r"(o) : "r"(a), "r"(cmp), "r"(val) : "memory");
    return o;
}
__device__ __forceinline__ void red_shared_add_u32(uint32_t a, uint32_t x) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(a), "r"(x) : "memory");
}
__device__ __forceinline__ void red_shared_or_b32(uint32_t a, uint32_t x) {
    asm volatile("red.shared.or.b32 [%0], %1;" ::"r"(a), "r"(x) : "memory");
}

// tinsert on a shared-memory table of u64 keys; created reports whether this call made the entry
__device__ __forceinline__ int64_t tinsert_shared(const Table<uint64_t> &t, uint64_t key, unsigned *status,
                                                  bool &created) {
    uint32_t s = slot_of(key, t.cap);
    const uint32_t kb = smem_addr(t.keys);
    created = false;
    for (uint32_t probe = 0; probe < t.cap; probe++) {
        const uint64_t kk = lds_u64(kb + 8u * s);
        if (kk == key) return s;
        if (kk == ~0ull) {
            const uint64_t old = cas_shared_u64(kb + 8u * s, ~0ull, key);
            if (old == ~0ull) {
                created = true;
                return s;
            }
            if (old == key) return s;
        }
        s = next_slot(s, t.cap);
    }
    atomicOr(status, kStatusTableFull);
    return -1;
}

// MapEntry::get_kmer_multiplicity (map_entry.rs:79-84): halve when both ends were ignored.
__device__ __forceinline__ uint32_t val_mult(uint32_t v) {
    uint32_t c = v & kCountMask;
    return (v >> 30) == 3u ? (c >> 1) : c;
}

// The k-mer graph of one unit's table.  Canonical builds key a k-mer and its reverse
// complement by the smaller of the two and walk both orientations; forward-only builds
// (fwd = 1, the forward seq-hash / Rabin-Karp families) key and walk k-mers as read.
template <typename KT>
struct Graph {
    Table<KT> t;
    int k;
    uint32_t min_mult;
    int fwd;

    __device__ __forceinline__ KT rc(KT v) const { return KeyOps<KT>::rc(v, k); }
    // even k: a k-mer equal to its reverse complement; a walk starts at it and a walk that
    // enters it stops there (its successor is the mirror of where the walk came from)
    __device__ __forceinline__ bool pal(KT v) const { return !fwd && v == rc(v); }
    __device__ __forceinline__ KT canon(KT v) const {
        if (fwd) return v;
        const KT r = rc(v);
        return v < r ? v : r;
    }
    // slot of an oriented k-mer if present and surviving, else -1
    __device__ __forceinline__ int64_t alive(KT v) const {
        int64_t s = tfind(t, canon(v));
        if (s < 0) return -1;
        return val_mult(t.vals[s]) >= min_mult ? s : -1;
    }
    // surviving successors of oriented v; *only receives the last one found
    __device__ __forceinline__ int succ(KT v, KT &only) const {
        int d = 0;
        const KT base = v >> 2;
#pragma unroll
        for (uint32_t b = 0; b < 4; b++) {
            const KT u = base | ((KT)b << (2 * (k - 1)));
            if (alive(u) >= 0) {
                d++;
                only = u;
            }
        }
        return d;
    }
    // surviving predecessors of oriented v; *only receives the last one found, oriented
    // towards v
    __device__ __forceinline__ int pred(KT v, KT &only) const {
        if (fwd) {
            int d = 0;
            const KT base = (v << 2) & KeyOps<KT>::mask(k);
#pragma unroll
            for (uint32_t b = 0; b < 4; b++) {
                const KT u = base | (KT)b;
                if (alive(u) >= 0) {
                    d++;
                    only = u;
                }
            }
            return d;
        }
        KT w;
        const int d = succ(rc(v), w);
        only = rc(w);
        return d;
    }
    // ignored-side flags in the orientation of v (hashmap.rs:453-465):
    // canonical orientation: flags == 1 -> left boundary, flags == 2 -> right boundary.
    // A k-mer equal to its reverse complement blocks no edge: a walk that enters it takes it
    // and stops there whatever its flags (hashmap.rs:162-297 tests the flags of a k-mer only
    // after appending it), and a walk leaving it is the mirror of one that enters it.
    __device__ __forceinline__ bool right_boundary(KT v, int64_t slot) const {
        if (pal(v)) return false;
        uint32_t f = t.vals[slot] >> 30;
        bool is_canon = fwd || v <= rc(v);
        return is_canon ? f == 2u : f == 1u;
    }
    __device__ __forceinline__ bool left_boundary(KT v, int64_t slot) const {
        if (pal(v)) return false;
        uint32_t f = t.vals[slot] >> 30;
        bool is_canon = fwd || v <= rc(v);
        return is_canon ? f == 1u : f == 2u;
    }
    // link flags of an emitted path from v to e (bit0 left end, bit1 right end).  A
    // reverse-complement-symmetric end is a link end when exactly one of its flags is set; a
    // path of that k-mer alone takes the sides a walk started on it gives (hashmap.rs:453-465
    // with is_forward false: flags 1 -> right end, flags 2 -> left end).
    __device__ __forceinline__ uint8_t path_flags(KT v, int64_t sv, KT e, int64_t se, uint32_t steps) const {
        if (steps == 0 && pal(v)) {
            const uint32_t f = t.vals[sv] >> 30;
            return (uint8_t)((f == 2u ? 1u : 0u) | (f == 1u ? 2u : 0u));
        }
        const uint32_t fv = t.vals[sv] >> 30, fe = t.vals[se] >> 30;
        const bool lb = pal(v) ? (fv == 1u || fv == 2u) : left_boundary(v, sv);
        const bool rb = pal(e) ? (fe == 1u || fe == 2u) : right_boundary(e, se);
        return (uint8_t)((lb ? 1u : 0u) | (rb ? 2u : 0u));
    }
    // Traversable successor: unique surviving successor u with a unique surviving
    // predecessor, no bucket boundary between them, and not the same k-mer.
    __device__ __forceinline__ bool next(KT v, int64_t sv, KT &u, int64_t &su) const {
        if (right_boundary(v, sv)) return false;
        if (succ(v, u) != 1) return false;
        su = tfind(t, canon(u));
        if (su == sv) return false;
        KT w;
        if (pred(u, w) != 1) return false;
        if (left_boundary(u, su)) return false;
        return true;
    }
    __device__ __forceinline__ bool is_start(KT v, int64_t sv) const {
        if (pal(v)) return true;
        if (left_boundary(v, sv)) return true;
        KT y;  // the unique predecessor, oriented towards v
        if (pred(v, y) != 1) return true;
        int64_t sy = tfind(t, canon(y));
        if (sy == sv) return true;
        KT z;
        if (succ(y, z) != 1) return true;
        if (right_boundary(y, sy)) return true;
        return false;
    }
};

__device__ __forceinline__ char base_char(uint32_t c) { return "ACTG"[c & 3]; }

// Walk a path from start v; returns the end node and the number of steps.
template <typename KT>
__device__ __forceinline__ uint32_t walk_to_end(const Graph<KT> &g, KT v, int64_t sv, KT &end, int64_t &send,
                                                unsigned *status) {
    uint32_t steps = 0;
    KT cur = v;
    int64_t scur = sv;
    for (;;) {
        KT u;
        int64_t su;
        if (steps > 0 && g.pal(cur)) break;  // entered a reverse-complement-symmetric k-mer
        if (!g.next(cur, scur, u, su)) break;
        cur = u;
        scur = su;
        if (++steps > g.t.cap) {
            atomicOr(status, kStatusWalkLimit);
            break;
        }
    }
    end = cur;
    send = scur;
    return steps;
}

// Emit the path (or cycle of `steps` edges when circular) starting at v.
template <typename KT>
__device__ void emit_walk(const Graph<KT> &g, KT v, int64_t sv, uint32_t steps, uint8_t flags, const MergeOut &o) {
    const int k = g.k;
    uint64_t len = (uint64_t)k + steps;
    unsigned long long off = atomicAdd(&o.counters[1], (unsigned long long)len);
    unsigned long long idx = atomicAdd(&o.counters[0], 1ull);
    bool ok = (off + len <= o.bases_cap) && (idx < o.u_cap);
    if (!ok) atomicOr(o.status, kStatusOutOverflow);
    if (ok) {
        o.u_off[idx] = off;
        o.u_len[idx] = (uint32_t)len;
        o.u_flags[idx] = flags;
        for (int i = 0; i < k; i++) o.bases[off + i] = base_char((uint32_t)(v >> (2 * i)));
    }
    g.t.vis[sv] = 1;
    KT cur = v;
    int64_t scur = sv;
    for (uint32_t s = 0; s < steps; s++) {
        KT u;
        int64_t su;
        if (!g.next(cur, scur, u, su)) break;
        if (ok) o.bases[off + k + s] = base_char((uint32_t)(u >> (2 * (k - 1))));
        g.t.vis[su] = 1;
        cur = u;
        scur = su;
    }
}

// Which of a k-mer's ignored ends sets which MapEntry flag bit (hashmap.rs:393-396: begin <<
// !is_forward, end << is_forward, in the record's stored orientation).  The k-mers are read in
// text orientation; a reverse-complemented record swaps begin and end and flips is_forward,
// which cancels, except for a k-mer equal to its reverse complement (even k): its is_forward
// (fw < rc) is false in both orientations, so in a reverse-complemented record the text-order
// ends map to the bits as if it were forward.
__device__ __forceinline__ uint32_t flag_orientation(uint32_t isf, bool symmetric, uint32_t rcf) {
    return isf | ((symmetric && rcf) ? 1u : 0u);
}

// Insert all k-mers of one superkmer record (hashmap.rs:361-431 add_sequence), processing
// the bases in text orientation with the flags mapped from the stored orientation.
template <typename KT>
__device__ __forceinline__ void insert_record(const Table<KT> &t, const uint64_t *__restrict__ packed, const SkRec r,
                                              int k, int fwd, unsigned *status) {
    const uint64_t start = rec_start(r);
    const uint32_t len = rec_len(r);
    const uint32_t fl = rec_flags(r), rcf = rec_rc(r);
    // text-orientation included flags: begin <- stored end when reverse-complemented
    const uint32_t inc_begin = rcf ? (fl >> 1) & 1u : fl & 1u;
    const uint32_t inc_end = rcf ? fl & 1u : (fl >> 1) & 1u;
    const KT mask = KeyOps<KT>::mask(k);
    KT fw = 0, rc = 0;
    uint64_t cur_word = ~0ull, pw = 0;
    const uint32_t last = len - (uint32_t)k;
    for (uint32_t i = 0; i < len; i++) {
        uint64_t p = start + i;
        uint64_t wi = p >> 5;
        if (wi != cur_word) {
            cur_word = wi;
            pw = packed[wi];
        }
        const uint32_t c = (uint32_t)(pw >> (2 * (p & 31))) & 3u;
        fw = (fw >> 2) | ((KT)c << (2 * (k - 1)));
        rc = ((rc << 2) | (KT)(c ^ 2u)) & mask;
        if (i + 1 < (uint32_t)k) continue;
        uint32_t idx = i + 1 - (uint32_t)k;
        bool begin_ignored = (idx == 0) && !inc_begin;
        bool end_ignored = (idx == last) && !inc_end;
        uint32_t isf = (fwd || fw < rc) ? 1u : 0u;
        const KT key = isf ? fw : rc;
        int64_t s = tinsert(t, key, status);
        if (s < 0) continue;
        const uint32_t fo = flag_orientation(isf, fw == rc, rcf);
        uint32_t fbits = ((uint32_t)begin_ignored << (fo ^ 1u)) | ((uint32_t)end_ignored << fo);
        if (fbits) atomicOr(&t.vals[s], fbits << 30);
        atomicAdd(&t.vals[s], 1u);
    }
}

// Per-slot work of the extension phase: k-mer dump, then path starts in both orientations.
template <typename KT>
__device__ __forceinline__ void extend_slot(const Graph<KT> &g, uint32_t s, const MergeOut &o, int keep_kmers,
                                            uint32_t min_mult) {
    const KT key = g.t.keys[s];
    if (key == KeyOps<KT>::empty()) return;
    uint32_t mult = val_mult(g.t.vals[s]);
    if (mult < min_mult) return;
    if (keep_kmers) {
        unsigned long long i = atomicAdd(&o.counters[2], 1ull);
        if (i < o.kmer_cap) {
            KeyOps<KT>::store(o.kmer_keys, i, key);
            o.kmer_mult[i] = mult;
        } else {
            atomicOr(o.status, kStatusKmerOverflow);
        }
    }
    for (int orient = 0; orient < (g.fwd ? 1 : 2); orient++) {
        const KT v = orient ? g.rc(key) : key;
        if (orient && v == key) break;  // reverse-complement-symmetric: one orientation
        if (!g.is_start(v, s)) continue;
        KT e;
        int64_t se;
        uint32_t steps = walk_to_end(g, v, (int64_t)s, e, se, o.status);
        // canonical: a path is found from both ends, the lower slot emits it; forward-only: it
        // is found from its start only
        bool owner = g.fwd || ((int64_t)s < se) || ((int64_t)s == se && orient == 0);
        if (!owner) continue;
        emit_walk(g, v, (int64_t)s, steps, g.path_flags(v, (int64_t)s, e, se, steps), o);
    }
}

// Cycle phase: surviving k-mers not covered by any path lie on cycles; the cycle is
// emitted once, from its smallest slot.
template <typename KT>
__device__ __forceinline__ void cycle_slot(const Graph<KT> &g, uint32_t s, const MergeOut &o, uint32_t min_mult) {
    const KT key = g.t.keys[s];
    if (key == KeyOps<KT>::empty() || g.t.vis[s]) return;
    if (val_mult(g.t.vals[s]) < min_mult) return;
    KT cur = key;
    int64_t scur = s;
    uint32_t steps = 0;
    int64_t min_slot = s;
    bool closed = false;
    for (;;) {
        KT u;
        int64_t su;
        if (!g.next(cur, scur, u, su)) break;
        if (su == (int64_t)s) {
            closed = (u == key);
            steps++;
            break;
        }
        if (su < min_slot) min_slot = su;
        cur = u;
        scur = su;
        if (++steps > g.t.cap) {
            atomicOr(o.status, kStatusWalkLimit);
            return;
        }
    }
    if (!closed) {
        atomicOr(o.status, kStatusWalkLimit);
        return;
    }
    if (min_slot != (int64_t)s) return;
    // a cycle of `steps` k-mers: k + steps - 1 bases, circular flag
    emit_walk(g, key, (int64_t)s, steps - 1, (uint8_t)4u, o);
}

// ---------------------------------------------------------------------------
// classify: pack consecutive sub-bins of each bucket into merge units of three tiers
//   S: <= small_limit k-mer instances, packed up to unit_target, shared-memory table
//   M: one sub-bin up to medium_limit instances, one CTA with a global-memory table
//   L: larger sub-bins, global-memory table processed grid-wide
// ---------------------------------------------------------------------------
// global-memory table capacity of a unit of kk instances: a power of two >= kk / load + 64
__device__ __forceinline__ uint32_t table_cap_for(uint64_t kk, uint32_t load_pct) {
    uint64_t cap = 64;
    const uint64_t want = kk * 100 / load_pct + 64;
    while (cap < want) cap <<= 1;
    return (uint32_t)cap;
}

// One warp per bucket: the lanes load 32 sub-bins' counts and offsets at a time (coalesced)
// and the warp walks them in order with the counts in registers (the same greedy packing on
// every lane; lane 0 writes the units).
__global__ void __launch_bounds__(128) classify_units_kernel(
    const unsigned long long *__restrict__ bin_off, const unsigned long long *__restrict__ kmer_off, uint32_t n_buckets,
    int fbits, uint64_t small_limit, uint64_t unit_target, uint64_t wide_limit, uint64_t medium_limit, uint32_t load_pct,
    MergeUnit *small_units, MergeUnit *wide_units, MergeUnit *medium_units, MergeUnit *large_units, uint64_t max_units,
    uint64_t pool_slots, unsigned long long *counters, unsigned *status) {
    const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (b >= n_buckets) return;
    const uint32_t nsub = 1u << fbits;
    uint64_t cur_begin = 0, cur_end = 0, cur_k = 0;
    bool open = false;
    auto close_small = [&]() {
        if (!open) return;
        if (lane == 0) {
            unsigned long long i = atomicAdd(&counters[kCntSmall], 1ull);
            if (i >= max_units) atomicOr(status, kStatusTableFull);
            if (i < max_units) {
                MergeUnit u;
                u.rec_begin = cur_begin;
                u.rec_end = cur_end;
                u.kmers = cur_k;
                u.table_off = 0;
                u.table_cap = 0;
                u.bucket = b;
                small_units[i] = u;
            }
        }
        open = false;
        cur_k = 0;
    };
    for (uint32_t j0 = 0; j0 < nsub; j0 += 32) {
        const uint64_t my_bin = (uint64_t)b * nsub + j0 + (uint32_t)lane;
        const bool in = j0 + (uint32_t)lane < nsub;
        const uint64_t my_k = in ? kmer_off[my_bin + 1] - kmer_off[my_bin] : 0ull;
        const uint64_t my_beg = in ? bin_off[my_bin] : 0ull;
        const uint64_t my_end = in ? bin_off[my_bin + 1] : 0ull;
        if (__ballot_sync(0xffffffffu, my_k != 0) == 0) continue;
        const uint32_t cnt = min(32u, nsub - j0);
        for (uint32_t i = 0; i < cnt; i++) {
            const uint64_t kk = __shfl_sync(0xffffffffu, my_k, (int)i);
            const uint64_t beg = __shfl_sync(0xffffffffu, my_beg, (int)i);
            const uint64_t end = __shfl_sync(0xffffffffu, my_end, (int)i);
            if (kk == 0) continue;
            if (kk > small_limit) {
                close_small();
                // wide: a W unit tries the shared-memory table first (it fits when the sub-bin
                // repeats its k-mers enough) and moves to the M tier with this reserved table when
                // its distinct k-mers overflow the shared-memory table
                if (lane == 0) {
                    const bool wide = kk <= wide_limit;
                    const bool medium = kk <= medium_limit;
                    unsigned long long ui =
                        atomicAdd(&counters[wide ? kCntWide : medium ? kCntMedium : kCntLarge], 1ull);
                    uint32_t cap = table_cap_for(kk, load_pct);
                    unsigned long long off = atomicAdd(&counters[kCntSlots], (unsigned long long)cap);
                    if (off + cap > pool_slots || ui >= max_units) {
                        atomicOr(status, kStatusTableFull);
                    } else {
                        MergeUnit u;
                        u.rec_begin = beg;
                        u.rec_end = end;
                        u.kmers = kk;
                        u.table_off = off;
                        u.table_cap = cap;
                        u.bucket = b;
                        (wide ? wide_units : medium ? medium_units : large_units)[ui] = u;
                    }
                }
                continue;
            }
            if (open && cur_k + kk > unit_target) close_small();
            if (!open) {
                open = true;
                cur_begin = beg;
            }
            cur_k += kk;
            cur_end = end;
        }
    }
    close_small();
}

// ---------------------------------------------------------------------------
// small units: persistent CTAs, shared-memory table, device work queue
// ---------------------------------------------------------------------------
// Tiers of merge_unit_kernel (one unit per CTA, persistent over a device work queue):
//   S: many sub-bins packed per unit, hash table in shared memory; u64 keys: 512 threads,
//      2 CTAs/SM (u128: 256 threads, 2 CTAs/SM);
//   W: one sub-bin of up to 65536 (u128: 16384) instances, the largest shared-memory table;
//      u64 keys: 1024 threads and 11264 slots, u128: 1024 threads and 7936 slots, 1 CTA/SM; a
//      unit whose distinct k-mers overflow the table moves to the M queue (with a reserved
//      global table);
//   M: table in the global pool (L2-resident), 512 threads, 2 CTAs/SM, shared memory for the
//      list-ranking arrays of up to 2048 (u128: 1536) survivors.
// The phases of a unit are separated by block barriers and bound by shared-memory latency, so
// the u64 tiers and the u128 W tier run 32 warps per SM (the kernel fits 64 registers per
// thread; u128 W keeps shared ranking arrays for 1024 survivors to make room for them).  S and W reuse
// the table bytes for the list-ranking arrays once the successor phase is done (union).  Units
// with more survivors than kSurv rank in the CTA's global scratch (extend_unit).
enum : int { kTierS = 0, kTierW = 1, kTierM = 2 };
template <typename KT, int kTier>
struct TierCfg;
template <>
struct TierCfg<uint64_t, kTierS> {
    static constexpr int NT = 512, kSlots = kSmallSlots, kSurv = 2048, kMinBlocks = 2;
};
template <>
struct TierCfg<u128, kTierS> {
    static constexpr int NT = 256, kSlots = kSmallSlots / 2, kSurv = 1024, kMinBlocks = 2;
};
template <>
struct TierCfg<uint64_t, kTierW> {
    static constexpr int NT = 1024, kSlots = 11264, kSurv = 4096, kMinBlocks = 1;
};
template <>
struct TierCfg<u128, kTierW> {
    static constexpr int NT = 1024, kSlots = 7936, kSurv = 1024, kMinBlocks = 1;
};
template <>
struct TierCfg<uint64_t, kTierM> {
    static constexpr int NT = 512, kSlots = 0, kSurv = 2048, kMinBlocks = 2;
};
template <>
struct TierCfg<u128, kTierM> {
    static constexpr int NT = 512, kSlots = 0, kSurv = 1536, kMinBlocks = 2;
};
// k > 64: every unit runs in this tier (or the grid-wide L kernels)
template <>
struct TierCfg<u256, kTierM> {
    static constexpr int NT = 512, kSlots = 0, kSurv = 1536, kMinBlocks = 1;
};
constexpr uint16_t kNone16 = 0xffff, kMulti16 = 0xfffe;

template <int N>
struct RankView {
    uint16_t jump[2 * N];     // pointer jumping: ends point to themselves
    uint16_t rank[2 * N];     // distance to the path end
    uint32_t offs[2 * N];     // local base offset of owner starts
    uint16_t uidx[2 * N];     // local unitig index of owner starts
    uint8_t haspred[2 * N];
};
template <typename KT, int kSlots>
struct SmemTableView {
    KT keys[kSlots];
    uint32_t vals[kSlots];  // count|flags<<30, then alive<<31|flags<<28|dense index
};

// packed words staged per record in the insert phase (records spanning more read global
// memory): k <= 32 superkmers are short; k > 32 superkmers of long reads often span 5-6 words,
// k > 64 ones up to 8
template <typename KT>
constexpr int stage_words() {
    return std::is_same<KT, uint64_t>::value ? 4 : std::is_same<KT, u128>::value ? 6 : 8;
}
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// colour of the sequence holding text position pos (the last sequence starting at or before it)
__device__ __forceinline__ uint32_t colour_at(const MergeArgs &a, uint64_t pos) {
    uint32_t lo = 0, hi = a.n_seq;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a.seq_off[mid] <= pos)
            lo = mid;
        else
            hi = mid;
    }
    return a.seq_color[lo];
}

// block-shared scalars of the extension phase
struct ExtShared {
    uint32_t n_surv, loc_bases, loc_count, ok;
    unsigned long long gbase, gidx;
};

template <typename KT, int N, int NT>
struct UnitSmemCommon {
    uint64_t stage[NT][stage_words<KT>()];  // per lane: the packed words of its record (insert phase)
    KT sk[N];              // survivor canonical k-mers (dense order)
    uint16_t succ[2 * N];  // traversable successor of each oriented node
    uint8_t bflag[2 * N];  // bit0 left boundary, bit1 right boundary (oriented)
    uint32_t warp_tmp[NT / 32 + 1];
    uint64_t unit;
    uint32_t distinct;  // entries created (optimistic units)
    uint32_t batch_head;  // next record batch of the insert phase
    ExtShared x;
};
template <typename KT, int kTier, bool kShared = (kTier != kTierM)>
struct UnitSmem;
template <typename KT, int kTier>
struct UnitSmem<KT, kTier, true> : UnitSmemCommon<KT, TierCfg<KT, kTier>::kSurv, TierCfg<KT, kTier>::NT> {
    using C = TierCfg<KT, kTier>;
    static_assert(sizeof(RankView<C::kSurv>) <= sizeof(SmemTableView<KT, C::kSlots>),
                  "rank view must fit in the table bytes");
    union {
        SmemTableView<KT, C::kSlots> t;
        RankView<C::kSurv> r;
    } u;
};
template <typename KT, int kTier>
struct UnitSmem<KT, kTier, false> : UnitSmemCommon<KT, TierCfg<KT, kTier>::kSurv, TierCfg<KT, kTier>::NT> {
    union {
        RankView<TierCfg<KT, kTier>::kSurv> r;
    } u;
};
static_assert(sizeof(UnitSmem<uint64_t, kTierW>) <= 227 * 1024 && sizeof(UnitSmem<u128, kTierW>) <= 227 * 1024 &&
                  sizeof(UnitSmem<uint64_t, kTierM>) <= 227 * 1024 && sizeof(UnitSmem<u128, kTierM>) <= 227 * 1024 &&
                  2 * sizeof(UnitSmem<uint64_t, kTierS>) <= 227 * 1024 && 2 * sizeof(UnitSmem<u128, kTierS>) <= 227 * 1024 &&
                  sizeof(UnitSmem<u256, kTierM>) <= 227 * 1024,
              "shared memory of a merge CTA");
// a shared-memory table never holds more survivors than the extension scratch of its CTA
static_assert(TierCfg<uint64_t, kTierS>::kSlots <= (int)kExtCapShared && TierCfg<uint64_t, kTierW>::kSlots <= (int)kExtCapShared &&
                  TierCfg<u128, kTierS>::kSlots <= (int)kExtCapShared && TierCfg<u128, kTierW>::kSlots <= (int)kExtCapShared,
              "extension scratch of the shared-memory tiers");

// exclusive block scan of one u32 per thread (blockDim.x == NT); all threads call it
template <int NT>
__device__ __forceinline__ uint32_t block_scan_u32(uint32_t v, uint32_t *warp_tmp, uint32_t &total) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_tmp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < NW ? warp_tmp[lane] : 0u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        if (lane < NW) warp_tmp[lane] = t;
    }
    __syncthreads();
    total = warp_tmp[NW - 1];
    uint32_t r = (wid > 0 ? warp_tmp[wid - 1] : 0u) + x - v;
    __syncthreads();
    return r;
}

__device__ __forceinline__ bool val_alive(uint32_t v) { return (v >> 31) != 0; }

// number of alive successors of oriented v (rv = its reverse complement); *s_only receives
// the slot of the last one found and *fw_only whether it is in canonical orientation.  The
// successor's reverse complement follows from rv: rc(v[1..] + b) = comp(b) + rc(v)[..k-1].
template <typename KT>
__device__ __forceinline__ int alive_succ(const Table<KT> &t, KT v, KT rv, int k, int64_t &s_only, bool &fw_only) {
    int d = 0;
    const KT bse = v >> 2;
    const KT rbase = (rv << 2) & KeyOps<KT>::mask(k);
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) {
        const KT w = bse | ((KT)b << (2 * (k - 1)));
        const KT rw = rbase | (KT)(b ^ 2u);
        const int64_t sw = tfind(t, w < rw ? w : rw);
        if (sw >= 0 && val_alive(t.vals[sw])) {
            d++;
            s_only = sw;
            fw_only = w < rw;
        }
    }
    return d;
}

// alive_succ on a shared-memory table of u64 keys: the four first probes (key and value words)
// are issued together; a collision continues probing
__device__ __forceinline__ int alive_succ_shared(const Table<uint64_t> &t, uint64_t v, uint64_t rv, int k,
                                                 uint32_t &v_only, bool &fw_only) {
    const uint64_t bse = v >> 2;
    const uint64_t rbase = (rv << 2) & kmer_mask(k);
    const uint32_t kb = smem_addr(t.keys), vb = smem_addr(t.vals);
    uint64_t key[4], got[4];
    uint32_t slot[4], val[4];
    bool isfw[4];
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) {
        const uint64_t w = bse | ((uint64_t)b << (2 * (k - 1)));
        const uint64_t rw = rbase | (uint64_t)(b ^ 2u);
        isfw[b] = w < rw;
        key[b] = isfw[b] ? w : rw;
        slot[b] = slot_of(key[b], t.cap);
    }
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) {
        got[b] = lds_u64(kb + 8u * slot[b]);
        val[b] = lds_u32(vb + 4u * slot[b]);
    }
    int d = 0;
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) {
        bool hit = got[b] == key[b];
        uint32_t vw = val[b];
        if (!hit && got[b] != ~0ull) {
            uint32_t s = slot[b];
            for (uint32_t probe = 1; probe < t.cap; probe++) {
                s = next_slot(s, t.cap);
                const uint64_t kk = lds_u64(kb + 8u * s);
                if (kk == key[b]) {
                    hit = true;
                    vw = lds_u32(vb + 4u * s);
                    break;
                }
                if (kk == ~0ull) break;
            }
        }
        if (hit && val_alive(vw)) {
            d++;
            v_only = vw;
            fw_only = isfw[b];
        }
    }
    return d;
}

// forward-only builds: surviving successors of the k-mer x read forward (back = 0) or its
// predecessors (back = 1, the node that walks x backwards); v_only receives the value word of
// the last one found
template <typename KT>
__device__ __forceinline__ int alive_succ_fwd(const Table<KT> &t, KT x, bool back, int k, uint32_t &v_only,
                                              bool &fw_only) {
    int d = 0;
    const KT mask = KeyOps<KT>::mask(k);
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) {
        const KT w = back ? (((x << 2) & mask) | (KT)b) : ((x >> 2) | ((KT)b << (2 * (k - 1))));
        const int64_t sw = tfind(t, w);
        if (sw >= 0) {
            const uint32_t vw = t.vals[sw];
            if (val_alive(vw)) {
                d++;
                v_only = vw;
            }
        }
    }
    fw_only = !back;
    return d;
}

template <typename KT>
__device__ __forceinline__ KT oriented(const KT *sk, uint32_t u, int k) {
    const KT x = sk[u >> 1];
    return (u & 1) ? KeyOps<KT>::rc(x, k) : x;
}

// Arrays of the extension phase of one unit: the survivors in dense order, and per oriented
// node u = 2*dense + (0 canonical, 1 reverse complement) the successor code, boundary sides,
// pointer-jumping state and emission slots.  IT is the node index type: u16 for the arrays in
// shared memory, u32 for the per-CTA scratch in global memory that units with more survivors
// than the shared-memory arrays hold use.
template <typename KT, typename IT>
struct ExtArrays {
    KT *sk;
    IT *succ;
    uint8_t *bflag;   // bit0 left boundary, bit1 right boundary (oriented)
    IT *jump, *rank;
    IT *jump2, *rank2;  // second pointer-jumping buffer (global scratch; the shared path uses registers)
    uint32_t *offs;   // local base offset of owner starts
    IT *uidx;         // local unitig index of owner starts
    uint8_t *haspred;
};

// Global scratch of one CTA for up to `cap` survivors: keys, then seven u32 and two u8 arrays
// of 2*cap oriented nodes.
__host__ __device__ constexpr uint64_t ext_bytes_per_survivor(uint64_t key_bytes) { return key_bytes + 2 * (7 * 4 + 2); }

template <typename KT>
__device__ __forceinline__ ExtArrays<KT, uint32_t> ext_global_arrays(uint8_t *base, uint32_t cap) {
    ExtArrays<KT, uint32_t> A;
    const size_t nn = 2 * (size_t)cap;
    A.sk = reinterpret_cast<KT *>(base);
    uint32_t *w = reinterpret_cast<uint32_t *>(base + sizeof(KT) * (size_t)cap);
    A.succ = w;
    A.jump = w + nn;
    A.rank = w + 2 * nn;
    A.jump2 = w + 3 * nn;
    A.rank2 = w + 4 * nn;
    A.offs = w + 5 * nn;
    A.uidx = w + 6 * nn;
    uint8_t *b = reinterpret_cast<uint8_t *>(w + 7 * nn);
    A.bflag = b;
    A.haspred = b + nn;
    return A;
}

// Extension of one unit after the survivor count (the extension rules of
// try_extend_function, hashmap.rs:162-297): dense numbering of the survivors, successor of
// every oriented node, list ranking by pointer jumping, emission of every path once (from the
// end with the smaller node) and of every cycle once.  All threads of the CTA call it.
//   list_scan: the survivor scan visits t_list[seg] (created-entry list) instead of slots
//   warp_base: this warp's first dense index (lane 0 of the block scan of survivor counts)
//   kRegJ:     per-thread register buffer of the shared-memory pointer jumping
template <typename KT, typename IT, int NT, int kRegJ, bool kGlobalArr, bool kSharedTable>
__device__ __forceinline__ void extend_unit(const Table<KT> &t, const uint32_t *t_list, bool list_scan,
                                            uint32_t seg_lo, uint32_t seg_hi, uint32_t warp_base, uint32_t n_surv,
                                            const ExtArrays<KT, IT> &A, ExtShared &X, int k, uint32_t min_mult,
                                            int keep_kmers, int fwd, const MergeOut &o, uint32_t *bm_cta = nullptr,
                                            int bm_words = 0, uint32_t *bm_out = nullptr) {
    using K = KeyOps<KT>;
    constexpr IT kNone = (IT)~(IT)0;
    constexpr IT kMulti = (IT)(kNone - 1);
    constexpr uint32_t kIdxMask = sizeof(IT) == 2 ? 0xffffu : 0x0fffffffu;
    const int lane = threadIdx.x & 31;

    // dense numbering in slot order; vals become alive<<31 | flags<<28 | dense index
    {
        uint32_t base = __shfl_sync(0xffffffffu, warp_base, 0);
        for (uint32_t b0 = seg_lo; b0 < seg_hi; b0 += 32) {
            const uint32_t ix = b0 + lane;
            const uint32_t sl = ix < seg_hi ? (list_scan ? t_list[ix] : ix) : 0u;
            bool alive = false;
            uint32_t v = 0;
            if (ix < seg_hi) {
                v = t.vals[sl];
                alive = val_mult(v) >= min_mult;
            }
            const unsigned bm = __ballot_sync(0xffffffffu, alive);
            const uint32_t idx = base + __popc(bm & ((1u << lane) - 1u));
            if (alive) {
                const KT key = t.keys[sl];
                A.sk[idx] = key;
                // boundary sides of both orientations (MapEntry flags in canonical
                // orientation: 1 = left side ignored, 2 = right side ignored)
                const uint32_t fv = v >> 30;
                if (!fwd && !(k & 1) && key == K::rc(key, k)) {
                    // reverse-complement-symmetric (even k): edges enter its odd node and leave
                    // its even node whatever its flags; a single flag makes the path end there
                    // (odd node) and the mirror path start there (even node) link ends.  Bit 2
                    // marks the k-mer, bits 3-4 keep the flags for a path of it alone.
                    const uint32_t one = (fv == 1u || fv == 2u) ? 1u : 0u;
                    A.bflag[2 * idx] = (uint8_t)(one | 4u | (fv << 3));
                    A.bflag[2 * idx + 1] = (uint8_t)((one << 1) | 4u | (fv << 3));
                } else {
                    A.bflag[2 * idx] = (uint8_t)((fv == 1u ? 1u : 0u) | (fv == 2u ? 2u : 0u));
                    A.bflag[2 * idx + 1] = (uint8_t)((fv == 2u ? 1u : 0u) | (fv == 1u ? 2u : 0u));
                }
                if (keep_kmers) {
                    const unsigned long long di = atomicAdd(&o.counters[kCntKmers], 1ull);
                    if (di < o.kmer_cap) {
                        K::store(o.kmer_keys, di, key);
                        o.kmer_mult[di] = val_mult(v);
                        if (bm_cta)  // the colours collected by the insert
                            for (int w = 0; w < bm_words; w++)
                                bm_out[di * (uint64_t)bm_words + w] = bm_cta[(uint64_t)sl * bm_words + w];
                    } else {
                        atomicOr(o.status, kStatusKmerOverflow);
                    }
                }
            }
            if (ix < seg_hi) t.vals[sl] = alive ? (0x80000000u | ((v >> 30) << 28) | idx) : 0u;
            if (bm_cta && ix < seg_hi && v != 0)  // the scratch stays zero for the next unit
                for (int w = 0; w < bm_words; w++) bm_cta[(uint64_t)sl * bm_words + w] = 0u;
            base += __popc(bm);
        }
        if (threadIdx.x == 0) X.n_surv = n_surv;
        __syncthreads();
    }
    const uint32_t ns = X.n_surv;
    const uint32_t nn = 2 * ns;

    // ---- successors.  Degrees first: per survivor, the surviving successors of both
    //      orientations (4 probes each); code = unique successor node, kNone (none) or kMulti.
    //      A node u -> w is traversable iff u's right side and w's left side are no bucket
    //      boundary, w is u's only successor, u is w's only predecessor (the mirror of w has
    //      one successor) and w is another k-mer. ----
    bool adj = false;
    if constexpr (kSharedTable && std::is_same<KT, uint64_t>::value)
        adj = !fwd && nn < (1u << 14) && 20u * ns <= 7u * t.cap;
    if constexpr (kSharedTable && std::is_same<KT, uint64_t>::value) {
        if (adj) {
            // The k-mer table is dead once the survivors are numbered: its slots become a table
            // of (k-1)-mers.  Node v's successors are the nodes whose first k-1 bases are v's
            // last k-1 bases.  Every survivor enters the canonical form of the first k-1 bases
            // of each of its nodes, with the orientation in which they match; a slot's value
            // word keeps per orientation a count (0, 1, 2 = more) and the last node, so one
            // lookup per node gives its unique successor or its degree.  An rc-symmetric
            // k-mer enters its odd node only (edges into it reach that node).
            const uint32_t vb = smem_addr(t.vals);
            for (uint32_t i = threadIdx.x; i < t.cap; i += NT) {
                t.keys[i] = ~0ull;
                t.vals[i] = 0u;
            }
            __syncthreads();
            const int k1 = k - 1;
            const uint64_t m1 = kmer_mask(k1);
            for (uint32_t i = threadIdx.x; i < ns; i += NT) {
                const uint64_t x = A.sk[i];
                const uint64_t rx = rc_packed(x, k);
                for (uint32_t side = (!(k & 1) && x == rx) ? 1u : 0u; side < 2; side++) {
                    const uint64_t pre = (side ? rx : x) & m1;
                    const uint64_t rpre = rc_packed(pre, k1);
                    const uint64_t key = pre < rpre ? pre : rpre;
                    const uint32_t ori = pre == key ? 1u : 0u;
                    bool created;
                    const int64_t sl = tinsert_shared(t, key, o.status, created);
                    if (sl < 0) continue;
                    const uint32_t a = vb + 4u * (uint32_t)sl;
                    uint32_t old = lds_u32(a);
                    for (;;) {
                        const uint32_t c = (old >> (2 * ori)) & 3u;
                        uint32_t nv = (old & ~(3u << (2 * ori))) | ((c < 2u ? c + 1u : 2u) << (2 * ori));
                        nv = (nv & ~(0x3fffu << (4 + 14 * ori))) | ((2u * i + side) << (4 + 14 * ori));
                        const uint32_t seen = cas_shared_u32(a, old, nv);
                        if (seen == old) break;
                        old = seen;
                    }
                }
            }
            __syncthreads();
            for (uint32_t u = threadIdx.x; u < nn; u += NT) {
                const uint64_t x = A.sk[u >> 1];
                const uint64_t rx = rc_packed(x, k);
                const uint64_t sfx = ((u & 1) ? rx : x) >> 2;
                const uint64_t rsfx = rc_packed(sfx, k1);
                const uint64_t key = sfx < rsfx ? sfx : rsfx;
                const uint32_t ori = sfx == key ? 1u : 0u;
                const int64_t sl = tfind(t, key);
                IT code = kNone;
                if (sl >= 0) {
                    const uint32_t w = t.vals[sl];
                    const uint32_t c = (w >> (2 * ori)) & 3u;
                    if (c == 1u) code = (IT)((w >> (4 + 14 * ori)) & 0x3fffu);
                    else if (c >= 2u) code = kMulti;
                }
                if ((u & 1) && x == rx) code = kNone;  // rc-symmetric k-mer: its odd node ends paths
                A.succ[u] = code;
            }
        }
    }
    if (!adj)
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        const KT x = A.sk[u >> 1];
        const KT rx = K::rc(x, k);
        bool fw_only = true;
        const bool odd = (u & 1) != 0;  // select the operands, not the call: lanes alternate parity
        int d;
        uint32_t v_only = 0;
        if (fwd) {
            // forward-only: even node = x read forward, odd node = x walked backwards
            d = alive_succ_fwd(t, x, odd, k, v_only, fw_only);
        } else if constexpr (kSharedTable && std::is_same<KT, uint64_t>::value) {
            d = alive_succ_shared(t, odd ? rx : x, odd ? x : rx, k, v_only, fw_only);
        } else {
            int64_t s_only = -1;
            d = alive_succ(t, odd ? rx : x, odd ? x : rx, k, s_only, fw_only);
            if (d == 1) v_only = t.vals[s_only];
        }
        IT code = d == 0 ? kNone : kMulti;
        if (d == 1) code = (IT)(2u * (v_only & kIdxMask) + (fw_only ? 0u : 1u));
        // even k: a k-mer equal to its reverse complement (both nodes read it the same way).
        // Edges into it always reach its odd node (a successor search finds it with
        // fw_only = false), so the odd node ends paths and the even node starts them: a walk
        // that enters it stops there, as the hash-map walk does when the next k-mer (the
        // mirror of the one it came from) is already used
        if (odd && !fwd && x == rx) code = kNone;
        A.succ[u] = code;
    }
    __syncthreads();  // the hash table is dead from here on

    // ---- list ranking by pointer jumping ----
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        const IT c = A.succ[u];
        IT nx = kNone;
        if (c < kMulti && !(A.bflag[u] & 2u) && (uint32_t)(c >> 1) != (u >> 1) && A.succ[c ^ 1u] < kMulti &&
            !(A.bflag[c] & 1u))
            nx = c;
        A.jump[u] = nx == kNone ? (IT)u : nx;
        A.rank[u] = nx == kNone ? (IT)0 : (IT)1;
        A.haspred[u] = 0;
    }
    __syncthreads();
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        const IT j = A.jump[u];
        A.succ[u] = j == (IT)u ? kNone : j;
        if (j != (IT)u) A.haspred[j] = 1;
    }
    __syncthreads();
    IT *J = A.jump, *Rk = A.rank;
    // (stops as soon as every jump reaches its path end: log2 of the longest path rounds)
    if constexpr (kGlobalArr) {
        IT *Jn = A.jump2, *Rn = A.rank2;
        for (uint32_t len = 1; len < nn; len <<= 1) {
            int moved = 0;
            for (uint32_t u = threadIdx.x; u < nn; u += NT) {
                const IT j = J[u];
                const uint32_t rr = (uint32_t)Rk[u] + (uint32_t)Rk[j];
                Rn[u] = (IT)(rr > (uint32_t)kMulti ? (uint32_t)kMulti : rr);
                const IT nj = J[j];
                Jn[u] = nj;
                moved |= nj != j;
            }
            IT *tj = J, *tr = Rk;
            J = Jn;
            Rk = Rn;
            Jn = tj;
            Rn = tr;
            if (!__syncthreads_or(moved)) break;
        }
    } else {
        for (uint32_t len = 1; len < nn; len <<= 1) {
            IT nj[kRegJ];
            IT nr[kRegJ];
            int c = 0;
            int moved = 0;
            for (uint32_t u = threadIdx.x; u < nn; u += NT, c++) {
                const IT j = J[u];
                const uint32_t rr = (uint32_t)Rk[u] + (uint32_t)Rk[j];
                nr[c] = (IT)(rr > (uint32_t)kMulti ? (uint32_t)kMulti : rr);
                nj[c] = J[j];
                moved |= nj[c] != j;
            }
            __syncthreads();
            c = 0;
            for (uint32_t u = threadIdx.x; u < nn; u += NT, c++) {
                Rk[u] = nr[c];
                J[u] = nj[c];
            }
            if (!__syncthreads_or(moved)) break;
        }
    }

    // ---- owner starts: one per path (the end with the smaller node, hashmap.rs walks a
    //      path once), local offsets via shared atomics ----
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        if (A.haspred[u]) continue;
        const IT e = J[u];
        if (A.succ[e] != kNone) continue;  // on a cycle (handled below)
        const uint32_t su = u >> 1, se = (uint32_t)e >> 1;
        // a path and its mirror: the one starting lower (forward-only: the one read forward)
        const bool owner = fwd ? (u & 1) == 0 : (su < se || (su == se && (u & 1) == 0));
        if (!owner) continue;
        const uint32_t len = (uint32_t)k + (uint32_t)Rk[u];
        A.offs[u] = atomicAdd(&X.loc_bases, len);
        A.uidx[u] = (IT)atomicAdd(&X.loc_count, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        X.gbase = atomicAdd(&o.counters[kCntBases], (unsigned long long)X.loc_bases);
        X.gidx = atomicAdd(&o.counters[kCntUnitigs], (unsigned long long)X.loc_count);
        X.ok = (X.gbase + X.loc_bases <= o.bases_cap) && (X.gidx + X.loc_count <= o.u_cap);
        if (!X.ok) atomicOr(o.status, kStatusOutOverflow);
    }
    __syncthreads();
    const bool ok = X.ok != 0;
    const unsigned long long gbase = X.gbase, gidx = X.gidx;

    // ---- emission: every node of an owned path writes its base(s) ----
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        const uint32_t mu = u ^ 1u;                 // mirror node
        const IT me = J[mu];                        // end of the mirror path = mirror of u's start
        if (A.succ[me] != kNone) continue;          // cycle node
        const uint32_t s0 = (uint32_t)me ^ 1u;      // start of u's path
        const IT e = J[u];
        const uint32_t ss = s0 >> 1, se = (uint32_t)e >> 1;
        const bool owner = fwd ? (s0 & 1) == 0 : (ss < se || (ss == se && (s0 & 1) == 0));
        if (!owner || !ok) continue;
        const uint32_t dist = Rk[mu];               // distance from the start
        const unsigned long long off = gbase + A.offs[s0];
        const KT v = oriented(A.sk, u, k);
        if (dist == 0) {
            for (int i = 0; i < k; i++) o.bases[off + i] = base_char((uint32_t)(v >> (2 * i)));
            const unsigned long long ix = gidx + A.uidx[u];
            o.u_off[ix] = off;
            o.u_len[ix] = (uint32_t)k + (uint32_t)Rk[u];
            const uint8_t bu = A.bflag[u];
            if (Rk[u] == 0 && (bu & 4u)) {
                // a reverse-complement-symmetric k-mer alone: the sides a walk started on it
                // gives (flags 1 -> right end, flags 2 -> left end)
                const uint32_t fv = (bu >> 3) & 3u;
                o.u_flags[ix] = (uint8_t)((fv == 2u ? 1u : 0u) | (fv == 1u ? 2u : 0u));
            } else {
                o.u_flags[ix] = (uint8_t)((bu & 1u) | (A.bflag[e] & 2u));
            }
        } else {
            o.bases[off + (uint32_t)k - 1 + dist] = base_char((uint32_t)(v >> (2 * (k - 1))));
        }
    }

    // ---- cycles (rare): every node has a successor and a predecessor; the cycle and its
    //      mirror are emitted once, from the smallest node of the pair ----
    for (uint32_t u = threadIdx.x; u < nn; u += NT) {
        if (A.succ[J[u]] == kNone) continue;
        uint32_t minc = u, minm = u ^ 1u, n = 1;
        uint32_t cur = A.succ[u];
        bool closed = false;
        while (n <= nn) {
            if (cur == (uint32_t)kNone) break;
            if (cur == u) {
                closed = true;
                break;
            }
            minc = min(minc, cur);
            minm = min(minm, cur ^ 1u);
            cur = A.succ[cur];
            n++;
        }
        if (!closed) {
            atomicOr(o.status, kStatusWalkLimit);
            continue;
        }
        if (u != minc || minc > minm) continue;
        const uint64_t len = (uint64_t)k + n - 1;
        const unsigned long long off = atomicAdd(&o.counters[kCntBases], len);
        const unsigned long long ix = atomicAdd(&o.counters[kCntUnitigs], 1ull);
        if (off + len > o.bases_cap || ix >= o.u_cap) {
            atomicOr(o.status, kStatusOutOverflow);
            continue;
        }
        KT v = oriented(A.sk, u, k);
        for (int i = 0; i < k; i++) o.bases[off + i] = base_char((uint32_t)(v >> (2 * i)));
        cur = A.succ[u];
        for (uint32_t i = 1; i < n; i++) {
            v = oriented(A.sk, cur, k);
            o.bases[off + (uint32_t)k - 1 + i] = base_char((uint32_t)(v >> (2 * (k - 1))));
            cur = A.succ[cur];
        }
        o.u_off[ix] = off;
        o.u_len[ix] = (uint32_t)len;
        o.u_flags[ix] = 4;
    }
}

// One merge unit per CTA, persistent over a device work queue (tiers above).  All tiers use
// the shared-memory list-ranking arrays for the extension.  kColors: the instantiation that
// collects colours (the uncoloured one carries none of that code).
template <typename KT, int kTier, bool kColors = false>
__global__ void __launch_bounds__(TierCfg<KT, kTier>::NT, TierCfg<KT, kTier>::kMinBlocks)
    merge_unit_kernel(MergeArgs a, const MergeUnit *__restrict__ units, const unsigned long long *__restrict__ counters_ro,
                      KT *pool_keys, uint32_t *pool_vals, uint8_t *pool_vis, uint32_t *pool_list, MergeUnit *spill,
                      uint64_t max_units, MergeOut o) {
    using Cfg = TierCfg<KT, kTier>;
    using Smem = UnitSmem<KT, kTier>;
    using K = KeyOps<KT>;
    constexpr int NT = Cfg::NT;
    constexpr bool kGlobalTable = kTier == kTierM;
    constexpr int kMaxSurv = Cfg::kSurv;
    constexpr int kCount = kTier == kTierS ? kCntSmall : kTier == kTierW ? kCntWide : kCntMedium;
    constexpr int kHead = kTier == kTierS ? kCntSmallHead : kTier == kTierW ? kCntWideHead : kCntMediumHead;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(smem_raw);
    const uint64_t n_units = counters_ro[kCount];
    const int k = a.k;
    const uint32_t min_mult = (uint32_t)a.min_mult;
    // this CTA's colour bitmaps, one row of bm_words per table slot (colours collected here)
    uint32_t *const bm_cta = kColors ? a.bm_scratch + (uint64_t)blockIdx.x * a.bm_stride : nullptr;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) S.unit = atomicAdd(&o.counters[kHead], 1ull);
        __syncthreads();
        const uint64_t ui = S.unit;
        if (ui >= n_units) break;
        const MergeUnit U = units[ui];
        uint32_t cap;
        Table<KT> t;
        uint32_t *t_list = nullptr;  // M units: slots of the created entries (in creation order)
        if constexpr (kGlobalTable) {
            t_list = pool_list + U.table_off;
            cap = U.table_cap;
            t = Table<KT>{pool_keys + U.table_off, pool_vals + U.table_off, pool_vis + U.table_off, cap};
        } else {
            cap = 64;
            while (cap < U.kmers + U.kmers / 4 + 8) cap <<= 1;
            if (cap > (uint32_t)Cfg::kSlots) cap = Cfg::kSlots;
            t = Table<KT>{S.u.t.keys, S.u.t.vals, nullptr, cap};  // (visited marks: walk fallback only)
        }
        // optimistic unit (W tier, or a unit with a reserved global table): stop creating
        // entries at kOptLimit (<= 0.8 load with the at most NT - 1 creations in flight when
        // the count is reached) and spill to the M queue
        const bool optimistic = !kGlobalTable && U.table_cap != 0;
        constexpr uint32_t kOptLimit = kGlobalTable ? 0xffffffffu : (uint32_t)Cfg::kSlots * 4 / 5 - NT;
        for (uint32_t i = threadIdx.x; i < cap; i += blockDim.x) {
            t.keys[i] = K::empty();
            t.vals[i] = 0;
            if constexpr (kGlobalTable) t.vis[i] = 0;
        }
        if (threadIdx.x == 0) {
            S.x.n_surv = 0;
            S.x.loc_bases = 0;
            S.x.loc_count = 0;
            S.distinct = 0;
            S.batch_head = 0;
        }
        __syncthreads();

        const uint64_t n_items = U.rec_end - U.rec_begin;
        // records per insert batch of a warp (<= 32): the launch's choice in the shared-memory
        // tiers (default 16: their units give each warp one or two batches, and smaller batches
        // even out the warps at the barrier that ends the insert), 32 in the M tier
        const int rec_batch = kGlobalTable ? 32 : a.rec_batch;
        if constexpr (!kGlobalTable) {
            // warm L2 with the packed words of the unit's records before the insert batches
            // load them: one dependent round trip (record, then its words) per unit instead of
            // one per batch
            for (uint64_t r0 = threadIdx.x; r0 < n_items; r0 += 4 * NT) {
                uint64_t w0s[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint64_t r = r0 + (uint64_t)q * NT;
                    w0s[q] = r < n_items ? a.recs[U.rec_begin + r].w0 : ~0ull;
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (w0s[q] == ~0ull) continue;
                    const SkRec rr{w0s[q], 0};
                    const uint64_t wb = rec_start(rr) >> 5, we = (rec_start(rr) + rec_len(rr) - 1) >> 5;
                    prefetch_l2(a.packed + wb);
                    if ((we >> 4) != (wb >> 4)) prefetch_l2(a.packed + we);  // another 128-byte line
                }
            }
        }

        // ---- insert (add_sequence, hashmap.rs:361-431).  Each warp takes rec_batch records at
        //      a time and deals their k-mers to its lanes 32 at a time; the record of k-mer j is
        //      found from the mask of record starts in the current 32-k-mer window, so the
        //      insert phase needs no block barrier. ----
        {
            const int lane = threadIdx.x & 31;
            const unsigned full = 0xffffffffu;
            bool stop = false;
            for (;;) {
                // batches of rec_batch records, claimed dynamically (no static warp imbalance at
                // the barrier that ends the phase)
                uint32_t bi = 0;
                if (lane == 0) bi = atomicAdd(&S.batch_head, 1u);
                bi = __shfl_sync(full, bi, 0);
                const uint64_t ib = (uint64_t)bi * rec_batch;
                if (ib >= n_items || stop) break;
                const uint64_t item = ib + lane;
                uint64_t w0 = 0;
                uint32_t fr = 0, nk = 0;
                if (lane < rec_batch && item < n_items) {
                    const SkRec rr = a.recs[U.rec_begin + item];
                    w0 = rr.w0;
                    fr = rec_flags(rr) | (rec_rc(rr) << 2);
                    if (bm_cta) fr |= colour_at(a, rec_start(rr)) << 4;  // bits 4-31: the record's colour
                    nk = rec_len(rr) - (uint32_t)k + 1;  // >= 1: records hold at least one k-mer
                    // stage the record's packed words in shared memory (one round of independent
                    // loads per 32 records instead of one dependent load per k-mer window)
                    const uint64_t st = rec_start(rr);
                    const uint64_t wb = st >> 5, we = (st + rec_len(rr) - 1) >> 5;
                    if (we - wb < (uint64_t)stage_words<KT>()) {
#pragma unroll
                        for (int q = 0; q < stage_words<KT>(); q++)
                            if (wb + q <= we) S.stage[threadIdx.x][q] = a.packed[wb + q];
                    } else {
                        fr |= 8u;  // long record: k-mers read from global memory
                    }
                }
                __syncwarp();
                uint32_t incl = nk;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t y = __shfl_up_sync(full, incl, d);
                    if (lane >= d) incl += y;
                }
                const uint32_t ex = incl - nk;
                const uint32_t total = __shfl_sync(full, incl, 31);
                for (uint32_t J = 0; J < total; J += 32) {
                    if (optimistic) {
                        const bool over = *(volatile uint32_t *)&S.distinct >= kOptLimit;
                        if (__any_sync(full, over)) {
                            stop = true;
                            break;
                        }
                    }
                    // records are in lane order with nk >= 1; record of k-mer J + lane =
                    // (records starting at or before it) - 1
                    const bool starts = nk > 0 && ex >= J && ex < J + 32u;
                    const uint32_t smask = __reduce_or_sync(full, starts ? 1u << (ex - J) : 0u);
                    const uint32_t before = __popc(__ballot_sync(full, nk > 0 && ex < J));
                    const uint32_t j = J + (uint32_t)lane;
                    const bool have = j < total;
                    const uint32_t ri = have ? before + __popc(smask & ((2u << lane) - 1u)) - 1u : 0u;
                    const uint64_t rw0 = __shfl_sync(full, w0, (int)ri);
                    const uint32_t rfr = __shfl_sync(full, fr, (int)ri);
                    const uint32_t rex = __shfl_sync(full, ex, (int)ri);
                    int64_t sl = -1;
                    bool created = false;
                    uint32_t fbits = 0;
                    if (have) {
                    const uint32_t off = j - rex;
                    const uint32_t last = (uint32_t)(rw0 >> 40) - (uint32_t)k;
                    const uint32_t fl = rfr & 3u, rcf = (rfr >> 2) & 1u;
                    // text-orientation included flags (begin <- stored end when reverse-complemented)
                    const uint32_t inc_begin = rcf ? (fl >> 1) & 1u : fl & 1u;
                    const uint32_t inc_end = rcf ? fl & 1u : (fl >> 1) & 1u;
                    const uint64_t pos = (rw0 & ((1ull << 40) - 1)) + off;
                    const KT fw = (rfr & 8u) ? K::load(a.packed, pos, k)
                                             : K::load(S.stage[(threadIdx.x & ~31u) + ri],
                                                       pos - ((rw0 & ((1ull << 40) - 1)) & ~31ull), k);
                    const KT rc = K::rc(fw, k);
                    const uint32_t isf = (a.forward || fw < rc) ? 1u : 0u;
                    if constexpr (!kGlobalTable && std::is_same<KT, uint64_t>::value)
                        sl = tinsert_shared(t, isf ? fw : rc, o.status, created);
                    else if (optimistic || kGlobalTable)
                        sl = tinsert_created(t, isf ? fw : rc, o.status, created);
                    else
                        sl = tinsert(t, isf ? fw : rc, o.status);
                    const bool bi = (off == 0) && !inc_begin, ei = (off == last) && !inc_end;
                    const uint32_t fo = flag_orientation(isf, fw == rc, rcf);
                    fbits = ((uint32_t)bi << (fo ^ 1u)) | ((uint32_t)ei << fo);
                    }
                    if (optimistic || kGlobalTable) {
                        // created entries: counted (W spill test) and, for global tables, listed
                        // so the survivor scan visits entries instead of every slot
                        const unsigned cm = __ballot_sync(full, created);
                        if (cm) {
                            const int leader = __ffs(cm) - 1;
                            uint32_t base = 0;
                            if (lane == leader) base = atomicAdd(&S.distinct, (uint32_t)__popc(cm));
                            base = __shfl_sync(full, base, leader);
                            if (kGlobalTable && created) t_list[base + __popc(cm & ((1u << lane) - 1u))] = (uint32_t)sl;
                        }
                    }
                    if (sl < 0) continue;
                    if (bm_cta) {
                        const uint32_t col = rfr >> 4;
                        atomicOr(bm_cta + (uint64_t)sl * a.bm_words + (col >> 5), 1u << (col & 31));
                    }
                    if constexpr (!kGlobalTable) {
                        const uint32_t va = smem_addr(t.vals + sl);
                        if (fbits) red_shared_or_b32(va, fbits << 30);
                        red_shared_add_u32(va, 1u);
                    } else {
                        if (fbits) atomicOr(&t.vals[sl], fbits << 30);
                        atomicAdd(&t.vals[sl], 1u);
                    }
                }
                __syncwarp();  // the next batch overwrites this warp's staged words
            }
            __syncthreads();
        }
        if (optimistic && S.distinct >= kOptLimit) {
            // too many distinct k-mers for the shared-memory table: the M tier redoes the
            // unit with its reserved global table (the colour scratch is left zero)
            if (bm_cta)
                for (uint32_t sl = threadIdx.x; sl < cap; sl += NT)
                    if (t.keys[sl] != K::empty())
                        for (int w = 0; w < a.bm_words; w++) bm_cta[(uint64_t)sl * a.bm_words + w] = 0u;
            if (threadIdx.x == 0) {
                atomicAdd(&o.counters[kCntSpilled], 1ull);
                const unsigned long long i = atomicAdd(&o.counters[kCntMedium], 1ull);
                if (i < max_units)
                    spill[i] = U;
                else
                    atomicOr(o.status, kStatusTableFull);
            }
            continue;
        }

        // ---- survivors (min-multiplicity filter): each warp scans a contiguous segment of
        //      slots (shared-memory tables) or of the created-entry list (global tables) 32 at
        //      a time, counting with ballots ----
        constexpr int NW = NT / 32;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        const uint32_t n_scan = kGlobalTable ? S.distinct : cap;
        const uint32_t seg = (((n_scan + NW - 1) / NW) + 31) & ~31u;
        const uint32_t seg_lo = min(n_scan, (uint32_t)wid * seg), seg_hi = min(n_scan, seg_lo + seg);
        // (an entry's count is >= 1 from its creation, so the value word alone tells empty
        // from occupied)
        uint32_t warp_surv = 0, warp_occ = 0;
        for (uint32_t b0 = seg_lo; b0 < seg_hi; b0 += 32) {
            const uint32_t ix = b0 + lane;
            bool alive = false, occ = false;
            if (ix < seg_hi) {
                const uint32_t v = t.vals[kGlobalTable ? t_list[ix] : ix];
                occ = v != 0;
                alive = val_mult(v) >= min_mult;
            }
            warp_surv += __popc(__ballot_sync(0xffffffffu, alive));
            warp_occ += __popc(__ballot_sync(0xffffffffu, occ));
        }
        if (lane == 0 && warp_occ) atomicAdd(&o.counters[kCntDistinct], (unsigned long long)warp_occ);
        uint32_t n_surv;
        const uint32_t warp_base = block_scan_u32<NT>(lane == 0 ? warp_surv : 0u, S.warp_tmp, n_surv);
        if (n_surv <= (uint32_t)kMaxSurv) {
            ExtArrays<KT, uint16_t> A{S.sk,          S.succ,    S.bflag,      S.u.r.jump, S.u.r.rank,
                                      nullptr,       nullptr,   S.u.r.offs,   S.u.r.uidx, S.u.r.haspred};
            extend_unit<KT, uint16_t, NT, (kMaxSurv * 2 + NT - 1) / NT, false, !kGlobalTable>(
                t, t_list, kGlobalTable, seg_lo, seg_hi, warp_base, n_surv, A, S.x, k, min_mult, a.keep_kmers, a.forward, o,
                bm_cta, a.bm_words, a.bm_out);
        } else if (a.ext_scratch != nullptr && n_surv <= a.ext_cap) {
            // more survivors than the shared-memory arrays hold: the same ranking on this
            // CTA's scratch in global memory
            if (threadIdx.x == 0) atomicAdd(&o.counters[kCntExtGlobal], 1ull);
            const ExtArrays<KT, uint32_t> A =
                ext_global_arrays<KT>(a.ext_scratch + (size_t)blockIdx.x * a.ext_stride, a.ext_cap);
            extend_unit<KT, uint32_t, NT, 1, true, !kGlobalTable>(t, t_list, kGlobalTable, seg_lo, seg_hi, warp_base, n_surv, A, S.x,
                                                  k, min_mult, a.keep_kmers, a.forward, o, bm_cta, a.bm_words,
                                                  a.bm_out);
        } else {
            // walk fallback (no scratch for this many survivors; a shared-memory table never has
            // more survivors than the scratch holds)
            if (threadIdx.x == 0) atomicAdd(&o.counters[kCntWalk], 1ull);
            if constexpr (kGlobalTable) {
                Graph<KT> g{t, k, min_mult, a.forward};
                for (uint32_t sl = threadIdx.x; sl < cap; sl += blockDim.x)
                    extend_slot(g, sl, o, a.keep_kmers, min_mult);
                __syncthreads();
                for (uint32_t sl = threadIdx.x; sl < cap; sl += blockDim.x) cycle_slot(g, sl, o, min_mult);
                // (these k-mers get no collected colours: the host falls back to the text pass)
                if (bm_cta)
                    for (uint32_t sl = threadIdx.x; sl < cap; sl += blockDim.x)
                        if (t.keys[sl] != K::empty())
                            for (int w = 0; w < a.bm_words; w++) bm_cta[(uint64_t)sl * a.bm_words + w] = 0u;
            } else {
                if (threadIdx.x == 0) atomicOr(o.status, kStatusWalkLimit);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// large units: global-memory tables, grid-wide phases
// ---------------------------------------------------------------------------
template <typename KT>
__global__ void init_tables_kernel(KT *keys, uint32_t *vals, uint8_t *vis, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        keys[i] = KeyOps<KT>::empty();
        vals[i] = 0;
        vis[i] = 0;
    }
}

template <typename KT>
__global__ void init_unit_tables_kernel(const MergeUnit *__restrict__ units, const unsigned long long *__restrict__ n_units_dev,
                                        KT *keys, uint32_t *vals, uint8_t *vis) {
    const uint64_t n_units = *n_units_dev;
    const uint64_t gt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u = 0; u < n_units; u++) {
        const MergeUnit U = units[u];
        for (uint64_t i = gt; i < U.table_cap; i += gs) {
            keys[U.table_off + i] = KeyOps<KT>::empty();
            vals[U.table_off + i] = 0;
            vis[U.table_off + i] = 0;
        }
    }
}

template <typename KT>
__global__ void __launch_bounds__(256) large_insert_kernel(MergeArgs a, const MergeUnit *__restrict__ units,
                                                           const unsigned long long *__restrict__ n_units_dev,
                                                           KT *keys, uint32_t *vals, uint8_t *vis, MergeOut o) {
    const uint64_t n_units = *n_units_dev;
    const uint64_t gt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u = 0; u < n_units; u++) {
        const MergeUnit U = units[u];
        Table<KT> t{keys + U.table_off, vals + U.table_off, vis + U.table_off, U.table_cap};
        for (uint64_t r = U.rec_begin + gt; r < U.rec_end; r += gs) insert_record(t, a.packed, a.recs[r], a.k, a.forward, o.status);
    }
}

template <typename KT>
__global__ void __launch_bounds__(256) large_extend_kernel(MergeArgs a, const MergeUnit *__restrict__ units,
                                                           const unsigned long long *__restrict__ n_units_dev,
                                                           KT *keys, uint32_t *vals, uint8_t *vis, MergeOut o,
                                                           int phase) {
    const uint64_t n_units = *n_units_dev;
    const uint64_t gt = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u = 0; u < n_units; u++) {
        const MergeUnit U = units[u];
        Table<KT> t{keys + U.table_off, vals + U.table_off, vis + U.table_off, U.table_cap};
        Graph<KT> g{t, a.k, (uint32_t)a.min_mult, a.forward};
        unsigned long long occ = 0;
        for (uint64_t s = gt; s < U.table_cap; s += gs) {
            if (phase == 0) {
                occ += keys[U.table_off + s] != KeyOps<KT>::empty();
                extend_slot(g, (uint32_t)s, o, a.keep_kmers, (uint32_t)a.min_mult);
            } else {
                cycle_slot(g, (uint32_t)s, o, (uint32_t)a.min_mult);
            }
        }
        if (occ) atomicAdd(&o.counters[kCntDistinct], occ);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_classify_units(const unsigned long long *bin_off, const unsigned long long *kmer_off, uint32_t n_buckets,
                          int fbits, uint64_t small_limit, uint64_t unit_target, uint64_t wide_limit,
                          uint64_t medium_limit, uint32_t load_pct, MergeUnit *small_units, MergeUnit *wide_units,
                          MergeUnit *medium_units, MergeUnit *large_units, uint64_t max_units, uint64_t pool_slots,
                          unsigned long long *counters, unsigned *status, cudaStream_t s) {
    classify_units_kernel<<<(n_buckets + 3) / 4, 128, 0, s>>>(
        bin_off, kmer_off, n_buckets, fbits, small_limit, unit_target, wide_limit, medium_limit, load_pct, small_units,
        wide_units, medium_units, large_units, max_units, pool_slots, counters, status);
    return 1;
}

template <typename KT, int kTier>
static void merge_tier_t(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters, KT *keys,
                         uint32_t *vals, uint8_t *vis, uint32_t *list, MergeUnit *spill, uint64_t max_units,
                         const MergeOut &o, int sms, cudaStream_t s) {
    using Cfg = TierCfg<KT, kTier>;
    const int smem = (int)sizeof(UnitSmem<KT, kTier>);
    if constexpr (!std::is_same<KT, u256>::value) {
        if (a.bm_words) {  // colours collected (k <= 64)
            merge_unit_kernel<KT, kTier, true><<<sms * Cfg::kMinBlocks, Cfg::NT, smem, s>>>(
                a, units, counters, keys, vals, vis, list, spill, max_units, o);
            return;
        }
    }
    merge_unit_kernel<KT, kTier>
        <<<sms * Cfg::kMinBlocks, Cfg::NT, smem, s>>>(a, units, counters, keys, vals, vis, list, spill, max_units, o);
}

template <typename KT, int kTier, bool kColors = false>
static cudaError_t merge_attr_t() {
    return cudaFuncSetAttribute(merge_unit_kernel<KT, kTier, kColors>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(UnitSmem<KT, kTier>));
}

cudaError_t merge_configure() {
    const cudaError_t e[13] = {merge_attr_t<uint64_t, kTierS>(),       merge_attr_t<uint64_t, kTierW>(),
                               merge_attr_t<uint64_t, kTierM>(),       merge_attr_t<u128, kTierS>(),
                               merge_attr_t<u128, kTierW>(),           merge_attr_t<u128, kTierM>(),
                               merge_attr_t<u256, kTierM>(),           merge_attr_t<uint64_t, kTierS, true>(),
                               merge_attr_t<uint64_t, kTierW, true>(), merge_attr_t<uint64_t, kTierM, true>(),
                               merge_attr_t<u128, kTierS, true>(),     merge_attr_t<u128, kTierW, true>(),
                               merge_attr_t<u128, kTierM, true>()};
    for (cudaError_t x : e)
        if (x != cudaSuccess) return x;
    return cudaSuccess;
}

int launch_merge_medium(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters, void *keys,
                        uint32_t *vals, uint8_t *vis, uint32_t *list, const MergeOut &o, int sms, cudaStream_t s) {
    if (a.wide == 2)
        merge_tier_t<u256, kTierM>(a, units, counters, static_cast<u256 *>(keys), vals, vis, list, nullptr, 0, o, sms,
                                   s);
    else if (a.wide)
        merge_tier_t<u128, kTierM>(a, units, counters, static_cast<u128 *>(keys), vals, vis, list, nullptr, 0, o, sms,
                                   s);
    else
        merge_tier_t<uint64_t, kTierM>(a, units, counters, static_cast<uint64_t *>(keys), vals, vis, list, nullptr, 0, o,
                                       sms, s);
    return 1;
}

int launch_merge_small(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters,
                       const MergeOut &o, int sms, cudaStream_t s) {
    if (a.wide == 2) return 0;  // k > 64: no shared-memory tiers
    if (a.wide)
        merge_tier_t<u128, kTierS>(a, units, counters, nullptr, nullptr, nullptr, nullptr, nullptr, 0, o, sms, s);
    else
        merge_tier_t<uint64_t, kTierS>(a, units, counters, nullptr, nullptr, nullptr, nullptr, nullptr, 0, o, sms, s);
    return 1;
}

int launch_merge_wide(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters,
                      MergeUnit *spill, uint64_t max_units, const MergeOut &o, int sms, cudaStream_t s) {
    if (a.wide == 2) return 0;
    if (a.wide)
        merge_tier_t<u128, kTierW>(a, units, counters, nullptr, nullptr, nullptr, nullptr, spill, max_units, o, sms, s);
    else
        merge_tier_t<uint64_t, kTierW>(a, units, counters, nullptr, nullptr, nullptr, nullptr, spill, max_units, o, sms,
                                       s);
    return 1;
}

int merge_ctas_per_sm(int tier, int wide) {
    if (wide == 2) return TierCfg<u256, kTierM>::kMinBlocks;
    if (wide)
        return tier == 0 ? TierCfg<u128, kTierS>::kMinBlocks
                         : tier == 1 ? TierCfg<u128, kTierW>::kMinBlocks : TierCfg<u128, kTierM>::kMinBlocks;
    return tier == 0 ? TierCfg<uint64_t, kTierS>::kMinBlocks
                     : tier == 1 ? TierCfg<uint64_t, kTierW>::kMinBlocks : TierCfg<uint64_t, kTierM>::kMinBlocks;
}

uint64_t merge_wide_limit(int wide) { return wide == 2 ? 0 : wide ? 16384 : 65536; }

uint64_t merge_small_limit(int wide) {
    // instances of an S unit, so that its table (Tier slots) stays at load <= 0.8
    static_assert(3200 * 5 <= TierCfg<uint64_t, kTierS>::kSlots * 4 && 1600 * 5 <= TierCfg<u128, kTierS>::kSlots * 4,
                  "S table load");
    return wide == 2 ? 0 : wide ? 1600 : 3200;
}

int launch_init_tables(void *keys, int wide, uint32_t *vals, uint8_t *vis, uint64_t slots, int sms, cudaStream_t s) {
    if (slots == 0) return 0;
    if (wide == 2)
        init_tables_kernel<u256><<<sms * 4, 256, 0, s>>>(static_cast<u256 *>(keys), vals, vis, slots);
    else if (wide)
        init_tables_kernel<u128><<<sms * 4, 256, 0, s>>>(static_cast<u128 *>(keys), vals, vis, slots);
    else
        init_tables_kernel<uint64_t><<<sms * 4, 256, 0, s>>>(static_cast<uint64_t *>(keys), vals, vis, slots);
    return 1;
}

int launch_init_unit_tables(const MergeUnit *units, const unsigned long long *n_units_dev, void *keys, int wide,
                            uint32_t *vals, uint8_t *vis, int sms, cudaStream_t s) {
    if (wide == 2)
        init_unit_tables_kernel<u256><<<sms * 4, 256, 0, s>>>(units, n_units_dev, static_cast<u256 *>(keys), vals, vis);
    else if (wide)
        init_unit_tables_kernel<u128><<<sms * 4, 256, 0, s>>>(units, n_units_dev, static_cast<u128 *>(keys), vals, vis);
    else
        init_unit_tables_kernel<uint64_t>
            <<<sms * 4, 256, 0, s>>>(units, n_units_dev, static_cast<uint64_t *>(keys), vals, vis);
    return 1;
}

template <typename KT>
static void merge_large_t(const MergeArgs &a, const MergeUnit *units, const unsigned long long *n_units_dev, KT *keys,
                          uint32_t *vals, uint8_t *vis, const MergeOut &o, int sms, cudaStream_t s) {
    large_insert_kernel<KT><<<sms * 4, 256, 0, s>>>(a, units, n_units_dev, keys, vals, vis, o);
    large_extend_kernel<KT><<<sms * 4, 256, 0, s>>>(a, units, n_units_dev, keys, vals, vis, o, 0);
    large_extend_kernel<KT><<<sms * 4, 256, 0, s>>>(a, units, n_units_dev, keys, vals, vis, o, 1);
}

int launch_merge_large(const MergeArgs &a, const MergeUnit *units, const unsigned long long *n_units_dev,
                       uint64_t n_units_host_hint, void *keys, uint32_t *vals, uint8_t *vis, const MergeOut &o,
                       int sms, cudaStream_t s) {
    (void)n_units_host_hint;
    if (a.wide == 2)
        merge_large_t<u256>(a, units, n_units_dev, static_cast<u256 *>(keys), vals, vis, o, sms, s);
    else if (a.wide)
        merge_large_t<u128>(a, units, n_units_dev, static_cast<u128 *>(keys), vals, vis, o, sms, s);
    else
        merge_large_t<uint64_t>(a, units, n_units_dev, static_cast<uint64_t *>(keys), vals, vis, o, sms, s);
    return 3;
}

}  // namespace ggcat
