// Colour-subset deduplication on sm_103a.
//
// Replaces the per-k-mer colour collection and subset dedup of the reference's
// MultipleColorsManager (crates/colors/src/managers/multiple.rs:99-228: colours of every
// occurrence are collected per k-mer, sorted, deduplicated, and the set is mapped to a
// subset id by ColorsMemMapWriter::get_id, crates/colors/src/colors_memmap_writer.rs:43-61).
// A k-mer's colour set is the set of colours (input files) of all its occurrences, which
// this phase computes globally instead of per bucket:
//   1. the surviving k-mers of the merge go into one device table (key -> id, the dump index
//      of the entry that inserted the key),
//   2. one pass over the input text sets bit `colour` of the k-mer's bitmap for every
//      occurrence (the occurrence's colour is that of the sequence containing it),
//   3. every bitmap is deduplicated into a subset table (exact: hash, then compare).
// Subset ids are assigned in arrival order (as in the reference they are not deterministic);
// the sets they decode to are.
#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace ggcat {

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t *p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// 128-bit compare-and-swap on a global 16-byte word pair; returns the previous pair
__device__ __forceinline__ void cas_pair(uint64_t *slot, uint64_t c0, uint64_t c1, uint64_t v0, uint64_t v1,
                                         uint64_t &o0, uint64_t &o1) {
    asm volatile(
        "{\n\t.reg .b128 c, v, d;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(o0), "=l"(o1)
        : "l"(c0), "l"(c1), "l"(v0), "l"(v1), "l"(slot)
        : "memory");
}

// The k-mer table, empty = all-ones.  A k-mer's id is the dump index of the thread that
// inserted it (its owner), so no numbering pass is needed; ids of k-mers dumped twice are
// holes whose colour bitmap stays empty.
//   u64 keys (k <= 32):  16-byte slots {key, id}, key and id claimed together by one 128-bit
//                        compare-and-swap (a failed compare returns the owner's pair);
//   u128 keys (k <= 64): 32-byte slots {key lo, key hi, id, -}, the key claimed by a 128-bit
//                        compare-and-swap and the id stored right after it; a thread that
//                        finds the key waits (bounded) for the id.
// A lookup reads one slot (one 32-byte sector).
template <typename KT>
struct ColorTable;

template <>
struct ColorTable<uint64_t> {
    static constexpr int kWords = 2;
    __device__ static __forceinline__ uint64_t slot(uint64_t key, uint64_t mask) { return mix64(key) & mask; }
    __device__ static __forceinline__ uint64_t dumped(const uint64_t *kmers, uint64_t i) { return kmers[i]; }
    // owner id of key, inserting it as dump entry i; kEmptyKey on failure
    __device__ static __forceinline__ uint64_t insert(uint64_t *slots, uint64_t mask, uint64_t key, uint64_t i,
                                                      bool &waited_out) {
        uint64_t s = slot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const uint64_t kk = slots[2 * s];
            if (kk == key || kk == kEmptyKey) {
                uint64_t ok, oid;
                cas_pair(slots + 2 * s, kEmptyKey, kEmptyKey, key, i, ok, oid);
                if (ok == kEmptyKey) return i;
                if (ok == key) return oid;
            }
            s = (s + 1) & mask;
        }
        waited_out = false;
        return kEmptyKey;
    }
    // id of key or -1; the table is read-only while this runs
    __device__ static __forceinline__ int64_t find(const uint64_t *__restrict__ slots, uint64_t mask, uint64_t key) {
        uint64_t s = slot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const ulonglong2 e = __ldg(reinterpret_cast<const ulonglong2 *>(slots) + s);
            if (e.x == key) return (int64_t)e.y;
            if (e.x == kEmptyKey) return -1;
            s = (s + 1) & mask;
        }
        return -1;
    }
};

template <>
struct ColorTable<u128> {
    static constexpr int kWords = 4;
    __device__ static __forceinline__ uint64_t slot(u128 key, uint64_t mask) {
        return mix64((uint64_t)key ^ ((uint64_t)(key >> 64) * 0x9E3779B97F4A7C15ull)) & mask;
    }
    __device__ static __forceinline__ u128 dumped(const uint64_t *kmers, uint64_t i) {
        return ((u128)kmers[2 * i + 1] << 64) | (u128)kmers[2 * i];
    }
    __device__ static __forceinline__ uint64_t insert(uint64_t *slots, uint64_t mask, u128 key, uint64_t i,
                                                      bool &waited_out) {
        const uint64_t lo = (uint64_t)key, hi = (uint64_t)(key >> 64);
        uint64_t s = slot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            uint64_t *sp = slots + 4 * s;
            // the key pair is only ever read whole, through the compare-and-swap
            uint64_t o0, o1;
            cas_pair(sp, kEmptyKey, kEmptyKey, lo, hi, o0, o1);
            if (o0 == kEmptyKey && o1 == kEmptyKey) {
                st_relaxed_u64(sp + 2, i);
                return i;
            }
            if (o0 == lo && o1 == hi) {
                uint64_t v = ld_relaxed_u64(sp + 2);
                for (int spin = 0; v == kEmptyKey && spin < (1 << 22); spin++) {
                    __nanosleep(32);
                    v = ld_relaxed_u64(sp + 2);
                }
                waited_out = v == kEmptyKey;
                return v;
            }
            s = (s + 1) & mask;
        }
        waited_out = false;
        return kEmptyKey;
    }
    __device__ static __forceinline__ int64_t find(const uint64_t *__restrict__ slots, uint64_t mask, u128 key) {
        const uint64_t lo = (uint64_t)key, hi = (uint64_t)(key >> 64);
        uint64_t s = slot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const ulonglong2 kk = __ldg(reinterpret_cast<const ulonglong2 *>(slots + 4 * s));
            const ulonglong2 id = __ldg(reinterpret_cast<const ulonglong2 *>(slots + 4 * s + 2));
            if (kk.x == lo && kk.y == hi) return (int64_t)id.x;
            if (kk.x == kEmptyKey && kk.y == kEmptyKey) return -1;
            s = (s + 1) & mask;
        }
        return -1;
    }
};

// 1. insert the dumped survivors; owner[i] = id of dump entry i's k-mer (i itself unless the
//    k-mer was dumped twice)
template <typename KT>
__global__ void color_kmer_insert_kernel(const uint64_t *__restrict__ kmers, uint64_t n, uint64_t *slots,
                                         uint64_t mask, uint32_t *owner, unsigned *status) {
    using T = ColorTable<KT>;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        bool waited_out = false;
        const uint64_t own = T::insert(slots, mask, T::dumped(kmers, i), i, waited_out);
        if (own == kEmptyKey) atomicOr(status, waited_out ? kStatusWalkLimit : kStatusTableFull);
        owner[i] = (uint32_t)own;
    }
}

// 2. occurrences: every k-mer of the text sets its sequence's colour bit
constexpr uint64_t kOccMaxRows = 65536;
template <typename KT>
__global__ void __launch_bounds__(256) color_occ_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                       int canonical, uint64_t chunk,
                                                       const uint64_t *__restrict__ seq_off,
                                                       const uint32_t *__restrict__ seq_color, uint64_t n_seq,
                                                       const uint64_t *__restrict__ slots, uint64_t mask,
                                                       uint32_t *bitmaps, int words, uint64_t rows,
                                                       uint64_t row_chunks, int seq_rows) {
    // chunk order: `rows` rows of `row_chunks` chunks walked column by column.  With one row per
    // sequence (seq_rows: row r = sequence r from its first base) chunk c of every sequence is
    // in flight at once, so related genomes touch the same table slots and bitmaps while those
    // are in L2; otherwise the rows are equal slices of the text.
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t column = tid / rows;
    if (column >= row_chunks) return;
    const uint64_t row = tid - column * rows;
    uint64_t x0, x1, seq;
    if (seq_rows) {
        const uint64_t end = row + 1 < n_seq ? seq_off[row + 1] : n;
        x0 = seq_off[row] + column * chunk;
        if (x0 >= end) return;
        x1 = min(x0 + chunk, end);
        seq = row;
    } else {
        x0 = (row * row_chunks + column) * chunk;
        if (x0 >= n) return;
        x1 = min(x0 + chunk, n);
        uint64_t lo = 0, hi = n_seq - 1;  // sequence containing x0
        while (lo < hi) {
            const uint64_t mid = (lo + hi + 1) >> 1;
            if (seq_off[mid] <= x0) lo = mid; else hi = mid - 1;
        }
        seq = lo;
    }
    uint64_t next_off = seq + 1 < n_seq ? seq_off[seq + 1] : ~0ull;
    uint32_t col = seq_color[seq];
    const KT kmask = KeyOps<KT>::mask(k);
    KT fw = 0, rc = 0;
    uint64_t run = 0;
    const uint64_t pend = min(x1 + (uint64_t)k - 1, n);
    // the text is read 16 bytes per aligned load into registers: one byte per load would
    // refetch each sector from DRAM, as the table traffic evicts it
    for (uint64_t q = x0; q < pend;) {
        uint64_t wlo, whi;
        int nb;
        if (((reinterpret_cast<uintptr_t>(text) + q) & 15u) == 0 && q + 16 <= n) {
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(text + q));
            wlo = (uint64_t)v.x | ((uint64_t)v.y << 32);
            whi = (uint64_t)v.z | ((uint64_t)v.w << 32);
            nb = pend - q < 16 ? (int)(pend - q) : 16;
        } else {
            wlo = text[q];
            whi = 0;
            nb = 1;
        }
        for (int j = 0; j < nb; j++) {
            const uint32_t c = (uint32_t)(wlo & 0xffu);
            wlo = (wlo >> 8) | (whi << 56);
            whi >>= 8;
            const uint32_t u = c & 0xDFu;
            if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
                run = 0;
                continue;
            }
            const uint32_t b = (c >> 1) & 3u;
            fw = (fw >> 2) | ((KT)b << (2 * (k - 1)));
            rc = ((rc << 2) | (KT)(b ^ 2u)) & kmask;
            if (++run < (uint64_t)k) continue;
            const uint64_t start = q + j + 1 - (uint64_t)k;
            while (start >= next_off) {
                seq++;
                next_off = seq + 1 < n_seq ? seq_off[seq + 1] : ~0ull;
                col = seq_color[seq];
            }
            const int64_t id = ColorTable<KT>::find(slots, mask, (canonical && rc < fw) ? rc : fw);
            if (id < 0) continue;  // not a surviving k-mer
            atomicOr(&bitmaps[(uint64_t)id * words + (col >> 5)], 1u << (col & 31));
        }
        q += nb;
    }
}

__device__ __forceinline__ uint64_t bitmap_hash(const uint32_t *bm, int words) {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    for (int w = 0; w < words; w++) h = mix64(h ^ (bm[w] + 0x632be59bd9b4e019ull * (uint64_t)(w + 1)));
    return h | 1ull;  // never 0 (0 marks an empty subset slot)
}

// 3. subset dedup: a subset slot holds (hash, state) and its bitmap in the arena; the
//    inserting thread publishes the bitmap before the ready flag, readers wait (bounded)
//    for ready and compare the whole bitmap, so equal hashes of different sets stay apart.
//    Ids with an empty bitmap are holes (see the k-mer table) and get no subset.
__global__ void color_subset_kernel(const uint32_t *__restrict__ bitmaps, uint64_t n_ids, int words,
                                    unsigned long long *sub_hash, uint32_t *sub_state, uint32_t *sub_arena,
                                    uint64_t sub_mask, unsigned long long *sub_count, uint32_t *id_subset,
                                    unsigned *status) {
    for (uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; id < n_ids;
         id += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t *bm = bitmaps + id * words;
        uint32_t any = 0;
        for (int w = 0; w < words; w++) any |= bm[w];
        if (!any) {
            id_subset[id] = 0xffffffffu;
            continue;
        }
        const uint64_t h = bitmap_hash(bm, words);
        uint64_t s = h & sub_mask;
        uint32_t result = 0xffffffffu;
        for (uint64_t probe = 0; probe <= sub_mask && result == 0xffffffffu; probe++) {
            unsigned long long cur = sub_hash[s];
            if (cur == 0ull) {
                cur = atomicCAS(&sub_hash[s], 0ull, (unsigned long long)h);
                if (cur == 0ull) {
                    // claimed: a new id (one counter atomic for the threads claiming together),
                    // its bitmap in the arena, then the ready flag
                    const cg::coalesced_group g = cg::coalesced_threads();
                    unsigned long long base = 0;
                    if (g.thread_rank() == 0) base = atomicAdd(sub_count, (unsigned long long)g.size());
                    const unsigned long long sid = g.shfl(base, 0) + g.thread_rank();
                    for (int w = 0; w < words; w++) sub_arena[sid * words + w] = bm[w];
                    __threadfence();
                    atomicExch(&sub_state[s], (uint32_t)sid | 0x80000000u);
                    result = (uint32_t)sid;
                    break;
                }
            }
            if (cur == h) {
                // acquire load, not an atomic: the popular subsets (one colour, all colours) are
                // polled by millions of threads, and same-address atomics serialise in L2
                uint32_t st = ld_acquire_u32(&sub_state[s]);
                for (int spin = 0; !(st & 0x80000000u) && spin < (1 << 22); spin++) {
                    __nanosleep(32);
                    st = ld_acquire_u32(&sub_state[s]);
                }
                if (!(st & 0x80000000u)) {
                    atomicOr(status, kStatusWalkLimit);  // the waited-for publisher never finished
                    break;
                }
                const uint64_t sid = st & 0x7fffffffu;
                bool same = true;
                for (int w = 0; w < words && same; w++) same = sub_arena[sid * words + w] == bm[w];
                if (same) {
                    result = (uint32_t)sid;
                    break;
                }
            }
            s = (s + 1) & sub_mask;
        }
        if (result == 0xffffffffu) atomicOr(status, kStatusTableFull);
        id_subset[id] = result;
    }
}

// Colours collected by the merge: every dumped copy of a k-mer holds the colours of the
// occurrences its sub-bucket saw (its own sub-bucket sees all of them, a neighbouring one only
// the occurrences where it is a superkmer's ignored end); the union goes to the owner's row,
// and the other copies' rows are cleared so that they are holes for the subset pass.
__global__ void color_union_copies_kernel(const uint32_t *__restrict__ owner, uint64_t n, int words,
                                          uint32_t *bitmaps) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t o = owner[i];
        if (o == i) continue;
        for (int w = 0; w < words; w++) {
            const uint32_t v = bitmaps[i * words + w];
            if (v) atomicOr(&bitmaps[o * words + w], v);
            bitmaps[i * words + w] = 0u;
        }
    }
}

// subset id of every dumped k-mer: a gather through its owner (almost always itself)
__global__ void color_dump_subsets_kernel(const uint32_t *__restrict__ owner, uint64_t n,
                                          const uint32_t *__restrict__ id_subset, uint32_t *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = id_subset[owner[i]];
}

// ---------------------------------------------------------------------------
int launch_color_phase_collected(const uint64_t *dump, uint64_t n_dump, int wide, int words, uint64_t *slots,
                                 uint64_t mask, uint32_t *owner, uint32_t *bitmaps, unsigned long long *sub_count,
                                 unsigned long long *sub_hash, uint32_t *sub_state, uint32_t *sub_arena,
                                 uint64_t sub_mask, uint32_t *id_subset, uint32_t *dump_subset, unsigned *status,
                                 int sms, cudaStream_t s) {
    if (!n_dump) return 0;
    if (wide)
        color_kmer_insert_kernel<u128><<<sms * 8, 256, 0, s>>>(dump, n_dump, slots, mask, owner, status);
    else
        color_kmer_insert_kernel<uint64_t><<<sms * 8, 256, 0, s>>>(dump, n_dump, slots, mask, owner, status);
    color_union_copies_kernel<<<sms * 8, 256, 0, s>>>(owner, n_dump, words, bitmaps);
    color_subset_kernel<<<sms * 8, 256, 0, s>>>(bitmaps, n_dump, words, sub_hash, sub_state, sub_arena, sub_mask,
                                                sub_count, id_subset, status);
    color_dump_subsets_kernel<<<sms * 8, 256, 0, s>>>(owner, n_dump, id_subset, dump_subset);
    return 4;
}

int launch_color_phase(const uint64_t *dump, uint64_t n_dump, const uint8_t *text, uint64_t n_text, int k,
                       int canonical, int wide, const uint64_t *seq_off, const uint32_t *seq_color,
                       uint64_t n_seq, uint64_t max_seq_len, int words, uint64_t *slots, uint64_t mask, uint32_t *owner, uint32_t *bitmaps,
                       unsigned long long *sub_count, unsigned long long *sub_hash, uint32_t *sub_state,
                       uint32_t *sub_arena, uint64_t sub_mask, uint32_t *id_subset, uint32_t *dump_subset,
                       unsigned *status, int sms, cudaStream_t s) {
    int n = 0;
    if (n_dump) {
        if (wide)
            color_kmer_insert_kernel<u128><<<sms * 8, 256, 0, s>>>(dump, n_dump, slots, mask, owner, status);
        else
            color_kmer_insert_kernel<uint64_t><<<sms * 8, 256, 0, s>>>(dump, n_dump, slots, mask, owner, status);
        n++;
    }
    const uint64_t chunk = 256;
    const uint64_t chunks = (n_text + chunk - 1) / chunk;
    if (chunks && n_dump) {
        // collections of genomes: one row per sequence, from its first base, when the lengths
        // are alike (rows x the longest sequence's chunks <= 2 x the text's chunks); else equal
        // slices of the text, one per sequence; read sets (many sequences) keep text order
        const uint64_t max_chunks = (max_seq_len + chunk - 1) / chunk;
        const int seq_rows = max_seq_len > 0 && n_seq <= kOccMaxRows && n_seq * max_chunks <= 2 * chunks;
        const uint64_t rows =
            seq_rows ? n_seq : std::max<uint64_t>(1, std::min<uint64_t>(n_seq <= kOccMaxRows ? n_seq : 1, chunks));
        const uint64_t row_chunks = seq_rows ? max_chunks : (chunks + rows - 1) / rows;
        const uint64_t threads = rows * row_chunks;
        const unsigned grid = (unsigned)((threads + 255) / 256);
        if (wide)
            color_occ_kernel<u128><<<grid, 256, 0, s>>>(text, n_text, k, canonical, chunk, seq_off, seq_color, n_seq,
                                                        slots, mask, bitmaps, words, rows, row_chunks, seq_rows);
        else
            color_occ_kernel<uint64_t><<<grid, 256, 0, s>>>(text, n_text, k, canonical, chunk, seq_off, seq_color,
                                                            n_seq, slots, mask, bitmaps, words, rows, row_chunks,
                                                            seq_rows);
        n++;
    }
    if (n_dump) {
        color_subset_kernel<<<sms * 8, 256, 0, s>>>(bitmaps, n_dump, words, sub_hash, sub_state, sub_arena, sub_mask,
                                                    sub_count, id_subset, status);
        color_dump_subsets_kernel<<<sms * 8, 256, 0, s>>>(owner, n_dump, id_subset, dump_subset);
        n += 2;
    }
    return n;
}

}  // namespace ggcat
