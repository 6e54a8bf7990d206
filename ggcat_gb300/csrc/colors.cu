// Colour-subset deduplication on sm_103a.
//
// Replaces the per-k-mer colour collection and subset dedup of the reference's
// MultipleColorsManager (crates/colors/src/managers/multiple.rs:99-228: colours of every
// occurrence are collected per k-mer, sorted, deduplicated, and the set is mapped to a
// subset id by ColorsMemMapWriter::get_id, crates/colors/src/colors_memmap_writer.rs:43-61).
// A k-mer's colour set is the set of colours (input files) of all its occurrences, which
// this phase computes globally instead of per bucket:
//   1. the surviving k-mers of the merge go into one device table (key -> dense id),
//   2. one pass over the input text sets bit `colour` of the k-mer's bitmap for every
//      occurrence (the occurrence's colour is that of the sequence containing it),
//   3. every bitmap is deduplicated into a subset table (exact: hash, then compare).
// Subset ids are assigned in arrival order (as in the reference they are not deterministic);
// the sets they decode to are.
#include "common.cuh"
#include "kernels.h"

namespace ggcat {

__device__ __forceinline__ uint64_t cslot(uint64_t key, uint64_t mask) { return mix64(key) & mask; }

// 1a. insert the dumped survivors (duplicates across sub-buckets collapse)
__global__ void color_kmer_insert_kernel(const uint64_t *__restrict__ kmers, uint64_t n, uint64_t *keys,
                                         uint32_t *vals, uint64_t mask, unsigned *status) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = kmers[i];
        uint64_t s = cslot(key, mask);
        for (uint64_t probe = 0;; probe++) {
            if (probe > mask) {
                atomicOr(status, kStatusTableFull);
                break;
            }
            const uint64_t kk = keys[s];
            if (kk == key) break;
            if (kk == kEmptyKey) {
                const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long *>(&keys[s]),
                                                         (unsigned long long)kEmptyKey, (unsigned long long)key);
                if (old == kEmptyKey || old == key) break;
            }
            s = (s + 1) & mask;
        }
    }
}

// 1b. dense ids for the occupied slots (warp-aggregated counter)
__global__ void color_kmer_number_kernel(const uint64_t *__restrict__ keys, uint32_t *vals, uint64_t cap,
                                         unsigned long long *counter) {
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < cap; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t s = base + threadIdx.x;
        const bool occ = s < cap && keys[s] != kEmptyKey;
        const unsigned bm = __ballot_sync(0xffffffffu, occ);
        const int lane = threadIdx.x & 31;
        unsigned long long b = 0;
        if (lane == 0 && bm) b = atomicAdd(counter, (unsigned long long)__popc(bm));
        b = __shfl_sync(0xffffffffu, b, 0);
        if (occ) vals[s] = (uint32_t)(b + __popc(bm & ((1u << lane) - 1u)));
    }
}

__device__ __forceinline__ int64_t color_find(const uint64_t *keys, uint64_t mask, uint64_t key) {
    uint64_t s = cslot(key, mask);
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const uint64_t kk = keys[s];
        if (kk == key) return (int64_t)s;
        if (kk == kEmptyKey) return -1;
        s = (s + 1) & mask;
    }
    return -1;
}

// 2. occurrences: every k-mer of the text sets its sequence's colour bit
__global__ void __launch_bounds__(256) color_occ_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                       uint64_t chunk, const uint64_t *__restrict__ seq_off,
                                                       const uint32_t *__restrict__ seq_color, uint64_t n_seq,
                                                       const uint64_t *__restrict__ keys,
                                                       const uint32_t *__restrict__ vals, uint64_t mask,
                                                       uint32_t *bitmaps, int words) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    uint64_t lo = 0, hi = n_seq - 1;  // sequence containing x0
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (seq_off[mid] <= x0) lo = mid; else hi = mid - 1;
    }
    uint64_t seq = lo;
    const uint64_t kmask = kmer_mask(k);
    uint64_t fw = 0, rc = 0, run = 0;
    const uint64_t pend = min(x1 + (uint64_t)k - 1, n);
    for (uint64_t p = x0; p < pend; p++) {
        const uint32_t c = text[p];
        const uint32_t u = c & 0xDFu;
        if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
            run = 0;
            continue;
        }
        const uint64_t b = (c >> 1) & 3u;
        fw = (fw >> 2) | (b << (2 * (k - 1)));
        rc = ((rc << 2) | (b ^ 2u)) & kmask;
        if (++run < (uint64_t)k) continue;
        const uint64_t start = p + 1 - (uint64_t)k;
        while (seq + 1 < n_seq && seq_off[seq + 1] <= start) seq++;
        const int64_t s = color_find(keys, mask, fw < rc ? fw : rc);
        if (s < 0) continue;  // not a surviving k-mer
        const uint32_t col = seq_color[seq];
        atomicOr(&bitmaps[(uint64_t)vals[s] * words + (col >> 5)], 1u << (col & 31));
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
__global__ void color_subset_kernel(const uint32_t *__restrict__ bitmaps, const unsigned long long *n_ids_dev, int words,
                                    unsigned long long *sub_hash, uint32_t *sub_state, uint32_t *sub_arena,
                                    uint64_t sub_mask, unsigned long long *sub_count, uint32_t *id_subset,
                                    unsigned *status) {
    const uint64_t n_ids = *n_ids_dev;
    for (uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; id < n_ids;
         id += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t *bm = bitmaps + id * words;
        const uint64_t h = bitmap_hash(bm, words);
        uint64_t s = h & sub_mask;
        uint32_t result = 0xffffffffu;
        for (uint64_t probe = 0; probe <= sub_mask && result == 0xffffffffu; probe++) {
            unsigned long long cur = sub_hash[s];
            if (cur == 0ull) {
                cur = atomicCAS(&sub_hash[s], 0ull, (unsigned long long)h);
                if (cur == 0ull) {
                    // claimed: a new id, its bitmap in the arena, then the ready flag
                    const unsigned long long sid = atomicAdd(sub_count, 1ull);
                    for (int w = 0; w < words; w++) sub_arena[sid * words + w] = bm[w];
                    __threadfence();
                    atomicExch(&sub_state[s], (uint32_t)sid | 0x80000000u);
                    result = (uint32_t)sid;
                    break;
                }
            }
            if (cur == h) {
                uint32_t st = 0;
                for (int spin = 0; spin < (1 << 22); spin++) {
                    st = atomicAdd(&sub_state[s], 0u);
                    if (st & 0x80000000u) break;
                    __nanosleep(32);
                }
                if (!(st & 0x80000000u)) {
                    atomicOr(status, kStatusWalkLimit);  // the waited-for publisher never finished
                    break;
                }
                __threadfence();
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

// subset id of every dumped k-mer
__global__ void color_dump_subsets_kernel(const uint64_t *__restrict__ kmers, uint64_t n,
                                          const uint64_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                          uint64_t mask, const uint32_t *__restrict__ id_subset, uint32_t *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t s = color_find(keys, mask, kmers[i]);
        out[i] = s < 0 ? 0xffffffffu : id_subset[vals[s]];
    }
}

// per k-mer start position of a text (e.g. the final unitigs): subset id or ~0
__global__ void __launch_bounds__(256) color_text_subsets_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                                uint64_t chunk, const uint64_t *__restrict__ keys,
                                                                const uint32_t *__restrict__ vals, uint64_t mask,
                                                                const uint32_t *__restrict__ id_subset,
                                                                uint32_t *out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    const uint64_t kmask = kmer_mask(k);
    uint64_t fw = 0, rc = 0, run = 0;
    for (uint64_t p = x0; p < x1; p++) out[p] = 0xffffffffu;
    const uint64_t pend = min(x1 + (uint64_t)k - 1, n);
    for (uint64_t p = x0; p < pend; p++) {
        const uint32_t c = text[p];
        const uint32_t u = c & 0xDFu;
        if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
            run = 0;
            continue;
        }
        const uint64_t b = (c >> 1) & 3u;
        fw = (fw >> 2) | (b << (2 * (k - 1)));
        rc = ((rc << 2) | (b ^ 2u)) & kmask;
        if (++run < (uint64_t)k) continue;
        const uint64_t start = p + 1 - (uint64_t)k;
        const int64_t s = color_find(keys, mask, fw < rc ? fw : rc);
        out[start] = s < 0 ? 0xffffffffu : id_subset[vals[s]];
    }
}

// ---------------------------------------------------------------------------
int launch_color_phase(const uint64_t *dump, uint64_t n_dump, const uint8_t *text, uint64_t n_text, int k,
                       const uint64_t *seq_off, const uint32_t *seq_color, uint64_t n_seq, int words, uint64_t *keys,
                       uint32_t *vals, uint64_t mask, uint32_t *bitmaps, unsigned long long *counters,
                       unsigned long long *sub_hash, uint32_t *sub_state, uint32_t *sub_arena, uint64_t sub_mask,
                       uint32_t *id_subset, uint32_t *dump_subset, unsigned *status, uint64_t n_ids_upper, int sms,
                       cudaStream_t s) {
    int n = 0;
    color_kmer_insert_kernel<<<sms * 8, 256, 0, s>>>(dump, n_dump, keys, vals, mask, status);
    n++;
    color_kmer_number_kernel<<<sms * 8, 256, 0, s>>>(keys, vals, mask + 1, counters);
    n++;
    const uint64_t chunk = 256;
    const uint64_t threads = (n_text + chunk - 1) / chunk;
    if (threads) {
        color_occ_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(text, n_text, k, chunk, seq_off, seq_color,
                                                                          n_seq, keys, vals, mask, bitmaps, words);
        n++;
    }
    (void)n_ids_upper;
    color_subset_kernel<<<sms * 8, 256, 0, s>>>(bitmaps, counters, words, sub_hash, sub_state, sub_arena, sub_mask,
                                                counters + 1, id_subset, status);
    n++;
    color_dump_subsets_kernel<<<sms * 8, 256, 0, s>>>(dump, n_dump, keys, vals, mask, id_subset, dump_subset);
    n++;
    return n;
}

int launch_color_text_subsets(const uint8_t *text, uint64_t n, int k, const uint64_t *keys, const uint32_t *vals,
                              uint64_t mask, const uint32_t *id_subset, uint32_t *out, cudaStream_t s) {
    const uint64_t chunk = 256;
    const uint64_t threads = (n + chunk - 1) / chunk;
    if (!threads) return 0;
    color_text_subsets_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(text, n, k, chunk, keys, vals, mask,
                                                                               id_subset, out);
    return 1;
}

}  // namespace ggcat
