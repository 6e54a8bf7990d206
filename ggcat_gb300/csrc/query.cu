// Graph query lookup on sm_103a.
//
// Replaces the querier's k-mer lookup (ParallelKmersQueryMapProcessor / FinalExecutor,
// crates/querier/src/pipeline/parallel_kmers_query.rs:362-471, with the bucketing of
// querier_minimizer_bucketing.rs:182-230 and the per-query sums of counters_sorting.rs:106-273).
// The reference buckets graph and query k-mers by minimizer so each lookup is local to a
// sub-bucket; here the graph's canonical k-mers stay resident in one device hash table, so a
// query k-mer is one probe and no bucketing pass is needed.  Every query k-mer occurrence
// that does not span a non-ACGT base is looked up (duplicates included), and the matches of
// each query are summed (per colour subset when the graph is coloured).
#include "common.cuh"
#include "kernels.h"

namespace ggcat {

__device__ __forceinline__ uint32_t qslot(uint64_t key, uint64_t mask) { return (uint32_t)(mix64(key) & mask); }

// Insert every canonical k-mer of the graph text (pieces separated by non-ACGT bytes) with the
// colour subset of its sequence (subset_of_seq[seq], seq from a binary search of seq_off) or 0.
__global__ void __launch_bounds__(256) index_insert_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                           uint64_t chunk, const uint64_t *__restrict__ seq_off,
                                                           const uint32_t *__restrict__ seq_subset, uint64_t n_seq,
                                                           uint64_t *keys, uint32_t *vals, uint64_t mask,
                                                           unsigned *status) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;  // k-mer start positions [x0, x1)
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    const uint64_t kmask = kmer_mask(k);
    uint64_t fw = 0, rc = 0, run = 0;
    uint64_t seq = 0;
    if (seq_subset) {  // sequence containing x0
        uint64_t lo = 0, hi = n_seq - 1;
        while (lo < hi) {
            const uint64_t mid = (lo + hi + 1) >> 1;
            if (seq_off[mid] <= x0) lo = mid; else hi = mid - 1;
        }
        seq = lo;
    }
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
        if (seq_subset)
            while (seq + 1 < n_seq && seq_off[seq + 1] <= start) seq++;
        const uint64_t key = fw < rc ? fw : rc;
        uint64_t s = qslot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const uint64_t kk = keys[s];
            if (kk == key) break;
            if (kk == kEmptyKey) {
                const unsigned long long old = atomicCAS(reinterpret_cast<unsigned long long *>(&keys[s]),
                                                         (unsigned long long)kEmptyKey, (unsigned long long)key);
                if (old == kEmptyKey) {
                    vals[s] = seq_subset ? seq_subset[seq] : 0u;
                    break;
                }
                if (old == key) break;
            }
            s = (s + 1) & mask;
            if (probe == mask) atomicOr(status, kStatusTableFull);
        }
    }
}

// One work item = a run of k-mer positions of one query.  Matches are summed per query;
// with a coloured graph, runs of equal subset ids are emitted as (query, subset, count).
__global__ void __launch_bounds__(256) query_kernel(const uint8_t *__restrict__ text, int k,
                                                   const uint32_t *__restrict__ item_query,
                                                   const uint64_t *__restrict__ item_start,
                                                   const uint32_t *__restrict__ item_len, uint64_t n_items,
                                                   const uint64_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                                   uint64_t mask, unsigned long long *__restrict__ matched,
                                                   int colored, uint4 *__restrict__ runs, unsigned long long runs_cap,
                                                   unsigned long long *__restrict__ runs_cursor,
                                                   unsigned *__restrict__ status) {
    const uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n_items) return;
    const uint32_t q = item_query[it];
    const uint64_t x0 = item_start[it];
    const uint64_t x1 = x0 + item_len[it];  // k-mer start positions
    const uint64_t kmask = kmer_mask(k);
    uint64_t fw = 0, rc = 0, run = 0, hits = 0;
    uint32_t cur_subset = 0xffffffffu, cur_count = 0;
    auto flush_run = [&]() {
        if (cur_count == 0) return;
        const unsigned long long i = atomicAdd(runs_cursor, 1ull);
        if (i < runs_cap)
            runs[i] = make_uint4(q, cur_subset, cur_count, 0u);
        else
            atomicOr(status, kStatusOutOverflow);
        cur_count = 0;
    };
    for (uint64_t p = x0; p < x1 + (uint64_t)k - 1; p++) {
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
        const uint64_t key = fw < rc ? fw : rc;
        uint64_t s = qslot(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const uint64_t kk = keys[s];
            if (kk == key) {
                hits++;
                if (colored) {
                    const uint32_t sub = vals[s];
                    if (sub != cur_subset) {
                        flush_run();
                        cur_subset = sub;
                    }
                    cur_count++;
                }
                break;
            }
            if (kk == kEmptyKey) break;
            s = (s + 1) & mask;
        }
    }
    if (colored) flush_run();
    if (hits) atomicAdd(&matched[q], (unsigned long long)hits);
}

int launch_index_insert(const uint8_t *text, uint64_t n, int k, const uint64_t *seq_off, const uint32_t *seq_subset,
                        uint64_t n_seq, uint64_t *keys, uint32_t *vals, uint64_t mask, unsigned *status, cudaStream_t s) {
    const uint64_t chunk = 256;
    const uint64_t threads = (n + chunk - 1) / chunk;
    if (threads == 0) return 0;
    index_insert_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(text, n, k, chunk, seq_off, seq_subset, n_seq,
                                                                          keys, vals, mask, status);
    return 1;
}

int launch_query(const uint8_t *text, int k, const uint32_t *item_query, const uint64_t *item_start,
                 const uint32_t *item_len, uint64_t n_items, const uint64_t *keys, const uint32_t *vals, uint64_t mask,
                 unsigned long long *matched, int colored, uint4 *runs, unsigned long long runs_cap,
                 unsigned long long *runs_cursor, unsigned *status, cudaStream_t s) {
    if (n_items == 0) return 0;
    query_kernel<<<(unsigned)((n_items + 255) / 256), 256, 0, s>>>(text, k, item_query, item_start, item_len, n_items,
                                                                  keys, vals, mask, matched, colored, runs, runs_cap,
                                                                  runs_cursor, status);
    return 1;
}

}  // namespace ggcat
