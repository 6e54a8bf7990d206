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
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace ggcat {

__device__ __forceinline__ uint32_t qslot(uint64_t key, uint64_t mask) { return (uint32_t)(mix64(key) & mask); }

// slot of a key in the uncoloured index (u64 keys for k <= 32, u128 for k <= 64)
__device__ __forceinline__ uint32_t qslot_key(uint64_t key, uint64_t mask) { return qslot(key, mask); }
__device__ __forceinline__ uint32_t qslot_key(u128 key, uint64_t mask) {
    return (uint32_t)(mix64((uint64_t)key ^ ((uint64_t)(key >> 64) * 0x9E3779B97F4A7C15ull)) & mask);
}

// Insert every canonical k-mer of the graph text (pieces separated by non-ACGT bytes); the
// value of the k-mer starting at text position p is pos_val[p] (the colour subset of a coloured
// graph's k-mer), or 0 without pos_val.
template <typename KT>
__global__ void __launch_bounds__(256) index_insert_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                           uint64_t chunk, const uint32_t *__restrict__ pos_val,
                                                           KT *keys, uint32_t *vals, uint64_t mask,
                                                           unsigned *status) {
    using K = KeyOps<KT>;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;  // k-mer start positions [x0, x1)
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    const KT kmask = K::mask(k);
    KT fw = 0, rc = 0;
    uint64_t run = 0;
    const uint64_t pend = min(x1 + (uint64_t)k - 1, n);
    for (uint64_t p = x0; p < pend; p++) {
        const uint32_t c = text[p];
        const uint32_t u = c & 0xDFu;
        if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
            run = 0;
            continue;
        }
        const uint32_t b = (c >> 1) & 3u;
        fw = (fw >> 2) | ((KT)b << (2 * (k - 1)));
        rc = ((rc << 2) | (KT)(b ^ 2u)) & kmask;
        if (++run < (uint64_t)k) continue;
        const KT key = fw < rc ? fw : rc;
        uint64_t s = qslot_key(key, mask);
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const KT kk = keys[s];
            if (kk == key) break;
            if (kk == K::empty()) {
                const KT old = K::cas(&keys[s], K::empty(), key);
                if (old == K::empty()) {
                    vals[s] = pos_val ? pos_val[p + 1 - (uint64_t)k] : 0u;
                    break;
                }
                if (old == key) break;
            }
            s = (s + 1) & mask;
            if (probe == mask) atomicOr(status, kStatusTableFull);
        }
    }
}

// Coloured index: the colour phase's k-mer table ({key, id} slots: 2 words for u64 keys, 4
// for u128) re-keyed into the query table with value = colour subset id.
template <typename KT>
__global__ void index_from_colors_kernel(const uint64_t *__restrict__ cslots, uint64_t ccap,
                                         const uint32_t *__restrict__ id_subset, KT *keys, uint32_t *vals,
                                         uint64_t mask, unsigned *status) {
    using K = KeyOps<KT>;
    constexpr int kSlotWords = sizeof(KT) == 8 ? 2 : 4;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ccap; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t *e = cslots + kSlotWords * i;
        KT key;
        if constexpr (sizeof(KT) == 8) key = e[0];
        else key = ((u128)e[1] << 64) | (u128)e[0];
        if (key == K::empty()) continue;
        const uint32_t id = (uint32_t)e[kSlotWords / 2];
        uint64_t s = qslot_key(key, mask);
        for (uint64_t probe = 0;; probe++) {
            if (probe > mask) {
                atomicOr(status, kStatusTableFull);
                break;
            }
            if (keys[s] == K::empty()) {
                const KT old = K::cas(&keys[s], K::empty(), key);
                if (old == K::empty()) {
                    vals[s] = id_subset[id];
                    break;
                }
            }
            s = (s + 1) & mask;
        }
    }
}

// Lookups of an uncoloured query run are issued four at a time: the canonical keys of the next
// four valid k-mers are rolled first, their first slots loaded together, and only collisions
// probe on (one round trip to memory per four k-mers instead of one per k-mer).
constexpr int kQueryIlp = 4;

// slot of key in the index given its first probe's key (first); -1 when absent
template <typename KT>
__device__ __forceinline__ int64_t query_resolve(const KT *__restrict__ keys, uint64_t mask, const KT &key, uint64_t s,
                                                 const KT &first) {
    using K = KeyOps<KT>;
    if (first == key) return (int64_t)s;
    if (first == K::empty()) return -1;
    for (uint64_t probe = 1; probe <= mask; probe++) {
        s = (s + 1) & mask;
        const KT kk = keys[s];
        if (kk == key) return (int64_t)s;
        if (kk == K::empty()) return -1;
    }
    return -1;
}

// One work item = a run of k-mer positions of one query; matches are summed per query.
template <typename KT>
__global__ void __launch_bounds__(256) query_kernel(const uint8_t *__restrict__ text, int k,
                                                   const uint32_t *__restrict__ item_query,
                                                   const uint64_t *__restrict__ item_start,
                                                   const uint32_t *__restrict__ item_len, uint64_t n_items,
                                                   const KT *__restrict__ keys, uint64_t mask,
                                                   unsigned long long *__restrict__ matched) {
    using K = KeyOps<KT>;
    const uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n_items) return;
    const uint32_t q = item_query[it];
    const uint64_t x0 = item_start[it];
    const uint64_t x1 = x0 + item_len[it];  // k-mer start positions
    const KT kmask = K::mask(k);
    KT fw = 0, rc = 0;
    uint64_t run = 0, hits = 0;
    const uint64_t pend = x1 + (uint64_t)k - 1;
    uint64_t p = x0;
    for (;;) {
        KT key[kQueryIlp];
        int nk = 0;
#pragma unroll
        for (int j = 0; j < kQueryIlp; j++) {  // (static indices keep key[] in registers)
            bool got = false;
            while (!got && p < pend) {
                const uint32_t c = text[p++];
                const uint32_t u = c & 0xDFu;
                if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
                    run = 0;
                    continue;
                }
                const uint32_t b = (c >> 1) & 3u;
                fw = (fw >> 2) | ((KT)b << (2 * (k - 1)));
                rc = ((rc << 2) | (KT)(b ^ 2u)) & kmask;
                if (++run >= (uint64_t)k) got = true;
            }
            if (!got) break;
            key[j] = fw < rc ? fw : rc;
            nk = j + 1;
        }
        if (nk == 0) break;
        uint64_t sl[kQueryIlp];
        KT first[kQueryIlp];
#pragma unroll
        for (int j = 0; j < kQueryIlp; j++)
            if (j < nk) {
                sl[j] = qslot_key(key[j], mask);
                first[j] = keys[sl[j]];
            }
#pragma unroll
        for (int j = 0; j < kQueryIlp; j++)
            if (j < nk && query_resolve(keys, mask, key[j], sl[j], first[j]) >= 0) hits++;
    }
    if (hits) atomicAdd(&matched[q], (unsigned long long)hits);
}

// Coloured lookup for up to 32 * W colours (W bitmap words per subset), one warp per work item
// (a run of at most kColorChunk k-mer positions of one query; colored_query_output.rs:264-309
// sums the per-subset counters of a query per colour).  Each lane rolls a contiguous span of
// the run and merges its consecutive equal subset ids; a changed id is emitted with its
// multiplicity: the lane stages the subset's words in shared memory and the warp walks the
// emitting lanes, lane l adding bit l of every word (colours 32 w + l) into its own register
// counters.  Counting therefore costs ~3 W instructions per emitted run and no atomics; each
// item adds its counters to the query's row once.
constexpr uint32_t kColorChunk = 4096;
constexpr int kColorWarps = 8;  // warps per CTA

template <typename KT, int W>
__global__ void __launch_bounds__(32 * kColorWarps) query_color_warp_kernel(
    const uint8_t *__restrict__ text, int k, const uint32_t *__restrict__ item_query,
    const uint64_t *__restrict__ item_start, const uint32_t *__restrict__ item_len, uint64_t n_items,
    const KT *__restrict__ keys, const uint32_t *__restrict__ vals, uint64_t mask,
    const uint32_t *__restrict__ sub_arena, int words, uint32_t n_colors, unsigned long long *__restrict__ matched,
    unsigned long long *__restrict__ counts) {
    using K = KeyOps<KT>;
    constexpr uint32_t kNone = 0xffffffffu;
    __shared__ __align__(16) uint32_t stage[kColorWarps][32][W];
    __shared__ uint32_t stage_mult[kColorWarps][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const KT kmask = K::mask(k);
    const uint64_t nwarps = (uint64_t)gridDim.x * kColorWarps;
    for (uint64_t it = (uint64_t)blockIdx.x * kColorWarps + wib; it < n_items; it += nwarps) {
        const uint32_t q = item_query[it];
        const uint64_t x0 = item_start[it];
        const uint32_t len = item_len[it];
        const uint32_t per = (len + 31) / 32;
        const uint32_t a = min(len, (uint32_t)lane * per), b = min(len, a + per);
        uint32_t cnt[W];
#pragma unroll
        for (int w = 0; w < W; w++) cnt[w] = 0;
        // warp-collective: adds every emitting lane's run (e_sub, e_mult) to the counters
        auto emit = [&](uint32_t e_sub, uint32_t e_mult) {
            const unsigned ball = __ballot_sync(0xffffffffu, e_sub != kNone);
            if (!ball) return;
            if (e_sub != kNone) {
                const uint32_t *bm = sub_arena + (uint64_t)e_sub * (uint64_t)words;
#pragma unroll
                for (int w = 0; w < W; w++) stage[wib][lane][w] = w < words ? bm[w] : 0u;
                stage_mult[wib][lane] = e_mult;
            }
            __syncwarp();
            for (unsigned m = ball; m; m &= m - 1) {
                const int j = __ffs(m) - 1;
                const uint32_t mj = stage_mult[wib][j];
#pragma unroll
                for (int w = 0; w < W; w++) cnt[w] += ((stage[wib][j][w] >> lane) & 1u) * mj;
            }
            __syncwarp();
        };
        KT fw = 0, rc = 0;
        uint32_t run = 0, hits = 0, cur = kNone, mult = 0;
        uint64_t p = x0 + a;
        for (uint32_t i = 0; i < per; i++) {  // the same trip count on every lane
            uint32_t sub = kNone;
            if (a + i < b) {
                const uint64_t e = x0 + a + i + (uint64_t)k - 1;  // last base of k-mer a + i
                while (p <= e) {
                    const uint32_t c = text[p++];
                    const uint32_t u = c & 0xDFu;
                    if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
                        run = 0;
                        continue;
                    }
                    const uint32_t bb = (c >> 1) & 3u;
                    fw = (fw >> 2) | ((KT)bb << (2 * (k - 1)));
                    rc = ((rc << 2) | (KT)(bb ^ 2u)) & kmask;
                    run++;
                }
                if (run >= (uint32_t)k) {
                    const KT key = fw < rc ? fw : rc;
                    const uint64_t s0 = qslot_key(key, mask);
                    const int64_t sl = query_resolve(keys, mask, key, s0, keys[s0]);
                    if (sl >= 0) {
                        sub = vals[sl];
                        hits++;
                    }
                }
            }
            uint32_t e_sub = kNone, e_mult = 0;
            if (sub != cur) {
                e_sub = cur;
                e_mult = mult;
                cur = sub;
                mult = sub != kNone ? 1u : 0u;
            } else if (sub != kNone) {
                mult++;
            }
            emit(e_sub, e_mult);
        }
        emit(cur, mult);
        unsigned long long *row = counts + (uint64_t)q * n_colors;
#pragma unroll
        for (int w = 0; w < W; w++) {
            const uint32_t c = 32u * w + lane;
            if (cnt[w] && c < n_colors) atomicAdd(&row[c], (unsigned long long)cnt[w]);
        }
        for (int o = 16; o; o >>= 1) hits += __shfl_xor_sync(0xffffffffu, hits, o);
        if (lane == 0 && hits) atomicAdd(&matched[q], (unsigned long long)hits);
    }
}

// Coloured lookup for any number of colours, one CTA per query from a device queue: runs of
// equal subset ids are expanded into per-colour counts in shared memory.
template <typename KT>
__global__ void __launch_bounds__(256) query_color_kernel(const uint8_t *__restrict__ text, int k,
                                                         const uint64_t *__restrict__ q_off,
                                                         const uint64_t *__restrict__ q_len, uint64_t nq,
                                                         const KT *__restrict__ keys,
                                                         const uint32_t *__restrict__ vals, uint64_t mask,
                                                         const uint32_t *__restrict__ sub_arena, int words,
                                                         uint32_t n_colors, unsigned long long *__restrict__ matched,
                                                         unsigned long long *__restrict__ counts,
                                                         unsigned long long *__restrict__ queue) {
    using K = KeyOps<KT>;
    extern __shared__ uint32_t cnt[];  // n_colors counters
    __shared__ unsigned long long q_cur;
    __shared__ unsigned long long hits_sh;
    const KT kmask = K::mask(k);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            q_cur = atomicAdd(queue, 1ull);
            hits_sh = 0;
        }
        for (uint32_t c = threadIdx.x; c < n_colors; c += blockDim.x) cnt[c] = 0;
        __syncthreads();
        const uint64_t q = q_cur;
        if (q >= nq) break;
        const uint64_t L = q_len[q];
        const uint64_t nk = L >= (uint64_t)k ? L - (uint64_t)k + 1 : 0;
        const uint64_t per = (nk + blockDim.x - 1) / blockDim.x;
        const uint64_t a = min(nk, (uint64_t)threadIdx.x * per), b = min(nk, a + per);
        KT fw = 0, rc = 0;
        uint64_t run = 0, hits = 0;
        uint32_t cur_sub = 0xffffffffu, cur_cnt = 0;
        auto flush = [&]() {
            if (!cur_cnt) return;
            const uint32_t *bm = sub_arena + (uint64_t)cur_sub * words;
            for (int w = 0; w < words; w++) {
                uint32_t bits = bm[w];
                while (bits) {
                    const int c = __ffs(bits) - 1;
                    bits &= bits - 1;
                    atomicAdd(&cnt[w * 32 + c], cur_cnt);
                }
            }
            cur_cnt = 0;
        };
        if (a < b) {
            const uint64_t base = q_off[q];
            for (uint64_t p = base + a; p < base + b + (uint64_t)k - 1; p++) {
                const uint32_t c = text[p];
                const uint32_t u = c & 0xDFu;
                if (!((u == 'A') | (u == 'C') | (u == 'G') | (u == 'T'))) {
                    run = 0;
                    continue;
                }
                const uint32_t bb = (c >> 1) & 3u;
                fw = (fw >> 2) | ((KT)bb << (2 * (k - 1)));
                rc = ((rc << 2) | (KT)(bb ^ 2u)) & kmask;
                if (++run < (uint64_t)k) continue;
                const KT key = fw < rc ? fw : rc;
                uint64_t s = qslot_key(key, mask);
                for (uint64_t probe = 0; probe <= mask; probe++) {
                    const KT kk = keys[s];
                    if (kk == key) {
                        hits++;
                        const uint32_t sub = vals[s];
                        if (sub != cur_sub) {
                            flush();
                            cur_sub = sub;
                        }
                        cur_cnt++;
                        break;
                    }
                    if (kk == K::empty()) break;
                    s = (s + 1) & mask;
                }
            }
            flush();
        }
        if (hits) atomicAdd(&hits_sh, hits);
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < n_colors; c += blockDim.x) counts[q * n_colors + c] = cnt[c];
        if (threadIdx.x == 0) matched[q] = hits_sh;
    }
}

// Colour subset of every k-mer of the final unitigs, the C: runs of a coloured graph's FASTA
// (UnitigColorData::write_as_ident, crates/colors/src/managers/multiple.rs:705-740).  Item i
// covers k-mers [item_first[i], item_first[i] + item_count[i]) of unitig item_unitig[i]
// (bases[u_off[u], u_off[u] + u_len[u])); k-mer j of unitig u goes to out[kmer_base[u] + j].
// The lookup is the coloured index (canonical k-mer -> subset id); a k-mer missing from it
// gets 0xffffffff.
template <typename KT>
__global__ void __launch_bounds__(256) unitig_subsets_kernel(
    const uint8_t *__restrict__ bases, const uint64_t *__restrict__ u_off, const uint32_t *__restrict__ u_len,
    const uint32_t *__restrict__ item_unitig, const uint32_t *__restrict__ item_first,
    const uint32_t *__restrict__ item_count, uint64_t n_items, const uint64_t *__restrict__ kmer_base, int k,
    const KT *__restrict__ keys, const uint32_t *__restrict__ vals, uint64_t mask, uint32_t *__restrict__ out) {
    using K = KeyOps<KT>;
    const uint64_t it = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= n_items) return;
    const uint32_t u = item_unitig[it], j0 = item_first[it], cnt = item_count[it];
    const uint8_t *seq = bases + u_off[u];
    if ((uint64_t)j0 + cnt + (uint64_t)k - 1 > u_len[u]) return;
    const KT kmask = K::mask(k);
    KT fw = 0, rc = 0;
    uint64_t run = 0;
    for (uint32_t p = j0; p < j0 + cnt + (uint32_t)k - 1; p++) {
        const uint32_t c = seq[p];
        const uint32_t uc = c & 0xDFu;
        if (!((uc == 'A') | (uc == 'C') | (uc == 'G') | (uc == 'T'))) {
            run = 0;
            if (p + 1 >= j0 + (uint32_t)k) out[kmer_base[u] + p + 1 - (uint32_t)k] = 0xffffffffu;
            continue;
        }
        const uint32_t b = (c >> 1) & 3u;
        fw = (fw >> 2) | ((KT)b << (2 * (k - 1)));
        rc = ((rc << 2) | (KT)(b ^ 2u)) & kmask;
        if (++run < (uint64_t)k) {
            if (p + 1 >= j0 + (uint32_t)k) out[kmer_base[u] + p + 1 - (uint32_t)k] = 0xffffffffu;
            continue;
        }
        const KT key = fw < rc ? fw : rc;
        uint64_t sl = qslot_key(key, mask);
        uint32_t sub = 0xffffffffu;
        for (uint64_t probe = 0; probe <= mask; probe++) {
            const KT kk = keys[sl];
            if (kk == key) {
                sub = vals[sl];
                break;
            }
            if (kk == K::empty()) break;
            sl = (sl + 1) & mask;
        }
        out[kmer_base[u] + p + 1 - (uint32_t)k] = sub;
    }
}

int launch_unitig_subsets(const uint8_t *bases, const uint64_t *u_off, const uint32_t *u_len,
                          const uint32_t *item_unitig, const uint32_t *item_first, const uint32_t *item_count,
                          uint64_t n_items, const uint64_t *kmer_base, int k, const void *keys, const uint32_t *vals,
                          uint64_t mask, uint32_t *out, cudaStream_t s) {
    if (n_items == 0) return 0;
    const unsigned grid = (unsigned)((n_items + 255) / 256);
    if (k > 32)
        unitig_subsets_kernel<u128><<<grid, 256, 0, s>>>(bases, u_off, u_len, item_unitig, item_first, item_count,
                                                         n_items, kmer_base, k, static_cast<const u128 *>(keys),
                                                         vals, mask, out);
    else
        unitig_subsets_kernel<uint64_t><<<grid, 256, 0, s>>>(bases, u_off, u_len, item_unitig, item_first,
                                                             item_count, n_items, kmer_base, k,
                                                             static_cast<const uint64_t *>(keys), vals, mask, out);
    return 1;
}

int launch_index_insert(const uint8_t *text, uint64_t n, int k, void *keys, uint32_t *vals, uint64_t mask,
                        unsigned *status, cudaStream_t s, const uint32_t *pos_val) {
    const uint64_t chunk = 256;
    const uint64_t threads = (n + chunk - 1) / chunk;
    if (threads == 0) return 0;
    const unsigned grid = (unsigned)((threads + 255) / 256);
    if (k > 32)
        index_insert_kernel<u128>
            <<<grid, 256, 0, s>>>(text, n, k, chunk, pos_val, static_cast<u128 *>(keys), vals, mask, status);
    else
        index_insert_kernel<uint64_t>
            <<<grid, 256, 0, s>>>(text, n, k, chunk, pos_val, static_cast<uint64_t *>(keys), vals, mask, status);
    return 1;
}

int launch_index_from_colors(const uint64_t *cslots, uint64_t ccap, const uint32_t *id_subset, int wide, void *keys,
                             uint32_t *vals, uint64_t mask, unsigned *status, int sms, cudaStream_t s) {
    if (wide)
        index_from_colors_kernel<u128><<<sms * 8, 256, 0, s>>>(cslots, ccap, id_subset, static_cast<u128 *>(keys), vals,
                                                               mask, status);
    else
        index_from_colors_kernel<uint64_t><<<sms * 8, 256, 0, s>>>(cslots, ccap, id_subset,
                                                                   static_cast<uint64_t *>(keys), vals, mask, status);
    return 1;
}

int launch_query(const uint8_t *text, int k, const uint32_t *item_query, const uint64_t *item_start,
                 const uint32_t *item_len, uint64_t n_items, const void *keys, uint64_t mask,
                 unsigned long long *matched, cudaStream_t s) {
    if (n_items == 0) return 0;
    const unsigned grid = (unsigned)((n_items + 255) / 256);
    if (k > 32)
        query_kernel<u128><<<grid, 256, 0, s>>>(text, k, item_query, item_start, item_len, n_items,
                                                static_cast<const u128 *>(keys), mask, matched);
    else
        query_kernel<uint64_t><<<grid, 256, 0, s>>>(text, k, item_query, item_start, item_len, n_items,
                                                    static_cast<const uint64_t *>(keys), mask, matched);
    return 1;
}

uint32_t query_color_chunk() { return kColorChunk; }

template <typename KT, int W>
static void color_warp_launch(const uint8_t *text, int k, const uint32_t *iq, const uint64_t *is, const uint32_t *il,
                              uint64_t n_items, const void *keys, const uint32_t *vals, uint64_t mask,
                              const uint32_t *sub_arena, int words, uint32_t n_colors, unsigned long long *matched,
                              unsigned long long *counts, int sms, cudaStream_t s) {
    const uint64_t blocks = (n_items + kColorWarps - 1) / kColorWarps;
    const unsigned grid = (unsigned)std::min<uint64_t>(blocks, (uint64_t)sms * 8);
    query_color_warp_kernel<KT, W><<<grid, 32 * kColorWarps, 0, s>>>(text, k, iq, is, il, n_items,
                                                                     static_cast<const KT *>(keys), vals, mask,
                                                                     sub_arena, words, n_colors, matched, counts);
}

template <typename KT>
static int color_warp_dispatch(const uint8_t *text, int k, const uint32_t *iq, const uint64_t *is, const uint32_t *il,
                               uint64_t n_items, const void *keys, const uint32_t *vals, uint64_t mask,
                               const uint32_t *sub_arena, int words, uint32_t n_colors, unsigned long long *matched,
                               unsigned long long *counts, int sms, cudaStream_t s) {
    if (words <= 1)
        color_warp_launch<KT, 1>(text, k, iq, is, il, n_items, keys, vals, mask, sub_arena, words, n_colors, matched,
                                 counts, sms, s);
    else if (words <= 2)
        color_warp_launch<KT, 2>(text, k, iq, is, il, n_items, keys, vals, mask, sub_arena, words, n_colors, matched,
                                 counts, sms, s);
    else if (words <= 4)
        color_warp_launch<KT, 4>(text, k, iq, is, il, n_items, keys, vals, mask, sub_arena, words, n_colors, matched,
                                 counts, sms, s);
    else
        color_warp_launch<KT, 8>(text, k, iq, is, il, n_items, keys, vals, mask, sub_arena, words, n_colors, matched,
                                 counts, sms, s);
    return 1;
}

int launch_query_color_items(const uint8_t *text, int k, const uint32_t *item_query, const uint64_t *item_start,
                             const uint32_t *item_len, uint64_t n_items, const void *keys, const uint32_t *vals,
                             uint64_t mask, const uint32_t *sub_arena, int words, uint32_t n_colors,
                             unsigned long long *matched, unsigned long long *counts, int sms, cudaStream_t s) {
    if (n_items == 0 || words > kColorWarpMaxWords) return 0;
    if (k > 32)
        return color_warp_dispatch<u128>(text, k, item_query, item_start, item_len, n_items, keys, vals, mask,
                                         sub_arena, words, n_colors, matched, counts, sms, s);
    return color_warp_dispatch<uint64_t>(text, k, item_query, item_start, item_len, n_items, keys, vals, mask,
                                         sub_arena, words, n_colors, matched, counts, sms, s);
}

int launch_query_color(const uint8_t *text, int k, const uint64_t *q_off, const uint64_t *q_len, uint64_t nq,
                       const void *keys, const uint32_t *vals, uint64_t mask, const uint32_t *sub_arena, int words,
                       uint32_t n_colors, unsigned long long *matched, unsigned long long *counts,
                       unsigned long long *queue, int sms, cudaStream_t s) {
    if (nq == 0) return 0;
    const size_t smem = (size_t)n_colors * sizeof(uint32_t);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(query_color_kernel<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(query_color_kernel<u128>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    const unsigned grid = (unsigned)std::min<uint64_t>(nq, (uint64_t)sms * 8);
    if (k > 32)
        query_color_kernel<u128><<<grid, 256, smem, s>>>(text, k, q_off, q_len, nq, static_cast<const u128 *>(keys),
                                                         vals, mask, sub_arena, words, n_colors, matched, counts, queue);
    else
        query_color_kernel<uint64_t><<<grid, 256, smem, s>>>(text, k, q_off, q_len, nq,
                                                             static_cast<const uint64_t *>(keys), vals, mask, sub_arena,
                                                             words, n_colors, matched, counts, queue);
    return 1;
}

}  // namespace ggcat
