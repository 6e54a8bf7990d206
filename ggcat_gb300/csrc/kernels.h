// Host-side launchers of the device kernels (internal to the library).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace ggcat {

// bucketing.cu — each launcher returns the number of kernels it launched
int launch_pack(const uint8_t *d_text, uint64_t n, uint64_t *packed, uint32_t *valid, cudaStream_t s, int sms);
// Launch geometry of bucketize_kernel: thread t owns `chunk` window starts and walks
// `lookback` bases before them; block b stores its records in staging region b
// (region_cap records), the rest in the overflow area after the regions.
struct BucketizeGeometry {
    uint32_t threads_per_block, chunk, lookback, blocks, region_cap;
    size_t smem;
};
BucketizeGeometry bucketize_geometry(uint64_t n, int k, int m);
// kernel attributes (dynamic shared memory limits) of the current device; called once per
// context, outside any stream capture
cudaError_t bucketize_configure();
cudaError_t merge_configure();
// bin_counts: per sub-bin records << 32 | k-mer instances (one packed atomic per superkmer),
// or with split_counts records only and k-mer instances in bin_kmers; total_recs receives the
// record total of all blocks (a packed count that overflowed shows as a smaller scanned total).
// The staging array holds the regions of blocks [stage_block0, stage_block0 + stage_blocks)
// (default: all blocks) followed by the overflow area.
int launch_bucketize(const uint64_t *packed, const uint32_t *valid, uint64_t n, int k, int m, int bbits, int sbits,
                     int fbits, int canonical, const BucketizeGeometry &g, unsigned long long *bin_counts,
                     unsigned long long *bin_kmers, int split_counts, unsigned long long *total_recs, SkRec *stage,
                     unsigned long long *block_count, unsigned long long ovf_cap, unsigned long long *ovf_cursor,
                     unsigned *status, uint32_t block_base, uint32_t n_blocks, cudaStream_t s,
                     uint32_t stage_block0 = 0, uint32_t stage_blocks = 0);
// text bases covered by one bucketize block (pieces of a pipelined launch are multiples of it)
inline uint64_t bucketize_block_bases(const BucketizeGeometry &g) { return (uint64_t)g.threads_per_block * g.chunk; }
int launch_partition(const SkRec *stage, const BucketizeGeometry &g, const unsigned long long *block_count,
                     const unsigned long long *ovf_cursor, unsigned long long ovf_cap, int fbits,
                     const unsigned long long *bin_off, unsigned *bin_cursor, SkRec *recs, unsigned *status,
                     cudaStream_t s, uint32_t stage_blocks = 0);
uint64_t scan_temp_elems(uint64_t n);
// out has n+1 entries: exclusive prefix sums and the total at out[n]; field 0 scans the words,
// 1 their high halves, 2 their low halves
int launch_exclusive_scan(const unsigned long long *in, uint64_t n, unsigned long long *out,
                          unsigned long long *tmp, cudaStream_t s, int field = 0);

// merge.cu
struct MergeUnit {
    uint64_t rec_begin, rec_end;  // record range in the bucket store
    uint64_t kmers;               // k-mer instances
    uint64_t table_off;           // large units: slot offset in the global table pool
    uint32_t table_cap;           // large units: capacity (power of two)
    uint32_t bucket;
};

struct MergeOut {
    uint8_t *bases;               // partial unitig bases (ASCII)
    unsigned long long bases_cap;
    uint64_t *u_off;              // per partial unitig: offset into bases
    uint32_t *u_len;
    uint8_t *u_flags;             // bit0 bw link, bit1 fw link, bit2 circular
    unsigned long long u_cap;
    unsigned long long *counters; // see kCnt*
    uint64_t *kmer_keys;          // optional k-mer dump (u128 keys: (lo, hi) word pairs)
    uint32_t *kmer_mult;
    unsigned long long kmer_cap;
    unsigned *status;
};

struct MergeArgs {
    const uint64_t *packed;
    const SkRec *recs;
    int k;
    int min_mult;
    int keep_kmers;
    int wide;  // key words as a power of two: 0 u64 (k <= 32), 1 u128 (k <= 64), 2 u256 (k <= 127)
    int forward;  // 1: forward-only build (k-mers keyed and extended as read, not canonicalised)
    // per-CTA global scratch of the extension phase for units with more survivors than the
    // shared-memory arrays hold (CTA i uses ext_scratch + i * ext_stride, up to ext_cap survivors)
    uint8_t *ext_scratch;
    uint64_t ext_stride;
    uint32_t ext_cap;
    int rec_batch;  // superkmer records per insert batch of a warp (1-32; shared-memory tiers)
    // colours collected during the merge (bm_words = 0: off).  A superkmer's colour is that of
    // the sequence holding its first base (seq_off ascending); every k-mer instance sets its
    // colour's bit in the CTA's bitmap scratch (bm_stride words per CTA, bm_words per table
    // slot), and the dense numbering moves a surviving k-mer's bitmap to bm_out at its dump
    // index, leaving the scratch zero for the next unit
    const uint64_t *seq_off = nullptr;
    const uint32_t *seq_color = nullptr;
    uint32_t n_seq = 0;
    int bm_words = 0;
    uint32_t *bm_scratch = nullptr;
    uint64_t bm_stride = 0;
    uint32_t *bm_out = nullptr;
};

// bytes of extension scratch per survivor (keys of key_bytes, 2 oriented nodes of 30 bytes)
inline uint64_t merge_ext_bytes_per_survivor(int wide) { return (8u << wide) + 60; }
// survivors per CTA the extension scratch is sized for: S and W tiers / M tier
constexpr uint32_t kExtCapShared = 16384;
constexpr uint32_t kExtCapMedium = 1u << 18;

// merge counters (device array of 16 u64)
enum : int {
    kCntUnitigs = 0,      // partial unitigs emitted
    kCntBases = 1,        // partial unitig bases emitted
    kCntKmers = 2,        // k-mers dumped
    kCntSmallHead = 3,    // work-queue head of S units
    kCntSmall = 4,        // number of S units
    kCntLarge = 5,        // number of L units
    kCntSlots = 6,        // global table slots claimed by M and L units
    kCntMediumHead = 7,   // work-queue head of M units
    kCntMedium = 8,       // number of M units (including spilled optimistic S units)
    kCntDistinct = 9,     // distinct k-mers summed over units (table entries)
    kCntSpilled = 10,     // W units moved to the M tier
    kCntWide = 11,        // number of W units
    kCntWideHead = 12,    // work-queue head of W units
    kCntExtGlobal = 13,   // units extended with the global-memory scratch arrays
    kCntWalk = 14,        // units extended by the per-thread walk fallback
};

constexpr int kSmallSlots = 4096;     // shared-memory table capacity of one merge CTA
constexpr int kMergeThreads = 256;

// Sub-bins of <= small_limit instances are packed into S units (up to unit_target); single
// sub-bins of <= wide_limit instances are W units (shared-memory table first, spill to the M
// queue); <= medium_limit: M units; larger: L units.  W, M and L units reserve a global table.
// kmer_off: exclusive prefix sums of the per-sub-bin k-mer instances
int launch_classify_units(const unsigned long long *bin_off, const unsigned long long *kmer_off, uint32_t n_buckets,
                          int fbits, uint64_t small_limit, uint64_t unit_target, uint64_t wide_limit,
                          uint64_t medium_limit, uint32_t load_pct, MergeUnit *small_units, MergeUnit *wide_units,
                          MergeUnit *medium_units, MergeUnit *large_units, uint64_t max_units, uint64_t pool_slots,
                          unsigned long long *counters, unsigned *status, cudaStream_t s);
int launch_merge_small(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters,
                       const MergeOut &o, int sms, cudaStream_t s);
// spill: the M-unit array (W units whose distinct k-mers overflow are appended to it)
int launch_merge_wide(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters,
                      MergeUnit *spill, uint64_t max_units, const MergeOut &o, int sms, cudaStream_t s);
// Table keys are u64 (a.wide == 0) or u128 (a.wide == 1, 16-byte aligned) slots.
// list: one u32 per pool slot (created-entry lists of the units)
int launch_merge_medium(const MergeArgs &a, const MergeUnit *units, const unsigned long long *counters, void *keys,
                        uint32_t *vals, uint8_t *vis, uint32_t *list, const MergeOut &o, int sms, cudaStream_t s);
// grid-wide insert/extend/cycles over the units [0, *n_units_dev)
int launch_merge_large(const MergeArgs &a, const MergeUnit *units, const unsigned long long *n_units_dev,
                       uint64_t n_units_host_hint, void *keys, uint32_t *vals, uint8_t *vis, const MergeOut &o,
                       int sms, cudaStream_t s);
int launch_init_tables(void *keys, int wide, uint32_t *vals, uint8_t *vis, uint64_t slots, int sms, cudaStream_t s);
int launch_init_unit_tables(const MergeUnit *units, const unsigned long long *n_units_dev, void *keys, int wide,
                            uint32_t *vals, uint8_t *vis, int sms, cudaStream_t s);
// largest number of k-mer instances of an S unit / of an optimistic S unit
uint64_t merge_small_limit(int wide);
uint64_t merge_wide_limit(int wide);
// CTAs per SM of a merge tier (0 = S, 1 = W, 2 = M): the persistent grids are SMs x this
int merge_ctas_per_sm(int tier, int wide);

// query.cu
// uncoloured index keys: u64 for k <= 32, u128 (16-byte aligned) for k <= 64
// pos_val (optional): the value of the k-mer starting at each text position (else 0)
int launch_index_insert(const uint8_t *text, uint64_t n, int k, void *keys, uint32_t *vals, uint64_t mask,
                        unsigned *status, cudaStream_t s, const uint32_t *pos_val = nullptr);
// cslots: the colour phase's {key, id} table of ccap slots
// keys: u64 (wide = 0) or u128 query table keys, 16-byte aligned
int launch_index_from_colors(const uint64_t *cslots, uint64_t ccap, const uint32_t *id_subset, int wide, void *keys,
                             uint32_t *vals, uint64_t mask, unsigned *status, int sms, cudaStream_t s);
int launch_query(const uint8_t *text, int k, const uint32_t *item_query, const uint64_t *item_start,
                 const uint32_t *item_len, uint64_t n_items, const void *keys, uint64_t mask,
                 unsigned long long *matched, cudaStream_t s);
// Coloured lookup over work items (runs of at most query_color_chunk() k-mer positions of one
// query, as for launch_query), for subsets of at most kColorWarpMaxWords bitmap words (256
// colours); matched and counts (nq x n_colors) must be zeroed first.  Returns 0 (nothing
// launched) above that width: launch_query_color covers any width.
constexpr int kColorWarpMaxWords = 8;
uint32_t query_color_chunk();
int launch_query_color_items(const uint8_t *text, int k, const uint32_t *item_query, const uint64_t *item_start,
                             const uint32_t *item_len, uint64_t n_items, const void *keys, const uint32_t *vals,
                             uint64_t mask, const uint32_t *sub_arena, int words, uint32_t n_colors,
                             unsigned long long *matched, unsigned long long *counts, int sms, cudaStream_t s);
int launch_query_color(const uint8_t *text, int k, const uint64_t *q_off, const uint64_t *q_len, uint64_t nq,
                       const void *keys, const uint32_t *vals, uint64_t mask, const uint32_t *sub_arena, int words,
                       uint32_t n_colors, unsigned long long *matched, unsigned long long *counts,
                       unsigned long long *queue, int sms, cudaStream_t s);

// per-k-mer colour subsets of the final unitigs through the coloured index (items of at most
// a few hundred k-mers of one unitig)
int launch_unitig_subsets(const uint8_t *bases, const uint64_t *u_off, const uint32_t *u_len,
                          const uint32_t *item_unitig, const uint32_t *item_first, const uint32_t *item_count,
                          uint64_t n_items, const uint64_t *kmer_base, int k, const void *keys, const uint32_t *vals,
                          uint64_t mask, uint32_t *out, cudaStream_t s);

// link.cu — cross-bucket link stage (each launcher returns the kernels it launched)
int launch_link_endpoints(const uint8_t *bases, const uint64_t *off, const uint32_t *len, const uint8_t *flags,
                          uint64_t n, int k, int fwd, void *keys, uint32_t *min1, uint64_t mask, uint32_t *eslot,
                          unsigned *status, int sms, cudaStream_t s);
int launch_link_succ(const uint32_t *eslot, const uint32_t *min1, const uint32_t *min2, uint64_t nn,
                     uint32_t *succ, uint32_t *jump, int sms, cudaStream_t s);
int launch_link_jump(const uint32_t *succ, const uint32_t *jump, uint32_t *jump_n, uint64_t nn,
                     unsigned long long *unresolved, int sms, cudaStream_t s);
int launch_link_cycle_list(const uint32_t *succ, const uint32_t *jump, uint64_t nn, uint32_t *list,
                           unsigned long long *count, uint32_t *cyc_jump, uint32_t *cyc_min, int sms, cudaStream_t s);
int launch_link_cycle_min(const uint32_t *list, uint64_t nc, const uint32_t *cj, const uint32_t *cm, uint32_t *cj_n,
                          uint32_t *cm_n, int sms, cudaStream_t s);
int launch_link_cycle_cut(const uint32_t *list, uint64_t nc, const uint32_t *cm, uint32_t *succ, uint8_t *node_state,
                          int sms, cudaStream_t s);
int launch_link_pred_init(const uint32_t *succ, const uint8_t *node_state, const uint32_t *len, uint64_t nn, int k,
                          uint32_t *pjump, unsigned long long *prank, int sms, cudaStream_t s);
int launch_link_pred_jump(const uint32_t *pj, const unsigned long long *pr, uint32_t *pj_n, unsigned long long *pr_n,
                          uint64_t nn, unsigned long long *changed, int sms, cudaStream_t s);
int launch_link_reserve(const uint32_t *succ, const uint8_t *node_state, const uint32_t *pj,
                        const unsigned long long *pr, const uint32_t *len, const uint8_t *pflags, uint64_t nn,
                        unsigned long long *chain_off, uint64_t *u_off, uint32_t *u_len, uint8_t *u_flags,
                        unsigned long long *counters, unsigned long long bases_cap, unsigned long long u_cap,
                        unsigned *status, int sms, cudaStream_t s);
int launch_link_write(const uint8_t *bases, const uint64_t *off, const uint32_t *len, const uint8_t *node_state,
                      const uint32_t *pj, const unsigned long long *pr, const unsigned long long *chain_off,
                      uint64_t nn, int k, uint8_t *out, int sms, cudaStream_t s);

// hashes.cu
int launch_kmer_hash(const uint8_t *text, uint64_t n, int k, int kind, uint64_t *out, cudaStream_t s);

// colors.cu
// dump: the merge's k-mer dump (u64 keys, or (lo, hi) pairs when wide, k > 32); slots:
// (wide ? 4 : 2) x (mask + 1) words ({key, id} slots, all-ones when empty); owner, id_subset,
// dump_subset: n_dump entries; bitmaps: n_dump x words (zeroed); max_seq_len: the longest
// sequence (seq_off[i + 1] - seq_off[i], the last one up to n_text), 0 when seq_off[0] > 0
// the colour phase when the merge collected every dumped copy's colours (ggcat_gpu_colors_prepare):
// k-mer table (owners), union of the copies into their owner, subset dedup, per-copy subset
int launch_color_phase_collected(const uint64_t *dump, uint64_t n_dump, int wide, int words, uint64_t *slots,
                                 uint64_t mask, uint32_t *owner, uint32_t *bitmaps, unsigned long long *sub_count,
                                 unsigned long long *sub_hash, uint32_t *sub_state, uint32_t *sub_arena,
                                 uint64_t sub_mask, uint32_t *id_subset, uint32_t *dump_subset, unsigned *status,
                                 int sms, cudaStream_t s);
int launch_color_phase(const uint64_t *dump, uint64_t n_dump, const uint8_t *text, uint64_t n_text, int k,
                       int canonical, int wide, const uint64_t *seq_off, const uint32_t *seq_color,
                       uint64_t n_seq, uint64_t max_seq_len, int words, uint64_t *slots, uint64_t mask, uint32_t *owner, uint32_t *bitmaps,
                       unsigned long long *sub_count, unsigned long long *sub_hash, uint32_t *sub_state,
                       uint32_t *sub_arena, uint64_t sub_mask, uint32_t *id_subset, uint32_t *dump_subset,
                       unsigned *status, int sms, cudaStream_t s);

}  // namespace ggcat
