// C ABI of ggcat_gb300: context, device buffers, orchestration of the bucketing and merge
// kernels, the host link stage, the FASTA reader and the file-level build entry point.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <cmath>
#include <vector>

#include "../../include/ggcat_gb300.h"
#include "colormap.h"
#include "graph_out.h"
#include "input.h"
#include "kernels.h"

using namespace ggcat;

namespace {

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t want = cnt ? cnt : 1;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

constexpr int kFeedPieces = 16;  // pieces of build_text's pipelined host text copy

struct PinnedBuf {
    uint8_t *p = nullptr;
    size_t n = 0;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t ensure(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMallocHost(&p, cnt ? cnt : 1);
        if (e == cudaSuccess) n = cnt ? cnt : 1;
        return e;
    }
};

// Host array in pinned memory for device results: it only grows (with 1/8 headroom) and
// resize() leaves the elements uninitialised, since a device copy fills them, so reading back
// a result is one direct DMA and no host-side fill.
template <typename T>
struct PinnedArray {
    T *p = nullptr;
    size_t n = 0, cap = 0;
    PinnedArray() = default;
    PinnedArray(const PinnedArray &) = delete;
    PinnedArray &operator=(const PinnedArray &) = delete;
    ~PinnedArray() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t resize(size_t cnt) {
        if (cnt > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            n = cap = 0;
            const size_t want = cnt + cnt / 8;
            cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(&p), want * sizeof(T));
            if (e != cudaSuccess) return e;
            cap = want;
        }
        n = cnt;
        return cudaSuccess;
    }
    void clear() { n = 0; }
    T *data() { return p; }
    const T *data() const { return p; }
    size_t size() const { return n; }
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
};

struct HostUnitigs {
    PinnedArray<uint8_t> bases;
    PinnedArray<uint64_t> off;
    PinnedArray<uint32_t> len;
    PinnedArray<uint8_t> flags;
    void clear() {
        bases.clear();
        off.clear();
        len.clear();
        flags.clear();
    }
};

}  // namespace

// Everything the captured merge launches depend on: a replay is valid while all of it is
// unchanged (zero-initialised with memset so padding compares equal).
struct MergeGraphKey {
    const void *ptr[32];
    uint64_t val[32];
};

// device buffers of the link stage
struct LinkBufs {
    DevBuf<uint64_t> keys;  // endpoint table keys (u64, or u128 as word pairs)
    DevBuf<uint32_t> min12, eslot, succ, jump, jump2, list, cj, cm, cj2, cm2;
    DevBuf<uint8_t> state;
    DevBuf<unsigned long long> pr, pr2, chain_off, counters;
    DevBuf<uint8_t> out_bases;
    DevBuf<uint64_t> out_off;
    DevBuf<uint32_t> out_len;
    DevBuf<uint8_t> out_flags;
};

struct ggcat_gpu_ctx {
    int device = 0;
    int sms = 1;
    std::string err;
    uint64_t launches = 0;

    // input staging
    DevBuf<uint8_t> d_text;
    PinnedBuf h_stage;

    // bucketing
    DevBuf<uint64_t> packed;
    DevBuf<uint32_t> valid;
    // per sub-bin: bin_count = records << 32 | k-mer instances (packed), or records only with the
    // k-mer instances in bin_kmers (split counters, after a packed count overflowed)
    DevBuf<unsigned long long> bin_count, bin_kmers, bin_off, kmer_off, scan_tmp, rec_total;
    DevBuf<unsigned> bin_cursor;  // records placed per sub-bin by the partition
    DevBuf<SkRec> recs, stage;
    DevBuf<unsigned long long> ovf_cursor, block_count;  // staging overflow cursor, records per region
    DevBuf<unsigned> status;
    uint64_t n_text = 0, n_recs = 0, n_kmers = 0, n_bins = 0;
    uint32_t n_buckets = 0;
    int fine_bits = 8;
    ggcat_gpu_params last_params{};
    bool have_buckets = false;
    const uint8_t *last_text = nullptr;  // device text of the last bucketize

    // colour phase
    DevBuf<uint64_t> cslots;  // {key, id} pairs
    DevBuf<uint32_t> cowner, cbitmaps, cid_subset, cdump_subset, csub_state, csub_arena;
    DevBuf<unsigned long long> csub_hash, ccounters;
    DevBuf<uint64_t> cseq_off;
    DevBuf<uint32_t> cseq_color;
    uint64_t cmask = 0, c_n_ids = 0, c_n_subsets = 0;
    uint32_t c_colors = 0;
    int c_words = 0;
    bool have_colors = false;
    // colours announced before the build (ggcat_gpu_colors_prepare): the merge collects them
    bool cprep = false;
    std::vector<uint64_t> cprep_off;
    std::vector<uint32_t> cprep_col;
    uint32_t cprep_colors = 0;
    DevBuf<uint64_t> cprep_off_d;
    DevBuf<uint32_t> cprep_col_d;
    DevBuf<uint32_t> cbm_scratch;  // per merge CTA, one bitmap row per table slot
    bool collect_now = false;      // this merge collects colours
    bool merge_collected = false;  // the last merge collected every dumped k-mer's colours

    // merge
    DevBuf<MergeUnit> small_units, wide_units, medium_units, large_units, bucket_units;
    DevBuf<unsigned long long> counters, ones;
    DevBuf<uint64_t> tkeys;
    DevBuf<uint32_t> tvals;
    DevBuf<uint8_t> tvis;
    DevBuf<uint32_t> tlist;  // created-entry lists of the M units
    DevBuf<uint8_t> ext_scratch;  // per-CTA extension scratch of units with many survivors
    LinkBufs lk;
    DevBuf<uint8_t> qgraph;  // graph text of the file-level query
    uint64_t n_final = 0, n_final_bases = 0;
    // the batched merge phase as a CUDA graph, captured once per buffer/parameter layout
    cudaStream_t cap_stream = nullptr;
    cudaStream_t copy_stream = nullptr;         // pipelined host text copies of build_text
    cudaStream_t piece_stream[kFeedPieces] = {};  // pack + bucketize of each piece (they overlap)
    cudaEvent_t pack_ev[kFeedPieces] = {}, piece_done_ev[kFeedPieces] = {}, feed_start_ev = nullptr;
    cudaEvent_t feed_ev[kFeedPieces + 1] = {};  // [0]: compute stream ready, [1 + i]: piece i copied
    cudaGraphExec_t merge_exec = nullptr;
    MergeGraphKey merge_key{};
    int merge_graph_kernels = 0;
    uint64_t merge_graph_captures = 0, merge_graph_replays = 0;
    DevBuf<uint8_t> out_bases;
    DevBuf<uint64_t> out_off;
    DevBuf<uint32_t> out_len;
    DevBuf<uint8_t> out_flags;
    DevBuf<uint64_t> kmer_keys;
    DevBuf<uint32_t> kmer_mult;
    uint64_t n_partial = 0, n_partial_bases = 0, n_kmers_out = 0;
    bool have_merge = false;

    HostUnitigs partial;  // copied back by build_text / on demand
    bool partial_on_host = false;
    HostUnitigs final_u;

    // host bucket store of a spilled bucketize: per piece of the text, its records partitioned
    // by (bucket, sub-bin) with the piece's sub-bin offsets (empty: the store is in HBM)
    struct SpillPiece {
        PinnedArray<SkRec> recs;
        std::vector<unsigned long long> bin_off, kmer_off;
    };
    std::vector<std::unique_ptr<SpillPiece>> spill;
    uint64_t spill_budget = 0;  // device bytes of the bucket store the spill was sized for

    cudaEvent_t ev[8] = {};
    cudaEvent_t tier_ev[5] = {};  // batched merge: before S, after S, W, M and L (graph event nodes)
    ggcat_gpu_stats stats{};

    // query: resident graph index and in-flight batch slots
    DevBuf<uint64_t> qkeys;
    DevBuf<uint32_t> qvals;
    uint64_t qmask = 0;
    int qk = 0;
    bool qcolored = false, qready = false;
    struct QuerySlot {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        DevBuf<uint8_t> d_text;
        DevBuf<uint32_t> d_iq, d_il;
        DevBuf<uint64_t> d_is;
        DevBuf<unsigned long long> d_matched, d_counts, d_queue;
        DevBuf<uint64_t> d_qoff, d_qlen;
        DevBuf<unsigned> d_status;
        PinnedBuf h_text, h_items, h_out, h_counts;
        uint64_t nq = 0, n_items = 0;
        bool busy = false, colored = false;
    };
    QuerySlot qslots[GGCAT_GPU_QUERY_SLOTS];

    ~ggcat_gpu_ctx() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : tier_ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : feed_ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : pack_ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : piece_done_ev)
            if (e) cudaEventDestroy(e);
        if (feed_start_ev) cudaEventDestroy(feed_start_ev);
        for (auto &q : piece_stream)
            if (q) cudaStreamDestroy(q);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        for (auto &q : qslots) {
            if (q.done) cudaEventDestroy(q.done);
            if (q.stream) cudaStreamDestroy(q.stream);
        }
    }
};

// Host copy split over up to 8 threads when large (one core copies ~14 GB/s, a batch of query
// text is a few hundred MB).
static void par_memcpy(void *dst, const void *src, uint64_t n) {
    const uint64_t kMin = 32ull << 20;
    const int t = (int)std::min<uint64_t>({8, n / kMin, (uint64_t)std::max(1u, std::thread::hardware_concurrency())});
    if (t <= 1) {
        if (n) memcpy(dst, src, n);
        return;
    }
    const uint64_t per = (n + t - 1) / t;
    std::vector<std::thread> th;
    for (int i = 1; i < t; i++) {
        const uint64_t a = std::min<uint64_t>(n, per * i), b = std::min<uint64_t>(n, a + per);
        th.emplace_back([=] { memcpy(static_cast<uint8_t *>(dst) + a, static_cast<const uint8_t *>(src) + a, b - a); });
    }
    memcpy(dst, src, std::min<uint64_t>(n, per));
    for (auto &x : th) x.join();
}

static int fail(ggcat_gpu_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? GGCAT_GPU_ENOMEM : GGCAT_GPU_ECUDA,     \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);   \
    } while (0)

static cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" int ggcat_gpu_create(int device, ggcat_gpu_ctx **out) {
    if (!out) return GGCAT_GPU_EINVAL;
    *out = nullptr;
    auto *ctx = new ggcat_gpu_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete ctx;
        return GGCAT_GPU_ECUDA;
    }
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    ctx->sms = sms > 0 ? sms : 1;
    for (auto &ev : ctx->ev) {
        if (cudaEventCreate(&ev) != cudaSuccess) {
            delete ctx;
            return GGCAT_GPU_ECUDA;
        }
    }
    for (auto &ev : ctx->tier_ev) {
        if (cudaEventCreate(&ev) != cudaSuccess) {
            delete ctx;
            return GGCAT_GPU_ECUDA;
        }
    }
    if (ctx->status.ensure(2) != cudaSuccess || ctx->counters.ensure(16) != cudaSuccess ||
        ctx->ones.ensure(1) != cudaSuccess) {
        delete ctx;
        return GGCAT_GPU_ENOMEM;
    }
    unsigned long long one = 1;
    cudaMemcpy(ctx->ones.p, &one, sizeof one, cudaMemcpyHostToDevice);
    if (bucketize_configure() != cudaSuccess || merge_configure() != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return GGCAT_GPU_ECUDA;
    }
    *out = ctx;
    return GGCAT_GPU_OK;
}

extern "C" void ggcat_gpu_destroy(ggcat_gpu_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->merge_exec) cudaGraphExecDestroy(ctx->merge_exec);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    delete ctx;
}

extern "C" const char *ggcat_gpu_last_error(const ggcat_gpu_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" uint64_t ggcat_gpu_kernel_launches(const ggcat_gpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

// merge-table key words as a power of two: u64 (k <= 32), u128 (k <= 64), u256 (k <= 127)
static int key_width(int k) { return k > 64 ? 2 : k > 32 ? 1 : 0; }

// Defaults of the tuning knobs (0 in ggcat_gpu_params).  Above k = 32 they are the autotuner's
// choice on the 2 Gbp long-k reads (k = 63, 250-bp reads): sub-bins of 4096 text bytes, 90 %
// global-table load, 8-record insert batches, W units up to 8192 instances (longer records
// carry more k-mers each, so smaller batches and units balance the warps).
static uint64_t default_subbin_bytes(int k) { return k > 32 ? 4096 : 1024; }
static uint32_t default_load_pct(int k) { return k > 32 ? 90 : 80; }
static int default_rec_batch(int k) { return k > 32 ? 8 : 16; }
static uint64_t default_wide_limit(int k, uint64_t tier_max) { return k > 32 ? std::min<uint64_t>(8192, tier_max) : tier_max; }

static int check_params(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p) {
    if (!p) return fail(ctx, GGCAT_GPU_EINVAL, "null params");
    if (p->m < 2 || p->m > 32) return fail(ctx, GGCAT_GPU_EINVAL, "minimizer length m=%d outside [2, 32]", p->m);
    if (p->k - p->m < 2) return fail(ctx, GGCAT_GPU_EINVAL, "need k - m >= 2 (k=%d, m=%d)", p->k, p->m);
    if (p->k > 127) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "k=%d > 127 is not supported on the device", p->k);
    // the reference's sequence hashes stop at k = 64; longer k-mers take the Rabin-Karp family
    // (crates/api/src/utils.rs:10-69)
    if (p->k > 64 && p->hash_kind == GGCAT_HASH_SEQHASH)
        return fail(ctx, GGCAT_GPU_EINVAL, "sequence hash for k=%d > 64 (use the Rabin-Karp hash)", p->k);
    if (p->bucket_bits < 1 || p->bucket_bits > 15)
        return fail(ctx, GGCAT_GPU_EINVAL, "bucket_bits=%d outside [1, 15]", p->bucket_bits);
    if (p->second_bits < 0 || p->second_bits > 8)
        return fail(ctx, GGCAT_GPU_EINVAL, "second_bits=%d outside [0, 8]", p->second_bits);
    if (p->subbin_bytes < 0 || p->table_load_pct < 0 || p->table_load_pct > 95 ||
        (p->table_load_pct > 0 && p->table_load_pct < 10) || p->small_limit < 0 || p->copy_pieces < 0 ||
        p->copy_pieces > kFeedPieces || p->small_batch < 0 || p->small_batch > 32 || p->wide_batch < 0 ||
        p->wide_batch > 32 || p->wide_limit < 0)
        return fail(ctx, GGCAT_GPU_EINVAL,
                    "tuning knob out of range (subbin_bytes=%d, table_load_pct=%d, small_limit=%d, copy_pieces=%d, "
                    "small_batch=%d, wide_batch=%d, wide_limit=%d)",
                    p->subbin_bytes, p->table_load_pct, p->small_limit, p->copy_pieces, p->small_batch,
                    p->wide_batch, p->wide_limit);
    return GGCAT_GPU_OK;
}

static int read_status(ggcat_gpu_ctx *ctx, unsigned *st) {
    CK(cudaMemcpy(st, ctx->status.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    return GGCAT_GPU_OK;
}

// Text arriving on the device in pieces (the pipelined host copy of build_text): piece i is
// [off[i], off[i + 1]), the offsets are multiples of a bucketize block's bases, and the piece is
// in place once ev[i] has completed.  Piece i is packed when it arrives and its blocks are
// bucketized once piece i + 1 is packed too: a block reads at most k - 1 bases and one
// prefetched 32-base word past its last window start, and any amount before its first one.
struct TextFeed {
    int pieces;
    const uint64_t *off;
    const cudaEvent_t *ev;
};

// Bucketize with the bucket store in pinned host memory: the text (packed whole, it stays on the
// device for the merge) is bucketized in pieces of bucketize blocks, each sized so that its
// staging and partitioned records fit `budget` bytes; every piece's records, partitioned by
// (bucket, sub-bin) with its own sub-bin offsets, are copied to host memory.  The merge then
// works bucket range by bucket range (merge_spill).  The records equal those of the resident
// path (each block's superkmers do not depend on the launch it runs in).
static int bucketize_spill(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len, const ggcat_gpu_params *p,
                           cudaStream_t s, const TextFeed *feed, uint64_t budget, uint64_t *n_superkmers) {
    const uint64_t n_words = (text_len + 31) / 32 + 1;
    CK(ctx->packed.ensure(n_words));
    CK(ctx->valid.ensure(n_words));
    const uint64_t nb = ctx->n_bins;
    CK(ctx->bin_count.ensure(nb + 1));
    CK(ctx->bin_off.ensure(nb + 1));
    CK(ctx->kmer_off.ensure(nb + 1));
    CK(ctx->bin_cursor.ensure(nb + 1));
    CK(ctx->scan_tmp.ensure(scan_temp_elems(nb) + 2));
    CK(ctx->rec_total.ensure(1));
    CK(ctx->ovf_cursor.ensure(1));
    const int canonical = p->forward_only ? 0 : 1;
    const BucketizeGeometry geo = bucketize_geometry(text_len, p->k, p->m);
    const uint64_t block_bases = bucketize_block_bases(geo);
    CK(cudaEventRecord(ctx->ev[0], s));
    if (feed)
        for (int i = 0; i < feed->pieces; i++) CK(cudaStreamWaitEvent(s, feed->ev[i], 0));
    ctx->launches += launch_pack(d_text, text_len, ctx->packed.p, ctx->valid.p, s, ctx->sms);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], s));
    // a block's staging region and, at most, as many partitioned records
    const uint64_t per_block = (uint64_t)geo.region_cap * sizeof(SkRec) * 2 + block_bases / 32;
    const uint64_t piece_blocks = std::max<uint64_t>(1, budget / per_block);
    ctx->spill.clear();
    ctx->spill_budget = budget;
    uint64_t tot_recs = 0, tot_kmers = 0;
    for (uint64_t B0 = 0; B0 < geo.blocks; B0 += piece_blocks) {
        const uint64_t B1 = std::min<uint64_t>(geo.blocks, B0 + piece_blocks), nbp = B1 - B0;
        uint64_t ovf_cap = nbp * block_bases / 64 + 4096;
        int split_counts = 0;
        unsigned long long totals[4] = {0, 0, 0, 0};
        CK(ctx->block_count.ensure(nbp + 1));
        for (int attempt = 0; attempt < 3; attempt++) {
            CK(ctx->stage.ensure(nbp * geo.region_cap + ovf_cap));
            if (split_counts) CK(ctx->bin_kmers.ensure(nb + 1));
            CK(cudaMemsetAsync(ctx->bin_count.p, 0, (nb + 1) * sizeof(unsigned long long), s));
            if (split_counts) CK(cudaMemsetAsync(ctx->bin_kmers.p, 0, (nb + 1) * sizeof(unsigned long long), s));
            CK(cudaMemsetAsync(ctx->rec_total.p, 0, sizeof(unsigned long long), s));
            CK(cudaMemsetAsync(ctx->bin_cursor.p, 0, (nb + 1) * sizeof(unsigned), s));
            CK(cudaMemsetAsync(ctx->ovf_cursor.p, 0, sizeof(unsigned long long), s));
            CK(cudaMemsetAsync(ctx->status.p, 0, 2 * sizeof(unsigned), s));
            ctx->launches += launch_bucketize(ctx->packed.p, ctx->valid.p, text_len, p->k, p->m, p->bucket_bits,
                                              p->second_bits, ctx->fine_bits, canonical, geo, ctx->bin_count.p,
                                              ctx->bin_kmers.p, split_counts, ctx->rec_total.p, ctx->stage.p,
                                              ctx->block_count.p, ovf_cap, ctx->ovf_cursor.p, ctx->status.p,
                                              (uint32_t)B0, (uint32_t)nbp, s, (uint32_t)B0, (uint32_t)nbp);
            CK(cudaGetLastError());
            ctx->launches += launch_exclusive_scan(ctx->bin_count.p, nb, ctx->bin_off.p, ctx->scan_tmp.p, s,
                                                   split_counts ? 0 : 1);
            ctx->launches += launch_exclusive_scan(split_counts ? ctx->bin_kmers.p : ctx->bin_count.p, nb,
                                                   ctx->kmer_off.p, ctx->scan_tmp.p, s, split_counts ? 0 : 2);
            CK(cudaMemcpyAsync(&totals[0], ctx->bin_off.p + nb, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(&totals[1], ctx->kmer_off.p + nb, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(&totals[2], ctx->ovf_cursor.p, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(&totals[3], ctx->rec_total.p, 8, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            bool again = false;
            if (!split_counts && totals[0] != totals[3]) {
                split_counts = 1;
                again = true;
            }
            if (totals[2] > ovf_cap) {
                ovf_cap = totals[2] + 1024;
                again = true;
            }
            if (!again) break;
        }
        if (totals[0] != totals[3] || totals[2] > ovf_cap)
            return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize (spill): staging or count overflow");
        const uint64_t nr = totals[0];
        CK(ctx->recs.ensure(nr + 1));
        ctx->launches += launch_partition(ctx->stage.p, geo, ctx->block_count.p, ctx->ovf_cursor.p, ovf_cap,
                                          ctx->fine_bits, ctx->bin_off.p, ctx->bin_cursor.p, ctx->recs.p,
                                          ctx->status.p, s, (uint32_t)nbp);
        CK(cudaGetLastError());
        auto piece = std::make_unique<ggcat_gpu_ctx::SpillPiece>();
        CK(piece->recs.resize(nr));
        piece->bin_off.resize(nb + 1);
        piece->kmer_off.resize(nb + 1);
        if (nr) CK(cudaMemcpyAsync(piece->recs.data(), ctx->recs.p, nr * sizeof(SkRec), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(piece->bin_off.data(), ctx->bin_off.p, (nb + 1) * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(piece->kmer_off.data(), ctx->kmer_off.p, (nb + 1) * 8, cudaMemcpyDeviceToHost, s));
        unsigned st = 0;
        CK(cudaMemcpyAsync(&st, ctx->status.p, sizeof st, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (st & (kStatusLookback | kStatusStageOverflow))
            return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize (spill): internal error (status %u)", st);
        tot_recs += nr;
        tot_kmers += totals[1];
        ctx->spill.push_back(std::move(piece));
    }
    CK(cudaEventRecord(ctx->ev[2], s));
    ctx->n_text = text_len;
    ctx->last_text = d_text;
    ctx->have_colors = false;
    ctx->last_params = *p;
    ctx->n_recs = tot_recs;
    ctx->n_kmers = tot_kmers;
    ctx->have_buckets = true;
    ctx->stats = ggcat_gpu_stats{};
    ctx->stats.text_bytes = text_len;
    ctx->stats.superkmers = tot_recs;
    ctx->stats.kmer_instances = tot_kmers;
    ctx->stats.spill_pieces = ctx->spill.size();
    ctx->stats.spill_bytes = tot_recs * sizeof(SkRec);
    if (n_superkmers) *n_superkmers = tot_recs;
    return GGCAT_GPU_OK;
}

static int bucketize_impl(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len, const ggcat_gpu_params *p,
                          void *stream, uint64_t *n_superkmers, const TextFeed *feed) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (text_len >= (1ull << 40)) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "text longer than 2^40 bytes");
    if (text_len > 0 && !d_text) return fail(ctx, GGCAT_GPU_EINVAL, "null text");
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    ctx->have_buckets = false;
    ctx->have_merge = false;
    ctx->partial_on_host = false;
    const uint64_t n_words = (text_len + 31) / 32 + 1;
    CK(ctx->packed.ensure(n_words));
    CK(ctx->valid.ensure(n_words));
    ctx->n_buckets = (1u << p->bucket_bits) + 1;
    // sub-bins per bucket: about subbin_bytes (default 1K) text bytes per sub-bin on average
    const uint64_t subbin = p->subbin_bytes > 0 ? (uint64_t)p->subbin_bytes : default_subbin_bytes(p->k);
    int fb = 0;
    while (fb < kMaxFineBits && ((uint64_t)ctx->n_buckets << fb) * subbin < text_len) fb++;
    ctx->fine_bits = fb < 4 ? 4 : fb;
    ctx->n_bins = (uint64_t)ctx->n_buckets << ctx->fine_bits;
    ctx->spill.clear();
    {
        // the bucket store goes to host memory when its records (with their staging) would pass
        // the spill_mb budget or half of the device's free memory
        const uint64_t est = text_len / (uint64_t)(p->k - p->m + 1) * 3 + 4096;  // 1.5x density 2/(w+1)
        const uint64_t need = est * sizeof(SkRec) * 2;
        uint64_t budget = p->spill_mb > 0 ? ((uint64_t)p->spill_mb << 20) : 0;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
            const uint64_t have = (uint64_t)free_b / 2 + ctx->stage.n * sizeof(SkRec) + ctx->recs.n * sizeof(SkRec);
            if (need > have && (budget == 0 || budget > have)) budget = std::max<uint64_t>(have, 64ull << 20);
        }
        if (budget && need > budget) return bucketize_spill(ctx, d_text, text_len, p, s, feed, budget, n_superkmers);
    }
    const uint64_t nb = ctx->n_bins;
    CK(ctx->bin_count.ensure(nb + 1));
    CK(ctx->bin_off.ensure(nb + 1));
    CK(ctx->kmer_off.ensure(nb + 1));
    CK(ctx->bin_cursor.ensure(nb + 1));
    CK(ctx->scan_tmp.ensure(scan_temp_elems(nb) + 2));
    const int canonical = p->forward_only ? 0 : 1;
    const BucketizeGeometry geo = bucketize_geometry(text_len, p->k, p->m);
    CK(ctx->ovf_cursor.ensure(1));
    CK(ctx->block_count.ensure((size_t)geo.blocks + 1));
    // overflow area of the staging array (records beyond a block's region); retried when exceeded
    uint64_t ovf_cap = text_len / 64 + 4096;
    const uint64_t block_bases = bucketize_block_bases(geo);
    CK(ctx->rec_total.ensure(1));
    int split_counts = 0;
    auto bucketize_blocks = [&](uint64_t b0, uint64_t b1, cudaStream_t q) {
        return launch_bucketize(ctx->packed.p, ctx->valid.p, text_len, p->k, p->m, p->bucket_bits, p->second_bits,
                                ctx->fine_bits, canonical, geo, ctx->bin_count.p, ctx->bin_kmers.p, split_counts,
                                ctx->rec_total.p, ctx->stage.p, ctx->block_count.p, ovf_cap, ctx->ovf_cursor.p,
                                ctx->status.p, (uint32_t)b0, (uint32_t)(b1 - b0), q);
    };
    auto clear_counts = [&]() -> int {
        CK(ctx->stage.ensure((uint64_t)geo.blocks * geo.region_cap + ovf_cap));
        CK(cudaMemsetAsync(ctx->bin_count.p, 0, (nb + 1) * sizeof(unsigned long long), s));
        if (split_counts) CK(cudaMemsetAsync(ctx->bin_kmers.p, 0, (nb + 1) * sizeof(unsigned long long), s));
        CK(cudaMemsetAsync(ctx->rec_total.p, 0, sizeof(unsigned long long), s));
        CK(cudaMemsetAsync(ctx->bin_cursor.p, 0, (nb + 1) * sizeof(unsigned), s));
        CK(cudaMemsetAsync(ctx->ovf_cursor.p, 0, sizeof(unsigned long long), s));
        CK(cudaMemsetAsync(ctx->status.p, 0, 2 * sizeof(unsigned), s));
        return GGCAT_GPU_OK;
    };
    CK(cudaEventRecord(ctx->ev[0], s));
    if (feed) {
        // pipelined: each piece on its own stream, packed when it arrives and bucketized once the
        // next piece is packed too (a block reads k - 1 bases and a prefetched word past its
        // last window); the pieces' kernels overlap, so a piece may be smaller than a wave.
        // (ms_pack stays 0; ms_bucketize covers the whole pipeline, copy waits included)
        CK(cudaEventRecord(ctx->ev[1], s));
        rc = clear_counts();
        if (rc) return rc;
        if (!ctx->feed_start_ev) CK(cudaEventCreateWithFlags(&ctx->feed_start_ev, cudaEventDisableTiming));
        CK(cudaEventRecord(ctx->feed_start_ev, s));  // the counters are clear
        const int np = feed->pieces;
        for (int i = 0; i < np; i++) {
            if (!ctx->piece_stream[i]) CK(cudaStreamCreateWithFlags(&ctx->piece_stream[i], cudaStreamNonBlocking));
            if (!ctx->pack_ev[i]) CK(cudaEventCreateWithFlags(&ctx->pack_ev[i], cudaEventDisableTiming));
            if (!ctx->piece_done_ev[i]) CK(cudaEventCreateWithFlags(&ctx->piece_done_ev[i], cudaEventDisableTiming));
            cudaStream_t q = ctx->piece_stream[i];
            const uint64_t o0 = feed->off[i], o1 = feed->off[i + 1];
            CK(cudaStreamWaitEvent(q, ctx->feed_start_ev, 0));
            CK(cudaStreamWaitEvent(q, feed->ev[i], 0));
            ctx->launches += launch_pack(d_text + o0, o1 - o0, ctx->packed.p + o0 / 32, ctx->valid.p + o0 / 32, q,
                                         ctx->sms);
            CK(cudaEventRecord(ctx->pack_ev[i], q));
        }
        for (int i = 0; i < np; i++) {
            cudaStream_t q = ctx->piece_stream[i];
            if (i + 1 < np) CK(cudaStreamWaitEvent(q, ctx->pack_ev[i + 1], 0));
            const uint64_t b0 = feed->off[i] / block_bases, b1 = i + 1 < np ? feed->off[i + 1] / block_bases : geo.blocks;
            ctx->launches += bucketize_blocks(b0, b1, q);
            CK(cudaEventRecord(ctx->piece_done_ev[i], q));
        }
        for (int i = 0; i < np; i++) CK(cudaStreamWaitEvent(s, ctx->piece_done_ev[i], 0));
        CK(cudaGetLastError());
    } else {
        ctx->launches += launch_pack(d_text, text_len, ctx->packed.p, ctx->valid.p, s, ctx->sms);
        CK(cudaGetLastError());
        CK(cudaEventRecord(ctx->ev[1], s));
    }
    unsigned long long totals[4];
    for (int attempt = 0; attempt < 3; attempt++) {
        if (attempt > 0 || !feed) {
            rc = clear_counts();
            if (rc) return rc;
            ctx->launches += bucketize_blocks(0, geo.blocks, s);
        }
        CK(cudaGetLastError());
        ctx->launches += launch_exclusive_scan(ctx->bin_count.p, nb, ctx->bin_off.p, ctx->scan_tmp.p, s,
                                               split_counts ? 0 : 1);
        ctx->launches += launch_exclusive_scan(split_counts ? ctx->bin_kmers.p : ctx->bin_count.p, nb,
                                               ctx->kmer_off.p, ctx->scan_tmp.p, s, split_counts ? 0 : 2);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&totals[0], ctx->bin_off.p + nb, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(&totals[1], ctx->kmer_off.p + nb, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(&totals[2], ctx->ovf_cursor.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(&totals[3], ctx->rec_total.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        bool again = false;
        if (!split_counts && totals[0] != totals[3]) {
            // a packed per-sub-bin count overflowed its 32-bit half: count again with separate
            // counters
            split_counts = 1;
            CK(ctx->bin_kmers.ensure(nb + 1));
            again = true;
        }
        if (totals[2] > ovf_cap) {
            ovf_cap = totals[2] + 1024;
            again = true;
        }
        if (!again) break;
    }
    if (totals[0] != totals[3])
        return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize: record count mismatch (%llu vs %llu)", totals[0], totals[3]);
    if (totals[2] > ovf_cap)
        return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize: staging overflow (%llu overflow records)", totals[2]);
    ctx->n_recs = totals[0];
    ctx->n_kmers = totals[1];
    CK(ctx->recs.ensure(ctx->n_recs + 1));
    ctx->launches += launch_partition(ctx->stage.p, geo, ctx->block_count.p, ctx->ovf_cursor.p, ovf_cap,
                                      ctx->fine_bits, ctx->bin_off.p, ctx->bin_cursor.p, ctx->recs.p, ctx->status.p,
                                      s);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[2], s));
    ctx->n_text = text_len;
    ctx->last_text = d_text;
    ctx->have_colors = false;
    ctx->last_params = *p;
    ctx->have_buckets = true;
    ctx->stats = ggcat_gpu_stats{};
    ctx->stats.text_bytes = text_len;
    ctx->stats.superkmers = ctx->n_recs;
    ctx->stats.kmer_instances = ctx->n_kmers;
    if (n_superkmers) *n_superkmers = ctx->n_recs;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_bucketize(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len,
                                   const ggcat_gpu_params *p, void *stream, uint64_t *n_superkmers) {
    return bucketize_impl(ctx, d_text, text_len, p, stream, n_superkmers, nullptr);
}

extern "C" int ggcat_gpu_superkmers_copy(ggcat_gpu_ctx *ctx, ggcat_gpu_superkmer *h_out, uint64_t cap, uint64_t *n) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_buckets) return fail(ctx, GGCAT_GPU_EINVAL, "no bucketize result");
    CK(cudaSetDevice(ctx->device));
    CK(cudaDeviceSynchronize());
    unsigned st = 0;
    int rc = read_status(ctx, &st);
    if (rc) return rc;
    if (st & kStatusLookback) return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize: lookback limit exceeded");
    if (n) *n = ctx->n_recs;
    if (!h_out) return GGCAT_GPU_OK;
    uint64_t cnt = std::min<uint64_t>(cap, ctx->n_recs);
    std::vector<SkRec> tmp(cnt);
    if (!ctx->spill.empty()) {
        // spilled store: the pieces' records sub-bin by sub-bin
        uint64_t pos = 0;
        for (uint64_t bin = 0; bin < ctx->n_bins && pos < cnt; bin++)
            for (const auto &pc : ctx->spill)
                for (uint64_t i = pc->bin_off[bin]; i < pc->bin_off[bin + 1] && pos < cnt; i++) tmp[pos++] = pc->recs[i];
    } else if (cnt) {
        CK(cudaMemcpy(tmp.data(), ctx->recs.p, cnt * sizeof(SkRec), cudaMemcpyDeviceToHost));
    }
    for (uint64_t i = 0; i < cnt; i++) {
        const SkRec &r = tmp[i];
        ggcat_gpu_superkmer o;
        o.start = rec_start(r);
        o.len = rec_len(r);
        o.bucket = (uint16_t)rec_bucket(r);
        o.second_bucket = (uint16_t)rec_second(r);
        o.minimizer_pos = (uint16_t)rec_minpos(r);
        o.rc = (uint8_t)rec_rc(r);
        o.flags = (uint8_t)rec_flags(r);
        h_out[i] = o;
    }
    return GGCAT_GPU_OK;
}

// ---------------------------------------------------------------------------
// merge
// ---------------------------------------------------------------------------
static int merge_once(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p, cudaStream_t s, uint64_t bases_cap,
                      uint64_t u_cap, uint64_t kmer_cap, unsigned *st_out) {
    CK(ctx->out_bases.ensure(bases_cap));
    CK(ctx->out_off.ensure(u_cap));
    CK(ctx->out_len.ensure(u_cap));
    CK(ctx->out_flags.ensure(u_cap));
    const int wide = key_width(p->k);  // table key words: 1 << wide
    if (p->keep_kmers) {
        CK(ctx->kmer_keys.ensure(kmer_cap << wide));
        CK(ctx->kmer_mult.ensure(kmer_cap));
    }
    const uint64_t max_units = ctx->n_bins + 1;
    CK(ctx->small_units.ensure(max_units));
    CK(ctx->wide_units.ensure(max_units));
    CK(ctx->medium_units.ensure(max_units));
    CK(ctx->large_units.ensure(max_units));
    const uint64_t small_limit = p->small_limit > 0 ? std::min<uint64_t>((uint64_t)p->small_limit, merge_small_limit(wide))
                                                    : merge_small_limit(wide);
    // worst-case slot pool of the global-memory tables: cap < 2 * (x * 100 / load + 64) per unit,
    // units of more than small_limit instances each
    const uint32_t load_pct = p->table_load_pct > 0 ? (uint32_t)p->table_load_pct : default_load_pct(p->k);
    const uint64_t max_big_units = std::min<uint64_t>(ctx->n_bins, ctx->n_kmers / small_limit + 1);
    uint64_t pool = ctx->n_kmers * 200 / load_pct + 2 + 128ull * (ctx->n_buckets + max_big_units) + 1024;
    CK(ctx->tkeys.ensure(pool << wide));
    CK(ctx->tvals.ensure(pool));
    CK(ctx->tvis.ensure(pool));
    CK(ctx->tlist.ensure(pool));
    // extension scratch: one region per CTA of the tier running (the tiers run one after
    // another): S/W CTAs up to kExtCapShared survivors each, M CTAs up to kExtCapMedium (the
    // instances of an M unit)
    const uint64_t bps = merge_ext_bytes_per_survivor(wide);
    const uint64_t stride_sw = ((uint64_t)kExtCapShared * bps + 255) & ~255ull;
    const uint64_t stride_m = ((uint64_t)kExtCapMedium * bps + 255) & ~255ull;
    const uint64_t ctas_sw = (uint64_t)ctx->sms * std::max(merge_ctas_per_sm(0, wide), merge_ctas_per_sm(1, wide));
    const uint64_t ctas_m = (uint64_t)ctx->sms * merge_ctas_per_sm(2, wide);
    CK(ctx->ext_scratch.ensure(std::max<uint64_t>(ctas_sw * stride_sw, ctas_m * stride_m)));
    // forward-only builds (forward seq-hash / Rabin-Karp, crates/hashes/src/fw_seqhash.rs) count
    // and extend k-mers as read, without canonicalisation
    MergeArgs a{ctx->packed.p, ctx->recs.p, p->k, p->min_multiplicity, p->keep_kmers, wide, p->forward_only ? 1 : 0,
                ctx->ext_scratch.p, stride_sw, kExtCapShared, 32};
    if (ctx->collect_now) {
        // colours collected by the merge: one bitmap row per table slot and CTA, sized for the
        // largest table of the shared-memory tiers and of the M tier (units up to 2^18 instances)
        const int words = (int)((ctx->cprep_colors + 31) / 32);
        const uint32_t load = p->table_load_pct > 0 ? (uint32_t)p->table_load_pct : default_load_pct(p->k);
        uint64_t mcap = 64;
        while (mcap < (1ull << 18) * 100 / load + 64) mcap <<= 1;
        const uint64_t rows = std::max<uint64_t>(mcap, 11264);
        const uint64_t ctas = (uint64_t)ctx->sms * 2;  // S and M: 2 CTAs per SM, W: 1
        if (ctx->cbm_scratch.ensure(ctas * rows * (uint64_t)words) != cudaSuccess ||
            ctx->cbitmaps.ensure((kmer_cap + 1) * (uint64_t)words) != cudaSuccess) {
            cudaGetLastError();  // no room: the colour phase reads the text instead
            ctx->cbm_scratch.release();
            ctx->collect_now = false;
        }
    }
    if (ctx->collect_now) {
        const int words = (int)((ctx->cprep_colors + 31) / 32);
        const uint64_t rows = ctx->cbm_scratch.n / ((uint64_t)ctx->sms * 2 * (uint64_t)words);
        CK(cudaMemsetAsync(ctx->cbm_scratch.p, 0, ctx->cbm_scratch.n * sizeof(uint32_t), s));
        a.seq_off = ctx->cprep_off_d.p;
        a.seq_color = ctx->cprep_col_d.p;
        a.n_seq = (uint32_t)ctx->cprep_off.size();
        a.bm_words = words;
        a.bm_scratch = ctx->cbm_scratch.p;
        a.bm_stride = rows * (uint64_t)words;
        a.bm_out = ctx->cbitmaps.p;
    }
    // per-class insert batches of the shared-memory tiers
    MergeArgs a_small = a, a_wide = a;
    a_small.rec_batch = p->small_batch > 0 ? p->small_batch : default_rec_batch(p->k);
    a_wide.rec_batch = p->wide_batch > 0 ? p->wide_batch : default_rec_batch(p->k);
    MergeArgs am = a;
    am.ext_stride = stride_m;
    am.ext_cap = kExtCapMedium;
    MergeOut o{ctx->out_bases.p, bases_cap,       ctx->out_off.p,   ctx->out_len.p, ctx->out_flags.p,
               u_cap,            ctx->counters.p, ctx->kmer_keys.p, ctx->kmer_mult.p,
               p->keep_kmers ? kmer_cap : 0,      ctx->status.p + 1};
    // S packing target: the size limit itself (fewer, fuller S units; the tuner's choice on the
    // skewed reads, S class 2.16 -> 1.95 ms, and on the long-k reads)
    uint64_t target = p->unit_target > 0 ? (uint64_t)p->unit_target : (wide ? 1600 : 3200);
    if (target > small_limit) target = small_limit;

    if (p->merge_mode == GGCAT_MERGE_PER_BUCKET) {
        CK(cudaMemsetAsync(ctx->counters.p, 0, 16 * sizeof(unsigned long long), s));
        CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
        CK(cudaEventRecord(ctx->ev[3], s));
        // plain form: every bucket is one unit with a global-memory table, three launches per bucket
        std::vector<unsigned long long> hoff(ctx->n_bins + 1), hk(ctx->n_bins + 1);
        CK(cudaMemcpyAsync(hoff.data(), ctx->bin_off.p, (ctx->n_bins + 1) * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hk.data(), ctx->kmer_off.p, (ctx->n_bins + 1) * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        std::vector<MergeUnit> units(ctx->n_buckets);
        uint64_t slot = 0;
        for (uint32_t b = 0; b < ctx->n_buckets; b++) {
            uint64_t b0 = (uint64_t)b << ctx->fine_bits, b1 = (uint64_t)(b + 1) << ctx->fine_bits;
            MergeUnit u{};
            u.rec_begin = hoff[b0];
            u.rec_end = hoff[b1];
            u.kmers = hk[b1] - hk[b0];
            uint64_t cap = 64;
            while (cap < u.kmers + u.kmers / 4 + 64) cap <<= 1;
            u.table_off = slot;
            u.table_cap = (uint32_t)cap;
            u.bucket = b;
            slot += cap;
            units[b] = u;
        }
        if (slot > pool) return fail(ctx, GGCAT_GPU_EDEVICE, "per-bucket table pool too small");
        CK(ctx->bucket_units.ensure(ctx->n_buckets));
        CK(cudaMemcpyAsync(ctx->bucket_units.p, units.data(), units.size() * sizeof(MergeUnit),
                           cudaMemcpyHostToDevice, s));
        ctx->launches += launch_init_tables(ctx->tkeys.p, wide, ctx->tvals.p, ctx->tvis.p, slot, ctx->sms, s);
        for (uint32_t b = 0; b < ctx->n_buckets; b++) {
            if (units[b].rec_end == units[b].rec_begin) continue;
            ctx->launches += launch_merge_large(a, ctx->bucket_units.p + b, ctx->ones.p, 1, ctx->tkeys.p, ctx->tvals.p,
                                                ctx->tvis.p, o, ctx->sms, s);
        }
        CK(cudaGetLastError());
        ctx->stats.merge_units_small = 0;
        ctx->stats.merge_units_large = ctx->n_buckets;
    } else {
        const uint64_t medium_limit = 1ull << 18;
        const uint64_t wide_limit =
            p->unit_target < 0 ? 0
                               : std::min<uint64_t>(merge_wide_limit(wide),
                                                    p->wide_limit > 0 ? (uint64_t)p->wide_limit
                                                                      : default_wide_limit(p->k, merge_wide_limit(wide)));
        // the whole batched merge phase: counter reset, classification, the S/W/M persistent
        // kernels fed by device work queues and the grid-wide L kernels
        auto enqueue = [&](cudaStream_t q) -> int {
            int n = 0;
            if (cudaMemsetAsync(ctx->counters.p, 0, 16 * sizeof(unsigned long long), q) != cudaSuccess) return -1;
            if (cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), q) != cudaSuccess) return -1;
            n += launch_classify_units(ctx->bin_off.p, ctx->kmer_off.p, ctx->n_buckets, ctx->fine_bits, small_limit,
                                       target, wide_limit, medium_limit, load_pct, ctx->small_units.p, ctx->wide_units.p,
                                       ctx->medium_units.p, ctx->large_units.p, max_units, pool, ctx->counters.p,
                                       ctx->status.p + 1, q);
            // event record nodes (external records: captured, an ordinary record only orders the
            // capture) between the classes time each class's kernels (per-class tuning)
            if (cudaEventRecordWithFlags(ctx->tier_ev[0], q, cudaEventRecordExternal) != cudaSuccess) return -1;
            n += launch_merge_small(a_small, ctx->small_units.p, ctx->counters.p, o, ctx->sms, q);
            if (cudaEventRecordWithFlags(ctx->tier_ev[1], q, cudaEventRecordExternal) != cudaSuccess) return -1;
            n += launch_merge_wide(a_wide, ctx->wide_units.p, ctx->counters.p, ctx->medium_units.p, max_units, o,
                                   ctx->sms, q);
            if (cudaEventRecordWithFlags(ctx->tier_ev[2], q, cudaEventRecordExternal) != cudaSuccess) return -1;
            n += launch_merge_medium(am, ctx->medium_units.p, ctx->counters.p, ctx->tkeys.p, ctx->tvals.p,
                                     ctx->tvis.p, ctx->tlist.p, o, ctx->sms, q);
            if (cudaEventRecordWithFlags(ctx->tier_ev[3], q, cudaEventRecordExternal) != cudaSuccess) return -1;
            n += launch_init_unit_tables(ctx->large_units.p, ctx->counters.p + kCntLarge, ctx->tkeys.p, wide,
                                         ctx->tvals.p, ctx->tvis.p, ctx->sms, q);
            n += launch_merge_large(a, ctx->large_units.p, ctx->counters.p + kCntLarge, 0, ctx->tkeys.p, ctx->tvals.p,
                                    ctx->tvis.p, o, ctx->sms, q);
            if (cudaEventRecordWithFlags(ctx->tier_ev[4], q, cudaEventRecordExternal) != cudaSuccess) return -1;
            return n;
        };
        MergeGraphKey key;
        memset(&key, 0, sizeof key);
        const void *ptrs[] = {ctx->packed.p,       ctx->recs.p,        ctx->ext_scratch.p,  ctx->out_bases.p,
                              ctx->out_off.p,      ctx->out_len.p,     ctx->out_flags.p,    ctx->kmer_keys.p,
                              ctx->kmer_mult.p,    ctx->counters.p,    ctx->status.p,       ctx->bin_off.p,
                              ctx->kmer_off.p,     ctx->small_units.p, ctx->wide_units.p,   ctx->medium_units.p,
                              ctx->large_units.p,  ctx->tkeys.p,       ctx->tvals.p,        ctx->tvis.p,
                              ctx->tlist.p,        a.bm_scratch,       a.bm_out,            a.seq_off,
                              a.seq_color};
        static_assert(sizeof(ptrs) / sizeof(ptrs[0]) <= sizeof(key.ptr) / sizeof(key.ptr[0]), "graph key");
        memcpy(key.ptr, ptrs, sizeof ptrs);
        const uint64_t vals[] = {(uint64_t)p->k,     (uint64_t)p->min_multiplicity, (uint64_t)p->keep_kmers,
                                 (uint64_t)wide,     bases_cap,                     u_cap,
                                 p->keep_kmers ? kmer_cap : 0, ctx->n_buckets,      (uint64_t)ctx->fine_bits,
                                 target,             wide_limit,                    max_units,
                                 pool,               stride_sw,                     stride_m,
                                 (uint64_t)ctx->sms, small_limit,                   load_pct,
                                 (uint64_t)a.forward, (uint64_t)a_small.rec_batch,  (uint64_t)a_wide.rec_batch,
                                 (uint64_t)a.bm_words, a.bm_stride,                 (uint64_t)a.n_seq};
        static_assert(sizeof(vals) / sizeof(vals[0]) <= sizeof(key.val) / sizeof(key.val[0]), "graph key");
        memcpy(key.val, vals, sizeof vals);
        if (!ctx->merge_exec || memcmp(&key, &ctx->merge_key, sizeof key) != 0) {
            if (ctx->merge_exec) {
                cudaGraphExecDestroy(ctx->merge_exec);
                ctx->merge_exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeThreadLocal));
            const int n = enqueue(ctx->cap_stream);
            const cudaError_t ec = cudaStreamEndCapture(ctx->cap_stream, &g);
            if (n < 0 || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return fail(ctx, GGCAT_GPU_ECUDA, "merge graph capture failed (%s)", cudaGetErrorString(ec));
            }
            const cudaError_t ei = cudaGraphInstantiate(&ctx->merge_exec, g, 0);
            cudaGraphDestroy(g);
            CK(ei);
            ctx->merge_key = key;
            ctx->merge_graph_kernels = n;
            ctx->merge_graph_captures++;
        }
        CK(cudaEventRecord(ctx->ev[3], s));
        CK(cudaGraphLaunch(ctx->merge_exec, s));
        ctx->launches += (uint64_t)ctx->merge_graph_kernels;
        ctx->merge_graph_replays++;
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ctx->ev[4], s));
    unsigned long long cnt[16];
    CK(cudaMemcpyAsync(cnt, ctx->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, s));
    unsigned stw[2] = {0, 0};
    CK(cudaMemcpyAsync(stw, ctx->status.p, sizeof stw, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    unsigned st = stw[0] | stw[1];
    ctx->n_partial = cnt[kCntUnitigs];
    ctx->n_partial_bases = cnt[kCntBases];
    ctx->n_kmers_out = cnt[kCntKmers];
    ctx->stats.distinct_kmers = cnt[kCntDistinct];
    if (p->merge_mode != GGCAT_MERGE_PER_BUCKET) {
        ctx->stats.merge_units_small = cnt[kCntSmall];
        ctx->stats.merge_units_large = cnt[kCntWide] + cnt[kCntMedium] + cnt[kCntLarge] - cnt[kCntSpilled];
        ctx->stats.merge_units_spilled = cnt[kCntSpilled];
        ctx->stats.merge_units_ext_global = cnt[kCntExtGlobal];
        ctx->stats.merge_units_walk = cnt[kCntWalk] + cnt[kCntLarge];
        // collected colours are complete unless a unit ran in the grid-wide L kernels or the
        // walk fallback, which do not collect them
        ctx->merge_collected = ctx->collect_now && cnt[kCntWalk] == 0 && cnt[kCntLarge] == 0;
        if (cnt[kCntSlots] > pool) return fail(ctx, GGCAT_GPU_EDEVICE, "table pool exceeded");
    }
    *st_out = st;
    return GGCAT_GPU_OK;
}

// merge_once with the output capacities grown until nothing overflows
static int merge_retry(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p, cudaStream_t s) {
    uint64_t bases_cap = ctx->n_kmers / 2 + (uint64_t)p->k * (ctx->n_recs / 2) + 4096;
    uint64_t u_cap = ctx->n_recs + 1024;
    uint64_t kmer_cap = ctx->n_kmers + 1024;
    unsigned st = 0;
    for (int attempt = 0; attempt < 3; attempt++) {
        const int rc = merge_once(ctx, p, s, bases_cap, u_cap, kmer_cap, &st);
        if (rc) return rc;
        if (!(st & (kStatusOutOverflow | kStatusKmerOverflow))) break;
        bases_cap = std::max<uint64_t>(bases_cap, ctx->n_partial_bases + 4096);
        u_cap = std::max<uint64_t>(u_cap, ctx->n_partial + 1024);
        kmer_cap = std::max<uint64_t>(kmer_cap, ctx->n_kmers_out + 1024);
    }
    if (st & (kStatusOutOverflow | kStatusKmerOverflow)) return fail(ctx, GGCAT_GPU_EDEVICE, "merge output overflow");
    if (st & kStatusTableFull) return fail(ctx, GGCAT_GPU_EDEVICE, "merge: hash table full");
    if (st & kStatusWalkLimit) return fail(ctx, GGCAT_GPU_EDEVICE, "merge: unitig walk bound exceeded");
    if (st & kStatusLookback) return fail(ctx, GGCAT_GPU_EDEVICE, "bucketize: internal lookback/partition error");
    return GGCAT_GPU_OK;
}

// The merge of a spilled bucket store: consecutive bucket ranges whose records (over all
// pieces) fit the spill budget, one after another.  A range's records are gathered on the host
// in (sub-bin, piece) order, so that every sub-bin is contiguous, copied to the device in one
// copy with offsets that leave the other buckets empty, and merged by the usual merge phase;
// its partial unitigs (and dumped k-mers) are appended on the host and finally put back on the
// device for the link and colour stages.  Every merge unit lies inside one bucket, so the
// result is the resident path's.
static int merge_spill(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p, cudaStream_t s) {
    const uint64_t nb = ctx->n_bins, nbk = ctx->n_buckets;
    const int fb = ctx->fine_bits;
    const uint64_t kw = 1ull << key_width(p->k);
    const uint64_t tot_recs = ctx->n_recs, tot_kmers = ctx->n_kmers;
    std::vector<uint64_t> brec(nbk, 0);
    for (const auto &pc : ctx->spill)
        for (uint64_t b = 0; b < nbk; b++) brec[b] += pc->bin_off[(b + 1) << fb] - pc->bin_off[b << fb];
    const uint64_t budget_recs = std::max<uint64_t>(1, ctx->spill_budget / (2 * sizeof(SkRec)));
    std::vector<uint8_t> a_bases, a_flags;
    std::vector<uint64_t> a_off, kkeys;
    std::vector<uint32_t> a_len, kmult;
    PinnedArray<SkRec> gather;
    std::vector<unsigned long long> roff(nb + 1), rkoff(nb + 1);
    double ms_merge = 0;
    uint64_t ranges = 0, distinct = 0, small_u = 0, large_u = 0, spilled_u = 0, extg = 0, walk = 0;
    auto restore = [&]() {
        ctx->n_recs = tot_recs;
        ctx->n_kmers = tot_kmers;
    };
    for (uint64_t b0 = 0; b0 < nbk;) {
        uint64_t b1 = b0 + 1, nr = brec[b0];
        while (b1 < nbk && nr + brec[b1] <= budget_recs) nr += brec[b1++];
        // gather the range's records and its offsets (empty sub-bins outside the range)
        CK(gather.resize(nr));
        uint64_t pos = 0, kpos = 0;
        const uint64_t bin0 = b0 << fb, bin1 = b1 << fb;
        for (uint64_t bin = 0; bin <= nb; bin++) {
            roff[bin] = pos;
            rkoff[bin] = kpos;
            if (bin < bin0 || bin >= bin1) continue;
            for (const auto &pc : ctx->spill) {
                const uint64_t a = pc->bin_off[bin], e = pc->bin_off[bin + 1];
                if (e > a) memcpy(gather.data() + pos, pc->recs.data() + a, (e - a) * sizeof(SkRec));
                pos += e - a;
                kpos += pc->kmer_off[bin + 1] - pc->kmer_off[bin];
            }
        }
        CK(ctx->recs.ensure(nr + 1));
        if (nr) CK(cudaMemcpyAsync(ctx->recs.p, gather.data(), nr * sizeof(SkRec), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->bin_off.p, roff.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->kmer_off.p, rkoff.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
        ctx->n_recs = nr;
        ctx->n_kmers = kpos;
        const int rc = merge_retry(ctx, p, s);
        if (rc) {
            restore();
            return rc;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[3], ctx->ev[4]);
        ms_merge += ms;
        distinct += ctx->stats.distinct_kmers;
        small_u += ctx->stats.merge_units_small;
        large_u += ctx->stats.merge_units_large;
        spilled_u += ctx->stats.merge_units_spilled;
        extg += ctx->stats.merge_units_ext_global;
        walk += ctx->stats.merge_units_walk;
        // append the range's partial unitigs and k-mers
        const uint64_t nu = ctx->n_partial, nbs = ctx->n_partial_bases, base0 = a_bases.size(), u0 = a_off.size();
        a_bases.resize(base0 + nbs);
        a_off.resize(u0 + nu);
        a_len.resize(u0 + nu);
        a_flags.resize(u0 + nu);
        if (nbs) CK(cudaMemcpy(a_bases.data() + base0, ctx->out_bases.p, nbs, cudaMemcpyDeviceToHost));
        if (nu) {
            CK(cudaMemcpy(a_off.data() + u0, ctx->out_off.p, nu * 8, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(a_len.data() + u0, ctx->out_len.p, nu * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(a_flags.data() + u0, ctx->out_flags.p, nu, cudaMemcpyDeviceToHost));
            for (uint64_t i = u0; i < u0 + nu; i++) a_off[i] += base0;
        }
        if (p->keep_kmers && ctx->n_kmers_out) {
            const uint64_t nk = ctx->n_kmers_out, k0 = kmult.size();
            kkeys.resize((k0 + nk) * kw);
            kmult.resize(k0 + nk);
            CK(cudaMemcpy(kkeys.data() + k0 * kw, ctx->kmer_keys.p, nk * kw * 8, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(kmult.data() + k0, ctx->kmer_mult.p, nk * 4, cudaMemcpyDeviceToHost));
        }
        ranges++;
        b0 = b1;
    }
    restore();
    // the appended partial unitigs (and k-mers) back on the device for the link and colour
    // stages, and in the pinned host arrays the partial-unitig copy reads
    const uint64_t nu = a_off.size(), nbs = a_bases.size();
    CK(ctx->out_bases.ensure(nbs + 1));
    CK(ctx->out_off.ensure(nu + 1));
    CK(ctx->out_len.ensure(nu + 1));
    CK(ctx->out_flags.ensure(nu + 1));
    if (nbs) CK(cudaMemcpy(ctx->out_bases.p, a_bases.data(), nbs, cudaMemcpyHostToDevice));
    if (nu) {
        CK(cudaMemcpy(ctx->out_off.p, a_off.data(), nu * 8, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->out_len.p, a_len.data(), nu * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->out_flags.p, a_flags.data(), nu, cudaMemcpyHostToDevice));
    }
    HostUnitigs &h = ctx->partial;
    CK(h.bases.resize(nbs));
    CK(h.off.resize(nu));
    CK(h.len.resize(nu));
    CK(h.flags.resize(nu));
    if (nbs) memcpy(h.bases.data(), a_bases.data(), nbs);
    if (nu) {
        memcpy(h.off.data(), a_off.data(), nu * 8);
        memcpy(h.len.data(), a_len.data(), nu * 4);
        memcpy(h.flags.data(), a_flags.data(), nu);
    }
    ctx->n_partial = nu;
    ctx->n_partial_bases = nbs;
    ctx->n_kmers_out = kmult.size();
    if (p->keep_kmers) {
        CK(ctx->kmer_keys.ensure(kmult.size() * kw + 1));
        CK(ctx->kmer_mult.ensure(kmult.size() + 1));
        if (!kmult.empty()) {
            CK(cudaMemcpy(ctx->kmer_keys.p, kkeys.data(), kkeys.size() * 8, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(ctx->kmer_mult.p, kmult.data(), kmult.size() * 4, cudaMemcpyHostToDevice));
        }
    }
    ctx->partial_on_host = true;
    ctx->stats.ms_merge = ms_merge;
    ctx->stats.distinct_kmers = distinct;
    ctx->stats.merge_units_small = small_u;
    ctx->stats.merge_units_large = large_u;
    ctx->stats.merge_units_spilled = spilled_u;
    ctx->stats.merge_units_ext_global = extg;
    ctx->stats.merge_units_walk = walk;
    ctx->stats.spill_ranges = ranges;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_merge(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p, void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (!ctx->have_buckets) return fail(ctx, GGCAT_GPU_EINVAL, "merge needs a bucketize result");
    if (p->k != ctx->last_params.k || p->m != ctx->last_params.m || p->bucket_bits != ctx->last_params.bucket_bits)
        return fail(ctx, GGCAT_GPU_EINVAL, "merge parameters differ from the bucketize parameters");
    if (p->k > 127) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "device merge supports k <= 127 (k=%d)", p->k);
    // a forward-only k-mer of all G at k = 32 / 64 is the tables' empty key (all ones); canonical
    // keys never are (the reverse complement, all C, is smaller)
    if (p->forward_only && (p->k == 32 || p->k == 64))
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "forward-only builds at k = %d are not supported", p->k);
    // Tables are keyed by the canonical packed k-mer (the seq-hash value).  The Rabin-Karp
    // u128 hash is injective on the k-mers of any input short of a 128-bit collision, so it
    // selects the same k-mer identities and gives the same result.
    if (p->hash_kind != GGCAT_HASH_SEQHASH && p->hash_kind != GGCAT_HASH_RABIN_KARP128 && p->hash_kind != 0)
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "unknown merge hash kind %d", p->hash_kind);
    if (p->min_multiplicity < 1) return fail(ctx, GGCAT_GPU_EINVAL, "min_multiplicity must be >= 1");
    if (ctx->n_kmers >= (1ull << 29) * 1024ull) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "input too large");
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    ctx->have_merge = false;
    ctx->partial_on_host = false;
    ctx->merge_collected = false;
    // colours announced before the build are collected by the batched, resident merge when its
    // bitmap buffers can be allocated (else ggcat_gpu_colors reads them from the text)
    ctx->collect_now = ctx->cprep && p->keep_kmers && p->k <= 64 && p->merge_mode == GGCAT_MERGE_BATCHED &&
                       ctx->spill.empty() && !ctx->cprep_off.empty() && ctx->cprep_off.back() < ctx->n_text;
    rc = ctx->spill.empty() ? merge_retry(ctx, p, s) : merge_spill(ctx, p, s);
    if (rc) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    ctx->stats.ms_pack = ms;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    ctx->stats.ms_bucketize = ms;
    if (ctx->spill.empty()) {
        cudaEventElapsedTime(&ms, ctx->ev[3], ctx->ev[4]);
        ctx->stats.ms_merge = ms;
    }
    for (int c = 0; c < 4; c++) {
        float mt = 0;
        if (p->merge_mode != GGCAT_MERGE_PER_BUCKET && ctx->spill.empty() &&
            cudaEventElapsedTime(&mt, ctx->tier_ev[c], ctx->tier_ev[c + 1]) != cudaSuccess) {
            cudaGetLastError();  // a class time is a statistic: its failure must not fail the next call
            mt = 0;
        }
        ctx->stats.ms_tier[c] = mt;
    }
    ctx->stats.partial_unitigs = ctx->n_partial;
    ctx->stats.partial_bases = ctx->n_partial_bases;
    ctx->stats.surviving_kmers = ctx->n_kmers_out;
    ctx->have_merge = true;
    return GGCAT_GPU_OK;
}

// ---------------------------------------------------------------------------
// autotuner: the tuning knobs of the build hot path chosen by measurement
// ---------------------------------------------------------------------------
extern "C" int ggcat_gpu_autotune(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len,
                                  const ggcat_gpu_params *p, uint64_t sample_bytes, void *stream,
                                  ggcat_gpu_params *best, double *default_ms, double *best_ms) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    int rc = check_params(ctx, p);
    if (rc) return rc;
    if (!best) return fail(ctx, GGCAT_GPU_EINVAL, "null output params");
    if (p->merge_mode == GGCAT_MERGE_PER_BUCKET) return fail(ctx, GGCAT_GPU_EINVAL, "autotune tunes the batched merge");
    const uint64_t n = sample_bytes ? std::min(sample_bytes, text_len) : text_len;
    const int wide = p->k > 32;
    // device time of one candidate: the better of two runs (by merge time, with that run's
    // per-class times); bucketize is redone only when the candidate changes the sub-bin digit width
    struct Trial {
        double bucket = 1e30, merge = 1e30, tier[4] = {0, 0, 0, 0};
    };
    auto trial = [&](const ggcat_gpu_params &q, bool rebucket, Trial &t) -> int {
        t = Trial{};
        for (int rep = 0; rep < 2; rep++) {
            if (rebucket || rep == 0) {
                uint64_t nsk = 0;
                int r = ggcat_gpu_bucketize(ctx, d_text, n, &q, stream, &nsk);
                if (r) return r;
            }
            int r = ggcat_gpu_merge(ctx, &q, stream);
            if (r) return r;
            if (rebucket) t.bucket = std::min(t.bucket, ctx->stats.ms_pack + ctx->stats.ms_bucketize);
            if (ctx->stats.ms_merge < t.merge) {
                t.merge = ctx->stats.ms_merge;
                for (int c = 0; c < 4; c++) t.tier[c] = ctx->stats.ms_tier[c];
            }
        }
        return GGCAT_GPU_OK;
    };
    ggcat_gpu_params cur = *p;
    Trial t0;
    rc = trial(cur, true, t0);
    if (rc) return rc;
    const double d_ms = t0.bucket + t0.merge;
    // 1. the sub-bin digit width of the bucket store (bucketize + merge)
    double best_total = d_ms, best_bucket = t0.bucket;
    int best_sb = cur.subbin_bytes;
    for (int sb : {256, 512, 1024, 2048, 4096}) {
        ggcat_gpu_params q = cur;
        q.subbin_bytes = sb;
        Trial t;
        rc = trial(q, true, t);
        if (rc) return rc;
        if (t.bucket + t.merge < best_total) {
            best_total = t.bucket + t.merge;
            best_bucket = t.bucket;
            best_sb = sb;
        }
    }
    cur.subbin_bytes = best_sb;
    {
        uint64_t nsk = 0;
        rc = ggcat_gpu_bucketize(ctx, d_text, n, &cur, stream, &nsk);
        if (rc) return rc;
    }
    // 2. per bucket-size class, each knob judged by the device time of the classes it moves work
    //    between (bit c of `classes`: 0 S units, 1 W units, 2 M units, 3 L units):
    //    S: unit packing target (-1: no W tier), S sub-bin limit, S insert batch;
    //    W: W insert batch, W sub-bin limit; M/L: global-table load
    struct Knob {
        int32_t ggcat_gpu_params::*field;
        unsigned classes;
        std::vector<int32_t> vals;
    };
    const int32_t wl = (int32_t)merge_wide_limit(wide);
    const std::vector<Knob> knobs = {
        {&ggcat_gpu_params::unit_target, 0x7u, wide ? std::vector<int32_t>{0, -1, 512, 1024}
                                                    : std::vector<int32_t>{0, -1, 1024, 2048}},
        {&ggcat_gpu_params::small_limit, 0x3u, wide ? std::vector<int32_t>{0, 1200, 800}
                                                    : std::vector<int32_t>{0, 2400, 1600}},
        {&ggcat_gpu_params::small_batch, 0x1u, {0, 8, 16, 32}},
        {&ggcat_gpu_params::wide_batch, 0x2u, {0, 8, 12, 16, 24, 32}},
        {&ggcat_gpu_params::wide_limit, 0x6u, {0, wl / 2, wl / 4}},
        {&ggcat_gpu_params::table_load_pct, 0xcu, {0, 50, 65, 90}},
    };
    auto class_ms = [](const Trial &t, unsigned classes) {
        double ms = 0;
        for (int c = 0; c < 4; c++)
            if (classes >> c & 1u) ms += t.tier[c];
        return ms;
    };
    for (const Knob &kb : knobs) {
        Trial base;
        rc = trial(cur, false, base);
        if (rc) return rc;
        double best_v_ms = class_ms(base, kb.classes);
        int32_t best_v = cur.*kb.field;
        for (int32_t v : kb.vals) {
            if (v == cur.*kb.field) continue;
            ggcat_gpu_params q = cur;
            q.*kb.field = v;
            Trial t;
            rc = trial(q, false, t);
            if (rc) return rc;
            const double ms = class_ms(t, kb.classes);
            if (ms < best_v_ms) {
                best_v_ms = ms;
                best_v = v;
            }
        }
        cur.*kb.field = best_v;
    }
    Trial fin;
    rc = trial(cur, false, fin);
    if (rc) return rc;
    const double best_merge = fin.merge;
    *best = cur;
    if (default_ms) *default_ms = d_ms;
    if (best_ms) *best_ms = best_bucket + best_merge;
    return GGCAT_GPU_OK;
}

static int fetch_partial(ggcat_gpu_ctx *ctx) {
    if (ctx->partial_on_host) return GGCAT_GPU_OK;
    HostUnitigs &h = ctx->partial;
    CK(cudaSetDevice(ctx->device));
    CK(h.bases.resize(ctx->n_partial_bases));
    CK(h.off.resize(ctx->n_partial));
    CK(h.len.resize(ctx->n_partial));
    CK(h.flags.resize(ctx->n_partial));
    // the merge has completed (its output counts were read on the host), so any stream will do
    if (ctx->n_partial_bases)
        CK(cudaMemcpyAsync(h.bases.data(), ctx->out_bases.p, ctx->n_partial_bases, cudaMemcpyDeviceToHost, 0));
    if (ctx->n_partial) {
        CK(cudaMemcpyAsync(h.off.data(), ctx->out_off.p, ctx->n_partial * sizeof(uint64_t), cudaMemcpyDeviceToHost, 0));
        CK(cudaMemcpyAsync(h.len.data(), ctx->out_len.p, ctx->n_partial * sizeof(uint32_t), cudaMemcpyDeviceToHost, 0));
        CK(cudaMemcpyAsync(h.flags.data(), ctx->out_flags.p, ctx->n_partial, cudaMemcpyDeviceToHost, 0));
    }
    CK(cudaStreamSynchronize(0));
    ctx->partial_on_host = true;
    return GGCAT_GPU_OK;
}

static int copy_unitigs_out(const HostUnitigs &h, uint8_t *h_bases, uint64_t bases_cap, uint64_t *h_off,
                            uint32_t *h_len, uint8_t *h_flags, uint64_t cap, uint64_t *n_unitigs, uint64_t *n_bases) {
    if (n_unitigs) *n_unitigs = h.off.size();
    if (n_bases) *n_bases = h.bases.size();
    if (h_bases) memcpy(h_bases, h.bases.data(), std::min<uint64_t>(bases_cap, h.bases.size()));
    uint64_t n = std::min<uint64_t>(cap, h.off.size());
    if (h_off) memcpy(h_off, h.off.data(), n * sizeof(uint64_t));
    if (h_len) memcpy(h_len, h.len.data(), n * sizeof(uint32_t));
    if (h_flags) memcpy(h_flags, h.flags.data(), n);
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_partial_unitigs_copy(ggcat_gpu_ctx *ctx, uint8_t *h_bases, uint64_t bases_cap,
                                              uint64_t *h_off, uint32_t *h_len, uint8_t *h_flags, uint64_t cap,
                                              uint64_t *n_unitigs, uint64_t *n_bases) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_merge) return fail(ctx, GGCAT_GPU_EINVAL, "no merge result");
    int rc = fetch_partial(ctx);
    if (rc) return rc;
    return copy_unitigs_out(ctx->partial, h_bases, bases_cap, h_off, h_len, h_flags, cap, n_unitigs, n_bases);
}

extern "C" int ggcat_gpu_kmers_copy(ggcat_gpu_ctx *ctx, uint64_t *h_kmers, uint64_t *h_mult, uint64_t cap, uint64_t *n) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_merge) return fail(ctx, GGCAT_GPU_EINVAL, "no merge result");
    if (n) *n = ctx->n_kmers_out;
    if (!h_kmers) return GGCAT_GPU_OK;
    uint64_t cnt = std::min<uint64_t>(cap, ctx->n_kmers_out);
    const uint64_t words = 1ull << key_width(ctx->last_params.k);
    CK(cudaSetDevice(ctx->device));
    if (cnt) {
        CK(cudaMemcpy(h_kmers, ctx->kmer_keys.p, cnt * words * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        std::vector<uint32_t> m(cnt);
        CK(cudaMemcpy(m.data(), ctx->kmer_mult.p, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < cnt; i++) h_mult[i] = m[i];
    }
    return GGCAT_GPU_OK;
}

// ---------------------------------------------------------------------------
// link stage (device): the kernels of link.cu driven round by round
// ---------------------------------------------------------------------------
static int link_device(ggcat_gpu_ctx *ctx, int k, cudaStream_t s) {
    auto t0 = std::chrono::steady_clock::now();
    HostUnitigs &F = ctx->final_u;
    F.clear();
    const uint64_t n = ctx->n_partial, nn = 2 * n;
    if (nn >= 0xffffffffull) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "link stage: too many partial unitigs");
    const int wide = key_width(k);
    uint64_t cap = 1024;
    while (cap < 2 * nn) cap <<= 1;
    LinkBufs &L = ctx->lk;
    CK(L.keys.ensure(cap << wide));
    CK(L.min12.ensure(2 * cap));
    CK(L.eslot.ensure(nn + 1));
    CK(L.succ.ensure(nn + 1));
    CK(L.jump.ensure(nn + 1));
    CK(L.jump2.ensure(nn + 1));
    CK(L.list.ensure(nn + 1));
    CK(L.cj.ensure(nn + 1));
    CK(L.cm.ensure(nn + 1));
    CK(L.cj2.ensure(nn + 1));
    CK(L.cm2.ensure(nn + 1));
    CK(L.state.ensure(nn + 1));
    CK(L.pr.ensure(nn + 1));
    CK(L.pr2.ensure(nn + 1));
    CK(L.chain_off.ensure(nn + 1));
    CK(L.counters.ensure(8));
    CK(L.out_bases.ensure(ctx->n_partial_bases + 1));
    CK(L.out_off.ensure(n + 1));
    CK(L.out_len.ensure(n + 1));
    CK(L.out_flags.ensure(n + 1));
    CK(cudaMemsetAsync(L.keys.p, 0xff, (cap << wide) * sizeof(uint64_t), s));
    CK(cudaMemsetAsync(L.min12.p, 0xff, 2 * cap * sizeof(uint32_t), s));
    CK(cudaMemsetAsync(L.state.p, 0, nn + 1, s));
    CK(cudaMemsetAsync(L.chain_off.p, 0xff, (nn + 1) * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(L.counters.p, 0, 8 * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
    const int sms = ctx->sms;
    uint32_t *min1 = L.min12.p, *min2 = L.min12.p + cap;
    // pairing and successors (pj / pr start as "no predecessor")
    ctx->launches += launch_link_endpoints(ctx->out_bases.p, ctx->out_off.p, ctx->out_len.p, ctx->out_flags.p, n, k,
                                           ctx->last_params.forward_only ? 1 : 0, L.keys.p, min1, cap - 1, L.eslot.p,
                                           ctx->status.p + 1, sms, s);
    ctx->launches += launch_link_succ(L.eslot.p, min1, min2, nn, L.succ.p, L.jump.p, sms, s);
    auto read_counter = [&](int i, unsigned long long &v) -> int {
        CK(cudaMemcpyAsync(&v, L.counters.p + i, sizeof v, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        return GGCAT_GPU_OK;
    };
    // forward jumping until the unresolved count stops falling: the rest lie on cycles
    uint32_t *jc = L.jump.p, *jn = L.jump2.p;
    unsigned long long prev = ~0ull, cnt = 0;
    int rc = GGCAT_GPU_OK;
    for (int round = 0; round < 64 && nn; round++) {
        CK(cudaMemsetAsync(L.counters.p + 2, 0, sizeof(unsigned long long), s));
        ctx->launches += launch_link_jump(L.succ.p, jc, jn, nn, L.counters.p + 2, sms, s);
        std::swap(jc, jn);
        if ((rc = read_counter(2, cnt))) return rc;
        if (cnt == 0 || cnt == prev) break;
        prev = cnt;
    }
    unsigned long long nc = 0;
    if (cnt) {
        CK(cudaMemsetAsync(L.counters.p + 3, 0, sizeof(unsigned long long), s));
        ctx->launches +=
            launch_link_cycle_list(L.succ.p, jc, nn, L.list.p, L.counters.p + 3, L.cj.p, L.cm.p, sms, s);
        if ((rc = read_counter(3, nc))) return rc;
        uint32_t *a_j = L.cj.p, *a_m = L.cm.p, *b_j = L.cj2.p, *b_m = L.cm2.p;
        for (unsigned long long span = 1; span < 2 * nc; span <<= 1) {
            ctx->launches += launch_link_cycle_min(L.list.p, nc, a_j, a_m, b_j, b_m, sms, s);
            std::swap(a_j, b_j);
            std::swap(a_m, b_m);
        }
        ctx->launches += launch_link_cycle_cut(L.list.p, nc, a_m, L.succ.p, L.state.p, sms, s);
    }
    // predecessor jumping: chain start and base offset of every node
    ctx->launches += launch_link_pred_init(L.succ.p, L.state.p, ctx->out_len.p, nn, k, L.jump.p, L.pr.p, sms, s);
    uint32_t *pc = L.jump.p, *pn = L.jump2.p;
    unsigned long long *rcur = L.pr.p, *rnext = L.pr2.p;
    for (int round = 0; round < 64 && nn; round++) {
        CK(cudaMemsetAsync(L.counters.p + 4, 0, sizeof(unsigned long long), s));
        ctx->launches += launch_link_pred_jump(pc, rcur, pn, rnext, nn, L.counters.p + 4, sms, s);
        std::swap(pc, pn);
        std::swap(rcur, rnext);
        unsigned long long changed = 0;
        if ((rc = read_counter(4, changed))) return rc;
        if (changed == 0) break;
    }
    ctx->launches += launch_link_reserve(L.succ.p, L.state.p, pc, rcur, ctx->out_len.p, ctx->out_flags.p, nn,
                                         L.chain_off.p, L.out_off.p, L.out_len.p, L.out_flags.p, L.counters.p,
                                         ctx->n_partial_bases + 1, n + 1, ctx->status.p + 1, sms, s);
    ctx->launches += launch_link_write(ctx->out_bases.p, ctx->out_off.p, ctx->out_len.p, L.state.p, pc, rcur,
                                       L.chain_off.p, nn, k, L.out_bases.p, sms, s);
    CK(cudaGetLastError());
    unsigned long long tot[2] = {0, 0};
    unsigned st = 0;
    CK(cudaMemcpyAsync(tot, L.counters.p, sizeof tot, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&st, ctx->status.p + 1, sizeof st, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st & (kStatusOutOverflow | kStatusTableFull))
        return fail(ctx, GGCAT_GPU_EDEVICE, "link stage: internal overflow (status %u)", st);
    // the unitigs are packed in reservation order; bytes between them are never read
    CK(F.bases.resize(tot[0]));
    CK(F.off.resize(tot[1]));
    CK(F.len.resize(tot[1]));
    CK(F.flags.resize(tot[1]));
    if (tot[0]) CK(cudaMemcpy(F.bases.data(), L.out_bases.p, tot[0], cudaMemcpyDeviceToHost));
    if (tot[1]) {
        CK(cudaMemcpy(F.off.data(), L.out_off.p, tot[1] * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(F.len.data(), L.out_len.p, tot[1] * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(F.flags.data(), L.out_flags.p, tot[1], cudaMemcpyDeviceToHost));
    }
    ctx->n_final = tot[1];
    ctx->n_final_bases = tot[0];
    auto t1 = std::chrono::steady_clock::now();
    ctx->stats.ms_link = std::chrono::duration<double, std::milli>(t1 - t0).count();
    ctx->stats.final_unitigs = F.off.size();
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_link(ggcat_gpu_ctx *ctx, int k) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_merge) return fail(ctx, GGCAT_GPU_EINVAL, "no merge result");
    if (k < 3 || k > 127) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "link stage supports k <= 127");
    if (k != ctx->last_params.k) return fail(ctx, GGCAT_GPU_EINVAL, "link k=%d differs from the build k=%d", k,
                                             ctx->last_params.k);
    CK(cudaSetDevice(ctx->device));
    return link_device(ctx, k, ctx->cap_stream);
}

extern "C" int ggcat_gpu_unitigs_copy(ggcat_gpu_ctx *ctx, uint8_t *h_bases, uint64_t bases_cap, uint64_t *h_off,
                                      uint32_t *h_len, uint8_t *h_flags, uint64_t cap, uint64_t *n_unitigs,
                                      uint64_t *n_bases) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    return copy_unitigs_out(ctx->final_u, h_bases, bases_cap, h_off, h_len, h_flags, cap, n_unitigs, n_bases);
}

extern "C" int ggcat_gpu_get_stats(const ggcat_gpu_ctx *ctx, ggcat_gpu_stats *out) {
    if (!ctx || !out) return GGCAT_GPU_EINVAL;
    *out = ctx->stats;
    out->merge_graph_captures = ctx->merge_graph_captures;
    out->merge_graph_replays = ctx->merge_graph_replays;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_build_text(ggcat_gpu_ctx *ctx, const uint8_t *h_text, uint64_t text_len,
                                    const ggcat_gpu_params *p, void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (text_len > 0 && !h_text) return fail(ctx, GGCAT_GPU_EINVAL, "null text");
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    CK(ctx->d_text.ensure(text_len + 64));
    // stage through pinned memory so the copy is a true async DMA
    cudaPointerAttributes attr{};
    bool pinned = cudaPointerGetAttributes(&attr, h_text) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (pinned) {
        // pipelined: the copy runs on its own stream in kFeedPieces pieces (multiples of a
        // bucketize block), each packed and bucketized while the next ones are in flight
        int rc = check_params(ctx, p);
        if (rc) return rc;
        const BucketizeGeometry geo = bucketize_geometry(text_len, p->k, p->m);
        const uint64_t bb = bucketize_block_bases(geo);
        // every piece at least a wave of bucketize blocks (3 per SM): the pieces' kernels run on
        // their own streams and overlap, so smaller pieces start the bucketing earlier; a wave
        // per piece measured best at 1 Gbp (8 pieces: 31.8 ms per build from pinned memory, 4:
        // 32.9, 12: 32.6, 16: 33.3)
        const uint64_t wave = (uint64_t)ctx->sms * 3;
        const int want = p->copy_pieces > 0 ? (int)std::min<uint64_t>(p->copy_pieces, geo.blocks)
                                            : (int)std::min<uint64_t>(kFeedPieces, geo.blocks / wave);
        const uint64_t per = want > 1 ? (geo.blocks + want - 1) / want : geo.blocks;
        uint64_t off[kFeedPieces + 1];
        int pieces = 0;
        off[0] = 0;
        while (off[pieces] < text_len && pieces < kFeedPieces) {
            off[pieces + 1] = std::min<uint64_t>(text_len, off[pieces] + per * bb);
            pieces++;
        }
        if (pieces <= 1) {
            CK(cudaMemcpyAsync(ctx->d_text.p, h_text, text_len, cudaMemcpyHostToDevice, s));
        } else {
            if (!ctx->copy_stream) CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
            for (auto &e : ctx->feed_ev)
                if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            // the copies overwrite the text only after the work already queued on s
            CK(cudaEventRecord(ctx->feed_ev[0], s));
            CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->feed_ev[0], 0));
            for (int i = 0; i < pieces; i++) {
                CK(cudaMemcpyAsync(ctx->d_text.p + off[i], h_text + off[i], off[i + 1] - off[i], cudaMemcpyHostToDevice,
                                   ctx->copy_stream));
                CK(cudaEventRecord(ctx->feed_ev[1 + i], ctx->copy_stream));
            }
            const TextFeed feed{pieces, off, ctx->feed_ev + 1};
            uint64_t nsk = 0;
            rc = bucketize_impl(ctx, ctx->d_text.p, text_len, p, stream, &nsk, &feed);
            if (rc) return rc;
            rc = ggcat_gpu_merge(ctx, p, stream);
            if (rc) return rc;
            return fetch_partial(ctx);
        }
    } else {
        const uint64_t chunk = 64ull << 20;
        CK(ctx->h_stage.ensure(2 * chunk));
        for (uint64_t o = 0, i = 0; o < text_len; o += chunk, i++) {
            uint64_t nb = std::min<uint64_t>(chunk, text_len - o);
            uint8_t *st = ctx->h_stage.p + (i & 1) * chunk;
            if (i >= 2) CK(cudaStreamSynchronize(s));
            memcpy(st, h_text + o, nb);
            CK(cudaMemcpyAsync(ctx->d_text.p + o, st, nb, cudaMemcpyHostToDevice, s));
        }
    }
    uint64_t nsk = 0;
    int rc = ggcat_gpu_bucketize(ctx, ctx->d_text.p, text_len, p, stream, &nsk);
    if (rc) return rc;
    rc = ggcat_gpu_merge(ctx, p, stream);
    if (rc) return rc;
    return fetch_partial(ctx);
}

// buckets count heuristic of compute_stats_from_input_blocks (crates/io/src/lib.rs:67-140)
static void bucket_counts_for(uint64_t bases, int *bbits, int *sbits) {
    const uint64_t MAX_BUCKET_SIZE = 1ull << 30, MIN_BUCKET_SIZE = 512ull << 10;
    uint64_t bc = std::max<uint64_t>(std::min<uint64_t>(1024, bases / MIN_BUCKET_SIZE), bases / MAX_BUCKET_SIZE);
    uint64_t p2 = 1;
    while (p2 < bc) p2 <<= 1;
    p2 = std::max<uint64_t>(std::min<uint64_t>(p2, 1ull << 13), 1ull << 2);
    int b = 0;
    while ((1ull << b) < p2) b++;
    uint64_t per = bases / p2;
    uint64_t sc = std::max<uint64_t>(std::min<uint64_t>(64, per / (2 * 1024)), per / (4ull << 20));
    uint64_t s2 = 1;
    while (s2 < sc) s2 <<= 1;
    s2 = std::max<uint64_t>(std::min<uint64_t>(s2, 1ull << 8), 1ull << 1);
    int s = 0;
    while ((1ull << s) < s2) s++;
    *bbits = b;
    *sbits = s;
}

// Colour subset of every k-mer of the final unitigs of the last link stage, through the
// coloured index (built here from the last ggcat_gpu_colors result): subs[kbase[u] + j] is the
// subset of k-mer j of unitig u.
static int final_kmer_subsets(ggcat_gpu_ctx *ctx, std::vector<uint32_t> &subs, std::vector<uint64_t> &kbase) {
    const int k = ctx->last_params.k;
    int rc = ggcat_gpu_query_index_colored(ctx, nullptr);
    if (rc) return rc;
    const HostUnitigs &F = ctx->final_u;
    const uint64_t n = F.off.size();
    kbase.assign(n + 1, 0);
    std::vector<uint32_t> iu, ifirst, icnt;
    constexpr uint32_t kItem = 512;
    for (uint64_t u = 0; u < n; u++) {
        const uint64_t nk = F.len[u] >= (uint32_t)k ? F.len[u] - (uint32_t)k + 1 : 0;
        kbase[u + 1] = kbase[u] + nk;
        for (uint64_t j = 0; j < nk; j += kItem) {
            iu.push_back((uint32_t)u);
            ifirst.push_back((uint32_t)j);
            icnt.push_back((uint32_t)std::min<uint64_t>(kItem, nk - j));
        }
    }
    const uint64_t total = kbase[n], ni = iu.size();
    subs.assign(total, 0xffffffffu);
    if (!ni) return GGCAT_GPU_OK;
    DevBuf<uint32_t> d_iu, d_if, d_ic, d_out;
    DevBuf<uint64_t> d_kb;
    CK(d_iu.ensure(ni));
    CK(d_if.ensure(ni));
    CK(d_ic.ensure(ni));
    CK(d_kb.ensure(n + 1));
    CK(d_out.ensure(total));
    cudaStream_t s = ctx->cap_stream;
    CK(cudaMemcpyAsync(d_iu.p, iu.data(), ni * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_if.p, ifirst.data(), ni * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_ic.p, icnt.data(), ni * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_kb.p, kbase.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s));
    ctx->launches += launch_unitig_subsets(ctx->lk.out_bases.p, ctx->lk.out_off.p, ctx->lk.out_len.p, d_iu.p, d_if.p,
                                           d_ic.p, ni, d_kb.p, k, ctx->qkeys.p, ctx->qvals.p, ctx->qmask, d_out.p, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(subs.data(), d_out.p, total * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (uint64_t i = 0; i < total; i++)
        if (subs[i] == 0xffffffffu)
            return fail(ctx, GGCAT_GPU_EDEVICE, "a k-mer of the final unitigs has no colour subset");
    return GGCAT_GPU_OK;
}

// The colormap of the last colour result: subset i = the set bits of its bitmap.
static int write_colormap_of(ggcat_gpu_ctx *ctx, const std::string &path, const std::vector<std::string> &names) {
    const uint64_t ns = ctx->c_n_subsets;
    const int w = ctx->c_words;
    std::vector<uint32_t> bm(ns * (uint64_t)w);
    if (!bm.empty()) CK(cudaMemcpy(bm.data(), ctx->csub_arena.p, bm.size() * 4, cudaMemcpyDeviceToHost));
    const int rc = cmap::write(path.c_str(), names, ns, [&](uint64_t i, std::vector<uint32_t> &out) {
        out.clear();
        for (int j = 0; j < w; j++)
            for (uint32_t x = bm[i * (uint64_t)w + j]; x; x &= x - 1) out.push_back((uint32_t)(32 * j + __builtin_ctz(x)));
    });
    if (rc) return fail(ctx, rc, "cannot write the colormap %s", path.c_str());
    return GGCAT_GPU_OK;
}

// The build of ggcat_build_from_files / GGCATInstance::build_graph once its inputs are text:
// the parameters as the reference derives them, the device build (with colours: the colour
// subsets of every k-mer), the link stage, then the output: FASTA ">{id} LN:i:{len}" with the
// C:{subset}:{count} runs of a coloured graph and the L: annotations of ExtraElaboration::
// UnitigLinks, or GFA v1 / v2; with colours also the colormap "<output>.colors.dat".
// seq_off: with colours, the text offset where each colour's sequences start (colour i =
// input i, MinBkSingleColor).
static int build_and_write(ggcat_gpu_ctx *ctx, const std::vector<uint8_t> &text, const char *output_file,
                           size_t kmer_length, int forward_only, size_t minimizer_length, size_t min_multiplicity,
                           int colors = 0, const std::vector<uint64_t> *seq_off = nullptr,
                           const std::vector<std::string> *color_names = nullptr, int extra_elab = 0,
                           int gfa_output_version = 0) {
    if (colors && gfa_output_version) return fail(ctx, GGCAT_GPU_EINVAL, "GFA output is not supported with colors");
    if (colors && forward_only)
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "coloured forward-only builds are not built (canonical index)");
    const uint64_t est = text.size();
    ggcat_gpu_params p{};
    p.k = (int)kmer_length;
    // compute_best_m (crates/utils/src/lib.rs:29-40) when minimizer_length == SIZE_MAX
    if (minimizer_length == (size_t)-1) {
        int k = p.k;
        p.m = k <= 13   ? std::max(k / 2, k - 4)
              : k <= 15 ? 9
              : k <= 21 ? 10
              : k <= 30 ? 11
              : k <= 37 ? 12
              : k <= 42 ? 13
              : k <= 64 ? 14
                        : (k + 2) / 4;  // round(k / 4), halves away from zero
    } else {
        p.m = (int)minimizer_length;
    }
    bucket_counts_for(est, &p.bucket_bits, &p.second_bits);
    p.min_multiplicity = (int)min_multiplicity;
    // HashType::Auto (crates/api/src/utils.rs:17-25): sequence hash up to k = 64, Rabin-Karp above
    p.hash_kind = p.k <= 64 ? GGCAT_HASH_SEQHASH : GGCAT_HASH_RABIN_KARP128;
    p.forward_only = forward_only;
    p.merge_mode = GGCAT_MERGE_BATCHED;
    p.keep_kmers = colors ? 1 : 0;
    // colour i = input file i (MinBkSingleColor); announced so that the merge collects them
    const uint64_t nc = colors && seq_off ? seq_off->size() : 0;
    if (colors && (nc == 0 || nc > 65536))
        return fail(ctx, GGCAT_GPU_EINVAL, "colours need 1 to 65536 inputs (%llu)", (unsigned long long)nc);
    std::vector<uint32_t> col(nc);
    for (uint64_t i = 0; i < nc; i++) col[i] = (uint32_t)i;
    int rc = ggcat_gpu_colors_prepare(ctx, nc ? seq_off->data() : nullptr, col.data(), nc, (uint32_t)nc);
    if (rc) return rc;
    rc = ggcat_gpu_build_text(ctx, text.data(), text.size(), &p, nullptr);
    if (rc) return rc;
    std::vector<std::string> names;
    if (colors) {
        rc = ggcat_gpu_colors(ctx, seq_off->data(), col.data(), nc, (uint32_t)nc, nullptr);
        if (rc) return rc;
        if (color_names) names = *color_names;
    }
    rc = ggcat_gpu_link(ctx, p.k);
    if (rc) return rc;
    const HostUnitigs &F = ctx->final_u;
    const uint64_t n = F.off.size();
    std::vector<uint32_t> subs;
    std::vector<uint64_t> kbase;
    if (colors) {
        rc = final_kmer_subsets(ctx, subs, kbase);
        if (rc) return rc;
        rc = write_colormap_of(ctx, ggcat_colormap_path(output_file), names);
        if (rc) return rc;
    }
    // " C:{subset:x}:{count}" per run of equal subsets along the unitig (multiple.rs:705-740)
    HeaderExtra runs = [&](uint64_t u, std::string &line) {
        char buf[48];
        uint64_t j = kbase[u];
        while (j < kbase[u + 1]) {
            uint64_t e = j + 1;
            while (e < kbase[u + 1] && subs[e] == subs[j]) e++;
            snprintf(buf, sizeof buf, " C:%x:%llu", subs[j], (unsigned long long)(e - j));
            line += buf;
            j = e;
        }
    };
    std::vector<uint64_t> off64(F.off.data(), F.off.data() + n), len64(n);
    for (uint64_t i = 0; i < n; i++) len64[i] = F.len[i];
    std::string err;
    if (extra_elab >= 2) {
        // matchtigs / eulertigs / pathtigs of the final unitigs, written in their place; with
        // colours (eulertigs and pathtigs: every k-mer once, in the order of its unitig or
        // reversed) the runs of the k-mers' subsets along each string
        std::vector<uint8_t> tb;
        std::vector<uint64_t> to, tl, walk, walk_end;
        rc = ggcat::compute_tigs(F.bases.data(), off64.data(), len64.data(), n, p.k, extra_elab, tb, to, tl, err, &walk,
                                 &walk_end);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
        HeaderExtra tig_runs = [&](uint64_t t, std::string &line) {
            char buf[48];
            uint32_t cur = 0;
            uint64_t cnt = 0;
            auto flush = [&]() {
                if (!cnt) return;
                snprintf(buf, sizeof buf, " C:%x:%llu", cur, (unsigned long long)cnt);
                line += buf;
            };
            auto add = [&](uint32_t sub) {
                if (cnt && sub == cur) {
                    cnt++;
                    return;
                }
                flush();
                cur = sub;
                cnt = 1;
            };
            for (uint64_t w = t ? walk_end[t - 1] : 0; w < walk_end[t]; w++) {
                const uint64_t u = walk[w] >> 1;
                if (!(walk[w] & 1))
                    for (uint64_t j = kbase[u]; j < kbase[u + 1]; j++) add(subs[j]);
                else
                    for (uint64_t j = kbase[u + 1]; j-- > kbase[u];) add(subs[j]);
            }
            flush();
        };
        rc = ggcat::write_graph_arrays(tb.data(), to.data(), tl.data(), to.size(), p.k, 0, gfa_output_version,
                                       colors ? &tig_runs : nullptr, output_file, err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
        return GGCAT_GPU_OK;
    }
    rc = ggcat::write_graph_arrays(F.bases.data(), off64.data(), len64.data(), n, p.k, extra_elab == 1,
                                   gfa_output_version, colors ? &runs : nullptr, output_file, err);
    if (rc) return fail(ctx, rc, "%s", err.c_str());
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_build_from_files(ggcat_gpu_ctx *ctx, const char *const *input_files, size_t n_inputs,
                                          const char *output_file, size_t kmer_length, size_t threads_count,
                                          int forward_only, size_t minimizer_length, size_t min_multiplicity) {
    if (!ctx || !input_files || !output_file) return GGCAT_GPU_EINVAL;
    std::vector<uint8_t> text;
    {
        // FASTA / FASTQ by extension, decompressed by the last one, files on threads_count host
        // threads (all of them when 0) and concatenated in input order (input.cpp)
        const int nt = threads_count > 0 ? (int)std::min<size_t>(threads_count, 1024)
                                         : (int)std::max(1u, std::thread::hardware_concurrency());
        std::string err;
        const int rc = ggcat::read_sequences_files(input_files, n_inputs, (int64_t)kmer_length - 1, nt, text, err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
    }
    return build_and_write(ctx, text, output_file, kmer_length, forward_only, minimizer_length, min_multiplicity);
}

extern "C" int ggcat_gpu_build_from_streams(ggcat_gpu_ctx *ctx, const ggcat_gpu_stream *streams, size_t n_streams,
                                            const char *output_file, size_t kmer_length, size_t threads_count,
                                            int forward_only, size_t minimizer_length, size_t min_multiplicity) {
    (void)threads_count;  // the streams are read on the calling thread
    if (!ctx || (n_streams && !streams) || !output_file) return GGCAT_GPU_EINVAL;
    std::vector<uint8_t> text;
    const int rc = ggcat::collect_streams(streams, n_streams, (int64_t)kmer_length - 1, text);
    if (rc) return fail(ctx, rc, "a stream has no read_block function");
    return build_and_write(ctx, text, output_file, kmer_length, forward_only, minimizer_length, min_multiplicity);
}

// ggcat_build_from_files with every argument (crates/capi/src/lib.rs:58-139, same order):
// colour names and colours (colour i = input file i), extra_elab (0 none, 1 unitig links;
// 2-4 greedy matchtigs, eulertigs, pathtigs of an uncoloured graph) and gfa_output_version
// (0 FASTA, 1, 2)
extern "C" int ggcat_gpu_build_from_files_ex(ggcat_gpu_ctx *ctx, const char *const *input_files, size_t n_inputs,
                                             const char *output_file, const char *const *color_names,
                                             size_t n_color_names, size_t kmer_length, size_t threads_count,
                                             int forward_only, size_t minimizer_length, int colors,
                                             size_t min_multiplicity, int extra_elab, int gfa_output_version) {
    if (!ctx || !input_files || !output_file || (n_color_names && !color_names)) return GGCAT_GPU_EINVAL;
    if (extra_elab < 0 || extra_elab > 4 || gfa_output_version < 0 || gfa_output_version > 2)
        return fail(ctx, GGCAT_GPU_EINVAL, "extra_elab %d / gfa_output_version %d out of range", extra_elab,
                    gfa_output_version);
    if (extra_elab == GGCAT_GPU_TIGS_GREEDY_MATCHTIGS && colors)
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "greedy matchtigs of a coloured graph are not built");
    std::vector<uint8_t> text;
    std::vector<uint64_t> file_off;
    {
        const int nt = threads_count > 0 ? (int)std::min<size_t>(threads_count, 1024)
                                         : (int)std::max(1u, std::thread::hardware_concurrency());
        std::string err;
        const int rc = ggcat::read_sequences_files(input_files, n_inputs, (int64_t)kmer_length - 1, nt, text, err,
                                                   &file_off);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
    }
    std::vector<std::string> names;
    for (size_t i = 0; i < n_color_names; i++) names.emplace_back(color_names[i] ? color_names[i] : "");
    return build_and_write(ctx, text, output_file, kmer_length, forward_only, minimizer_length, min_multiplicity,
                           colors, &file_off, &names, extra_elab, gfa_output_version);
}

// ---------------------------------------------------------------------------
// colour subsets
// ---------------------------------------------------------------------------
extern "C" int ggcat_gpu_colors_prepare(ggcat_gpu_ctx *ctx, const uint64_t *h_seq_off, const uint32_t *h_seq_color,
                                        uint64_t n_seq, uint32_t n_colors) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    ctx->cprep = false;
    if (n_seq == 0) return GGCAT_GPU_OK;  // withdraws an earlier announcement
    if (!h_seq_off || !h_seq_color || n_colors == 0 || n_colors > 65536 || n_seq >= 0xffffffffull)
        return fail(ctx, GGCAT_GPU_EINVAL, "bad colour table (n_seq=%llu, n_colors=%u)", (unsigned long long)n_seq,
                    n_colors);
    for (uint64_t i = 0; i < n_seq; i++) {
        if (h_seq_color[i] >= n_colors) return fail(ctx, GGCAT_GPU_EINVAL, "colour out of range at sequence %llu",
                                                    (unsigned long long)i);
        if (i && h_seq_off[i] < h_seq_off[i - 1]) return fail(ctx, GGCAT_GPU_EINVAL, "sequence offsets not sorted");
    }
    CK(cudaSetDevice(ctx->device));
    ctx->cprep_off.assign(h_seq_off, h_seq_off + n_seq);
    ctx->cprep_col.assign(h_seq_color, h_seq_color + n_seq);
    ctx->cprep_colors = n_colors;
    CK(ctx->cprep_off_d.ensure(n_seq));
    CK(ctx->cprep_col_d.ensure(n_seq));
    CK(cudaMemcpy(ctx->cprep_off_d.p, h_seq_off, n_seq * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->cprep_col_d.p, h_seq_color, n_seq * sizeof(uint32_t), cudaMemcpyHostToDevice));
    ctx->cprep = true;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_colors(ggcat_gpu_ctx *ctx, const uint64_t *h_seq_off, const uint32_t *h_seq_color,
                                uint64_t n_seq, uint32_t n_colors, void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_merge || !ctx->last_params.keep_kmers)
        return fail(ctx, GGCAT_GPU_EINVAL, "colours need a merge run with keep_kmers = 1");
    if (!h_seq_off || !h_seq_color || n_seq == 0 || n_colors == 0 || n_colors > 65536)
        return fail(ctx, GGCAT_GPU_EINVAL, "bad colour table (n_seq=%llu, n_colors=%u)", (unsigned long long)n_seq,
                    n_colors);
    uint64_t max_len = 0;
    for (uint64_t i = 0; i < n_seq; i++) {
        if (h_seq_color[i] >= n_colors) return fail(ctx, GGCAT_GPU_EINVAL, "colour out of range at sequence %llu",
                                                    (unsigned long long)i);
        if (i && h_seq_off[i] < h_seq_off[i - 1]) return fail(ctx, GGCAT_GPU_EINVAL, "sequence offsets not sorted");
        const uint64_t end = i + 1 < n_seq ? h_seq_off[i + 1] : ctx->n_text;
        if (end < h_seq_off[i] || end > ctx->n_text)
            return fail(ctx, GGCAT_GPU_EINVAL, "sequence %llu outside the text", (unsigned long long)i);
        max_len = std::max<uint64_t>(max_len, end - h_seq_off[i]);
    }
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    ctx->have_colors = false;
    const uint64_t nd = ctx->n_kmers_out;
    if (nd >= 0xffffffffull) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "colours support < 2^32 k-mers");
    if (ctx->last_params.k > 64) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "colours support k <= 64");
    const int words = (int)((n_colors + 31) / 32);
    uint64_t cap = 1024;
    while (cap < 2 * nd + 64) cap <<= 1;
    uint64_t scap = 1024;
    while (scap < 2 * nd + 64) scap <<= 1;
    const int wide = ctx->last_params.k > 32;
    const uint64_t slot_words = wide ? 4 : 2;
    CK(ctx->cslots.ensure(slot_words * cap));
    CK(ctx->cowner.ensure(nd + 1));
    CK(ctx->cbitmaps.ensure((nd + 1) * (uint64_t)words));
    CK(ctx->cid_subset.ensure(nd + 1));
    CK(ctx->cdump_subset.ensure(nd + 1));
    CK(ctx->csub_hash.ensure(scap));
    CK(ctx->csub_state.ensure(scap));
    CK(ctx->csub_arena.ensure((nd + 1) * (uint64_t)words));
    CK(ctx->ccounters.ensure(4));
    CK(ctx->cseq_off.ensure(n_seq));
    CK(ctx->cseq_color.ensure(n_seq));
    // the merge collected these colours (the same table was announced before the build): no
    // pass over the text, the dumped copies' bitmaps are merged into their owners
    const bool collected = ctx->merge_collected && ctx->cprep && ctx->cprep_colors == n_colors &&
                           ctx->cprep_off.size() == n_seq &&
                           std::equal(ctx->cprep_off.begin(), ctx->cprep_off.end(), h_seq_off) &&
                           std::equal(ctx->cprep_col.begin(), ctx->cprep_col.end(), h_seq_color);
    if (!collected) {
        CK(cudaMemcpyAsync(ctx->cseq_off.p, h_seq_off, n_seq * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->cseq_color.p, h_seq_color, n_seq * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(ctx->cbitmaps.p, 0, (nd + 1) * words * sizeof(uint32_t), s));
    }
    CK(cudaMemsetAsync(ctx->cslots.p, 0xff, slot_words * cap * sizeof(uint64_t), s));
    CK(cudaMemsetAsync(ctx->csub_hash.p, 0, scap * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(ctx->csub_state.p, 0, scap * sizeof(uint32_t), s));
    CK(cudaMemsetAsync(ctx->ccounters.p, 0, 4 * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
    if (collected)
        ctx->launches += launch_color_phase_collected(
            ctx->kmer_keys.p, nd, wide, words, ctx->cslots.p, cap - 1, ctx->cowner.p, ctx->cbitmaps.p,
            ctx->ccounters.p + 1, ctx->csub_hash.p, ctx->csub_state.p, ctx->csub_arena.p, scap - 1, ctx->cid_subset.p,
            ctx->cdump_subset.p, ctx->status.p + 1, ctx->sms, s);
    else
        ctx->launches += launch_color_phase(ctx->kmer_keys.p, nd, ctx->last_text, ctx->n_text, ctx->last_params.k,
                                            ctx->last_params.forward_only ? 0 : 1, wide, ctx->cseq_off.p,
                                            ctx->cseq_color.p, n_seq, h_seq_off[0] == 0 ? max_len : 0, words,
                                            ctx->cslots.p, cap - 1, ctx->cowner.p, ctx->cbitmaps.p,
                                            ctx->ccounters.p + 1, ctx->csub_hash.p, ctx->csub_state.p,
                                            ctx->csub_arena.p, scap - 1, ctx->cid_subset.p, ctx->cdump_subset.p,
                                            ctx->status.p + 1, ctx->sms, s);
    ctx->stats.colors_collected = collected ? 1 : 0;
    CK(cudaGetLastError());
    unsigned long long cnt[2];
    unsigned st = 0;
    CK(cudaMemcpyAsync(cnt, ctx->ccounters.p, sizeof cnt, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&st, ctx->status.p + 1, sizeof st, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st) return fail(ctx, GGCAT_GPU_EDEVICE, "colour phase: internal error (status %u)", st);
    ctx->cmask = cap - 1;
    ctx->c_n_ids = nd;  // ids are dump indices (holes for k-mers dumped twice)
    ctx->c_n_subsets = cnt[1];
    ctx->c_words = words;
    ctx->c_colors = n_colors;
    ctx->have_colors = true;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_kmer_subsets_copy(ggcat_gpu_ctx *ctx, uint32_t *h_subset, uint64_t cap, uint64_t *n) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_colors) return fail(ctx, GGCAT_GPU_EINVAL, "no colour result");
    if (n) *n = ctx->n_kmers_out;
    if (!h_subset) return GGCAT_GPU_OK;
    CK(cudaSetDevice(ctx->device));
    const uint64_t m = std::min<uint64_t>(cap, ctx->n_kmers_out);
    if (m) CK(cudaMemcpy(h_subset, ctx->cdump_subset.p, m * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_subsets_copy(ggcat_gpu_ctx *ctx, uint32_t *h_bitmaps, uint64_t cap_words, uint64_t *n_subsets,
                                      uint32_t *words_per_subset) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_colors) return fail(ctx, GGCAT_GPU_EINVAL, "no colour result");
    if (n_subsets) *n_subsets = ctx->c_n_subsets;
    if (words_per_subset) *words_per_subset = (uint32_t)ctx->c_words;
    if (!h_bitmaps) return GGCAT_GPU_OK;
    CK(cudaSetDevice(ctx->device));
    const uint64_t m = std::min<uint64_t>(cap_words, ctx->c_n_subsets * (uint64_t)ctx->c_words);
    if (m) CK(cudaMemcpy(h_bitmaps, ctx->csub_arena.p, m * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return GGCAT_GPU_OK;
}

// ---------------------------------------------------------------------------
// graph query lookup
// ---------------------------------------------------------------------------
extern "C" int ggcat_gpu_query_index(ggcat_gpu_ctx *ctx, const uint8_t *d_graph_text, uint64_t len, int k,
                                     void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (k < 3 || k > 64) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "query index supports k <= 64 (k=%d)", k);
    const uint64_t kw = k > 32 ? 2 : 1;  // key words (u128 keys above k = 32)
    if (len > 0 && !d_graph_text) return fail(ctx, GGCAT_GPU_EINVAL, "null graph text");
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    ctx->qready = false;
    uint64_t cap = 1024;
    while (cap < 2 * len + 64) cap <<= 1;  // one slot per k-mer position at load <= 0.5
    CK(ctx->qkeys.ensure(cap * kw));
    CK(ctx->qvals.ensure(cap));
    CK(cudaMemsetAsync(ctx->qkeys.p, 0xff, cap * kw * sizeof(uint64_t), s));
    CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
    ctx->launches += launch_index_insert(d_graph_text, len, k, ctx->qkeys.p, ctx->qvals.p, cap - 1, ctx->status.p + 1, s);
    CK(cudaGetLastError());
    unsigned st = 0;
    CK(cudaMemcpyAsync(&st, ctx->status.p + 1, sizeof st, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st) return fail(ctx, GGCAT_GPU_EDEVICE, "query index: table full");
    ctx->qmask = cap - 1;
    ctx->qk = k;
    ctx->qcolored = false;
    ctx->qready = true;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_index_colored(ggcat_gpu_ctx *ctx, void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->have_colors) return fail(ctx, GGCAT_GPU_EINVAL, "no colour result to index");
    if (ctx->last_params.forward_only)
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "the device query index is canonical (forward_only=1)");
    cudaStream_t s = as_stream(stream);
    CK(cudaSetDevice(ctx->device));
    ctx->qready = false;
    const int wide = ctx->last_params.k > 32;
    const uint64_t kw = wide ? 2 : 1;  // key words (u128 keys above k = 32)
    uint64_t cap = 1024;
    while (cap < 2 * ctx->c_n_ids + 64) cap <<= 1;
    CK(ctx->qkeys.ensure(cap * kw));
    CK(ctx->qvals.ensure(cap));
    CK(cudaMemsetAsync(ctx->qkeys.p, 0xff, cap * kw * sizeof(uint64_t), s));
    CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
    ctx->launches += launch_index_from_colors(ctx->cslots.p, ctx->cmask + 1, ctx->cid_subset.p, wide, ctx->qkeys.p,
                                              ctx->qvals.p, cap - 1, ctx->status.p + 1, ctx->sms, s);
    CK(cudaGetLastError());
    unsigned st = 0;
    CK(cudaMemcpyAsync(&st, ctx->status.p + 1, sizeof st, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (st) return fail(ctx, GGCAT_GPU_EDEVICE, "coloured query index: table full");
    ctx->qmask = cap - 1;
    ctx->qk = ctx->last_params.k;
    ctx->qcolored = true;
    ctx->qready = true;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_submit(ggcat_gpu_ctx *ctx, int slot, const uint8_t *h_text, uint64_t len,
                                      const uint64_t *h_off, const uint64_t *h_len, uint64_t nq) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!ctx->qready) return fail(ctx, GGCAT_GPU_EINVAL, "no query index");
    if (slot < 0 || slot >= GGCAT_GPU_QUERY_SLOTS) return fail(ctx, GGCAT_GPU_EINVAL, "bad slot %d", slot);
    if (nq >= (1ull << 32)) return fail(ctx, GGCAT_GPU_EINVAL, "too many queries in one batch");
    auto &q = ctx->qslots[slot];
    if (q.busy) return fail(ctx, GGCAT_GPU_EINVAL, "slot %d is busy", slot);
    CK(cudaSetDevice(ctx->device));
    if (!q.stream) {
        CK(cudaStreamCreateWithFlags(&q.stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&q.done, cudaEventDisableTiming));
    }
    const int k = ctx->qk;
    for (uint64_t i = 0; i < nq; i++)
        if (h_off[i] + h_len[i] > len)
            return fail(ctx, GGCAT_GPU_EINVAL, "query %llu outside the text", (unsigned long long)i);
    cudaStream_t s = q.stream;
    CK(q.h_text.ensure(len + 1));
    par_memcpy(q.h_text.p, h_text, len);
    CK(q.d_text.ensure(len + 1));
    CK(q.d_matched.ensure(nq + 1));
    CK(q.d_status.ensure(1));
    CK(q.h_out.ensure(nq * sizeof(unsigned long long) + 16));
    CK(cudaMemcpyAsync(q.d_text.p, q.h_text.p, len, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(q.d_matched.p, 0, nq * sizeof(unsigned long long), s));
    q.colored = ctx->qcolored;
    const bool warp_colored = ctx->qcolored && ctx->c_words <= kColorWarpMaxWords;
    if (!ctx->qcolored || warp_colored) {
        // work items: runs of at most kChunk k-mer positions of one query, sized so that a small
        // batch still spreads over every warp (coloured: one warp per item) or thread (one
        // thread per item) the GPU holds at once, and a large one takes the longest runs
        uint64_t total_nk = 0;
        for (uint64_t i = 0; i < nq; i++) total_nk += h_len[i] >= (uint64_t)k ? h_len[i] - (uint64_t)k + 1 : 0;
        const uint64_t workers = warp_colored ? (uint64_t)ctx->sms * 64 : (uint64_t)ctx->sms * 2048;
        const uint64_t lo_chunk = warp_colored ? 256 : 64, hi_chunk = warp_colored ? query_color_chunk() : 2048;
        const uint64_t kChunk = std::min<uint64_t>(hi_chunk, std::max<uint64_t>(lo_chunk, (total_nk / workers + 31) & ~(uint64_t)31));
        uint64_t n_items = 0;
        for (uint64_t i = 0; i < nq; i++) {
            const uint64_t nk = h_len[i] >= (uint64_t)k ? h_len[i] - (uint64_t)k + 1 : 0;
            n_items += (nk + kChunk - 1) / kChunk;
        }
        CK(q.h_items.ensure(n_items * 16 + 16));
        uint32_t *iq = reinterpret_cast<uint32_t *>(q.h_items.p);
        uint64_t *is = reinterpret_cast<uint64_t *>(q.h_items.p + n_items * 4);
        uint32_t *il = reinterpret_cast<uint32_t *>(q.h_items.p + n_items * 12);
        uint64_t it = 0;
        for (uint64_t i = 0; i < nq; i++) {
            const uint64_t nk = h_len[i] >= (uint64_t)k ? h_len[i] - (uint64_t)k + 1 : 0;
            for (uint64_t c = 0; c < nk; c += kChunk, it++) {
                iq[it] = (uint32_t)i;
                is[it] = h_off[i] + c;
                il[it] = (uint32_t)std::min<uint64_t>(kChunk, nk - c);
            }
        }
        CK(q.d_iq.ensure(n_items + 1));
        CK(q.d_is.ensure(n_items + 1));
        CK(q.d_il.ensure(n_items + 1));
        CK(cudaMemcpyAsync(q.d_iq.p, iq, n_items * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(q.d_is.p, is, n_items * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(q.d_il.p, il, n_items * 4, cudaMemcpyHostToDevice, s));
        if (!warp_colored) {
            ctx->launches += launch_query(q.d_text.p, k, q.d_iq.p, q.d_is.p, q.d_il.p, n_items, ctx->qkeys.p,
                                          ctx->qmask, q.d_matched.p, s);
        } else {
            const uint64_t nc = ctx->c_colors;
            CK(q.d_counts.ensure(nq * nc + 1));
            CK(q.h_counts.ensure(nq * nc * sizeof(unsigned long long) + 16));
            CK(cudaMemsetAsync(q.d_counts.p, 0, nq * nc * sizeof(unsigned long long), s));
            ctx->launches += launch_query_color_items(q.d_text.p, k, q.d_iq.p, q.d_is.p, q.d_il.p, n_items,
                                                      ctx->qkeys.p, ctx->qvals.p, ctx->qmask, ctx->csub_arena.p,
                                                      ctx->c_words, ctx->c_colors, q.d_matched.p, q.d_counts.p,
                                                      ctx->sms, s);
            CK(cudaMemcpyAsync(q.h_counts.p, q.d_counts.p, nq * nc * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, s));
        }
        q.n_items = n_items;
    } else {
        const uint64_t nc = ctx->c_colors;
        CK(q.h_items.ensure(nq * 16 + 16));
        memcpy(q.h_items.p, h_off, nq * 8);
        memcpy(q.h_items.p + nq * 8, h_len, nq * 8);
        CK(q.d_qoff.ensure(nq + 1));
        CK(q.d_qlen.ensure(nq + 1));
        CK(q.d_counts.ensure(nq * nc + 1));
        CK(q.d_queue.ensure(1));
        CK(q.h_counts.ensure(nq * nc * sizeof(unsigned long long) + 16));
        CK(cudaMemcpyAsync(q.d_qoff.p, q.h_items.p, nq * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(q.d_qlen.p, q.h_items.p + nq * 8, nq * 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(q.d_queue.p, 0, sizeof(unsigned long long), s));
        ctx->launches += launch_query_color(q.d_text.p, k, q.d_qoff.p, q.d_qlen.p, nq, ctx->qkeys.p, ctx->qvals.p,
                                            ctx->qmask, ctx->csub_arena.p, ctx->c_words, ctx->c_colors, q.d_matched.p,
                                            q.d_counts.p, q.d_queue.p, ctx->sms, s);
        CK(cudaMemcpyAsync(q.h_counts.p, q.d_counts.p, nq * nc * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           s));
        q.n_items = nq;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(q.h_out.p, q.d_matched.p, nq * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(q.done, s));
    q.nq = nq;
    q.busy = true;
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_poll(ggcat_gpu_ctx *ctx, int slot) {
    if (!ctx || slot < 0 || slot >= GGCAT_GPU_QUERY_SLOTS) return GGCAT_GPU_EINVAL;
    auto &q = ctx->qslots[slot];
    if (!q.busy) return 1;
    cudaError_t e = cudaEventQuery(q.done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return fail(ctx, GGCAT_GPU_ECUDA, "query poll: %s", cudaGetErrorString(e));
}

extern "C" int ggcat_gpu_query_wait(ggcat_gpu_ctx *ctx, int slot, uint64_t *h_matched, uint64_t cap, uint64_t *nq) {
    if (!ctx || slot < 0 || slot >= GGCAT_GPU_QUERY_SLOTS) return GGCAT_GPU_EINVAL;
    auto &q = ctx->qslots[slot];
    if (!q.busy) return fail(ctx, GGCAT_GPU_EINVAL, "slot %d has no batch", slot);
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventSynchronize(q.done));
    q.busy = false;
    if (nq) *nq = q.nq;
    if (h_matched) memcpy(h_matched, q.h_out.p, std::min<uint64_t>(cap, q.nq) * sizeof(uint64_t));
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_color_counts(ggcat_gpu_ctx *ctx, int slot, uint64_t *h_counts, uint64_t cap,
                                            uint32_t *n_colors) {
    if (!ctx || slot < 0 || slot >= GGCAT_GPU_QUERY_SLOTS) return GGCAT_GPU_EINVAL;
    auto &q = ctx->qslots[slot];
    if (q.busy) return fail(ctx, GGCAT_GPU_EINVAL, "slot %d still running; wait first", slot);
    if (!q.colored) return fail(ctx, GGCAT_GPU_EINVAL, "slot %d ran an uncoloured batch", slot);
    if (n_colors) *n_colors = ctx->c_colors;
    if (h_counts)
        par_memcpy(h_counts, q.h_counts.p,
                   std::min<uint64_t>(cap, q.nq * (uint64_t)ctx->c_colors) * sizeof(uint64_t));
    return GGCAT_GPU_OK;
}

// ---------------------------------------------------------------------------
// file-level query: GGCATInstance::query_graph
// ---------------------------------------------------------------------------

// A coloured graph's FASTA (as build_and_write or the reference writes it: ">{id} LN:i:{len}
// C:{subset:x}:{count}... [L:...]" then the bases, possibly over several lines, plain or
// compressed by its extension): the unitigs in the text layout and, per text position, the
// colour subset of the k-mer starting there.
static int read_colored_graph(const char *path, int k, std::vector<uint8_t> &text, std::vector<uint32_t> &pos_subset,
                              std::string &err) {
    std::vector<uint8_t> raw;
    int rc = ggcat::read_input_file(path, raw, err);
    if (rc) return rc;
    text.clear();
    pos_subset.clear();
    std::vector<std::pair<uint32_t, uint64_t>> runs;
    bool in_rec = false;
    uint64_t rec_start = 0;
    auto close_rec = [&]() -> bool {
        if (!in_rec) return true;
        const uint64_t len = text.size() - rec_start;
        uint64_t nk = len >= (uint64_t)k ? len - (uint64_t)k + 1 : 0, covered = 0;
        pos_subset.resize(text.size() + 1, 0xffffffffu);
        for (const auto &r : runs) {
            for (uint64_t j = 0; j < r.second && covered + j < nk; j++) pos_subset[rec_start + covered + j] = r.first;
            covered += r.second;
        }
        text.push_back('\n');
        in_rec = false;
        return covered == nk;
    };
    const uint8_t *p = raw.data(), *end = raw.data() + raw.size();
    while (p < end) {
        const uint8_t *nl = static_cast<const uint8_t *>(memchr(p, '\n', (size_t)(end - p)));
        const uint8_t *le = nl ? nl : end;
        const uint8_t *lend = (le > p && le[-1] == '\r') ? le - 1 : le;
        if (p < lend && *p == '>') {
            if (!close_rec()) return err = std::string(path) + ": colour runs do not cover a unitig", GGCAT_GPU_EIO;
            runs.clear();
            // tokens " C:{hex}:{count}"
            for (const uint8_t *q = p; q + 3 < lend; q++) {
                if (q[0] == ' ' && q[1] == 'C' && q[2] == ':') {
                    char *e1 = nullptr, *e2 = nullptr;
                    const std::string tok(reinterpret_cast<const char *>(q + 3), (size_t)(lend - q - 3));
                    const unsigned long sub = strtoul(tok.c_str(), &e1, 16);
                    if (!e1 || *e1 != ':') return err = std::string(path) + ": bad C: annotation", GGCAT_GPU_EIO;
                    const unsigned long long cnt = strtoull(e1 + 1, &e2, 10);
                    runs.emplace_back((uint32_t)sub, (uint64_t)cnt);
                }
            }
            rec_start = text.size();
            in_rec = true;
        } else if (in_rec) {
            for (const uint8_t *q = p; q < lend; q++) {
                const uint8_t c = *q & 0xDF;
                text.push_back((c == 'A' || c == 'C' || c == 'G' || c == 'T') ? c : 'N');
            }
        }
        p = nl ? nl + 1 : end;
    }
    if (!close_rec()) return err = std::string(path) + ": colour runs do not cover a unitig", GGCAT_GPU_EIO;
    pos_subset.resize(text.size(), 0xffffffffu);
    return GGCAT_GPU_OK;
}

// The coloured branch of ggcat_dump_unitigs (dumper::dump_unitigs,
// crates/dumper/src/pipeline/dumper_colormap_reading.rs:62-146): every k-mer of the graph once,
// in pieces of one colour subset (maximal runs of equal subsets along a unitig), grouped by
// subset in ascending order; colors = the subset's colours from the colormap, same_colors = 1
// for every piece of a group but the first.
int dump_colored_unitigs(const char *graph_input, int k, ggcat_gpu_dump_fn fn, void *fn_ctx) {
    std::vector<uint8_t> graph;
    std::vector<uint32_t> pos_subset;
    std::string err;
    int rc = read_colored_graph(graph_input, k, graph, pos_subset, err);
    if (rc) return rc;
    cmap::Reader cm;
    rc = cm.open(ggcat_colormap_path(graph_input).c_str(), &err);
    if (rc) return rc;
    struct Piece {
        uint32_t subset;
        uint64_t start, kmers;
    };
    std::vector<Piece> pieces;
    for (uint64_t p = 0; p < pos_subset.size();) {
        if (pos_subset[p] == 0xffffffffu) {
            p++;
            continue;
        }
        uint64_t e = p + 1;
        while (e < pos_subset.size() && pos_subset[e] == pos_subset[p]) e++;
        pieces.push_back(Piece{pos_subset[p], p, e - p});
        p = e;
    }
    std::stable_sort(pieces.begin(), pieces.end(), [](const Piece &a, const Piece &b) { return a.subset < b.subset; });
    std::vector<uint32_t> cols;
    for (size_t i = 0; i < pieces.size(); i++) {
        const bool same = i > 0 && pieces[i - 1].subset == pieces[i].subset;
        if (!same && !cm.get(pieces[i].subset, cols)) return GGCAT_GPU_EIO;
        fn(fn_ctx, graph.data() + pieces[i].start, pieces[i].kmers + (uint64_t)k - 1, cols.data(), cols.size(),
           same ? 1 : 0);
    }
    return GGCAT_GPU_OK;
}

// The query output path: output_file_prefix with `ext` when it has no extension
// (Path::with_extension of an extension-less path, querier/src/lib.rs:190)
static std::string query_output_path(const char *prefix, const char *ext) {
    std::string path = prefix;
    const size_t slash = path.find_last_of('/');
    const size_t dot = path.find_last_of('.');
    const size_t name = slash == std::string::npos ? 0 : slash + 1;
    if (dot == std::string::npos || dot < name || dot == name) path += std::string(".") + ext;
    return path;
}

// Rust's f64 "{:.2}" for the fractions of the query outputs
static void fmt_frac(char *num, size_t cap, double frac) {
    if (std::isnan(frac))
        snprintf(num, cap, "NaN");
    else if (std::isinf(frac))
        snprintf(num, cap, "inf");
    else
        snprintf(num, cap, "%.2f", frac);
}

static int query_graph_impl(ggcat_gpu_ctx *ctx, const char *graph_fasta, const char *query_fasta,
                            const char *output_prefix, int k, int colors, int color_output_format, char *out_path,
                            uint64_t out_cap) {
    CK(cudaSetDevice(ctx->device));
    std::vector<std::string> color_names;
    uint32_t n_colors = 0;
    if (!colors) {
        // graph: the unitigs as text (records cut like the reference's reader, k-1 copyback)
        std::vector<uint8_t> graph;
        std::string err;
        int rc = ggcat::read_sequences(graph_fasta, k - 1, graph, nullptr, nullptr, err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
        CK(ctx->qgraph.ensure(graph.size() + 64));
        if (!graph.empty()) CK(cudaMemcpy(ctx->qgraph.p, graph.data(), graph.size(), cudaMemcpyHostToDevice));
        rc = ggcat_gpu_query_index(ctx, ctx->qgraph.p, graph.size(), k, nullptr);
        if (rc) return rc;
    } else {
        // coloured graph: the k-mers' subsets from the C: runs, the subsets' colours from the
        // colormap beside the graph (colormap_reading.rs:28-183 reads the same two files)
        std::vector<uint8_t> graph;
        std::vector<uint32_t> pos_subset;
        std::string err;
        int rc = read_colored_graph(graph_fasta, k, graph, pos_subset, err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
        cmap::Reader cm;
        const std::string cpath = ggcat_colormap_path(graph_fasta);
        rc = cm.open(cpath.c_str(), &err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
        color_names = cm.names;
        n_colors = (uint32_t)std::max<uint64_t>(cm.colors_count, 1);
        const int words = (int)((n_colors + 31) / 32);
        std::vector<uint32_t> bm(cm.subsets_count * (uint64_t)words, 0), cols;
        for (uint64_t sidx = 0; sidx < cm.subsets_count; sidx++) {
            if (!cm.get((uint32_t)sidx, cols))
                return fail(ctx, GGCAT_GPU_EIO, "%s: bad subset %llu", cpath.c_str(), (unsigned long long)sidx);
            for (uint32_t c : cols) {
                if (c >= n_colors) return fail(ctx, GGCAT_GPU_EIO, "%s: colour %u out of range", cpath.c_str(), c);
                bm[sidx * words + c / 32] |= 1u << (c % 32);
            }
        }
        for (uint32_t v : pos_subset)
            if (v != 0xffffffffu && v >= cm.subsets_count)
                return fail(ctx, GGCAT_GPU_EIO, "%s: subset %u not in the colormap", graph_fasta, v);
        const uint64_t kw = k > 32 ? 2 : 1;
        uint64_t cap = 1024;
        while (cap < 2 * graph.size() + 64) cap <<= 1;
        CK(ctx->qgraph.ensure(graph.size() + 64));
        DevBuf<uint32_t> d_pos;
        CK(d_pos.ensure(graph.size() + 1));
        CK(ctx->qkeys.ensure(cap * kw));
        CK(ctx->qvals.ensure(cap));
        CK(ctx->csub_arena.ensure(bm.size() + 1));
        cudaStream_t s = ctx->cap_stream;
        if (!graph.empty()) {
            CK(cudaMemcpyAsync(ctx->qgraph.p, graph.data(), graph.size(), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(d_pos.p, pos_subset.data(), graph.size() * 4, cudaMemcpyHostToDevice, s));
        }
        if (!bm.empty()) CK(cudaMemcpyAsync(ctx->csub_arena.p, bm.data(), bm.size() * 4, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(ctx->qkeys.p, 0xff, cap * kw * sizeof(uint64_t), s));
        CK(cudaMemsetAsync(ctx->status.p + 1, 0, sizeof(unsigned), s));
        ctx->launches += launch_index_insert(ctx->qgraph.p, graph.size(), k, ctx->qkeys.p, ctx->qvals.p, cap - 1,
                                             ctx->status.p + 1, s, d_pos.p);
        CK(cudaGetLastError());
        unsigned st = 0;
        CK(cudaMemcpyAsync(&st, ctx->status.p + 1, sizeof st, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (st) return fail(ctx, GGCAT_GPU_EDEVICE, "query index: table full");
        ctx->have_colors = false;  // the colour state now describes the loaded graph's subsets
        ctx->c_words = words;
        ctx->c_colors = n_colors;
        ctx->c_n_subsets = cm.subsets_count;
        ctx->qmask = cap - 1;
        ctx->qk = k;
        ctx->qcolored = true;
        ctx->qready = true;
    }
    // queries: one per record the reader emits (FASTA records with bases, every FASTQ
    // record; never cut), submitted in batches of bounded text size
    std::vector<uint8_t> qtext;
    std::vector<uint64_t> qoff, qlen;
    {
        std::string err;
        const int rc = ggcat::read_sequences(query_fasta, -1, qtext, &qoff, &qlen, err);
        if (rc) return fail(ctx, rc, "%s", err.c_str());
    }
    const uint64_t nq = qoff.size();
    std::vector<uint64_t> matched(nq, 0), counts;
    if (colors) counts.assign(nq * (uint64_t)n_colors, 0);
    const uint64_t kBatchBytes = 256ull << 20;
    for (uint64_t a = 0; a < nq;) {
        uint64_t b = a + 1;
        while (b < nq && qoff[b] + qlen[b] - qoff[a] <= kBatchBytes) b++;
        const uint64_t lo = qoff[a], hi = qoff[b - 1] + qlen[b - 1];
        std::vector<uint64_t> o(b - a), l(b - a);
        for (uint64_t i = a; i < b; i++) {
            o[i - a] = qoff[i] - lo;
            l[i - a] = qlen[i];
        }
        int rc = ggcat_gpu_query_submit(ctx, 0, qtext.data() + lo, hi - lo, o.data(), l.data(), b - a);
        if (rc) return rc;
        uint64_t got = 0;
        rc = ggcat_gpu_query_wait(ctx, 0, matched.data() + a, b - a, &got);
        if (rc) return rc;
        if (colors) {
            uint32_t ncol = 0;
            rc = ggcat_gpu_query_color_counts(ctx, 0, counts.data() + a * n_colors, (b - a) * n_colors, &ncol);
            if (rc) return rc;
        }
        a = b;
    }
    const std::string path = query_output_path(output_prefix, colors ? "jsonl" : "csv");
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return fail(ctx, GGCAT_GPU_EIO, "cannot write %s", path.c_str());
    char num[64];
    if (!colors) {
        // the CSV of counters_sorting (crates/querier/src/pipeline/counters_sorting.rs:235-268):
        // query_index, matched_kmers, query_kmers = len - (k - 1), matched / query_kmers to 2 places
        fprintf(f, "query_index,matched_kmers,query_kmers,match_percentage\n");
        for (uint64_t i = 0; i < nq; i++) {
            const uint64_t qk = qlen[i] >= (uint64_t)(k - 1) ? qlen[i] - (uint64_t)(k - 1) : 0;
            fmt_frac(num, sizeof num, (double)matched[i] / (double)qk);
            fprintf(f, "%llu,%llu,%llu,%s\n", (unsigned long long)i, (unsigned long long)matched[i],
                    (unsigned long long)qk, num);
        }
    } else {
        // JSON lines of colored_query_output.rs:264-309: queries with at least one match, in
        // index order; per colour present, the query k-mers found in it over the query's k-mers
        // to 2 places, keyed by the colour index or its JSON-escaped name (the reference escapes
        // '"' first, then '\' -- also the backslash it has just added)
        std::vector<std::string> esc(color_names.size());
        for (size_t c = 0; c < color_names.size(); c++) {
            std::string a;
            for (char ch : color_names[c]) {
                if (ch == '"') a += "\\\"";
                else a += ch;
            }
            std::string b2;
            for (char ch : a) {
                if (ch == '\\') b2 += "\\\\";
                else b2 += ch;
            }
            esc[c] = b2;
        }
        for (uint64_t i = 0; i < nq; i++) {
            const uint64_t *cc = counts.data() + i * n_colors;
            bool any = false;
            for (uint32_t c = 0; c < n_colors && !any; c++) any = cc[c] != 0;
            if (!any) continue;
            const uint64_t qk = qlen[i] >= (uint64_t)(k - 1) ? qlen[i] - (uint64_t)(k - 1) : 0;
            fprintf(f, "{\"query_index\":%llu, \"matches\":{", (unsigned long long)i);
            bool first = true;
            for (uint32_t c = 0; c < n_colors; c++) {
                if (!cc[c]) continue;
                fmt_frac(num, sizeof num, (double)cc[c] / (double)qk);
                if (color_output_format == 1 && c < esc.size())
                    fprintf(f, "%s\"%s\": %s", first ? "" : ",", esc[c].c_str(), num);
                else
                    fprintf(f, "%s\"%u\": %s", first ? "" : ",", c, num);
                first = false;
            }
            fprintf(f, "}}\n");
        }
    }
    const bool werr = ferror(f) != 0;
    if (fclose(f) != 0 || werr) return fail(ctx, GGCAT_GPU_EIO, "error writing %s", path.c_str());
    if (out_path && out_cap) snprintf(out_path, out_cap, "%s", path.c_str());
    return GGCAT_GPU_OK;
}

extern "C" int ggcat_gpu_query_graph(ggcat_gpu_ctx *ctx, const char *input_graph, const char *input_query,
                                     const char *output_file_prefix, size_t kmer_length, size_t threads_count,
                                     int forward_only, size_t minimizer_length, int colors, size_t color_output_format,
                                     char *out_path, uint64_t out_cap) {
    (void)threads_count;     // the files are read on the calling thread; the lookup is on the device
    (void)minimizer_length;  // the device index needs no minimizer bucketing
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (!input_graph || !input_query || !output_file_prefix) return fail(ctx, GGCAT_GPU_EINVAL, "null path");
    if (kmer_length < 3 || kmer_length > 64)
        return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "query supports k <= 64 (k=%zu)", kmer_length);
    if (forward_only) return fail(ctx, GGCAT_GPU_EUNSUPPORTED, "the device query index is canonical (forward_only=1)");
    if (color_output_format > 1)
        return fail(ctx, GGCAT_GPU_EINVAL, "color_output_format %zu is not 0 (numbers) or 1 (names)",
                    color_output_format);
    return query_graph_impl(ctx, input_graph, input_query, output_file_prefix, (int)kmer_length, colors ? 1 : 0,
                            (int)color_output_format, out_path, out_cap);
}

extern "C" int ggcat_gpu_query_from_files(ggcat_gpu_ctx *ctx, const char *graph_fasta, const char *query_fasta,
                                          const char *output_prefix, int k, int forward_only, char *out_path,
                                          uint64_t out_cap) {
    return ggcat_gpu_query_graph(ctx, graph_fasta, query_fasta, output_prefix, (size_t)(k > 0 ? k : 0), 0,
                                 forward_only, (size_t)-1, 0, 0, out_path, out_cap);
}

// ---------------------------------------------------------------------------
// hash families
// ---------------------------------------------------------------------------
extern "C" int ggcat_gpu_kmer_hashes(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t len, int k, int kind,
                                     uint64_t *d_out, void *stream) {
    if (!ctx) return GGCAT_GPU_EINVAL;
    if (kind < 0 || kind > 6) return fail(ctx, GGCAT_GPU_EINVAL, "bad hash kind %d", kind);
    const int kmax = kind <= 1 ? 32 : kind <= 3 ? 64 : kind == 6 ? 64 : 127;
    if (k < 2 || k > kmax) return fail(ctx, GGCAT_GPU_EINVAL, "k=%d outside [2, %d] for hash kind %d", k, kmax, kind);
    if (len && (!d_text || !d_out)) return fail(ctx, GGCAT_GPU_EINVAL, "null buffer");
    CK(cudaSetDevice(ctx->device));
    ctx->launches += launch_kmer_hash(d_text, len, k, kind, d_out, as_stream(stream));
    CK(cudaGetLastError());
    return GGCAT_GPU_OK;
}
