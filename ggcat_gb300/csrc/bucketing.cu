// Minimizer bucketing on sm_103a.
//
// Replaces the CPU hot loop of GGCAT's bucketing (MinimizerBucketingExecWriter::execute,
// crates/minimizer_bucketing/src/lib.rs:296-376, with
// AssemblerMinimizerBucketingExecutor::process_sequence,
// crates/assembler_minimizer_bucketing/src/lib.rs:171-270) and its lz4 temp-file bucket
// store with a device radix partition kept in HBM.
//
// Layout: the ASCII text is packed once into 2-bit codes (32 bases per u64) and a
// validity bitmap (1 bit per base; ACGTacgt are valid).  Each thread then owns a chunk
// of (k-1)-mer window positions and walks its bases sequentially with a rolling nt-hash
// and a block-decomposed window minimum; the superkmers whose split point falls in the
// chunk are appended as 16-byte records to a staging array and counted per sub-bin in
// the same pass, and partition_kernel scatters them by sub-bin after an exclusive scan.
#include "common.cuh"
#include "kernels.h"

namespace ggcat {

// ---------------------------------------------------------------------------
// Pack: ASCII -> 2-bit codes (A0 C1 T2 G3 = (c >> 1) & 3) + validity bits.
// One thread per 32 bases: two 16-byte loads, one 8-byte and one 4-byte store.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) pack_kernel(const uint8_t *__restrict__ text, uint64_t n, uint64_t n_words,
                                                   int aligned16, uint64_t *__restrict__ packed,
                                                   uint32_t *__restrict__ valid) {
    uint64_t wi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; wi < n_words; wi += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t base = wi * 32;
        uint8_t b[32];
        if (aligned16 && base + 32 <= n) {
            uint4 a0 = reinterpret_cast<const uint4 *>(text + base)[0];
            uint4 a1 = reinterpret_cast<const uint4 *>(text + base)[1];
            const uint8_t *p0 = reinterpret_cast<const uint8_t *>(&a0);
            const uint8_t *p1 = reinterpret_cast<const uint8_t *>(&a1);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                b[i] = p0[i];
                b[16 + i] = p1[i];
            }
        } else {
#pragma unroll
            for (int i = 0; i < 32; i++) b[i] = (base + i < n) ? text[base + i] : (uint8_t)'\n';
        }
        uint64_t pw = 0;
        uint32_t vw = 0;
#pragma unroll
        for (int i = 0; i < 32; i++) {
            uint32_t c = b[i];
            uint32_t u = c & 0xDFu;  // upper case
            bool ok = (u == 'A') | (u == 'C') | (u == 'G') | (u == 'T');
            pw |= (uint64_t)((c >> 1) & 3u) << (2 * i);
            vw |= (uint32_t)ok << i;
        }
        packed[wi] = pw;
        valid[wi] = vw;
    }
}

// ---------------------------------------------------------------------------
// Bucketize
//
// Window minimum with the duplicate flag.  Each m-mer contributes v = (min(fw,rc) << 1) | u
// with u = 1 unless the m-mer is rc-symmetric (lib.rs:189-199).  Over a set of m-mers the
// batched queue (batch_minqueue.rs:37-120) reports the masked minimum mv with u = 1 exactly
// when mv occurs once and that occurrence has u = 1; this is the associative combine `cmb`
// below (equal masked minima from two disjoint sets clear u).  Canonical nt-hash values of
// distinct m-mers never collide for the minimizer lengths in use (checked by the oracle's
// tests), so the combine reproduces the queue's values exactly.
//
// The window of w = k-m m-mers ending at m-mer i is split van Herk / Gil-Werman style into
// blocks of w m-mers aligned at i % w == 0: window = suffix(previous block, from i-w+1)
// combined with prefix(current block, up to i).  Every thread's chunk starts at a multiple
// of w, so all lanes of a warp cross block boundaries on the same step and do identical
// work.  The per-thread block array (w entries) lives in shared memory, column-major.
// ---------------------------------------------------------------------------
struct NtTables {
    uint64_t h[4], rch[4], h_rot_m[4], rch_rot_m1[4];
};

struct CState {
    uint64_t v;    // masked minimum | unique bit
    uint64_t pos;  // absolute m-mer position of the minimum (meaningful when unique)
    uint32_t fw;   // is_forward of that m-mer
};

__device__ __forceinline__ CState cmb(CState a, const CState &b) {
    const uint64_t ma = a.v & ~1ull, mb = b.v & ~1ull;
    if (ma < mb) return a;
    if (mb < ma) return b;
    a.v = ma;  // the minimum occurs in both parts: not unique
    return a;
}

// Base of age a (0 = newest) in the 64-base history (r0 newest 32 bases, r1 older 32).
__device__ __forceinline__ uint32_t hist_base(uint64_t r0, uint64_t r1, int a) {
    return a < 32 ? (uint32_t)((r0 >> (2 * a)) & 3u) : (uint32_t)((r1 >> (2 * (a - 32))) & 3u);
}

// nt-hash of the m-mer whose first base has age `a_first` (its last base has age a_first-m+1).
__device__ __forceinline__ void nt_from_scratch(const NtTables &T, uint64_t r0, uint64_t r1, int a_first, int m,
                                                uint64_t &fw, uint64_t &rc) {
    fw = 0;
    rc = 0;
    for (int j = 0; j < m; j++) {
        uint32_t c = hist_base(r0, r1, a_first - j);
        fw ^= rotl64(T.h[c], (unsigned)(m - 1 - j));
        rc ^= rotl64(T.rch[c], (unsigned)j);
    }
}

__device__ __forceinline__ uint64_t nt_value(uint64_t fw, uint64_t rc) {
    uint64_t mn = fw < rc ? fw : rc;
    return (mn << 1) | (uint64_t)(fw != rc);
}

constexpr uint64_t kInf = ~0ull;

// Superkmers found by a lane wait in a per-lane queue in shared memory (column-major, one
// column per thread) and are built, counted and appended together by the whole warp: a split
// happens every ~(w+1)/2 positions per lane, so emitting at once would run the record code on
// almost every step with one or two lanes active.
constexpr int kEmitQueue = 8;   // entries per lane
constexpr int kEmitDrain = 4;   // the warp drains when a lane holds this many

// Single pass: superkmer records are appended to a staging array (warp-aggregated slot
// reservation) and counted per sub-bin; partition_kernel then scatters them by sub-bin.
__global__ void __launch_bounds__(256)
    bucketize_kernel(const uint64_t *__restrict__ packed, const uint32_t *__restrict__ valid, uint64_t n, int k, int m,
                     int bbits, int sbits, int fbits, int canonical, uint64_t chunk,
                     unsigned long long *__restrict__ bin_count, unsigned long long *__restrict__ bin_kmers,
                     SkRec *__restrict__ stage, unsigned long long stage_cap,
                     unsigned long long *__restrict__ stage_cursor, unsigned *__restrict__ status) {
    __shared__ NtTables T;
    extern __shared__ __align__(16) uint8_t bk_smem[];
    const int wn = k - m;
    const int nthr = blockDim.x;
    uint64_t *blk_v = reinterpret_cast<uint64_t *>(bk_smem);                                  // [wn][nthr]
    uint64_t *q_w0 = blk_v + (size_t)wn * nthr;                                              // [kEmitQueue][nthr]
    uint64_t *q_raw = q_w0 + (size_t)kEmitQueue * nthr;                                      // [kEmitQueue][nthr]
    uint32_t *q_meta = reinterpret_cast<uint32_t *>(q_raw + (size_t)kEmitQueue * nthr);      // [kEmitQueue][nthr]
    uint8_t *blk_meta = reinterpret_cast<uint8_t *>(q_meta + (size_t)kEmitQueue * nthr);     // [wn][nthr]
    if (threadIdx.x < 4) {
        uint32_t c = threadIdx.x;
        uint64_t h = (uint64_t)(2 * c + 1) * kNtMult;
        uint64_t r = (uint64_t)(((2 * c) ^ 4) + 1) * kNtMult;
        T.h[c] = h;
        T.rch[c] = r;
        T.h_rot_m[c] = rotl64(h, (unsigned)m);
        T.rch_rot_m1[c] = rotl64(r, (unsigned)(m - 1));
    }
    __syncthreads();

    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;  // chunk is a multiple of wn
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    const uint32_t dup_bucket = 1u << bbits;
    const uint64_t bmask = (1ull << bbits) - 1, smask = (1ull << sbits) - 1, fmask = (1ull << fbits) - 1;
    uint64_t *my_v = blk_v + threadIdx.x;
    uint8_t *my_meta = blk_meta + threadIdx.x;

    uint64_t lb = (uint64_t)wn * 6;
    for (int attempt = 0; attempt < 40; attempt++) {
        const uint64_t xb = x0 > lb ? x0 - lb : 0;  // multiple of wn
        bool anchored = (xb == 0);
        uint64_t run = 0;
        uint64_t r0 = 0, r1 = 0, fw = 0, rc = 0;
        uint64_t prev_raw = 0, prev_pos = 0;
        uint32_t prev_fw = 0;
        bool prev_valid = false;
        uint64_t c_prev = 0;
        bool c_known = false, first_sk = false, failed = false;
        bool have_prev_block = false;
        CState P{kInf, 0, 0};
        int o = 0;  // offset of the current m-mer inside its block

        uint64_t cur_word = ~0ull, pw = 0;
        uint32_t vw = 0;
        const uint64_t p_end = min(x1 + (uint64_t)k - 1, n + 1);

        int qlen = 0;  // superkmers waiting in this lane's queue
        // build, count and append one queued superkmer of every lane that has one, until all
        // queues of the warp are empty; one stage-cursor atomic per round
        auto drain = [&]() {
            const unsigned am = __activemask();
            const int lane = (int)(threadIdx.x & 31);
            for (;;) {
                const unsigned bm = __ballot_sync(am, qlen > 0);
                if (bm == 0) break;
                SkRec r{0, 0};
                if (qlen > 0) {
                    qlen--;
                    const size_t qi = (size_t)qlen * nthr + threadIdx.x;
                    const uint64_t w0 = q_w0[qi], raw = q_raw[qi];
                    const uint32_t meta = q_meta[qi];
                    // superkmer [start, start + len) with the minimizer of value raw at offset
                    // moff (lib.rs:207-267)
                    const uint32_t len = (uint32_t)(w0 >> 40);
                    const uint32_t moff = meta & 0xffffffu, mfw = (meta >> 24) & 1u;
                    const uint32_t inc_first = (meta >> 25) & 1u, inc_last = (meta >> 26) & 1u;
                    uint32_t bucket, rcf, pos;
                    if ((raw & 1ull) == 0) {
                        bucket = dup_bucket;
                        rcf = 0;
                        pos = 0;
                    } else {
                        rcf = (canonical && !mfw) ? 1u : 0u;
                        bucket = (uint32_t)((raw >> 1) & bmask);  // get_bucket(0, b, h), cn_nthash.rs:135-142
                        pos = rcf ? len - (moff + (uint32_t)m) : moff;
                    }
                    const uint32_t second = (uint32_t)((raw >> (bbits + 1)) & smask);
                    const uint32_t sub = (uint32_t)((raw >> (bbits + 1)) & fmask);
                    const uint32_t flags = (inc_first << rcf) | (inc_last << (rcf ^ 1u));
                    const uint64_t bin = ((uint64_t)bucket << fbits) | sub;
                    atomicAdd(&bin_count[bin], 1ull);
                    atomicAdd(&bin_kmers[bin], (unsigned long long)(len - (uint32_t)k + 1));
                    r.w0 = w0;
                    r.w1 = (uint64_t)bucket | ((uint64_t)(second & 0xff) << 16) | ((uint64_t)flags << 24) |
                           ((uint64_t)rcf << 26) | ((uint64_t)(pos & 0xffff) << 32) | ((uint64_t)sub << 48);
                }
                const int leader = __ffs(bm) - 1;
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(stage_cursor, (unsigned long long)__popc(bm));
                base = __shfl_sync(am, base, leader);
                if ((bm >> lane) & 1u) {
                    const unsigned long long idx = base + (unsigned long long)__popc(bm & ((1u << lane) - 1u));
                    if (idx < stage_cap)
                        stage[idx] = r;
                    else
                        atomicOr(status, kStatusStageOverflow);
                }
            }
        };

        auto emit = [&](uint64_t c, bool is_final) {
            // queue the superkmer [c_prev - 1, c + k - 1) with the minimizer of the window
            // before c (split) or of the last window (final)
            const uint64_t start = c_prev - 1, end = c + (uint64_t)k - 1;
            const size_t qi = (size_t)qlen * nthr + threadIdx.x;
            q_w0[qi] = start | ((end - start) << 40);
            q_raw[qi] = prev_raw;
            q_meta[qi] = (uint32_t)((prev_pos - start) & 0xffffffu) | (prev_fw << 24) | ((first_sk ? 1u : 0u) << 25) |
                         ((is_final ? 1u : 0u) << 26);
            qlen++;
            first_sk = false;
        };

        for (uint64_t p = xb; p < p_end; p++) {
            // the warp drains its queues once a lane's queue is half full (loop stays in lockstep)
            if (__any_sync(__activemask(), qlen >= kEmitDrain)) drain();
            const uint64_t wi = p >> 5;
            if (wi != cur_word) {
                cur_word = wi;
                if (p < n) {
                    pw = packed[wi];
                    vw = valid[wi];
                } else {
                    pw = 0;
                    vw = 0;
                }
            }
            const uint32_t sh = (uint32_t)(p & 31);
            const bool ok = (p < n) && ((vw >> sh) & 1u);
            uint64_t e_v = kInf;
            uint32_t e_fw = 0;
            if (ok) {
                const uint32_t c = (uint32_t)((pw >> (2 * sh)) & 3u);
                r1 = (r1 << 2) | (r0 >> 62);
                r0 = (r0 << 2) | c;
                run++;
                if (run == (uint64_t)m) {
                    nt_from_scratch(T, r0, r1, m - 1, m, fw, rc);
                } else if (run > (uint64_t)m) {
                    uint32_t out = hist_base(r0, r1, m);
                    fw = rotl64(fw, 1) ^ T.h_rot_m[out] ^ T.h[c];
                    rc = rotr64(rc ^ T.rch[out], 1) ^ T.rch_rot_m1[c];
                }
                if (run >= (uint64_t)m) {
                    e_v = nt_value(fw, rc);
                    e_fw = (uint32_t)(fw < rc);
                }
            } else {
                if (run >= (uint64_t)k && prev_valid) {
                    const uint64_t x_last = p - (uint64_t)k + 1;
                    if (x_last >= x0 && x_last < x1) {
                        if (!c_known) failed = true;
                        else emit(x_last, true);
                    }
                }
                run = 0;
                anchored = true;
                prev_valid = false;
                c_known = false;
            }
            if (failed) break;
            // block bookkeeping over m-mer positions i = p - m + 1 (aligned: xb % wn == 0)
            if (p + 1 < xb + (uint64_t)m) continue;  // no m-mer position >= xb yet
            const uint64_t i = p + 1 - (uint64_t)m;
            if (o == 0 && i > xb) {
                // the previous block [i - wn, i) is complete: suffix-combine it in place
                CState s{my_v[(size_t)(wn - 1) * nthr], 0, 0};
                {
                    uint8_t mt = my_meta[(size_t)(wn - 1) * nthr];
                    s.pos = (uint64_t)(mt & 0x7f);
                    s.fw = mt >> 7;
                }
                for (int j = wn - 2; j >= 0; j--) {
                    uint8_t mt = my_meta[(size_t)j * nthr];
                    CState c{my_v[(size_t)j * nthr], (uint64_t)(mt & 0x7f), (uint32_t)(mt >> 7)};
                    s = cmb(c, s);
                    my_v[(size_t)j * nthr] = s.v;
                    my_meta[(size_t)j * nthr] = (uint8_t)((s.pos & 0x7f) | (s.fw << 7));
                }
                have_prev_block = true;
            }
            const CState e{e_v, i, e_fw};
            P = (o == 0) ? e : cmb(P, e);
            CState win = P;
            bool win_avail = (o == wn - 1);
            if (!win_avail && have_prev_block) {
                uint8_t mt = my_meta[(size_t)(o + 1) * nthr];
                CState sp{my_v[(size_t)(o + 1) * nthr], i - (uint64_t)o - (uint64_t)wn + (uint64_t)(mt & 0x7f),
                          (uint32_t)(mt >> 7)};
                win = cmb(sp, P);
                win_avail = true;
            }
            my_v[(size_t)o * nthr] = e_v;
            my_meta[(size_t)o * nthr] = (uint8_t)(o | (e_fw << 7));
            o = (o + 1 == wn) ? 0 : o + 1;

            if (!ok || run < (uint64_t)(k - 1) || !win_avail) continue;
            const uint64_t x = p - (uint64_t)k + 2;  // window start
            const uint64_t cur_raw = win.v, cur_pos = win.pos;
            const uint32_t cur_fw = win.fw;
            if (run == (uint64_t)(k - 1)) {
                if (anchored) {
                    c_prev = x + 1;  // virtual first callback: the first superkmer starts at x
                    c_known = true;
                    first_sk = true;
                } else {
                    c_known = false;
                }
            } else {
                // get_minimizer_splits split rule, batch_minqueue.rs:146-152
                const bool split = (cur_raw != prev_raw) || ((cur_raw & 1ull) && cur_pos != prev_pos);
                if (split) {
                    if (x >= x0 && x < x1) {
                        if (!c_known) {
                            failed = true;
                            break;
                        }
                        emit(x, false);
                    }
                    c_prev = x;
                    c_known = true;
                    first_sk = false;
                }
            }
            prev_raw = cur_raw;
            prev_pos = cur_pos;
            prev_fw = cur_fw;
            prev_valid = true;
        }
        drain();
        if (!failed) return;
        if (xb == 0) break;  // cannot look back further
        lb *= 4;
    }
    atomicOr(status, kStatusLookback);
}

// Scatter of the staged records into their sub-bin ranges (the device radix partition).
__global__ void __launch_bounds__(256) partition_kernel(const SkRec *__restrict__ stage, uint64_t n_stage, int fbits,
                                                        const unsigned long long *__restrict__ bin_off,
                                                        unsigned long long *__restrict__ bin_cursor,
                                                        SkRec *__restrict__ recs, unsigned *__restrict__ status) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_stage;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const SkRec r = stage[i];
        const uint64_t bin = ((uint64_t)rec_bucket(r) << fbits) | ((r.w1 >> 48) & 0xffffull);
        const unsigned long long slot = bin_off[bin] + atomicAdd(&bin_cursor[bin], 1ull);
        if (slot >= bin_off[bin + 1]) {
            atomicOr(status, kStatusLookback);
            continue;
        }
        recs[slot] = r;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan over u64 counts (3 phases; n up to a few million)
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;

__device__ unsigned long long block_excl_scan(unsigned long long v, unsigned long long *tmp, unsigned long long &total) {
    // warp scan
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) tmp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned long long s = lane < (int)(blockDim.x >> 5) ? tmp[lane] : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        tmp[lane] = s;
    }
    __syncthreads();
    unsigned long long base = wid > 0 ? tmp[wid - 1] : 0ull;
    total = tmp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void __launch_bounds__(kScanBlock) scan_partials_kernel(const unsigned long long *__restrict__ in, uint64_t n,
                                                                   unsigned long long *__restrict__ block_sums) {
    __shared__ unsigned long long tmp[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanBlock * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if (base + j < n) s += in[base + j];
    unsigned long long total;
    block_excl_scan(s, tmp, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_top_kernel(unsigned long long *__restrict__ block_sums, uint64_t nb,
                                                              unsigned long long *__restrict__ grand_total) {
    __shared__ unsigned long long tmp[32];
    unsigned long long carry = 0;
    for (uint64_t s = 0; s < nb; s += kScanBlock) {
        uint64_t i = s + threadIdx.x;
        unsigned long long v = i < nb ? block_sums[i] : 0ull;
        unsigned long long total;
        unsigned long long ex = block_excl_scan(v, tmp, total);
        if (i < nb) block_sums[i] = ex + carry;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && grand_total) *grand_total = carry;
}

__global__ void __launch_bounds__(kScanBlock) scan_final_kernel(const unsigned long long *__restrict__ in, uint64_t n,
                                                                const unsigned long long *__restrict__ block_sums,
                                                                unsigned long long *__restrict__ out) {
    __shared__ unsigned long long tmp[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanBlock * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long v[kScanItems];
    unsigned long long s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = base + j < n ? in[base + j] : 0ull;
        s += v[j];
    }
    unsigned long long total;
    unsigned long long ex = block_excl_scan(s, tmp, total) + block_sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) out[base + j] = ex;
        ex += v[j];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = ex;  // total at out[n]
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
int launch_pack(const uint8_t *d_text, uint64_t n, uint64_t *packed, uint32_t *valid, cudaStream_t s, int sms) {
    uint64_t n_words = (n + 31) / 32;
    if (n_words == 0) return 0;
    int aligned = ((uintptr_t)d_text % 16) == 0;
    uint64_t blocks = (n_words + 255) / 256;
    uint64_t cap = (uint64_t)sms * 16;
    if (blocks > cap) blocks = cap;
    pack_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_text, n, n_words, aligned, packed, valid);
    return 1;
}

int launch_bucketize(const uint64_t *packed, const uint32_t *valid, uint64_t n, int k, int m, int bbits, int sbits,
                     int fbits, int canonical, uint64_t chunk_hint, unsigned long long *bin_count,
                     unsigned long long *bin_kmers, SkRec *stage, unsigned long long stage_cap,
                     unsigned long long *stage_cursor, unsigned *status, cudaStream_t s) {
    const int wn = k - m;
    const uint64_t chunk = ((chunk_hint + wn - 1) / wn) * wn;
    uint64_t threads = (n + chunk - 1) / chunk;
    if (threads == 0) return 0;
    const int tpb = wn <= 24 ? 256 : 128;
    const size_t smem = (size_t)wn * tpb * 9 + (size_t)kEmitQueue * tpb * 20;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(bucketize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    uint64_t blocks = (threads + tpb - 1) / tpb;
    bucketize_kernel<<<(unsigned)blocks, tpb, smem, s>>>(packed, valid, n, k, m, bbits, sbits, fbits, canonical, chunk,
                                                         bin_count, bin_kmers, stage, stage_cap, stage_cursor, status);
    return 1;
}

int launch_partition(const SkRec *stage, uint64_t n_stage, int fbits, const unsigned long long *bin_off,
                     unsigned long long *bin_cursor, SkRec *recs, unsigned *status, int sms, cudaStream_t s) {
    if (n_stage == 0) return 0;
    uint64_t blocks = (n_stage + 255) / 256;
    const uint64_t cap = (uint64_t)sms * 8;
    if (blocks > cap) blocks = cap;
    partition_kernel<<<(unsigned)blocks, 256, 0, s>>>(stage, n_stage, fbits, bin_off, bin_cursor, recs, status);
    return 1;
}

uint64_t scan_temp_elems(uint64_t n) { return (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems) + 1; }

int launch_exclusive_scan(const unsigned long long *in, uint64_t n, unsigned long long *out,
                          unsigned long long *tmp, cudaStream_t s) {
    if (n == 0) {
        cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
        return 0;
    }
    uint64_t nb = (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
    scan_partials_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(in, n, tmp);
    scan_top_kernel<<<1, kScanBlock, 0, s>>>(tmp, nb, nullptr);
    scan_final_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(in, n, tmp, out);
    return 3;
}

}  // namespace ggcat
