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
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace ggcat {

// ---------------------------------------------------------------------------
// Pack: ASCII -> 2-bit codes (A0 C1 T2 G3 = (c >> 1) & 3) + validity bits.
// One thread per 32 bases: two 16-byte loads, one 8-byte and one 4-byte store; the bytes are
// processed four at a time inside 32-bit words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack4_codes(uint32_t w) {
    // byte i's code (bits 1-2 of the ASCII letter) moves to bits 2i..2i+1
    const uint32_t x = (w >> 1) & 0x03030303u;
    return (x | (x >> 6) | (x >> 12) | (x >> 18)) & 0xFFu;
}
__device__ __forceinline__ uint32_t pack4_valid(uint32_t w) {
    // one bit per byte: ACGT in either case (upper-cased by clearing bit 5)
    const uint32_t u = w & 0xDFDFDFDFu;
    const uint32_t m = __vcmpeq4(u, 0x41414141u) | __vcmpeq4(u, 0x43434343u) | __vcmpeq4(u, 0x47474747u) |
                       __vcmpeq4(u, 0x54545454u);
    const uint32_t y = m & 0x01010101u;
    return (y | (y >> 7) | (y >> 14) | (y >> 21)) & 0xFu;
}

__global__ void __launch_bounds__(256) pack_kernel(const uint8_t *__restrict__ text, uint64_t n, uint64_t n_words,
                                                   int aligned16, uint64_t *__restrict__ packed,
                                                   uint32_t *__restrict__ valid) {
    uint64_t wi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; wi < n_words; wi += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t base = wi * 32;
        uint32_t w[8];
        if (aligned16 && base + 32 <= n) {
            const uint4 a0 = reinterpret_cast<const uint4 *>(text + base)[0];
            const uint4 a1 = reinterpret_cast<const uint4 *>(text + base)[1];
            w[0] = a0.x, w[1] = a0.y, w[2] = a0.z, w[3] = a0.w;
            w[4] = a1.x, w[5] = a1.y, w[6] = a1.z, w[7] = a1.w;
        } else {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                uint32_t x = 0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const uint64_t p = base + 4 * j + i;
                    x |= (uint32_t)(p < n ? text[p] : (uint8_t)'\n') << (8 * i);
                }
                w[j] = x;
            }
        }
        uint64_t pw = 0;
        uint32_t vw = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            pw |= (uint64_t)pack4_codes(w[j]) << (8 * j);
            vw |= pack4_valid(w[j]) << (4 * j);
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
// blocks of w m-mers counted from the thread's first base: window = suffix(previous block,
// from i-w+1) combined with prefix(current block, up to i).  M-mers are indexed by their
// last base, counted from the walk's first base; a window is only used when its k-1 bases
// are valid, which puts it in the second block or later and makes all its m-mers valid.
// All lanes of a warp start the same number of bases before a multiple of 32, so they load
// packed words and cross block boundaries on the same steps.  The per-thread block array (w
// entries: value, and a byte with the offset of the suffix minimum and its orientation) lives
// in shared memory, column-major.
//
// The nt-hash rolls over every code, valid or not, starting from the state of an all-'A'
// history: the rolling update is exact for any code sequence, so m steps after a separator
// or an N the value is the m-mer's hash again without a recomputation; validity is tracked
// by the run length.  One 16-byte table entry per (leaving code, entering code) pair holds
// both XOR terms of the roll.
// ---------------------------------------------------------------------------
// Roll terms (cn_nthash.rs:19-58) of the pair (out, in): f = rotl(h(out), m) ^ h(in),
// r = rotr(rch(out), 1) ^ rotl(rch(in), m - 1); fw' = rotl(fw, 1) ^ f, rc' = rotr(rc, 1) ^ r.
struct __align__(16) NtRoll {
    uint64_t f, r;
};

// Window-minimum state: v = masked minimum | unique bit, pf = (last base of the m-mer) << 1 |
// is_forward
struct CState {
    uint64_t v;
    uint32_t pf;
};

__device__ __forceinline__ CState cmb(const CState &a, const CState &b) {
    const uint64_t ma = a.v & ~1ull, mb = b.v & ~1ull;
    const bool lt = mb < ma, eq = ma == mb;
    CState r;
    r.v = lt ? b.v : (eq ? ma : a.v);  // equal minima from two parts: not unique
    r.pf = lt ? b.pf : a.pf;
    return r;
}

// Superkmers found by a lane wait in a per-lane queue in shared memory (column-major, one
// column per thread) and are built, counted and stored together by the whole warp: a split
// happens every ~(w+1)/2 positions per lane, so emitting at once would run the record code on
// almost every step with one or two lanes active.  The queues are checked every kCheck steps
// (a lane gains at most kCheck entries in between) and drained while some lane holds
// kEmitDrain or more, one entry of every non-empty lane per round.
constexpr int kEmitQueue = 6;
constexpr int kCheck = 2;
constexpr int kEmitDrain = kEmitQueue - kCheck;

// Per-sub-bin counts: one 64-bit atomic per superkmer, records in the high half and k-mer
// instances in the low half (packed).  A count that does not fit its half carries into the
// other one or out of the word; the host detects that from the record total and runs again
// with separate counters (split).
struct BinCounters {
    unsigned long long *packed;  // packed mode: records << 32 | k-mers
    unsigned long long *kmers;   // split mode: k-mers (records in `packed`)
    unsigned long long *total;   // records of all CTAs
    int split;
};

// Single pass over the 2-bit text.  Thread t owns the window starts [t*chunk, (t+1)*chunk)
// (chunk a multiple of 32) and walks the bases from lb (a multiple of 32) before its range,
// one packed word (32 bases) per outer iteration.  Superkmer records go to the block's
// region of the staging array (block-shared cursor), or to the overflow area when the region
// is full; partition_kernel scatters them by sub-bin after an exclusive scan of the
// per-sub-bin counts.
template <int kTPB, bool kLongM>  // kLongM: m > 16, the last m codes need a 64-bit shift register
__global__ void __launch_bounds__(kTPB, kTPB == 256 ? 3 : 6)
    bucketize_kernel(const uint64_t *__restrict__ packed, const uint32_t *__restrict__ valid, uint64_t n, int k,
                     int m, int bbits, int sbits, int fbits, int canonical, uint32_t chunk, uint32_t lb0,
                     BinCounters bc, SkRec *__restrict__ stage, uint32_t region_cap,
                     unsigned long long *__restrict__ block_count, unsigned long long ovf_cap,
                     unsigned long long *__restrict__ ovf_cursor, unsigned *__restrict__ status, uint32_t block_base,
                     uint32_t stage_block0, uint32_t stage_blocks) {
    __shared__ NtRoll tab[16];
    __shared__ unsigned s_cnt;
    extern __shared__ __align__(16) uint8_t bk_smem[];
    const uint32_t wn = (uint32_t)(k - m);
    uint64_t *blk_v = reinterpret_cast<uint64_t *>(bk_smem);                       // [wn][kTPB]
    uint4 *que = reinterpret_cast<uint4 *>(blk_v + (size_t)wn * kTPB);             // [kEmitQueue][kTPB]
    uint8_t *blk_m = reinterpret_cast<uint8_t *>(que + (size_t)kEmitQueue * kTPB); // [wn][kTPB]
    if (threadIdx.x < 16) {
        const uint32_t out = threadIdx.x >> 2, in = threadIdx.x & 3;
        const uint64_t ho = (uint64_t)(2 * out + 1) * kNtMult, ro = (uint64_t)(((2 * out) ^ 4) + 1) * kNtMult;
        const uint64_t hi = (uint64_t)(2 * in + 1) * kNtMult, ri = (uint64_t)(((2 * in) ^ 4) + 1) * kNtMult;
        tab[threadIdx.x] = NtRoll{rotl64(ho, (unsigned)m) ^ hi, rotr64(ro, 1) ^ rotl64(ri, (unsigned)(m - 1))};
    }
    if (threadIdx.x == 0) s_cnt = 0;
    // rolling state of an all-'A' history (code 0): nt-hash of m A's
    uint64_t fw_a = 0, rc_a = 0;
    {
        const uint64_t h0 = kNtMult, r0 = 5ull * kNtMult;
        for (int j = 0; j < m; j++) {
            fw_a ^= rotl64(h0, (unsigned)(m - 1 - j));
            rc_a ^= rotl64(r0, (unsigned)j);
        }
    }
    __syncthreads();

    const uint32_t dup_bucket = 1u << bbits;
    const uint32_t bmask = (1u << bbits) - 1, smask = (1u << sbits) - 1, fmask = (1u << fbits) - 1;
    const uint64_t n_words = (n + 31) >> 5;
    const int lane = (int)(threadIdx.x & 31);
    // this launch covers blocks [block_base, block_base + gridDim.x); the staging array holds the
    // regions of blocks [stage_block0, stage_block0 + stage_blocks), then the overflow area
    const uint64_t bid = (uint64_t)blockIdx.x + block_base;
    const uint64_t region = (bid - stage_block0) * region_cap;
    uint64_t *my_v = blk_v + threadIdx.x;
    uint8_t *my_m = blk_m + threadIdx.x;
    uint4 *my_q = que + threadIdx.x;
    const uint32_t top_sh = 2u * (uint32_t)(m - 1);
    const uint32_t km1 = (uint32_t)(k - 1);

    const uint64_t tid = bid * kTPB + threadIdx.x;
    const uint64_t x0 = tid * chunk;
    int qlen = 0;     // superkmers waiting in this lane's queue
    uint64_t xb = 0;  // first base of the current attempt (queue positions are relative to it)

    // Builds, counts and stores one queued superkmer of every lane that has one, in rounds,
    // while some lane holds at least `keep` entries (keep = 1: until all queues are empty).
    auto drain = [&](int keep) {
        const unsigned am = __activemask();
        for (;;) {
            if (!__any_sync(am, qlen >= keep)) break;
            const unsigned bm = __ballot_sync(am, qlen > 0);
            SkRec rec{0, 0};
            if (qlen > 0) {
                qlen--;
                const uint4 e = my_q[(size_t)qlen * kTPB];
                // superkmer [start, end) whose last window's minimum (value raw, last base of
                // the m-mer and is_forward in pf) is the minimizer (lib.rs:207-267)
                const uint32_t start_r = e.x, end_r = e.y & 0x3fffffffu;
                const uint32_t inc_first = (e.y >> 30) & 1u, inc_last = e.y >> 31;
                const uint32_t len = end_r - start_r;
                const uint32_t moff = (e.z >> 1) + 1u - (uint32_t)m - start_r, mfw = e.z & 1u;
                const uint32_t raw = e.w;
                uint32_t bucket, rcf, pos;
                if ((raw & 1u) == 0) {
                    bucket = dup_bucket;
                    rcf = 0;
                    pos = 0;
                } else {
                    rcf = (canonical && !mfw) ? 1u : 0u;
                    bucket = (raw >> 1) & bmask;  // get_bucket(0, b, h), cn_nthash.rs:135-142
                    pos = rcf ? len - (moff + (uint32_t)m) : moff;
                }
                const uint32_t second = (raw >> (bbits + 1)) & smask;
                const uint32_t sub = (raw >> (bbits + 1)) & fmask;
                const uint32_t flags = (inc_first << rcf) | (inc_last << (rcf ^ 1u));
                const uint64_t bin = ((uint64_t)bucket << fbits) | sub;
                const unsigned long long nk = (unsigned long long)(len - (uint32_t)k + 1);
                if (bc.split) {
                    atomicAdd(&bc.packed[bin], 1ull);
                    atomicAdd(&bc.kmers[bin], nk);
                } else {
                    atomicAdd(&bc.packed[bin], (1ull << 32) + nk);
                }
                rec.w0 = (xb + start_r) | ((uint64_t)len << 40);
                rec.w1 = (uint64_t)bucket | ((uint64_t)(second & 0xff) << 16) | ((uint64_t)flags << 24) |
                         ((uint64_t)rcf << 26) | ((uint64_t)(pos & 0xffff) << 32) | ((uint64_t)sub << 48);
            }
            const int leader = __ffs(bm) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(&s_cnt, (unsigned)__popc(bm));
            base = __shfl_sync(am, base, leader);
            if ((bm >> lane) & 1u) {
                const unsigned idx = base + (unsigned)__popc(bm & ((1u << lane) - 1u));
                if (idx < region_cap) {
                    stage[region + idx] = rec;
                } else {
                    const unsigned long long oi = atomicAdd(ovf_cursor, 1ull);
                    if (oi < ovf_cap)
                        stage[(uint64_t)stage_blocks * region_cap + oi] = rec;
                    else
                        atomicOr(status, kStatusStageOverflow);
                }
            }
        }
    };

    if (x0 < n) {
        const uint64_t x1 = min(x0 + chunk, n);
        uint64_t lb = lb0;
        bool done = false;
        // (relative positions stay below 2^30: queue entries keep two flags above them)
        for (int attempt = 0; attempt < 24 && !done && lb <= (1ull << 28); attempt++) {
            xb = x0 > lb ? x0 - lb : 0;  // a multiple of 32
            const uint32_t lo_r = (uint32_t)(x0 - xb);
            uint32_t hi_r = (uint32_t)(x1 - xb);
            const uint32_t r_end = (uint32_t)(min(x1 + (uint64_t)k - 1, n + 1) - xb);
            bool anchored = (xb == 0), c_known = false, first_sk = false, failed = false;
            uint32_t run = 0, c_prev = 0;
            uint64_t fw = fw_a, rc = rc_a;
            uint64_t hist = 0;  // codes of the last m bases, oldest in the low bits
            CState P{~0ull, 0}, prev{0, 0};
            uint32_t o = 0;  // offset of the current m-mer inside its block
            for (uint32_t j = 0; j < wn; j++) {
                my_v[(size_t)j * kTPB] = ~0ull;
                my_m[(size_t)j * kTPB] = 0;
            }

            // one base: c its 2-bit code, ok its validity, r its offset from xb
            auto step = [&](uint32_t c, bool ok, uint32_t r) {
                if (!ok) {
                    // end of a run: the last superkmer closes at its last window (x_last)
                    if (run >= (uint32_t)k) {
                        const uint32_t x_last = r - (uint32_t)k + 1;
                        if (x_last >= lo_r && x_last < hi_r) {
                            if (!c_known) {
                                failed = true;
                                hi_r = 0;  // no further records in this attempt
                            } else {
                                my_q[(size_t)qlen * kTPB] =
                                    make_uint4(c_prev - 1, (x_last + (uint32_t)k - 1) | ((first_sk ? 1u : 0u) << 30) |
                                                               (1u << 31),
                                               prev.pf, (uint32_t)prev.v);
                                qlen++;
                                first_sk = false;
                            }
                        }
                    }
                    anchored = true;
                    c_known = false;
                }
                run = ok ? run + 1 : 0u;
                // rolling nt-hash of the m-mer ending here (every code rolls, valid or not)
                uint32_t out;
                if constexpr (kLongM) {
                    out = (uint32_t)hist & 3u;
                    hist = (hist >> 2) | ((uint64_t)c << top_sh);
                } else {
                    out = (uint32_t)hist & 3u;
                    hist = (uint64_t)(((uint32_t)hist >> 2) | (c << top_sh));
                }
                const NtRoll t = tab[(out << 2) | c];
                fw = rotl64(fw, 1) ^ t.f;
                rc = rotr64(rc, 1) ^ t.r;
                const bool isf = fw < rc;
                const uint64_t mn = isf ? fw : rc;
                // (an m-mer over a non-ACGT byte gets a meaningless value: the windows that are
                // used hold valid m-mers only, and the van Herk parts of a window cover exactly
                // its m-mers, so such values never reach a used window)
                const CState e{(mn << 1) | (uint64_t)(fw != rc), (r << 1) | (isf ? 1u : 0u)};
                // van Herk block window minimum
                if (o == 0) {  // the previous block is complete: suffix minima in place (offset 0 unused)
                    CState sfx{my_v[(size_t)(wn - 1) * kTPB], my_m[(size_t)(wn - 1) * kTPB]};
                    for (uint32_t j = wn - 2; j >= 1; j--) {
                        const CState cj{my_v[(size_t)j * kTPB], my_m[(size_t)j * kTPB]};
                        sfx = cmb(cj, sfx);
                        my_v[(size_t)j * kTPB] = sfx.v;
                        my_m[(size_t)j * kTPB] = (uint8_t)sfx.pf;
                    }
                    P = e;
                } else {
                    P = cmb(P, e);
                }
                CState win = P;
                if (o + 1 < wn) {  // suffix of the previous block from offset o + 1
                    const uint8_t mt = my_m[(size_t)(o + 1) * kTPB];
                    const uint32_t ps = r - o - wn + (uint32_t)(mt & 0x7f);
                    win = cmb(CState{my_v[(size_t)(o + 1) * kTPB], (ps << 1) | (uint32_t)(mt >> 7)}, P);
                }
                my_v[(size_t)o * kTPB] = e.v;
                my_m[(size_t)o * kTPB] = (uint8_t)(o | ((e.pf & 1u) << 7));
                o = (o + 1 == wn) ? 0 : o + 1;

                // Superkmer bookkeeping as predicated assignments (some lane of a warp splits on
                // almost every step, so a divergent branch would run nearly always):
                //   a run starts (first valid window): with an anchor, a virtual first callback
                //     (the first superkmer starts at x); otherwise the start is not known yet;
                //   a split (get_minimizer_splits split rule, batch_minqueue.rs:146-152) closes
                //     the current superkmer at the window before x.
                const bool wv = ok && run >= km1;  // the (k-1)-mer ending here is a valid window
                const uint32_t x = r - (uint32_t)k + 2;
                const bool first = wv && run == km1;
                const bool split = wv && !first && ((win.v != prev.v) || ((win.v & 1ull) && win.pf != prev.pf));
                const bool inr = split && x >= lo_r && x < hi_r;
                if (inr && c_known) {
                    my_q[(size_t)qlen * kTPB] = make_uint4(
                        c_prev - 1, (x + (uint32_t)k - 1) | ((first_sk ? 1u : 0u) << 30), prev.pf, (uint32_t)prev.v);
                    qlen++;
                }
                if (inr && !c_known) {
                    failed = true;
                    hi_r = 0;
                }
                c_prev = first ? x + 1 : (split ? x : c_prev);
                first_sk = first ? anchored : (first_sk && !split);
                c_known = first ? anchored : (c_known || split);
                if (wv) prev = win;
            };

            uint64_t wi = xb >> 5;
            uint64_t pw_next = wi < n_words ? packed[wi] : 0ull;
            uint32_t vw_next = wi < n_words ? valid[wi] : 0u;
            for (uint32_t r0 = 0; r0 < r_end && !failed; r0 += 32) {  // the same words on every lane
                uint64_t pw = pw_next;
                uint32_t vw = vw_next;
                wi++;
                pw_next = wi < n_words ? packed[wi] : 0ull;
                vw_next = wi < n_words ? valid[wi] : 0u;
#pragma unroll 1
                for (uint32_t j = 0; j < 32; j += kCheck) {
                    // a lane gains at most kCheck queue entries between two checks
                    if (__any_sync(__activemask(), qlen >= kEmitDrain)) drain(kEmitDrain);
#pragma unroll
                    for (uint32_t t = 0; t < (uint32_t)kCheck; t++) {
                        step((uint32_t)pw & 3u, (vw & 1u) != 0, r0 + j + t);
                        pw >>= 2;
                        vw >>= 1;
                    }
                }
            }
            drain(1);
            if (!failed) {
                done = true;
            } else {
                if (xb == 0) break;  // cannot look back further
                lb *= 4;
            }
        }
        if (!done) atomicOr(status, kStatusLookback);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        block_count[bid - stage_block0] = min(s_cnt, region_cap);
        atomicAdd(bc.total, (unsigned long long)s_cnt);
    }
}

// Scatter of the staged records into their sub-bin ranges (the device radix partition).
// CTA b < n_regions reads the first block_count[b] records of staging region b; the CTAs
// after them read slices of kOvfSlice records of the overflow area.
constexpr uint32_t kOvfSlice = 8192;

__global__ void __launch_bounds__(256) partition_kernel(const SkRec *__restrict__ stage, uint32_t n_regions,
                                                        uint32_t region_cap,
                                                        const unsigned long long *__restrict__ block_count,
                                                        const unsigned long long *__restrict__ ovf_cursor,
                                                        unsigned long long ovf_cap, int fbits,
                                                        const unsigned long long *__restrict__ bin_off,
                                                        unsigned *__restrict__ bin_cursor,
                                                        SkRec *__restrict__ recs, unsigned *__restrict__ status) {
    uint64_t begin, end;
    if (blockIdx.x < n_regions) {
        begin = (uint64_t)blockIdx.x * region_cap;
        end = begin + min((unsigned long long)region_cap, block_count[blockIdx.x]);
    } else {
        const uint64_t used = min(*ovf_cursor, ovf_cap);
        const uint64_t s0 = (uint64_t)(blockIdx.x - n_regions) * kOvfSlice;
        if (s0 >= used) return;
        begin = (uint64_t)n_regions * region_cap + s0;
        end = (uint64_t)n_regions * region_cap + min(used, s0 + kOvfSlice);
    }
    // four records per thread in flight: their cursor atomics and offset loads are independent,
    // so one round trip to L2 serves four scatters
    constexpr int kIlp = 4;
    for (uint64_t i0 = begin + threadIdx.x; i0 < end; i0 += kIlp * blockDim.x) {
        SkRec r[kIlp];
        uint64_t bin[kIlp];
        unsigned long long slot[kIlp], lim[kIlp];
#pragma unroll
        for (int q = 0; q < kIlp; q++) {
            const uint64_t i = i0 + (uint64_t)q * blockDim.x;
            if (i < end) r[q] = stage[i];
        }
#pragma unroll
        for (int q = 0; q < kIlp; q++) {
            if (i0 + (uint64_t)q * blockDim.x >= end) continue;
            bin[q] = ((uint64_t)rec_bucket(r[q]) << fbits) | ((r[q].w1 >> 48) & 0xffffull);
            slot[q] = atomicAdd(&bin_cursor[bin[q]], 1u);
            lim[q] = bin_off[bin[q] + 1];
            slot[q] += bin_off[bin[q]];
        }
#pragma unroll
        for (int q = 0; q < kIlp; q++) {
            if (i0 + (uint64_t)q * blockDim.x >= end) continue;
            if (slot[q] >= lim[q]) {
                atomicOr(status, kStatusLookback);
                continue;
            }
            recs[slot[q]] = r[q];
        }
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

// field of a scanned word: the whole word, or one half of a packed (high << 32 | low) count
__device__ __forceinline__ unsigned long long scan_field(unsigned long long x, int field) {
    return field == 0 ? x : (field == 1 ? (x >> 32) : (x & 0xffffffffull));
}

__global__ void __launch_bounds__(kScanBlock) scan_partials_kernel(const unsigned long long *__restrict__ in, uint64_t n,
                                                                   int field, unsigned long long *__restrict__ block_sums) {
    __shared__ unsigned long long tmp[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanBlock * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if (base + j < n) s += scan_field(in[base + j], field);
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
                                                                int field,
                                                                const unsigned long long *__restrict__ block_sums,
                                                                unsigned long long *__restrict__ out) {
    __shared__ unsigned long long tmp[32];
    uint64_t base = (uint64_t)blockIdx.x * kScanBlock * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    unsigned long long v[kScanItems];
    unsigned long long s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = base + j < n ? scan_field(in[base + j], field) : 0ull;
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

cudaError_t bucketize_configure() {
    cudaError_t e = cudaFuncSetAttribute(bucketize_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(bucketize_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(bucketize_kernel<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(bucketize_kernel<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    return e;
}

BucketizeGeometry bucketize_geometry(uint64_t n, int k, int m) {
    BucketizeGeometry g{};
    const int wn = k - m;
    g.threads_per_block = wn <= 24 ? 256 : 128;
    g.chunk = wn <= 24 ? 1024u : 2048u;
    g.lookback = (uint32_t)(((2 * wn + 8) + 31) / 32 * 32);
    const uint64_t threads = (n + g.chunk - 1) / g.chunk;
    g.blocks = (uint32_t)((threads + g.threads_per_block - 1) / g.threads_per_block);
    // 1.5x the expected superkmer density 2/(w+1) of random sequence; excess goes to the
    // overflow area
    g.region_cap = (uint32_t)((uint64_t)g.threads_per_block * g.chunk * 3 / (uint64_t)(wn + 1) + 64);
    g.smem = (size_t)wn * g.threads_per_block * 9 + (size_t)kEmitQueue * g.threads_per_block * 16;
    return g;
}

int launch_bucketize(const uint64_t *packed, const uint32_t *valid, uint64_t n, int k, int m, int bbits, int sbits,
                     int fbits, int canonical, const BucketizeGeometry &g, unsigned long long *bin_counts,
                     unsigned long long *bin_kmers, int split_counts, unsigned long long *total_recs, SkRec *stage,
                     unsigned long long *block_count, unsigned long long ovf_cap, unsigned long long *ovf_cursor,
                     unsigned *status, uint32_t block_base, uint32_t n_blocks, cudaStream_t s, uint32_t stage_block0,
                     uint32_t stage_blocks) {
    if (block_base >= g.blocks) return 0;
    if (stage_blocks == 0) stage_blocks = g.blocks;
    n_blocks = std::min(n_blocks, g.blocks - block_base);
    if (n_blocks == 0) return 0;
    const BinCounters bc{bin_counts, bin_kmers, total_recs, split_counts};
#define GGCAT_BUCKETIZE_LAUNCH(TPB, LONGM)                                                                        \
    bucketize_kernel<TPB, LONGM><<<n_blocks, TPB, g.smem, s>>>(packed, valid, n, k, m, bbits, sbits, fbits,       \
                                                              canonical, g.chunk, g.lookback, bc, stage,          \
                                                              g.region_cap, block_count, ovf_cap, ovf_cursor,     \
                                                              status, block_base, stage_block0, stage_blocks)
    if (g.threads_per_block == 256) {
        if (m > 16)
            GGCAT_BUCKETIZE_LAUNCH(256, true);
        else
            GGCAT_BUCKETIZE_LAUNCH(256, false);
    } else {
        if (m > 16)
            GGCAT_BUCKETIZE_LAUNCH(128, true);
        else
            GGCAT_BUCKETIZE_LAUNCH(128, false);
    }
#undef GGCAT_BUCKETIZE_LAUNCH
    return 1;
}

int launch_partition(const SkRec *stage, const BucketizeGeometry &g, const unsigned long long *block_count,
                     const unsigned long long *ovf_cursor, unsigned long long ovf_cap, int fbits,
                     const unsigned long long *bin_off, unsigned *bin_cursor, SkRec *recs, unsigned *status,
                     cudaStream_t s, uint32_t stage_blocks) {
    if (stage_blocks == 0) stage_blocks = g.blocks;
    const uint64_t grid = (uint64_t)stage_blocks + (ovf_cap + kOvfSlice - 1) / kOvfSlice;
    if (grid == 0) return 0;
    partition_kernel<<<(unsigned)grid, 256, 0, s>>>(stage, stage_blocks, g.region_cap, block_count, ovf_cursor,
                                                    ovf_cap, fbits, bin_off, bin_cursor, recs, status);
    return 1;
}

uint64_t scan_temp_elems(uint64_t n) { return (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems) + 1; }

int launch_exclusive_scan(const unsigned long long *in, uint64_t n, unsigned long long *out,
                          unsigned long long *tmp, cudaStream_t s, int field) {
    if (n == 0) {
        cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
        return 0;
    }
    uint64_t nb = (n + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
    scan_partials_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(in, n, field, tmp);
    scan_top_kernel<<<1, kScanBlock, 0, s>>>(tmp, nb, nullptr);
    scan_final_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(in, n, field, tmp, out);
    return 3;
}

}  // namespace ggcat
