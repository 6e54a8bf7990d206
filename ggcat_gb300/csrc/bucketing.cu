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
// blocks of w m-mers counted from the thread's first m-mer: window = suffix(previous block,
// from i-w+1) combined with prefix(current block, up to i).  All lanes of a warp start the
// same number of bases before a multiple of 32, so they cross block and packed-word
// boundaries on the same steps and do identical work.  The per-thread block array (w
// entries) lives in shared memory, column-major.
//
// The nt-hash rolls over every code, valid or not, starting from the state of an all-'A'
// history: the rolling update is exact for any code sequence, so m steps after a separator
// or an N the value is the m-mer's hash again without a recomputation; validity is tracked
// by the run length.
// ---------------------------------------------------------------------------
// Rolling nt-hash tables per 2-bit code (cn_nthash.rs:19-58): the leaving base contributes
// {rotl(h, m), rch} and the entering base {h, rotl(rch, m - 1)}.
struct __align__(16) NtPair {
    uint64_t a, b;
};

// Window-minimum state: v = masked minimum | unique bit, pf = position << 1 | is_forward
struct CState {
    uint64_t v;
    uint32_t pf;
};

__device__ __forceinline__ CState cmb(const CState &a, const CState &b) {
    const uint64_t ma = a.v & ~1ull, mb = b.v & ~1ull;
    CState r;
    r.v = ma < mb ? a.v : (mb < ma ? b.v : ma);  // equal minima from two parts: not unique
    r.pf = mb < ma ? b.pf : a.pf;
    return r;
}

constexpr uint64_t kInf = ~0ull;

// Superkmers found by a lane wait in a per-lane queue in shared memory (column-major, one
// column per thread) and are built, counted and stored together by the whole warp: a split
// happens every ~(w+1)/2 positions per lane, so emitting at once would run the record code on
// almost every step with one or two lanes active.  A lane gains at most one entry per step
// and the warp drains as soon as a lane holds kEmitDrain, so kEmitQueue entries suffice; six
// entries keep three 256-thread CTAs per SM (k - m = 21) and halve the drain rounds of four.
constexpr int kEmitQueue = 6;
constexpr int kEmitDrain = 5;

// Single pass over the 2-bit text.  Thread t owns the window starts [t*chunk, (t+1)*chunk)
// (chunk a multiple of 32) and walks the bases from lb (a multiple of 32) before its range,
// so all lanes of a warp load packed words and cross van Herk block boundaries on the same
// steps.  Superkmer records go to the block's region of the staging array (block-shared
// cursor), or to the overflow area when the region is full; partition_kernel scatters them
// by sub-bin after an exclusive scan of the per-sub-bin counts.
template <bool kLongM>  // m > 16: the last m codes need a 64-bit shift register
__global__ void __launch_bounds__(256, 3)
    bucketize_kernel(const uint64_t *__restrict__ packed, const uint32_t *__restrict__ valid, uint64_t n, int k,
                     int m, int bbits, int sbits, int fbits, int canonical, uint32_t chunk, uint32_t lb0,
                     unsigned long long *__restrict__ bin_count, unsigned long long *__restrict__ bin_kmers,
                     SkRec *__restrict__ stage, uint32_t region_cap, unsigned long long *__restrict__ block_count,
                     unsigned long long ovf_cap, unsigned long long *__restrict__ ovf_cursor,
                     unsigned *__restrict__ status, uint32_t block_base, uint32_t total_blocks) {
    __shared__ NtPair t_out[4], t_in[4];
    __shared__ unsigned s_cnt;
    extern __shared__ __align__(16) uint8_t bk_smem[];
    const int wn = k - m;
    const int nthr = blockDim.x;
    uint64_t *blk_v = reinterpret_cast<uint64_t *>(bk_smem);                          // [wn][nthr]
    uint4 *que = reinterpret_cast<uint4 *>(blk_v + (size_t)wn * nthr);                // [kEmitQueue][nthr]
    uint8_t *blk_m = reinterpret_cast<uint8_t *>(que + (size_t)kEmitQueue * nthr);    // [wn][nthr]
    if (threadIdx.x < 4) {
        const uint32_t c = threadIdx.x;
        const uint64_t h = (uint64_t)(2 * c + 1) * kNtMult;
        const uint64_t r = (uint64_t)(((2 * c) ^ 4) + 1) * kNtMult;
        t_out[c] = NtPair{rotl64(h, (unsigned)m), r};
        t_in[c] = NtPair{h, rotl64(r, (unsigned)(m - 1))};
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
    // this launch covers blocks [block_base, block_base + gridDim.x) of total_blocks
    const uint64_t bid = (uint64_t)blockIdx.x + block_base;
    const uint64_t region = bid * region_cap;
    uint64_t *my_v = blk_v + threadIdx.x;
    uint8_t *my_m = blk_m + threadIdx.x;
    uint4 *my_q = que + threadIdx.x;
    const uint32_t top_sh = 2u * (uint32_t)(m - 1);

    const uint64_t tid = bid * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;
    int qlen = 0;     // superkmers waiting in this lane's queue
    uint64_t xb = 0;  // first base of the current attempt (queue positions are relative to it)

    // build, count and store one queued superkmer of every lane that has one, until all
    // queues of the active lanes are empty
    auto drain = [&]() {
        const unsigned am = __activemask();
        for (;;) {
            const unsigned bm = __ballot_sync(am, qlen > 0);
            if (bm == 0) break;
            SkRec rec{0, 0};
            if (qlen > 0) {
                qlen--;
                const uint4 e = my_q[(size_t)qlen * nthr];
                // superkmer [start, end) whose last window's minimum (value raw, m-mer
                // position pos, is_forward mfw) is the minimizer (lib.rs:207-267)
                const uint32_t start_r = e.x, end_r = e.y & 0x3fffffffu;
                const uint32_t inc_first = (e.y >> 30) & 1u, inc_last = e.y >> 31;
                const uint32_t len = end_r - start_r;
                const uint32_t moff = (e.z >> 1) - start_r, mfw = e.z & 1u;
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
                atomicAdd(&bin_count[bin], 1ull);
                atomicAdd(&bin_kmers[bin], (unsigned long long)(len - (uint32_t)k + 1));
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
                        stage[(uint64_t)total_blocks * region_cap + oi] = rec;
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
            const uint32_t lo_r = (uint32_t)(x0 - xb), hi_r = (uint32_t)(x1 - xb);
            const uint32_t r_end = (uint32_t)(min(x1 + (uint64_t)k - 1, n + 1) - xb);
            bool anchored = (xb == 0);
            uint32_t run = 0;
            uint64_t fw = fw_a, rc = rc_a;
            uint64_t hist = 0;  // codes of the last m bases, oldest in the low bits
            CState P{kInf, 0}, prev{0, 0};
            bool prev_valid = false, c_known = false, first_sk = false, failed = false, have_prev_block = false;
            uint32_t c_prev = 0;
            int o = 0;  // offset of the current m-mer inside its block

            uint64_t wi = xb >> 5;
            uint64_t pw = 0, pw_next = wi < n_words ? packed[wi] : 0ull;
            uint32_t vw = 0, vw_next = wi < n_words ? valid[wi] : 0u;

            auto push = [&](uint32_t start_r, uint32_t end_r, uint32_t fin) {
                my_q[(size_t)qlen * nthr] = make_uint4(start_r, end_r | ((first_sk ? 1u : 0u) << 30) | (fin << 31),
                                                       prev.pf, (uint32_t)prev.v);
                qlen++;
                first_sk = false;
            };

            for (uint32_t r = 0; r < r_end; r++) {
                // the warp drains its queues once a lane's queue reaches kEmitDrain
                if (__any_sync(__activemask(), qlen >= kEmitDrain)) drain();
                if ((r & 31u) == 0) {  // the same step on every lane
                    pw = pw_next;
                    vw = vw_next;
                    wi++;
                    pw_next = wi < n_words ? packed[wi] : 0ull;
                    vw_next = wi < n_words ? valid[wi] : 0u;
                }
                const uint32_t c = (uint32_t)pw & 3u;
                pw >>= 2;
                const bool ok = (vw & 1u) != 0;
                vw >>= 1;
                if (!ok) {
                    // end of a run: the last superkmer closes at its last window (x_last)
                    if (run >= (uint32_t)k && prev_valid) {
                        const uint32_t x_last = r - (uint32_t)k + 1;
                        if (x_last >= lo_r && x_last < hi_r) {
                            if (!c_known) {
                                failed = true;
                                break;
                            }
                            push(c_prev - 1, x_last + (uint32_t)k - 1, 1u);
                        }
                    }
                    anchored = true;
                    prev_valid = false;
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
                const NtPair to = t_out[out], ti = t_in[c];
                fw = rotl64(fw, 1) ^ to.a ^ ti.a;
                rc = rotr64(rc ^ to.b, 1) ^ ti.b;
                if (r + 1 < (uint32_t)m) continue;  // no m-mer yet (the same steps on every lane)
                const bool mv = run >= (uint32_t)m;
                const bool isf = fw < rc;
                const uint64_t mn = isf ? fw : rc;
                const CState e{mv ? ((mn << 1) | (uint64_t)(fw != rc)) : kInf,
                               ((r + 1 - (uint32_t)m) << 1) | (isf ? 1u : 0u)};
                // van Herk block window minimum over m-mer indices relative to xb
                uint64_t *vo = my_v + (size_t)o * nthr;
                uint8_t *mo = my_m + (size_t)o * nthr;
                if (o == 0) {
                    if (r + 1 > (uint32_t)m) {
                        // the previous block is complete: suffix minima in place (offset 0 unused)
                        CState s{my_v[(size_t)(wn - 1) * nthr], my_m[(size_t)(wn - 1) * nthr]};
                        for (int j = wn - 2; j >= 1; j--) {
                            const CState cj{my_v[(size_t)j * nthr], my_m[(size_t)j * nthr]};
                            s = cmb(cj, s);
                            my_v[(size_t)j * nthr] = s.v;
                            my_m[(size_t)j * nthr] = (uint8_t)s.pf;
                        }
                        have_prev_block = true;
                    }
                    P = e;
                } else {
                    P = cmb(P, e);
                }
                CState win = P;
                bool win_avail = (o == wn - 1);
                if (!win_avail && have_prev_block) {
                    const uint8_t mt = mo[nthr];
                    // suffix of the previous block from offset o + 1: position = block start + offset
                    const uint32_t ps = (r + 1 - (uint32_t)m) - (uint32_t)o - (uint32_t)wn + (uint32_t)(mt & 0x7f);
                    win = cmb(CState{vo[nthr], (ps << 1) | (uint32_t)(mt >> 7)}, P);
                    win_avail = true;
                }
                *vo = e.v;
                *mo = (uint8_t)((uint32_t)o | ((e.pf & 1u) << 7));
                o = (o + 1 == wn) ? 0 : o + 1;

                if (!ok || run < (uint32_t)(k - 1) || !win_avail) continue;
                const uint32_t x = r - (uint32_t)k + 2;  // window start
                if (run == (uint32_t)(k - 1)) {
                    if (anchored) {
                        c_prev = x + 1;  // virtual first callback: the first superkmer starts at x
                        c_known = true;
                        first_sk = true;
                    } else {
                        c_known = false;
                    }
                } else {
                    // get_minimizer_splits split rule, batch_minqueue.rs:146-152
                    const bool split = (win.v != prev.v) || ((win.v & 1ull) && win.pf != prev.pf);
                    if (split) {
                        if (x >= lo_r && x < hi_r) {
                            if (!c_known) {
                                failed = true;
                                break;
                            }
                            push(c_prev - 1, x + (uint32_t)k - 1, 0u);
                        }
                        c_prev = x;
                        c_known = true;
                        first_sk = false;
                    }
                }
                prev = win;
                prev_valid = true;
            }
            drain();
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
    if (threadIdx.x == 0) block_count[bid] = min(s_cnt, region_cap);
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
    for (uint64_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const SkRec r = stage[i];
        const uint64_t bin = ((uint64_t)rec_bucket(r) << fbits) | ((r.w1 >> 48) & 0xffffull);
        const unsigned long long slot = bin_off[bin] + atomicAdd(&bin_cursor[bin], 1u);
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

cudaError_t bucketize_configure() {
    cudaError_t e = cudaFuncSetAttribute(bucketize_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(bucketize_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
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
                     int fbits, int canonical, const BucketizeGeometry &g, unsigned long long *bin_count,
                     unsigned long long *bin_kmers, SkRec *stage, unsigned long long *block_count,
                     unsigned long long ovf_cap, unsigned long long *ovf_cursor, unsigned *status, uint32_t block_base,
                     uint32_t n_blocks, cudaStream_t s) {
    if (block_base >= g.blocks) return 0;
    n_blocks = std::min(n_blocks, g.blocks - block_base);
    if (n_blocks == 0) return 0;
    if (m > 16)
        bucketize_kernel<true><<<n_blocks, g.threads_per_block, g.smem, s>>>(
            packed, valid, n, k, m, bbits, sbits, fbits, canonical, g.chunk, g.lookback, bin_count, bin_kmers, stage,
            g.region_cap, block_count, ovf_cap, ovf_cursor, status, block_base, g.blocks);
    else
        bucketize_kernel<false><<<n_blocks, g.threads_per_block, g.smem, s>>>(
            packed, valid, n, k, m, bbits, sbits, fbits, canonical, g.chunk, g.lookback, bin_count, bin_kmers, stage,
            g.region_cap, block_count, ovf_cap, ovf_cursor, status, block_base, g.blocks);
    return 1;
}

int launch_partition(const SkRec *stage, const BucketizeGeometry &g, const unsigned long long *block_count,
                     const unsigned long long *ovf_cursor, unsigned long long ovf_cap, int fbits,
                     const unsigned long long *bin_off, unsigned *bin_cursor, SkRec *recs, unsigned *status,
                     cudaStream_t s) {
    const uint64_t grid = (uint64_t)g.blocks + (ovf_cap + kOvfSlice - 1) / kOvfSlice;
    if (grid == 0) return 0;
    partition_kernel<<<(unsigned)grid, 256, 0, s>>>(stage, g.blocks, g.region_cap, block_count, ovf_cursor, ovf_cap,
                                                    fbits, bin_off, bin_cursor, recs, status);
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
