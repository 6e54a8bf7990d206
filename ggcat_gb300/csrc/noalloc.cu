// Bucket-size histogram that allocates no device memory.
//
// Some callers cannot allocate device memory at all: a host pipeline whose device memory is
// owned by another allocator (a framework's caching pool), code running inside a region
// where allocation is forbidden, or a caller that only wants to size its own bucket store
// before committing memory.  For them this file provides one entry point that takes device
// input and output pointers and uses, as its only scratch, the file-scope static array
// below.  It has no counterpart in the reference.
//
// The kernel is a variant of the bucketize count pass: it reads the ASCII text directly
// (instead of the 2-bit copy the main path allocates), and accumulates per-bucket superkmer
// and k-mer counts into the static scratch; a second kernel writes the caller's count arrays
// and the exclusive prefix sums of the superkmer counts.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ggcat_gb300.h"
#include "common.cuh"

namespace ggcat {
namespace noalloc {

// Largest supported first-level bucket count: 2^13 normal buckets + the duplicates bucket
// (the reference's MAX_BUCKETS_COUNT_LOG = 13, crates/config/src/lib.rs:73).
constexpr int kMaxBucketBits = 13;
constexpr uint32_t kMaxBuckets = (1u << kMaxBucketBits) + 1;

// Scratch: [0, kMaxBuckets) superkmers per bucket, [kMaxBuckets, 2*kMaxBuckets) k-mers per
// bucket.  131 KB, held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned long long g_scratch[2 * kMaxBuckets];

struct NtT {
    uint64_t h[4], rch[4], h_rot_m[4], rch_rot_m1[4];
};
struct CSt {
    uint64_t v, pos;
    uint32_t fw;
};
__device__ __forceinline__ CSt cmb2(CSt a, const CSt &b) {
    const uint64_t ma = a.v & ~1ull, mb = b.v & ~1ull;
    if (ma < mb) return a;
    if (mb < ma) return b;
    a.v = ma;
    return a;
}
__device__ __forceinline__ uint32_t hbase(uint64_t r0, uint64_t r1, int a) {
    return a < 32 ? (uint32_t)((r0 >> (2 * a)) & 3u) : (uint32_t)((r1 >> (2 * (a - 32))) & 3u);
}
__device__ __forceinline__ bool text_base(const uint8_t *text, uint64_t n, uint64_t p, uint32_t &code) {
    if (p >= n) return false;
    const uint32_t c = text[p];
    const uint32_t u = c & 0xDFu;
    code = (c >> 1) & 3u;
    return (u == 'A') | (u == 'C') | (u == 'G') | (u == 'T');
}

__global__ void clear_kernel(unsigned long long *scratch, uint32_t nb) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
        scratch[i] = 0;
        scratch[kMaxBuckets + i] = 0;
    }
}

// Per thread: window positions [x0, x1), chunk a multiple of w = k - m.  Accounting without
// superkmer starts: a superkmer spanning W windows has W - 1 k-mers, so per bucket
//   k-mers = (own windows) + (splits that start a superkmer there) - (pieces ending there),
// and one superkmer per split or piece end (the callbacks of get_minimizer_splits).
__global__ void __launch_bounds__(256) histogram_kernel(const uint8_t *__restrict__ text, uint64_t n, int k, int m,
                                                        int bbits, uint64_t chunk, unsigned long long *scratch) {
    __shared__ NtT T;
    extern __shared__ __align__(16) uint8_t na_smem[];
    const int wn = k - m;
    const int nthr = blockDim.x;
    uint64_t *blk_v = reinterpret_cast<uint64_t *>(na_smem);
    uint8_t *blk_meta = reinterpret_cast<uint8_t *>(blk_v + (size_t)wn * nthr);
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
    const uint64_t x0 = tid * chunk;
    if (x0 >= n) return;
    const uint64_t x1 = min(x0 + chunk, n);
    const uint32_t dup_bucket = 1u << bbits;
    const uint64_t bmask = (1ull << bbits) - 1;
    unsigned long long *cnt = scratch, *kms = scratch + kMaxBuckets;
    uint64_t *my_v = blk_v + threadIdx.x;
    uint8_t *my_meta = blk_meta + threadIdx.x;
    auto bucket_of = [&](uint64_t raw) -> uint32_t {
        return (raw & 1ull) ? (uint32_t)((raw >> 1) & bmask) : dup_bucket;
    };

    const uint64_t xb = x0 >= (uint64_t)wn ? x0 - (uint64_t)wn : 0;
    uint32_t code;
    // a run that already covers base xb - 1 is not starting inside this chunk's view
    bool continued = xb > 0 && text_base(text, n, xb - 1, code);
    uint64_t run = 0, r0 = 0, r1 = 0, fw = 0, rc = 0;
    uint64_t prev_raw = 0, prev_pos = 0;
    bool prev_valid = false, pending_first = false;
    bool have_prev_block = false;
    CSt P{~0ull, 0, 0};
    int o = 0;
    const uint64_t p_end = min(x1 + (uint64_t)k - 1, n + 1);
    for (uint64_t p = xb; p < p_end; p++) {
        const bool ok = text_base(text, n, p, code);
        uint64_t e_v = ~0ull;
        uint32_t e_fw = 0;
        if (ok) {
            r1 = (r1 << 2) | (r0 >> 62);
            r0 = (r0 << 2) | code;
            run++;
            if (run == (uint64_t)m) {
                fw = 0;
                rc = 0;
                for (int j = 0; j < m; j++) {
                    uint32_t c = hbase(r0, r1, m - 1 - j);
                    fw ^= rotl64(T.h[c], (unsigned)(m - 1 - j));
                    rc ^= rotl64(T.rch[c], (unsigned)j);
                }
            } else if (run > (uint64_t)m) {
                uint32_t out = hbase(r0, r1, m);
                fw = rotl64(fw, 1) ^ T.h_rot_m[out] ^ T.h[code];
                rc = rotr64(rc ^ T.rch[out], 1) ^ T.rch_rot_m1[code];
            }
            if (run >= (uint64_t)m) {
                uint64_t mn = fw < rc ? fw : rc;
                e_v = (mn << 1) | (uint64_t)(fw != rc);
                e_fw = (uint32_t)(fw < rc);
            }
        } else {
            // the piece ended: its last window is x_last (a piece has >= 2 windows when its
            // length is >= k; shorter pieces are dropped and contributed nothing)
            if (prev_valid && (run >= (uint64_t)k || continued)) {
                const uint64_t x_last = p - (uint64_t)k + 1;
                if (x_last >= x0 && x_last < x1) {
                    const uint32_t b = bucket_of(prev_raw);
                    atomicAdd(&cnt[b], 1ull);
                    atomicAdd(&kms[b], ~0ull);  // -1
                }
            }
            run = 0;
            continued = false;
            prev_valid = false;
            pending_first = false;
        }
        if (p + 1 < xb + (uint64_t)m) continue;
        const uint64_t i = p + 1 - (uint64_t)m;
        if (o == 0 && i > xb) {
            uint8_t mt = my_meta[(size_t)(wn - 1) * nthr];
            CSt s{my_v[(size_t)(wn - 1) * nthr], (uint64_t)(mt & 0x7f), (uint32_t)(mt >> 7)};
            for (int j = wn - 2; j >= 0; j--) {
                uint8_t mj = my_meta[(size_t)j * nthr];
                CSt c{my_v[(size_t)j * nthr], (uint64_t)(mj & 0x7f), (uint32_t)(mj >> 7)};
                s = cmb2(c, s);
                my_v[(size_t)j * nthr] = s.v;
                my_meta[(size_t)j * nthr] = (uint8_t)((s.pos & 0x7f) | (s.fw << 7));
            }
            have_prev_block = true;
        }
        const CSt e{e_v, i, e_fw};
        P = (o == 0) ? e : cmb2(P, e);
        CSt win = P;
        bool win_avail = (o == wn - 1);
        if (!win_avail && have_prev_block) {
            uint8_t mt = my_meta[(size_t)(o + 1) * nthr];
            CSt sp{my_v[(size_t)(o + 1) * nthr], i - (uint64_t)o - (uint64_t)wn + (uint64_t)(mt & 0x7f),
                   (uint32_t)(mt >> 7)};
            win = cmb2(sp, P);
            win_avail = true;
        }
        my_v[(size_t)o * nthr] = e_v;
        my_meta[(size_t)o * nthr] = (uint8_t)(o | (e_fw << 7));
        o = (o + 1 == wn) ? 0 : o + 1;

        if (!ok || run < (uint64_t)(k - 1) || !win_avail) continue;
        const uint64_t x = p - (uint64_t)k + 2;
        const uint64_t cur_raw = win.v, cur_pos = win.pos;
        const bool owned = x >= x0 && x < x1;
        if (run == (uint64_t)(k - 1) && !continued) {
            // first window of a piece: counted once the piece is known to have >= k bases
            pending_first = owned;
        } else {
            if (pending_first) {
                // the previous window (first of its piece) is owned and the piece is kept
                atomicAdd(&kms[bucket_of(prev_raw)], 1ull);
                pending_first = false;
            } else if (run == (uint64_t)(k - 1)) {
                // unreachable: a continued run never has a first window here
            }
            if (owned) atomicAdd(&kms[bucket_of(cur_raw)], 1ull);
            const bool split = (cur_raw != prev_raw) || ((cur_raw & 1ull) && cur_pos != prev_pos);
            if (split && owned) {
                atomicAdd(&cnt[bucket_of(prev_raw)], 1ull);  // the superkmer ending here
                atomicAdd(&kms[bucket_of(cur_raw)], 1ull);   // the next one starts with an extra window
            }
        }
        prev_raw = cur_raw;
        prev_pos = cur_pos;
        prev_valid = true;
    }
}

__global__ void __launch_bounds__(1024) finalize_kernel(const unsigned long long *scratch, uint32_t nb,
                                                        uint64_t *out_superkmers, uint64_t *out_kmers,
                                                        uint64_t *out_offsets) {
    __shared__ unsigned long long warp_tot[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nb; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const unsigned long long v = i < nb ? scratch[i] : 0ull;
        if (i < nb) {
            out_superkmers[i] = v;
            out_kmers[i] = scratch[kMaxBuckets + i];
        }
        unsigned long long x = v;
        for (int d = 1; d < 32; d <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            unsigned long long t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0ull;
            for (int d = 1; d < 32; d <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const unsigned long long before = (wid > 0 ? warp_tot[wid - 1] : 0ull) + carry;
        if (i < nb) out_offsets[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) out_offsets[nb] = carry;
}

// Device address of g_scratch per device, looked up once with that device current.
static std::mutex g_mu;
static unsigned long long *g_addr[256];

}  // namespace noalloc
}  // namespace ggcat

using namespace ggcat;

extern "C" int ggcat_gpu_bucket_histogram_noalloc(const uint8_t *d_text, uint64_t text_len, int32_t k, int32_t m,
                                                  int32_t bucket_bits, uint64_t *d_superkmers, uint64_t *d_kmers,
                                                  uint64_t *d_offsets, void *stream) {
    if (m < 2 || m > 32 || k - m < 2 || k > 64 || bucket_bits < 1) return GGCAT_GPU_EINVAL;
    if (bucket_bits > noalloc::kMaxBucketBits) return GGCAT_GPU_ETOOLARGE;
    if (text_len >= (1ull << 40)) return GGCAT_GPU_ETOOLARGE;
    if (!d_superkmers || !d_kmers || !d_offsets || (text_len && !d_text)) return GGCAT_GPU_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return GGCAT_GPU_ECUDA;
    unsigned long long *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(noalloc::g_mu);
        if (!noalloc::g_addr[dev]) {
            void *ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, noalloc::g_scratch) != cudaSuccess || !ptr) return GGCAT_GPU_ECUDA;
            noalloc::g_addr[dev] = static_cast<unsigned long long *>(ptr);
        }
        scratch = noalloc::g_addr[dev];
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // an error left by earlier work is not this call's: report it without clearing it
    if (cudaPeekAtLastError() != cudaSuccess) return GGCAT_GPU_ECUDA;
    const uint32_t nb = (1u << bucket_bits) + 1;
    const int wn = k - m;
    noalloc::clear_kernel<<<(nb + 255) / 256, 256, 0, s>>>(scratch, nb);
    if (cudaGetLastError() != cudaSuccess) return GGCAT_GPU_ECUDA;
    if (text_len > 0) {
        const uint64_t chunk = ((512 + wn - 1) / wn) * wn;
        const uint64_t threads = (text_len + chunk - 1) / chunk;
        const int tpb = wn <= 24 ? 256 : 128;
        const size_t smem = (size_t)wn * tpb * 9;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(noalloc::histogram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
            return GGCAT_GPU_ECUDA;
        noalloc::histogram_kernel<<<(unsigned)((threads + tpb - 1) / tpb), tpb, smem, s>>>(d_text, text_len, k, m,
                                                                                         bucket_bits, chunk, scratch);
        if (cudaGetLastError() != cudaSuccess) return GGCAT_GPU_ECUDA;
    }
    noalloc::finalize_kernel<<<1, 1024, 0, s>>>(scratch, nb, d_superkmers, d_kmers, d_offsets);
    return cudaGetLastError() == cudaSuccess ? GGCAT_GPU_OK : GGCAT_GPU_ECUDA;
}
