// Device helpers shared by the bucketing, merge and query kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ggcat {

constexpr uint64_t kEmptyKey = ~0ull;  // never a canonical 2-bit k-mer (canonical(G..G) = C..C)

// nt-hash base terms, crates/hashes/src/nthash_base.rs:49-61: h(c) = (2c+1)*M,
// rc(c) = ((2c ^ 4) + 1) * M with the 2-bit code c (A0 C1 T2 G3).
constexpr uint64_t kNtMult = 0x397f178c6ae330f9ull;

__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x << r) | (x >> (64u - r)) : x;
}
__host__ __device__ __forceinline__ uint64_t rotr64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x >> r) | (x << (64u - r)) : x;
}

// splitmix64 finaliser: slot hash of a table key
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// Reverse complement of a 2-bit packed k-mer in seq-hash layout (base i at bits 2i),
// k <= 32.  Complement of a code is code ^ 2.
__device__ __forceinline__ uint64_t rc_packed(uint64_t v, int k) {
    uint64_t x = __brevll(v);                                                     // reverse all bits
    x = ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);  // restore bit order inside pairs
    x ^= 0xAAAAAAAAAAAAAAAAull;                                                   // complement every base
    return x >> (2 * (32 - k));
}

__device__ __forceinline__ uint64_t kmer_mask(int k) { return k >= 32 ? ~0ull : ((1ull << (2 * k)) - 1); }

// Superkmer record of the device bucket store (16 bytes):
//   w0 = start (40 bits) | len << 40 (24 bits)
//   w1 = bucket (16) | second_bucket << 16 (8) | flags << 24 (2) | rc << 26 (1)
//        | minimizer_pos << 32 (16) | sub-bin << 48 (16)
struct __align__(16) SkRec {
    uint64_t w0, w1;
};
__host__ __device__ __forceinline__ uint64_t rec_start(const SkRec &r) { return r.w0 & ((1ull << 40) - 1); }
__host__ __device__ __forceinline__ uint32_t rec_len(const SkRec &r) { return (uint32_t)(r.w0 >> 40); }
__host__ __device__ __forceinline__ uint32_t rec_bucket(const SkRec &r) { return (uint32_t)(r.w1 & 0xffff); }
__host__ __device__ __forceinline__ uint32_t rec_second(const SkRec &r) { return (uint32_t)((r.w1 >> 16) & 0xff); }
__host__ __device__ __forceinline__ uint32_t rec_flags(const SkRec &r) { return (uint32_t)((r.w1 >> 24) & 3); }
__host__ __device__ __forceinline__ uint32_t rec_rc(const SkRec &r) { return (uint32_t)((r.w1 >> 26) & 1); }
__host__ __device__ __forceinline__ uint32_t rec_minpos(const SkRec &r) { return (uint32_t)((r.w1 >> 32) & 0xffff); }

// Sub-bins per bucket = 2^fine_bits (chosen per input, <= kMaxFineBits); the bucket store
// is partitioned by (bucket, sub-bin) and merge units are runs of sub-bins of one bucket.
constexpr int kMaxFineBits = 12;

// Device status word bits (set with atomicOr, read by the host after a sync)
enum : unsigned {
    kStatusOutOverflow = 1u,    // partial-unitig output buffer too small (host retries)
    kStatusKmerOverflow = 2u,   // k-mer dump buffer too small (host retries)
    kStatusTableFull = 4u,      // a hash table probe ran past its capacity (internal error)
    kStatusWalkLimit = 8u,      // a unitig walk exceeded its bound (internal error)
    kStatusLookback = 16u,      // bucketing needed more than the maximum lookback (internal error)
    kStatusStageOverflow = 32u, // staging array of the bucket store too small (host retries)
};

}  // namespace ggcat
