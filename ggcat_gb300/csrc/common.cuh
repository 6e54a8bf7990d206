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

// ---------------------------------------------------------------------------
// k-mer key types of the merge tables: u64 for k <= 32, u128 for 32 < k <= 64.  Both hold the
// canonical 2-bit packed k-mer (base i at bits 2i), i.e. the seq-hash value of the reference
// (crates/hashes/src/base/cn_seqhash_base.rs:22-69, u64 and u128 variants).
// ---------------------------------------------------------------------------
typedef unsigned __int128 u128;

template <typename KT>
struct KeyOps;

template <>
struct KeyOps<uint64_t> {
    static constexpr int kMaxK = 32;
    __device__ static __forceinline__ uint64_t empty() { return ~0ull; }
    // high half of a multiplicative hash; table slots take its top bits
    __device__ static __forceinline__ uint32_t hash(uint64_t x) { return (uint32_t)((x * 0x9E3779B97F4A7C15ull) >> 32); }
    __device__ static __forceinline__ uint64_t rc(uint64_t v, int k) { return rc_packed(v, k); }
    __device__ static __forceinline__ uint64_t mask(int k) { return kmer_mask(k); }
    __device__ static __forceinline__ uint64_t cas(uint64_t *a, uint64_t cmp, uint64_t val) {
        return atomicCAS(reinterpret_cast<unsigned long long *>(a), (unsigned long long)cmp, (unsigned long long)val);
    }
    // k bases starting at base p of the packed text
    __device__ static __forceinline__ uint64_t load(const uint64_t *__restrict__ packed, uint64_t p, int k) {
        const uint64_t w = p >> 5;
        const uint32_t sh = (uint32_t)(p & 31) * 2u;
        uint64_t v = packed[w] >> sh;
        if (sh + 2u * (uint32_t)k > 64u) v |= packed[w + 1] << (64u - sh);
        return v & kmer_mask(k);
    }
    __device__ static __forceinline__ void store(uint64_t *arr, uint64_t i, uint64_t key) { arr[i] = key; }
};

// 128-bit compare-and-swap (PTX atom.cas.b128, sm_90 and later; generic address, so it works on
// shared and global memory); the address is 16-byte aligned
__device__ __forceinline__ u128 cas_u128(u128 *addr, u128 cmp, u128 val) {
    const uint64_t clo = (uint64_t)cmp, chi = (uint64_t)(cmp >> 64), vlo = (uint64_t)val, vhi = (uint64_t)(val >> 64);
    uint64_t olo, ohi;
    asm volatile(
        "{\n\t.reg .b128 d, b, c;\n\t"
        "mov.b128 b, {%2, %3};\n\t"
        "mov.b128 c, {%4, %5};\n\t"
        "atom.cas.b128 d, [%6], b, c;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}\n"
        : "=l"(olo), "=l"(ohi)
        : "l"(clo), "l"(chi), "l"(vlo), "l"(vhi), "l"(addr)
        : "memory");
    return ((u128)ohi << 64) | (u128)olo;
}

template <>
struct KeyOps<u128> {
    static constexpr int kMaxK = 64;
    __device__ static __forceinline__ u128 empty() { return ~(u128)0; }
    __device__ static __forceinline__ uint32_t hash(u128 x) {
        const uint64_t f = (uint64_t)x ^ ((uint64_t)(x >> 64) * 0xC2B2AE3D27D4EB4Full);
        return (uint32_t)((f * 0x9E3779B97F4A7C15ull) >> 32);
    }
    // the 64-base reverse complement is the rc of the two 32-base halves, swapped
    __device__ static __forceinline__ u128 rc(u128 v, int k) {
        const uint64_t rlo = rc_packed((uint64_t)(v >> 64), 32), rhi = rc_packed((uint64_t)v, 32);
        return (((u128)rhi << 64) | (u128)rlo) >> (2 * (64 - k));
    }
    __device__ static __forceinline__ u128 mask(int k) { return k >= 64 ? ~(u128)0 : (((u128)1 << (2 * k)) - 1); }
    __device__ static __forceinline__ u128 cas(u128 *a, u128 cmp, u128 val) { return cas_u128(a, cmp, val); }
    __device__ static __forceinline__ u128 load(const uint64_t *__restrict__ packed, uint64_t p, int k) {
        const uint64_t w = p >> 5;
        const uint32_t sh = (uint32_t)(p & 31) * 2u;
        const uint32_t need = sh + 2u * (uint32_t)k;  // bits used from word w on
        uint64_t lo = packed[w] >> sh, hi = 0;
        if (need > 64u) {
            const uint64_t a1 = packed[w + 1];
            if (sh) lo |= a1 << (64u - sh);
            hi = sh ? a1 >> sh : a1;
            if (need > 128u) hi |= packed[w + 2] << (64u - sh);  // need > 128 implies sh > 0
        }
        return (((u128)hi << 64) | (u128)lo) & mask(k);
    }
    // dumped keys are stored as (lo, hi) word pairs
    __device__ static __forceinline__ void store(uint64_t *arr, uint64_t i, u128 key) {
        arr[2 * i] = (uint64_t)key;
        arr[2 * i + 1] = (uint64_t)(key >> 64);
    }
};

// ---------------------------------------------------------------------------
// k > 64 (the Rabin-Karp families of the reference, crates/api/src/utils.rs:10-69): the
// canonical packed k-mer in four 64-bit words, base i at bit 2i of the 256-bit value (w[0]
// holds bases 0-31), k <= 127.  The top bit of w[3] is never set by a k-mer, which leaves the
// all-ones word for an empty slot and kU256Claim for a slot being written.
// ---------------------------------------------------------------------------
struct __align__(32) u256 {
    uint64_t w[4];
    u256() = default;
    __host__ __device__ constexpr u256(uint64_t x) : w{x, 0, 0, 0} {}
    __host__ __device__ constexpr u256(uint64_t a, uint64_t b, uint64_t c, uint64_t d) : w{a, b, c, d} {}
    __host__ __device__ explicit operator uint64_t() const { return w[0]; }
    __host__ __device__ explicit operator uint32_t() const { return (uint32_t)w[0]; }
};
__host__ __device__ __forceinline__ u256 operator|(const u256 &a, const u256 &b) {
    return u256(a.w[0] | b.w[0], a.w[1] | b.w[1], a.w[2] | b.w[2], a.w[3] | b.w[3]);
}
__host__ __device__ __forceinline__ u256 operator&(const u256 &a, const u256 &b) {
    return u256(a.w[0] & b.w[0], a.w[1] & b.w[1], a.w[2] & b.w[2], a.w[3] & b.w[3]);
}
__host__ __device__ __forceinline__ u256 operator^(const u256 &a, const u256 &b) {
    return u256(a.w[0] ^ b.w[0], a.w[1] ^ b.w[1], a.w[2] ^ b.w[2], a.w[3] ^ b.w[3]);
}
__host__ __device__ __forceinline__ bool operator==(const u256 &a, const u256 &b) {
    return ((a.w[0] ^ b.w[0]) | (a.w[1] ^ b.w[1]) | (a.w[2] ^ b.w[2]) | (a.w[3] ^ b.w[3])) == 0;
}
__host__ __device__ __forceinline__ bool operator!=(const u256 &a, const u256 &b) { return !(a == b); }
__host__ __device__ __forceinline__ bool operator<(const u256 &a, const u256 &b) {
    if (a.w[3] != b.w[3]) return a.w[3] < b.w[3];
    if (a.w[2] != b.w[2]) return a.w[2] < b.w[2];
    if (a.w[1] != b.w[1]) return a.w[1] < b.w[1];
    return a.w[0] < b.w[0];
}
__host__ __device__ __forceinline__ bool operator<=(const u256 &a, const u256 &b) { return !(b < a); }
__host__ __device__ __forceinline__ bool operator>(const u256 &a, const u256 &b) { return b < a; }
// shifts by 0 <= n < 256 bits
__host__ __device__ __forceinline__ u256 operator>>(const u256 &a, int n) {
    const int q = n >> 6, r = n & 63;
    u256 o(0);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int j = i + q;
        uint64_t v = j < 4 ? a.w[j] >> r : 0;
        if (r && j + 1 < 4) v |= a.w[j + 1] << (64 - r);
        o.w[i] = v;
    }
    return o;
}
__host__ __device__ __forceinline__ u256 operator<<(const u256 &a, int n) {
    const int q = n >> 6, r = n & 63;
    u256 o(0);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int j = i - q;
        uint64_t v = j >= 0 ? a.w[j] << r : 0;
        if (r && j - 1 >= 0) v |= a.w[j - 1] >> (64 - r);
        o.w[i] = v;
    }
    return o;
}

__host__ __device__ __forceinline__ u256 &operator|=(u256 &a, const u256 &b) { return a = a | b; }
__host__ __device__ __forceinline__ u256 &operator&=(u256 &a, const u256 &b) { return a = a & b; }
__host__ __device__ __forceinline__ u256 &operator>>=(u256 &a, int n) { return a = a >> n; }
__host__ __device__ __forceinline__ u256 &operator<<=(u256 &a, int n) { return a = a << n; }

constexpr uint64_t kU256Claim = 0xfffffffffffffffeull;  // w[3] of a slot whose key is being written

__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

template <>
struct KeyOps<u256> {
    static constexpr int kMaxK = 127;
    __device__ static __forceinline__ u256 empty() { return u256(~0ull, ~0ull, ~0ull, ~0ull); }
    __device__ static __forceinline__ uint32_t hash(const u256 &x) {
        const uint64_t f = mix64(x.w[0] ^ mix64(x.w[1] ^ mix64(x.w[2] ^ mix64(x.w[3]))));
        return (uint32_t)(f >> 32);
    }
    // the 128-base reverse complement is the rc of the four 32-base words in reverse order
    __device__ static __forceinline__ u256 rc(const u256 &v, int k) {
        const u256 r(rc_packed(v.w[3], 32), rc_packed(v.w[2], 32), rc_packed(v.w[1], 32), rc_packed(v.w[0], 32));
        return r >> (2 * (128 - k));
    }
    __device__ static __forceinline__ u256 mask(int k) {
        u256 m(0);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int bits = 2 * k - 64 * i;
            m.w[i] = bits >= 64 ? ~0ull : bits > 0 ? ((1ull << bits) - 1) : 0ull;
        }
        return m;
    }
    // k bases starting at base p of the packed text (up to five words)
    __device__ static __forceinline__ u256 load(const uint64_t *__restrict__ packed, uint64_t p, int k) {
        const uint64_t w = p >> 5;
        const uint32_t sh = (uint32_t)(p & 31) * 2u;
        const uint32_t need = sh + 2u * (uint32_t)k;  // bits used from word w on
        u256 o(0);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (64u * (uint32_t)i >= need) break;
            uint64_t v = packed[w + i] >> sh;
            if (sh && 64u * (uint32_t)(i + 1) < need) v |= packed[w + i + 1] << (64u - sh);
            o.w[i] = v;
        }
        return o & mask(k);
    }
    __device__ static __forceinline__ void store(uint64_t *arr, uint64_t i, const u256 &key) {
#pragma unroll
        for (int j = 0; j < 4; j++) arr[4 * i + j] = key.w[j];
    }
};

// Find-or-insert of `key` at one slot of an open-addressing key array: 1 when the slot holds
// key (*created when this call wrote it), 0 when it holds another key, -1 when a bounded wait
// for another thread's write gave up.  Keys of one or two words are claimed by one
// compare-and-swap.
template <typename KT>
__device__ __forceinline__ int slot_claim(KT *slot, const KT &key, bool &created) {
    const KT kk = *slot;
    if (kk == key) return 1;
    if (kk == KeyOps<KT>::empty()) {
        const KT old = KeyOps<KT>::cas(slot, KeyOps<KT>::empty(), key);
        if (old == KeyOps<KT>::empty()) {
            created = true;
            return 1;
        }
        if (old == key) return 1;
    }
    return 0;
}
// Four-word keys: the writer claims the slot by a compare-and-swap of w[3] from empty to
// kU256Claim, stores w[0..2], and releases w[3] = key.w[3] after a fence; readers acquire w[3]
// and wait (bounded) while it reads kU256Claim.
template <>
__device__ __forceinline__ int slot_claim<u256>(u256 *slot, const u256 &key, bool &created) {
    uint64_t w3 = ld_acquire_u64(&slot->w[3]);
    for (int spin = 0;; spin++) {
        if (w3 == ~0ull) {
            const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long *>(&slot->w[3]), ~0ull,
                                                      (unsigned long long)kU256Claim);
            if (prev == ~0ull) {
                volatile uint64_t *vw = slot->w;
                vw[0] = key.w[0];
                vw[1] = key.w[1];
                vw[2] = key.w[2];
                __threadfence();
                atomicExch(reinterpret_cast<unsigned long long *>(&slot->w[3]), (unsigned long long)key.w[3]);
                created = true;
                return 1;
            }
            w3 = prev;
        }
        if (w3 != kU256Claim) break;
        if (spin >= (1 << 20)) return -1;
        __nanosleep(32);
        w3 = ld_acquire_u64(&slot->w[3]);
    }
    if (w3 != key.w[3]) return 0;
    const volatile uint64_t *vw = slot->w;
    return (vw[0] == key.w[0] && vw[1] == key.w[1] && vw[2] == key.w[2]) ? 1 : 0;
}

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
    kStatusWaitLimit = 64u,     // a bounded wait for another thread's table slot gave up (internal error)
};

}  // namespace ggcat
