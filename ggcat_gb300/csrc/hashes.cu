// Rolling k-mer / m-mer hashes of GGCAT on sm_103a, as a standalone device pass.
//
// Restates the hash families of crates/hashes on the device, one thread per run of
// positions, each thread rolling its window exactly like the reference iterators:
//   seq-hash u64/u128 (base/cn_seqhash_base.rs:23-69, base/fw_seqhash_base.rs:18-59),
//   Rabin-Karp u128 (base/cn_rkhash_base.rs:62-109, base/fw_rkhash_base.rs:40-69; rmmult =
//   MULTIPLIER^(k-1), lib.rs:169-191), and the canonical nt-hash of m-mers
//   (cn_nthash.rs:21-58, value (min(fw,rc) << 1) | unique flag).
// The merge keys its tables by the canonical 2-bit packed k-mer, which equals the seq-hash
// value; this pass exposes every family so hash values can be checked bit for bit.
#include "common.cuh"
#include "kernels.h"

namespace ggcat {

typedef unsigned __int128 u128;

__device__ __forceinline__ u128 mk128(uint64_t hi, uint64_t lo) { return ((u128)hi << 64) | (u128)lo; }

// Rabin-Karp constants (crates/hashes/src/cn_rkhash.rs:58-78): the hash definition.
__device__ __forceinline__ u128 rk_mult() { return mk128(0x3eb9402f3e733993ull, 0xadd64d3ca00e1b6bull); }
__device__ __forceinline__ u128 rk_inv() { return mk128(0x09cb6ff6f1b1a6d7ull, 0x33e0952e899c3943ull); }
// FWD_LOOKUP over 2-bit codes A0 C1 T2 G3 (cn_rkhash_base.rs:10-25)
__device__ __forceinline__ u128 rk_fwd(uint32_t c) {
    switch (c & 3u) {
    case 0: return mk128(0x4751137d01d863c5ull, 0xb8c36de2b7d399dfull);   // A
    case 1: return mk128(0x37ea3a13226503fbull, 0x783f5cb69f4552bdull);   // C
    case 2: return mk128(0x1e62d96a5e1f5adeull, 0x2d4e68d8f88110b7ull);   // T
    default: return mk128(0x50796b285343f09aull, 0x0c53113ae736572bull); // G
    }
}
__device__ __forceinline__ u128 rk_bkw(uint32_t c) { return rk_fwd((c & 3u) ^ 2u); }

__device__ __forceinline__ u128 rk_pow(u128 b, uint32_t e) {
    u128 r = 1;
    while (e) {
        if (e & 1u) r *= b;
        b *= b;
        e >>= 1;
    }
    return r;
}

__device__ __forceinline__ bool base_at(const uint8_t *text, uint64_t p, uint32_t &code) {
    const uint32_t c = text[p];
    const uint32_t u = c & 0xDFu;
    code = (c >> 1) & 3u;
    return (u == 'A') | (u == 'C') | (u == 'G') | (u == 'T');
}

// kind: 0 cn seq u64, 1 fw seq u64, 2 cn seq u128, 3 fw seq u128, 4 cn rk u128, 5 fw rk u128,
// 6 nt-hash m-mer values (k = m).  out[2*i], out[2*i+1] = (lo, hi) of the unextendable hash
// of the window starting at i; windows that span a non-ACGT byte get (~0, ~0).
__global__ void __launch_bounds__(256) kmer_hash_kernel(const uint8_t *__restrict__ text, uint64_t n, int k,
                                                        int kind, uint64_t chunk, uint64_t *__restrict__ out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t x0 = tid * chunk;
    if (x0 >= n) return;
    const uint64_t n_win = n >= (uint64_t)k ? n - (uint64_t)k + 1 : 0;
    const uint64_t x1 = min(x0 + chunk, n_win);
    for (uint64_t i = x0; i < min(x0 + chunk, n); i++) {
        out[2 * i] = ~0ull;
        out[2 * i + 1] = ~0ull;
    }
    if (x0 >= x1) return;
    const bool canon = (kind % 2) == 0;
    const u128 all = ~(u128)0;
    const int words = (kind <= 1) ? 32 : 64;
    const u128 wmask = words == 32 ? (u128)~0ull : all;
    const u128 smask = (kind < 4) ? (wmask >> (2 * (words - k))) : all;
    const u128 M = rk_mult(), INV = rk_inv();
    const u128 rm = rk_pow(M, (uint32_t)(k - 1));
    u128 fw = 0, rc = 0;
    uint64_t ntf = 0, ntr = 0;
    uint64_t run = 0;
    uint32_t code;
    // history of the last k codes for the rolling updates that need the outgoing base
    uint32_t hist[128];
    for (uint64_t p = x0; p < x1 + (uint64_t)k - 1; p++) {
        if (!base_at(text, p, code)) {
            run = 0;
            continue;
        }
        hist[p % 128] = code;
        run++;
        if (run < (uint64_t)k) continue;
        const uint64_t start = p + 1 - (uint64_t)k;
        if (run == (uint64_t)k) {
            // window from scratch
            fw = 0;
            rc = 0;
            ntf = 0;
            ntr = 0;
            for (int j = 0; j < k; j++) {
                const uint32_t c = hist[(start + j) % 128];
                if (kind < 4) {
                    fw |= (u128)c << (2 * j);
                    rc = ((rc << 2) | (u128)(c ^ 2u)) & smask;
                } else if (kind < 6) {
                    fw = fw * M + rk_fwd(c);
                } else {
                    ntf ^= rotl64((uint64_t)(2 * c + 1) * kNtMult, (unsigned)(k - 1 - j));
                    ntr ^= rotl64((uint64_t)(((2 * c) ^ 4) + 1) * kNtMult, (unsigned)j);
                }
            }
            if (kind >= 4 && kind < 6)
                for (int j = k - 1; j >= 0; j--) rc = rc * M + rk_bkw(hist[(start + j) % 128]);
        } else {
            const uint32_t in = code, ob = hist[(start - 1) % 128];
            if (kind < 4) {
                fw = ((fw >> 2) | ((u128)in << (2 * (k - 1)))) & wmask;
                rc = ((rc << 2) | (u128)(in ^ 2u)) & smask;
            } else if (kind < 6) {
                fw = (fw - rk_fwd(ob) * rm) * M + rk_fwd(in);
                rc = (rc - rk_bkw(ob)) * INV + rk_bkw(in) * rm;
            } else {
                ntf = rotl64(ntf, 1) ^ rotl64((uint64_t)(2 * ob + 1) * kNtMult, (unsigned)k) ^
                      ((uint64_t)(2 * in + 1) * kNtMult);
                ntr = rotr64(ntr ^ ((uint64_t)(((2 * ob) ^ 4) + 1) * kNtMult), 1) ^
                      rotl64((uint64_t)(((2 * in) ^ 4) + 1) * kNtMult, (unsigned)(k - 1));
            }
        }
        if (start < x0) continue;
        u128 h;
        if (kind == 6) {
            const uint64_t mn = ntf < ntr ? ntf : ntr;
            h = (u128)((mn << 1) | (uint64_t)(ntf != ntr));
        } else {
            h = (canon && rc < fw) ? rc : fw;
        }
        out[2 * start] = (uint64_t)h;
        out[2 * start + 1] = (uint64_t)(h >> 64);
    }
}

int launch_kmer_hash(const uint8_t *text, uint64_t n, int k, int kind, uint64_t *out, cudaStream_t s) {
    const uint64_t chunk = 256;
    const uint64_t threads = (n + chunk - 1) / chunk;
    if (!threads) return 0;
    kmer_hash_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(text, n, k, kind, chunk, out);
    return 1;
}

}  // namespace ggcat
