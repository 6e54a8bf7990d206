/*
 * ORACLE (test infrastructure only).  CPU restatement of GGCAT's rolling hash
 * families, used by the tests and by the CPU-baseline leg of bench.py as the
 * checker for the CUDA path.  Nothing in the product links or calls this code.
 *
 * Restated from (paths inside algbio/ggcat):
 *   crates/hashes/src/nthash_base.rs:49-61      nt-hash base terms h()/rc()
 *   crates/hashes/src/cn_nthash.rs:19-58         canonical nt-hash iterator
 *   crates/hashes/src/cn_nthash.rs:96-99,135-142 to_unextendable / get_bucket
 *   crates/hashes/src/base/cn_seqhash_base.rs    canonical seq-hash (u64/u128)
 *   crates/hashes/src/base/fw_seqhash_base.rs    forward seq-hash
 *   crates/hashes/src/cn_seqhash.rs:1-27         FNV bucket constants
 *   crates/hashes/src/base/cn_rkhash_base.rs     canonical Rabin-Karp
 *   crates/hashes/src/base/fw_rkhash_base.rs     forward Rabin-Karp
 *   crates/hashes/src/cn_rkhash.rs:1-78          Rabin-Karp constants
 *   crates/hashes/src/lib.rs:169-191             rmmult = MULTIPLIER^(k-1)
 */
#ifndef GGCAT_ORACLE_HASHES_H
#define GGCAT_ORACLE_HASHES_H
#include <stdint.h>
#include <stddef.h>

typedef unsigned __int128 u128;

static inline uint64_t orc_rotl64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x << r) | (x >> (64u - r)) : x;
}
static inline uint64_t orc_rotr64(uint64_t x, unsigned r) {
    r &= 63u;
    return r ? (x >> r) | (x << (64u - r)) : x;
}
static inline u128 orc_rotr128(u128 x, unsigned r) {
    r &= 127u;
    return r ? (x >> r) | (x << (128u - r)) : x;
}

/* 2-bit code of GGCAT: A0 C1 T2 G3 == (ascii >> 1) & 3 (crates/utils/src/lib.rs:44-56). */
static inline uint8_t orc_compress_base(uint8_t ascii) { return (uint8_t)((ascii >> 1) & 3u); }

/* ---------------- nt-hash (m-mer / minimizer hash) ---------------- */
#define ORC_NT_MULT 0x397f178c6ae330f9ULL
static inline uint64_t orc_nt_h(uint8_t c) { return (uint64_t)(((uint64_t)c << 1) + 1u) * ORC_NT_MULT; }
static inline uint64_t orc_nt_rc(uint8_t c) { return (uint64_t)((((uint64_t)c << 1) ^ 4u) + 1u) * ORC_NT_MULT; }

/* Hash kinds of the k-mer ("merging") hash, crates/api/src/utils.rs:10-69. */
enum {
    ORC_H_CN_SEQ64 = 0,
    ORC_H_FW_SEQ64 = 1,
    ORC_H_CN_SEQ128 = 2,
    ORC_H_FW_SEQ128 = 3,
    ORC_H_CN_RK128 = 4,
    ORC_H_FW_RK128 = 5,
    ORC_H_CN_RK64 = 6,
    ORC_H_FW_RK64 = 7,
};

/* An extendable hash: forward and reverse-complement words (fw only for forward kinds). */
typedef struct { u128 fw, rc; } orc_ext_hash;

void orc_hash_init_k(int kind, int k);
int orc_hash_is_canonical(int kind);
int orc_hash_is_invertible(int kind);
int orc_hash_usable_bits(int kind);
u128 orc_hash_unext(int kind, orc_ext_hash h);
int orc_hash_is_forward(int kind, orc_ext_hash h);
int orc_hash_is_symmetric(int kind, orc_ext_hash h);
uint32_t orc_hash_get_bucket(int kind, int used_bits, int req_bits, u128 h);
/* Iterate all k-mers of a 2-bit sequence (one code per byte). Returns count. */
size_t orc_hash_iter(int kind, const uint8_t *cbases, size_t n, int k, orc_ext_hash *out);
orc_ext_hash orc_hash_roll_fw(int kind, orc_ext_hash h, int k, uint8_t out_b, uint8_t in_b);
orc_ext_hash orc_hash_roll_bw(int kind, orc_ext_hash h, int k, uint8_t out_b, uint8_t in_b);
orc_ext_hash orc_hash_remove_fw(int kind, orc_ext_hash h, int k, uint8_t out_b);
orc_ext_hash orc_hash_remove_bw(int kind, orc_ext_hash h, int k, uint8_t out_b);

/* nt-hash iterator over m-mers of a 2-bit sequence. Returns count of m-mers. */
size_t orc_nthash_iter(const uint8_t *cbases, size_t n, int m, uint64_t *out_fw, uint64_t *out_rc);

#endif
