/*
 * ORACLE (test infrastructure only): CPU restatement of GGCAT's hash families.
 * See oracle_hashes.h for the list of reference files this follows.
 */
#include "oracle_hashes.h"

/* ---- Rabin-Karp constants: crates/hashes/src/cn_rkhash.rs:17-78 (same for fw_rkhash.rs) ---- */
#define U128C(hi, lo) ((((u128)(hi)) << 64) | (u128)(lo))
static const uint64_t RK64_MULT = 0x660b123642ca9149ULL;
static const uint64_t RK64_INV = 0x397f178c6ae330f9ULL;
static const uint64_t RK64_A = 0x34889973de695e1bULL, RK64_C = 0x72dacb3a60672825ULL,
                      RK64_G = 0x61bf33e452d231a5ULL, RK64_T = 0x759db32ccd931bb5ULL;
#define RK128_MULT U128C(0x3eb9402f3e733993ULL, 0xadd64d3ca00e1b6bULL)
#define RK128_INV U128C(0x09cb6ff6f1b1a6d7ULL, 0x33e0952e899c3943ULL)
#define RK128_A U128C(0x4751137d01d863c5ULL, 0xb8c36de2b7d399dfULL)
#define RK128_C U128C(0x37ea3a13226503fbULL, 0x783f5cb69f4552bdULL)
#define RK128_G U128C(0x50796b285343f09aULL, 0x0c53113ae736572bULL)
#define RK128_T U128C(0x1e62d96a5e1f5adeULL, 0x2d4e68d8f88110b7ULL)

/* seq-hash bucket constants: crates/hashes/src/cn_seqhash.rs:15-27 */
static const uint64_t SEQ64_BMULT = 0x00000100000001b3ULL, SEQ64_BBASIS = 0xcbf29ce484222325ULL;
#define SEQ128_BMULT U128C(0x0000000001000000ULL, 0x000000000000013bULL)
#define SEQ128_BBASIS U128C(0x6c62272e07bb0142ULL, 0x62b821756295c58dULL)

/* rmmult cache, crates/hashes/src/lib.rs:169-191: rmmult(k) = MULTIPLIER^(k-1) */
static u128 rk_pow(u128 base, size_t exp) {
    u128 r = 1, s = base;
    while (exp) {
        if (exp & 1) r *= s;
        exp >>= 1;
        s *= s;
    }
    return r;
}

static inline int is_rk(int kind) {
    return kind == ORC_H_CN_RK128 || kind == ORC_H_FW_RK128 || kind == ORC_H_CN_RK64 || kind == ORC_H_FW_RK64;
}
static inline int is_64(int kind) {
    return kind == ORC_H_CN_SEQ64 || kind == ORC_H_FW_SEQ64 || kind == ORC_H_CN_RK64 || kind == ORC_H_FW_RK64;
}
static inline u128 wmask(int kind) { return is_64(kind) ? (u128)UINT64_MAX : ~(u128)0; }

static u128 rk_mult(int kind) { return is_64(kind) ? (u128)RK64_MULT : RK128_MULT; }
static u128 rk_inv(int kind) { return is_64(kind) ? (u128)RK64_INV : RK128_INV; }
/* FWD_LOOKUP / BKW_LOOKUP of cn_rkhash_base.rs:10-44 restricted to 2-bit codes (A0 C1 T2 G3). */
static u128 rk_fwd(int kind, uint8_t c) {
    if (is_64(kind)) {
        static const uint64_t t[4] = {0x34889973de695e1bULL, 0x72dacb3a60672825ULL, 0x759db32ccd931bb5ULL,
                                      0x61bf33e452d231a5ULL};
        (void)RK64_A; (void)RK64_C; (void)RK64_G; (void)RK64_T;
        return t[c & 3];
    } else {
        const u128 t[4] = {RK128_A, RK128_C, RK128_T, RK128_G};
        return t[c & 3];
    }
}
static u128 rk_bkw(int kind, uint8_t c) { return rk_fwd(kind, (uint8_t)((c & 3) ^ 2)); }
static u128 rk_rmmult(int kind, int k) { return rk_pow(rk_mult(kind), (size_t)(k > 0 ? k - 1 : 0)) & wmask(kind); }

static inline u128 seq_mask(int kind, int k) {
    int words = is_64(kind) ? 32 : 64;
    u128 all = wmask(kind);
    return all >> ((unsigned)(words - k) * 2u);
}

void orc_hash_init_k(int kind, int k) { (void)kind; (void)k; }

int orc_hash_is_canonical(int kind) {
    return kind == ORC_H_CN_SEQ64 || kind == ORC_H_CN_SEQ128 || kind == ORC_H_CN_RK128 || kind == ORC_H_CN_RK64;
}
int orc_hash_is_invertible(int kind) { return !is_rk(kind); }
int orc_hash_usable_bits(int kind) {
    int bits = is_64(kind) ? 64 : 128;
    return is_rk(kind) ? bits - 1 : bits;
}

u128 orc_hash_unext(int kind, orc_ext_hash h) {
    if (!orc_hash_is_canonical(kind)) return h.fw;
    return h.fw < h.rc ? h.fw : h.rc;
}
int orc_hash_is_forward(int kind, orc_ext_hash h) { return orc_hash_is_canonical(kind) ? h.fw < h.rc : 1; }
int orc_hash_is_symmetric(int kind, orc_ext_hash h) { return orc_hash_is_canonical(kind) ? h.fw == h.rc : 0; }

uint32_t orc_hash_get_bucket(int kind, int used_bits, int req_bits, u128 h) {
    u128 mod = ((u128)1) << req_bits;
    if (is_rk(kind)) return (uint32_t)((h >> (used_bits + 1)) % mod);
    if (is_64(kind)) {
        uint64_t x = (uint64_t)h * SEQ64_BMULT + SEQ64_BBASIS;
        x = orc_rotr64(x, 3);
        return (uint32_t)((x >> used_bits) % (uint64_t)mod);
    } else {
        u128 x = h * SEQ128_BMULT + SEQ128_BBASIS;
        x = orc_rotr128(x, 3);
        return (uint32_t)((x >> used_bits) % mod);
    }
}

/* Iterators: cn_seqhash_base.rs:23-69, fw_seqhash_base.rs:18-59, cn_rkhash_base.rs:62-109,
 * fw_rkhash_base.rs:40-69.  out[i] is the hash of the k-mer starting at base i. */
size_t orc_hash_iter(int kind, const uint8_t *cb, size_t n, int k, orc_ext_hash *out) {
    if (k <= 0 || (size_t)k > n) return 0;
    size_t cnt = n - (size_t)k + 1;
    u128 M = wmask(kind);
    if (!is_rk(kind)) {
        u128 mask = seq_mask(kind, k);
        u128 fh = 0, bw = 0;
        for (int i = 0; i < k - 1; i++) {
            u128 b = cb[i] & 3;
            fh |= b << (2 * i);
            bw = ((bw << 2) | (b ^ 2)) & M;
        }
        fh = (fh << 2) & M;
        u128 rc = bw & mask;
        for (size_t idx = (size_t)k - 1; idx < n; idx++) {
            u128 b = cb[idx] & 3;
            fh = ((fh >> 2) | (b << (2 * (k - 1)))) & M;
            rc = ((rc << 2) | (b ^ 2)) & mask;
            out[idx - (size_t)k + 1].fw = fh;
            out[idx - (size_t)k + 1].rc = orc_hash_is_canonical(kind) ? rc : 0;
        }
    } else {
        u128 mult = rk_mult(kind), inv = rk_inv(kind), rm = rk_rmmult(kind, k);
        u128 fh = 0, bw = 0;
        for (int i = 0; i < k - 1; i++) fh = (fh * mult + rk_fwd(kind, cb[i])) & M;
        for (int i = k - 2; i >= 0; i--) bw = (bw * mult + rk_bkw(kind, cb[i])) & M;
        bw = (bw * mult) & M;
        u128 rc = bw;
        for (size_t idx = (size_t)k - 1; idx < n; idx++) {
            uint8_t in = cb[idx], ob = cb[idx - (size_t)k + 1];
            u128 cur_fh = (fh * mult + rk_fwd(kind, in)) & M;
            fh = (cur_fh - rk_fwd(kind, ob) * rm) & M;
            u128 cur_bk = (rc * inv + rk_bkw(kind, in) * rm) & M;
            rc = (cur_bk - rk_bkw(kind, ob)) & M;
            out[idx - (size_t)k + 1].fw = cur_fh;
            out[idx - (size_t)k + 1].rc = orc_hash_is_canonical(kind) ? cur_bk : 0;
        }
    }
    return cnt;
}

/* manual_roll_forward (cn_seqhash_base.rs:160-177, cn_rkhash_base.rs:217-236, fw variants) */
orc_ext_hash orc_hash_roll_fw(int kind, orc_ext_hash h, int k, uint8_t ob, uint8_t ib) {
    u128 M = wmask(kind);
    orc_ext_hash r = {0, 0};
    if (!is_rk(kind)) {
        u128 mask = seq_mask(kind, k);
        r.fw = ((h.fw >> 2) | ((u128)(ib & 3) << (2 * (k - 1)))) & M;
        if (orc_hash_is_canonical(kind)) r.rc = ((h.rc << 2) | (u128)((ib & 3) ^ 2)) & mask;
    } else {
        u128 rm = rk_rmmult(kind, k), mult = rk_mult(kind), inv = rk_inv(kind);
        r.fw = ((h.fw - rk_fwd(kind, ob) * rm) * mult + rk_fwd(kind, ib)) & M;
        if (orc_hash_is_canonical(kind)) r.rc = ((h.rc - rk_bkw(kind, ob)) * inv + rk_bkw(kind, ib) * rm) & M;
    }
    return r;
}

/* manual_roll_reverse (cn_seqhash_base.rs:179-197, cn_rkhash_base.rs:238-258, fw variants) */
orc_ext_hash orc_hash_roll_bw(int kind, orc_ext_hash h, int k, uint8_t ob, uint8_t ib) {
    u128 M = wmask(kind);
    orc_ext_hash r = {0, 0};
    if (!is_rk(kind)) {
        u128 mask = seq_mask(kind, k);
        r.fw = ((h.fw << 2) | (u128)(ib & 3)) & mask;
        if (orc_hash_is_canonical(kind)) r.rc = ((h.rc >> 2) | ((u128)((ib & 3) ^ 2) << (2 * (k - 1)))) & M;
    } else {
        u128 rm = rk_rmmult(kind, k), mult = rk_mult(kind), inv = rk_inv(kind);
        r.fw = ((h.fw - rk_fwd(kind, ob)) * inv + rk_fwd(kind, ib) * rm) & M;
        if (orc_hash_is_canonical(kind)) r.rc = ((h.rc - rk_bkw(kind, ob) * rm) * mult + rk_bkw(kind, ib)) & M;
    }
    return r;
}

/* manual_remove_only_forward (cn_seqhash_base.rs:199-211, cn_rkhash_base.rs:260-274) */
orc_ext_hash orc_hash_remove_fw(int kind, orc_ext_hash h, int k, uint8_t ob) {
    u128 M = wmask(kind);
    orc_ext_hash r = {0, 0};
    if (!is_rk(kind)) {
        r.fw = h.fw >> 2;
        if (orc_hash_is_canonical(kind)) r.rc = h.rc & seq_mask(kind, k - 1);
    } else {
        u128 rm = rk_rmmult(kind, k), inv = rk_inv(kind);
        r.fw = (h.fw - rm * rk_fwd(kind, ob)) & M;
        if (orc_hash_is_canonical(kind)) r.rc = ((h.rc - rk_bkw(kind, ob)) * inv) & M;
    }
    return r;
}

/* manual_remove_only_reverse (cn_seqhash_base.rs:213-225, cn_rkhash_base.rs:276-290) */
orc_ext_hash orc_hash_remove_bw(int kind, orc_ext_hash h, int k, uint8_t ob) {
    u128 M = wmask(kind);
    orc_ext_hash r = {0, 0};
    if (!is_rk(kind)) {
        r.fw = h.fw & seq_mask(kind, k - 1);
        if (orc_hash_is_canonical(kind)) r.rc = h.rc >> 2;
    } else {
        u128 rm = rk_rmmult(kind, k), inv = rk_inv(kind);
        r.fw = ((h.fw - rk_fwd(kind, ob)) * inv) & M;
        if (orc_hash_is_canonical(kind)) r.rc = (h.rc - rm * rk_bkw(kind, ob)) & M;
    }
    return r;
}

/* CanonicalNtHashIterator::new/roll_hash, crates/hashes/src/cn_nthash.rs:21-58 */
size_t orc_nthash_iter(const uint8_t *cb, size_t n, int m, uint64_t *out_fw, uint64_t *out_rc) {
    if (m <= 0 || (size_t)m > n) return 0;
    uint64_t fh = 0, bw = 0;
    for (int i = 0; i < m - 1; i++) {
        fh ^= orc_rotl64(orc_nt_h(cb[i]), (unsigned)(m - i - 2));
        bw ^= orc_rotl64(orc_nt_rc(cb[i]), (unsigned)i);
    }
    size_t cnt = n - (size_t)m + 1;
    for (size_t i = 0; i < cnt; i++) {
        uint8_t bi = cb[i], bk = cb[i + (size_t)m - 1];
        uint64_t res = orc_rotl64(fh, 1) ^ orc_nt_h(bk);
        fh = res ^ orc_rotl64(orc_nt_h(bi), (unsigned)(m - 1));
        uint64_t res_rc = bw ^ orc_rotl64(orc_nt_rc(bk), (unsigned)(m - 1));
        bw = orc_rotr64(res_rc ^ orc_nt_rc(bi), 1);
        out_fw[i] = res;
        out_rc[i] = res_rc;
    }
    return cnt;
}
