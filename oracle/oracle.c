/*
 * ORACLE (test infrastructure only): CPU restatement of GGCAT's minimizer bucketing,
 * per-sub-bucket k-mer merge, link stage and query lookup.  See oracle.h.
 *
 * Each function names the reference lines it restates (paths inside algbio/ggcat).
 */
#define _GNU_SOURCE
#include "oracle.h"
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define READ_FLAG_INCL_BEGIN 1u /* crates/config/src/lib.rs:93 */
#define READ_FLAG_INCL_END 2u   /* crates/config/src/lib.rs:94 */

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) {
        fprintf(stderr, "oracle: out of memory (%zu bytes)\n", n);
        abort();
    }
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        abort();
    }
    return p;
}
static void *xrealloc(void *q, size_t n) {
    void *p = realloc(q, n ? n : 1);
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        abort();
    }
    return p;
}

/* ======================================================================
 * BatchMinQueue — crates/hashes/src/rolling/batch_minqueue.rs:37-188
 * ====================================================================== */
static inline int item_x_eq(const orc_mq_item *a, const orc_mq_item *b) {
    return a->index == b->index && a->is_forward == b->is_forward;
}
/* std::cmp::min_by_key keeps the first argument on equal keys */
static inline orc_mq_item min_by_v(orc_mq_item a, orc_mq_item b) { return a.v <= b.v ? a : b; }

typedef struct {
    size_t *pos;
    orc_mq_item *val;
    uint8_t *last;
    size_t n, cap;
} split_sink;

/* get_minimizers: batch_minqueue.rs:37-120.  min_cb receives (value, offset);
 * flush_cb receives is_last. */
typedef void (*mq_min_cb)(void *ctx, orc_mq_item m, size_t index);
typedef void (*mq_flush_cb)(void *ctx, int is_last);

static void mq_get_minimizers(size_t size, orc_mq_item *backward, const orc_mq_item *iter, size_t len,
                              size_t skip_ending, int dup, mq_min_cb min_cb, mq_flush_cb flush_cb, void *ctx) {
    const size_t bl = size - 1;
    if (len < skip_ending) return;
    size_t total = len - skip_ending;
    if (total < bl) return;
    size_t pos = 0;
    for (size_t i = 0; i < bl; i++) backward[i] = iter[pos++];
    size_t offset = 0;
    const size_t S = total - bl;
    const uint64_t mask = dup ? ~(uint64_t)1 : ~(uint64_t)0;
    while (offset < S) {
        size_t remaining = S - offset < bl ? S - offset : bl;
        for (size_t ii = bl - 1; ii-- > 0;) {
            orc_mq_item current = backward[ii];
            orc_mq_item next = backward[ii + 1];
            if (dup && current.v == next.v) current.v &= mask;
            backward[ii] = min_by_v(current, next);
        }
        orc_mq_item new_item = iter[pos++];
        orc_mq_item first_min = min_by_v(new_item, backward[0]);
        if (dup && new_item.v == backward[0].v) first_min.v &= mask;
        min_cb(ctx, first_min, offset);
        orc_mq_item last_forward = new_item;
        backward[0] = new_item;
        for (size_t i = 1; i < remaining; i++) {
            new_item = iter[pos++];
            if (dup && new_item.v == last_forward.v) last_forward.v &= mask;
            last_forward = min_by_v(last_forward, new_item);
            orc_mq_item cur = min_by_v(last_forward, backward[i]);
            if (dup && last_forward.v == backward[i].v) cur.v &= mask;
            min_cb(ctx, cur, offset + i);
            backward[i] = new_item;
        }
        offset += remaining;
        flush_cb(ctx, offset == S);
    }
}

/* get_minimizer_splits: batch_minqueue.rs:122-188 */
typedef void (*mq_split_cb)(void *ctx, size_t position, orc_mq_item value, int is_last);
typedef struct {
    orc_mq_item last_value;
    int is_first;
    size_t last_index, skip_b;
    int dup;
    /* pending split buffer (self.splits) */
    size_t *sp_pos;
    orc_mq_item *sp_val;
    size_t sp_n, sp_cap;
    mq_split_cb cb;
    void *cb_ctx;
} split_state;

static void split_push(split_state *s, orc_mq_item v, size_t position, int advance) {
    if (s->sp_n >= s->sp_cap) {
        s->sp_cap = s->sp_cap ? s->sp_cap * 2 : 64;
        s->sp_pos = xrealloc(s->sp_pos, s->sp_cap * sizeof(size_t));
        s->sp_val = xrealloc(s->sp_val, s->sp_cap * sizeof(orc_mq_item));
    }
    s->sp_val[s->sp_n] = v;
    s->sp_pos[s->sp_n] = position;
    if (advance) s->sp_n++;
}
static void split_min_cb(void *ctx, orc_mq_item m, size_t index) {
    split_state *s = ctx;
    const uint64_t uf = s->dup ? 1u : 0u;
    int has_diff = !s->is_first && (s->last_value.v != m.v || (!item_x_eq(&s->last_value, &m) && (m.v & uf) == uf));
    split_push(s, s->last_value, index + s->skip_b, has_diff);
    s->is_first = 0;
    s->last_value = m;
}
static void split_flush_cb(void *ctx, int is_last) {
    split_state *s = ctx;
    if (is_last) split_push(s, s->last_value, s->last_index, 1);
    for (size_t i = 0; i < s->sp_n; i++) {
        int last = (i + 1 == s->sp_n);
        s->cb(s->cb_ctx, s->sp_pos[i], s->sp_val[i], last && is_last);
    }
    s->sp_n = 0;
}

static void mq_get_minimizer_splits(size_t size, orc_mq_item *backward, const orc_mq_item *items, size_t n,
                                    size_t skip_b, size_t skip_e, int dup, mq_split_cb cb, void *ctx,
                                    split_state *st) {
    st->last_value = (orc_mq_item){0, 0, 0, {0, 0, 0}};
    st->is_first = 1;
    st->last_index = n - size;
    st->skip_b = skip_b;
    st->dup = dup;
    st->sp_n = 0;
    st->cb = cb;
    st->cb_ctx = ctx;
    if (skip_b > n) return;
    mq_get_minimizers(size, backward, items + skip_b, n - skip_b, skip_e, dup, split_min_cb, split_flush_cb, st);
}

typedef struct {
    size_t *pos;
    orc_mq_item *val;
    uint8_t *last;
    size_t n, cap;
} collect_ctx;
static void collect_split(void *ctx, size_t position, orc_mq_item value, int is_last) {
    collect_ctx *c = ctx;
    if (c->n < c->cap) {
        c->pos[c->n] = position;
        c->val[c->n] = value;
        c->last[c->n] = (uint8_t)is_last;
    }
    c->n++;
}
size_t orc_minqueue_splits(size_t size, const orc_mq_item *items, size_t n, size_t skip_b, size_t skip_e,
                           int dup_check, size_t *out_pos, orc_mq_item *out_val, uint8_t *out_last, size_t cap) {
    if (size < 2) return 0;
    orc_mq_item *backward = xmalloc(size * sizeof(orc_mq_item));
    split_state st;
    memset(&st, 0, sizeof st);
    collect_ctx c = {out_pos, out_val, out_last, 0, cap};
    mq_get_minimizer_splits(size, backward, items, n, skip_b, skip_e, dup_check, collect_split, &c, &st);
    free(backward);
    free(st.sp_pos);
    free(st.sp_val);
    return c.n;
}

typedef struct {
    orc_mq_item *out;
    size_t n, cap;
} collect_min_ctx;
static void collect_min(void *ctx, orc_mq_item m, size_t index) {
    collect_min_ctx *c = ctx;
    if (index < c->cap) c->out[index] = m;
    if (index + 1 > c->n) c->n = index + 1;
}
static void noop_flush(void *ctx, int is_last) {
    (void)ctx;
    (void)is_last;
}
size_t orc_minqueue_minimizers(size_t size, const orc_mq_item *items, size_t n, size_t skip_e, int dup_check,
                               orc_mq_item *out, size_t cap) {
    if (size < 2) return 0;
    orc_mq_item *backward = xmalloc(size * sizeof(orc_mq_item));
    collect_min_ctx c = {out, 0, cap};
    mq_get_minimizers(size, backward, items, n, skip_e, dup_check, collect_min, noop_flush, &c);
    free(backward);
    return c.n;
}

/* ======================================================================
 * Minimizer bucketing
 * ====================================================================== */

/* SEQ_LETTERS_MAPPING, crates/io/src/sequences_reader.rs:26-37 */
static uint8_t norm_table[256];
static pthread_once_t norm_once = PTHREAD_ONCE_INIT;
static void norm_init(void) {
    for (int i = 0; i < 256; i++) norm_table[i] = 'N';
    norm_table['A'] = 'A';
    norm_table['C'] = 'C';
    norm_table['G'] = 'G';
    norm_table['T'] = 'T';
    norm_table['a'] = 'A';
    norm_table['c'] = 'C';
    norm_table['g'] = 'G';
    norm_table['t'] = 'T';
}

/* nt-hash get_bucket: crates/hashes/src/cn_nthash.rs:135-142 (one discarded bit) */
static inline uint32_t nt_get_bucket(int used_bits, int req_bits, uint64_t h) {
    return (uint32_t)((h >> (used_bits + 1)) % (1ULL << req_bits));
}

typedef struct {
    orc_superkmer *v;
    size_t n, cap;
} sk_vec;
static void sk_push(sk_vec *vec, const orc_superkmer *s) {
    if (vec->n == vec->cap) {
        vec->cap = vec->cap ? vec->cap * 2 : 1024;
        vec->v = xrealloc(vec->v, vec->cap * sizeof(orc_superkmer));
    }
    vec->v[vec->n++] = *s;
}

typedef struct {
    const orc_params *p;
    uint64_t piece_abs;   /* absolute offset of the piece in the text */
    uint32_t seq_index;
    size_t last_index;    /* process_sequence: last_index */
    int include_first;
    int include_last_pre; /* preprocess_info.include_last */
    uint16_t dup_bucket;
    sk_vec *out;
} proc_ctx;

/* AssemblerMinimizerBucketingExecutor::process_sequence split callback,
 * crates/assembler_minimizer_bucketing/src/lib.rs:207-267 */
static void process_split_cb(void *vctx, size_t index, orc_mq_item mh, int is_last) {
    proc_ctx *c = vctx;
    const orc_params *p = c->p;
    int include_last = c->include_last_pre && is_last;
    uint16_t bucket, pos;
    int rc;
    if ((mh.v & 1u) == 0) {
        bucket = c->dup_bucket;
        rc = 0;
        pos = 0;
    } else {
        rc = p->canonical && !mh.is_forward;
        bucket = (uint16_t)nt_get_bucket(0, p->bucket_bits, mh.v);
        if (rc)
            pos = (uint16_t)(index + (size_t)p->k - 1 - (size_t)mh.index - (size_t)p->m);
        else
            pos = (uint16_t)(mh.index - (uint32_t)(c->last_index - 1));
    }
    orc_superkmer s;
    memset(&s, 0, sizeof s);
    size_t b = c->last_index - 1, e = index + (size_t)p->k - 1;
    s.start = c->piece_abs + b;
    s.len = (uint32_t)(e - b);
    s.bucket = bucket;
    s.second_bucket = (uint16_t)nt_get_bucket(p->bucket_bits, p->second_bits, mh.v);
    s.minimizer_pos = pos;
    s.rc = (uint8_t)rc;
    s.flags = (uint8_t)(((unsigned)c->include_first << (unsigned)rc) | ((unsigned)include_last << (unsigned)!rc));
    s.seq_index = c->seq_index;
    s.minimizer = mh.v;
    sk_push(c->out, &s);
    c->last_index = index;
    c->include_first = 0;
}

typedef struct {
    uint8_t *cb;
    uint64_t *fw, *rc;
    orc_mq_item *items, *backward;
    size_t cap, bcap;
    split_state st;
} proc_scratch;

static void scratch_reserve(proc_scratch *s, size_t n, size_t w) {
    if (n > s->cap) {
        s->cap = n * 2;
        s->cb = xrealloc(s->cb, s->cap);
        s->fw = xrealloc(s->fw, s->cap * sizeof(uint64_t));
        s->rc = xrealloc(s->rc, s->cap * sizeof(uint64_t));
        s->items = xrealloc(s->items, s->cap * sizeof(orc_mq_item));
    }
    if (w > s->bcap) {
        s->bcap = w;
        s->backward = xrealloc(s->backward, w * sizeof(orc_mq_item));
    }
}
static void scratch_free(proc_scratch *s) {
    free(s->cb);
    free(s->fw);
    free(s->rc);
    free(s->items);
    free(s->backward);
    free(s->st.sp_pos);
    free(s->st.sp_val);
}

/* One piece (a run without N, length >= k): process_sequence with include_first =
 * include_last = true (preprocess_dna_sequence, lib.rs:120-151). */
static void process_piece(const uint8_t *text, uint64_t abs, size_t len, uint32_t seq_index, const orc_params *p,
                          proc_scratch *sc, sk_vec *out) {
    const size_t w = (size_t)(p->k - p->m);
    scratch_reserve(sc, len, w);
    for (size_t i = 0; i < len; i++) sc->cb[i] = orc_compress_base(norm_table[text[abs + i]]);
    size_t nm = orc_nthash_iter(sc->cb, len, p->m, sc->fw, sc->rc);
    for (size_t i = 0; i < nm; i++) {
        uint64_t f = sc->fw[i], r = sc->rc[i];
        uint64_t mn = f < r ? f : r;
        /* to_unextendable (cn_nthash.rs:96-99) | unique flag when not rc-symmetric (lib.rs:189-199) */
        sc->items[i].v = (mn << 1) | (uint64_t)(f != r);
        sc->items[i].index = (uint32_t)i;
        sc->items[i].is_forward = (uint8_t)(f < r);
    }
    proc_ctx c;
    c.p = p;
    c.piece_abs = abs;
    c.seq_index = seq_index;
    c.last_index = 1;
    c.include_first = 1;
    c.include_last_pre = 1;
    c.dup_bucket = (uint16_t)(1u << p->bucket_bits);
    c.out = out;
    mq_get_minimizer_splits(w, sc->backward, sc->items, nm, 0, 0, 1, process_split_cb, &c, &sc->st);
}

/* SequencesSplitter::process_sequences, crates/minimizer_bucketing/src/sequences_splitter.rs:15-40,
 * on the normalised sequence. */
static void process_sequence_all(const uint8_t *text, uint64_t off, uint64_t len, uint32_t seq_index,
                                 const orc_params *p, proc_scratch *sc, sk_vec *out) {
    uint64_t end = 0;
    while (end < len) {
        uint64_t start = end;
        while (start < len && ((norm_table[text[off + start]] ^ 'N') & 7) == 0) start++;
        end = start;
        while (end < len && ((norm_table[text[off + end]] ^ 'N') & 7) != 0) end++;
        if (end - start >= (uint64_t)p->k) process_piece(text, off + start, (size_t)(end - start), seq_index, p, sc, out);
    }
}

typedef struct {
    const uint8_t *text;
    const uint64_t *off, *len;
    size_t nseq;
    const orc_params *p;
    size_t tid, nthreads;
    sk_vec out;
} bucketize_job;

static void *bucketize_worker(void *arg) {
    bucketize_job *j = arg;
    proc_scratch sc;
    memset(&sc, 0, sizeof sc);
    size_t per = (j->nseq + j->nthreads - 1) / j->nthreads;
    size_t a = j->tid * per, b = a + per < j->nseq ? a + per : j->nseq;
    for (size_t s = a; s < b; s++) process_sequence_all(j->text, j->off[s], j->len[s], (uint32_t)s, j->p, &sc, &j->out);
    scratch_free(&sc);
    return NULL;
}

static sk_vec bucketize_vec(const uint8_t *text, const uint64_t *seq_off, const uint64_t *seq_len, size_t nseq,
                            const orc_params *p) {
    pthread_once(&norm_once, norm_init);
    int nt = p->threads > 0 ? p->threads : 1;
    if ((size_t)nt > nseq && nseq > 0) nt = (int)nseq;
    bucketize_job *jobs = xcalloc((size_t)nt, sizeof(bucketize_job));
    pthread_t *th = xcalloc((size_t)nt, sizeof(pthread_t));
    for (int t = 0; t < nt; t++) {
        jobs[t].text = text;
        jobs[t].off = seq_off;
        jobs[t].len = seq_len;
        jobs[t].nseq = nseq;
        jobs[t].p = p;
        jobs[t].tid = (size_t)t;
        jobs[t].nthreads = (size_t)nt;
        if (nt > 1)
            pthread_create(&th[t], NULL, bucketize_worker, &jobs[t]);
        else
            bucketize_worker(&jobs[t]);
    }
    sk_vec all = {0, 0, 0};
    for (int t = 0; t < nt; t++) {
        if (nt > 1) pthread_join(th[t], NULL);
        for (size_t i = 0; i < jobs[t].out.n; i++) sk_push(&all, &jobs[t].out.v[i]);
        free(jobs[t].out.v);
    }
    free(jobs);
    free(th);
    return all;
}

size_t orc_bucketize(const uint8_t *text, const uint64_t *seq_off, const uint64_t *seq_len, size_t nseq,
                     const orc_params *p, orc_superkmer *out, size_t cap) {
    if (p->k - p->m < 2) return 0;
    sk_vec v = bucketize_vec(text, seq_off, seq_len, nseq, p);
    size_t n = v.n;
    if (out) memcpy(out, v.v, (n < cap ? n : cap) * sizeof(orc_superkmer));
    free(v.v);
    return n;
}

/* ======================================================================
 * FASTA reader: SequencesReader::process_fasta (crates/io/src/sequences_reader.rs:106-182)
 * over LinesReader::process_lines (crates/io/src/lines_reader.rs:147-213) with
 * DEFAULT_OUTPUT_BUFFER_SIZE = 4 MiB read buffers (crates/config/src/lib.rs:51).
 * ====================================================================== */
#define ORC_READ_BUF (4u << 20)
typedef struct {
    uint8_t *seq;
    size_t seq_len, seq_cap;
    int on_comment, state, new_line;
    long copyback;
    size_t flush_size;
    uint8_t *out_text;
    size_t text_cap, text_used;
    uint64_t *out_off, *out_len;
    size_t cap, n;
} fasta_state;

static void fasta_emit(fasta_state *s) {
    /* normalize_sequence then func(DnaSequence) */
    if (s->n < s->cap) {
        s->out_off[s->n] = s->text_used;
        s->out_len[s->n] = s->seq_len;
    }
    if (s->text_used + s->seq_len <= s->text_cap) {
        for (size_t i = 0; i < s->seq_len; i++) s->out_text[s->text_used + i] = norm_table[s->seq[i]];
    }
    s->text_used += s->seq_len;
    s->n++;
}
static void seq_append(fasta_state *s, const uint8_t *line, size_t len) {
    if (s->seq_len + len > s->seq_cap) {
        s->seq_cap = (s->seq_len + len) * 2 + 64;
        s->seq = xrealloc(s->seq, s->seq_cap);
    }
    memcpy(s->seq + s->seq_len, line, len);
    s->seq_len += len;
}
/* the process_fasta line closure, sequences_reader.rs:129-180 */
static void fasta_line(fasta_state *s, const uint8_t *line, size_t len, int partial, int finished) {
    enum { IDENT = 0, SEQ = 1 };
    if (s->on_comment) {
        s->on_comment = !partial;
    } else if (finished || (s->new_line && len > 0 && line[0] == '>')) {
        if (s->seq_len > 0) fasta_emit(s);
        s->seq_len = 0;
        s->state = partial ? IDENT : SEQ;
    } else if (s->new_line && len > 0 && line[0] == ';') {
        s->on_comment = 1;
    } else if (s->state == IDENT) {
        if (!partial) s->state = SEQ;
    } else {
        seq_append(s, line, len);
    }
    if (s->copyback >= 0) {
        if (s->seq_len >= s->flush_size) {
            fasta_emit(s);
            size_t cb = (size_t)s->copyback;
            memmove(s->seq, s->seq + s->seq_len - cb, cb);
            s->seq_len = cb;
        }
    }
    s->new_line = !partial;
}

size_t orc_fasta_parse(const uint8_t *file, size_t file_len, long copyback, uint8_t *out_text, size_t text_cap,
                       uint64_t *out_off, uint64_t *out_len, size_t cap, size_t *out_text_used) {
    pthread_once(&norm_once, norm_init);
    fasta_state s;
    memset(&s, 0, sizeof s);
    s.state = 1;
    s.new_line = 1;
    s.copyback = copyback;
    size_t cbz = copyback > 0 ? (size_t)copyback * 2 : 0;
    s.flush_size = ORC_READ_BUF > cbz ? ORC_READ_BUF : cbz;
    s.out_text = out_text;
    s.text_cap = text_cap;
    s.out_off = out_off;
    s.out_len = out_len;
    s.cap = cap;
    /* line_pending tracking of process_lines; buffer boundaries every 4 MiB */
    for (size_t base = 0; base < file_len; base += ORC_READ_BUF) {
        size_t blen = file_len - base < ORC_READ_BUF ? file_len - base : ORC_READ_BUF;
        const uint8_t *buf = file + base;
        size_t p = 0;
        for (;;) {
            const uint8_t *nl = memchr(buf + p, '\n', blen - p);
            if (nl) {
                size_t pos = (size_t)(nl - buf);
                size_t bpos = pos;
                if (bpos != p && buf[bpos - 1] == '\r') bpos--;
                fasta_line(&s, buf + p, bpos - p, 0, 0);
                p = pos + 1;
            } else {
                size_t l = blen - p;
                if (l > 0 && buf[blen - 1] == '\r') l--;
                if (l > 0) fasta_line(&s, buf + p, l, 1, 0);
                break;
            }
        }
    }
    fasta_line(&s, (const uint8_t *)"", 0, 0, 1);
    free(s.seq);
    if (out_text_used) *out_text_used = s.text_used;
    return s.n;
}

/* ======================================================================
 * K-mer merge: HashMapUnitigsExtender
 * (crates/assembler_kmers_merge/src/unitigs_extender/hashmap.rs:361-601)
 * with MapEntry (crates/structs/src/map_entry.rs:5-85).  The reference runs the
 * sorting extender on normal groups and this extender on duplicate / outlier
 * sub-buckets; both define the same k-mer multiplicities and the same maximal
 * unitigs, and this one is restated for every sub-bucket here.
 * ====================================================================== */

/* a packed k-mer of up to 128 bases, base i at bits 2i of (lo | hi << 128) */
typedef struct {
    u128 lo, hi;
} okey;
static inline int okey_cmp(okey a, okey b) {
    if (a.hi != b.hi) return a.hi < b.hi ? -1 : 1;
    if (a.lo != b.lo) return a.lo < b.lo ? -1 : 1;
    return 0;
}

typedef struct {
    u128 key;      /* MH unextendable hash */
    u128 packed;   /* canonical 2-bit packed k-mer, bases 0-63 (seq-hash layout); bases 64-127 of
                      a k > 64 k-mer in the merge's side array, by ordinal */
    uint64_t count;
    uint8_t flags, used, occupied;
    uint32_t ordinal;    /* creation order; stable across kmap_grow (colour pairs refer to it) */
} kentry;

typedef struct {
    kentry *e;
    size_t cap, n;
} kmap;

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}
static inline size_t khash(u128 k) { return (size_t)mix64((uint64_t)k ^ mix64((uint64_t)(k >> 64))); }

static void kmap_init(kmap *m, size_t expect) {
    size_t c = 64;
    while (c < expect * 2) c <<= 1;
    m->cap = c;
    m->n = 0;
    m->e = xcalloc(c, sizeof(kentry));
}
static kentry *kmap_find(const kmap *m, u128 key) {
    size_t mask = m->cap - 1, i = khash(key) & mask;
    while (m->e[i].occupied) {
        if (m->e[i].key == key) return &m->e[i];
        i = (i + 1) & mask;
    }
    return NULL;
}
static kentry *kmap_insert(kmap *m, u128 key, int *created);
static void kmap_grow(kmap *m) {
    kmap n2;
    n2.cap = m->cap * 2;
    n2.n = 0;
    n2.e = xcalloc(n2.cap, sizeof(kentry));
    for (size_t i = 0; i < m->cap; i++)
        if (m->e[i].occupied) {
            int c;
            kentry *d = kmap_insert(&n2, m->e[i].key, &c);
            *d = m->e[i];
        }
    free(m->e);
    *m = n2;
}
static kentry *kmap_insert(kmap *m, u128 key, int *created) {
    if ((m->n + 1) * 2 > m->cap) kmap_grow(m);
    size_t mask = m->cap - 1, i = khash(key) & mask;
    while (m->e[i].occupied) {
        if (m->e[i].key == key) {
            *created = 0;
            return &m->e[i];
        }
        i = (i + 1) & mask;
    }
    m->e[i].occupied = 1;
    m->e[i].key = key;
    m->n++;
    *created = 1;
    return &m->e[i];
}

/* MapEntry::get_kmer_multiplicity, map_entry.rs:79-84 */
static inline uint64_t entry_mult(const kentry *e) {
    return e->count >> (e->flags == (READ_FLAG_INCL_BEGIN | READ_FLAG_INCL_END));
}

/* packed canonical k-mer in seq-hash layout (base i at bits 2i) for k <= 128; for k <= 64
 * the seq-hash value itself (hi = 0) */
static okey pack_canonical(const uint8_t *cb, int k, int canonical) {
    if (k <= 64) {  /* the seq-hash value (one 128-bit word) */
        u128 f = 0, r = 0;
        for (int i = 0; i < k; i++) {
            f |= (u128)(cb[i] & 3) << (2 * i);
            r |= (u128)((cb[k - 1 - i] & 3) ^ 2) << (2 * i);
        }
        okey o = {canonical && r < f ? r : f, 0};
        return o;
    }
    okey fw = {0, 0}, rc = {0, 0};
    for (int i = 0; i < k; i++) {
        const u128 f = (u128)(cb[i] & 3), r = (u128)((cb[k - 1 - i] & 3) ^ 2);
        if (i < 64) {
            fw.lo |= f << (2 * i);
            rc.lo |= r << (2 * i);
        } else {
            fw.hi |= f << (2 * (i - 64));
            rc.hi |= r << (2 * (i - 64));
        }
    }
    if (!canonical) return fw;
    return okey_cmp(fw, rc) < 0 ? fw : rc;
}
static inline size_t okey_hash(okey k) { return khash(k.lo) ^ (size_t)mix64((uint64_t)k.hi ^ mix64((uint64_t)(k.hi >> 64))); }

typedef struct {
    uint8_t *seq; /* ASCII */
    size_t len;
    uint8_t fw_link, bw_link, circular;
} unitig_t;

typedef struct {
    unitig_t *v;
    size_t n, cap;
} unitig_vec;
static void ut_push(unitig_vec *v, unitig_t u) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 256;
        v->v = xrealloc(v->v, v->cap * sizeof(unitig_t));
    }
    v->v[v->n++] = u;
}

typedef struct {
    u128 packed; /* bases 0-63; bases 64-127 of a k > 64 k-mer in the vector's hi array */
    uint64_t mult;
    uint32_t color_off, color_n;
} kmer_out;

typedef struct {
    kmer_out *v;
    size_t n, cap;
    uint32_t *colors;
    size_t ncol, colcap;
    u128 *hi; /* k > 64 only, parallel to v */
} kmer_vec;
static void kv_push(kmer_vec *v, kmer_out k, int wide, u128 hi) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->v = xrealloc(v->v, v->cap * sizeof(kmer_out));
        if (wide) v->hi = xrealloc(v->hi, v->cap * sizeof(u128));
    }
    if (wide) v->hi[v->n] = hi;
    v->v[v->n++] = k;
}
static uint32_t kv_push_colors(kmer_vec *v, const uint32_t *c, size_t n) {
    if (v->ncol + n > v->colcap) {
        v->colcap = (v->ncol + n) * 2 + 256;
        v->colors = xrealloc(v->colors, v->colcap * sizeof(uint32_t));
    }
    uint32_t off = (uint32_t)v->ncol;
    memcpy(v->colors + v->ncol, c, n * sizeof(uint32_t));
    v->ncol += n;
    return off;
}

static const char DECOMP[4] = {'A', 'C', 'T', 'G'};

typedef struct {
    const orc_params *p;
    const kmap *m;
} ext_ctx;

static int entry_ok(const ext_ctx *c, orc_ext_hash h) {
    kentry *e = kmap_find(c->m, orc_hash_unext(c->p->hash_kind, h));
    return e && entry_mult(e) >= (uint64_t)c->p->min_multiplicity;
}

/* try_extend_function, hashmap.rs:162-297 (unitigs, not simplitigs).  Returns 1 with
 * *link set when the extension stopped at a bucket boundary (Some(hash)), 0 otherwise.
 * *hit_start is set when the walk stopped on the start k-mer (a closed cycle). */
static int try_extend(const ext_ctx *c, orc_ext_hash hash, uint8_t **out, size_t *out_len, size_t *out_cap, int fwdir,
                      orc_ext_hash start_hash, int *hit_start) {
    const int kind = c->p->hash_kind, k = c->p->k;
    orc_ext_hash temp = hash;
    uint8_t temp_base = 0;
    *hit_start = 0;
    for (;;) {
        int count = 0;
        orc_ext_hash cur = temp;
        uint8_t outb = orc_compress_base((*out)[*out_len - (size_t)k]);
        for (uint8_t idx = 0; idx < 4; idx++) {
            orc_ext_hash nh = fwdir ? orc_hash_roll_fw(kind, cur, k, outb, idx) : orc_hash_roll_bw(kind, cur, k, outb, idx);
            if (entry_ok(c, nh)) {
                count++;
                temp = nh;
                temp_base = idx;
            }
        }
        if (count != 1) return 0;
        int ocount = 0;
        for (uint8_t idx = 0; idx < 4; idx++) {
            orc_ext_hash bh = fwdir ? orc_hash_roll_bw(kind, temp, k, temp_base, idx)
                                    : orc_hash_roll_fw(kind, temp, k, temp_base, idx);
            if (entry_ok(c, bh)) {
                if (ocount > 0) return 0;
                ocount++;
            }
        }
        kentry *e = kmap_find(c->m, orc_hash_unext(kind, temp));
        if (e->used) {
            if (temp.fw == start_hash.fw && temp.rc == start_hash.rc) *hit_start = 1;
            return 0;
        }
        e->used = 1;
        if (*out_len == *out_cap) {
            *out_cap *= 2;
            *out = xrealloc(*out, *out_cap);
        }
        (*out)[(*out_len)++] = (uint8_t)DECOMP[temp_base];
        if (e->flags == READ_FLAG_INCL_BEGIN || e->flags == READ_FLAG_INCL_END) return 1;
    }
}

/* per-sub-bucket processing: add_sequence for every superkmer, then compute_unitigs */
typedef struct {
    const uint8_t *text;
    const uint32_t *seq_colors;
    const orc_params *p;
    const orc_superkmer *recs;
    const size_t *unit_off;
    size_t nunits;
    size_t next_unit;
    pthread_mutex_t lock;
} merge_shared;

typedef struct {
    merge_shared *sh;
    unitig_vec unitigs;
    kmer_vec kmers;
} merge_job;

typedef struct {
    uint32_t entry_slot; /* kentry ordinal */
    uint32_t color;
} color_pair;

static int cmp_color_pair(const void *a, const void *b) {
    const color_pair *x = a, *y = b;
    if (x->entry_slot != y->entry_slot) return x->entry_slot < y->entry_slot ? -1 : 1;
    return x->color < y->color ? -1 : x->color > y->color;
}

static void merge_unit(merge_job *job, const orc_superkmer *recs, size_t nrec) {
    const orc_params *p = job->sh->p;
    const int k = p->k, kind = p->hash_kind;
    size_t total = 0;
    for (size_t i = 0; i < nrec; i++) total += recs[i].len - (size_t)k + 1;
    kmap m;
    kmap_init(&m, total / 2 + 16);
    uint8_t *cb = NULL;
    orc_ext_hash *hs = NULL;
    size_t cap = 0;
    color_pair *cpairs = NULL;
    size_t ncp = 0, cpcap = 0;
    u128 *packed_hi = NULL; /* k > 64: bases 64-127 of each entry, by ordinal */
    size_t hi_cap = 0;
    /* add_sequence, hashmap.rs:361-431; reads in stored orientation (rc applied) */
    for (size_t r = 0; r < nrec; r++) {
        const orc_superkmer *s = &recs[r];
        size_t L = s->len;
        if (L > cap) {
            cap = L * 2;
            cb = xrealloc(cb, cap);
            hs = xrealloc(hs, cap * sizeof(orc_ext_hash));
        }
        for (size_t i = 0; i < L; i++) {
            uint8_t c = orc_compress_base(norm_table[job->sh->text[s->start + i]]);
            if (s->rc)
                cb[L - 1 - i] = c ^ 2;
            else
                cb[i] = c;
        }
        size_t nk = orc_hash_iter(kind, cb, L, k, hs);
        size_t last = L - (size_t)k;
        for (size_t idx = 0; idx < nk; idx++) {
            int begin_ignored = (s->flags & READ_FLAG_INCL_BEGIN) == 0 && idx == 0;
            int end_ignored = (s->flags & READ_FLAG_INCL_END) == 0 && idx == last;
            int isf = orc_hash_is_forward(kind, hs[idx]);
            int created;
            kentry *e = kmap_insert(&m, orc_hash_unext(kind, hs[idx]), &created);
            if (created) {
                const okey q = pack_canonical(cb + idx, k, orc_hash_is_canonical(kind));
                e->packed = q.lo;
                e->ordinal = (uint32_t)(m.n - 1);
                if (k > 64) {
                    if (e->ordinal >= hi_cap) {
                        hi_cap = hi_cap ? hi_cap * 2 : 1024;
                        packed_hi = xrealloc(packed_hi, hi_cap * sizeof(u128));
                    }
                    packed_hi[e->ordinal] = q.hi;
                }
            }
            e->flags |= (uint8_t)(((unsigned)begin_ignored << (unsigned)!isf) | ((unsigned)end_ignored << (unsigned)isf));
            e->count += 1; /* every record has multiplicity 1 (no compaction) */
            if (p->colors) {
                if (ncp == cpcap) {
                    cpcap = cpcap ? cpcap * 2 : 1024;
                    cpairs = xrealloc(cpairs, cpcap * sizeof(color_pair));
                }
                cpairs[ncp].entry_slot = e->ordinal;
                cpairs[ncp].color = job->sh->seq_colors ? job->sh->seq_colors[s->seq_index] : 0;
                ncp++;
            }
        }
    }
    /* kmer colour subsets: sorted, deduplicated colours of all occurrences
     * (MultipleColorsManager::process_colors, crates/colors/src/managers/multiple.rs:175-214) */
    uint32_t *slot_col_off = NULL, *slot_col_n = NULL;
    uint32_t *ucolors = NULL;
    if (p->colors) {
        qsort(cpairs, ncp, sizeof(color_pair), cmp_color_pair);
        slot_col_off = xcalloc(m.n + 1, sizeof(uint32_t));
        slot_col_n = xcalloc(m.n + 1, sizeof(uint32_t));
        ucolors = xmalloc((ncp + 1) * sizeof(uint32_t));
        size_t nu = 0;
        for (size_t i = 0; i < ncp; i++) {
            if (i == 0 || cpairs[i].entry_slot != cpairs[i - 1].entry_slot) {
                slot_col_off[cpairs[i].entry_slot] = (uint32_t)nu;
            } else if (cpairs[i].color == cpairs[i - 1].color)
                continue;
            ucolors[nu++] = cpairs[i].color;
            slot_col_n[cpairs[i].entry_slot]++;
        }
    }
    for (size_t i = 0; i < m.cap; i++) {
        kentry *e = &m.e[i];
        if (!e->occupied || entry_mult(e) < (uint64_t)p->min_multiplicity) continue;
        kmer_out ko = {e->packed, entry_mult(e), 0, 0};
        if (p->colors) {
            ko.color_off = kv_push_colors(&job->kmers, ucolors + slot_col_off[e->ordinal], slot_col_n[e->ordinal]);
            ko.color_n = slot_col_n[e->ordinal];
        }
        kv_push(&job->kmers, ko, k > 64, k > 64 ? packed_hi[e->ordinal] : 0);
    }

    /* compute_unitigs, hashmap.rs:442-601; k-mers visited in read order (get_kmers,
     * hashmap.rs:76-160), which starts walks at the same k-mers for every hash kind. */
    ext_ctx ec = {p, &m};
    size_t fcap = (size_t)k * 4, bcap = (size_t)k * 4;
    uint8_t *fseq = xmalloc(fcap), *bseq = xmalloc(bcap);
    for (size_t r = 0; r < nrec; r++) {
        const orc_superkmer *s = &recs[r];
        size_t L = s->len;
        for (size_t i = 0; i < L; i++) {
            uint8_t c = orc_compress_base(norm_table[job->sh->text[s->start + i]]);
            if (s->rc)
                cb[L - 1 - i] = c ^ 2;
            else
                cb[i] = c;
        }
        size_t nk = orc_hash_iter(kind, cb, L, k, hs);
        for (size_t idx = 0; idx < nk; idx++) {
            orc_ext_hash hash = hs[idx];
            kentry *e = kmap_find(&m, orc_hash_unext(kind, hash));
            if (entry_mult(e) < (uint64_t)p->min_multiplicity || e->used) continue;
            int isf = orc_hash_is_forward(kind, hash);
            int begin_ignored, end_ignored;
            if (isf) {
                begin_ignored = e->flags == READ_FLAG_INCL_BEGIN;
                end_ignored = e->flags == READ_FLAG_INCL_END;
            } else {
                begin_ignored = e->flags == READ_FLAG_INCL_END;
                end_ignored = e->flags == READ_FLAG_INCL_BEGIN;
            }
            size_t flen = (size_t)k, blen = (size_t)k;
            for (int i = 0; i < k; i++) {
                fseq[i] = (uint8_t)DECOMP[cb[idx + (size_t)i]];
                bseq[k - 1 - i] = fseq[i];
            }
            e->used = 1;
            int fw_link, bw_link, hit_f = 0, hit_b = 0;
            if (end_ignored)
                fw_link = 1;
            else
                fw_link = try_extend(&ec, hash, &fseq, &flen, &fcap, 1, hash, &hit_f);
            if (begin_ignored)
                bw_link = 1;
            else
                bw_link = try_extend(&ec, hash, &bseq, &blen, &bcap, 0, hash, &hit_b);
            unitig_t u;
            u.len = blen + flen - (size_t)k;
            u.seq = xmalloc(u.len);
            for (size_t i = 0; i < blen; i++) u.seq[i] = bseq[blen - 1 - i];
            memcpy(u.seq + blen, fseq + k, flen - (size_t)k);
            u.fw_link = (uint8_t)fw_link;
            u.bw_link = (uint8_t)bw_link;
            u.circular = (uint8_t)(hit_f && !fw_link && !bw_link);
            ut_push(&job->unitigs, u);
        }
    }
    free(fseq);
    free(bseq);
    free(cb);
    free(hs);
    free(m.e);
    free(cpairs);
    free(packed_hi);
    free(slot_col_off);
    free(slot_col_n);
    free(ucolors);
}

static void *merge_worker(void *arg) {
    merge_job *j = arg;
    merge_shared *sh = j->sh;
    for (;;) {
        pthread_mutex_lock(&sh->lock);
        size_t u = sh->next_unit++;
        pthread_mutex_unlock(&sh->lock);
        if (u >= sh->nunits) break;
        size_t a = sh->unit_off[u], b = sh->unit_off[u + 1];
        if (b > a) merge_unit(j, sh->recs + a, b - a);
    }
    return NULL;
}

/* ---- link stage: joins partial unitigs at their shared boundary k-mers.  The result
 * is the set produced by build_final_unitigs / extend_unitigs
 * (crates/assembler_pipeline/src/extend_unitigs.rs:348-993). ---- */
static void rc_ascii(uint8_t *s, size_t n) {
    for (size_t i = 0, j = n ? n - 1 : 0; i < j; i++, j--) {
        uint8_t t = s[i];
        s[i] = s[j];
        s[j] = t;
    }
    for (size_t i = 0; i < n; i++) {
        switch (s[i]) {
        case 'A': s[i] = 'T'; break;
        case 'C': s[i] = 'G'; break;
        case 'G': s[i] = 'C'; break;
        case 'T': s[i] = 'A'; break;
        }
    }
}
/* link key of a boundary k-mer: its unextendable hash identity, i.e. the canonical packed
 * k-mer for the canonical hash families and the k-mer as read for the forward ones
 * (extend_unitigs.rs:142-147, 196-240 key the extremities by hash.to_unextendable()) */
static okey pack_ascii_key(const uint8_t *a, int k, int canonical) {
    uint8_t tmp[128];
    for (int i = 0; i < k; i++) tmp[i] = orc_compress_base(a[i]);
    return pack_canonical(tmp, k, canonical);
}

typedef struct {
    okey key;
    int32_t ends[2]; /* endpoint ids (unitig*2 + side), -1 if unused */
    uint8_t occupied;
} link_entry;

static void link_stage(unitig_vec *in, int k, int canonical, unitig_vec *out) {
    size_t n = in->n;
    /* endpoint 2i = left end (bw link), 2i+1 = right end (fw link) */
    size_t cap = 64;
    while (cap < n * 4 + 16) cap <<= 1;
    link_entry *tab = xcalloc(cap, sizeof(link_entry));
    int32_t *partner = xmalloc(n * 2 * sizeof(int32_t));
    for (size_t i = 0; i < n * 2; i++) partner[i] = -1;
    for (size_t i = 0; i < n; i++) {
        for (int side = 0; side < 2; side++) {
            unitig_t *u = &in->v[i];
            if (!(side ? u->fw_link : u->bw_link)) continue;
            const uint8_t *km = side ? u->seq + u->len - k : u->seq;
            okey key = pack_ascii_key(km, k, canonical);
            size_t h = okey_hash(key) & (cap - 1);
            while (tab[h].occupied && okey_cmp(tab[h].key, key) != 0) h = (h + 1) & (cap - 1);
            if (!tab[h].occupied) {
                tab[h].occupied = 1;
                tab[h].key = key;
                tab[h].ends[0] = (int32_t)(i * 2 + side);
                tab[h].ends[1] = -1;
            } else if (tab[h].ends[1] < 0) {
                tab[h].ends[1] = (int32_t)(i * 2 + side);
                partner[tab[h].ends[0]] = tab[h].ends[1];
                partner[tab[h].ends[1]] = tab[h].ends[0];
            }
        }
    }
    uint8_t *done = xcalloc(n ? n : 1, 1);
    /* walk chains from unitigs with a free endpoint, then the remaining cycles */
    for (int pass = 0; pass < 2; pass++) {
        for (size_t i = 0; i < n; i++) {
            if (done[i]) continue;
            int start_side = -1;
            if (pass == 0) {
                if (partner[i * 2] < 0)
                    start_side = 0; /* enter from the left: traverse forward */
                else if (partner[i * 2 + 1] < 0)
                    start_side = 1;
                else
                    continue;
            } else {
                start_side = 0;
            }
            size_t cap_s = 1024, len_s = 0;
            uint8_t *s = xmalloc(cap_s);
            size_t cur = i;
            int enter = start_side;
            int circ = 0;
            for (;;) {
                done[cur] = 1;
                unitig_t *u = &in->v[cur];
                uint8_t *tmp = xmalloc(u->len);
                memcpy(tmp, u->seq, u->len);
                if (enter == 1) rc_ascii(tmp, u->len);
                size_t skip = len_s ? (size_t)k : 0;
                if (len_s + u->len > cap_s) {
                    cap_s = (len_s + u->len) * 2;
                    s = xrealloc(s, cap_s);
                }
                memcpy(s + len_s, tmp + skip, u->len - skip);
                len_s += u->len - skip;
                free(tmp);
                int exit_ep = (int)(cur * 2 + (enter == 0 ? 1 : 0));
                int nxt = partner[exit_ep];
                if (nxt < 0) break;
                size_t nu = (size_t)nxt / 2;
                if (done[nu]) {
                    if (nu == i) circ = 1;
                    break;
                }
                cur = nu;
                enter = nxt % 2; /* entering at its left end => forward */
            }
            unitig_t o;
            if (circ) {
                /* the joined string ends with the k-mer it starts with */
                len_s -= (size_t)k;
                len_s += (size_t)k - 1;
            }
            o.seq = s;
            o.len = len_s;
            o.fw_link = o.bw_link = 0;
            o.circular = (uint8_t)circ;
            ut_push(out, o);
        }
    }
    free(done);
    free(partner);
    free(tab);
}

/* ---- canonical form of a unitig set ---- */
static int cmp_bytes(const uint8_t *a, size_t al, const uint8_t *b, size_t bl) {
    size_t n = al < bl ? al : bl;
    int c = memcmp(a, b, n);
    if (c) return c;
    return al < bl ? -1 : al > bl;
}
static uint8_t *canon_unitig(const uint8_t *seq, size_t len, int circular, int k) {
    uint8_t *best = xmalloc(len);
    memcpy(best, seq, len);
    uint8_t *r = xmalloc(len);
    memcpy(r, seq, len);
    rc_ascii(r, len);
    if (!circular || len < (size_t)k) {
        if (cmp_bytes(r, len, best, len) < 0) memcpy(best, r, len);
        free(r);
        return best;
    }
    size_t nk = len - (size_t)k + 1; /* cycle length in k-mers */
    uint8_t *cand = xmalloc(len);
    for (int o = 0; o < 2; o++) {
        const uint8_t *src = o ? r : seq;
        for (size_t rot = 0; rot < nk; rot++) {
            for (size_t i = 0; i < len; i++) cand[i] = src[(rot + i) % nk];
            if (cmp_bytes(cand, len, best, len) < 0) memcpy(best, cand, len);
        }
    }
    free(cand);
    free(r);
    return best;
}

typedef struct {
    uint8_t *s;
    size_t n;
} bstr;
static int cmp_bstr(const void *a, const void *b) {
    const bstr *x = a, *y = b;
    return cmp_bytes(x->s, x->n, y->s, y->n);
}

static size_t emit_canonical(unitig_vec *v, int k, uint8_t *out, size_t cap) {
    bstr *arr = xmalloc((v->n + 1) * sizeof(bstr));
    for (size_t i = 0; i < v->n; i++) {
        arr[i].s = canon_unitig(v->v[i].seq, v->v[i].len, v->v[i].circular, k);
        arr[i].n = v->v[i].len;
    }
    qsort(arr, v->n, sizeof(bstr), cmp_bstr);
    size_t used = 0;
    for (size_t i = 0; i < v->n; i++) {
        if (out && used + arr[i].n + 1 <= cap) {
            memcpy(out + used, arr[i].s, arr[i].n);
            out[used + arr[i].n] = '\n';
        }
        used += arr[i].n + 1;
        free(arr[i].s);
    }
    free(arr);
    return used;
}

size_t orc_canonicalize_unitigs(const uint8_t *lines, size_t len, const uint8_t *circular, size_t nlines, int k,
                                uint8_t *out, size_t cap) {
    unitig_vec v = {0, 0, 0};
    size_t p = 0, li = 0;
    while (p < len && li < nlines) {
        const uint8_t *nl = memchr(lines + p, '\n', len - p);
        size_t e = nl ? (size_t)(nl - lines) : len;
        unitig_t u;
        u.seq = (uint8_t *)(lines + p);
        u.len = e - p;
        u.circular = circular ? circular[li] : 0;
        u.fw_link = u.bw_link = 0;
        ut_push(&v, u);
        p = e + 1;
        li++;
    }
    size_t r = emit_canonical(&v, k, out, cap);
    free(v.v);
    return r;
}

/* ---- full build ---- */
struct orc_build_result {
    int k;
    kmer_out *kmers;
    u128 *kmers_hi; /* k > 64: bases 64-127 of each k-mer */
    size_t nkmers;
    uint32_t *colors;
    size_t ncolors;
    unitig_vec final_unitigs;
    size_t partial_count;
};

static int cmp_kmer_out(const void *a, const void *b) {
    const kmer_out *x = a, *y = b;
    return x->packed < y->packed ? -1 : x->packed > y->packed;
}
/* k > 64: the k-mers sorted by (lo, hi) through an index */
typedef struct {
    u128 lo, hi;
    size_t i;
} wide_ref;
static int cmp_wide_ref(const void *a, const void *b) {
    const wide_ref *x = a, *y = b;
    if (x->lo != y->lo) return x->lo < y->lo ? -1 : 1;
    if (x->hi != y->hi) return x->hi < y->hi ? -1 : 1;
    return 0;
}

orc_build_result *orc_build(const uint8_t *text, const uint64_t *seq_off, const uint64_t *seq_len,
                            const uint32_t *seq_colors, size_t nseq, const orc_params *p) {
    /* packed k-mers up to 128 bases; above 64 only the Rabin-Karp families key them
     * (crates/api/src/utils.rs:10-69: sequence hashes stop at k = 64) */
    if (p->k - p->m < 2 || p->k > 128) return NULL;
    if (p->k > 64 && p->hash_kind != ORC_H_CN_RK128 && p->hash_kind != ORC_H_FW_RK128) return NULL;
    orc_hash_init_k(p->hash_kind, p->k);
    sk_vec sk = bucketize_vec(text, seq_off, seq_len, nseq, p);
    /* group by sub-bucket (bucket, second_bucket): counting sort */
    size_t nb = ((size_t)1 << p->bucket_bits) + 1, ns = (size_t)1 << p->second_bits;
    size_t nunits = nb * ns;
    size_t *cnt = xcalloc(nunits + 1, sizeof(size_t));
    for (size_t i = 0; i < sk.n; i++) cnt[(size_t)sk.v[i].bucket * ns + sk.v[i].second_bucket + 1]++;
    for (size_t u = 0; u < nunits; u++) cnt[u + 1] += cnt[u];
    size_t *cur = xmalloc((nunits + 1) * sizeof(size_t));
    memcpy(cur, cnt, (nunits + 1) * sizeof(size_t));
    orc_superkmer *sorted = xmalloc((sk.n + 1) * sizeof(orc_superkmer));
    for (size_t i = 0; i < sk.n; i++) sorted[cur[(size_t)sk.v[i].bucket * ns + sk.v[i].second_bucket]++] = sk.v[i];
    free(cur);
    free(sk.v);

    merge_shared sh;
    sh.text = text;
    sh.seq_colors = seq_colors;
    sh.p = p;
    sh.recs = sorted;
    sh.unit_off = cnt;
    sh.nunits = nunits;
    sh.next_unit = 0;
    pthread_mutex_init(&sh.lock, NULL);
    int nt = p->threads > 0 ? p->threads : 1;
    merge_job *jobs = xcalloc((size_t)nt, sizeof(merge_job));
    pthread_t *th = xcalloc((size_t)nt, sizeof(pthread_t));
    for (int t = 0; t < nt; t++) {
        jobs[t].sh = &sh;
        if (nt > 1)
            pthread_create(&th[t], NULL, merge_worker, &jobs[t]);
        else
            merge_worker(&jobs[t]);
    }
    unitig_vec partial = {0, 0, 0};
    kmer_vec kv = {0, 0, 0, 0, 0, 0, 0};
    for (int t = 0; t < nt; t++) {
        if (nt > 1) pthread_join(th[t], NULL);
        for (size_t i = 0; i < jobs[t].unitigs.n; i++) ut_push(&partial, jobs[t].unitigs.v[i]);
        for (size_t i = 0; i < jobs[t].kmers.n; i++) {
            kmer_out ko = jobs[t].kmers.v[i];
            if (ko.color_n) ko.color_off = kv_push_colors(&kv, jobs[t].kmers.colors + ko.color_off, ko.color_n);
            kv_push(&kv, ko, p->k > 64, p->k > 64 ? jobs[t].kmers.hi[i] : 0);
        }
        free(jobs[t].unitigs.v);
        free(jobs[t].kmers.v);
        free(jobs[t].kmers.hi);
        free(jobs[t].kmers.colors);
    }
    pthread_mutex_destroy(&sh.lock);
    free(jobs);
    free(th);
    free(sorted);
    free(cnt);

    orc_build_result *res = xcalloc(1, sizeof(orc_build_result));
    res->k = p->k;
    /* k-mers at a sub-bucket boundary are counted in both sub-buckets with the same
     * multiplicity: keep one copy. */
    if (p->k > 64) {
        wide_ref *ref = xmalloc((kv.n + 1) * sizeof(wide_ref));
        for (size_t i = 0; i < kv.n; i++) ref[i] = (wide_ref){kv.v[i].packed, kv.hi[i], i};
        qsort(ref, kv.n, sizeof(wide_ref), cmp_wide_ref);
        kmer_out *sv = xmalloc((kv.n + 1) * sizeof(kmer_out));
        u128 *sh = xmalloc((kv.n + 1) * sizeof(u128));
        for (size_t i = 0; i < kv.n; i++) {
            sv[i] = kv.v[ref[i].i];
            sh[i] = ref[i].hi;
        }
        free(ref);
        free(kv.v);
        free(kv.hi);
        kv.v = sv;
        kv.hi = sh;
    } else {
        qsort(kv.v, kv.n, sizeof(kmer_out), cmp_kmer_out);
    }
    size_t w = 0;
    for (size_t i = 0; i < kv.n; i++) {
        if (w > 0 && kv.v[w - 1].packed == kv.v[i].packed && (p->k <= 64 || kv.hi[w - 1] == kv.hi[i])) {
            if (kv.v[w - 1].mult != kv.v[i].mult) kv.v[w - 1].mult = UINT64_MAX; /* inconsistency marker */
            continue;
        }
        if (p->k > 64) kv.hi[w] = kv.hi[i];
        kv.v[w++] = kv.v[i];
    }
    res->kmers = kv.v;
    res->kmers_hi = kv.hi;
    res->nkmers = w;
    res->colors = kv.colors;
    res->ncolors = kv.ncol;
    res->partial_count = partial.n;
    unitig_vec fin = {0, 0, 0};
    unitig_vec linked = {0, 0, 0};
    for (size_t i = 0; i < partial.n; i++) {
        if (partial.v[i].fw_link || partial.v[i].bw_link)
            ut_push(&linked, partial.v[i]);
        else
            ut_push(&fin, partial.v[i]);
    }
    link_stage(&linked, p->k, orc_hash_is_canonical(p->hash_kind), &fin);
    for (size_t i = 0; i < linked.n; i++) free(linked.v[i].seq);
    free(linked.v);
    free(partial.v);
    res->final_unitigs = fin;
    return res;
}

void orc_build_free(orc_build_result *r) {
    if (!r) return;
    for (size_t i = 0; i < r->final_unitigs.n; i++) free(r->final_unitigs.v[i].seq);
    free(r->final_unitigs.v);
    free(r->kmers);
    free(r->kmers_hi);
    free(r->colors);
    free(r);
}

size_t orc_build_kmers(const orc_build_result *r, uint64_t *lo, uint64_t *hi, uint64_t *mult, size_t cap) {
    if (lo)
        for (size_t i = 0; i < r->nkmers && i < cap; i++) {
            lo[i] = (uint64_t)r->kmers[i].packed;
            hi[i] = (uint64_t)(r->kmers[i].packed >> 64);
            mult[i] = r->kmers[i].mult;
        }
    return r->nkmers;
}

/* the surviving k-mers as four 64-bit words each (bases 0-31, 32-63, 64-95, 96-127) */
size_t orc_build_kmers_wide(const orc_build_result *r, uint64_t *words, uint64_t *mult, size_t cap) {
    if (words)
        for (size_t i = 0; i < r->nkmers && i < cap; i++) {
            const u128 lo = r->kmers[i].packed, hi = r->kmers_hi ? r->kmers_hi[i] : 0;
            words[4 * i] = (uint64_t)lo;
            words[4 * i + 1] = (uint64_t)(lo >> 64);
            words[4 * i + 2] = (uint64_t)hi;
            words[4 * i + 3] = (uint64_t)(hi >> 64);
            mult[i] = r->kmers[i].mult;
        }
    return r->nkmers;
}

size_t orc_build_kmer_colors(const orc_build_result *r, uint64_t *off, uint32_t *colors, size_t cap) {
    size_t used = 0;
    for (size_t i = 0; i < r->nkmers; i++) {
        if (off) off[i] = used;
        for (uint32_t j = 0; j < r->kmers[i].color_n; j++) {
            if (colors && used < cap) colors[used] = r->colors[r->kmers[i].color_off + j];
            used++;
        }
    }
    if (off) off[r->nkmers] = used;
    return used;
}

size_t orc_build_unitigs(const orc_build_result *r, uint8_t *buf, size_t cap) {
    unitig_vec v = r->final_unitigs;
    return emit_canonical(&v, r->k, buf, cap);
}

size_t orc_build_partial_count(const orc_build_result *r) { return r->partial_count; }

/* ======================================================================
 * Query: the querier counts every query k-mer occurrence (split at N) whose canonical
 * merging hash is a graph k-mer, per colour subset, then sums per colour
 * (crates/querier/src/pipeline/querier_minimizer_bucketing.rs:182-230,
 *  parallel_kmers_query.rs:362-471, counters_sorting.rs:106-273,
 *  colored_query_output.rs:264-309; query_kmers = len - k + 1, lib.rs:138-150).
 * ====================================================================== */
typedef struct {
    u128 key;
    uint32_t idx;
    uint8_t occupied;
} qentry;

int orc_query(const uint64_t *graph_lo, const uint64_t *graph_hi, size_t ngraph, const uint64_t *gc_off,
              const uint32_t *gc_colors, uint32_t ncolors, const uint8_t *qtext, const uint64_t *q_off,
              const uint64_t *q_len, size_t nq, int k, int hash_kind, uint64_t *out_matched, uint64_t *out_qkmers,
              uint64_t *out_percolor) {
    pthread_once(&norm_once, norm_init);
    (void)hash_kind;
    size_t cap = 64;
    while (cap < ngraph * 2 + 16) cap <<= 1;
    qentry *tab = xcalloc(cap, sizeof(qentry));
    for (size_t i = 0; i < ngraph; i++) {
        u128 key = ((u128)graph_hi[i] << 64) | graph_lo[i];
        size_t h = khash(key) & (cap - 1);
        while (tab[h].occupied && tab[h].key != key) h = (h + 1) & (cap - 1);
        tab[h].occupied = 1;
        tab[h].key = key;
        tab[h].idx = (uint32_t)i;
    }
    uint8_t *cb = NULL;
    size_t cbcap = 0;
    for (size_t q = 0; q < nq; q++) {
        const uint8_t *s = qtext + q_off[q];
        size_t L = q_len[q];
        out_qkmers[q] = L >= (size_t)k ? L - (size_t)k + 1 : 0;
        out_matched[q] = 0;
        if (out_percolor) memset(out_percolor + q * ncolors, 0, ncolors * sizeof(uint64_t));
        if (L > cbcap) {
            cbcap = L * 2;
            cb = xrealloc(cb, cbcap);
        }
        size_t run = 0;
        for (size_t i = 0; i < L; i++) {
            uint8_t c = norm_table[s[i]];
            if (c == 'N') {
                run = 0;
                continue;
            }
            cb[i] = orc_compress_base(c);
            run++;
            if (run >= (size_t)k) {
                u128 key = pack_canonical(cb + i + 1 - (size_t)k, k, 1).lo;
                size_t h = khash(key) & (cap - 1);
                while (tab[h].occupied && tab[h].key != key) h = (h + 1) & (cap - 1);
                if (tab[h].occupied) {
                    out_matched[q]++;
                    if (out_percolor && gc_off) {
                        uint32_t gi = tab[h].idx;
                        for (uint64_t j = gc_off[gi]; j < gc_off[gi + 1]; j++) out_percolor[q * ncolors + gc_colors[j]]++;
                    }
                }
            }
        }
    }
    free(cb);
    free(tab);
    return 0;
}
