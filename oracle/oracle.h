/*
 * ORACLE (test infrastructure only).  A CPU restatement of GGCAT's build hot path
 * (minimizer bucketing -> per-bucket k-mer merge -> link) and of its query lookup.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and
 * only as the checker or as the timed CPU baseline.  The product never links it.
 *
 * Parity status: the hash families and the sliding-window minimum are pinned by a
 * port of the reference's own property tests (crates/hashes/src/lib.rs:265-454,
 * crates/hashes/src/rolling/minqueue_testing.rs:335-370) and the reference's
 * known-answer 2-bit/rc packing vector (crates/io/src/compressed_read.rs:1011-1023).
 * End-to-end outputs are NOT pinned against reference runs: the reference is Rust
 * and cannot be compiled in this environment (no cargo/rustc, empty submodules).
 */
#ifndef GGCAT_ORACLE_H
#define GGCAT_ORACLE_H
#include "oracle_hashes.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One superkmer record, in the semantic form of PushSequenceInfo
 * (crates/minimizer_bucketing/src/lib.rs:101-110).  The bases are
 * text[start .. start+len) of the input text; when rc != 0 the reference stores
 * their reverse complement (flags then refer to the stored orientation). */
typedef struct {
    uint64_t start;
    uint32_t len;
    uint16_t bucket;
    uint16_t second_bucket;
    uint16_t minimizer_pos;
    uint8_t rc;
    uint8_t flags;
    uint32_t seq_index;
    uint64_t minimizer; /* minimizer value including the unique flag in bit 0 */
} orc_superkmer;

typedef struct {
    int k, m;
    int bucket_bits;      /* first-level buckets = 2^bucket_bits (+1 duplicates bucket) */
    int second_bits;      /* second-level (sub-bucket) bits */
    int canonical;        /* !forward_only */
    int hash_kind;        /* ORC_H_* merging hash */
    int min_multiplicity;
    int threads;
    int colors;           /* colour per input sequence (seq_colors) */
} orc_params;

/* ---- sliding-window minimum, exact restatement of BatchMinQueue ---- */
typedef struct { uint64_t v; uint32_t index; uint8_t is_forward; uint8_t pad[3]; } orc_mq_item;
/* Returns number of split records written (position, value). last flag in out_last. */
size_t orc_minqueue_splits(size_t size, const orc_mq_item *items, size_t n, size_t skip_b, size_t skip_e,
                           int dup_check, size_t *out_pos, orc_mq_item *out_val, uint8_t *out_last, size_t cap);
/* Plain per-window minima (get_minimizers): value per window. Returns window count. */
size_t orc_minqueue_minimizers(size_t size, const orc_mq_item *items, size_t n, size_t skip_e, int dup_check,
                               orc_mq_item *out, size_t cap);

/* ---- minimizer bucketing ---- */
/* text: concatenated sequences; seq_off/seq_len describe each input sequence (already
 * cut into pieces by the FASTA reader).  Returns the number of superkmers; writes at
 * most cap records. */
size_t orc_bucketize(const uint8_t *text, const uint64_t *seq_off, const uint64_t *seq_len, size_t nseq,
                     const orc_params *p, orc_superkmer *out, size_t cap);

/* ---- FASTA reader with the 4 MiB + (k-1) copyback chunking ---- */
/* Parses a FASTA buffer exactly like SequencesReader::process_fasta with read buffers of
 * 4 MiB.  Writes the normalised sequence pieces into out_text (capacity text_cap) and
 * (offset, len) pairs into out_off/out_len.  Returns the number of pieces. */
size_t orc_fasta_parse(const uint8_t *file, size_t file_len, long copyback, uint8_t *out_text, size_t text_cap,
                       uint64_t *out_off, uint64_t *out_len, size_t cap, size_t *out_text_used);

/* ---- k-mer merge + link ---- */
typedef struct orc_build_result orc_build_result;
orc_build_result *orc_build(const uint8_t *text, const uint64_t *seq_off, const uint64_t *seq_len,
                            const uint32_t *seq_colors, size_t nseq, const orc_params *p);
void orc_build_free(orc_build_result *r);
/* surviving canonical k-mers: 2-bit packed canonical k-mer (lo, hi words, seq-hash layout)
 * and multiplicity, sorted by (hi, lo). */
size_t orc_build_kmers(const orc_build_result *r, uint64_t *lo, uint64_t *hi, uint64_t *mult, size_t cap);
/* the same with four 64-bit words per k-mer (k <= 128: bases 0-31, 32-63, 64-95, 96-127) */
size_t orc_build_kmers_wide(const orc_build_result *r, uint64_t *words, uint64_t *mult, size_t cap);
/* colour subset of each surviving k-mer, same order: offsets into a flat colour list */
size_t orc_build_kmer_colors(const orc_build_result *r, uint64_t *off, uint32_t *colors, size_t cap);
/* canonical, sorted maximal-unitig set as '\n'-terminated ASCII lines; returns bytes. */
size_t orc_build_unitigs(const orc_build_result *r, uint8_t *buf, size_t cap);
/* partial (per sub-bucket) unitig count before linking, for diagnostics */
size_t orc_build_partial_count(const orc_build_result *r);

/* Canonicalise a unitig list given as '\n'-terminated lines with a circular flag per line;
 * returns bytes written (sorted, '\n'-terminated). */
size_t orc_canonicalize_unitigs(const uint8_t *lines, size_t len, const uint8_t *circular, size_t nlines, int k,
                                uint8_t *out, size_t cap);

/* ---- query ---- */
/* For each query sequence, count its k-mers (split at N) present in the graph k-mer set;
 * graph_colors (optional) gives the colour-subset of each graph k-mer as offsets into a
 * flat colour list; then per_colour counts are written (nq x ncolors). */
int orc_query(const uint64_t *graph_lo, const uint64_t *graph_hi, size_t ngraph, const uint64_t *gc_off,
              const uint32_t *gc_colors, uint32_t ncolors, const uint8_t *qtext, const uint64_t *q_off,
              const uint64_t *q_len, size_t nq, int k, int hash_kind, uint64_t *out_matched, uint64_t *out_qkmers,
              uint64_t *out_percolor);

#ifdef __cplusplus
}
#endif
#endif
