/*
 * ggcat_gb300 — C ABI of the GB300 (sm_103a) implementation of GGCAT's build hot path
 * (minimizer bucketing -> per-bucket k-mer merge) and graph query lookup.
 *
 * Plain C types only (pointers, sizes, status codes).  Every call returns 0 on success
 * or a negative GGCAT_GPU_E* code; ggcat_gpu_last_error() describes the last failure.
 * Calls on one context are not thread-safe; use one context per host thread.
 *
 * Device pointers are marked d_, host pointers h_.  `stream` is a cudaStream_t (NULL =
 * the legacy default stream).  Functions that return results to the host synchronise
 * the stream.
 */
#ifndef GGCAT_GB300_H
#define GGCAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GGCAT_GPU_OK 0
#define GGCAT_GPU_EINVAL -1      /* bad argument */
#define GGCAT_GPU_ECUDA -2       /* CUDA runtime error */
#define GGCAT_GPU_ENOMEM -3      /* device allocation failed */
#define GGCAT_GPU_EDEVICE -4     /* a kernel reported an internal error (see last_error) */
#define GGCAT_GPU_EUNSUPPORTED -5 /* parameters outside what this build supports */
#define GGCAT_GPU_EIO -6         /* file read/write error */
#define GGCAT_GPU_ETOOLARGE -7   /* size beyond a fixed maximum of the entry point */

/* Merging-hash kinds (crates/api/src/utils.rs:10-69). */
#define GGCAT_HASH_SEQHASH 1
#define GGCAT_HASH_RABIN_KARP128 4

/* Merge scheduling (both give identical results). */
#define GGCAT_MERGE_BATCHED 0    /* persistent kernel over a device work queue */
#define GGCAT_MERGE_PER_BUCKET 1 /* plain form: one launch group per bucket */

typedef struct ggcat_gpu_ctx ggcat_gpu_ctx;

typedef struct {
    int32_t k;                /* k-mer length <= 127, odd or even: merge tables keyed by the canonical packed
                                 k-mer in one word (k <= 32), two (k <= 64) or four (k > 64, global-memory
                                 tables only; the Rabin-Karp hash_kind, as the reference requires above 64;
                                 colours and queries stop at 64); forward-only merges exclude
                                 k = 32 and 64 (their all-G k-mer is the tables' empty key) */
    int32_t m;                /* minimizer length, 2 <= m <= 32, k - m >= 2 */
    int32_t bucket_bits;      /* first-level buckets = 2^bucket_bits (+1 duplicates bucket) */
    int32_t second_bits;      /* second-level bucket bits reported in superkmer records */
    int32_t min_multiplicity; /* keep k-mers with multiplicity >= this */
    int32_t hash_kind;        /* GGCAT_HASH_* */
    int32_t forward_only;     /* 1 = do not canonicalise (rc never applied) */
    int32_t merge_mode;       /* GGCAT_MERGE_* */
    int32_t unit_target;      /* target k-mer instances per merge unit (0 = auto; -1 = auto without the
                                 shared-memory attempt for sub-buckets above the S-unit size) */
    int32_t keep_kmers;       /* 1 = also output the surviving k-mers and multiplicities */
    /* tuning knobs (0 = default; ggcat_gpu_autotune chooses them), results are identical for any value */
    int32_t subbin_bytes;     /* text bytes per sub-bin: sets the sub-bin digit width of the bucket store
                                 partition (default 1024, 4096 for k > 32) */
    int32_t table_load_pct;   /* largest load of a global-memory merge table, percent (default 80, 90 for
                                 k > 32) */
    int32_t small_limit;      /* largest sub-bin, in k-mer instances, merged in a shared-memory S unit
                                 (default and maximum 3200, 1600 for k > 32) */
    int32_t copy_pieces;      /* pieces of the host text copy of ggcat_gpu_build_text from pinned memory,
                                 each packed and bucketized on its own stream while the next ones are in
                                 flight (0 = auto: up to 16, each at least a wave of bucketize blocks;
                                 1 = one copy; at most 16) */
    int32_t spill_mb;         /* device memory for the bucket store, MiB (0 = no limit).  When the superkmer
                                 records would exceed it, or do not fit the device's free memory, the text is
                                 bucketized in pieces whose partitioned records go to pinned host memory, and
                                 the merge runs bucket range by bucket range, each range's records copied back
                                 to the device (the reference's bucket files spilled from its in-memory
                                 store, crates/minimizer_bucketing/src/lib.rs:569-586).  Results are the same. */
    /* per bucket-size-class knobs (0 = default), results identical for any value */
    int32_t small_batch;      /* superkmer records per insert batch of a warp in S units, 1-32 (default 16,
                                 8 for k > 32) */
    int32_t wide_batch;       /* the same in W units, 1-32 (default 16, 8 for k > 32) */
    int32_t wide_limit;       /* largest sub-bin, in k-mer instances, tried in a shared-memory W unit before
                                 a global-memory table (default and maximum 65536; k > 32: default 8192,
                                 maximum 16384) */
} ggcat_gpu_params;

/* One superkmer in the semantic form of PushSequenceInfo
 * (crates/minimizer_bucketing/src/lib.rs:101-110): bases text[start, start+len);
 * when rc != 0 the reference stores their reverse complement and flags refer to the
 * stored orientation (bit0 = begin included, bit1 = end included). */
typedef struct {
    uint64_t start;
    uint32_t len;
    uint16_t bucket;
    uint16_t second_bucket;
    uint16_t minimizer_pos;
    uint8_t rc;
    uint8_t flags;
} ggcat_gpu_superkmer;

typedef struct {
    uint64_t text_bytes;
    uint64_t superkmers;
    uint64_t kmer_instances;
    uint64_t merge_units_small;
    uint64_t merge_units_large;
    uint64_t partial_unitigs;
    uint64_t partial_bases;
    uint64_t surviving_kmers;   /* counted once per (k-mer, sub-bucket) */
    uint64_t final_unitigs;
    double ms_pack, ms_bucketize, ms_merge, ms_link; /* device times (events) and host link time */
    uint64_t distinct_kmers;    /* table entries summed over merge units */
    uint64_t merge_units_spilled; /* shared-memory attempts that moved to a global-memory table */
    uint64_t merge_units_ext_global; /* units ranked in global-memory scratch (many survivors) */
    uint64_t merge_units_walk;  /* units extended by per-thread walks (grid-wide tier, fallback) */
    uint64_t merge_graph_captures; /* captures of the batched merge phase as a CUDA graph (context lifetime) */
    uint64_t merge_graph_replays;  /* launches of that graph (context lifetime) */
    uint64_t spill_pieces;      /* bucketize pieces whose records went to host memory (0: resident store) */
    uint64_t spill_ranges;      /* bucket ranges merged one after another from the host store */
    uint64_t spill_bytes;       /* record bytes held in host memory */
    double ms_tier[4];          /* device time of each bucket-size class of the batched merge: S units,
                                   W units, M units (global tables), L units (grid-wide kernels) */
    uint64_t colors_collected;  /* 1 when the last ggcat_gpu_colors used the colours collected by the merge */
} ggcat_gpu_stats;

/* ---- context ---- */
/* Creates a context on `device`.  All device memory of the context is owned by it. */
int ggcat_gpu_create(int device, ggcat_gpu_ctx **out);
void ggcat_gpu_destroy(ggcat_gpu_ctx *ctx);
const char *ggcat_gpu_last_error(const ggcat_gpu_ctx *ctx);
/* Number of kernels this context launched since creation (all entry points). */
uint64_t ggcat_gpu_kernel_launches(const ggcat_gpu_ctx *ctx);

/* ---- build hot path, device-resident input ----
 * Input "text": all sequences concatenated, each followed by at least one byte that is
 * not ACGTacgt (a separator, e.g. '\n'); any such byte splits k-mers like an N
 * (SequencesSplitter, crates/minimizer_bucketing/src/sequences_splitter.rs:15-40).
 * Long FASTA records must already be cut into pieces by the FASTA reader
 * (ggcat_gpu_fasta_parse does this exactly like the reference). */

/* Replaces assembler_minimizer_bucketing::minimizer_bucketing
 * (crates/assembler_minimizer_bucketing/src/lib.rs:279-340): 2-bit packing, nt-hash
 * m-mers, (k-1)-mer window minimizers with the duplicate flag, superkmer splitting,
 * bucket ids, and a device radix partition of the superkmer records (the bucket store,
 * kept in HBM).  *n_superkmers receives the record count. */
int ggcat_gpu_bucketize(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len, const ggcat_gpu_params *p,
                        void *stream, uint64_t *n_superkmers);

/* Copies the superkmer records of the last bucketize (ordered by bucket, then by an
 * internal sub-bucket; order inside a sub-bucket is unspecified) to the host. */
int ggcat_gpu_superkmers_copy(ggcat_gpu_ctx *ctx, ggcat_gpu_superkmer *h_out, uint64_t cap, uint64_t *n);

/* Replaces assembler_kmers_merge::kmers_merge (crates/assembler_kmers_merge/src/lib.rs:159-284):
 * per sub-bucket canonical k-mer counting with the MapEntry flag/halving rule, the
 * min-multiplicity filter and within-sub-bucket unitig extension.  Produces partial
 * unitigs (with open-end link flags) for the link stage.  Runs on the bucket store of
 * the last ggcat_gpu_bucketize. */
int ggcat_gpu_merge(ggcat_gpu_ctx *ctx, const ggcat_gpu_params *p, void *stream);

/* Chooses the tuning knobs of p by measurement on the first sample_bytes of d_text (all of it
 * when 0), coordinate descent with two runs per candidate: first the sub-bin digit width
 * (subbin_bytes) by the device time of bucketize + merge, then per bucket-size class, each knob
 * by the device time (ggcat_gpu_stats.ms_tier) of the classes it moves work between: S units
 * (unit_target, small_limit, small_batch), W units (wide_batch, wide_limit), M and L units
 * (table_load_pct).  *best receives p with the chosen knobs, *default_ms / *best_ms the device
 * times of p as given and of *best.  Stands where
 * the reference sizes its buckets by heuristics (compute_stats_from_input_blocks,
 * crates/io/src/lib.rs:67-140; second-level bucket count, crates/assembler/src/lib.rs:155).
 * Leaves the bucket store of its last trial; outputs do not depend on the knobs. */
int ggcat_gpu_autotune(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t text_len, const ggcat_gpu_params *p,
                       uint64_t sample_bytes, void *stream, ggcat_gpu_params *best, double *default_ms,
                       double *best_ms);

/* Partial unitigs of the last merge: concatenated ASCII bases, and per unitig
 * (offset, length, flags) with flags bit0 = backward link, bit1 = forward link,
 * bit2 = circular.  Pass NULL buffers to query the sizes. */
int ggcat_gpu_partial_unitigs_copy(ggcat_gpu_ctx *ctx, uint8_t *h_bases, uint64_t bases_cap, uint64_t *h_off,
                                   uint32_t *h_len, uint8_t *h_flags, uint64_t cap, uint64_t *n_unitigs,
                                   uint64_t *n_bases);

/* Surviving k-mers of the last merge (needs keep_kmers = 1): canonical 2-bit packed
 * k-mer (seq-hash layout, base i at bits 2i) and multiplicity.  For k > 32 every k-mer takes
 * two words of h_kmers (low, high), so h_kmers holds 2 * cap words.  A k-mer on a sub-bucket
 * boundary is reported once per sub-bucket.  Pass NULL to query the count. */
int ggcat_gpu_kmers_copy(ggcat_gpu_ctx *ctx, uint64_t *h_kmers, uint64_t *h_mult, uint64_t cap, uint64_t *n);

/* Host link stage (crates/assembler_pipeline/src/extend_unitigs.rs:348-993 semantics):
 * joins the partial unitigs of the last merge at their link k-mers into the maximal
 * unitigs.  Output as for ggcat_gpu_partial_unitigs_copy (flags bit2 = circular). */
int ggcat_gpu_link(ggcat_gpu_ctx *ctx, int k);
int ggcat_gpu_unitigs_copy(ggcat_gpu_ctx *ctx, uint8_t *h_bases, uint64_t bases_cap, uint64_t *h_off,
                           uint32_t *h_len, uint8_t *h_flags, uint64_t cap, uint64_t *n_unitigs, uint64_t *n_bases);

/* Statistics of the last bucketize/merge/link. */
int ggcat_gpu_get_stats(const ggcat_gpu_ctx *ctx, ggcat_gpu_stats *out);

/* ---- end to end, host input ----
 * Copies the host text to the device (pinned staging, cudaMemcpyAsync), runs bucketize
 * + merge on `stream`, and copies the partial unitigs back to host memory owned by the
 * context (read them with ggcat_gpu_partial_unitigs_copy, or link them with
 * ggcat_gpu_link).  This is the call the reference's kmers pipeline would make. */
int ggcat_gpu_build_text(ggcat_gpu_ctx *ctx, const uint8_t *h_text, uint64_t text_len, const ggcat_gpu_params *p,
                         void *stream);

/* FASTA parsing with the reference's 4 MiB + (k-1) copyback record chunking
 * (SequencesReader::process_fasta, crates/io/src/sequences_reader.rs:106-182).
 * Produces the device text layout (pieces separated by '\n').  Pass h_text = NULL to
 * query the needed capacity. */
int ggcat_gpu_fasta_parse(const uint8_t *h_file, uint64_t file_len, int64_t copyback, uint8_t *h_text,
                          uint64_t text_cap, uint64_t *text_len, uint64_t *n_pieces);

/* FASTQ parsing (SequencesReader::process_fastq, crates/io/src/sequences_reader.rs:183-241):
 * four-line records, one piece per record (never cut), the same text layout. */
int ggcat_gpu_fastq_parse(const uint8_t *h_file, uint64_t file_len, uint8_t *h_text, uint64_t text_cap,
                          uint64_t *text_len, uint64_t *n_records);

/* One input file the way the reference's SequencesReader reads it
 * (process_file_extended, sequences_reader.rs:56-104; LinesReader::read_binary_file,
 * crates/io/src/lines_reader.rs:60-143): FASTA (fa, fasta, fna, ffn) or FASTQ (fq, fastq)
 * by the extension chain, decompressed by the last extension (gz, lz4, bz2, xz, zst/zstd;
 * the system's libz / liblz4 / libbz2 / liblzma / libzstd, opened at run time).  FASTA
 * records are cut with `copyback` (< 0: whole records).  h_text = NULL queries the size; err
 * (optional) receives the reason of a failure (GGCAT_GPU_EUNSUPPORTED: unknown file type or
 * missing decompressor; GGCAT_GPU_EIO: unreadable or corrupt file). */
int ggcat_gpu_read_sequences_file(const char *path, int64_t copyback, uint8_t *h_text, uint64_t text_cap,
                                  uint64_t *text_len, uint64_t *n_pieces, char *err, uint64_t err_cap);

/* Several input files read like ggcat_gpu_read_sequences_file on up to `threads` host
 * threads (the reference's reader threads) and concatenated in input order: the text of
 * ggcat_gpu_build_from_files.  h_text = NULL queries the size. */
int ggcat_gpu_read_sequences_files(const char *const *paths, uint64_t n, int64_t copyback, int threads,
                                   uint8_t *h_text, uint64_t text_cap, uint64_t *text_len, char *err,
                                   uint64_t err_cap);

/* Spectrum-preserving string sets over n unitigs bases[off[i], off[i] + len[i]) (ACGT,
 * len >= k, 3 <= k <= 127): the matchtigs family of ExtraElaboration (crates/api/src/lib.rs:101-116;
 * compute_matchtigs_thread, crates/assembler_pipeline/src/compute_matchtigs.rs:380-537, which
 * runs the third-party matchtigs crate 2.1.x; the published algorithms are restated here):
 *   GGCAT_GPU_TIGS_EULERTIGS: the minimum number of strings with every k-mer once (per
 *     connected component max(1, sum of binode imbalances / 2));
 *   GGCAT_GPU_TIGS_PATHTIGS: a greedy walk cover, every k-mer once;
 *   GGCAT_GPU_TIGS_GREEDY_MATCHTIGS: eulertigs whose walks are first joined, cheapest first,
 *     through at most k-2 repeated k-mers when that is shorter than a new string.
 * Strings are walks of unitigs overlapping by k-1 bases (a join of w repeated k-mers by
 * k-1-w).  Output: out_bases[out_off[i], out_off[i] + out_len[i]) for i < *n_out, *bases_out
 * bytes in all; Σ len bytes and n entries always suffice.  NULL outputs query the sizes. */
#define GGCAT_GPU_TIGS_GREEDY_MATCHTIGS 2
#define GGCAT_GPU_TIGS_EULERTIGS 3
#define GGCAT_GPU_TIGS_PATHTIGS 4
int ggcat_gpu_compute_tigs(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k, int mode,
                           uint8_t *out_bases, uint64_t bases_cap, uint64_t *out_off, uint64_t *out_len,
                           uint64_t n_cap, uint64_t *n_out, uint64_t *bases_out);

/* Maximal-unitig links (build_maximal_unitigs_links,
 * crates/assembler_pipeline/src/maximal_unitig_links.rs:55-417) of n unitigs
 * bases[off[i], off[i] + len[i]) (ACGT, len >= k, k <= 127): list 2i = links from unitig i's
 * end, list 2i + 1 = from its beginning, entries [list_off[l], list_off[l + 1]) (list_off:
 * 2n + 1 entries).  Per link: the other unitig, the start of the shared (k-1)-mer in it, flags
 * bit 0 = flip_current, bit 1 = flip_other.  Pass other = NULL to query *n_links. */
int ggcat_gpu_unitig_links(const uint8_t *bases, const uint64_t *off, const uint64_t *len, uint64_t n, int k,
                           uint64_t *list_off, uint64_t *other, uint64_t *overlap, uint8_t *flags, uint64_t cap,
                           uint64_t *n_links);

/* Rewrites a FASTA of unitigs (">i LN:i:len" records in index order, as ggcat_gpu_build_from_files
 * writes them) as FASTA with the links in the headers (" L:+:j:-", gfa_version = 0,
 * unitig_links = 1) or as GFA v1 / v2 (gfa_version 1 / 2; L / E lines when unitig_links): the
 * output of ExtraElaboration::UnitigLinks and of gfa_output_version in
 * GGCATInstance::build_graph (crates/api/src/lib.rs:217-322; writers in
 * crates/sequence_output/src/structured_sequences/{fasta,gfa}.rs). */
int ggcat_gpu_write_graph(const char *unitigs_fasta, const char *output_file, int k, int unitig_links,
                          int gfa_version, char *err, uint64_t err_cap);

/* ggcat_dump_unitigs (crates/capi/src/lib.rs:407-452; GGCATInstance::dump_unitigs,
 * crates/api/src/lib.rs:434-477), on the calling thread.  Uncoloured (colors = 0): fn once per
 * piece of the graph FASTA, read like the reference's reader with a k-1 copyback, with colors =
 * NULL, n_colors = 0, same_colors = 0 (the reference's uncoloured branch hands the function the
 * record's identifier buffer, which its reader leaves empty there; this hands it the piece's
 * bases).  Coloured (colors = 1; dumper_colormap_reading.rs:62-146): every k-mer once, in
 * pieces of one colour subset (runs of the " C:" annotations), grouped by subset in ascending
 * order; colors = the subset's colours from the colormap beside the graph, same_colors = 1 for
 * every piece of a group but the first.  As in the reference, pieces are not maximal unitigs. */
typedef void (*ggcat_gpu_dump_fn)(void *fn_ctx, const uint8_t *seq, uint64_t len, const uint32_t *colors,
                                  uint64_t n_colors, int same_colors);
int ggcat_gpu_dump_unitigs(const char *graph_input, int k, int colors, ggcat_gpu_dump_fn fn, void *fn_ctx);

/* A sequence source (InputStreamFFI of ggcat_build_from_streams, crates/capi/src/lib.rs:226-292,
 * 551-558): read_block calls emit once per sequence, on the calling thread; a sequence is any
 * bytes (ACGTacgt are bases, anything else splits k-mers like an N); partial_read_copyback is
 * the overlap (k - 1) a stream that cuts long sequences keeps between the pieces. */
typedef void (*ggcat_gpu_seq_fn)(void *emit_ctx, const uint8_t *seq, uint64_t len);
typedef struct {
    void *stream_ctx;
    void (*read_block)(void *stream_ctx, int64_t partial_read_copyback, ggcat_gpu_seq_fn emit, void *emit_ctx);
} ggcat_gpu_stream;

/* The text a build from streams starts from: every emitted sequence normalised like the
 * reader (ACGTacgt -> upper case, anything else -> N), each followed by '\n'.  h_text = NULL
 * queries the size. */
int ggcat_gpu_collect_streams(const ggcat_gpu_stream *streams, uint64_t n, int64_t copyback, uint8_t *h_text,
                              uint64_t text_cap, uint64_t *text_len);

/* ggcat_build_from_streams (crates/capi/src/lib.rs:226-292): ggcat_gpu_build_from_files with
 * the sequences of the streams instead of files. */
int ggcat_gpu_build_from_streams(ggcat_gpu_ctx *ctx, const ggcat_gpu_stream *streams, size_t n_streams,
                                 const char *output_file, size_t kmer_length, size_t threads_count, int forward_only,
                                 size_t minimizer_length, size_t min_multiplicity);

/* Mirrors ggcat_build_from_files (crates/capi/src/lib.rs:58-139, api/src/lib.rs:217-322)
 * for the uncoloured, no-extra-elaboration case: reads the input files like
 * ggcat_gpu_read_sequences_file (FASTA / FASTQ, plain or compressed), builds the graph on
 * the GPU and writes the maximal unitigs as FASTA ">{id} LN:i:{len}" to output_file.
 * threads_count = host threads reading the input files (0: all).  Returns 0 or a negative code. */
int ggcat_gpu_build_from_files(ggcat_gpu_ctx *ctx, const char *const *input_files, size_t n_inputs,
                               const char *output_file, size_t kmer_length, size_t threads_count, int forward_only,
                               size_t minimizer_length, size_t min_multiplicity);

/* ggcat_build_from_files with all its arguments, in its order (crates/capi/src/lib.rs:58-139;
 * GGCATInstance::build_graph, crates/api/src/lib.rs:217-322):
 *   color_names / n_color_names: the names written to the colormap (colour i = input i);
 *   colors: 1 = coloured graph: every k-mer's colour set (the inputs it occurs in) is deduped
 *     into subsets, the FASTA headers carry " C:{subset:x}:{count}" runs of the k-mers' subsets
 *     (UnitigColorData::write_as_ident, crates/colors/src/managers/multiple.rs:705-740) and the
 *     subsets go to the colormap "<output_file without its extension>.colors.dat"
 *     (ggcat_gpu_colormap_file); canonical builds only;
 *   extra_elab: 0 none, 1 unitig links (" L:+:j:-" after the colour runs, or GFA L / E lines),
 *     2 greedy matchtigs, 3 eulertigs, 4 pathtigs (ggcat_gpu_compute_tigs over the final
 *     unitigs, written as ">{i} LN:i:{len}" records, with the C: runs of their k-mers along
 *     each string when coloured, or GFA segments without links; greedy matchtigs not with
 *     colours: the reference's writer stops on coloured joins, compute_matchtigs.rs:496-503);
 *   gfa_output_version: 0 FASTA, 1 GFA v1, 2 GFA v2 (not with colours, as in the reference). */
int ggcat_gpu_build_from_files_ex(ggcat_gpu_ctx *ctx, const char *const *input_files, size_t n_inputs,
                                  const char *output_file, const char *const *color_names, size_t n_color_names,
                                  size_t kmer_length, size_t threads_count, int forward_only, size_t minimizer_length,
                                  int colors, size_t min_multiplicity, int extra_elab, int gfa_output_version);

/* Announces the colour table of the next build (the arguments of ggcat_gpu_colors, before
 * ggcat_gpu_build_text / ggcat_gpu_merge): the batched merge then collects every k-mer
 * instance's colour into its table entry, like the reference's buckets carry each superkmer's
 * colour into the merge (MinimizerBucketingMultipleSeqColorDataType, add_temp_buffer_structure_el,
 * crates/assembler_kmers_merge/src/unitigs_extender/hashmap.rs:361-431), and ggcat_gpu_colors
 * called with the same table merges the dumped copies instead of reading the text again.
 * Results are identical either way; the merge skips the collection (and ggcat_gpu_colors reads
 * the text) when its bitmap scratch would pass a quarter of the free device memory, for the
 * spilled store, the per-bucket form or k > 64.  n_seq = 0 withdraws the announcement. */
int ggcat_gpu_colors_prepare(ggcat_gpu_ctx *ctx, const uint64_t *h_seq_off, const uint32_t *h_seq_color,
                             uint64_t n_seq, uint32_t n_colors);

/* ---- colour subsets ----
 * Replaces the per-k-mer colour sets and subset dedup of MultipleColorsManager
 * (crates/colors/src/managers/multiple.rs:99-228) and ColorsMemMapWriter::get_id
 * (crates/colors/src/colors_memmap_writer.rs:43-61).  Needs the last merge run with
 * keep_kmers = 1 and the input text of the last bucketize still on the device
 * (ggcat_gpu_build_text keeps its copy; with ggcat_gpu_bucketize the caller's d_text must stay
 * valid).  Sequence i starts at text byte h_seq_off[i] (non-decreasing) and has colour
 * h_seq_color[i] < n_colors <= 65536 (the input file index, MinBkSingleColor).  A k-mer's
 * colour set is the set of colours of all its occurrences; equal sets share one subset id. */
int ggcat_gpu_colors(ggcat_gpu_ctx *ctx, const uint64_t *h_seq_off, const uint32_t *h_seq_color, uint64_t n_seq,
                     uint32_t n_colors, void *stream);
/* Subset id of every k-mer of ggcat_gpu_kmers_copy (same order). */
int ggcat_gpu_kmer_subsets_copy(ggcat_gpu_ctx *ctx, uint32_t *h_subset, uint64_t cap, uint64_t *n);
/* Subsets as colour bitmaps: subset i is words [i*w, (i+1)*w), bit c of word c/32 = colour c. */
int ggcat_gpu_subsets_copy(ggcat_gpu_ctx *ctx, uint32_t *h_bitmaps, uint64_t cap_words, uint64_t *n_subsets,
                           uint32_t *words_per_subset);

/* ---- colormap file (the colour subsets of a coloured graph) ----
 * "<graph>.colors.dat" in the reference's run-length colormap layout
 * (crates/colors/src/storage/{serializer,run_length,deserializer}.rs): header, LZ4 frame of the
 * colour names, LZ4 frames of 20000 encoded subsets each, chunk index.  Frames are written with
 * uncompressed blocks; compressed frames (as the reference writes them) are read too. */

/* GGCATInstance::get_colormap_file / ggcat_get_colormap_file (crates/api/src/lib.rs:385-387,
 * crates/capi/src/lib.rs:384-390): the graph path with its last extension replaced by
 * "colors.dat". */
int ggcat_gpu_colormap_file(const char *graph_file, char *out, uint64_t out_cap);

/* Writes a colormap: colour names, and subset i = colours subset_colors[subset_off[i] ..
 * subset_off[i + 1]) (strictly ascending, non-empty; subset_off has n_subsets + 1 entries).
 * The writer half of ColorsSerializer (serializer.rs:56-241). */
int ggcat_gpu_write_colormap(const char *path, const char *const *color_names, uint64_t n_colors,
                             const uint64_t *subset_off, const uint32_t *subset_colors, uint64_t n_subsets);

/* ggcat_dump_colors (crates/capi/src/lib.rs:392-401; GGCATInstance::dump_colors,
 * crates/api/src/lib.rs:392-408): the colour names of a colormap, each '\0'-terminated, in colour
 * index order.  h_names = NULL queries *names_bytes and *n_colors. */
int ggcat_gpu_dump_colors(const char *colormap, char *h_names, uint64_t cap, uint64_t *names_bytes,
                          uint64_t *n_colors);

/* ggcat_query_colormap (crates/capi/src/lib.rs:454-490; dump_colormap_query,
 * crates/dumper/src/pipeline/dumper_colormap_querying.rs:11-61): fn(fn_ctx, subset, colors,
 * n_colors) once per distinct requested subset, in ascending subset order, on the calling
 * thread (so single_thread_output_function holds either way).  A subset id the colormap does
 * not hold returns GGCAT_GPU_EINVAL. */
typedef void (*ggcat_gpu_colormap_fn)(void *fn_ctx, uint32_t subset, const uint32_t *colors, uint64_t n_colors);
int ggcat_gpu_query_colormap(const char *colormap, const uint32_t *subsets, uint64_t n_subsets,
                             int single_thread_output_function, ggcat_gpu_colormap_fn fn, void *fn_ctx);

/* ---- graph query lookup (querier::run_query, crates/querier/src/lib.rs:54-199) ----
 * The graph's canonical k-mers stay resident in a device hash table; batches of queries are
 * looked up asynchronously in up to GGCAT_GPU_QUERY_SLOTS in-flight slots (each with its own
 * stream and buffers), which is what a continuous-batching serving loop needs. */
#define GGCAT_GPU_QUERY_SLOTS 4

/* Uncoloured index from the graph's unitigs in the text layout (device memory); replaces the
 * graph side of the querier's bucketing and per-bucket maps (querier_minimizer_bucketing.rs:233-288,
 * parallel_kmers_query.rs:362-403).  k <= 64 (u128 keys above 32). */
int ggcat_gpu_query_index(ggcat_gpu_ctx *ctx, const uint8_t *d_graph_text, uint64_t len, int k, void *stream);
/* Coloured index from the last ggcat_gpu_colors result (the build's k-mers and subsets). */
int ggcat_gpu_query_index_colored(ggcat_gpu_ctx *ctx, void *stream);

/* Replaces ggcat_query_graph (crates/capi/src/lib.rs:324-380) / GGCATInstance::query_graph
 * (crates/api/src/lib.rs:325-382) for uncoloured graphs: indexes the unitigs of graph_fasta,
 * looks up every k-mer of every record of query_fasta (both read like
 * ggcat_gpu_read_sequences_file: FASTA / FASTQ, plain or compressed; one query per record
 * the reader emits) and writes the querier's CSV
 * (query_index,matched_kmers,query_kmers,match_percentage; counters_sorting.rs:235-268) to
 * output_prefix, ".csv" appended when it has no extension; the written path is copied to
 * out_path.  Canonical k-mers, k <= 64. */
int ggcat_gpu_query_from_files(ggcat_gpu_ctx *ctx, const char *graph_fasta, const char *query_fasta,
                               const char *output_prefix, int k, int forward_only, char *out_path, uint64_t out_cap);

/* ggcat_query_graph with all its arguments, in its order (crates/capi/src/lib.rs:324-380;
 * GGCATInstance::query_graph, crates/api/src/lib.rs:325-382).  The graph's canonical k-mers are
 * indexed on the device and every k-mer of every query record (FASTA / FASTQ, plain or
 * compressed) is looked up.  colors = 0: the querier's CSV
 * (query_index,matched_kmers,query_kmers,match_percentage; counters_sorting.rs:235-268) at
 * output_file_prefix (".csv" appended when it has no extension).  colors = 1: the graph's
 * " C:" runs give every k-mer's subset and the colormap beside the graph the subsets' colours;
 * the JSON lines of colored_query_output.rs:264-309 at output_file_prefix (".jsonl" appended
 * when it has no extension): {"query_index":i, "matches":{"c": f, ...}} for every query with a
 * match, f = the query's k-mers found in colour c over its k-mers, to 2 places; c is the colour
 * index (color_output_format 0) or its name (1).  threads_count and minimizer_length are
 * accepted and unused (no host threads, no minimizer bucketing).  The written path is copied to
 * out_path.  k <= 64, canonical only. */
int ggcat_gpu_query_graph(ggcat_gpu_ctx *ctx, const char *input_graph, const char *input_query,
                          const char *output_file_prefix, size_t kmer_length, size_t threads_count, int forward_only,
                          size_t minimizer_length, int colors, size_t color_output_format, char *out_path,
                          uint64_t out_cap);

/* Submits a batch of queries (host text layout; query i = h_text[h_off[i], h_off[i]+h_len[i]))
 * to slot `slot` and returns without waiting.  The slot's H2D copy, lookup kernel and D2H
 * copy run on the slot's own stream. */
int ggcat_gpu_query_submit(ggcat_gpu_ctx *ctx, int slot, const uint8_t *h_text, uint64_t len, const uint64_t *h_off,
                           const uint64_t *h_len, uint64_t nq);
/* 1 = the slot's batch has completed (or the slot is idle), 0 = still running, < 0 error. */
int ggcat_gpu_query_poll(ggcat_gpu_ctx *ctx, int slot);
/* Waits for the slot's batch; h_matched[i] = number of k-mer occurrences of query i present
 * in the graph (parallel_kmers_query.rs:437-471 + counters_sorting.rs:106-273). */
int ggcat_gpu_query_wait(ggcat_gpu_ctx *ctx, int slot, uint64_t *h_matched, uint64_t cap, uint64_t *nq);
/* Coloured index: per query and colour, the number of query k-mer occurrences present in
 * that colour (h_counts[q * n_colors + c]); colored_query_output.rs:264-309 prints these
 * divided by the query's k-mer count. */
int ggcat_gpu_query_color_counts(ggcat_gpu_ctx *ctx, int slot, uint64_t *h_counts, uint64_t cap, uint32_t *n_colors);

/* ---- hash families (crates/hashes) ----
 * Writes, for every window start i of d_text, the unextendable hash of the window as
 * d_out[2i] (low 64 bits), d_out[2i+1] (high 64 bits); windows spanning a non-ACGT byte give
 * all-ones.  kind: 0 canonical seq-hash u64 (k <= 32), 1 forward seq-hash u64, 2 canonical
 * seq-hash u128 (k <= 64), 3 forward seq-hash u128, 4 canonical Rabin-Karp u128 (k <= 127),
 * 5 forward Rabin-Karp u128, 6 canonical nt-hash m-mer value (min(fw,rc) << 1 | unique
 * flag, the minimizer ordering of cn_nthash.rs:96-99 and lib.rs:189-199; k = m <= 64). */
int ggcat_gpu_kmer_hashes(ggcat_gpu_ctx *ctx, const uint8_t *d_text, uint64_t len, int k, int kind, uint64_t *d_out,
                          void *stream);

/* ---- bucket-size histogram without device allocation ----
 * For callers that cannot allocate device memory (their memory belongs to another
 * allocator, or they run where allocating is not allowed, or they only want to size their
 * own bucket store first).  No counterpart in the reference.
 *
 * Runs the superkmer split of ggcat_gpu_bucketize over d_text (device, layout as above)
 * and writes, for each of the 2^bucket_bits + 1 first-level buckets, the number of
 * superkmers (d_superkmers) and of k-mer instances (d_kmers), plus d_offsets, the
 * exclusive prefix sums of d_superkmers with the total in d_offsets[2^bucket_bits + 1].
 * All three are caller-owned device arrays.  The values equal those of the records
 * ggcat_gpu_bucketize produces.
 *
 * Allocates nothing: its only scratch is a static 131 KB device array (room for
 * 2^13 + 1 buckets) that every GPU loading the library keeps until exit.  bucket_bits > 13
 * or text_len >= 2^40 returns GGCAT_GPU_ETOOLARGE.  The first call on each device looks up
 * the scratch's device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  Every call clears and reuses the same scratch, so
 * calls that overlap on the GPU (other streams, other host threads) race: serialise them.
 * Runs on the current device; stream is a cudaStream_t (NULL = legacy default stream). */
int ggcat_gpu_bucket_histogram_noalloc(const uint8_t *d_text, uint64_t text_len, int32_t k, int32_t m,
                                       int32_t bucket_bits, uint64_t *d_superkmers, uint64_t *d_kmers,
                                       uint64_t *d_offsets, void *stream);

#ifdef __cplusplus
}
#endif
#endif
