// Host input readers (input.cpp): files of the build and query paths into the device text
// layout (normalised pieces, each followed by '\n').
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "ggcat_gb300.h"

namespace ggcat {

enum : int { kFormatUnknown = 0, kFormatFasta = 1, kFormatFastq = 2 };

// FASTA or FASTQ from the file name's extension chain (kFormatUnknown otherwise)
int sequence_format(const char *path);
// the whole file, decompressed by its last extension (gz, lz4, bz2, xz, zst/zstd)
int read_input_file(const char *path, std::vector<uint8_t> &out, std::string &err);
// parses n bytes of the given format: FASTA records cut with the copyback (< 0: whole
// records), FASTQ records whole; h_text = null counts only; off/len (optional) receive each
// piece's offset and length
int parse_sequences(const uint8_t *data, uint64_t n, int format, int64_t copyback, uint8_t *h_text, uint64_t cap,
                    uint64_t *text_len, uint64_t *n_pieces, std::vector<uint64_t> *off, std::vector<uint64_t> *len);
// read + parse, appending to text (off, len: pieces, offsets into text); FASTA files of
// 16 MiB or more are parsed on `threads` threads (the same output)
int read_sequences(const char *path, int64_t copyback, std::vector<uint8_t> &text, std::vector<uint64_t> *off,
                   std::vector<uint64_t> *len, std::string &err, int threads = 1);
// the sequences the streams emit, normalised, each followed by '\n', appended to text
int collect_streams(const ggcat_gpu_stream *streams, size_t n, int64_t copyback, std::vector<uint8_t> &text);
// several files on up to `threads` threads, concatenated in input order into text; file_off
// (optional) receives the text offset where each file's sequences start
int read_sequences_files(const char *const *paths, size_t n, int64_t copyback, int threads, std::vector<uint8_t> &text,
                         std::string &err, std::vector<uint64_t> *file_off = nullptr);

}  // namespace ggcat
