// Colour-subset map file (run-length colormap layout of the reference); see colormap.cpp.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <utility>
#include <vector>

namespace ggcat {
namespace cmap {

void lz4_frame_store(std::vector<uint8_t> &out, const uint8_t *data, size_t n);
bool lz4_frame_decode(const uint8_t *in, size_t n, size_t *used, std::vector<uint8_t> &out);
void varint_put(std::vector<uint8_t> &o, uint64_t v);
bool varint_get(const uint8_t *&p, const uint8_t *end, uint64_t *v);
void subset_encode(std::vector<uint8_t> &o, const uint32_t *colors, size_t n);
bool subset_decode(const uint8_t *&p, const uint8_t *end, std::vector<uint32_t> &out);

// Writes the colormap of n_subsets subsets; subset(i, out) fills subset i's colours (sorted
// ascending, at least one).  Returns a GGCAT_GPU_* code.
int write(const char *path, const std::vector<std::string> &names, uint64_t n_subsets,
          const std::function<void(uint64_t, std::vector<uint32_t> &)> &subset);

// Whole-file reader; get() decodes subsets sequentially inside a chunk (cheap for ascending
// requests, like the reference's deserializer).
struct Reader {
    std::vector<uint8_t> data;
    std::vector<std::string> names;
    std::vector<std::pair<uint32_t, uint64_t>> chunks;  // (first subset, file offset)
    uint64_t index_offset = 0, colors_count = 0, subsets_count = 0;
    std::vector<uint8_t> chunk_raw;
    size_t cur_chunk = (size_t)-1, cur_pos = 0;
    uint32_t cur_index = 0;
    int open(const char *path, std::string *err);
    bool get(uint32_t subset, std::vector<uint32_t> &out);
};

}  // namespace cmap
}  // namespace ggcat

// the colormap path of a graph file (GGCATInstance::get_colormap_file)
std::string ggcat_colormap_path(const std::string &graph);
