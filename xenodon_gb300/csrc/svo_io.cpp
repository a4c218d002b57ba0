// XNDN-SVO file I/O (src/model/Octree.cpp:21,50-114): "XNDN-SVO", u64 side,
// u64 node count, then per node 8 child words, the packed colour and
// is_leaf_depth, all little-endian u32.  The byte order is written out
// explicitly so the files are identical on x86 and Arm hosts.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/xenodon.h"
#include "xn_ctx.h"

namespace {

const char SVO_ID[8] = {'X', 'N', 'D', 'N', '-', 'S', 'V', 'O'};

uint64_t get_le64(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

void put_le64(unsigned char* p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}

struct File {
    std::FILE* f;
    explicit File(std::FILE* f) : f(f) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace

using xn::fail;

XN_API int xn_svo_load(const char* path, uint32_t** nodes_out, uint64_t* n_nodes, uint64_t* side) {
    if (!path || !nodes_out || !n_nodes || !side) return fail(XN_ERR_ARG, "xn_svo_load: NULL argument");
    *nodes_out = nullptr;
    File in(std::fopen(path, "rb"));
    if (!in.f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    unsigned char hdr[24];
    if (std::fread(hdr, 1, 24, in.f) != 24) return fail(XN_ERR_FORMAT, "'%s': truncated header", path);
    if (std::memcmp(hdr, SVO_ID, 8) != 0) return fail(XN_ERR_FORMAT, "'%s': Invalid format id", path);
    uint64_t dim = get_le64(hdr + 8);
    uint64_t n = get_le64(hdr + 16);
    if (std::fseek(in.f, 0, SEEK_END) != 0) return fail(XN_ERR_IO, "'%s': Failed to tell", path);
    long end = std::ftell(in.f);
    if (end < 0) return fail(XN_ERR_IO, "'%s': Failed to tell", path);
    uint64_t remaining = (uint64_t)end - 24;
    if (n > UINT64_MAX / 40 || remaining != 40 * n)
        return fail(XN_ERR_FORMAT, "'%s': File size does not match number of nodes", path);
    if (std::fseek(in.f, 24, SEEK_SET) != 0) return fail(XN_ERR_IO, "'%s': seek failed", path);
    uint32_t* nodes = static_cast<uint32_t*>(std::malloc(n ? n * 40 : 1));
    if (!nodes) return fail(XN_ERR_NOMEM, "'%s': out of host memory for %llu nodes", path, (unsigned long long)n);
    const uint64_t chunk_words = 1u << 20;
    unsigned char* buf = static_cast<unsigned char*>(std::malloc(chunk_words * 4));
    if (!buf) {
        std::free(nodes);
        return fail(XN_ERR_NOMEM, "xn_svo_load: out of host memory");
    }
    uint64_t words = n * 10;
    for (uint64_t done = 0; done < words;) {
        uint64_t take = words - done < chunk_words ? words - done : chunk_words;
        if (std::fread(buf, 4, take, in.f) != take) {
            std::free(buf);
            std::free(nodes);
            return fail(XN_ERR_IO, "'%s': short read", path);
        }
        for (uint64_t i = 0; i < take; ++i) {
            const unsigned char* p = buf + 4 * i;
            nodes[done + i] = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
        }
        done += take;
    }
    std::free(buf);
    *nodes_out = nodes;
    *n_nodes = n;
    *side = dim;
    return XN_OK;
}

XN_API int xn_svo_save(const char* path, const uint32_t* nodes, uint64_t n_nodes, uint64_t side) {
    if (!path || (!nodes && n_nodes)) return fail(XN_ERR_ARG, "xn_svo_save: NULL argument");
    File out(std::fopen(path, "wb"));
    if (!out.f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    unsigned char hdr[24];
    std::memcpy(hdr, SVO_ID, 8);
    put_le64(hdr + 8, side);
    put_le64(hdr + 16, n_nodes);
    if (std::fwrite(hdr, 1, 24, out.f) != 24) return fail(XN_ERR_IO, "'%s': write failed", path);
    const uint64_t chunk_words = 1u << 20;
    unsigned char* buf = static_cast<unsigned char*>(std::malloc(chunk_words * 4));
    if (!buf) return fail(XN_ERR_NOMEM, "xn_svo_save: out of host memory");
    uint64_t words = n_nodes * 10;
    for (uint64_t done = 0; done < words;) {
        uint64_t take = words - done < chunk_words ? words - done : chunk_words;
        for (uint64_t i = 0; i < take; ++i) {
            uint32_t w = nodes[done + i];
            unsigned char* p = buf + 4 * i;
            p[0] = (unsigned char)w;
            p[1] = (unsigned char)(w >> 8);
            p[2] = (unsigned char)(w >> 16);
            p[3] = (unsigned char)(w >> 24);
        }
        if (std::fwrite(buf, 4, take, out.f) != take) {
            std::free(buf);
            return fail(XN_ERR_IO, "'%s': write failed", path);
        }
        done += take;
    }
    std::free(buf);
    if (std::fflush(out.f) != 0) return fail(XN_ERR_IO, "'%s': write failed", path);
    return XN_OK;
}
