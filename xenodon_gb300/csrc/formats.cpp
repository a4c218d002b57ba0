// Host file formats: stacked TIFF volumes and PNG frames.
//
// Stacked TIFF (Grid::load_tiff, src/model/Grid.cpp:27-79).  libtiff is not
// available, so this is a reader of its own for the files the reference's
// tools write (tifffile: classic or BigTIFF, one page per z slice,
// uncompressed, 8-bit gray / RGB / RGBA, strips or tiles, contiguous
// samples).  It returns what TIFFReadRGBAImage hands the reference:
//   - rows bottom-up: grid row y of a layer is image row height-1-y
//     (TIFFReadRGBAImage's default ORIENTATION_BOTLEFT raster);
//   - gray -> R=G=B=gray, A=255; RGB -> A=255;
//   - RGBA with unassociated alpha is premultiplied, (c*a + 127)/255, as
//     libtiff's RGBA interface does; associated alpha is kept as stored.
// The layer-size check copies the reference's `&&` (a layer is rejected only
// when both width and height differ, Grid.cpp:47); later layers must still
// hold at least width*height pixels here, where the reference would read past
// them.
//
// PNG: RGBA8, non-interlaced, deflate "stored" blocks (the reference uses
// lodepng, src/backend/headless/HeadlessDisplay.cpp:80-85; any conforming
// decoder reads the same pixels).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/xenodon.h"
#include "xn_ctx.h"

using xn::fail;

namespace {

struct Reader {
    std::FILE* f = nullptr;
    bool le = true;
    bool big = false;
    uint64_t size = 0;
    ~Reader() {
        if (f) std::fclose(f);
    }
    bool read_at(uint64_t off, void* dst, uint64_t n) {
        if (off > size || n > size - off) return false;
        if (fseeko(f, (off_t)off, SEEK_SET) != 0) return false;
        return std::fread(dst, 1, n, f) == n;
    }
    uint64_t get(const unsigned char* p, int bytes) const {
        uint64_t v = 0;
        if (le)
            for (int i = bytes - 1; i >= 0; --i) v = (v << 8) | p[i];
        else
            for (int i = 0; i < bytes; ++i) v = (v << 8) | p[i];
        return v;
    }
};

struct Ifd {
    uint32_t width = 0, height = 0;
    uint16_t bits = 1, spp = 1, compression = 1, photometric = 1, planar = 1;
    uint16_t extra = 0;  // first ExtraSamples value
    uint32_t rows_per_strip = 0xFFFFFFFFu;
    uint32_t tile_w = 0, tile_h = 0;
    std::vector<uint64_t> offsets, counts;
    uint64_t next = 0;
};

const int TYPE_SIZE[19] = {0, 1, 1, 2, 4, 8, 1, 1, 2, 4, 8, 4, 8, 4, 0, 0, 8, 8, 8};

// Reads the values of one IFD entry as unsigned integers.
bool entry_values(Reader& r, const unsigned char* e, std::vector<uint64_t>& out) {
    const int tb = r.big ? 8 : 4;  // size of the count / inline value field
    const uint16_t type = (uint16_t)r.get(e + 2, 2);
    const uint64_t count = r.get(e + 4, tb);
    if (type >= 19 || TYPE_SIZE[type] == 0) return false;
    const int sz = TYPE_SIZE[type];
    if (count > (1ull << 32)) return false;
    const uint64_t total = count * sz;
    std::vector<unsigned char> buf(total ? total : 1);
    const unsigned char* field = e + 4 + tb;
    if (total <= (uint64_t)tb) {
        std::memcpy(buf.data(), field, total);
    } else if (!r.read_at(r.get(field, tb), buf.data(), total)) {
        return false;
    }
    out.resize(count);
    for (uint64_t i = 0; i < count; ++i) out[i] = r.get(buf.data() + i * sz, sz);
    return true;
}

int read_ifd(Reader& r, uint64_t off, Ifd& d, const char* path) {
    const int cb = r.big ? 8 : 2, eb = r.big ? 20 : 12, nb = r.big ? 8 : 4;
    unsigned char hdr[8];
    if (!r.read_at(off, hdr, cb)) return fail(XN_ERR_FORMAT, "'%s': truncated directory", path);
    const uint64_t n = r.get(hdr, cb);
    if (n == 0 || n > 4096) return fail(XN_ERR_FORMAT, "'%s': bad directory entry count", path);
    std::vector<unsigned char> ents(n * eb + nb);
    if (!r.read_at(off + cb, ents.data(), ents.size())) return fail(XN_ERR_FORMAT, "'%s': truncated directory", path);
    for (uint64_t i = 0; i < n; ++i) {
        const unsigned char* e = ents.data() + i * eb;
        const uint16_t tag = (uint16_t)r.get(e, 2);
        std::vector<uint64_t> v;
        switch (tag) {
        case 256: case 257: case 258: case 259: case 262: case 273: case 277: case 278: case 279:
        case 284: case 322: case 323: case 324: case 325: case 338:
            if (!entry_values(r, e, v) || v.empty()) return fail(XN_ERR_FORMAT, "'%s': bad value of tag %u", path, tag);
            break;
        default:
            continue;
        }
        switch (tag) {
        case 256: d.width = (uint32_t)v[0]; break;
        case 257: d.height = (uint32_t)v[0]; break;
        case 258:
            d.bits = (uint16_t)v[0];
            for (uint64_t b : v)
                if (b != v[0]) return fail(XN_ERR_FORMAT, "'%s': mixed bits per sample", path);
            break;
        case 259: d.compression = (uint16_t)v[0]; break;
        case 262: d.photometric = (uint16_t)v[0]; break;
        case 273: case 324: d.offsets = v; break;
        case 277: d.spp = (uint16_t)v[0]; break;
        case 278: d.rows_per_strip = (uint32_t)std::min<uint64_t>(v[0], 0xFFFFFFFFu); break;
        case 279: case 325: d.counts = v; break;
        case 284: d.planar = (uint16_t)v[0]; break;
        case 322: d.tile_w = (uint32_t)v[0]; break;
        case 323: d.tile_h = (uint32_t)v[0]; break;
        case 338: d.extra = (uint16_t)v[0]; break;
        }
    }
    d.next = r.get(ents.data() + n * eb, nb);
    return XN_OK;
}

// Decodes one page into RGBA rows, bottom-up (TIFFReadRGBAImage's raster).
int decode_page(Reader& r, const Ifd& d, uint32_t width, uint32_t height, uint8_t* out, const char* path) {
    if (d.compression != 1) return fail(XN_ERR_FORMAT, "'%s': compressed TIFF (compression %u) is not supported", path, d.compression);
    if (d.bits != 8) return fail(XN_ERR_FORMAT, "'%s': only 8-bit samples are supported (got %u)", path, d.bits);
    if (d.planar != 1 && d.spp > 1) return fail(XN_ERR_FORMAT, "'%s': planar TIFF is not supported", path);
    const bool gray = d.photometric == 0 || d.photometric == 1;
    if (!gray && d.photometric != 2) return fail(XN_ERR_FORMAT, "'%s': photometric %u is not supported", path, d.photometric);
    if ((gray && d.spp < 1) || (!gray && d.spp < 3)) return fail(XN_ERR_FORMAT, "'%s': unsupported samples per pixel", path);
    const uint32_t spp = d.spp;
    const bool invert = d.photometric == 0;  // WhiteIsZero
    const bool has_alpha = !gray && spp >= 4;
    const bool premultiply = has_alpha && d.extra == 2;
    // the page as stored, top row first
    std::vector<uint8_t> px((uint64_t)d.width * d.height * spp);
    if (d.tile_w && d.tile_h) {
        const uint32_t tx = (d.width + d.tile_w - 1) / d.tile_w, ty = (d.height + d.tile_h - 1) / d.tile_h;
        if (d.offsets.size() < (uint64_t)tx * ty) return fail(XN_ERR_FORMAT, "'%s': missing tiles", path);
        std::vector<uint8_t> tile((uint64_t)d.tile_w * d.tile_h * spp);
        for (uint32_t j = 0; j < ty; ++j)
            for (uint32_t i = 0; i < tx; ++i) {
                if (!r.read_at(d.offsets[(uint64_t)j * tx + i], tile.data(), tile.size()))
                    return fail(XN_ERR_FORMAT, "'%s': truncated tile", path);
                for (uint32_t y = 0; y < d.tile_h && j * d.tile_h + y < d.height; ++y) {
                    const uint32_t w = std::min(d.tile_w, d.width - i * d.tile_w);
                    std::memcpy(&px[(((uint64_t)(j * d.tile_h + y)) * d.width + i * d.tile_w) * spp],
                                &tile[(uint64_t)y * d.tile_w * spp], (uint64_t)w * spp);
                }
            }
    } else {
        const uint64_t rps = std::min<uint64_t>(d.rows_per_strip ? d.rows_per_strip : 1, d.height);
        const uint64_t strips = (d.height + rps - 1) / rps;
        if (d.offsets.size() < strips) return fail(XN_ERR_FORMAT, "'%s': missing strips", path);
        for (uint64_t s = 0; s < strips; ++s) {
            const uint64_t rows = std::min<uint64_t>(rps, d.height - s * rps);
            if (!r.read_at(d.offsets[s], &px[s * rps * d.width * spp], rows * d.width * spp))
                return fail(XN_ERR_FORMAT, "'%s': truncated strip", path);
        }
    }
    for (uint32_t y = 0; y < height; ++y) {
        // raster row y holds image row d.height-1-y (rows past the page stay 0)
        const uint64_t src_row = y < d.height ? (uint64_t)d.height - 1 - y : ~0ull;
        for (uint32_t x = 0; x < width; ++x) {
            uint8_t* o = out + 4 * ((uint64_t)y * width + x);
            if (src_row >= d.height || x >= d.width) {
                o[0] = o[1] = o[2] = o[3] = 0;
                continue;
            }
            const uint8_t* p = &px[((uint64_t)src_row * d.width + x) * spp];
            if (gray) {
                uint8_t g = invert ? (uint8_t)(255 - p[0]) : p[0];
                o[0] = o[1] = o[2] = g;
                o[3] = 255;
            } else if (!has_alpha) {
                o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = 255;
            } else if (premultiply) {
                const uint32_t a = p[3];
                o[0] = (uint8_t)((p[0] * a + 127) / 255);
                o[1] = (uint8_t)((p[1] * a + 127) / 255);
                o[2] = (uint8_t)((p[2] * a + 127) / 255);
                o[3] = (uint8_t)a;
            } else {
                o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = p[3];
            }
        }
    }
    return XN_OK;
}

uint32_t crc_table[256];
bool crc_ready = false;

uint32_t crc32_update(uint32_t c, const uint8_t* p, size_t n) {
    if (!crc_ready) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            crc_table[i] = v;
        }
        crc_ready = true;
    }
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

bool write_chunk(std::FILE* f, const char* type, const std::vector<uint8_t>& data) {
    std::vector<uint8_t> head;
    put_be32(head, (uint32_t)data.size());
    head.insert(head.end(), type, type + 4);
    uint32_t c = crc32_update(0xFFFFFFFFu, reinterpret_cast<const uint8_t*>(type), 4);
    c = crc32_update(c, data.data(), data.size()) ^ 0xFFFFFFFFu;
    std::vector<uint8_t> tail;
    put_be32(tail, c);
    return std::fwrite(head.data(), 1, head.size(), f) == head.size() &&
           (data.empty() || std::fwrite(data.data(), 1, data.size(), f) == data.size()) &&
           std::fwrite(tail.data(), 1, 4, f) == 4;
}

}  // namespace

XN_API int xn_tiff_load(const char* path, uint8_t** rgba_out, uint32_t dims_out[3]) {
    if (!path || !rgba_out || !dims_out) return fail(XN_ERR_ARG, "xn_tiff_load: NULL argument");
    *rgba_out = nullptr;
    Reader r;
    r.f = std::fopen(path, "rb");
    if (!r.f) return fail(XN_ERR_IO, "Failed to open");
    if (fseeko(r.f, 0, SEEK_END) != 0) return fail(XN_ERR_IO, "'%s': seek failed", path);
    r.size = (uint64_t)ftello(r.f);
    unsigned char h[16];
    if (!r.read_at(0, h, 8)) return fail(XN_ERR_FORMAT, "'%s': not a TIFF file", path);
    if (h[0] == 'I' && h[1] == 'I') r.le = true;
    else if (h[0] == 'M' && h[1] == 'M') r.le = false;
    else return fail(XN_ERR_FORMAT, "'%s': not a TIFF file", path);
    const uint16_t magic = (uint16_t)r.get(h + 2, 2);
    uint64_t off;
    if (magic == 42) {
        off = r.get(h + 4, 4);
    } else if (magic == 43) {
        if (!r.read_at(0, h, 16)) return fail(XN_ERR_FORMAT, "'%s': truncated BigTIFF header", path);
        r.big = true;
        off = r.get(h + 8, 8);
    } else {
        return fail(XN_ERR_FORMAT, "'%s': not a TIFF file", path);
    }
    std::vector<Ifd> pages;
    uint32_t width = 0, height = 0;
    while (off) {
        if (pages.size() >= 65535) return fail(XN_ERR_FORMAT, "'%s': more than 65535 layers", path);  // uint16_t depth
        Ifd d;
        int rc = read_ifd(r, off, d, path);
        if (rc) return rc;
        if (d.width == 0 || d.height == 0)
            return fail(XN_ERR_FORMAT, "Layer %zu has invalid dimensions (%ux%u)", pages.size(), d.width, d.height);
        if (width == 0) {
            width = d.width;
            height = d.height;
        } else if (d.width != width && d.height != height) {  // Grid.cpp:47 uses &&
            return fail(XN_ERR_FORMAT, "Dimensions of layer %zu differ from previous dimensions (%ux%u, previously %ux%u)",
                        pages.size(), d.width, d.height, width, height);
        }
        for (const Ifd& p : pages)
            if (p.next == d.next && d.next) return fail(XN_ERR_FORMAT, "'%s': directory loop", path);
        pages.push_back(d);
        off = d.next;
    }
    if (pages.empty()) return fail(XN_ERR_FORMAT, "'%s': no image", path);
    const uint64_t layer = (uint64_t)width * height * 4;
    uint8_t* out = static_cast<uint8_t*>(std::malloc(layer * pages.size()));
    if (!out) return fail(XN_ERR_NOMEM, "'%s': out of host memory", path);
    for (size_t z = 0; z < pages.size(); ++z) {
        int rc = decode_page(r, pages[z], width, height, out + z * layer, path);
        if (rc) {
            std::free(out);
            return rc;
        }
    }
    dims_out[0] = width;
    dims_out[1] = height;
    dims_out[2] = (uint32_t)pages.size();
    *rgba_out = out;
    return XN_OK;
}

XN_API int xn_tiff_save(const char* path, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz) {
    if (!path || !rgba) return fail(XN_ERR_ARG, "xn_tiff_save: NULL argument");
    if (!dx || !dy || !dz || dz > 65535) return fail(XN_ERR_ARG, "xn_tiff_save: bad dimensions %ux%ux%u", dx, dy, dz);
    const uint64_t layer = (uint64_t)dx * dy * 4;
    // BigTIFF, little-endian; per page: one strip of RGBA rows stored top row
    // first, so that the bottom-up raster read back is the grid.
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    auto le = [](std::vector<uint8_t>& v, uint64_t x, int n) {
        for (int i = 0; i < n; ++i) v.push_back((uint8_t)(x >> (8 * i)));
    };
    const int NE = 11;
    const uint64_t ifd_size = 8 + NE * 20 + 8;
    std::vector<uint8_t> hdr;
    hdr.insert(hdr.end(), {'I', 'I'});
    le(hdr, 43, 2);
    le(hdr, 8, 2);
    le(hdr, 0, 2);
    const uint64_t first = 16;
    le(hdr, first, 8);
    bool ok = std::fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
    std::vector<uint8_t> row((uint64_t)dx * 4);
    for (uint32_t z = 0; z < dz && ok; ++z) {
        const uint64_t base = first + (uint64_t)z * (ifd_size + layer);
        const uint64_t data_off = base + ifd_size;
        const uint64_t next = z + 1 < dz ? data_off + layer : 0;
        std::vector<uint8_t> d;
        le(d, NE, 8);
        auto ent = [&](uint16_t tag, uint16_t type, uint64_t count, uint64_t value) {
            le(d, tag, 2);
            le(d, type, 2);
            le(d, count, 8);
            le(d, value, 8);
        };
        ent(256, 4, 1, dx);
        ent(257, 4, 1, dy);
        ent(258, 3, 4, 0x0008000800080008ull);  // four 8-bit samples, inline
        ent(259, 3, 1, 1);
        ent(262, 3, 1, 2);
        ent(273, 16, 1, data_off);
        ent(277, 3, 1, 4);
        ent(278, 4, 1, dy);
        ent(279, 16, 1, layer);
        ent(284, 3, 1, 1);
        ent(338, 3, 1, 2);  // unassociated alpha
        le(d, next, 8);
        ok = std::fwrite(d.data(), 1, d.size(), f) == d.size();
        for (uint32_t y = 0; y < dy && ok; ++y) {
            const uint8_t* src = rgba + z * layer + (uint64_t)(dy - 1 - y) * dx * 4;
            ok = std::fwrite(src, 1, (size_t)dx * 4, f) == (size_t)dx * 4;
        }
    }
    if (std::fclose(f) != 0) ok = false;
    return ok ? XN_OK : fail(XN_ERR_IO, "'%s': write failed", path);
}

XN_API int xn_png_save(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height) {
    if (!path || !rgba) return fail(XN_ERR_ARG, "xn_png_save: NULL argument");
    if (!width || !height) return fail(XN_ERR_ARG, "xn_png_save: empty image");
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    bool ok = std::fwrite(sig, 1, 8, f) == 8;
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, no filter method extras, no interlace
    ok = ok && write_chunk(f, "IHDR", ihdr);
    // zlib stream of stored blocks over the filtered scanlines (filter 0)
    const uint64_t stride = (uint64_t)width * 4 + 1;
    const uint64_t raw = stride * height;
    std::vector<uint8_t> z;
    z.reserve(raw + raw / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    uint32_t s1 = 1, s2 = 0;
    uint64_t pos = 0;
    std::vector<uint8_t> line(stride);
    uint64_t in_block = 0;
    size_t block_len_at = 0;
    for (uint32_t y = 0; y < height; ++y) {
        line[0] = 0;
        std::memcpy(&line[1], rgba + (uint64_t)y * width * 4, (size_t)width * 4);
        for (uint64_t i = 0; i < stride; ++i) {
            if (in_block == 0) {
                const uint64_t left = raw - pos;
                const uint16_t len = (uint16_t)(left < 65535 ? left : 65535);
                z.push_back(left <= 65535 ? 1 : 0);
                block_len_at = z.size();
                z.push_back((uint8_t)len);
                z.push_back((uint8_t)(len >> 8));
                z.push_back((uint8_t)~len);
                z.push_back((uint8_t)(~len >> 8));
                in_block = len;
            }
            const uint8_t b = line[i];
            z.push_back(b);
            s1 = (s1 + b) % 65521;
            s2 = (s2 + s1) % 65521;
            --in_block;
            ++pos;
        }
    }
    (void)block_len_at;
    put_be32(z, (s2 << 16) | s1);
    ok = ok && write_chunk(f, "IDAT", z);
    ok = ok && write_chunk(f, "IEND", {});
    if (std::fclose(f) != 0) ok = false;
    return ok ? XN_OK : fail(XN_ERR_IO, "'%s': write failed", path);
}
