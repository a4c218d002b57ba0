// Host file formats: stacked TIFF volumes (PNG frames are in png.cpp).
//
// Stacked TIFF (Grid::load_tiff, src/model/Grid.cpp:27-79).  libtiff is not
// available, so this is a reader of its own for the files the reference's
// tools write (tifffile: classic or BigTIFF, one page per z slice, 8-bit
// gray / RGB / RGBA, strips or tiles, contiguous samples), uncompressed or
// with the codecs libtiff decodes for such files: LZW (5, libtiff's MSB-first
// form with the code width growing one code early), Deflate (8 and the old
// 32946; zlib streams, inflated by an RFC 1950/1951 decoder of its own) and
// PackBits (32773), each optionally with the horizontal predictor (2).  It
// returns what TIFFReadRGBAImage hands the reference:
//   - rows bottom-up: grid row y of a layer is image row height-1-y
//     (TIFFReadRGBAImage's default ORIENTATION_BOTLEFT raster);
//   - gray -> R=G=B=gray, A=255; RGB -> A=255;
//   - RGBA with unassociated alpha is premultiplied, (c*a + 127)/255, as
//     libtiff's RGBA interface does; associated alpha is kept as stored.
// The layer-size check copies the reference's `&&` (a layer is rejected only
// when both width and height differ, Grid.cpp:47); later layers must still
// hold at least width*height pixels here, where the reference would read past
// them.

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
    uint16_t predictor = 1;
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
        case 284: case 317: case 322: case 323: case 324: case 325: case 338:
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
        case 317: d.predictor = (uint16_t)v[0]; break;
        case 322: d.tile_w = (uint32_t)v[0]; break;
        case 323: d.tile_h = (uint32_t)v[0]; break;
        case 338: d.extra = (uint16_t)v[0]; break;
        }
    }
    d.next = r.get(ents.data() + n * eb, nb);
    return XN_OK;
}

// ------------------------------------------------------------- codecs ---

// Inflate (RFC 1951) with 15-bit lookup tables: each table entry holds the
// symbol and the code length for every 15-bit window whose low bits start
// with that code (deflate packs Huffman codes most-significant bit first
// into a least-significant-bit-first stream, so codes are bit-reversed).
struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;
    uint64_t buf = 0, used = 0;  // used: bits consumed
    int cnt = 0;                 // bits in buf (bytes past the end read as 0)
    BitIn(const uint8_t* d, size_t len) : p(d), n(len) {}
    uint32_t peek(int k) {
        while (cnt <= 56) {
            buf |= (uint64_t)(pos < n ? p[pos] : 0) << cnt;
            ++pos;
            cnt += 8;
        }
        return (uint32_t)(buf & ((1ull << k) - 1));
    }
    void skip(int k) {
        buf >>= k;
        cnt -= k;
        used += (uint64_t)k;
    }
    uint32_t bits(int k) {
        if (k == 0) return 0;
        const uint32_t v = peek(k);
        skip(k);
        return v;
    }
    bool over() const { return used > (uint64_t)n * 8; }
    void align() { skip((int)((8 - (used & 7)) & 7)); }
};

struct Huffman {
    std::vector<uint32_t> table;  // symbol << 4 | length, 0 = no code
    bool build(const uint8_t* lengths, int n) {
        uint16_t count[16] = {0};
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = (left << 1) - count[l];
            if (left < 0) return false;  // over-subscribed
        }
        uint32_t next[16];
        uint32_t code = 0;
        for (int l = 1; l < 16; ++l) {
            code = (code + count[l - 1]) << 1;
            next[l] = code;
        }
        table.assign(1u << 15, 0u);
        for (int s = 0; s < n; ++s) {
            const int l = lengths[s];
            if (!l) continue;
            const uint32_t c = next[l]++;
            uint32_t r = 0;
            for (int b = 0; b < l; ++b) r |= ((c >> b) & 1u) << (l - 1 - b);
            for (uint32_t k = r; k < (1u << 15); k += 1u << l) table[k] = ((uint32_t)s << 4) | (uint32_t)l;
        }
        return true;
    }
    int decode(BitIn& in) const {
        const uint32_t e = table[in.peek(15)];
        if (!e) return -1;
        in.skip((int)(e & 15u));
        return (int)(e >> 4);
    }
};

const uint16_t LEN_BASE[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t DIST_BASE[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

// Inflates a zlib stream into out (exactly out.size() bytes expected).
bool inflate_zlib(const uint8_t* src, size_t n, std::vector<uint8_t>& out) {
    if (n < 2) return false;
    const uint32_t cmf = src[0], flg = src[1];
    if ((cmf & 15u) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
    BitIn in(src + 2, n - 2);
    size_t o = 0;
    const size_t cap = out.size();
    Huffman lit, dist;
    for (;;) {
        const uint32_t last = in.bits(1);
        const uint32_t type = in.bits(2);
        if (type == 0) {
            in.align();
            const uint32_t len = in.bits(16), nlen = in.bits(16);
            if ((len ^ 0xFFFFu) != nlen) return false;
            for (uint32_t i = 0; i < len; ++i) {
                if (o >= cap) return false;
                out[o++] = (uint8_t)in.bits(8);
            }
        } else if (type == 1 || type == 2) {
            uint8_t lengths[320];
            int nlit = 288, ndist = 30;
            if (type == 1) {
                for (int i = 0; i < 144; ++i) lengths[i] = 8;
                for (int i = 144; i < 256; ++i) lengths[i] = 9;
                for (int i = 256; i < 280; ++i) lengths[i] = 7;
                for (int i = 280; i < 288; ++i) lengths[i] = 8;
                for (int i = 0; i < 30; ++i) lengths[288 + i] = 5;
            } else {
                nlit = (int)in.bits(5) + 257;
                ndist = (int)in.bits(5) + 1;
                const int ncode = (int)in.bits(4) + 4;
                static const uint8_t ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
                uint8_t cl[19] = {0};
                for (int i = 0; i < ncode; ++i) cl[ORDER[i]] = (uint8_t)in.bits(3);
                Huffman clh;
                if (nlit > 286 || ndist > 30 || !clh.build(cl, 19)) return false;
                int i = 0;
                while (i < nlit + ndist) {
                    const int sym = clh.decode(in);
                    if (sym < 0) return false;
                    if (sym < 16) { lengths[i++] = (uint8_t)sym; continue; }
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (i == 0) return false;
                        val = lengths[i - 1];
                        rep = 3 + (int)in.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)in.bits(3);
                    } else {
                        rep = 11 + (int)in.bits(7);
                    }
                    if (i + rep > nlit + ndist) return false;
                    while (rep--) lengths[i++] = val;
                }
                if (lengths[256] == 0) return false;
                // the distance lengths follow the literal lengths directly
                std::memmove(lengths + 288, lengths + nlit, (size_t)ndist);
                for (int k = nlit; k < 288; ++k) lengths[k] = 0;
            }
            if (!lit.build(lengths, 288) || !dist.build(lengths + 288, ndist)) return false;
            for (;;) {
                const int sym = lit.decode(in);
                if (sym < 0 || in.over()) return false;
                if (sym < 256) {
                    if (o >= cap) return false;
                    out[o++] = (uint8_t)sym;
                } else if (sym == 256) {
                    break;
                } else {
                    const int li = sym - 257;
                    if (li >= 29) return false;
                    const uint32_t len = LEN_BASE[li] + in.bits(LEN_EXTRA[li]);
                    const int di = dist.decode(in);
                    if (di < 0 || di >= 30) return false;
                    const uint32_t d = DIST_BASE[di] + in.bits(DIST_EXTRA[di]);
                    if (d > o || len > cap - o) return false;
                    for (uint32_t k = 0; k < len; ++k, ++o) out[o] = out[o - d];
                }
            }
        } else {
            return false;
        }
        if (in.over()) return false;
        if (last) break;
    }
    if (o != cap) return false;
    // zlib trailer: Adler-32 of the output, big-endian (zlib reports a mismatch as an error)
    in.align();
    uint32_t want = 0;
    for (int k = 0; k < 4; ++k) want = (want << 8) | in.bits(8);
    if (in.over()) return false;
    uint32_t a = 1, b = 0;
    for (size_t k = 0; k < o; ++k) {
        a = (a + out[k]) % 65521u;
        b = (b + a) % 65521u;
    }
    return ((b << 16) | a) == want;
}

// TIFF LZW (compression 5): MSB-first codes of 9..12 bits, Clear = 256,
// EndOfInformation = 257; the width grows when the next free entry reaches
// 2^width - 1 (one code early, as libtiff's decoder and every TIFF writer do).
bool lzw_decode(const uint8_t* src, size_t n, std::vector<uint8_t>& out) {
    const size_t cap = out.size();
    std::vector<uint16_t> prefix(4096), len(4096);
    std::vector<uint8_t> suffix(4096), first(4096);
    for (int i = 0; i < 256; ++i) {
        prefix[i] = 0xFFFF;
        suffix[i] = first[i] = (uint8_t)i;
        len[i] = 1;
    }
    size_t o = 0;
    uint64_t bitpos = 0;
    const uint64_t nbits_total = (uint64_t)n * 8;
    int width = 9;
    uint32_t next = 258;
    int old = -1;
    auto emit = [&](uint32_t code) -> bool {
        const uint32_t l = len[code];
        if (l > cap - o) return false;
        uint32_t c = code;
        for (uint32_t k = l; k-- > 0;) {
            out[o + k] = suffix[c];
            c = prefix[c];
        }
        o += l;
        return true;
    };
    while (bitpos + width <= nbits_total) {
        uint32_t code = 0;
        for (int b = 0; b < width; ++b, ++bitpos) code = (code << 1) | ((src[bitpos >> 3] >> (7 - (bitpos & 7))) & 1u);
        if (code == 257) break;
        if (code == 256) {
            width = 9;
            next = 258;
            old = -1;
            continue;
        }
        if (old < 0) {
            if (code > 255 || !emit(code)) return false;
            old = (int)code;
            continue;
        }
        uint8_t head;
        if (code < next) {
            if (!emit(code)) return false;
            head = first[code];
        } else if (code == next && next < 4096) {
            head = first[old];
            // the new entry is old's string plus its own first byte
            const uint32_t l = len[old];
            if (l + 1 > cap - o) return false;
            const size_t start = o;
            if (!emit((uint32_t)old)) return false;
            out[start + l] = head;
            ++o;
        } else {
            return false;
        }
        if (next < 4096) {
            prefix[next] = (uint16_t)old;
            suffix[next] = head;
            first[next] = first[old];
            len[next] = (uint16_t)(len[old] + 1);
            ++next;
            if (next >= 2047) width = 12;
            else if (next >= 1023) width = 11;
            else if (next >= 511) width = 10;
        }
        old = (int)code;
    }
    return o == cap;
}

// PackBits (compression 32773): a signed header byte h; 0..127 copies the
// next h+1 bytes, -127..-1 repeats the next byte 1-h times, -128 is skipped.
bool packbits_decode(const uint8_t* src, size_t n, std::vector<uint8_t>& out) {
    const size_t cap = out.size();
    size_t i = 0, o = 0;
    while (i < n && o < cap) {
        const int h = (int)(int8_t)src[i++];
        if (h >= 0) {
            const size_t k = (size_t)h + 1;
            if (k > n - i || k > cap - o) return false;
            std::memcpy(&out[o], &src[i], k);
            i += k;
            o += k;
        } else if (h != -128) {
            const size_t k = (size_t)(1 - h);
            if (i >= n || k > cap - o) return false;
            std::memset(&out[o], src[i++], k);
            o += k;
        }
    }
    return o == cap;
}

// Reads one strip or tile (bytes stored at off, count of them) and decodes it
// into out (its uncompressed size); row_bytes = one row of the strip / tile.
int read_chunk(Reader& r, const Ifd& d, uint64_t off, uint64_t count, std::vector<uint8_t>& out, uint64_t row_bytes,
               const char* path, const char* what) {
    if (d.compression == 1) {
        if (!r.read_at(off, out.data(), out.size())) return fail(XN_ERR_FORMAT, "'%s': truncated %s", path, what);
    } else {
        std::vector<uint8_t> raw(count ? count : 1);
        if (!count || !r.read_at(off, raw.data(), count)) return fail(XN_ERR_FORMAT, "'%s': truncated %s", path, what);
        bool ok;
        if (d.compression == 5) ok = lzw_decode(raw.data(), count, out);
        else if (d.compression == 8 || d.compression == 32946) ok = inflate_zlib(raw.data(), count, out);
        else ok = packbits_decode(raw.data(), count, out);
        if (!ok) return fail(XN_ERR_FORMAT, "'%s': corrupt compressed %s (compression %u)", path, what, d.compression);
    }
    if (d.predictor == 2) {
        // horizontal differencing: each sample is stored minus the same sample of the previous pixel
        for (uint64_t row = 0; row + row_bytes <= out.size(); row += row_bytes)
            for (uint64_t i = d.spp; i < row_bytes; ++i) out[row + i] = (uint8_t)(out[row + i] + out[row + i - d.spp]);
    }
    return XN_OK;
}

// Decodes one page into RGBA rows, bottom-up (TIFFReadRGBAImage's raster).
int decode_page(Reader& r, const Ifd& d, uint32_t width, uint32_t height, uint8_t* out, const char* path) {
    if (d.compression != 1 && d.compression != 5 && d.compression != 8 && d.compression != 32946 &&
        d.compression != 32773)
        return fail(XN_ERR_FORMAT, "'%s': TIFF compression %u is not supported", path, d.compression);
    if (d.predictor != 1 && d.predictor != 2)
        return fail(XN_ERR_FORMAT, "'%s': TIFF predictor %u is not supported", path, d.predictor);
    if (d.compression != 1 && d.counts.size() < d.offsets.size())
        return fail(XN_ERR_FORMAT, "'%s': compressed TIFF without byte counts", path);
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
                const uint64_t t = (uint64_t)j * tx + i;
                const int rc = read_chunk(r, d, d.offsets[t], t < d.counts.size() ? d.counts[t] : 0, tile,
                                          (uint64_t)d.tile_w * spp, path, "tile");
                if (rc) return rc;
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
        std::vector<uint8_t> strip;
        for (uint64_t s = 0; s < strips; ++s) {
            const uint64_t rows = std::min<uint64_t>(rps, d.height - s * rps);
            strip.resize(rows * d.width * spp);
            const int rc = read_chunk(r, d, d.offsets[s], s < d.counts.size() ? d.counts[s] : 0, strip,
                                      (uint64_t)d.width * spp, path, "strip");
            if (rc) return rc;
            std::memcpy(&px[s * rps * d.width * spp], strip.data(), strip.size());
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
