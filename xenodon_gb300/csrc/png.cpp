// PNG output of rendered frames (the headless backend's frame files,
// src/backend/headless/HeadlessDisplay.cpp:80-85, which the reference writes
// with lodepng).  Own encoder:
//
//  - each scanline gets the PNG filter (None, Sub, Up, Average, Paeth) with
//    the smallest sum of absolute residuals, the usual heuristic;
//  - the filtered bytes are cut into bands of whole rows, and every band is
//    deflated on its own thread: LZ77 over a 32 KiB window with hash chains,
//    then one dynamic-Huffman block per band (RFC 1951 3.2.7).  A band that is
//    not the last one ends with an empty stored block, which byte-aligns it,
//    so the bands' bit streams concatenate into one zlib stream (the method
//    parallel gzip tools use);
//  - the Adler-32 of the whole stream closes it (RFC 1950).
//
// A rendered frame is mostly black background, which the filters turn into
// runs of zeros and LZ77 into long matches.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/xenodon.h"
#include "xn_ctx.h"

using xn::fail;

namespace {

// ------------------------------------------------------------ bit writer ---

struct BitWriter {
    std::vector<uint8_t>& out;
    uint64_t acc = 0;
    int n = 0;
    explicit BitWriter(std::vector<uint8_t>& o) : out(o) {}
    // `bits` LSB first (deflate's order for everything but Huffman codes)
    void put(uint32_t bits, int count) {
        acc |= (uint64_t)bits << n;
        n += count;
        while (n >= 8) {
            out.push_back((uint8_t)acc);
            acc >>= 8;
            n -= 8;
        }
    }
    void align() {
        if (n > 0) put(0, 8 - n);
    }
};

// Huffman codes are sent most significant bit first: store them reversed.
uint32_t reverse_bits(uint32_t code, int len) {
    uint32_t r = 0;
    for (int i = 0; i < len; ++i) r |= ((code >> i) & 1u) << (len - 1 - i);
    return r;
}

// ------------------------------------------------------ Huffman lengths ---

// Code lengths of at most max_len bits for the given symbol counts (0 for an
// unused symbol).  A plain Huffman construction; while the longest code is too
// long, the counts are halved (keeping used symbols at >= 1) and the code is
// built again, which flattens the tree.
void huffman_lengths(const std::vector<uint32_t>& freq_in, int max_len, std::vector<uint8_t>& len) {
    const int n = (int)freq_in.size();
    len.assign(n, 0);
    std::vector<uint64_t> freq(freq_in.begin(), freq_in.end());
    int used = 0;
    for (uint64_t f : freq) used += f > 0;
    if (used == 0) return;
    if (used == 1) {
        // two codes of one bit: a complete code, which every inflater accepts
        // (zlib refuses an incomplete code-length code)
        for (int i = 0; i < n; ++i)
            if (freq[i]) len[i] = 1;
        len[len[0] ? 1 : 0] = 1;
        return;
    }
    for (;;) {
        // nodes: leaves 0..n-1, internal n..; parent links give the depths
        struct Node {
            uint64_t w;
            int id;
        };
        std::vector<Node> heap;
        std::vector<int> parent(2 * n, -1);
        for (int i = 0; i < n; ++i)
            if (freq[i]) heap.push_back({freq[i], i});
        auto cmp = [](const Node& a, const Node& b) { return a.w != b.w ? a.w > b.w : a.id > b.id; };
        std::make_heap(heap.begin(), heap.end(), cmp);
        int next = n;
        while (heap.size() > 1) {
            std::pop_heap(heap.begin(), heap.end(), cmp);
            Node a = heap.back();
            heap.pop_back();
            std::pop_heap(heap.begin(), heap.end(), cmp);
            Node b = heap.back();
            heap.pop_back();
            parent[a.id] = next;
            parent[b.id] = next;
            heap.push_back({a.w + b.w, next});
            std::push_heap(heap.begin(), heap.end(), cmp);
            ++next;
        }
        int longest = 0;
        for (int i = 0; i < n; ++i) {
            if (!freq[i]) continue;
            int d = 0;
            for (int p = parent[i]; p != -1; p = parent[p]) ++d;
            len[i] = (uint8_t)d;
            longest = std::max(longest, d);
        }
        if (longest <= max_len) return;
        for (auto& f : freq)
            if (f) f = std::max<uint64_t>(1, f >> 1);
    }
}

// Canonical codes from lengths (RFC 1951 3.2.2), already bit-reversed.
void canonical_codes(const std::vector<uint8_t>& len, std::vector<uint32_t>& code) {
    int bl_count[16] = {0};
    for (uint8_t l : len) bl_count[l]++;
    bl_count[0] = 0;
    uint32_t next_code[16] = {0};
    uint32_t c = 0;
    for (int bits = 1; bits < 16; ++bits) {
        c = (c + bl_count[bits - 1]) << 1;
        next_code[bits] = c;
    }
    code.assign(len.size(), 0);
    for (size_t i = 0; i < len.size(); ++i)
        if (len[i]) code[i] = reverse_bits(next_code[len[i]]++, len[i]);
}

// ------------------------------------------------------------------ LZ77 ---

// RFC 1951 3.2.5 length and distance code tables (the format's constants).
constexpr uint16_t LEN_BASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

int length_code(int len) {  // 3..258 -> 0..28
    int i = 28;
    while (LEN_BASE[i] > len) --i;
    return i;
}
int dist_code(int d) {  // 1..32768 -> 0..29
    int i = 29;
    while (DIST_BASE[i] > d) --i;
    return i;
}

// One token: a literal (dist == 0) or a match.
struct Token {
    uint16_t lit_or_len;
    uint16_t dist;
};

constexpr int WINDOW = 32768;
constexpr int MIN_MATCH = 3, MAX_MATCH = 258;
constexpr int HASH_BITS = 15;
constexpr int MAX_CHAIN = 48;

void lz77(const uint8_t* p, size_t n, std::vector<Token>& tok) {
    tok.clear();
    tok.reserve(n / 4 + 16);
    std::vector<int32_t> head(1u << HASH_BITS, -1);
    std::vector<int32_t> prev(n ? n : 1, -1);
    auto hash = [&](size_t i) { return ((uint32_t)p[i] << 10 ^ (uint32_t)p[i + 1] << 5 ^ p[i + 2]) & ((1u << HASH_BITS) - 1); };
    auto insert = [&](size_t i) {
        if (i + MIN_MATCH > n) return;
        const uint32_t h = hash(i);
        prev[i] = head[h];
        head[h] = (int32_t)i;
    };
    size_t i = 0;
    while (i < n) {
        int best = 0, best_d = 0;
        if (i + MIN_MATCH <= n) {
            const uint32_t h = hash(i);
            int32_t c = head[h];
            const size_t lim = std::min<size_t>(MAX_MATCH, n - i);
            for (int chain = 0; c >= 0 && chain < MAX_CHAIN; ++chain, c = prev[c]) {
                const size_t d = i - (size_t)c;
                if (d > WINDOW) break;
                if (p[c + best] != p[i + best]) continue;
                size_t l = 0;
                while (l < lim && p[c + l] == p[i + l]) ++l;
                if ((int)l > best) {
                    best = (int)l;
                    best_d = (int)d;
                    if (l == lim) break;
                }
            }
        }
        if (best >= MIN_MATCH) {
            tok.push_back({(uint16_t)best, (uint16_t)best_d});
            // index the matched positions (all of them for short matches, the
            // ends of long ones: a run of zeros needs no dense chain)
            const size_t end = i + (size_t)best;
            if (best <= 32) {
                for (size_t k = i; k < end; ++k) insert(k);
            } else {
                insert(i);
                for (size_t k = end - 3; k < end; ++k) insert(k);
            }
            i = end;
        } else {
            tok.push_back({p[i], 0});
            insert(i);
            ++i;
        }
    }
}

// One dynamic-Huffman block of the tokens (final or not).
void write_dynamic_block(BitWriter& bw, const std::vector<Token>& tok, bool final) {
    std::vector<uint32_t> lf(286, 0), df(30, 0);
    for (const Token& t : tok) {
        if (t.dist == 0) {
            lf[t.lit_or_len]++;
        } else {
            lf[257 + length_code(t.lit_or_len)]++;
            df[dist_code(t.dist)]++;
        }
    }
    lf[256] = 1;
    bool any_dist = false;
    for (uint32_t f : df) any_dist |= f > 0;
    if (!any_dist) df[0] = 1;  // the distance tree needs one code
    std::vector<uint8_t> ll, dl;
    huffman_lengths(lf, 15, ll);
    huffman_lengths(df, 15, dl);
    int hlit = 286, hdist = 30;
    while (hlit > 257 && ll[hlit - 1] == 0) --hlit;
    while (hdist > 1 && dl[hdist - 1] == 0) --hdist;
    // run-length code the two length sequences together (codes 16, 17, 18)
    std::vector<uint8_t> seq(ll.begin(), ll.begin() + hlit);
    seq.insert(seq.end(), dl.begin(), dl.begin() + hdist);
    struct Rl {
        uint8_t sym, extra;
    };
    std::vector<Rl> rl;
    for (size_t i = 0; i < seq.size();) {
        const uint8_t v = seq[i];
        size_t run = 1;
        while (i + run < seq.size() && seq[i + run] == v) ++run;
        size_t left = run;
        if (v == 0) {
            while (left >= 11) {
                const size_t k = std::min<size_t>(left, 138);
                rl.push_back({18, (uint8_t)(k - 11)});
                left -= k;
            }
            if (left >= 3) {
                rl.push_back({17, (uint8_t)(left - 3)});
                left = 0;
            }
        } else {
            rl.push_back({v, 0});
            --left;
            while (left >= 3) {
                const size_t k = std::min<size_t>(left, 6);
                rl.push_back({16, (uint8_t)(k - 3)});
                left -= k;
            }
        }
        for (; left > 0; --left) rl.push_back({v, 0});
        i += run;
    }
    std::vector<uint32_t> cf(19, 0);
    for (const Rl& r : rl) cf[r.sym]++;
    std::vector<uint8_t> cl;
    huffman_lengths(cf, 7, cl);
    static const uint8_t ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    int hclen = 19;
    while (hclen > 4 && cl[ORDER[hclen - 1]] == 0) --hclen;
    std::vector<uint32_t> lc, dc, cc;
    canonical_codes(ll, lc);
    canonical_codes(dl, dc);
    canonical_codes(cl, cc);

    bw.put(final ? 1 : 0, 1);
    bw.put(2, 2);
    bw.put((uint32_t)(hlit - 257), 5);
    bw.put((uint32_t)(hdist - 1), 5);
    bw.put((uint32_t)(hclen - 4), 4);
    for (int i = 0; i < hclen; ++i) bw.put(cl[ORDER[i]], 3);
    for (const Rl& r : rl) {
        bw.put(cc[r.sym], cl[r.sym]);
        if (r.sym == 16) bw.put(r.extra, 2);
        if (r.sym == 17) bw.put(r.extra, 3);
        if (r.sym == 18) bw.put(r.extra, 7);
    }
    for (const Token& t : tok) {
        if (t.dist == 0) {
            bw.put(lc[t.lit_or_len], ll[t.lit_or_len]);
        } else {
            const int c = length_code(t.lit_or_len);
            bw.put(lc[257 + c], ll[257 + c]);
            if (LEN_EXTRA[c]) bw.put((uint32_t)(t.lit_or_len - LEN_BASE[c]), LEN_EXTRA[c]);
            const int d = dist_code(t.dist);
            bw.put(dc[d], dl[d]);
            if (DIST_EXTRA[d]) bw.put((uint32_t)(t.dist - DIST_BASE[d]), DIST_EXTRA[d]);
        }
    }
    bw.put(lc[256], ll[256]);
}

// A band's deflate stream: its tokens in dynamic blocks of at most 1 Mi
// tokens; a band that is not the last ends byte-aligned with an empty stored
// block, so the next band's stream can follow it directly.
void deflate_band(const uint8_t* p, size_t n, bool last, std::vector<uint8_t>& out) {
    std::vector<Token> tok;
    lz77(p, n, tok);
    BitWriter bw(out);
    const size_t BLOCK = 1u << 20;
    if (tok.empty()) {
        if (last) {
            write_dynamic_block(bw, tok, true);
            bw.align();
        }
        return;
    }
    for (size_t b = 0; b < tok.size(); b += BLOCK) {
        std::vector<Token> part(tok.begin() + b, tok.begin() + std::min(tok.size(), b + BLOCK));
        write_dynamic_block(bw, part, last && b + BLOCK >= tok.size());
    }
    if (!last) {
        bw.put(0, 1);  // BFINAL 0
        bw.put(0, 2);  // stored
        bw.align();
        out.push_back(0x00);
        out.push_back(0x00);
        out.push_back(0xFF);
        out.push_back(0xFF);
    } else {
        bw.align();
    }
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n > 0) {
        const size_t k = std::min<size_t>(n, 5552);  // the largest run without overflow before the modulo
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521;
        b %= 65521;
        p += k;
        n -= k;
    }
    return (b << 16) | a;
}

// ----------------------------------------------------------- PNG pieces ---

struct Crc {
    uint32_t table[256];
    Crc() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
    }
    uint32_t update(uint32_t c, const uint8_t* p, size_t n) const {
        for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
        return c;
    }
};
const Crc g_crc;

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

bool write_chunk(std::FILE* f, const char* type, const uint8_t* data, size_t n) {
    std::vector<uint8_t> head;
    put_be32(head, (uint32_t)n);
    head.insert(head.end(), type, type + 4);
    uint32_t c = g_crc.update(0xFFFFFFFFu, reinterpret_cast<const uint8_t*>(type), 4);
    c = g_crc.update(c, data, n) ^ 0xFFFFFFFFu;
    std::vector<uint8_t> tail;
    put_be32(tail, c);
    return std::fwrite(head.data(), 1, head.size(), f) == head.size() && (n == 0 || std::fwrite(data, 1, n, f) == n) &&
           std::fwrite(tail.data(), 1, 4, f) == 4;
}

uint8_t paeth(uint8_t a, uint8_t b, uint8_t c) {
    const int p = (int)a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

// Filters row y (RGBA8, 4 bytes per pixel) into out[0..stride): the filter
// type byte, then the residuals of the filter with the smallest sum of
// absolute values (residuals read as signed bytes).
void filter_row(const uint8_t* cur, const uint8_t* up, uint32_t width, uint8_t* out, std::vector<uint8_t>& tmp) {
    const size_t n = (size_t)width * 4;
    tmp.resize(5 * n);
    uint64_t best_sum = ~0ull;
    int best = 0;
    for (int f = 0; f < 5; ++f) {
        if (!up && (f == 2 || f == 4)) continue;  // the first row: Up is None, Paeth is Sub
        uint8_t* r = tmp.data() + f * n;
        uint64_t sum = 0;
        for (size_t i = 0; i < n; ++i) {
            const uint8_t a = i >= 4 ? cur[i - 4] : 0;
            const uint8_t b = up ? up[i] : 0;
            const uint8_t c = (up && i >= 4) ? up[i - 4] : 0;
            uint8_t v = cur[i];
            switch (f) {
                case 1: v = (uint8_t)(v - a); break;
                case 2: v = (uint8_t)(v - b); break;
                case 3: v = (uint8_t)(v - (uint8_t)(((unsigned)a + b) >> 1)); break;
                case 4: v = (uint8_t)(v - paeth(a, b, c)); break;
                default: break;
            }
            r[i] = v;
            sum += (uint64_t)std::abs((int)(int8_t)v);
        }
        if (sum < best_sum) {
            best_sum = sum;
            best = f;
        }
    }
    out[0] = (uint8_t)best;
    std::memcpy(out + 1, tmp.data() + best * n, n);
}

}  // namespace

XN_API int xn_png_save(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height) {
    if (!path || !rgba) return fail(XN_ERR_ARG, "xn_png_save: NULL argument");
    if (!width || !height) return fail(XN_ERR_ARG, "xn_png_save: empty image");
    if ((uint64_t)width * 4 + 1 > 0x7FFFFFFFull) return fail(XN_ERR_ARG, "xn_png_save: image too wide");
    const size_t stride = (size_t)width * 4 + 1;
    const size_t raw_n = stride * height;
    std::vector<uint8_t> raw;
    try {
        raw.resize(raw_n);
    } catch (const std::bad_alloc&) {
        return fail(XN_ERR_NOMEM, "xn_png_save: out of host memory");
    }
    // bands of whole rows, at least 256 KiB each, at most one per host thread
    const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint32_t min_rows = (uint32_t)std::max<size_t>(1, (256u << 10) / stride);
    uint32_t bands = std::max(1u, std::min<uint32_t>(hw, height / min_rows));
    // and at most 1 GiB each (the match finder indexes a band with 32 bits)
    bands = std::min<uint64_t>(height, std::max<uint64_t>(bands, (raw_n >> 30) + 1));
    std::vector<std::vector<uint8_t>> out(bands);
    auto work = [&](uint32_t b) {
        const uint32_t y0 = (uint32_t)((uint64_t)height * b / bands), y1 = (uint32_t)((uint64_t)height * (b + 1) / bands);
        std::vector<uint8_t> tmp;
        for (uint32_t y = y0; y < y1; ++y) {
            const uint8_t* cur = rgba + (uint64_t)y * width * 4;
            const uint8_t* up = y ? cur - (uint64_t)width * 4 : nullptr;
            filter_row(cur, up, width, raw.data() + (size_t)y * stride, tmp);
        }
        deflate_band(raw.data() + (size_t)y0 * stride, (size_t)(y1 - y0) * stride, b + 1 == bands, out[b]);
    };
    std::vector<std::thread> th;
    try {
        for (uint32_t b = 1; b < bands; ++b) th.emplace_back(work, b);
    } catch (...) {
        for (auto& t : th) t.join();
        return fail(XN_ERR_NOMEM, "xn_png_save: could not start encoder threads");
    }
    work(0);
    for (auto& t : th) t.join();

    std::vector<uint8_t> z;
    size_t total = 2 + 4;
    for (auto& o : out) total += o.size();
    z.reserve(total);
    z.push_back(0x78);  // deflate, 32 KiB window
    z.push_back(0x9C);  // default level; (0x78 << 8 | 0x9C) % 31 == 0
    for (auto& o : out) z.insert(z.end(), o.begin(), o.end());
    put_be32(z, adler32(raw.data(), raw_n));

    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    bool ok = std::fwrite(sig, 1, 8, f) == 8;
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, adaptive filtering, no interlace
    ok = ok && write_chunk(f, "IHDR", ihdr.data(), ihdr.size());
    // IDAT chunks of at most 1 GiB (a chunk length is 31 bits)
    const size_t CH = 1u << 30;
    for (size_t off = 0; off < z.size() && ok; off += CH)
        ok = write_chunk(f, "IDAT", z.data() + off, std::min(CH, z.size() - off));
    ok = ok && write_chunk(f, "IEND", nullptr, 0);
    if (std::fclose(f) != 0) ok = false;
    return ok ? XN_OK : fail(XN_ERR_IO, "'%s': write failed", path);
}
