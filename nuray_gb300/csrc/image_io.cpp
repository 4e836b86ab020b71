// PNG codec for textures and output images; see image_io.h.
#include "image_io.h"

#include <cstring>

namespace nr {

namespace {

// ------------------------------------------------------------ bit input
// DEFLATE packs bits least-significant first; Huffman codes are read one
// bit at a time from the most significant bit of the code.
struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool over = false;
    Bits(const uint8_t* d, size_t len) : p(d), n(len) {}
    uint32_t take(int k) {  // k <= 32
        while (cnt < k) {
            uint64_t byte = 0;
            if (pos < n) byte = p[pos++];
            else over = true;
            buf |= byte << cnt;
            cnt += 8;
        }
        uint32_t v = (uint32_t)(buf & ((k == 32) ? 0xffffffffull : ((1ull << k) - 1)));
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() {  // drop to the next byte boundary
        int drop = cnt & 7;
        buf >>= drop;
        cnt -= drop;
    }
};

// Canonical Huffman code: the number of codes of each length and the
// symbols sorted by (length, value).
struct Code {
    uint16_t count[16];
    uint16_t sym[320];
};

// Builds a code from per-symbol lengths. Fails on an over-subscribed set;
// an incomplete set is accepted (RFC 1951 allows one distance code).
bool build(Code& c, const uint8_t* len, int n) {
    std::memset(c.count, 0, sizeof(c.count));
    for (int i = 0; i < n; ++i) c.count[len[i]]++;
    c.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= c.count[l];
        if (left < 0) return false;
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = off[l] + c.count[l];
    for (int i = 0; i < n; ++i)
        if (len[i]) c.sym[off[len[i]]++] = (uint16_t)i;
    return true;
}

// Reads one symbol: walks the code lengths, comparing the code read so far
// with the first code of each length.
int decode(Bits& b, const Code& c) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)b.take(1);
        int cnt = c.count[l];
        if (code - first < cnt) return c.sym[index + (code - first)];
        index += cnt;
        first = (first + cnt) << 1;
        code <<= 1;
        if (b.over) return -1;
    }
    return -1;
}

// RFC 1951 3.2.5: base values and extra bits of length codes 257..285 and
// distance codes 0..29.
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// RFC 1951 3.2.7: order of the code-length code lengths.
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

std::string inflate_codes(Bits& b, const Code& lit, const Code& dist, std::vector<uint8_t>& out, size_t limit) {
    while (true) {
        int s = decode(b, lit);
        if (s < 0 || b.over) return "corrupt deflate data (literal/length code)";
        if (s < 256) {
            if (out.size() >= limit) return "deflate data longer than expected";
            out.push_back((uint8_t)s);
            continue;
        }
        if (s == 256) return "";
        s -= 257;
        if (s >= 29) return "corrupt deflate data (length symbol)";
        size_t len = kLenBase[s] + b.take(kLenExtra[s]);
        int ds = decode(b, dist);
        if (ds < 0 || ds >= 30 || b.over) return "corrupt deflate data (distance code)";
        size_t d = kDistBase[ds] + b.take(kDistExtra[ds]);
        if (d > out.size()) return "corrupt deflate data (distance beyond output)";
        if (len > limit - out.size()) return "deflate data longer than expected";
        size_t from = out.size() - d;
        for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);  // overlapping copies repeat
    }
}

std::string inflate_raw(Bits& b, std::vector<uint8_t>& out, size_t limit) {
    bool last = false;
    while (!last) {
        last = b.take(1) != 0;
        const uint32_t type = b.take(2);
        if (b.over) return "truncated deflate data";
        if (type == 0) {  // stored
            b.align();
            uint32_t len = b.take(16), nlen = b.take(16);
            if (b.over || (len ^ 0xffffu) != nlen) return "corrupt stored block";
            if (len > limit - out.size()) return "deflate data longer than expected";
            for (uint32_t i = 0; i < len; ++i) out.push_back((uint8_t)b.take(8));
            if (b.over) return "truncated stored block";
        } else if (type == 1) {  // fixed Huffman codes (RFC 1951 3.2.6)
            static const Code lit = [] {
                Code c;
                uint8_t l[288];
                for (int i = 0; i < 144; ++i) l[i] = 8;
                for (int i = 144; i < 256; ++i) l[i] = 9;
                for (int i = 256; i < 280; ++i) l[i] = 7;
                for (int i = 280; i < 288; ++i) l[i] = 8;
                build(c, l, 288);
                return c;
            }();
            static const Code dist = [] {
                Code c;
                uint8_t l[30];
                for (int i = 0; i < 30; ++i) l[i] = 5;
                build(c, l, 30);
                return c;
            }();
            std::string e = inflate_codes(b, lit, dist, out, limit);
            if (!e.empty()) return e;
        } else if (type == 2) {  // dynamic Huffman codes (RFC 1951 3.2.7)
            const int hlit = (int)b.take(5) + 257, hdist = (int)b.take(5) + 1, hclen = (int)b.take(4) + 4;
            if (hlit > 286 || hdist > 30) return "corrupt dynamic block header";
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = (uint8_t)b.take(3);
            Code clc;
            if (!build(clc, cl, 19)) return "corrupt code-length code";
            uint8_t lens[320] = {0};
            int i = 0;
            while (i < hlit + hdist) {
                int s = decode(b, clc);
                if (s < 0 || b.over) return "corrupt code lengths";
                if (s < 16) { lens[i++] = (uint8_t)s; continue; }
                int rep = 0;
                uint8_t val = 0;
                if (s == 16) {
                    if (i == 0) return "repeat with no previous length";
                    val = lens[i - 1];
                    rep = 3 + (int)b.take(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.take(3);
                } else {
                    rep = 11 + (int)b.take(7);
                }
                if (i + rep > hlit + hdist) return "code lengths overrun";
                while (rep--) lens[i++] = val;
            }
            if (lens[256] == 0) return "no end-of-block code";
            Code lit, dist;
            if (!build(lit, lens, hlit) || !build(dist, lens + hlit, hdist)) return "corrupt Huffman lengths";
            std::string e = inflate_codes(b, lit, dist, out, limit);
            if (!e.empty()) return e;
        } else {
            return "reserved deflate block type";
        }
    }
    return "";
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
    int p = a + b - c;
    int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

}  // namespace

uint32_t crc32_png(const uint8_t* p, size_t n, uint32_t crc) {
    struct Table {
        uint32_t t[256];
        Table() {
            for (uint32_t i = 0; i < 256; ++i) {
                uint32_t c = i;
                for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
                t[i] = c;
            }
        }
    };
    static const Table table;
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table.t[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}

std::string zlib_inflate(const uint8_t* data, size_t n, std::vector<uint8_t>& out, size_t limit) {
    if (n < 6) return "zlib stream too short";
    const uint8_t cmf = data[0], flg = data[1];
    if ((cmf & 0x0f) != 8 || (cmf >> 4) > 7) return "not a deflate zlib stream";
    if (((uint32_t)cmf * 256u + flg) % 31u != 0) return "bad zlib header check";
    if (flg & 0x20) return "zlib preset dictionary not supported";
    Bits b(data + 2, n - 2);
    out.clear();
    std::string e = inflate_raw(b, out, limit);
    if (!e.empty()) return e;
    b.align();
    const size_t used = 2 + b.pos - (size_t)(b.cnt / 8);
    if (used + 4 > n) return "missing zlib checksum";
    if (be32(data + used) != adler32(out.data(), out.size())) return "zlib checksum mismatch";
    return "";
}

std::string png_decode(const std::vector<uint8_t>& f, int& width, int& height, std::vector<uint8_t>& rgba) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    if (f.size() < 8 || std::memcmp(f.data(), sig, 8) != 0) return "not a PNG file";
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette, trns;
    bool seen_end = false;
    for (size_t pos = 8; pos + 12 <= f.size();) {
        const uint32_t len = be32(&f[pos]);
        if (len > f.size() - pos - 12) return "truncated PNG chunk";
        const uint8_t* type = &f[pos + 4];
        const uint8_t* data = &f[pos + 8];
        if (crc32_png(type, 4 + (size_t)len) != be32(data + len)) return "PNG chunk CRC mismatch";
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) return "bad IHDR";
            w = be32(data);
            h = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            if (data[10] != 0 || data[11] != 0) return "unknown PNG compression or filter method";
            interlace = data[12];
            if (interlace > 1) return "unknown PNG interlace method";
        } else if (!std::memcmp(type, "PLTE", 4)) {
            palette.assign(data, data + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(data, data + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            seen_end = true;
            break;
        } else if (!(type[0] & 0x20)) {
            return "unknown critical PNG chunk";
        }
        pos += 12 + (size_t)len;
    }
    if (!seen_end) return "PNG without IEND";
    if (w == 0 || h == 0 || w > (1u << 24) || h > (1u << 24) || (uint64_t)w * h > (1ull << 30)) return "bad PNG size";
    int channels = 0;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: return "unknown PNG colour type";
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok) return "bad PNG bit depth for its colour type";
    if (ctype == 3 && (palette.empty() || palette.size() % 3 != 0)) return "palette image without PLTE";
    // The filtered rows' size, from the header: the inflater stops past it
    // (a small stream cannot expand without bound), and the image is only
    // allocated once all of its rows are there.
    uint64_t need = 0;
    {
        static const uint32_t a7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                          {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
        for (int p = 0; p < (interlace ? 7 : 1); ++p) {
            const uint32_t x0 = interlace ? a7[p][0] : 0, y0 = interlace ? a7[p][1] : 0;
            const uint32_t dx = interlace ? a7[p][2] : 1, dy = interlace ? a7[p][3] : 1;
            if (x0 >= w || y0 >= h) continue;
            const uint64_t pw = (w - x0 + dx - 1) / dx, ph = (h - y0 + dy - 1) / dy;
            need += ph * (1 + (pw * channels * depth + 7) / 8);
        }
    }
    std::vector<uint8_t> raw;
    std::string e = zlib_inflate(idat.data(), idat.size(), raw, (size_t)need + 65536);
    if (!e.empty()) return e;
    if (raw.size() < need) return "truncated PNG image data";

    const int bpp = (channels * depth + 7) / 8;  // filter byte distance
    rgba.assign((size_t)w * h * 4, 0);
    // one sample of row `line` at index i (in samples), scaled to 8 bits
    auto sample = [&](const uint8_t* line, size_t i) -> uint32_t {
        if (depth == 8) return line[i];
        if (depth == 16) return ((uint32_t)line[2 * i] << 8) | line[2 * i + 1];
        const size_t bit = i * (size_t)depth;
        return (uint32_t)(line[bit >> 3] >> (8 - depth - (int)(bit & 7))) & ((1u << depth) - 1u);
    };
    auto to8 = [&](uint32_t v) -> uint8_t {
        if (depth == 16) return (uint8_t)(v >> 8);
        if (depth == 8) return (uint8_t)v;
        return (uint8_t)(v * 255u / ((1u << depth) - 1u));
    };
    auto put = [&](const uint8_t* line, uint32_t x, uint32_t px, uint32_t py) {
        uint8_t* o = &rgba[((size_t)py * w + px) * 4];
        if (ctype == 3) {
            uint32_t idx = sample(line, x);
            if (3 * (size_t)idx + 2 >= palette.size()) { o[0] = o[1] = o[2] = 0; o[3] = 255; return; }
            o[0] = palette[3 * idx]; o[1] = palette[3 * idx + 1]; o[2] = palette[3 * idx + 2];
            o[3] = idx < trns.size() ? trns[idx] : 255;
        } else if (ctype == 0 || ctype == 4) {
            uint32_t g = sample(line, (size_t)x * channels);
            o[0] = o[1] = o[2] = to8(g);
            if (ctype == 4) o[3] = to8(sample(line, (size_t)x * channels + 1));
            else o[3] = (trns.size() >= 2 && g == (((uint32_t)trns[0] << 8) | trns[1])) ? 0 : 255;
        } else {
            uint32_t r = sample(line, (size_t)x * channels), g = sample(line, (size_t)x * channels + 1),
                     b = sample(line, (size_t)x * channels + 2);
            o[0] = to8(r); o[1] = to8(g); o[2] = to8(b);
            if (ctype == 6) o[3] = to8(sample(line, (size_t)x * channels + 3));
            else o[3] = (trns.size() >= 6 && r == (((uint32_t)trns[0] << 8) | trns[1]) &&
                         g == (((uint32_t)trns[2] << 8) | trns[3]) && b == (((uint32_t)trns[4] << 8) | trns[5])) ? 0 : 255;
        }
    };
    // Adam7 passes: (x0, y0, dx, dy); a non-interlaced image is one pass
    static const uint32_t adam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                         {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const int passes = interlace ? 7 : 1;
    size_t off = 0;
    for (int p = 0; p < passes; ++p) {
        const uint32_t x0 = interlace ? adam7[p][0] : 0, y0 = interlace ? adam7[p][1] : 0;
        const uint32_t dx = interlace ? adam7[p][2] : 1, dy = interlace ? adam7[p][3] : 1;
        if (x0 >= w || y0 >= h) continue;
        const uint32_t pw = (w - x0 + dx - 1) / dx, ph = (h - y0 + dy - 1) / dy;
        const size_t stride = ((size_t)pw * channels * depth + 7) / 8;
        std::vector<uint8_t> prev(stride, 0), cur(stride);
        for (uint32_t y = 0; y < ph; ++y) {
            if (off + 1 + stride > raw.size()) return "truncated PNG image data";
            const int filter = raw[off];
            std::memcpy(cur.data(), &raw[off + 1], stride);
            off += 1 + stride;
            for (size_t i = 0; i < stride; ++i) {
                const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= (size_t)bpp ? prev[i - bpp] : 0;
                int v = cur[i];
                switch (filter) {
                    case 0: break;
                    case 1: v += a; break;
                    case 2: v += b; break;
                    case 3: v += (a + b) >> 1; break;
                    case 4: v += paeth(a, b, c); break;
                    default: return "unknown PNG filter type";
                }
                cur[i] = (uint8_t)v;
            }
            for (uint32_t x = 0; x < pw; ++x) put(cur.data(), x, x0 + x * dx, y0 + y * dy);
            std::swap(prev, cur);
        }
    }
    width = (int)w;
    height = (int)h;
    return "";
}

std::vector<uint8_t> png_encode_rgb8(const uint8_t* rgb, int w, int h) {
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    auto put32 = [](std::vector<uint8_t>& v, uint32_t x) {
        v.push_back((uint8_t)(x >> 24)); v.push_back((uint8_t)(x >> 16)); v.push_back((uint8_t)(x >> 8)); v.push_back((uint8_t)x);
    };
    auto chunk = [&](const char* type, const std::vector<uint8_t>& data) {
        put32(out, (uint32_t)data.size());
        const size_t start = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), data.begin(), data.end());
        put32(out, crc32_png(&out[start], 4 + data.size()));
    };
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    chunk("IHDR", ihdr);
    // scanlines with filter 0
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (1 + 3 * (size_t)w));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb + (size_t)y * w * 3, rgb + (size_t)(y + 1) * w * 3);
    }
    // zlib: header, stored blocks of at most 65535 bytes, Adler-32
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {
        const size_t len = raw.size() - pos < 65535 ? raw.size() - pos : 65535;
        z.push_back(pos + len == raw.size() ? 1 : 0);
        z.push_back((uint8_t)len); z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len); z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + (long)pos, raw.begin() + (long)(pos + len));
        pos += len;
    } while (pos < raw.size());
    put32(z, adler32(raw.data(), raw.size()));
    chunk("IDAT", z);
    chunk("IEND", {});
    return out;
}

}  // namespace nr
