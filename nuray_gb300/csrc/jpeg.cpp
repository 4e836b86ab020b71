// JPEG decoding for textures: the JPG branch of the reference's texture
// decode through Qt (Texture::load, src/scene/texture.cpp:5-31:
// QImage(file).convertToFormat(Format_RGBA8888), then pixelColor).
//
// ITU-T T.81 Huffman processes with 8-bit samples: baseline and extended
// sequential (SOF0, SOF1) and progressive (SOF2, spectral selection and
// successive approximation), any sampling factors up to 4, restart
// intervals, one to three components (grayscale, YCbCr, or RGB when an
// Adobe APP14 segment says so or the component ids are 'R', 'G', 'B').
// Arithmetic coding, lossless, hierarchical, 12-bit and four-component
// files are refused with an error.
//
// Reconstruction: all coefficients of the file are gathered first (both
// processes), then each block is dequantised and inverse-transformed with
// the 2-D IDCT of T.81 A.3.3 evaluated in double precision, level-shifted,
// rounded to nearest and clamped to 8 bits. Subsampled components are
// brought to full size by centred linear interpolation (weights 3/4 and
// 1/4 at 2:1, the same as libjpeg's default "fancy" upsampling up to its
// alternating rounding) and YCbCr is converted to RGB by the JFIF
// equations. Qt decodes JPEG through libjpeg, whose default integer IDCT
// and fixed-point colour conversion may differ from these by one or two
// levels on some pixels.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "image_io.h"

namespace nr {
namespace {

// zig-zag position -> row-major index within the 8x8 block
const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

const double kPi = 3.14159265358979323846;

struct JError {
    std::string msg;
};

// Canonical Huffman table (T.81 C and F.2.2.3): codes of each length are
// consecutive; a code of length l is valid when it is <= maxcode[l].
struct Huffman {
    bool defined = false;
    int32_t mincode[17], maxcode[18], valptr[17];
    uint8_t vals[256];
    // 9-bit lookahead: (length << 8) | symbol, or 0 when the code is longer
    uint16_t fast[512];
};

void build_huffman(Huffman& H, const uint8_t* counts, const uint8_t* symbols, int nsym) {
    int code = 0, k = 0;
    std::memset(H.fast, 0, sizeof(H.fast));
    for (int l = 1; l <= 16; ++l) {
        H.valptr[l] = k;
        H.mincode[l] = code;
        for (int i = 0; i < counts[l - 1]; ++i) {
            if (code >= (1 << l)) throw JError{"bad Huffman table (more codes than fit)"};
            if (l <= 9) {
                const int shift = 9 - l;
                for (int f = 0; f < (1 << shift); ++f) H.fast[(code << shift) | f] = (uint16_t)((l << 8) | symbols[k]);
            }
            ++code;
            ++k;
        }
        H.maxcode[l] = counts[l - 1] ? code - 1 : -1;
        code <<= 1;
    }
    H.maxcode[17] = INT32_MAX;
    std::memcpy(H.vals, symbols, (size_t)nsym);
    H.defined = true;
}

// Entropy-coded data: removes stuffed zero bytes, stops at markers (and
// then supplies zero bits, as decoders do for truncated data).
struct BitReader {
    const uint8_t* p;
    const uint8_t* end;
    uint32_t buf = 0;
    int nbits = 0;
    bool at_marker = false;

    void fill() {
        while (nbits <= 24) {
            uint32_t byte = 0;
            if (!at_marker && p < end) {
                byte = *p;
                if (byte == 0xFF) {
                    const uint8_t next = p + 1 < end ? p[1] : 0;
                    if (next == 0x00) {
                        p += 2;
                    } else {
                        at_marker = true;  // leave p on the marker
                        byte = 0;
                    }
                } else {
                    ++p;
                }
            }
            buf |= byte << (24 - nbits);
            nbits += 8;
        }
    }
    uint32_t peek(int n) {
        if (nbits < n) fill();
        return buf >> (32 - n);
    }
    void skip(int n) {
        buf <<= n;
        nbits -= n;
    }
    int bits(int n) {
        if (n == 0) return 0;
        const uint32_t v = peek(n);
        skip(n);
        return (int)v;
    }
    int bit() { return bits(1); }
    // receive + extend (T.81 F.2.2.1)
    int signed_bits(int s) {
        if (s == 0) return 0;
        const int v = bits(s);
        return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
    }
    int decode(const Huffman& H) {
        if (!H.defined) throw JError{"scan uses an undefined Huffman table"};
        const uint32_t look = peek(16);
        const uint16_t f = H.fast[look >> 7];
        if (f) {
            skip(f >> 8);
            return f & 0xFF;
        }
        int l = 10;
        int32_t code = (int32_t)(look >> (16 - l));
        while (l <= 16 && code > H.maxcode[l]) {
            ++l;
            code = (int32_t)(look >> (16 - l));
        }
        if (l > 16) throw JError{"bad Huffman code"};
        skip(l);
        return H.vals[H.valptr[l] + code - H.mincode[l]];
    }
    // byte-aligns and consumes the restart marker expected next
    void restart(int expected) {
        nbits = 0;
        buf = 0;
        if (at_marker && p + 1 < end && p[1] == 0xD0 + expected) {
            p += 2;
        } else {
            // tolerate a missing marker: resynchronise on the next RSTn
            while (p + 1 < end && !(p[0] == 0xFF && p[1] >= 0xD0 && p[1] <= 0xD7)) ++p;
            if (p + 1 < end) p += 2;
        }
        at_marker = false;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int td = 0, ta = 0;
    int bw = 0, bh = 0;    // blocks per row / column, padded to whole MCUs
    int cbw = 0, cbh = 0;  // blocks covering the component's own samples
    std::vector<int16_t> coef;  // bw * bh blocks of 64, row-major within a block
    int dc_pred = 0;
};

struct Decoder {
    const uint8_t* data = nullptr;
    size_t n = 0;
    size_t pos = 0;
    uint16_t qt[4][64];
    bool qt_defined[4] = {false, false, false, false};
    Huffman dc[4], ac[4];
    std::vector<Component> comps;
    int width = 0, height = 0;
    int hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool progressive = false, have_frame = false;
    int restart_interval = 0;
    int adobe_transform = -1;
    int eobrun = 0;

    int u8() {
        if (pos >= n) throw JError{"truncated JPEG"};
        return data[pos++];
    }
    int u16() {
        const int hi = u8();
        return (hi << 8) | u8();
    }

    void read_dqt(size_t end) {
        while (pos < end) {
            const int pq_tq = u8(), pq = pq_tq >> 4, tq = pq_tq & 15;
            if (tq > 3 || pq > 1) throw JError{"bad DQT"};
            for (int k = 0; k < 64; ++k) qt[tq][kZigzag[k]] = (uint16_t)(pq ? u16() : u8());
            qt_defined[tq] = true;
        }
    }
    void read_dht(size_t end) {
        while (pos < end) {
            const int tc_th = u8(), tc = tc_th >> 4, th = tc_th & 15;
            if (tc > 1 || th > 3) throw JError{"bad DHT"};
            uint8_t counts[16], syms[256];
            int total = 0;
            for (int i = 0; i < 16; ++i) total += counts[i] = (uint8_t)u8();
            if (total > 256) throw JError{"bad DHT"};
            for (int i = 0; i < total; ++i) syms[i] = (uint8_t)u8();
            build_huffman(tc ? ac[th] : dc[th], counts, syms, total);
        }
    }
    void read_sof(int marker) {
        if (have_frame) throw JError{"more than one frame"};
        if (marker != 0xC0 && marker != 0xC1 && marker != 0xC2)
            throw JError{"unsupported JPEG process (arithmetic, lossless or hierarchical)"};
        progressive = marker == 0xC2;
        if (u8() != 8) throw JError{"only 8-bit JPEG samples are supported"};
        height = u16();
        width = u16();
        const int nc = u8();
        if (width <= 0 || height <= 0) throw JError{"JPEG without dimensions (DNL) is not supported"};
        if (nc != 1 && nc != 3) throw JError{"only 1- or 3-component JPEG is supported"};
        comps.resize(nc);
        for (auto& c : comps) {
            c.id = u8();
            const int hv = u8();
            c.h = hv >> 4;
            c.v = hv & 15;
            c.tq = u8();
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) throw JError{"bad SOF"};
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        // At most 2^28 pixels (16384 x 16384), and the coefficient planes are
        // only allocated when the file can hold them: every coded block
        // takes at least one bit of entropy-coded data.
        if ((uint64_t)width * (uint64_t)height > (1ull << 28)) throw JError{"JPEG larger than 2^28 pixels"};
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        uint64_t coded_blocks = 0;
        for (auto& c : comps) {
            c.bw = mcux * c.h;
            c.bh = mcuy * c.v;
            c.cbw = ((width * c.h + hmax - 1) / hmax + 7) / 8;
            c.cbh = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            coded_blocks += (uint64_t)c.cbw * c.cbh;
        }
        if (coded_blocks > 8 * (uint64_t)(n - pos)) throw JError{"JPEG data too short for its frame size"};
        for (auto& c : comps) c.coef.assign((size_t)c.bw * c.bh * 64, 0);
        have_frame = true;
    }

    int16_t* block(Component& c, int bx, int by) { return &c.coef[((size_t)by * c.bw + bx) * 64]; }

    void decode_block_baseline(BitReader& br, Component& c, int16_t* b) {
        const int t = br.decode(dc[c.td]);
        if (t > 11) throw JError{"bad DC magnitude"};
        c.dc_pred += br.signed_bits(t);
        b[0] = (int16_t)c.dc_pred;
        for (int k = 1; k < 64;) {
            const int rs = br.decode(ac[c.ta]), r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;  // EOB
                k += 16;             // ZRL
                continue;
            }
            k += r;
            if (k > 63) throw JError{"AC coefficients past the block"};
            b[kZigzag[k]] = (int16_t)br.signed_bits(s);
            ++k;
        }
    }
    void decode_dc_first(BitReader& br, Component& c, int16_t* b, int al) {
        const int t = br.decode(dc[c.td]);
        if (t > 11) throw JError{"bad DC magnitude"};
        c.dc_pred += br.signed_bits(t);
        b[0] = (int16_t)(c.dc_pred * (1 << al));
    }
    void decode_dc_refine(BitReader& br, int16_t* b, int al) {
        if (br.bit()) b[0] = (int16_t)(b[0] | (1 << al));
    }
    void decode_ac_first(BitReader& br, Component& c, int16_t* b, int ss, int se, int al) {
        if (eobrun > 0) {
            --eobrun;
            return;
        }
        for (int k = ss; k <= se;) {
            const int rs = br.decode(ac[c.ta]), r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r < 15) {  // EOBr: this block and the next 2^r - 1 + bits end here
                    eobrun = (1 << r) - 1 + br.bits(r);
                    break;
                }
                k += 16;
                continue;
            }
            k += r;
            if (k > se) throw JError{"AC coefficients past the band"};
            b[kZigzag[k]] = (int16_t)(br.signed_bits(s) * (1 << al));
            ++k;
        }
    }
    // One correction bit for a coefficient already nonzero (T.81 G.1.2.3).
    void refine(BitReader& br, int16_t& c, int p1) {
        if (br.bit() && (c & p1) == 0) c = (int16_t)(c >= 0 ? c + p1 : c - p1);
    }
    void decode_ac_refine(BitReader& br, Component& c, int16_t* b, int ss, int se, int al) {
        const int p1 = 1 << al;
        int k = ss;
        if (eobrun == 0) {
            while (k <= se) {
                const int rs = br.decode(ac[c.ta]);
                int r = rs >> 4;
                const int s = rs & 15;
                int value = 0;
                if (s != 0) {
                    if (s != 1) throw JError{"bad refinement magnitude"};
                    value = br.bit() ? p1 : -p1;
                } else if (r != 15) {
                    eobrun = (1 << r) + br.bits(r);  // this block included
                    break;
                }
                // Skip r coefficients that are still zero, refining the
                // nonzero ones met on the way; the new coefficient (or, for
                // ZRL, the sixteenth zero) takes the next zero position.
                while (k <= se) {
                    int16_t& z = b[kZigzag[k]];
                    if (z != 0) {
                        refine(br, z, p1);
                    } else {
                        if (r == 0) {
                            if (value) z = (int16_t)value;
                            ++k;
                            break;
                        }
                        --r;
                    }
                    ++k;
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k) {
                int16_t& z = b[kZigzag[k]];
                if (z != 0) refine(br, z, p1);
            }
            --eobrun;
        }
    }

    void read_sos(size_t end) {
        if (!have_frame) throw JError{"scan before frame header"};
        const int ns = u8();
        if (ns < 1 || ns > 4) throw JError{"bad SOS"};
        std::vector<Component*> sc;
        for (int i = 0; i < ns; ++i) {
            const int id = u8(), t = u8();
            Component* c = nullptr;
            for (auto& x : comps)
                if (x.id == id) c = &x;
            if (!c) throw JError{"scan names an unknown component"};
            c->td = t >> 4;
            c->ta = t & 15;
            if (c->td > 3 || c->ta > 3) throw JError{"bad SOS table"};
            sc.push_back(c);
        }
        const int ss = u8(), se = u8(), a = u8(), ah = a >> 4, al = a & 15;
        if (pos != end) throw JError{"bad SOS length"};
        if (!progressive && (ss != 0 || se != 63 || a != 0)) throw JError{"bad sequential scan parameters"};
        if (progressive) {
            if (ss > se || se > 63 || al > 13 || (ss == 0 && se != 0) || (ss > 0 && ns != 1))
                throw JError{"bad progressive scan parameters"};
        }
        for (auto* c : sc) c->dc_pred = 0;
        eobrun = 0;

        BitReader br{data + pos, data + n};
        auto one = [&](Component& c, int bx, int by) {
            int16_t* b = block(c, bx, by);
            if (!progressive) decode_block_baseline(br, c, b);
            else if (ss == 0 && ah == 0) decode_dc_first(br, c, b, al);
            else if (ss == 0) decode_dc_refine(br, b, al);
            else if (ah == 0) decode_ac_first(br, c, b, ss, se, al);
            else decode_ac_refine(br, c, b, ss, se, al);
        };
        int rst = 0, left = restart_interval;
        auto after_mcu = [&](bool last) {
            if (restart_interval == 0 || last) return;
            if (--left == 0) {
                br.restart(rst);
                rst = (rst + 1) & 7;
                left = restart_interval;
                for (auto* c : sc) c->dc_pred = 0;
                eobrun = 0;
            }
        };
        if (ns == 1) {
            // non-interleaved: the component's own blocks in raster order
            Component& c = *sc[0];
            const int total = c.cbw * c.cbh;
            for (int i = 0; i < total; ++i) {
                one(c, i % c.cbw, i / c.cbw);
                after_mcu(i + 1 == total);
            }
        } else {
            const int total = mcux * mcuy;
            for (int m = 0; m < total; ++m) {
                const int mx = m % mcux, my = m / mcux;
                for (auto* c : sc)
                    for (int y = 0; y < c->v; ++y)
                        for (int x = 0; x < c->h; ++x) one(*c, mx * c->h + x, my * c->v + y);
                after_mcu(m + 1 == total);
            }
        }
        // continue after the entropy-coded segment: the next marker
        const uint8_t* p = br.p;
        while (p + 1 < data + n && !(p[0] == 0xFF && p[1] != 0x00 && !(p[1] >= 0xD0 && p[1] <= 0xD7))) ++p;
        pos = (size_t)(p - data);
    }

    void parse() {
        if (n < 4 || data[0] != 0xFF || data[1] != 0xD8) throw JError{"not a JPEG file"};
        pos = 2;
        while (true) {
            int b = u8();
            if (b != 0xFF) throw JError{"expected a marker"};
            int marker = u8();
            while (marker == 0xFF) marker = u8();  // fill bytes
            if (marker == 0xD9) break;            // EOI
            if (marker == 0xD8 || (marker >= 0xD0 && marker <= 0xD7) || marker == 0x01) continue;
            const int len = u16();
            if (len < 2 || pos + (size_t)len - 2 > n) throw JError{"truncated JPEG segment"};
            const size_t end = pos + (size_t)len - 2;
            if (marker == 0xDB) read_dqt(end);
            else if (marker == 0xC4) read_dht(end);
            else if (marker >= 0xC0 && marker <= 0xCF && marker != 0xC4 && marker != 0xC8 && marker != 0xCC) read_sof(marker);
            else if (marker == 0xDD) { restart_interval = u16(); }
            else if (marker == 0xDA) { read_sos(end); continue; }
            else if (marker == 0xEE && len >= 14) {  // Adobe APP14: transform flag in its last byte
                if (std::memcmp(data + pos, "Adobe", 5) == 0) adobe_transform = data[pos + 11];
            } else if (marker == 0xCC || marker == 0xC8) {
                throw JError{"arithmetic-coded JPEG is not supported"};
            } else if (marker == 0xDC) {
                throw JError{"JPEG with a DNL marker is not supported"};
            }
            pos = end;
            if (pos >= n) break;
        }
        if (!have_frame) throw JError{"JPEG without a frame"};
    }

    // dequantised IDCT of every block into an 8-bit plane per component
    void reconstruct(std::vector<std::vector<uint8_t>>& planes) {
        double cosv[8][8];  // cos((2x + 1) u pi / 16) * C(u) / 2
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                cosv[x][u] = std::cos((2 * x + 1) * u * kPi / 16.0) * (u == 0 ? std::sqrt(0.5) : 1.0) * 0.5;
        planes.resize(comps.size());
        for (size_t ci = 0; ci < comps.size(); ++ci) {
            Component& c = comps[ci];
            if (!qt_defined[c.tq]) throw JError{"component uses an undefined quantisation table"};
            const uint16_t* q = qt[c.tq];
            const int pw = c.bw * 8;
            std::vector<uint8_t>& out = planes[ci];
            out.assign((size_t)pw * c.bh * 8, 0);
            double F[64], tmp[64];
            for (int by = 0; by < c.bh; ++by)
                for (int bx = 0; bx < c.bw; ++bx) {
                    const int16_t* b = block(c, bx, by);
                    for (int k = 0; k < 64; ++k) F[k] = (double)b[k] * q[k];
                    // rows of F are v (vertical frequency), columns u
                    for (int v = 0; v < 8; ++v)
                        for (int x = 0; x < 8; ++x) {
                            double s = 0.0;
                            for (int u = 0; u < 8; ++u) s += cosv[x][u] * F[v * 8 + u];
                            tmp[v * 8 + x] = s;
                        }
                    for (int y = 0; y < 8; ++y)
                        for (int x = 0; x < 8; ++x) {
                            double s = 0.0;
                            for (int v = 0; v < 8; ++v) s += cosv[y][v] * tmp[v * 8 + x];
                            const double val = std::floor(s + 128.0 + 0.5);
                            out[(size_t)(by * 8 + y) * pw + bx * 8 + x] = (uint8_t)std::min(255.0, std::max(0.0, val));
                        }
                }
        }
    }
};

// Sample of component plane P (pw wide) at full-resolution pixel (x, y):
// centred linear interpolation between the component's samples, edges
// replicated.
uint8_t upsample(const std::vector<uint8_t>& P, int pw, int cw, int ch, int fx, int fy, int x, int y) {
    if (fx == 1 && fy == 1) return P[(size_t)y * pw + x];
    auto axis = [](int i, int f, int n, int& i0, int& i1, double& w1) {
        if (f == 1) {
            i0 = i1 = i;
            w1 = 0.0;
            return;
        }
        const double s = (i + 0.5) / f - 0.5;
        const double fl = std::floor(s);
        i0 = (int)fl;
        w1 = s - fl;
        i1 = i0 + 1;
        i0 = std::min(std::max(i0, 0), n - 1);
        i1 = std::min(std::max(i1, 0), n - 1);
    };
    int x0, x1, y0, y1;
    double wx, wy;
    axis(x, fx, cw, x0, x1, wx);
    axis(y, fy, ch, y0, y1, wy);
    auto at = [&](int xx, int yy) { return (double)P[(size_t)yy * pw + xx]; };
    const double top = at(x0, y0) * (1.0 - wx) + at(x1, y0) * wx;
    const double bot = at(x0, y1) * (1.0 - wx) + at(x1, y1) * wx;
    const double v = top * (1.0 - wy) + bot * wy;
    return (uint8_t)std::min(255.0, std::max(0.0, std::floor(v + 0.5)));
}

uint8_t clamp8(double v) { return (uint8_t)std::min(255.0, std::max(0.0, std::floor(v + 0.5))); }

}  // namespace

std::string jpeg_decode(const std::vector<uint8_t>& file, int& width, int& height, std::vector<uint8_t>& rgb) {
    try {
        Decoder D;
        D.data = file.data();
        D.n = file.size();
        D.parse();
        std::vector<std::vector<uint8_t>> planes;
        D.reconstruct(planes);
        width = D.width;
        height = D.height;
        rgb.assign((size_t)width * height * 3, 0);
        const size_t nc = D.comps.size();
        bool is_rgb = false;
        if (nc == 3) {
            if (D.adobe_transform >= 0) is_rgb = D.adobe_transform == 0;
            else is_rgb = D.comps[0].id == 'R' && D.comps[1].id == 'G' && D.comps[2].id == 'B';
        }
        int fx[3], fy[3], cw[3], ch[3];
        for (size_t c = 0; c < nc; ++c) {
            const Component& C = D.comps[c];
            fx[c] = D.hmax / C.h;
            fy[c] = D.vmax / C.v;
            if (fx[c] * C.h != D.hmax || fy[c] * C.v != D.vmax)
                throw JError{"sampling factors that do not divide the maximum are not supported"};
            cw[c] = (width * C.h + D.hmax - 1) / D.hmax;
            ch[c] = (height * C.v + D.vmax - 1) / D.vmax;
        }
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                double s[3];
                for (size_t c = 0; c < nc; ++c)
                    s[c] = upsample(planes[c], D.comps[c].bw * 8, cw[c], ch[c], fx[c], fy[c], x, y);
                uint8_t* o = &rgb[((size_t)y * width + x) * 3];
                if (nc == 1) {
                    o[0] = o[1] = o[2] = (uint8_t)s[0];
                } else if (is_rgb) {
                    o[0] = (uint8_t)s[0];
                    o[1] = (uint8_t)s[1];
                    o[2] = (uint8_t)s[2];
                } else {  // JFIF YCbCr -> RGB
                    const double Y = s[0], cb = s[1] - 128.0, cr = s[2] - 128.0;
                    o[0] = clamp8(Y + 1.402 * cr);
                    o[1] = clamp8(Y - 0.344136 * cb - 0.714136 * cr);
                    o[2] = clamp8(Y + 1.772 * cb);
                }
            }
        return "";
    } catch (const JError& e) {
        return e.msg;
    }
}

}  // namespace nr
