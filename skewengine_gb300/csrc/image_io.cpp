// Image input/output of the reference's image operators (kernelRADN, kernelBLUR):
// PNG reading and writing and the colourings its result writers apply.
//
//  * Reading: the reference loads its input with helper::read_png
//    (src/helper.h:167-184): the file decoded to 8-bit RGBA by its vendored PNG
//    library, then one value per pixel, R + G + B, used as the grid value
//    (configureRADN / configureCEPS, src/kernelRADN.h:77-87,
//    src/kernelBLUR.h:46-56).  The decoder here is written from the PNG
//    specification (ISO/IEC 15948) and DEFLATE/zlib (RFC 1950, RFC 1951): every
//    colour type and bit depth, both filter methods' five scanline filters,
//    Adam7 interlacing, tRNS transparency, CRC-32 and Adler-32 checks.  Its RGBA
//    conversion is the reference library's: samples of fewer than 8 bits scale
//    by 255 / (2^bits - 1), 16-bit samples keep their high byte, a colour equal
//    to the tRNS key gets alpha 0, palette indices past the palette are opaque
//    black.
//  * Writing: 8-bit grey or RGB, scanline filter 0, zlib stored blocks.  The
//    reference writes the same pixels compressed (salida1.png, salida2.png);
//    the decoded images are identical.
//  * Colourings (showResults, src/main.h:124-141; showResultsRADN,
//    src/kernelRADN.h:384-400; showResultsCEPS, src/kernelBLUR.h:396-410;
//    HSVtoRGB, src/color.cpp:80-115) restated with the reference's float
//    arithmetic and conversions.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/skewengine.h"
#include "image_io.h"

namespace {

// An image entry point's failure: the reason (and the file) become the calling
// thread's last error (ske_last_error).
int image_error(int code, const char* what, const char* path = nullptr) {
    std::string m = what;
    if (path) {
        m += ": ";
        m += path;
    }
    return ske::set_last_error(code, m.c_str());
}

// Largest image decoded: 2^31 pixels (8 GiB of RGBA).
constexpr uint64_t kMaxPixels = (uint64_t)1 << 31;

// ---------------------------------------------------------------- checksums
struct CrcTable {
    uint32_t v[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            v[i] = c;
        }
    }
};

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
    static const CrcTable table;  // initialised once, thread-safe
    crc ^= 0xffffffffu;
    for (size_t i = 0; i < n; i++) crc = table.v[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return crc ^ 0xffffffffu;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; i++) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ---------------------------------------------------------------- inflate
struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool overrun = false;
    int bits(int need) {
        while (cnt < need) {
            if (pos >= n) {
                overrun = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const int v = (int)(buf & ((1u << need) - 1u));
        buf >>= need;
        cnt -= need;
        return v;
    }
};

// Canonical Huffman code: counts per length and symbols in code order.
struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
};

// Returns false for an over-subscribed code (incomplete codes are allowed, as
// RFC 1951 permits for single-code distance trees).
bool build_huffman(Huffman& h, const uint8_t* lengths, int n) {
    memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; i++) h.count[lengths[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; len++) {
        left <<= 1;
        left -= h.count[len];
        if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; len++) offs[len + 1] = (uint16_t)(offs[len] + h.count[len]);
    for (int i = 0; i < n; i++)
        if (lengths[i]) h.symbol[offs[lengths[i]]++] = (uint16_t)i;
    return true;
}

// Decode one symbol, reading the code bit by bit (codes are stored MSB first).
int decode_symbol(BitReader& br, const Huffman& h) {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; len++) {
        code |= br.bits(1);
        if (br.overrun) return -1;
        const int c = h.count[len];
        if (code - c < first) return h.symbol[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return -1;
}

// RFC 1951 section 3.2.5: base lengths / distances and their extra bits.
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59,
                               67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitReader& br, std::vector<uint8_t>& out, const Huffman& lit, const Huffman& dist, size_t limit) {
    for (;;) {
        int sym = decode_symbol(br, lit);
        if (sym < 0) return false;
        if (sym < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) return false;
            const int len = kLenBase[sym] + br.bits(kLenExtra[sym]);
            const int ds = decode_symbol(br, dist);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = (size_t)kDistBase[ds] + (size_t)br.bits(kDistExtra[ds]);
            if (br.overrun || d > out.size()) return false;
            if (out.size() + len > limit) return false;
            const size_t from = out.size() - d;
            for (int i = 0; i < len; i++) out.push_back(out[from + i]);
        }
    }
}

// Stops (false) once the output would exceed `limit` bytes.
bool inflate(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit) {
    BitReader br{in, n};
    int last;
    do {
        last = br.bits(1);
        const int type = br.bits(2);
        if (br.overrun) return false;
        if (type == 0) {  // stored
            br.buf = 0;
            br.cnt = 0;
            if (br.pos + 4 > n) return false;
            const unsigned len = in[br.pos] | in[br.pos + 1] << 8;
            const unsigned nlen = in[br.pos + 2] | in[br.pos + 3] << 8;
            br.pos += 4;
            if ((len ^ 0xffffu) != nlen || br.pos + len > n) return false;
            if (out.size() + len > limit) return false;
            out.insert(out.end(), in + br.pos, in + br.pos + len);
            br.pos += len;
        } else if (type == 1) {  // fixed codes (RFC 1951 section 3.2.6)
            uint8_t l[288 + 30];
            for (int i = 0; i < 144; i++) l[i] = 8;
            for (int i = 144; i < 256; i++) l[i] = 9;
            for (int i = 256; i < 280; i++) l[i] = 7;
            for (int i = 280; i < 288; i++) l[i] = 8;
            for (int i = 0; i < 30; i++) l[288 + i] = 5;
            Huffman lit, dist;
            build_huffman(lit, l, 288);
            build_huffman(dist, l + 288, 30);
            if (!inflate_codes(br, out, lit, dist, limit)) return false;
        } else if (type == 2) {  // dynamic codes (RFC 1951 section 3.2.7)
            const int hlit = br.bits(5) + 257, hdist = br.bits(5) + 1, hclen = br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (br.overrun || hlit > 286 || hdist > 30 || !build_huffman(clh, cl, 19)) return false;
            uint8_t l[286 + 30];
            int i = 0;
            while (i < hlit + hdist) {
                const int sym = decode_symbol(br, clh);
                if (sym < 0) return false;
                if (sym < 16) {
                    l[i++] = (uint8_t)sym;
                    continue;
                }
                int rep;
                uint8_t val = 0;
                if (sym == 16) {
                    if (i == 0) return false;
                    val = l[i - 1];
                    rep = 3 + br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + br.bits(3);
                } else {
                    rep = 11 + br.bits(7);
                }
                if (br.overrun || i + rep > hlit + hdist) return false;
                while (rep--) l[i++] = val;
            }
            if (l[256] == 0) return false;  // no end-of-block code
            Huffman lit, dist;
            if (!build_huffman(lit, l, hlit) || !build_huffman(dist, l + hlit, hdist)) return false;
            if (!inflate_codes(br, out, lit, dist, limit)) return false;
        } else {
            return false;
        }
    } while (!last);
    return true;
}

bool zlib_decompress(const std::vector<uint8_t>& z, std::vector<uint8_t>& out, size_t limit) {
    if (z.size() < 6) return false;
    const unsigned cmf = z[0], flg = z[1];
    if ((cmf & 0x0fu) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20u)) return false;
    if (!inflate(z.data() + 2, z.size() - 6, out, limit)) return false;
    return adler32(out.data(), out.size()) == be32(z.data() + z.size() - 4);
}

// ---------------------------------------------------------------- PNG decode
struct PngImage {
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> palette;  // RGBA entries
    bool key = false;
    uint16_t key_r = 0, key_g = 0, key_b = 0;
};

int channels_of(int ctype) { return ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : 4; }

bool valid_depth(int ctype, int d) {
    switch (ctype) {
        case 0: return d == 1 || d == 2 || d == 4 || d == 8 || d == 16;
        case 3: return d == 1 || d == 2 || d == 4 || d == 8;
        case 2:
        case 4:
        case 6: return d == 8 || d == 16;
        default: return false;
    }
}

uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c, pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

// Undo the scanline filters of one (sub)image of w x h pixels in place; data
// holds h rows of 1 + stride bytes.  bpp: bytes per complete pixel (>= 1).
bool unfilter(uint8_t* data, size_t stride, uint32_t h, int bpp, std::vector<uint8_t>& rows) {
    rows.assign((size_t)h * stride, 0);
    const uint8_t* prev = nullptr;
    for (uint32_t y = 0; y < h; y++) {
        const uint8_t ft = data[(size_t)y * (stride + 1)];
        const uint8_t* in = data + (size_t)y * (stride + 1) + 1;
        uint8_t* out = rows.data() + (size_t)y * stride;
        for (size_t i = 0; i < stride; i++) {
            const int a = i >= (size_t)bpp ? out[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v = in[i];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return false;
            }
            out[i] = (uint8_t)v;
        }
        prev = out;
    }
    return true;
}

// Sample of `bits` bits at sample index k of a row (MSB-first packing).
unsigned sample_at(const uint8_t* row, size_t k, int bits) {
    if (bits == 8) return row[k];
    if (bits == 16) return (unsigned)row[2 * k] << 8 | row[2 * k + 1];
    const size_t bit = k * bits;
    return (row[bit >> 3] >> (8 - bits - (bit & 7))) & ((1u << bits) - 1u);
}

void to_rgba(const PngImage& im, const uint8_t* row, uint32_t x, uint8_t* o) {
    const int d = im.depth;
    switch (im.ctype) {
        case 0: {
            const unsigned v = sample_at(row, x, d);
            o[0] = o[1] = o[2] = (uint8_t)(d == 16 ? v >> 8 : d == 8 ? v : v * 255u / ((1u << d) - 1u));
            o[3] = (im.key && v == im.key_r) ? 0 : 255;
            break;
        }
        case 2: {
            const unsigned r = sample_at(row, 3 * (size_t)x, d), g = sample_at(row, 3 * (size_t)x + 1, d),
                           b = sample_at(row, 3 * (size_t)x + 2, d);
            const int sh = d == 16 ? 8 : 0;
            o[0] = (uint8_t)(r >> sh);
            o[1] = (uint8_t)(g >> sh);
            o[2] = (uint8_t)(b >> sh);
            o[3] = (im.key && r == im.key_r && g == im.key_g && b == im.key_b) ? 0 : 255;
            break;
        }
        case 3: {
            const unsigned i = sample_at(row, x, d);
            if ((size_t)i * 4 + 3 < im.palette.size()) {
                memcpy(o, im.palette.data() + (size_t)i * 4, 4);
            } else {
                o[0] = o[1] = o[2] = 0;
                o[3] = 255;
            }
            break;
        }
        case 4: {
            const int sh = d == 16 ? 8 : 0;
            o[0] = o[1] = o[2] = (uint8_t)(sample_at(row, 2 * (size_t)x, d) >> sh);
            o[3] = (uint8_t)(sample_at(row, 2 * (size_t)x + 1, d) >> sh);
            break;
        }
        default: {
            const int sh = d == 16 ? 8 : 0;
            for (int c = 0; c < 4; c++) o[c] = (uint8_t)(sample_at(row, 4 * (size_t)x + c, d) >> sh);
        }
    }
}

int read_file(const char* path, std::vector<uint8_t>& bytes) {
    FILE* f = fopen(path, "rb");
    if (!f) return SKE_ERR_INVALID;
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (n < 0) {
        fclose(f);
        return SKE_ERR_INVALID;
    }
    bytes.resize((size_t)n);
    const size_t got = n ? fread(bytes.data(), 1, (size_t)n, f) : 0;
    fclose(f);
    return got == (size_t)n ? SKE_OK : SKE_ERR_INVALID;
}

// Parse the chunks; with rgba set, also decode the pixels (8-bit RGBA).
int png_decode(const std::vector<uint8_t>& f, PngImage& im, std::vector<uint8_t>* rgba) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (f.size() < 8 || memcmp(f.data(), sig, 8) != 0) return SKE_ERR_INVALID;
    std::vector<uint8_t> idat;
    bool have_hdr = false, have_end = false;
    size_t pos = 8;
    while (pos + 12 <= f.size() && !have_end) {
        const uint32_t len = be32(f.data() + pos);
        if (len > f.size() - pos - 12) return SKE_ERR_INVALID;
        const uint8_t* type = f.data() + pos + 4;
        const uint8_t* data = type + 4;
        if (crc32_update(0, type, (size_t)len + 4) != be32(data + len)) return SKE_ERR_INVALID;
        if (!memcmp(type, "IHDR", 4)) {
            if (len != 13) return SKE_ERR_INVALID;
            im.w = be32(data);
            im.h = be32(data + 4);
            im.depth = data[8];
            im.ctype = data[9];
            im.interlace = data[12];
            if (!im.w || !im.h || !valid_depth(im.ctype, im.depth) || data[10] || data[11] || im.interlace > 1)
                return SKE_ERR_INVALID;
            have_hdr = true;
        } else if (!memcmp(type, "PLTE", 4)) {
            if (len % 3 || len > 768) return SKE_ERR_INVALID;
            im.palette.assign((size_t)len / 3 * 4, 255);
            for (uint32_t i = 0; i < len / 3; i++) memcpy(im.palette.data() + 4 * i, data + 3 * i, 3);
        } else if (!memcmp(type, "tRNS", 4)) {
            if (im.ctype == 3) {
                if (len > im.palette.size() / 4) return SKE_ERR_INVALID;
                for (uint32_t i = 0; i < len; i++) im.palette[4 * i + 3] = data[i];
            } else if (im.ctype == 0 && len == 2) {
                im.key = true;
                im.key_r = (uint16_t)(data[0] << 8 | data[1]);
            } else if (im.ctype == 2 && len == 6) {
                im.key = true;
                im.key_r = (uint16_t)(data[0] << 8 | data[1]);
                im.key_g = (uint16_t)(data[2] << 8 | data[3]);
                im.key_b = (uint16_t)(data[4] << 8 | data[5]);
            } else {
                return SKE_ERR_INVALID;
            }
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!memcmp(type, "IEND", 4)) {
            have_end = true;
        } else if (!(type[0] & 0x20)) {
            return SKE_ERR_INVALID;  // unknown critical chunk
        }
        pos += (size_t)len + 12;
    }
    if (!have_hdr || !have_end || idat.empty()) return SKE_ERR_INVALID;
    if (im.ctype == 3 && im.palette.empty()) return SKE_ERR_INVALID;
    if (!rgba) return SKE_OK;
    if ((uint64_t)im.w * im.h > kMaxPixels) return SKE_ERR_INVALID;

    const int bits_pp = channels_of(im.ctype) * im.depth;
    const int bpp = bits_pp < 8 ? 1 : bits_pp / 8;
    // The filtered scanlines' size follows from the header: decompress no more.
    size_t expect = 0;
    for (int p = 0; p < (im.interlace ? 7 : 1); p++) {
        static const int sx0[7] = {0, 4, 0, 2, 0, 1, 0}, sy0[7] = {0, 0, 4, 0, 2, 0, 1};
        static const int sdx[7] = {8, 8, 4, 4, 2, 2, 1}, sdy[7] = {8, 8, 8, 4, 4, 2, 2};
        const uint32_t x0 = im.interlace ? sx0[p] : 0, y0 = im.interlace ? sy0[p] : 0;
        const uint32_t dx = im.interlace ? sdx[p] : 1, dy = im.interlace ? sdy[p] : 1;
        if (im.w <= x0 || im.h <= y0) continue;
        const uint64_t pw = (im.w - x0 + dx - 1) / dx, ph = (im.h - y0 + dy - 1) / dy;
        expect += (size_t)((pw * bits_pp + 7) / 8 + 1) * ph;
    }
    std::vector<uint8_t> raw;
    if (!zlib_decompress(idat, raw, expect)) return SKE_ERR_INVALID;
    // Short scanline data fails the pass checks below in any case; refusing it
    // here keeps a damaged file from sizing the RGBA buffer by its header alone.
    if (raw.size() != expect) return SKE_ERR_INVALID;
    rgba->assign((size_t)im.w * im.h * 4, 0);
    // Adam7 passes (PNG specification 8.2): start and step in x and y.
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    const int passes = im.interlace ? 7 : 1;
    size_t off = 0;
    std::vector<uint8_t> rows;
    for (int p = 0; p < passes; p++) {
        const uint32_t x0 = im.interlace ? ax0[p] : 0, y0 = im.interlace ? ay0[p] : 0;
        const uint32_t dx = im.interlace ? adx[p] : 1, dy = im.interlace ? ady[p] : 1;
        if (im.w <= x0 || im.h <= y0) continue;
        const uint32_t pw = (im.w - x0 + dx - 1) / dx, ph = (im.h - y0 + dy - 1) / dy;
        const size_t stride = ((size_t)pw * bits_pp + 7) / 8;
        if (off + (stride + 1) * ph > raw.size()) return SKE_ERR_INVALID;
        if (!unfilter(raw.data() + off, stride, ph, bpp, rows)) return SKE_ERR_INVALID;
        off += (stride + 1) * ph;
        for (uint32_t y = 0; y < ph; y++)
            for (uint32_t x = 0; x < pw; x++)
                to_rgba(im, rows.data() + (size_t)y * stride, x,
                        rgba->data() + (((size_t)(y0 + y * dy) * im.w) + x0 + x * dx) * 4);
    }
    return SKE_OK;
}

int png_load(const char* path, PngImage& im, std::vector<uint8_t>* rgba) {
    if (!path) return SKE_ERR_INVALID;
    std::vector<uint8_t> f;
    const int rc = read_file(path, f);
    return rc != SKE_OK ? rc : png_decode(f, im, rgba);
}

// ---------------------------------------------------------------- PNG encode
void put32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void put_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
    put32(out, (uint32_t)data.size());
    const size_t at = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    put32(out, crc32_update(0, out.data() + at, data.size() + 4));
}

// ---------------------------------------------------------------- colourings
// getMinMax (src/helper.h:190-201): min starts at FLT_MAX, max at FLT_MIN (the
// smallest positive float, so an all-negative grid reports that as its max).
void min_max(const float* d, size_t n, float* mn, float* mx) {
    float lo = 3.40282347e+38f, hi = 1.17549435e-38f;
    for (size_t i = 0; i < n; i++) {
        lo = d[i] < lo ? d[i] : lo;
        hi = d[i] > hi ? d[i] : hi;
    }
    *mn = lo;
    *mx = hi;
}

// The reference converts a float to unsigned char; on its x86-64 build that is
// a truncation to int followed by the low byte.
uint8_t to_u8(float v) { return (uint8_t)(int)v; }

}  // namespace

namespace ske {

int png_read_grid(const char* path, int* width, int* height, std::vector<float>& grid) {
    PngImage im;
    std::vector<uint8_t> px;
    const int rc = png_load(path, im, &px);
    if (rc != SKE_OK) return rc;
    if (im.w > 0x7fffffffu || im.h > 0x7fffffffu) return SKE_ERR_INVALID;
    *width = (int)im.w;
    *height = (int)im.h;
    const size_t n = (size_t)im.w * im.h;
    grid.resize(n);
    // read_png: pixels[i] = R + G + B (a short); the grid value is that number.
    for (size_t i = 0; i < n; i++) grid[i] = (float)(short)(px[4 * i] + px[4 * i + 1] + px[4 * i + 2]);
    return SKE_OK;
}

}  // namespace ske

extern "C" {

void ske_hsv_to_rgb(float H, float S, float V, uint8_t* rgb) {
    // src/color.cpp:80-115.  The reference calls abs() with only <cmath>
    // included, which resolves to the C library's int abs: the argument
    // fmod(H/60, 2) - 1 is truncated to an integer first, so X is 0 when H/60 is
    // an even integer and C otherwise.
    if (H > 360 || H < 0 || S > 100 || S < 0 || V > 100 || V < 0) {
        rgb[0] = rgb[1] = rgb[2] = 0;
        return;
    }
    const float s = S / 100, v = V / 100;
    const float C = s * v;
    const int t = (int)(std::fmod(H / 60.0, 2) - 1);
    const float X = (float)(C * (1 - abs(t)));
    const float m = v - C;
    float r, g, b;
    if (H >= 0 && H < 60) r = C, g = X, b = 0;
    else if (H >= 60 && H < 120) r = X, g = C, b = 0;
    else if (H >= 120 && H < 180) r = 0, g = C, b = X;
    else if (H >= 180 && H < 240) r = 0, g = X, b = C;
    else if (H >= 240 && H < 300) r = X, g = 0, b = C;
    else r = C, g = 0, b = X;
    rgb[0] = (uint8_t)(int)((r + m) * 255);
    rgb[1] = (uint8_t)(int)((g + m) * 255);
    rgb[2] = (uint8_t)(int)((b + m) * 255);
}

int ske_png_size(const char* path, int* width, int* height) {
    if (!width || !height) return image_error(SKE_ERR_INVALID, "png_size: null width or height");
    try {
        PngImage im;
        const int rc = png_load(path, im, nullptr);
        if (rc != SKE_OK) return image_error(rc, "png_size: not a readable PNG file", path);
        // The size of an image the decoder takes (at most 2^31 pixels): a
        // caller sizes its buffers from it.
        if (im.w > 0x7fffffffu || im.h > 0x7fffffffu || (uint64_t)im.w * im.h > kMaxPixels)
            return image_error(SKE_ERR_INVALID, "png_size: more than 2^31 pixels", path);
        *width = (int)im.w;
        *height = (int)im.h;
        return SKE_OK;
    } catch (const std::exception&) {  // allocation failure: no exception crosses the C ABI
        return image_error(SKE_ERR_INVALID, "png_size: out of host memory", path);
    }
}

int ske_png_read_rgba(const char* path, uint8_t* rgba, size_t capacity) {
    if (!rgba) return image_error(SKE_ERR_INVALID, "png_read_rgba: null buffer");
    try {
        PngImage im;
        std::vector<uint8_t> px;
        const int rc = png_load(path, im, &px);
        if (rc != SKE_OK) return image_error(rc, "png_read_rgba: not a readable PNG file", path);
        if (px.size() > capacity) return image_error(SKE_ERR_INVALID, "png_read_rgba: buffer smaller than the image", path);
        memcpy(rgba, px.data(), px.size());
        return SKE_OK;
    } catch (const std::exception&) {
        return image_error(SKE_ERR_INVALID, "png_read_rgba: out of host memory", path);
    }
}

int ske_png_read_image(const char* path, float* image, size_t capacity) {
    if (!image) return image_error(SKE_ERR_INVALID, "png_read_image: null buffer");
    try {
        PngImage im;
        std::vector<uint8_t> px;
        const int rc = png_load(path, im, &px);
        if (rc != SKE_OK) return image_error(rc, "png_read_image: not a readable PNG file", path);
        const size_t n = (size_t)im.w * im.h;
        if (n > capacity) return image_error(SKE_ERR_INVALID, "png_read_image: buffer smaller than the image", path);
        // read_png: pixels[i] = R + G + B (a short); the grid value is that number.
        for (size_t i = 0; i < n; i++) image[i] = (float)(short)(px[4 * i] + px[4 * i + 1] + px[4 * i + 2]);
        return SKE_OK;
    } catch (const std::exception&) {
        return image_error(SKE_ERR_INVALID, "png_read_image: out of host memory", path);
    }
}

int ske_png_write(const char* path, const uint8_t* pixels, int width, int height, int channels) try {
    if (!path || !pixels || width <= 0 || height <= 0 || (channels != 1 && channels != 3))
        return image_error(SKE_ERR_INVALID, "png_write: bad argument (null, size, or channels not 1 or 3)");
    const size_t stride = (size_t)width * channels;
    std::vector<uint8_t> raw;
    raw.reserve((stride + 1) * height);
    for (int y = 0; y < height; y++) {
        raw.push_back(0);  // filter type None
        raw.insert(raw.end(), pixels + (size_t)y * stride, pixels + (size_t)(y + 1) * stride);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t at = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - at);
        z.push_back(at + len == raw.size() ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + at, raw.begin() + at + len);
        at += len;
    } while (at < raw.size());
    put32(z, adler32(raw.data(), raw.size()));
    std::vector<uint8_t> out = {137, 80, 78, 71, 13, 10, 26, 10}, hdr;
    put32(hdr, (uint32_t)width);
    put32(hdr, (uint32_t)height);
    hdr.push_back(8);
    hdr.push_back(channels == 1 ? 0 : 2);
    hdr.push_back(0);
    hdr.push_back(0);
    hdr.push_back(0);
    put_chunk(out, "IHDR", hdr);
    put_chunk(out, "IDAT", z);
    put_chunk(out, "IEND", {});
    FILE* f = fopen(path, "wb");
    if (!f) return image_error(SKE_ERR_INVALID, "png_write: cannot open", path);
    const size_t put = fwrite(out.data(), 1, out.size(), f);
    const int closed = fclose(f);
    return (put == out.size() && closed == 0) ? SKE_OK : image_error(SKE_ERR_INVALID, "png_write: cannot write", path);
} catch (const std::exception&) {  // allocation failure: no exception crosses the C ABI
    return image_error(SKE_ERR_INVALID, "png_write: out of host memory", path);
}

int ske_render_input(const float* image, int count, uint8_t* grey) {
    if (!image || !grey || count < 0) return image_error(SKE_ERR_INVALID, "render_input: bad argument");
    // grey.push_back(pixels[i] / 3): integer division of the R + G + B sum.
    for (int i = 0; i < count; i++) grey[i] = (uint8_t)((short)image[i] / 3);
    return SKE_OK;
}

int ske_render(int kernel, const float* out, int dimx, int dimy, uint8_t* rgb) {
    if (!out || !rgb || dimx <= 0 || dimy <= 0) return image_error(SKE_ERR_INVALID, "render: bad argument");
    const size_t n = (size_t)dimx * dimy;
    switch (kernel) {
        case SKE_KERNEL_RADON:
        case SKE_KERNEL_LOCAL_RADON:
        case SKE_KERNEL_IDENTITYIMG: {
            // showResults -> showResultsRADN: Radon with the automatic grey scale
            // 255 / (max - min) and shift min, the image identity with 1/540.
            float mn, mx;
            min_max(out, n, &mn, &mx);
            const bool radon = kernel != SKE_KERNEL_IDENTITYIMG;
            const float escala = radon ? 255 / (mx - mn) : (float)(1.0 / 540);
            const float shift = radon ? mn : 0.0f;
            for (size_t i = 0; i < n; i++) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = to_u8((int)(out[i] - shift) * escala);
            return SKE_OK;
        }
        case SKE_KERNEL_IDENTITYDEM:
        case SKE_KERNEL_CEPSTRUM: {
            // showResultsCEPS: hue = the output's integer part mod 360, value
            // min(100, out / 3000) (identity) or min(100, out / (180 * 3000)).
            const float div = kernel == SKE_KERNEL_CEPSTRUM ? 180 * 3000.0f : 3000.0f;
            for (size_t i = 0; i < n; i++) {
                const float v = out[i] / div;
                ske_hsv_to_rgb((float)(((int)out[i]) % 360), 100.0f, v < 100.0f ? v : 100.0f, rgb + 3 * i);
            }
            return SKE_OK;
        }
        default:  // the reference renders no image of a viewshed (it writes floats)
            return image_error(SKE_ERR_INVALID, "render: no image for this operator (a viewshed is written as floats)");
    }
}

}  // extern "C"
