// png.cpp — PNG decoding for texture images.
//
// The reference loads textures with stb_image (texturedata.cpp:30-48), asking
// for the file's channel count with 3 widened to 4; 16-bit samples keep their
// high byte, low bit depths are scaled to 8 bits, palettes expand to RGB or
// RGBA (with a tRNS chunk).  This decoder produces the same 8-bit texels from
// the PNG specification (RFC 1950/1951 zlib + deflate, the five scanline
// filters, Adam7 interlace).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "png.h"

namespace pt {
namespace host {

namespace {

struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool ok = true;
    uint32_t bits(int k)
    {
        while (bitcnt < k) {
            if (pos >= n) {
                ok = false;
                return 0;
            }
            bitbuf |= (uint32_t)p[pos++] << bitcnt;
            bitcnt += 8;
        }
        uint32_t v = bitbuf & ((1u << k) - 1u);
        bitbuf >>= k;
        bitcnt -= k;
        return v;
    }
    void align()
    {
        bitbuf = 0;
        bitcnt = 0;
    }
};

// Canonical Huffman code (RFC 1951 3.2.2): counts per length, symbols sorted.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t* lengths, int n)
    {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++)
            count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= count[len];
            if (left < 0)
                return false; // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++)
            offs[len + 1] = (uint16_t)(offs[len] + count[len]);
        symbol.assign(n, 0);
        for (int i = 0; i < n; i++)
            if (lengths[i])
                symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader& br) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= (int)br.bits(1);
            int c = count[len];
            if (code - c < first)
                return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (!br.ok)
                return -1;
        }
        return -1;
    }
};

const uint16_t LEN_BASE[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit)
{
    while (true) {
        int sym = lit.decode(br);
        if (sym < 0)
            return false;
        if (sym < 256) {
            if (out.size() >= limit)
                return false;
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29)
                return false;
            size_t len = LEN_BASE[sym] + br.bits(LEN_EXTRA[sym]);
            int ds = dist.decode(br);
            if (ds < 0 || ds >= 30)
                return false;
            size_t d = DIST_BASE[ds] + br.bits(DIST_EXTRA[ds]);
            if (!br.ok || d > out.size() || out.size() + len > limit)
                return false;
            size_t from = out.size() - d;
            for (size_t k = 0; k < len; k++)
                out.push_back(out[from + k]);
        }
    }
}

// zlib stream -> bytes (at most `limit`).
bool zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t limit, std::string& err)
{
    if (n < 2 || (p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) {
        err = "PNG: bad zlib header";
        return false;
    }
    BitReader br{p + 2, n - 2};
    bool last = false;
    while (!last) {
        last = br.bits(1) != 0;
        uint32_t type = br.bits(2);
        if (!br.ok)
            break;
        if (type == 0) {
            br.align();
            if (br.pos + 4 > br.n) {
                err = "PNG: truncated stored block";
                return false;
            }
            uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            uint32_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || br.pos + len > br.n || out.size() + len > limit) {
                err = "PNG: bad stored block";
                return false;
            }
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; i++)
                l[i] = 8;
            for (int i = 144; i < 256; i++)
                l[i] = 9;
            for (int i = 256; i < 280; i++)
                l[i] = 7;
            for (int i = 280; i < 288; i++)
                l[i] = 8;
            for (int i = 0; i < 30; i++)
                d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            if (!inflate_block(br, lit, dist, out, limit)) {
                err = "PNG: corrupt deflate data";
                return false;
            }
        } else if (type == 2) {
            int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; i++)
                cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) {
                err = "PNG: bad code-length code";
                return false;
            }
            uint8_t lens[320] = {};
            int k = 0;
            while (k < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 0) {
                    err = "PNG: corrupt code lengths";
                    return false;
                }
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) {
                            err = "PNG: repeat without a length";
                            return false;
                        }
                        val = lens[k - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (k + rep > hlit + hdist) {
                        err = "PNG: code lengths overflow";
                        return false;
                    }
                    while (rep--)
                        lens[k++] = val;
                }
            }
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist) ||
                !inflate_block(br, lit, dist, out, limit)) {
                err = "PNG: corrupt deflate data";
                return false;
            }
        } else {
            err = "PNG: reserved deflate block type";
            return false;
        }
    }
    if (!br.ok) {
        err = "PNG: truncated deflate data";
        return false;
    }
    return true;
}

uint32_t be32(const uint8_t* p)
{
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

int paeth(int a, int b, int c)
{
    int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc)
        return a;
    return pb <= pc ? b : c;
}

// Reverses the scanline filters of one (sub)image in place; rows of `stride` bytes.
bool unfilter(uint8_t* data, uint32_t rows, size_t stride, size_t bpp, std::vector<uint8_t>& out)
{
    out.assign((size_t)rows * stride, 0);
    const uint8_t* src = data;
    for (uint32_t y = 0; y < rows; y++) {
        uint8_t ft = *src++;
        uint8_t* row = out.data() + (size_t)y * stride;
        const uint8_t* prev = y ? row - stride : nullptr;
        for (size_t i = 0; i < stride; i++) {
            int a = i >= bpp ? row[i - bpp] : 0;
            int b = prev ? prev[i] : 0;
            int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
            int x = src[i], v;
            switch (ft) {
            case 0: v = x; break;
            case 1: v = x + a; break;
            case 2: v = x + b; break;
            case 3: v = x + ((a + b) >> 1); break;
            case 4: v = x + paeth(a, b, c); break;
            default: return false;
            }
            row[i] = (uint8_t)v;
        }
        src += stride;
    }
    return true;
}

} // namespace

bool png_decode(const uint8_t* data, size_t size, PngImage& img, std::string& err)
{
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (size < 8 || std::memcmp(data, sig, 8) != 0) {
        err = "not a PNG file";
        return false;
    }
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    size_t pos = 8;
    bool ended = false;
    while (pos + 12 <= size && !ended) {
        uint32_t len = be32(data + pos);
        const uint8_t* type = data + pos + 4;
        const uint8_t* body = data + pos + 8;
        if (len > size - pos - 12) {
            err = "PNG: truncated chunk";
            return false;
        }
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            if (body[10] != 0 || body[11] != 0 || interlace > 1) {
                err = "PNG: unsupported compression, filter or interlace method";
                return false;
            }
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            ended = true;
        }
        pos += 12 + (size_t)len;
    }
    static const int chans[7] = {1, 0, 3, 1, 2, 0, 4};
    if (w == 0 || h == 0 || w > (1u << 15) || h > (1u << 15) || ctype < 0 || ctype > 6 || chans[ctype] == 0) {
        err = "PNG: bad or missing header";
        return false;
    }
    const bool depth_ok = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (!depth_ok || (ctype == 3 && (depth == 16 || plte.size() < 3))) {
        err = "PNG: unsupported bit depth";
        return false;
    }
    const int src_ch = chans[ctype];
    const size_t bits_px = (size_t)src_ch * depth;
    const size_t bpp = (bits_px + 7) / 8;
    // passes: Adam7 or one full image
    static const int ax[7] = {0, 4, 0, 2, 0, 1, 0}, ay[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int sx[7] = {8, 8, 4, 4, 2, 2, 1}, sy[7] = {8, 8, 8, 4, 4, 2, 2};
    const int passes = interlace ? 7 : 1;
    size_t raw_total = 0;
    uint32_t pw[7], ph[7];
    for (int p = 0; p < passes; p++) {
        pw[p] = interlace ? (w + sx[p] - 1 - ax[p]) / sx[p] : w;
        ph[p] = interlace ? (h + sy[p] - 1 - ay[p]) / sy[p] : h;
        if (pw[p] && ph[p])
            raw_total += (size_t)ph[p] * (1 + (pw[p] * bits_px + 7) / 8);
    }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw, raw_total, err))
        return false;
    if (raw.size() != raw_total) {
        err = "PNG: image data has the wrong size";
        return false;
    }
    // output channels as the reference asks stb_image: 3 -> 4; palettes -> 3 or 4
    int out_ch = ctype == 3 ? (trns.empty() ? 3 : 4) : src_ch;
    img.file_channels = out_ch;
    if (out_ch == 3)
        out_ch = 4;
    img.width = w;
    img.height = h;
    img.channels = (uint32_t)out_ch;
    img.texels.assign((size_t)w * h * out_ch, 0);
    size_t off = 0;
    std::vector<uint8_t> rows;
    for (int p = 0; p < passes; p++) {
        if (!pw[p] || !ph[p])
            continue;
        const size_t stride = (pw[p] * bits_px + 7) / 8;
        if (!unfilter(raw.data() + off, ph[p], stride, bpp, rows)) {
            err = "PNG: bad filter type";
            return false;
        }
        off += (size_t)ph[p] * (1 + stride);
        for (uint32_t y = 0; y < ph[p]; y++) {
            const uint8_t* row = rows.data() + (size_t)y * stride;
            const uint32_t oy = interlace ? ay[p] + y * sy[p] : y;
            for (uint32_t x = 0; x < pw[p]; x++) {
                const uint32_t ox = interlace ? ax[p] + x * sx[p] : x;
                uint8_t* dst = img.texels.data() + ((size_t)oy * w + ox) * out_ch;
                uint8_t v[4] = {0, 0, 0, 255};
                if (depth < 8) {
                    const size_t bit = (size_t)x * depth;
                    const int s = (int)((row[bit >> 3] >> (8 - depth - (bit & 7))) & ((1 << depth) - 1));
                    if (ctype == 3) {
                        if ((size_t)s * 3 + 2 >= plte.size()) {
                            err = "PNG: palette index out of range";
                            return false;
                        }
                        v[0] = plte[3 * s];
                        v[1] = plte[3 * s + 1];
                        v[2] = plte[3 * s + 2];
                        v[3] = (size_t)s < trns.size() ? trns[s] : 255;
                    } else {
                        v[0] = (uint8_t)(s * 255 / ((1 << depth) - 1));
                    }
                } else if (ctype == 3) {
                    const int s = row[x];
                    if ((size_t)s * 3 + 2 >= plte.size()) {
                        err = "PNG: palette index out of range";
                        return false;
                    }
                    v[0] = plte[3 * s];
                    v[1] = plte[3 * s + 1];
                    v[2] = plte[3 * s + 2];
                    v[3] = (size_t)s < trns.size() ? trns[s] : 255;
                } else {
                    const size_t step = depth / 8;
                    for (int c = 0; c < src_ch; c++)
                        v[c] = row[((size_t)x * src_ch + c) * step]; // 16-bit: high byte
                }
                if (ctype == 3) {
                    for (int c = 0; c < out_ch; c++)
                        dst[c] = v[c];
                } else if (src_ch == 3) {
                    dst[0] = v[0];
                    dst[1] = v[1];
                    dst[2] = v[2];
                    dst[3] = 255;
                } else {
                    for (int c = 0; c < src_ch; c++)
                        dst[c] = v[c];
                }
            }
        }
    }
    return true;
}

} // namespace host
} // namespace pt
