// jpeg.cpp — baseline JPEG decoder for textures (ITU-T T.81 sequential
// Huffman mode, 8-bit samples), written from the specification:
//
//   markers        SOI, SOF0/SOF1, DHT, DQT, DRI, SOS, RSTn, EOI; APPn/COM skipped
//                  (APP14 "Adobe" read for its colour-transform flag)
//   entropy        canonical Huffman codes (T.81 Annex C) with a 9-bit lookup,
//                  byte stuffing (0xFF00), DC prediction, EXTEND (F.2.2.1),
//                  run-length AC coding with ZRL/EOB (F.2.2.2), restarts
//   dequantisation tables of 8- or 16-bit entries, coefficients in zig-zag order
//   inverse DCT    the exact 2-D IDCT of A.3.3 in double precision, level shift
//                  +128, rounded and clamped to 0..255
//   upsampling     chroma at half resolution is interpolated with the 3:1
//                  triangle filter (each output sample: 3/4 of the nearer and
//                  1/4 of the farther input sample, per direction; edges
//                  replicate), with the reference decoder's weighting of the
//                  second-to-last sample of 2:1 horizontal rows
//   colour         JFIF YCbCr -> RGB (R = Y + 1.402 Cr', G = Y - 0.344136 Cb'
//                  - 0.714136 Cr', B = Y + 1.772 Cb'), in 16.16 fixed point
//                  with rounding; RGB files (Adobe transform 0, or component
//                  ids 'R','G','B') are copied
//
// The reference decodes textures with stb_image (texturedata.cpp:30-48, 64-76);
// its integer IDCT and fixed-point colour conversion round differently from
// this decoder in places, so texels may differ from the reference's by a few
// units (the bound is tested against stb_image compiled from the reference's
// own tree).  The CUDA path and the oracle both sample this decoder's texels.
#include "jpeg.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace pt::host {
namespace {

struct ZigZag {
    uint8_t natural[64]; // coded position k -> row-major index
    ZigZag()
    {
        int k = 0;
        for (int s = 0; s < 15; s++) {
            const int lo = std::max(0, s - 7), hi = std::min(7, s);
            if (s & 1)
                for (int r = lo; r <= hi; r++)
                    natural[k++] = (uint8_t)(r * 8 + (s - r));
            else
                for (int r = hi; r >= lo; r--)
                    natural[k++] = (uint8_t)(r * 8 + (s - r));
        }
    }
};
const ZigZag kZig;

struct IdctTable {
    double c[8][8]; // c[u][x] = C(u)/2 cos((2x+1) u pi / 16)
    IdctTable()
    {
        const double pi = 3.14159265358979323846;
        for (int u = 0; u < 8; u++)
            for (int x = 0; x < 8; x++)
                c[u][x] = (u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * pi / 16.0);
    }
};
const IdctTable kIdct;

struct Huffman {
    bool present = false;
    uint8_t fast_len[512] = {}; // 0: code longer than 9 bits
    uint8_t fast_val[512] = {};
    int32_t mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
    uint8_t vals[256] = {};

    void build(const uint8_t counts[16], const uint8_t* values, int nvals)
    {
        std::memset(fast_len, 0, sizeof(fast_len));
        std::memcpy(vals, values, (size_t)nvals);
        int32_t code = 0;
        int k = 0;
        for (int len = 1; len <= 16; len++) {
            mincode[len] = code;
            valptr[len] = k;
            for (int i = 0; i < counts[len - 1]; i++, k++, code++) {
                if (code >= (1 << len))
                    throw std::runtime_error("over-subscribed Huffman table");
                if (len <= 9) {
                    const int shift = 9 - len;
                    for (int e = 0; e < (1 << shift); e++) {
                        fast_len[(code << shift) | e] = (uint8_t)len;
                        fast_val[(code << shift) | e] = values[k];
                    }
                }
            }
            maxcode[len] = counts[len - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        present = true;
    }
};

// Entropy-coded segment reader: MSB-first bits, 0xFF00 stuffing removed;
// at a marker it stops (pointer left on the 0xFF) and supplies zero bits.
struct BitReader {
    const uint8_t* p;
    const uint8_t* end;
    uint32_t acc = 0;
    int n = 0;
    bool at_marker = false;

    void fill()
    {
        while (n <= 24) {
            uint32_t b = 0;
            if (!at_marker && p < end) {
                b = *p++;
                if (b == 0xFF) {
                    const uint8_t next = p < end ? *p : 0xD9;
                    if (next == 0x00) {
                        p++;
                    } else {
                        at_marker = true;
                        p--;
                        b = 0;
                    }
                }
            }
            acc |= b << (24 - n);
            n += 8;
        }
    }
    uint32_t bits(int k)
    {
        fill();
        const uint32_t v = acc >> (32 - k);
        acc <<= k;
        n -= k;
        return v;
    }
    int extend(int s)
    {
        if (s == 0)
            return 0;
        if (s > 16)
            throw std::runtime_error("bad coefficient size");
        const int v = (int)bits(s);
        return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
    }
    int decode(const Huffman& h)
    {
        fill();
        const uint32_t look = acc >> 23;
        if (h.fast_len[look]) {
            const int l = h.fast_len[look];
            acc <<= l;
            n -= l;
            return h.fast_val[look];
        }
        for (int len = 10; len <= 16; len++) {
            const int32_t code = (int32_t)(acc >> (32 - len));
            if (code <= h.maxcode[len]) {
                acc <<= len;
                n -= len;
                return h.vals[h.valptr[len] + code - h.mincode[len]];
            }
        }
        throw std::runtime_error("bad Huffman code");
    }
    void reset()
    {
        acc = 0;
        n = 0;
        at_marker = false;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int dc_pred = 0;
    int stride = 0, rows = 0; // plane size in samples (whole MCUs)
    std::vector<uint8_t> plane;
};

struct Decoder {
    const uint8_t* data;
    size_t size;
    size_t pos = 0;
    int width = 0, height = 0;
    int hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool have_frame = false, adobe = false;
    int adobe_transform = -1;
    uint32_t restart_interval = 0;
    uint16_t qt[4][64] = {};
    bool qt_present[4] = {};
    Huffman dc[4], ac[4];
    std::vector<Component> comps;

    uint8_t byte()
    {
        if (pos >= size)
            throw std::runtime_error("truncated JPEG");
        return data[pos++];
    }
    int u16()
    {
        const int a = byte();
        return (a << 8) | byte();
    }
    // Segment body [pos, pos + len - 2) after its length field.
    size_t segment_end()
    {
        const int len = u16();
        if (len < 2 || pos + (size_t)len - 2 > size)
            throw std::runtime_error("truncated JPEG segment");
        return pos + (size_t)len - 2;
    }

    void read_dqt()
    {
        const size_t e = segment_end();
        while (pos < e) {
            const int pq_tq = byte(), pq = pq_tq >> 4, tq = pq_tq & 15;
            if (tq > 3 || pq > 1)
                throw std::runtime_error("bad quantisation table");
            for (int k = 0; k < 64; k++)
                qt[tq][k] = (uint16_t)(pq ? u16() : byte());
            qt_present[tq] = true;
        }
        pos = e;
    }
    void read_dht()
    {
        const size_t e = segment_end();
        while (pos < e) {
            const int tc_th = byte(), tc = tc_th >> 4, th = tc_th & 15;
            if (tc > 1 || th > 3)
                throw std::runtime_error("bad Huffman table");
            uint8_t counts[16];
            int total = 0;
            for (int i = 0; i < 16; i++)
                total += counts[i] = byte();
            if (total > 256 || pos + (size_t)total > e)
                throw std::runtime_error("bad Huffman table");
            (tc ? ac : dc)[th].build(counts, data + pos, total);
            pos += (size_t)total;
        }
        pos = e;
    }
    void read_sof()
    {
        const size_t e = segment_end();
        if (have_frame)
            throw std::runtime_error("more than one frame");
        if (byte() != 8)
            throw std::runtime_error("only 8-bit JPEG samples are supported");
        height = u16();
        width = u16();
        const int nf = byte();
        if (width == 0 || height == 0)
            throw std::runtime_error("JPEG without a size (DNL is not supported)");
        if ((uint64_t)width * height > (1ull << 28))
            throw std::runtime_error("JPEG image too large");
        if (nf != 1 && nf != 3)
            throw std::runtime_error("only greyscale and three-component JPEGs are supported");
        comps.resize((size_t)nf);
        for (Component& c : comps) {
            c.id = byte();
            const int hv = byte();
            c.h = hv >> 4;
            c.v = hv & 15;
            c.tq = byte();
            if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2 || c.tq > 3)
                throw std::runtime_error("unsupported JPEG sampling factors");
        }
        if (nf == 1)
            comps[0].h = comps[0].v = 1; // a single component is never interleaved
        hmax = vmax = 1;
        for (const Component& c : comps) {
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        for (Component& c : comps) {
            c.stride = mcux * c.h * 8;
            c.rows = mcuy * c.v * 8;
            c.plane.assign((size_t)c.stride * c.rows, 0);
        }
        have_frame = true;
        pos = e;
    }

    void idct_block(const int coef[64], Component& c, int bx, int by)
    {
        double tmp[8][8];
        for (int v = 0; v < 8; v++)
            for (int x = 0; x < 8; x++) {
                double s = 0.0;
                for (int u = 0; u < 8; u++)
                    s += kIdct.c[u][x] * coef[v * 8 + u];
                tmp[v][x] = s;
            }
        uint8_t* out = c.plane.data() + (size_t)by * 8 * c.stride + (size_t)bx * 8;
        for (int y = 0; y < 8; y++)
            for (int x = 0; x < 8; x++) {
                double s = 0.0;
                for (int v = 0; v < 8; v++)
                    s += kIdct.c[v][y] * tmp[v][x];
                const double px = std::floor(s + 128.5);
                out[(size_t)y * c.stride + x] = (uint8_t)std::min(255.0, std::max(0.0, px));
            }
    }

    void decode_block(BitReader& br, Component& c, int bx, int by)
    {
        const Huffman& hd = dc[c.td];
        const Huffman& ha = ac[c.ta];
        if (!hd.present || !ha.present || !qt_present[c.tq])
            throw std::runtime_error("scan uses a missing table");
        int coef[64] = {};
        const uint16_t* q = qt[c.tq];
        const int t = br.decode(hd);
        c.dc_pred += br.extend(t);
        coef[0] = c.dc_pred * q[0];
        for (int k = 1; k < 64;) {
            const int rs = br.decode(ha), r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15)
                    break; // EOB
                k += 16;   // ZRL
                continue;
            }
            k += r;
            if (k > 63)
                throw std::runtime_error("AC coefficient run past the block");
            coef[kZig.natural[k]] = br.extend(s) * q[k];
            k++;
        }
        idct_block(coef, c, bx, by);
    }

    // After a restart interval: skip to the RSTn marker, reset the predictors.
    void restart(BitReader& br)
    {
        br.reset();
        const uint8_t* p = br.p;
        while (p + 1 < br.end && !(p[0] == 0xFF && p[1] >= 0xD0 && p[1] <= 0xD7))
            p++;
        if (p + 1 >= br.end)
            throw std::runtime_error("missing restart marker");
        br.p = p + 2;
        for (Component& c : comps)
            c.dc_pred = 0;
    }

    void read_sos()
    {
        const size_t e = segment_end();
        if (!have_frame)
            throw std::runtime_error("scan before the frame header");
        const int ns = byte();
        if (ns < 1 || ns > (int)comps.size())
            throw std::runtime_error("bad scan header");
        std::vector<Component*> sc;
        for (int i = 0; i < ns; i++) {
            const int id = byte(), t = byte();
            Component* found = nullptr;
            for (Component& c : comps)
                if (c.id == id)
                    found = &c;
            if (!found)
                throw std::runtime_error("scan names a missing component");
            found->td = t >> 4;
            found->ta = t & 15;
            if (found->td > 3 || found->ta > 3)
                throw std::runtime_error("bad scan table selector");
            sc.push_back(found);
        }
        const int ss = byte(), se = byte(), a = byte();
        if (ss != 0 || se != 63 || a != 0)
            throw std::runtime_error("only sequential (baseline) JPEG scans are supported");
        pos = e;
        for (Component* c : sc)
            c->dc_pred = 0;
        BitReader br{data + pos, data + size};
        uint32_t mcus = 0;
        if (ns == 1) {
            Component& c = *sc[0];
            const int bw = ((width * c.h + hmax - 1) / hmax + 7) / 8;
            const int bh = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            const uint32_t total = (uint32_t)bw * bh;
            for (int by = 0; by < bh; by++)
                for (int bx = 0; bx < bw; bx++) {
                    decode_block(br, c, bx, by);
                    if (restart_interval && ++mcus % restart_interval == 0 && mcus < total)
                        restart(br);
                }
        } else {
            const uint32_t total = (uint32_t)mcux * mcuy;
            for (int my = 0; my < mcuy; my++)
                for (int mx = 0; mx < mcux; mx++) {
                    for (Component* c : sc)
                        for (int v = 0; v < c->v; v++)
                            for (int h = 0; h < c->h; h++)
                                decode_block(br, *c, mx * c->h + h, my * c->v + v);
                    if (restart_interval && ++mcus % restart_interval == 0 && mcus < total)
                        restart(br);
                }
        }
        // continue at the next marker that is not a restart
        size_t p = (size_t)(br.p - data);
        while (p + 1 < size && !(data[p] == 0xFF && data[p + 1] != 0x00 && data[p + 1] != 0xFF &&
                                 !(data[p + 1] >= 0xD0 && data[p + 1] <= 0xD7)))
            p++;
        pos = p;
    }

    // One component at full resolution, row y (0 <= y < height), into out[width].
    void upsample_row(const Component& c, int y, uint8_t* out) const
    {
        const int fx = hmax / c.h, fy = vmax / c.v;
        const int cw = (width * c.h + hmax - 1) / hmax, ch = (height * c.v + vmax - 1) / vmax;
        const uint8_t* plane = c.plane.data();
        auto at = [&](int xx, int yy) -> int {
            xx = std::min(std::max(xx, 0), cw - 1);
            yy = std::min(std::max(yy, 0), ch - 1);
            return plane[(size_t)yy * c.stride + xx];
        };
        if (fx == 1 && fy == 1) {
            std::memcpy(out, plane + (size_t)y * c.stride, (size_t)width);
            return;
        }
        // vertical: the chroma row at y / fy and its neighbour on y's side
        const int cy = y / fy;
        const int far_y = fy == 2 ? ((y & 1) ? cy + 1 : cy - 1) : cy;
        auto col = [&](int xx) -> int { // 4 x the vertically interpolated value
            return fy == 2 ? 3 * at(xx, cy) + at(xx, far_y) : 4 * at(xx, cy);
        };
        for (int x = 0; x < width; x++) {
            const int cx = x / fx;
            int v16; // 16 x the interpolated sample
            if (fx == 2) {
                const int far_x = (x & 1) ? cx + 1 : cx - 1;
                v16 = 3 * col(cx) + col(far_x);
                // The reference's decoder (stb_image 2.30) weights the
                // next-to-last sample 3/4 for the second-to-last output of a
                // row subsampled 2:1 horizontally only; kept for parity.
                if (fy == 1 && cw > 1 && cx == cw - 1 && !(x & 1))
                    v16 = 3 * col(cx - 1) + col(cx);
            } else {
                v16 = 4 * col(cx);
            }
            out[x] = (uint8_t)((v16 + 8) >> 4);
        }
    }

    void finish(JpegImage& img) const
    {
        img.width = (uint32_t)width;
        img.height = (uint32_t)height;
        img.file_channels = (uint32_t)comps.size();
        if (comps.size() == 1) {
            img.channels = 1;
            img.texels.resize((size_t)width * height);
            for (int y = 0; y < height; y++)
                std::memcpy(&img.texels[(size_t)y * width], comps[0].plane.data() + (size_t)y * comps[0].stride,
                            (size_t)width);
            return;
        }
        const bool rgb = (adobe && adobe_transform == 0) ||
                         (comps[0].id == 'R' && comps[1].id == 'G' && comps[2].id == 'B');
        img.channels = 4;
        img.texels.resize((size_t)width * height * 4);
        std::vector<uint8_t> r0((size_t)width), r1((size_t)width), r2((size_t)width);
        for (int y = 0; y < height; y++) {
            upsample_row(comps[0], y, r0.data());
            upsample_row(comps[1], y, r1.data());
            upsample_row(comps[2], y, r2.data());
            uint8_t* o = &img.texels[(size_t)y * width * 4];
            for (int x = 0; x < width; x++, o += 4) {
                if (rgb) {
                    o[0] = r0[x];
                    o[1] = r1[x];
                    o[2] = r2[x];
                } else {
                    const int32_t Y = (int32_t)r0[x] << 16, cb = (int32_t)r1[x] - 128, cr = (int32_t)r2[x] - 128;
                    const int32_t half = 1 << 15;
                    const int32_t R = (Y + 91881 * cr + half) >> 16;
                    const int32_t G = (Y - 22554 * cb - 46802 * cr + half) >> 16;
                    const int32_t B = (Y + 116130 * cb + half) >> 16;
                    o[0] = (uint8_t)std::min(255, std::max(0, R));
                    o[1] = (uint8_t)std::min(255, std::max(0, G));
                    o[2] = (uint8_t)std::min(255, std::max(0, B));
                }
                o[3] = 255;
            }
        }
    }

    void run(JpegImage& img)
    {
        if (size < 4 || data[0] != 0xFF || data[1] != 0xD8)
            throw std::runtime_error("not a JPEG file");
        pos = 2;
        bool scanned = false;
        for (;;) {
            uint8_t b = byte();
            if (b != 0xFF)
                throw std::runtime_error("expected a JPEG marker");
            uint8_t m = byte();
            while (m == 0xFF)
                m = byte();
            if (m == 0xD9)
                break; // EOI
            if (m == 0xC0 || m == 0xC1) {
                read_sof();
            } else if (m == 0xC2 || m == 0xC6 || m == 0xCA || m == 0xCE) {
                throw std::runtime_error("progressive JPEG is not supported");
            } else if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
                throw std::runtime_error("lossless or arithmetic-coded JPEG is not supported");
            } else if (m == 0xC4) {
                read_dht();
            } else if (m == 0xCC) {
                throw std::runtime_error("arithmetic-coded JPEG is not supported");
            } else if (m == 0xDB) {
                read_dqt();
            } else if (m == 0xDD) {
                const size_t e = segment_end();
                restart_interval = (uint32_t)u16();
                pos = e;
            } else if (m == 0xDA) {
                read_sos();
                scanned = true;
            } else if (m == 0xEE) {
                const size_t e = segment_end();
                if (e - pos >= 12 && std::memcmp(data + pos, "Adobe", 5) == 0) {
                    adobe = true;
                    adobe_transform = data[pos + 11];
                }
                pos = e;
            } else if ((m >= 0xE0 && m <= 0xEF) || m == 0xFE || m == 0xDC || m == 0xDE || m == 0xDF) {
                pos = segment_end();
            } else if (m >= 0xD0 && m <= 0xD7) {
                continue; // stray restart marker
            } else {
                throw std::runtime_error("unexpected JPEG marker");
            }
            if (pos >= size)
                break;
        }
        if (!have_frame || !scanned)
            throw std::runtime_error("JPEG without image data");
        finish(img);
    }
};

} // namespace

bool jpeg_decode(const uint8_t* data, size_t size, JpegImage& out, std::string& err)
{
    try {
        Decoder d{data, size};
        d.run(out);
        return true;
    } catch (const std::exception& e) {
        err = e.what();
        return false;
    }
}

} // namespace pt::host
