// imageio.cpp — output stage of the headless path (src/io/imagewrite.cpp:19-67).
//
// .hdr: Radiance RGBE (Ward, "Real Pixels", Graphics Gems II) of the RGB
//       channels, written with the run-length scanline encoding of the format
//       for widths in [8, 32767] and flat pixels otherwise.
// .png: 8-bit RGBA, each channel clamp(x * 255, 0, 255) truncated to u8 as the
//       reference does (imagewrite.cpp:39-42); zlib stream of stored blocks.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../../include/pt_scene.h"
#include "jpeg.h"
#include "png.h"

namespace {

void rgbe(const float* c, uint8_t out[4])
{
    float v = c[0];
    if (c[1] > v)
        v = c[1];
    if (c[2] > v)
        v = c[2];
    if (!(v >= 1e-32f)) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int e;
    float m = std::frexp(v, &e) * 256.0f / v;
    for (int k = 0; k < 3; k++) {
        float x = c[k] > 0.0f ? c[k] * m : 0.0f;
        out[k] = (uint8_t)(x > 255.0f ? 255.0f : x);
    }
    out[3] = (uint8_t)(e + 128);
}

void rle_channel(std::vector<uint8_t>& out, const uint8_t* data, int n)
{
    int i = 0;
    while (i < n) {
        // find the next run of at least 3 equal bytes
        int run_start = i, run_len = 0;
        while (run_start < n) {
            run_len = 1;
            while (run_start + run_len < n && run_len < 127 && data[run_start + run_len] == data[run_start])
                run_len++;
            if (run_len >= 3)
                break;
            run_start++;
        }
        if (run_start >= n)
            run_len = 0;
        // literal bytes before the run
        while (i < run_start) {
            int cnt = run_start - i;
            if (cnt > 128)
                cnt = 128;
            out.push_back((uint8_t)cnt);
            out.insert(out.end(), data + i, data + i + cnt);
            i += cnt;
        }
        if (run_len >= 3) {
            out.push_back((uint8_t)(128 + run_len));
            out.push_back(data[run_start]);
            i = run_start + run_len;
        }
    }
}

uint32_t crc_table[256];
bool crc_ready = false;
uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu)
{
    if (!crc_ready) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t x = i;
            for (int k = 0; k < 8; k++)
                x = (x & 1) ? 0xEDB88320u ^ (x >> 1) : x >> 1;
            crc_table[i] = x;
        }
        crc_ready = true;
    }
    for (size_t i = 0; i < n; i++)
        c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c;
}

void be32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& png, const char* type, const std::vector<uint8_t>& data)
{
    be32(png, (uint32_t)data.size());
    size_t start = png.size();
    png.insert(png.end(), type, type + 4);
    png.insert(png.end(), data.begin(), data.end());
    be32(png, crc32(png.data() + start, png.size() - start) ^ 0xFFFFFFFFu);
}

uint8_t float_to_byte(float x)
{
    float v = x * 255.0f;
    v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
    return (uint8_t)v;
}

bool write_all(const char* path, const std::vector<uint8_t>& bytes)
{
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return false;
    bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return std::fclose(f) == 0 && ok;
}

} // namespace

extern "C" {

int pt_write_hdr(const char* path, const float* rgba, uint32_t w, uint32_t h)
{
    if (!path || !rgba || w == 0 || h == 0)
        return PT_ERR_INVALID;
    std::vector<uint8_t> out;
    std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(h) + " +X " + std::to_string(w) + "\n";
    out.insert(out.end(), head.begin(), head.end());
    std::vector<uint8_t> px(4 * (size_t)w), ch(w);
    for (uint32_t y = 0; y < h; y++) {
        for (uint32_t x = 0; x < w; x++)
            rgbe(rgba + 4 * ((size_t)y * w + x), &px[4 * x]);
        if (w < 8 || w > 32767) {
            out.insert(out.end(), px.begin(), px.end());
            continue;
        }
        out.push_back(2);
        out.push_back(2);
        out.push_back((uint8_t)(w >> 8));
        out.push_back((uint8_t)(w & 0xFF));
        for (int c = 0; c < 4; c++) {
            for (uint32_t x = 0; x < w; x++)
                ch[x] = px[4 * x + c];
            rle_channel(out, ch.data(), (int)w);
        }
    }
    return write_all(path, out) ? PT_OK : PT_ERR_IO;
}

int pt_write_png(const char* path, const float* rgba, uint32_t w, uint32_t h)
{
    if (!path || !rgba || w == 0 || h == 0)
        return PT_ERR_INVALID;
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (4 * (size_t)w + 1));
    for (uint32_t y = 0; y < h; y++) {
        raw.push_back(0); // filter: none
        for (uint32_t x = 0; x < 4 * w; x++)
            raw.push_back(float_to_byte(rgba[(size_t)y * 4 * w + x]));
    }
    // zlib stream of stored deflate blocks
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {
        size_t n = raw.size() - pos;
        if (n > 65535)
            n = 65535;
        bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    be32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    be32(ihdr, w);
    be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    return write_all(path, png) ? PT_OK : PT_ERR_IO;
}

int pt_read_hdr(const char* path, float** rgba, uint32_t* width, uint32_t* height)
{
    if (!path || !rgba || !width || !height)
        return PT_ERR_INVALID;
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return PT_ERR_IO;
    std::vector<uint8_t> d;
    uint8_t buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0)
        d.insert(d.end(), buf, buf + n);
    std::fclose(f);
    size_t i = 0;
    auto line = [&]() {
        std::string s;
        while (i < d.size() && d[i] != '\n')
            s += (char)d[i++];
        i++;
        return s;
    };
    if (line().rfind("#?", 0) != 0)
        return PT_ERR_IO;
    while (i < d.size() && !line().empty()) {
    }
    std::string res = line();
    int H = 0, W = 0;
    if (std::sscanf(res.c_str(), "-Y %d +X %d", &H, &W) != 2 || W <= 0 || H <= 0)
        return PT_ERR_IO;
    std::vector<uint8_t> px(4 * (size_t)W * H);
    for (int y = 0; y < H; y++) {
        uint8_t* row = &px[4 * (size_t)y * W];
        if (W >= 8 && W <= 32767 && i + 4 <= d.size() && d[i] == 2 && d[i + 1] == 2 && (d[i + 2] & 0x80) == 0) {
            i += 4;
            for (int c = 0; c < 4; c++) {
                int x = 0;
                while (x < W) {
                    if (i >= d.size())
                        return PT_ERR_IO;
                    int cnt = d[i++];
                    if (cnt > 128) {
                        cnt -= 128;
                        if (i >= d.size() || x + cnt > W)
                            return PT_ERR_IO;
                        uint8_t v = d[i++];
                        for (int k = 0; k < cnt; k++)
                            row[4 * (x++) + c] = v;
                    } else {
                        if (cnt == 0 || x + cnt > W || i + cnt > d.size())
                            return PT_ERR_IO;
                        for (int k = 0; k < cnt; k++)
                            row[4 * (x++) + c] = d[i++];
                    }
                }
            }
        } else {
            if (i + 4 * (size_t)W > d.size())
                return PT_ERR_IO;
            std::memcpy(row, &d[i], 4 * (size_t)W);
            i += 4 * (size_t)W;
        }
    }
    float* out = (float*)std::malloc(sizeof(float) * 4 * (size_t)W * H);
    if (!out)
        return PT_ERR_OOM;
    for (size_t p = 0; p < (size_t)W * H; p++) {
        const uint8_t* q = &px[4 * p];
        if (q[3] == 0) {
            out[4 * p] = out[4 * p + 1] = out[4 * p + 2] = 0.0f;
        } else {
            float f1 = std::ldexp(1.0f, (int)q[3] - (128 + 8));
            out[4 * p + 0] = q[0] * f1;
            out[4 * p + 1] = q[1] * f1;
            out[4 * p + 2] = q[2] * f1;
        }
        out[4 * p + 3] = 1.0f;
    }
    *rgba = out;
    *width = (uint32_t)W;
    *height = (uint32_t)H;
    return PT_OK;
}

int pt_jpeg_decode(const uint8_t* data, size_t size, uint8_t** texels, uint32_t* width, uint32_t* height,
                   uint32_t* channels, uint32_t* file_channels)
{
    if (!data || !texels || !width || !height || !channels)
        return PT_ERR_INVALID;
    pt::host::JpegImage img;
    std::string err;
    if (!pt::host::jpeg_decode(data, size, img, err))
        return PT_ERR_IO;
    uint8_t* out = (uint8_t*)std::malloc(img.texels.size());
    if (!out)
        return PT_ERR_OOM;
    std::memcpy(out, img.texels.data(), img.texels.size());
    *texels = out;
    *width = img.width;
    *height = img.height;
    *channels = img.channels;
    if (file_channels)
        *file_channels = img.file_channels;
    return PT_OK;
}

void pt_host_free(void* p) { std::free(p); }

} // extern "C"

int pt_png_decode(const uint8_t* data, size_t size, uint8_t** texels, uint32_t* width, uint32_t* height,
                  uint32_t* channels, uint32_t* file_channels)
{
    if (!data || !texels || !width || !height || !channels)
        return PT_ERR_INVALID;
    pt::host::PngImage img;
    std::string err;
    if (!pt::host::png_decode(data, size, img, err))
        return PT_ERR_IO;
    uint8_t* out = (uint8_t*)std::malloc(img.texels.size());
    if (!out)
        return PT_ERR_OOM;
    std::memcpy(out, img.texels.data(), img.texels.size());
    *texels = out;
    *width = img.width;
    *height = img.height;
    *channels = img.channels;
    if (file_channels)
        *file_channels = img.file_channels;
    return PT_OK;
}
