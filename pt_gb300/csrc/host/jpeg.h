// jpeg.h — baseline JPEG decoding for textures (host side of libptgpu.so).
#ifndef PT_HOST_JPEG_H
#define PT_HOST_JPEG_H

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace pt::host {

// A decoded image as the reference's texture loader keeps it: 8-bit texels,
// rows from the top, 1 channel for greyscale files and 4 (RGB + alpha 255)
// for colour files (stb_image with the file's channel count, 3 widened to 4:
// texturedata.cpp:30-48).  `file_channels` is the file's own count (1 or 3).
struct JpegImage {
    uint32_t width = 0, height = 0, channels = 0, file_channels = 0;
    std::vector<uint8_t> texels;
};

// Decodes a baseline or extended-sequential Huffman JPEG (ITU-T T.81, SOF0 /
// SOF1, 8-bit samples): greyscale or three components (YCbCr, or RGB when the
// file says so), any sampling factors of 1 or 2, restart intervals.
// Progressive, lossless and arithmetic-coded files are refused.  Returns
// false with a message in `err` on malformed or unsupported input.
bool jpeg_decode(const uint8_t* data, size_t size, JpegImage& out, std::string& err);

} // namespace pt::host

#endif
