// png.h — PNG decoding for texture images (png.cpp).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace pt {
namespace host {

struct PngImage {
    uint32_t width = 0, height = 0;
    uint32_t channels = 0;      // 1, 2 or 4 stored per texel (3-channel files are widened to 4)
    uint32_t file_channels = 0; // channels the file holds (what stb_image reports)
    std::vector<uint8_t> texels; // rows from the top, 8 bits per channel
};

bool png_decode(const uint8_t* data, size_t size, PngImage& img, std::string& err);

} // namespace host
} // namespace pt
