// jpeg.h — JPEG decoding for `Image` textures (room.json:6 and the
// living-room materials): ITU-T T.81 Huffman-coded sequential (SOF0, SOF1)
// and progressive (SOF2) frames, 8-bit samples, one (grey) or three
// (YCbCr, JFIF) components, any sampling factors up to 4, restart intervals.
// Arithmetic coding, lossless and 12-bit frames are refused.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace aq {

struct JpegImage {
    int w = 0, h = 0;
    int components = 0;        // in the file: 1 (grey) or 3
    bool progressive = false;
    std::vector<uint8_t> rgb;  // w * h * 3, row 0 = top of the image
};

// Decodes `n` bytes. Returns "" on success, else why the data was refused.
std::string jpeg_decode(const uint8_t* data, size_t n, JpegImage& out);

}  // namespace aq
