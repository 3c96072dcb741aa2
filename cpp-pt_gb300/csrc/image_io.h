// Image files for textures: PNG (RFC 2083 / ISO 15948) and Radiance RGBE
// (.hdr), decoded by this library.  The reference reads textures through
// stb_image (src/image/rgb_image.h:160-205); the decoded samples here follow
// what it hands to Image<T>: 8-bit channels for PNG (16-bit samples keep
// their high byte, 1/2/4-bit grey is scaled to 0..255, palettes expand to
// RGB, or RGBA with a tRNS chunk), floats m * 2^(e - 136) for RGBE, and the
// channel count of the file (grey 1, grey+alpha 2, RGB 3, RGBA 4; RGBE 3).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cpppt_gb300 {

struct DecodedImage {
    int w = 0, h = 0, n = 0;  // n: channels per pixel
    bool hdr = false;         // f holds the samples (RGBE); else u8
    std::vector<uint8_t> u8;  // w * h * n, top row first
    std::vector<float> f;
};

// Throws std::runtime_error on unreadable, malformed or unsupported files.
DecodedImage decode_image_file(const std::string& path);
DecodedImage decode_png(const uint8_t* data, size_t size);
DecodedImage decode_rgbe(const uint8_t* data, size_t size);

// Texture pixels as the reference's Image<Vec3> (rgb = true; grey files
// replicate their first channel) or Image<float> (first channel) stores
// them: 8-bit samples as float(v) / 255.0, optionally converted from sRGB
// to linear (pixel_ops::srgb2linear); RGBE samples as decoded, converted
// the same way when srgb is set.  out: w * h * (rgb ? 3 : 1) floats.
void texture_pixels(const DecodedImage& im, bool rgb, bool srgb, std::vector<float>& out);

// pixel_ops::srgb2linear (rgb_image.h:122-128) with its double-precision
// intermediate steps.
float srgb_to_linear_ref(float a);

}  // namespace cpppt_gb300
