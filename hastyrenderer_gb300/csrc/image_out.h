// Output images of a render job: uncompressed scanline OpenEXR (FLOAT RGB,
// what OIIO writes for writeEXR, core/src/Image.cpp:140-152) and PFM
// (core/src/Image.cpp:52-73 layout, rows bottom-up as the format defines).
#pragma once
#include <string>

namespace hasty {
bool write_exr_rgb(const std::string& path, const float* rgb, int w, int h);
bool write_pfm_rgb(const std::string& path, const float* rgb, int w, int h);
}  // namespace hasty
