// Host image loading for OTF files (TIFF / .cimg); see otf_io.cpp.
#pragma once

#include <string>
#include <vector>

namespace cdx {

struct HostImage {
  int w = 0, h = 0, d = 0;  // CImg width (x, fastest), height, depth
  std::vector<float> data;
};

bool load_image_file(const char* path, HostImage& img, std::string& err);
// Little-endian uncompressed float32 TIFF, one page per z slice.
bool save_float_tiff(const char* path, const HostImage& img, std::string& err);

}  // namespace cdx
