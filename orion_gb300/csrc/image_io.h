// 8-bit image files (PNG, BMP, TGA, binary PPM) for environment maps and
// image textures.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace orion_gb300 {

struct Image8 {
  int width = 0, height = 0;
  int channels = 0;          // channels in the file (1-4); rgb always holds 3
  std::vector<uint8_t> rgb;  // width x height x 3, row 0 at the top
};

// Returns false with `err` set when the file cannot be read or decoded.
bool load_image8(const std::string& path, Image8* img, std::string* err);

}  // namespace orion_gb300
