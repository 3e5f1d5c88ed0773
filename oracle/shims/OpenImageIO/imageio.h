// Oracle stand-in for the OpenImageIO calls of core/src/Image.cpp:74-166.
// Reads PFM / binary PPM / PGM through the oracle's reader (PFM rows are
// returned top-down, as OIIO does); writes PFM.
#pragma once
#include <memory>
#include <string>
#include <vector>
#include "../../port/hor_io.hpp"

namespace OIIO {
struct TypeDesc {
  enum BASETYPE { UNKNOWN = 0, FLOAT = 11 };
  BASETYPE basetype;
  TypeDesc(BASETYPE b = FLOAT) : basetype(b) {}
};
struct ImageSpec {
  int width = 0, height = 0, nchannels = 0;
  ImageSpec() {}
  ImageSpec(int w, int h, int c, TypeDesc) : width(w), height(h), nchannels(c) {}
};
class ImageInput {
 public:
  static std::unique_ptr<ImageInput> open(const std::string& name) {
    std::unique_ptr<ImageInput> in(new ImageInput());
    std::string err;
    if (!hor::read_image(name, in->img_, err)) return nullptr;
    in->spec_ = ImageSpec(in->img_.width, in->img_.height, in->img_.channels, TypeDesc::FLOAT);
    return in;
  }
  const ImageSpec& spec() const { return spec_; }
  bool read_image(TypeDesc, void* data) {
    std::copy(img_.data.begin(), img_.data.end(), static_cast<float*>(data));
    return true;
  }
  void close() {}
 private:
  hor::ImageF img_;
  ImageSpec spec_;
};
class ImageOutput {
 public:
  static std::unique_ptr<ImageOutput> create(const std::string&) { return std::unique_ptr<ImageOutput>(new ImageOutput()); }
  bool open(const std::string& name, const ImageSpec& s) { name_ = name; spec_ = s; return true; }
  bool write_image(TypeDesc, const void* data) {
    FILE* f = std::fopen(name_.c_str(), "wb");
    if (!f) return false;
    std::fprintf(f, "%s\n%d %d\n-1.0\n", spec_.nchannels == 1 ? "Pf" : "PF", spec_.width, spec_.height);
    const float* p = static_cast<const float*>(data);
    int c = spec_.nchannels == 1 ? 1 : 3;
    for (int y = spec_.height - 1; y >= 0; --y)
      for (int x = 0; x < spec_.width; ++x) std::fwrite(p + (size_t(y) * spec_.width + x) * spec_.nchannels, sizeof(float), c, f);
    std::fclose(f);
    return true;
  }
  bool close() { return true; }
 private:
  std::string name_;
  ImageSpec spec_;
};
}  // namespace OIIO
