// EXR / PFM writers. See image_out.h.
#include "image_out.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace hasty {
namespace {
void put_u32(std::vector<uint8_t>& b, uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back(uint8_t(v >> (8 * i))); }
void put_u64(std::vector<uint8_t>& b, uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back(uint8_t(v >> (8 * i))); }
void put_f32(std::vector<uint8_t>& b, float f) { uint32_t u; std::memcpy(&u, &f, 4); put_u32(b, u); }
void put_str(std::vector<uint8_t>& b, const char* s) { while (*s) b.push_back(uint8_t(*s++)); b.push_back(0); }
void attr(std::vector<uint8_t>& b, const char* name, const char* type, const std::vector<uint8_t>& val) {
  put_str(b, name); put_str(b, type); put_u32(b, uint32_t(val.size())); b.insert(b.end(), val.begin(), val.end());
}
}  // namespace

bool write_exr_rgb(const std::string& path, const float* rgb, int w, int h) {
  std::vector<uint8_t> hd;
  put_u32(hd, 20000630u);   // magic
  put_u32(hd, 2u);          // version 2, single-part scanline
  std::vector<uint8_t> ch;
  for (const char* c : {"B", "G", "R"}) {   // channels in alphabetical order
    put_str(ch, c); put_u32(ch, 2u /*FLOAT*/); ch.push_back(0); ch.push_back(0); ch.push_back(0); ch.push_back(0);
    put_u32(ch, 1u); put_u32(ch, 1u);
  }
  ch.push_back(0);
  attr(hd, "channels", "chlist", ch);
  attr(hd, "compression", "compression", {0});
  std::vector<uint8_t> box;
  put_u32(box, 0); put_u32(box, 0); put_u32(box, uint32_t(w - 1)); put_u32(box, uint32_t(h - 1));
  attr(hd, "dataWindow", "box2i", box);
  attr(hd, "displayWindow", "box2i", box);
  attr(hd, "lineOrder", "lineOrder", {0});
  std::vector<uint8_t> one; put_f32(one, 1.0f);
  attr(hd, "pixelAspectRatio", "float", one);
  std::vector<uint8_t> cen; put_f32(cen, 0.f); put_f32(cen, 0.f);
  attr(hd, "screenWindowCenter", "v2f", cen);
  attr(hd, "screenWindowWidth", "float", one);
  hd.push_back(0);
  const uint64_t line_bytes = 8 + uint64_t(w) * 3 * 4;
  const uint64_t table_end = hd.size() + 8 * uint64_t(h);
  for (int y = 0; y < h; ++y) put_u64(hd, table_end + uint64_t(y) * line_bytes);
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = std::fwrite(hd.data(), 1, hd.size(), f) == hd.size();
  std::vector<uint8_t> line;
  for (int y = 0; y < h && ok; ++y) {
    line.clear();
    put_u32(line, uint32_t(y));
    put_u32(line, uint32_t(w * 3 * 4));
    for (int c = 2; c >= 0; --c)
      for (int x = 0; x < w; ++x) put_f32(line, rgb[3 * (size_t(y) * w + x) + size_t(c)]);
    ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
  }
  return std::fclose(f) == 0 && ok;
}

bool write_pfm_rgb(const std::string& path, const float* rgb, int w, int h) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  std::fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
  bool ok = true;
  for (int y = h - 1; y >= 0 && ok; --y) ok = std::fwrite(rgb + 3 * size_t(y) * w, sizeof(float), size_t(w) * 3, f) == size_t(w) * 3;
  return std::fclose(f) == 0 && ok;
}

}  // namespace hasty
