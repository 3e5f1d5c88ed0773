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
  // one chunk per line: y, byte count, then the B, G and R planes
  // (little-endian floats: the host's own layout on the supported machines)
  static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "EXR lines are written from host floats");
  std::vector<uint8_t> line(static_cast<size_t>(line_bytes));
  const uint32_t nbytes = uint32_t(w * 3 * 4);
  std::memcpy(line.data() + 4, &nbytes, 4);
  for (int y = 0; y < h && ok; ++y) {
    const uint32_t yy = uint32_t(y);
    std::memcpy(line.data(), &yy, 4);
    const float* row = rgb + 3 * size_t(y) * size_t(w);
    for (int c = 2; c >= 0; --c) {
      uint8_t* plane = line.data() + 8 + size_t(2 - c) * size_t(w) * 4;
      for (int x = 0; x < w; ++x) std::memcpy(plane + 4 * size_t(x), row + 3 * size_t(x) + size_t(c), 4);
    }
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
