// Oracle (test infrastructure only): readers for the render-job surface used by
// the CPU oracle and by the stand-in headers under oracle/shims/.
//  * JSON: a small DOM for renderJob.json and the scene JSON
//    (core/src/RenderJob.cpp:10-28, core/src/Scene.cpp:12-31, core/src/Camera.cpp:9-25).
//  * OBJ/MTL: the subset of tinyobjloader semantics the reference relies on
//    (core/src/Scene.cpp:31-118,122-189, core/src/tinyobj.cpp:7-89): shapes split
//    at o/g, per-face material ids from usemtl, smoothing-group ids from s,
//    negative (relative) indices, quads split on the shorter diagonal,
//    larger polygons fanned.
//  * Images: PFM (rows stored bottom-up, returned top-down as OIIO does),
//    binary PPM/PGM (8-bit, scaled by 1/255).
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <fstream>
#include <sstream>

namespace hor {

// ---------------------------------------------------------------- JSON ----
struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  const Json* find(const std::string& k) const {
    if (kind != Object) return nullptr;
    for (auto& kv : obj) if (kv.first == k) return &kv.second;
    return nullptr;
  }
  bool contains(const std::string& k) const { return find(k) != nullptr; }
  const Json& at(const std::string& k) const {
    const Json* j = find(k);
    if (!j) throw std::runtime_error("json: missing key '" + k + "'");
    return *j;
  }
  const Json& at(size_t i) const {
    if (kind != Array || i >= arr.size()) throw std::runtime_error("json: index out of range");
    return arr[i];
  }
  double as_number() const {
    if (kind == Number) return num;
    if (kind == Bool) return b ? 1.0 : 0.0;
    throw std::runtime_error("json: value is not a number");
  }
  bool as_bool() const {
    if (kind == Bool) return b;
    if (kind == Number) return num != 0.0;
    throw std::runtime_error("json: value is not a boolean");
  }
  const std::string& as_string() const {
    if (kind != String) throw std::runtime_error("json: value is not a string");
    return str;
  }
};

struct JsonParser {
  const char* p; const char* e;
  void ws() { while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p; }
  [[noreturn]] void fail(const char* m) { throw std::runtime_error(std::string("json parse error: ") + m); }
  Json value() {
    ws();
    if (p >= e) fail("unexpected end");
    Json j;
    char c = *p;
    if (c == '{') {
      j.kind = Json::Object; ++p; ws();
      if (p < e && *p == '}') { ++p; return j; }
      for (;;) {
        ws(); if (p >= e || *p != '"') fail("expected key");
        std::string k = string_lit(); ws();
        if (p >= e || *p != ':') fail("expected ':'");
        ++p;
        j.obj.emplace_back(k, value()); ws();
        if (p < e && *p == ',') { ++p; continue; }
        if (p < e && *p == '}') { ++p; break; }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      j.kind = Json::Array; ++p; ws();
      if (p < e && *p == ']') { ++p; return j; }
      for (;;) {
        j.arr.push_back(value()); ws();
        if (p < e && *p == ',') { ++p; continue; }
        if (p < e && *p == ']') { ++p; break; }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      j.kind = Json::String; j.str = string_lit();
    } else if (!strncmp(p, "true", 4)) { j.kind = Json::Bool; j.b = true; p += 4; }
    else if (!strncmp(p, "false", 5)) { j.kind = Json::Bool; j.b = false; p += 5; }
    else if (!strncmp(p, "null", 4)) { j.kind = Json::Null; p += 4; }
    else {
      char* end = nullptr;
      std::string tmp(p, std::min<size_t>(64, size_t(e - p)));
      double v = std::strtod(tmp.c_str(), &end);
      if (end == tmp.c_str()) fail("bad value");
      p += (end - tmp.c_str());
      j.kind = Json::Number; j.num = v;
    }
    return j;
  }
  std::string string_lit() {
    ++p; std::string s;
    while (p < e && *p != '"') {
      if (*p == '\\' && p + 1 < e) {
        ++p;
        switch (*p) {
          case 'n': s += '\n'; break; case 't': s += '\t'; break;
          case 'r': s += '\r'; break; case 'b': s += '\b'; break;
          case 'f': s += '\f'; break; case 'u': { s += '?'; p += 4; break; }
          default: s += *p;
        }
        ++p;
      } else s += *p++;
    }
    if (p >= e) fail("unterminated string");
    ++p;
    return s;
  }
};

inline Json parse_json_text(const std::string& text) {
  JsonParser ps{text.data(), text.data() + text.size()};
  Json j = ps.value();
  return j;
}

inline std::string read_text_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("could not open " + path + "  for reading ");
  std::stringstream ss; ss << f.rdbuf();
  return ss.str();
}

inline Json read_json_file(const std::string& path) { return parse_json_text(read_text_file(path)); }

inline std::string dir_of(const std::string& path) {
  size_t k = path.find_last_of('/');
  return k == std::string::npos ? std::string(".") : path.substr(0, k);
}
inline std::string join_path(const std::string& dir, const std::string& f) {
  if (!f.empty() && f[0] == '/') return f;
  return dir + "/" + f;
}

// ----------------------------------------------------------- OBJ / MTL ----
struct ObjIndex { int v = -1, vn = -1, vt = -1; };

struct ObjMaterial {
  std::string name;
  float ambient[3] = {0, 0, 0}, diffuse[3] = {0, 0, 0}, specular[3] = {0, 0, 0};
  float transmittance[3] = {0, 0, 0}, emission[3] = {0, 0, 0};
  float shininess = 1.0f, ior = 1.0f, dissolve = 1.0f, anisotropy = 0.0f;
  int illum = 0;
  std::string diffuse_texname, specular_highlight_texname, bump_texname, metallic_texname;
};

struct ObjShape {
  std::string name;
  std::vector<ObjIndex> indices;          // 3 per triangle
  std::vector<unsigned char> num_face_vertices;
  std::vector<int> material_ids;
  std::vector<unsigned int> smoothing_group_ids;
};

struct ObjData {
  std::vector<float> vertices, normals, texcoords;
  std::vector<ObjShape> shapes;
  std::vector<ObjMaterial> materials;
  std::string warning;
};

namespace objdetail {
inline const char* skip_ws(const char* s) { while (*s == ' ' || *s == '\t') ++s; return s; }
inline std::string next_tok(const char*& s) {
  s = skip_ws(s);
  const char* b = s;
  while (*s && *s != ' ' && *s != '\t' && *s != '\r' && *s != '\n') ++s;
  return std::string(b, s);
}
inline float parse_f(const char*& s, float def) {
  s = skip_ws(s);
  char* end = nullptr;
  float v = std::strtof(s, &end);
  if (end == s) return def;
  s = end;
  return v;
}
inline void parse3(const char*& s, float* out) {
  out[0] = parse_f(s, 0.0f); out[1] = parse_f(s, 0.0f); out[2] = parse_f(s, 0.0f);
}
// Texture statements may carry options (-bm 1.0 ...); the file name is the last token.
inline std::string tex_name(const char* s) {
  std::string last;
  for (;;) { std::string t = next_tok(s); if (t.empty()) break; last = t; }
  return last;
}
inline int fix_index(int idx, size_t n) {
  if (idx > 0) return idx - 1;
  if (idx < 0) return int(n) + idx;
  return -1;
}
}  // namespace objdetail

inline void parse_mtl(const std::string& path, ObjData& out, std::map<std::string, int>& matmap) {
  std::ifstream f(path);
  if (!f) { out.warning += "Material file [ " + path + " ] not found.\n"; return; }
  std::string line;
  ObjMaterial cur; bool have = false;
  auto flush = [&]() {
    if (have) { matmap[cur.name] = int(out.materials.size()); out.materials.push_back(cur); }
  };
  while (std::getline(f, line)) {
    const char* s = objdetail::skip_ws(line.c_str());
    if (!*s || *s == '#') continue;
    std::string key = objdetail::next_tok(s);
    if (key == "newmtl") { flush(); cur = ObjMaterial(); cur.name = objdetail::next_tok(s); have = true; }
    else if (key == "Ka") objdetail::parse3(s, cur.ambient);
    else if (key == "Kd") objdetail::parse3(s, cur.diffuse);
    else if (key == "Ks") objdetail::parse3(s, cur.specular);
    else if (key == "Kt" || key == "Tf") objdetail::parse3(s, cur.transmittance);
    else if (key == "Ke") objdetail::parse3(s, cur.emission);
    else if (key == "Ni") cur.ior = objdetail::parse_f(s, 0.0f);
    else if (key == "Ns") cur.shininess = objdetail::parse_f(s, 0.0f);
    else if (key == "illum") cur.illum = int(objdetail::parse_f(s, 0.0f));
    else if (key == "d") cur.dissolve = objdetail::parse_f(s, 0.0f);
    else if (key == "Tr") cur.dissolve = 1.0f - objdetail::parse_f(s, 0.0f);
    else if (key == "aniso") cur.anisotropy = objdetail::parse_f(s, 0.0f);
    else if (key == "map_Kd") cur.diffuse_texname = objdetail::tex_name(s);
    else if (key == "map_Ns") cur.specular_highlight_texname = objdetail::tex_name(s);
    else if (key == "map_Pm") cur.metallic_texname = objdetail::tex_name(s);
    else if (key == "map_bump" || key == "map_Bump" || key == "bump") cur.bump_texname = objdetail::tex_name(s);
  }
  flush();
}

inline bool parse_obj(const std::string& path, const std::string& mtl_dir, ObjData& out, std::string& err) {
  std::ifstream f(path);
  if (!f) { err = "Cannot open file [" + path + "]\n"; return false; }
  std::map<std::string, int> matmap;
  ObjShape cur;
  int cur_mat = -1;
  unsigned int cur_sg = 0;
  auto flush_shape = [&](const std::string& next_name) {
    if (!cur.indices.empty()) out.shapes.push_back(cur);
    cur = ObjShape(); cur.name = next_name;
  };
  std::string line;
  std::vector<ObjIndex> face;
  while (std::getline(f, line)) {
    const char* s = objdetail::skip_ws(line.c_str());
    if (!*s || *s == '#') continue;
    if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
      s += 2; float v[3]; objdetail::parse3(s, v);
      out.vertices.insert(out.vertices.end(), v, v + 3);
    } else if (s[0] == 'v' && s[1] == 'n' && (s[2] == ' ' || s[2] == '\t')) {
      s += 3; float v[3]; objdetail::parse3(s, v);
      out.normals.insert(out.normals.end(), v, v + 3);
    } else if (s[0] == 'v' && s[1] == 't' && (s[2] == ' ' || s[2] == '\t')) {
      s += 3; float u = objdetail::parse_f(s, 0.0f), v = objdetail::parse_f(s, 0.0f);
      out.texcoords.push_back(u); out.texcoords.push_back(v);
    } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
      s += 2; face.clear();
      for (;;) {
        std::string t = objdetail::next_tok(s);
        if (t.empty()) break;
        ObjIndex ix; int a = 0, b = 0, c = 0; int fields = 0;
        const char* q = t.c_str();
        a = std::atoi(q); fields = 1;
        const char* sl = std::strchr(q, '/');
        if (sl) {
          if (sl[1] != '/') { b = std::atoi(sl + 1); fields = 2; }
          const char* sl2 = std::strchr(sl + 1, '/');
          if (sl2) { c = std::atoi(sl2 + 1); fields = 3; }
        }
        ix.v = objdetail::fix_index(a, out.vertices.size() / 3);
        ix.vt = fields >= 2 && b != 0 ? objdetail::fix_index(b, out.texcoords.size() / 2) : -1;
        ix.vn = fields >= 3 && c != 0 ? objdetail::fix_index(c, out.normals.size() / 3) : -1;
        face.push_back(ix);
      }
      if (face.size() < 3) continue;
      auto emit = [&](const ObjIndex& i0, const ObjIndex& i1, const ObjIndex& i2) {
        cur.indices.push_back(i0); cur.indices.push_back(i1); cur.indices.push_back(i2);
        cur.num_face_vertices.push_back(3);
        cur.material_ids.push_back(cur_mat);
        cur.smoothing_group_ids.push_back(cur_sg);
      };
      if (face.size() == 3) emit(face[0], face[1], face[2]);
      else if (face.size() == 4) {
        auto P = [&](int k) { return &out.vertices[3 * size_t(face[k].v)]; };
        float d02[3], d13[3];
        for (int c2 = 0; c2 < 3; ++c2) { d02[c2] = P(2)[c2] - P(0)[c2]; d13[c2] = P(3)[c2] - P(1)[c2]; }
        float s02 = d02[0] * d02[0] + d02[1] * d02[1] + d02[2] * d02[2];
        float s13 = d13[0] * d13[0] + d13[1] * d13[1] + d13[2] * d13[2];
        if (s02 < s13) { emit(face[0], face[1], face[2]); emit(face[0], face[2], face[3]); }
        else { emit(face[0], face[1], face[3]); emit(face[1], face[2], face[3]); }
      } else {
        for (size_t k = 1; k + 1 < face.size(); ++k) emit(face[0], face[k], face[k + 1]);
      }
    } else {
      std::string key = objdetail::next_tok(s);
      if (key == "o" || key == "g") {
        std::string rest = objdetail::skip_ws(s);
        while (!rest.empty() && (rest.back() == '\r' || rest.back() == ' ')) rest.pop_back();
        flush_shape(rest);
      } else if (key == "usemtl") {
        std::string nm = objdetail::next_tok(s);
        auto it = matmap.find(nm);
        if (it == matmap.end()) { out.warning += "material [ '" + nm + "' ] not found in .mtl\n"; cur_mat = -1; }
        else cur_mat = it->second;
      } else if (key == "mtllib") {
        std::string nm = objdetail::next_tok(s);
        parse_mtl(join_path(mtl_dir, nm), out, matmap);
      } else if (key == "s") {
        std::string v = objdetail::next_tok(s);
        if (v == "off") cur_sg = 0; else cur_sg = (unsigned)std::strtoul(v.c_str(), nullptr, 10);
      }
    }
  }
  flush_shape("");
  return true;
}

// -------------------------------------------------------------- images ----
struct ImageF {
  int width = 0, height = 0, channels = 0;
  std::vector<float> data;   // row-major, row 0 = top of the picture
};

inline bool read_image(const std::string& path, ImageF& img, std::string& err) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) { err = "could not open file " + path + " for reading"; return false; }
  char magic[3] = {0, 0, 0};
  if (std::fscanf(fp, "%2s", magic) != 1) { std::fclose(fp); err = "bad image header " + path; return false; }
  std::string m(magic);
  auto read_int = [&](int& v) -> bool {
    int c;
    for (;;) {
      c = std::fgetc(fp);
      if (c == '#') { while (c != '\n' && c != EOF) c = std::fgetc(fp); continue; }
      if (c == ' ' || c == '\t' || c == '\n' || c == '\r') continue;
      break;
    }
    if (c == EOF) return false;
    std::ungetc(c, fp);
    return std::fscanf(fp, "%d", &v) == 1;
  };
  if (m == "PF" || m == "Pf") {
    int w, h; double scale;
    if (!read_int(w) || !read_int(h) || std::fscanf(fp, "%lf", &scale) != 1) { std::fclose(fp); err = "bad PFM header " + path; return false; }
    std::fgetc(fp);
    int ch = (m == "PF") ? 3 : 1;
    std::vector<float> raw(size_t(w) * h * ch);
    if (std::fread(raw.data(), sizeof(float), raw.size(), fp) != raw.size()) { std::fclose(fp); err = "short PFM " + path; return false; }
    std::fclose(fp);
    if (scale > 0) {  // big-endian payload
      for (float& v : raw) { uint32_t u; std::memcpy(&u, &v, 4); u = __builtin_bswap32(u); std::memcpy(&v, &u, 4); }
    }
    img.width = w; img.height = h; img.channels = ch; img.data.resize(raw.size());
    for (int y = 0; y < h; ++y)
      std::memcpy(&img.data[size_t(y) * w * ch], &raw[size_t(h - 1 - y) * w * ch], sizeof(float) * w * ch);
    return true;
  }
  if (m == "P6" || m == "P5" || m == "P7") {
    int w = 0, h = 0, maxv = 0, ch = 0;
    if (m == "P7") {             // PAM: KEY value lines up to ENDHDR
      char key[64], val[64];
      for (int guard = 0;; ++guard) {
        if (guard > 64 || std::fscanf(fp, "%63s", key) != 1) { std::fclose(fp); err = "bad PAM header " + path; return false; }
        if (std::string(key) == "ENDHDR") break;
        if (std::fscanf(fp, "%63s", val) != 1) { std::fclose(fp); err = "bad PAM header " + path; return false; }
        std::string k(key);
        if (k == "WIDTH") w = std::atoi(val);
        else if (k == "HEIGHT") h = std::atoi(val);
        else if (k == "DEPTH") ch = std::atoi(val);
        else if (k == "MAXVAL") maxv = std::atoi(val);
      }
      if (ch < 1 || ch > 4 || w <= 0 || h <= 0 || maxv <= 0) { std::fclose(fp); err = "bad PAM header " + path; return false; }
    } else {
      if (!read_int(w) || !read_int(h) || !read_int(maxv)) { std::fclose(fp); err = "bad PNM header " + path; return false; }
      ch = (m == "P6") ? 3 : 1;
    }
    std::fgetc(fp);
    size_t n = size_t(w) * h * ch;
    img.width = w; img.height = h; img.channels = ch; img.data.resize(n);
    if (maxv < 256) {
      std::vector<uint8_t> raw(n);
      if (std::fread(raw.data(), 1, n, fp) != n) { std::fclose(fp); err = "short PNM " + path; return false; }
      for (size_t i = 0; i < n; ++i) img.data[i] = float(raw[i]) / float(maxv);
    } else {
      std::vector<uint8_t> raw(2 * n);
      if (std::fread(raw.data(), 1, 2 * n, fp) != 2 * n) { std::fclose(fp); err = "short PNM " + path; return false; }
      for (size_t i = 0; i < n; ++i) img.data[i] = float((raw[2 * i] << 8) | raw[2 * i + 1]) / float(maxv);
    }
    std::fclose(fp);
    return true;
  }
  std::fclose(fp);
  err = "unsupported image format " + path + " (PFM, PPM, PGM and PAM are read)";
  return false;
}

}  // namespace hor
