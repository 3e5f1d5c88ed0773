// Host-side job loader: JSON, OBJ/MTL and image readers plus the scene
// assembly of core/src/Scene.cpp:12-194. See scene_load.h.
#include "scene_load.h"

#include <algorithm>
#include <cctype>
#include <charconv>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <exception>
#include <thread>
#include <unordered_map>
#include <unistd.h>
#include <sys/stat.h>
#include <sys/mman.h>
#include <fcntl.h>

namespace hasty {
namespace {

// ------------------------------------------------------------------ JSON --
struct JNode {
  enum T { NUL, BOOL, NUM, STR, ARR, OBJ } t = NUL;
  double num = 0; bool b = false; std::string s;
  std::vector<JNode> items;
  std::vector<std::string> keys;
  const JNode* get(const char* k) const {
    if (t != OBJ) return nullptr;
    for (size_t i = 0; i < keys.size(); ++i) if (keys[i] == k) return &items[i];
    return nullptr;
  }
  const JNode& req(const char* k) const {
    const JNode* n = get(k);
    if (!n) throw LoadError(std::string("json: key '") + k + "' not found");
    return *n;
  }
  double number() const {
    if (t == NUM) return num;
    if (t == BOOL) return b ? 1.0 : 0.0;
    throw LoadError("json: expected a number");
  }
  bool boolean() const { return t == BOOL ? b : number() != 0.0; }
  const std::string& str() const { if (t != STR) throw LoadError("json: expected a string"); return s; }
};

class JReader {
 public:
  explicit JReader(const std::string& txt) : p_(txt.c_str()), end_(txt.c_str() + txt.size()) {}
  JNode parse() { JNode n = val(); skip(); if (p_ != end_) bad("trailing characters"); return n; }
 private:
  const char* p_; const char* end_;
  [[noreturn]] void bad(const char* m) { throw LoadError(std::string("json syntax error: ") + m); }
  void skip() { while (p_ < end_ && std::strchr(" \t\r\n", *p_)) ++p_; }
  bool lit(const char* w) { size_t n = std::strlen(w); if (size_t(end_ - p_) >= n && !std::strncmp(p_, w, n)) { p_ += n; return true; } return false; }
  std::string str() {
    std::string o; ++p_;
    while (p_ < end_ && *p_ != '"') {
      char c = *p_++;
      if (c == '\\' && p_ < end_) {
        char e = *p_++;
        switch (e) { case 'n': o += '\n'; break; case 't': o += '\t'; break; case 'r': o += '\r'; break;
          case 'b': o += '\b'; break; case 'f': o += '\f'; break; case 'u': o += '?'; p_ += std::min<ptrdiff_t>(4, end_ - p_); break;
          default: o += e; }
      } else o += c;
    }
    if (p_ >= end_) bad("unterminated string");
    ++p_;
    return o;
  }
  JNode val() {
    skip();
    if (p_ >= end_) bad("unexpected end of input");
    JNode n;
    if (*p_ == '{') {
      n.t = JNode::OBJ; ++p_; skip();
      if (p_ < end_ && *p_ == '}') { ++p_; return n; }
      while (true) {
        skip(); if (p_ >= end_ || *p_ != '"') bad("object key expected");
        n.keys.push_back(str()); skip();
        if (p_ >= end_ || *p_ != ':') bad("':' expected");
        ++p_;
        n.items.push_back(val()); skip();
        if (p_ < end_ && *p_ == ',') { ++p_; continue; }
        if (p_ < end_ && *p_ == '}') { ++p_; break; }
        bad("',' or '}' expected");
      }
    } else if (*p_ == '[') {
      n.t = JNode::ARR; ++p_; skip();
      if (p_ < end_ && *p_ == ']') { ++p_; return n; }
      while (true) {
        n.items.push_back(val()); skip();
        if (p_ < end_ && *p_ == ',') { ++p_; continue; }
        if (p_ < end_ && *p_ == ']') { ++p_; break; }
        bad("',' or ']' expected");
      }
    } else if (*p_ == '"') { n.t = JNode::STR; n.s = str(); }
    else if (lit("true")) { n.t = JNode::BOOL; n.b = true; }
    else if (lit("false")) { n.t = JNode::BOOL; n.b = false; }
    else if (lit("null")) { n.t = JNode::NUL; }
    else {
      char buf[80]; size_t k = 0;
      while (p_ < end_ && k < 79 && std::strchr("+-0123456789.eE", *p_)) buf[k++] = *p_++;
      buf[k] = 0;
      char* e = nullptr; n.num = std::strtod(buf, &e);
      if (k == 0 || e != buf + k) bad("invalid number");
      n.t = JNode::NUM;
    }
    return n;
  }
};

std::string slurp(const std::string& path) {
  std::FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) throw LoadError("could not open " + path + " for reading");
  std::string data;
  long size = std::fseek(fp, 0, SEEK_END) == 0 ? std::ftell(fp) : -1;
  if (size > 0 && std::fseek(fp, 0, SEEK_SET) == 0) {
    data.resize(size_t(size));
    data.resize(std::fread(&data[0], 1, size_t(size), fp));
  }
  char chunk[1 << 16];     // whatever follows (or a stream without a size)
  for (size_t got; (got = std::fread(chunk, 1, sizeof(chunk), fp)) > 0;) data.append(chunk, got);
  std::fclose(fp);
  return data;
}
JNode read_json(const std::string& path) { return JReader(slurp(path)).parse(); }

std::string folder_of(const std::string& p) { size_t k = p.rfind('/'); return k == std::string::npos ? "." : p.substr(0, k); }
std::string resolve(const std::string& dir, const std::string& f) { return (!f.empty() && f[0] == '/') ? f : dir + "/" + f; }

void vec3_of(const JNode& n, float* out) {
  if (n.t != JNode::ARR || n.items.size() < 3) throw LoadError("json: expected a 3-vector");
  for (int i = 0; i < 3; ++i) out[i] = float(n.items[size_t(i)].number());
}

// ---------------------------------------------------------------- images --
// px: values as floats (PNM/PAM: v / maxval); u8: the raw bytes when the
// file stores 8-bit samples (maxval 255), for 8-bit device textures.
struct Img { int w = 0, h = 0, ch = 0; std::vector<float> px; std::vector<uint8_t> u8; };

// PFM (scanlines bottom-up in the file, returned top-down), binary PNM and
// PAM (P7: WIDTH/HEIGHT/DEPTH/MAXVAL header, e.g. RGB_ALPHA for RGBA8).
Img read_image(const std::string& path) {
  std::string data = slurp(path);
  const char* p = data.c_str(); const char* e = p + data.size();
  auto token = [&]() {
    while (p < e) {
      if (*p == '#') { while (p < e && *p != '\n') ++p; continue; }
      if (std::isspace(static_cast<unsigned char>(*p))) { ++p; continue; }
      break;
    }
    const char* b = p;
    while (p < e && !std::isspace(static_cast<unsigned char>(*p))) ++p;
    return std::string(b, p);
  };
  std::string magic = token();
  Img im;
  if (magic == "PF" || magic == "Pf") {
    im.w = std::atoi(token().c_str()); im.h = std::atoi(token().c_str());
    double scale = std::atof(token().c_str());
    ++p;
    im.ch = magic == "PF" ? 3 : 1;
    size_t n = size_t(im.w) * im.h * im.ch;
    if (im.w <= 0 || im.h <= 0 || size_t(e - p) < n * 4) throw LoadError("truncated PFM " + path);
    im.px.resize(n);
    size_t row = size_t(im.w) * im.ch;
    for (int y = 0; y < im.h; ++y) {
      const char* src = p + 4 * row * size_t(im.h - 1 - y);
      for (size_t i = 0; i < row; ++i) {
        uint32_t u; std::memcpy(&u, src + 4 * i, 4);
        if (scale > 0) u = (u >> 24) | ((u >> 8) & 0xFF00u) | ((u << 8) & 0xFF0000u) | (u << 24);
        float f; std::memcpy(&f, &u, 4);
        im.px[size_t(y) * row + i] = f;
      }
    }
    return im;
  }
  if (magic == "P6" || magic == "P5" || magic == "P7") {
    int maxv = 0;
    if (magic == "P7") {
      for (int guard = 0; guard < 64; ++guard) {
        std::string key = token();
        if (key == "ENDHDR") break;
        if (key.empty()) throw LoadError("truncated PAM header " + path);
        std::string val = token();
        if (key == "WIDTH") im.w = std::atoi(val.c_str());
        else if (key == "HEIGHT") im.h = std::atoi(val.c_str());
        else if (key == "DEPTH") im.ch = std::atoi(val.c_str());
        else if (key == "MAXVAL") maxv = std::atoi(val.c_str());
      }
      if (im.ch < 1 || im.ch > 4) throw LoadError("PAM depth must be 1..4: " + path);
    } else {
      im.w = std::atoi(token().c_str()); im.h = std::atoi(token().c_str());
      maxv = std::atoi(token().c_str());
      im.ch = magic == "P6" ? 3 : 1;
    }
    ++p;
    size_t n = size_t(im.w) * im.h * im.ch;
    size_t bps = maxv < 256 ? 1 : 2;
    if (im.w <= 0 || im.h <= 0 || maxv <= 0 || size_t(e - p) < n * bps) throw LoadError("truncated PNM " + path);
    im.px.resize(n);
    const unsigned char* q = reinterpret_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      unsigned v = bps == 1 ? q[i] : (unsigned(q[2 * i]) << 8 | q[2 * i + 1]);
      im.px[i] = float(v) / float(maxv);
    }
    if (maxv == 255) im.u8.assign(q, q + n);
    return im;
  }
  throw LoadError("unsupported image format: " + path + " (PFM, PPM, PGM, PAM are accepted)");
}

// ----------------------------------------------------------------- OBJ ----
struct MtlRec {
  std::string name;
  float Ka[3] = {0, 0, 0}, Kd[3] = {0, 0, 0}, Ks[3] = {0, 0, 0}, Ke[3] = {0, 0, 0};
  float Ns = 1.f, Ni = 1.f, d = 1.f, aniso = 0.f;
  std::string map_Kd, map_Ns, map_Pm, map_bump;
};
struct Corner { int v, vt, vn; };
// Triangles of all shapes in file order: corners (3 per triangle), material
// and smoothing group per triangle; shape s holds triangles
// [shape_first[s], shape_first[s + 1]).
struct ObjFile {
  std::vector<float> v, vn, vt;
  std::vector<Corner> corners;
  std::vector<int> mat;
  std::vector<uint32_t> sg;
  std::vector<size_t> shape_first{0};
  std::vector<MtlRec> mtls;
  size_t n_shapes() const { return shape_first.size() - 1; }
};

const char* ws(const char* s) { while (*s == ' ' || *s == '\t') ++s; return s; }
std::string word(const char*& s) {
  s = ws(s); const char* b = s;
  while (*s && *s != ' ' && *s != '\t' && *s != '\r' && *s != '\n') ++s;
  return std::string(b, s);
}
// A number as strtof reads it. Plain decimals go through std::from_chars
// (also correctly rounded, so the same float, but several times faster);
// the forms where the two differ (a leading '+' or extra whitespace, hex,
// out-of-range values) take strtof itself.
float num(const char*& s) {
  s = ws(s);
  const char* e = s;
  while (*e && !std::isspace(static_cast<unsigned char>(*e))) ++e;
  if (e > s && *s != '+') {
    float f = 0.0f;
    std::from_chars_result r = std::from_chars(s, e, f);
    if (r.ec == std::errc() && *r.ptr != 'x' && *r.ptr != 'X') { s = r.ptr; return f; }
  }
  char* se = nullptr; float f = std::strtof(s, &se);
  if (se == s) return 0.0f;
  s = se; return f;
}
void num3(const char*& s, float* o) { for (int i = 0; i < 3; ++i) o[i] = num(s); }
std::string last_word(const char* s) { std::string l; for (std::string t = word(s); !t.empty(); t = word(s)) l = t; return l; }

void read_mtl(const std::string& path, std::vector<MtlRec>& out, std::map<std::string, int>& index) {
  std::ifstream f(path);
  if (!f) return;   // tinyobj warns and continues without the library
  std::string line;
  MtlRec cur; bool open = false;
  auto close = [&]() { if (open) { index[cur.name] = int(out.size()); out.push_back(cur); } };
  while (std::getline(f, line)) {
    const char* s = ws(line.c_str());
    if (!*s || *s == '#') continue;
    std::string k = word(s);
    if (k == "newmtl") { close(); cur = MtlRec(); cur.name = word(s); open = true; }
    else if (k == "Ka") num3(s, cur.Ka);
    else if (k == "Kd") num3(s, cur.Kd);
    else if (k == "Ks") num3(s, cur.Ks);
    else if (k == "Ke") num3(s, cur.Ke);
    else if (k == "Ns") cur.Ns = num(s);
    else if (k == "Ni") cur.Ni = num(s);
    else if (k == "d") cur.d = num(s);
    else if (k == "Tr") cur.d = 1.0f - num(s);
    else if (k == "aniso") cur.aniso = num(s);
    else if (k == "map_Kd") cur.map_Kd = last_word(s);
    else if (k == "map_Ns") cur.map_Ns = last_word(s);
    else if (k == "map_Pm") cur.map_Pm = last_word(s);
    else if (k == "map_bump" || k == "map_Bump" || k == "bump") cur.map_bump = last_word(s);
  }
  close();
}

int rel_index(long idx, size_t count) {
  if (idx > 0) return int(idx - 1);
  if (idx < 0) return int(long(count) + idx);
  return -1;
}

// One chunk of an OBJ file, parsed on its own thread. Faces keep their raw
// indices (0 where absent, which resolves to -1 like an index of 0) and the
// chunk-local v/vt/vn counts at the face, so that relative (negative) indices
// can be resolved once the counts of the earlier chunks are known.
// Directives are kept in order with the number of faces before them.
struct ObjChunk {
  std::vector<float> v, vn, vt;
  struct Face { uint32_t first, n, lv, lvt, lvn; };
  struct RawCorner { long v, vt, vn; };
  std::vector<Face> faces;
  std::vector<RawCorner> corners;
  enum Kind { kFlush, kUseMtl, kMtlLib, kSmooth };
  struct Directive { size_t face_pos; Kind kind; std::string arg; uint32_t sg; };
  std::vector<Directive> directives;
};

// The line-by-line grammar of the reader, applied to the lines in
// [begin, end) (whole lines). Each line is copied to a NUL-terminated buffer
// first, so the scanning functions see exactly what a getline would give.
void parse_obj_lines(const char* begin, const char* end, ObjChunk& c) {
  std::string line;
  const char* p = begin;
  while (p < end) {
    const char* le = static_cast<const char*>(std::memchr(p, '\n', size_t(end - p)));
    if (!le) le = end;
    line.assign(p, le);
    p = le < end ? le + 1 : end;
    char* s0 = &line[0];
    const char* s = ws(s0);
    if (!*s || *s == '#') continue;
    if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) { s += 1; for (int i = 0; i < 3; ++i) c.v.push_back(num(s)); continue; }
    if (s[0] == 'v' && s[1] == 'n' && (s[2] == ' ' || s[2] == '\t')) { s += 2; for (int i = 0; i < 3; ++i) c.vn.push_back(num(s)); continue; }
    if (s[0] == 'v' && s[1] == 't' && (s[2] == ' ' || s[2] == '\t')) { s += 2; c.vt.push_back(num(s)); c.vt.push_back(num(s)); continue; }
    if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
      ObjChunk::Face f;
      f.first = uint32_t(c.corners.size());
      f.lv = uint32_t(c.v.size() / 3); f.lvt = uint32_t(c.vt.size() / 2); f.lvn = uint32_t(c.vn.size() / 3);
      char* q0 = s0 + (s - s0) + 1;
      for (;;) {
        // token = next run of non-blank characters, NUL-terminated in place
        while (*q0 == ' ' || *q0 == '\t') ++q0;
        char* te = q0;
        while (*te && *te != ' ' && *te != '\t' && *te != '\r' && *te != '\n') ++te;
        if (te == q0) break;
        const char saved = *te;
        *te = '\0';
        ObjChunk::RawCorner rc{0, 0, 0};
        const char* q = q0;
        char* e = nullptr;
        rc.v = std::strtol(q, &e, 10);
        if (*e == '/') {
          q = e + 1;
          if (*q != '/') { long b = std::strtol(q, &e, 10); if (e != q) rc.vt = b; q = e; }
          if (*q == '/') { ++q; long cc = std::strtol(q, &e, 10); if (e != q) rc.vn = cc; }
        }
        c.corners.push_back(rc);
        *te = saved;
        q0 = te;
      }
      f.n = uint32_t(c.corners.size()) - f.first;
      c.faces.push_back(f);
      continue;
    }
    std::string k = word(s);
    ObjChunk::Directive d{c.faces.size(), ObjChunk::kFlush, std::string(), 0u};
    if (k == "o" || k == "g") { c.directives.push_back(d); }
    else if (k == "usemtl") { d.kind = ObjChunk::kUseMtl; d.arg = word(s); c.directives.push_back(d); }
    else if (k == "mtllib") { d.kind = ObjChunk::kMtlLib; d.arg = word(s); c.directives.push_back(d); }
    else if (k == "s") {
      std::string v = word(s);
      d.kind = ObjChunk::kSmooth;
      d.sg = v == "off" ? 0u : uint32_t(std::strtoul(v.c_str(), nullptr, 10));
      c.directives.push_back(d);
    }
  }
}

// Wavefront OBJ with tinyobjloader's conventions (the reference's reader):
// polygons are fanned, quads split along the shorter diagonal, shapes cut at
// o/g, usemtl by name in the mtllib libraries read so far. The file is read
// at once and its lines are parsed on all host threads in chunks; a
// sequential merge then resolves indices and assembles shapes in file order,
// so the result is the one a single pass over the lines gives.
// An OBJ file's bytes: mapped read-only when it is a regular file (the parse
// threads then fault in their own parts of it), else read into memory.
struct FileBytes {
  const char* p = nullptr;
  size_t n = 0;
  void* map = nullptr;
  std::string buf;
  explicit FileBytes(const std::string& path) {
    const int fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) throw LoadError("TinyObjReader error Cannot open file [" + path + "]");
    struct stat st;
    if (::fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
      void* m = ::mmap(nullptr, size_t(st.st_size), PROT_READ, MAP_PRIVATE, fd, 0);
      if (m != MAP_FAILED) { map = m; p = static_cast<const char*>(m); n = size_t(st.st_size); }
    }
    ::close(fd);
    if (!map) {
      try {
        buf = slurp(path);
      } catch (const LoadError&) {
        throw LoadError("TinyObjReader error Cannot open file [" + path + "]");
      }
      p = buf.data(); n = buf.size();
    }
  }
  ~FileBytes() { if (map) ::munmap(map, n); }
  FileBytes(const FileBytes&) = delete;
  FileBytes& operator=(const FileBytes&) = delete;
};

// Triangles a face of n corners gives (tinyobjloader fans polygons; a quad
// is split in two): none below 3 corners.
inline size_t face_tris(uint32_t n) { return n >= 3 ? size_t(n) - 2 : 0; }

ObjFile read_obj(const std::string& path, const std::string& mtl_dir, size_t force_chunks = 0) {
  FileBytes file(path);
  const char* b0 = file.p;
  const char* b1 = b0 + file.n;
  unsigned hw = std::thread::hardware_concurrency();
  size_t n_chunks = std::max<size_t>(1, std::min<size_t>(hw ? hw : 4, file.n / (1u << 20) + 1));
  n_chunks = std::min<size_t>(n_chunks, 64);
  if (force_chunks) n_chunks = force_chunks;
  std::vector<const char*> cut(n_chunks + 1, b1);
  cut[0] = b0;
  for (size_t k = 1; k < n_chunks; ++k) {
    const char* t = b0 + file.n * k / n_chunks;
    if (t < cut[k - 1]) t = cut[k - 1];
    const char* nl = t < b1 ? static_cast<const char*>(std::memchr(t, '\n', size_t(b1 - t))) : nullptr;
    cut[k] = nl ? nl + 1 : b1;
  }
  std::vector<ObjChunk> chunks(n_chunks);
  auto on_chunks = [&](auto&& fn) {
    std::vector<std::thread> th;
    for (size_t k = 1; k < n_chunks; ++k) th.emplace_back(fn, k);
    fn(size_t(0));
    for (std::thread& t : th) t.join();
  };
  // Segments: the faces of a chunk between two directive positions, with
  // the number of triangles they give.
  struct Segment { size_t fa, fb, tris; size_t first_tri; int mat; uint32_t sg; };
  std::vector<std::vector<Segment>> segs(n_chunks);
  on_chunks([&](size_t k) {
    parse_obj_lines(cut[k], cut[k + 1], chunks[k]);
    const ObjChunk& c = chunks[k];
    size_t fa = 0, di = 0;
    while (fa <= c.faces.size()) {
      while (di < c.directives.size() && c.directives[di].face_pos == fa) ++di;
      const size_t fb = di < c.directives.size() ? c.directives[di].face_pos : c.faces.size();
      Segment sg{fa, fb, 0, 0, -1, 0};
      for (size_t f = fa; f < fb; ++f) sg.tris += face_tris(c.faces[f].n);
      segs[k].push_back(sg);
      if (fb == c.faces.size()) break;
      fa = fb;
    }
  });
  ObjFile o;
  size_t nv = 0, nvn = 0, nvt = 0;
  for (const ObjChunk& c : chunks) { nv += c.v.size(); nvn += c.vn.size(); nvt += c.vt.size(); }
  o.v.reserve(nv); o.vn.reserve(nvn); o.vt.reserve(nvt);
  for (const ObjChunk& c : chunks) {
    o.v.insert(o.v.end(), c.v.begin(), c.v.end());
    o.vn.insert(o.vn.end(), c.vn.begin(), c.vn.end());
    o.vt.insert(o.vt.end(), c.vt.begin(), c.vt.end());
  }
  // The reader's state machine over the directives in file order, one step
  // per segment: materials by name from the libraries read so far, the
  // smoothing group, and shapes cut at o/g when they hold triangles.
  std::map<std::string, int> mindex;
  int mat = -1; uint32_t sg = 0;
  size_t tris = 0, shape_tris = 0;
  auto apply = [&](const ObjChunk::Directive& d) {
    switch (d.kind) {
      case ObjChunk::kFlush:
        if (shape_tris) { o.shape_first.push_back(tris); shape_tris = 0; }
        break;
      case ObjChunk::kUseMtl: { auto it = mindex.find(d.arg); mat = it == mindex.end() ? -1 : it->second; break; }
      case ObjChunk::kMtlLib: read_mtl(resolve(mtl_dir, d.arg), o.mtls, mindex); break;
      case ObjChunk::kSmooth: sg = d.sg; break;
    }
  };
  for (size_t k = 0; k < n_chunks; ++k) {
    const ObjChunk& c = chunks[k];
    size_t di = 0;
    for (Segment& g : segs[k]) {
      while (di < c.directives.size() && c.directives[di].face_pos == g.fa) apply(c.directives[di++]);
      g.first_tri = tris; g.mat = mat; g.sg = sg;
      tris += g.tris; shape_tris += g.tris;
    }
    while (di < c.directives.size()) apply(c.directives[di++]);
  }
  if (shape_tris) o.shape_first.push_back(tris);
  o.corners.resize(3 * tris);
  o.mat.resize(tris);
  o.sg.resize(tris);
  // Faces to triangles on all threads, each segment at its place.
  std::vector<size_t> base_v(n_chunks + 1, 0), base_vt(n_chunks + 1, 0), base_vn(n_chunks + 1, 0);
  for (size_t k = 0; k < n_chunks; ++k) {
    base_v[k + 1] = base_v[k] + chunks[k].v.size() / 3;
    base_vt[k + 1] = base_vt[k] + chunks[k].vt.size() / 2;
    base_vn[k + 1] = base_vn[k] + chunks[k].vn.size() / 3;
  }
  on_chunks([&](size_t k) {
    const ObjChunk& c = chunks[k];
    std::vector<Corner> poly;
    for (const Segment& g : segs[k]) {
      size_t t = g.first_tri;
      auto tri = [&](size_t a, size_t b, size_t cc) {
        o.corners[3 * t] = poly[a]; o.corners[3 * t + 1] = poly[b]; o.corners[3 * t + 2] = poly[cc];
        o.mat[t] = g.mat; o.sg[t] = g.sg;
        ++t;
      };
      for (size_t fi = g.fa; fi < g.fb; ++fi) {
        const ObjChunk::Face& f = c.faces[fi];
        if (f.n < 3) continue;
        poly.clear();
        for (uint32_t q = 0; q < f.n; ++q) {
          const ObjChunk::RawCorner& r = c.corners[size_t(f.first) + q];
          Corner cr;
          cr.v = rel_index(r.v, base_v[k] + f.lv);
          cr.vt = rel_index(r.vt, base_vt[k] + f.lvt);
          cr.vn = rel_index(r.vn, base_vn[k] + f.lvn);
          poly.push_back(cr);
        }
        if (poly.size() == 3) {
          tri(0, 1, 2);
        } else if (poly.size() == 4) {
          // tinyobjloader splits a quad along its shorter diagonal
          auto P = [&](size_t q, int a) {
            const size_t i = 3 * size_t(poly[q].v) + size_t(a);
            return poly[q].v >= 0 && i < o.v.size() ? o.v[i] : 0.0f;
          };
          float d02 = 0, d13 = 0;
          for (int a = 0; a < 3; ++a) { float x = P(2, a) - P(0, a), y = P(3, a) - P(1, a); d02 += x * x; d13 += y * y; }
          if (d02 < d13) { tri(0, 1, 2); tri(0, 2, 3); } else { tri(0, 1, 3); tri(1, 2, 3); }
        } else {
          for (size_t q = 1; q + 1 < poly.size(); ++q) tri(0, q, q + 1);
        }
      }
    }
  });
  return o;
}

// The value of texel sample x after loading: sRGB albedo maps are raised to
// 2.2 (clampAndPowInplace(image, 0, FLT_MAX, 2.2), core/src/Texture.cpp:43).
float texel_value(float x, bool srgb) { return srgb ? std::pow(std::max(0.0f, std::min(FLT_MAX, x)), 2.2f) : x; }

int add_texture(HostScene& sc, const std::string& path, int want, bool srgb) {
  Img im = read_image(path);
  TextureDev t{};
  t.w = im.w; t.h = im.h;
  if (!im.u8.empty() && (want == 1 ? im.ch == 1 : (im.ch == 3 || im.ch == 4))) {
    // 8-bit texture: bytes on the device (4 per colour texel, 1 per scalar
    // texel) and a 256-entry table of the float each byte loads as, so a
    // lookup returns exactly what the float texture would hold.
    t.fmt = 1;
    t.ch = want == 1 ? 1 : 3;
    t.lut = int64_t(sc.tex_pool.size());
    for (int b = 0; b < 256; ++b) sc.tex_pool.push_back(texel_value(float(b) / float(255), srgb));
    t.offset = int64_t(sc.tex_pool8.size());
    size_t n = size_t(im.w) * im.h;
    if (want == 1) {
      sc.tex_pool8.insert(sc.tex_pool8.end(), im.u8.begin(), im.u8.end());
    } else {
      for (size_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) sc.tex_pool8.push_back(im.u8[i * size_t(im.ch) + size_t(c)]);
        sc.tex_pool8.push_back(0);
      }
    }
    sc.textures.push_back(t);
    return int(sc.textures.size() - 1);
  }
  t.offset = int64_t(sc.tex_pool.size());
  if (want == 1) {
    if (im.ch != 1) throw LoadError("could not read " + path + ", wrong number of channels, expected 1, found " + std::to_string(im.ch));
    t.ch = 1;
    sc.tex_pool.insert(sc.tex_pool.end(), im.px.begin(), im.px.end());
  } else {
    if (im.ch != 3 && im.ch != 4) throw LoadError("could not read " + path + ", wrong number of channels, expected 3 or 4, found " + std::to_string(im.ch));
    t.ch = 3;
    size_t n = size_t(im.w) * im.h;
    for (size_t i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) sc.tex_pool.push_back(im.px[i * size_t(im.ch) + size_t(c)]);
  }
  if (srgb)
    for (size_t i = size_t(t.offset); i < sc.tex_pool.size(); ++i) sc.tex_pool[i] = texel_value(sc.tex_pool[i], true);
  sc.textures.push_back(t);
  return int(sc.textures.size() - 1);
}

void setup_camera(const JNode& cj, CameraDev& c) {      // Camera.cpp:9-38
  float pos[3], look[3];
  vec3_of(cj.req("position"), pos);
  if (const JNode* la = cj.get("look_at")) vec3_of(*la, look);
  else { look[0] = pos[0]; look[1] = pos[1]; look[2] = pos[2] + -1.0f; }
  float f[3] = {look[0] - pos[0], look[1] - pos[1], look[2] - pos[2]};
  float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (float& x : f) x = x / fl;
  float up[3] = {0.f, 1.f, 0.f};
  float d = up[0] * f[0] + up[1] * f[1] + up[2] * f[2];
  for (int i = 0; i < 3; ++i) up[i] = up[i] - d * f[i];
  float ul = std::sqrt(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
  for (float& x : up) x = x / ul;
  float r[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  for (int i = 0; i < 3; ++i) { c.pos[i] = pos[i]; c.fwd[i] = f[i]; c.up[i] = up[i]; c.right[i] = r[i]; }
  c.aperture = cj.get("aperture") ? float(cj.get("aperture")->number()) : 0.0f;
  c.focal = cj.get("focal_distance") ? float(cj.get("focal_distance")->number()) : 1.0f;
  c.exposure = cj.get("exposure") ? float(cj.get("exposure")->number()) : 0.0f;
  c.blades = cj.get("num_blades") ? int(cj.get("num_blades")->number()) : 8;
  c.blade_rot = cj.get("blade_rotation") ? float(cj.get("blade_rotation")->number()) : 0.0f;
  if (c.aperture > 0.0f && c.blades < 3) throw LoadError("camera: num_blades must be at least 3");
  const double kPi = 3.1415926535897932384;
  float fov = float(kPi) * 45.0f / 180.0f;                // fixed 45 degrees, Camera.h:41
  c.q = std::tan(fov * 0.5f);
  c.ngon_per = float(2.0 * kPi / c.blades);
  c.ngon_nx = std::cos(c.ngon_per * 0.5f);
  c.ngon_ny = std::sin(c.ngon_per * 0.5f);
}

}  // namespace

uint64_t obj_digest(const std::string& path, size_t chunks, int64_t* n_tris, int64_t* n_shapes) {
  const ObjFile o = read_obj(path, folder_of(path), chunks);
  uint64_t h = 1469598103934665603ull;                       // FNV-1a over the words
  auto mix = [&](uint64_t w) { for (int b = 0; b < 8; ++b) { h ^= (w >> (8 * b)) & 0xFFu; h *= 1099511628211ull; } };
  for (const Corner& c : o.corners) { mix(uint32_t(c.v)); mix(uint32_t(c.vt)); mix(uint32_t(c.vn)); }
  for (size_t t = 0; t < o.mat.size(); ++t) { mix(uint32_t(o.mat[t])); mix(o.sg[t]); }
  for (size_t f : o.shape_first) mix(f);
  mix(o.v.size()); mix(o.vn.size()); mix(o.vt.size()); mix(o.mtls.size());
  if (n_tris) *n_tris = int64_t(o.mat.size());
  if (n_shapes) *n_shapes = int64_t(o.n_shapes());
  return h;
}

std::vector<double> build_discrete_cdf(const float* w, size_t n) {
  std::vector<double> cdf;
  if (n < 2) return cdf;
  double total = 0.0;
  for (size_t i = 0; i < n; ++i) total += double(w[i]);
  cdf.resize(n);
  double run = 0.0;
  for (size_t i = 0; i < n; ++i) { double p = double(w[i]) / total; run = i == 0 ? p : run + p; cdf[i] = run; }
  cdf[n - 1] = 1.0;
  return cdf;
}

std::vector<uint32_t> build_cdf_guide(const std::vector<double>& cdf, uint32_t& log2k) {
  std::vector<uint32_t> g;
  log2k = 0;
  size_t n = cdf.size();
  if (n < 2) return g;
  while ((size_t(1) << log2k) < n && log2k < 22) ++log2k;
  size_t K = size_t(1) << log2k;
  g.resize(K + 1);
  size_t i = 0;
  for (size_t k = 0; k <= K; ++k) {
    double x = double(k) / double(K);
    while (i < n - 1 && cdf[i] < x) ++i;
    g[k] = uint32_t(i);
  }
  return g;
}

float halton_value(uint32_t base, uint32_t k) {
  uint32_t i = k + 1, n = 0, d = 1;
  while (i) { n = n * base + i % base; i /= base; d *= base; }
  return float(n) / float(d);
}

void load_job_settings(const std::string& job_path, RenderSettingsH& st, std::string& scene_path) {
  JNode job = read_json(job_path);
  if (const JNode* s = job.get("settings")) {                 // RenderJob.cpp:10-20
    if (const JNode* v = s->get("roulette_start_depth")) st.roulette_start = int(v->number());
    if (const JNode* v = s->get("roulette_q")) st.roulette_q = float(v->number());
    if (const JNode* v = s->get("width")) st.width = uint32_t(v->number());
    if (const JNode* v = s->get("height")) st.height = uint32_t(v->number());
    if (const JNode* v = s->get("num_threads")) st.num_threads = uint32_t(v->number());
    if (const JNode* v = s->get("max_depth")) st.max_depth = int(v->number());
    if (const JNode* v = s->get("num_samples")) st.num_samples = int(v->number());
    if (const JNode* v = s->get("use_mis")) st.use_mis = v->boolean();
  }
  if (const JNode* g = job.get("gb300")) if (const JNode* v = g->get("seed")) st.seed = uint64_t(v->number());
  if (st.width == 0 || st.height == 0) throw LoadError("settings: width and height must be positive");
  scene_path = resolve(folder_of(job_path), job.req("scene").str());
}

void check_job_settings(const RenderSettingsH& st, const HostScene& sc) {
  // Constant non-black background, MIS on, no emissive triangle: the
  // reference exits at its first light sample (Scene.cpp:506-511).
  if (st.use_mis && sc.light_tris.empty() && !sc.env_texture && sc.has_light())
    throw LoadError("error: no light triangle found (constant background with MIS needs an emissive triangle)");
}

void load_render_job(const std::string& job_path, HostScene& sc) {
  std::string scene_path;
  load_job_settings(job_path, sc.settings, scene_path);
  load_scene_file(scene_path, sc);
  check_job_settings(sc.settings, sc);
}

// Environment texture (Environment.h:98-130): texels, pixel weights
// |rgb| sin(theta_center), the discrete distribution over them and their sum.
void load_environment(const std::string& path, HostScene& sc) {
  Img im = read_image(path);
  if (im.ch != 3 && im.ch != 4) throw LoadError("environment texture: expected 3 or 4 channels");
  sc.env_texture = true; sc.env_w = im.w; sc.env_h = im.h;
  size_t n = size_t(im.w) * im.h;
  sc.env_texels.resize(3 * n);
  for (size_t i = 0; i < n; ++i) for (int c = 0; c < 3; ++c) sc.env_texels[3 * i + size_t(c)] = im.px[i * size_t(im.ch) + size_t(c)];
  // pixel weights |rgb| sin(theta_center), Environment.h:107-112
  sc.env_weights.resize(n);
  const double kPi = 3.1415926535897932384;
  float hf = float(im.h);
  for (int y = 0; y < im.h; ++y) {
    float theta = ((float(y) + 0.5f) / hf) * float(kPi);
    float s = std::sin(theta);
    for (int x = 0; x < im.w; ++x) {
      const float* px = &sc.env_texels[3 * (size_t(y) * size_t(im.w) + size_t(x))];
      float nn = std::sqrt(px[0] * px[0] + px[1] * px[1] + px[2] * px[2]);
      sc.env_weights[size_t(y) * size_t(im.w) + size_t(x)] = nn * s;
    }
  }
  sc.env_cdf = build_discrete_cdf(sc.env_weights.data(), n);
  float vs = 0.f;
  for (float v : sc.env_weights) vs += v;
  sc.env_value_sum = vs;
  if (!(vs > 0.f)) throw LoadError("environment texture is black; it cannot be importance sampled");
}

void load_scene_file(const std::string& scene_path, HostScene& sc) {
  std::string folder = folder_of(scene_path);
  JNode scene = read_json(scene_path);
  setup_camera(scene.req("camera"), sc.cam);

  const JNode& world = scene.req("world");
  // The environment map is read and its sampling tables built on a thread of
  // its own while the mesh is parsed (they share nothing).
  std::exception_ptr env_error;
  std::thread env_thread;
  if (const JNode* bg = world.get("background_color")) {
    sc.env_texture = false; vec3_of(*bg, sc.bg);
  } else {
    const std::string env_path = resolve(folder, world.req("environment_texture").str());
    env_thread = std::thread([&sc, env_path, &env_error] {
      try {
        load_environment(env_path, sc);
      } catch (...) {
        env_error = std::current_exception();
      }
    });
  }
  // errors are reported in the reference's loading order: environment first
  std::exception_ptr main_error;
  ObjFile obj;
  try {
    if (const JNode* v = world.get("vary_glass_ior")) sc.vary_glass_ior = v->boolean();
    if (const JNode* dj = world.get("dispersion")) {      // extension: Cauchy bands
      const JNode& model = dj->req("model");
      if (model.str() == "cauchy") sc.cauchy = true;
      else if (model.str() != "ratio") throw LoadError("world.dispersion.model: expected \"cauchy\" or \"ratio\"");
      if (const JNode* b = dj->get("b")) sc.cauchy_b = float(b->number());
      if (const JNode* wv = dj->get("wavelengths")) {
        if (wv->t != JNode::ARR || wv->items.size() != 3) throw LoadError("world.dispersion.wavelengths: expected 3 values (um)");
        for (int k = 0; k < 3; ++k) {
          sc.band_um[k] = float(wv->items[size_t(k)].number());
          if (!(sc.band_um[k] > 0.0f)) throw LoadError("world.dispersion.wavelengths must be positive");
        }
      }
    }

    obj = read_obj(resolve(folder, scene.req("mesh").str()), folder);
  } catch (...) {
    main_error = std::current_exception();
  }
  if (env_thread.joinable()) env_thread.join();
  if (env_error) std::rethrow_exception(env_error);
  if (main_error) std::rethrow_exception(main_error);
  sc.vertices = std::move(obj.v); sc.normals = std::move(obj.vn); sc.texcoords = std::move(obj.vt);

  for (const MtlRec& m : obj.mtls) {                       // Scene.cpp:66-118
    MaterialDev d{};
    d.transmission = 1.0f - m.d;
    d.vary_ior = (sc.vary_glass_ior && d.transmission > 0.0f) ? 1 : 0;
    d.normal_tex = m.map_bump.empty() ? -1 : add_texture(sc, resolve(folder, m.map_bump), 3, false);
    d.albedo_tex = m.map_Kd.empty() ? -1 : add_texture(sc, resolve(folder, m.map_Kd), 3, true);
    for (int c = 0; c < 3; ++c) { d.albedo[c] = m.Kd[c]; d.emission[c] = m.Ke[c]; }
    d.roughness_tex = m.map_Ns.empty() ? -1 : add_texture(sc, resolve(folder, m.map_Ns), 1, false);
    d.roughness = 1.0f - std::sqrt(m.Ns / 1000.0f);
    d.metallic_tex = m.map_Pm.empty() ? -1 : add_texture(sc, resolve(folder, m.map_Pm), 1, false);
    d.metallic = m.Ka[0];
    d.specular = m.Ks[0];
    d.ior = m.Ni;
    d.anisotropy = m.aniso;
    d.is_light = (m.Ke[0] > 0.0f || m.Ke[1] > 0.0f || m.Ke[2] > 0.0f) ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
      const float ratio[3] = {1.43f / 1.45f, 1.45f / 1.45f, 1.47f / 1.45f};
      float lam = sc.band_um[k];
      d.ior_band[k] = sc.cauchy ? d.ior + sc.cauchy_b / (lam * lam) : d.ior * ratio[k];
    }
    // A transmissive surface with a rough lobe makes the reference throw
    // "not implemented" at the first shade (BRDF.cpp:386-389); refuse it here.
    if (d.transmission > 0.0f) {
      float a = d.roughness * d.roughness;
      if (d.roughness_tex >= 0 || a != 0.0f)
        throw LoadError("material '" + m.name + "': transmission > 0 needs roughness 0 (Ns 1000); rough dielectrics are not implemented");
    }
    sc.mats.push_back(d);
  }

  // Triangles in shape order (Scene.cpp:122-189), filled on all host
  // threads over contiguous ranges; the lights of each range are kept in
  // order and joined, and a bad face is reported as the first one in order.
  const std::vector<size_t>& shape_first = obj.shape_first;
  const size_t n_tris = shape_first.back();
  sc.tri_attr.resize(n_tris);
  sc.tri_pos.resize(9 * n_tris);
  struct Range { std::vector<int32_t> lights; std::vector<float> areas; size_t bad = SIZE_MAX; std::string msg; };
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t n_ranges = std::max<size_t>(1, std::min<size_t>(hw ? hw : 4, n_tris / 65536 + 1));
  std::vector<Range> ranges(n_ranges);
  auto fill = [&](size_t r) {
    Range& R = ranges[r];
    const size_t g0 = n_tris * r / n_ranges, g1 = n_tris * (r + 1) / n_ranges;
    size_t s = size_t(std::upper_bound(shape_first.begin(), shape_first.end(), g0) - shape_first.begin()) - 1;
    for (size_t g = g0; g < g1; ++g) {
      while (g >= shape_first[s + 1]) ++s;
      const size_t f = g - shape_first[s];
      TriAttr a{};
      for (int k = 0; k < 3; ++k) {
        const Corner& c = obj.corners[3 * g + size_t(k)];
        if (c.v < 0 || size_t(c.v) * 3 + 2 >= sc.vertices.size()) { R.bad = g; R.msg = "OBJ: vertex index out of range"; return; }
        if (c.vn >= 0 && size_t(c.vn) * 3 + 2 >= sc.normals.size()) { R.bad = g; R.msg = "OBJ: normal index out of range"; return; }
        a.vi[k] = c.v; a.ni[k] = c.vn; a.ti[k] = c.vt;
      }
      a.mat = obj.mat[g];
      if (a.mat < 0) { R.bad = g; R.msg = " error face has no material "; return; }
      a.geom = uint32_t(s); a.prim = uint32_t(f); a.smooth = obj.sg[g] != 0 ? 1u : 0u;
      float* q = &sc.tri_pos[9 * g];
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) q[3 * k + c] = sc.vertices[3 * size_t(a.vi[k]) + size_t(c)];
      const MtlRec& m = obj.mtls[size_t(a.mat)];
      if (m.Ke[0] > 0.0f || m.Ke[1] > 0.0f || m.Ke[2] > 0.0f) {
        if (m.Kd[0] > 0.0f || m.Kd[1] > 0.0f || m.Kd[2] > 0.0f || m.Ks[0] > 0.0f || m.Ks[1] > 0.0f || m.Ks[2] > 0.0f) {
          R.bad = g; R.msg = " don't support non black diffuse materials with emission "; return;
        }
        R.lights.push_back(int32_t(g));
        float e1[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]}, e2[3] = {q[6] - q[0], q[7] - q[1], q[8] - q[2]};
        float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
        R.areas.push_back(0.5f * std::sqrt(cx * cx + cy * cy + cz * cz));
      }
      sc.tri_attr[g] = a;
    }
  };
  {
    std::vector<std::thread> th;
    for (size_t r = 1; r < n_ranges; ++r) th.emplace_back(fill, r);
    fill(0);
    for (std::thread& t : th) t.join();
  }
  std::vector<float> areas;
  for (const Range& R : ranges) {
    if (R.bad != SIZE_MAX) throw LoadError(R.msg);     // ranges are in order: the first bad face
    sc.light_tris.insert(sc.light_tris.end(), R.lights.begin(), R.lights.end());
    areas.insert(areas.end(), R.areas.begin(), R.areas.end());
  }
  sc.n_shapes = uint32_t(obj.n_shapes());
  if (sc.tri_attr.empty()) throw LoadError("scene has no triangles");
  if (sc.tri_attr.size() >= (size_t(1) << 31) - 2) throw LoadError("scene has too many triangles");
  sc.light_cdf = build_discrete_cdf(areas.data(), areas.size());
  float ta = 0.f;
  for (float a : areas) ta += a;
  sc.total_light_area = ta;
}

}  // namespace hasty
