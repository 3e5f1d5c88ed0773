// Oracle stand-in for the nlohmann::json calls the reference makes
// (core/src/Json.cpp, core/include/Hasty/Json.h:12-23, core/src/VMath.cpp:10-16,
// core/src/Camera.cpp:9-25, core/src/Scene.cpp:12-31, core/src/RenderJob.cpp:10-28):
// stream parse, at(key|index), contains, find/end, operator[], get<T>().
#pragma once
#include <istream>
#include <iterator>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>
#include "../../port/hor_io.hpp"

namespace nlohmann {

class json {
 public:
  json() {}
  explicit json(const hor::Json& j) { assign(j); }

  struct const_iterator {
    const json* p;
    bool operator==(const const_iterator& o) const { return p == o.p; }
    bool operator!=(const const_iterator& o) const { return p != o.p; }
    const json& operator*() const { return *p; }
  };

  const json& at(const char* k) const { return at(std::string(k)); }
  const json& at(const std::string& k) const {
    for (auto& kv : obj_) if (kv.first == k) return kv.second;
    throw std::runtime_error("json: missing key " + k);
  }
  const json& at(int i) const { return at(size_t(i)); }
  const json& at(size_t i) const {
    if (i >= arr_.size()) throw std::runtime_error("json: index out of range");
    return arr_[i];
  }
  bool contains(const char* k) const {
    for (auto& kv : obj_) if (kv.first == k) return true;
    return false;
  }
  const_iterator find(const char* k) const {
    for (auto& kv : obj_) if (kv.first == k) return const_iterator{&kv.second};
    return end();
  }
  const_iterator end() const { return const_iterator{nullptr}; }
  json& operator[](const char* k) {
    for (auto& kv : obj_) if (kv.first == k) return kv.second;
    obj_.emplace_back(std::string(k), json());
    return obj_.back().second;
  }

  template <class T>
  T get() const {
    if constexpr (std::is_same<T, bool>::value) return kind_ == hor::Json::Bool ? b_ : num_ != 0.0;
    else if constexpr (std::is_arithmetic<T>::value) return static_cast<T>(kind_ == hor::Json::Bool ? (b_ ? 1.0 : 0.0) : num_);
    else if constexpr (std::is_same<T, std::string>::value) return str_;
    else { T v; from_json(*this, v); return v; }
  }

  friend std::istream& operator>>(std::istream& is, json& j) {
    std::string text((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    j = json(hor::parse_json_text(text));
    return is;
  }

 private:
  void assign(const hor::Json& j) {
    kind_ = j.kind; b_ = j.b; num_ = j.num; str_ = j.str;
    for (auto& a : j.arr) arr_.emplace_back(a);
    for (auto& kv : j.obj) obj_.emplace_back(kv.first, json(kv.second));
  }
  hor::Json::Kind kind_ = hor::Json::Null;
  bool b_ = false;
  double num_ = 0.0;
  std::string str_;
  std::vector<json> arr_;
  std::vector<std::pair<std::string, json>> obj_;
};

}  // namespace nlohmann
