// Test-only stand-in for the small part of nlohmann::json that the reference's logging and
// profiler sources use (the progress JSONL line and the profile blob). It exists so that the
// reference PDHG can be compiled offline from its own sources into oracle/_ref/ as a checker;
// it is never part of the GPU engine. Supports: null, numbers, strings, arrays, objects,
// operator[] on a string key, push_back, the {{"key", value}, ...} object literal, dump().
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json {
 public:
  enum class kind { null, number, integer, boolean, string, array, object };

  json() = default;
  json(std::nullptr_t) {}
  json(bool b) : kind_(kind::boolean), integer_(b ? 1 : 0) {}
  template <typename T,
            typename std::enable_if<std::is_integral<T>::value && !std::is_same<T, bool>::value,
                                    int>::type = 0>
  json(T v) : kind_(kind::integer), integer_(static_cast<long long>(v)) {}
  template <typename T,
            typename std::enable_if<std::is_floating_point<T>::value, int>::type = 0>
  json(T v) : kind_(kind::number), number_(static_cast<double>(v)) {}
  json(const char* s) : kind_(kind::string), string_(s) {}
  json(const std::string& s) : kind_(kind::string), string_(s) {}
  json(std::initializer_list<json> items) {
    bool pairs = items.size() > 0;
    for (const json& item : items) {
      if (item.kind_ != kind::array || item.items_.size() != 2 ||
          item.items_[0].kind_ != kind::string) {
        pairs = false;
      }
    }
    if (pairs) {
      kind_ = kind::object;
      for (const json& item : items) set(item.items_[0].string_, item.items_[1]);
    } else {
      kind_ = kind::array;
      items_.assign(items.begin(), items.end());
    }
  }

  static json array() {
    json j;
    j.kind_ = kind::array;
    return j;
  }
  static json object() {
    json j;
    j.kind_ = kind::object;
    return j;
  }

  json& operator[](const std::string& key) {
    if (kind_ == kind::null) kind_ = kind::object;
    for (std::size_t k = 0; k < keys_.size(); ++k) {
      if (keys_[k] == key) return items_[k];
    }
    keys_.push_back(key);
    items_.emplace_back();
    return items_.back();
  }
  json& operator[](const char* key) { return (*this)[std::string(key)]; }

  void push_back(const json& value) {
    if (kind_ == kind::null) kind_ = kind::array;
    items_.push_back(value);
  }

  std::string dump(int indent = -1) const {
    std::string out;
    write(out, indent, 0);
    return out;
  }

 private:
  void set(const std::string& key, const json& value) { (*this)[key] = value; }

  static void newline(std::string& out, int indent, int depth) {
    if (indent < 0) return;
    out += '\n';
    out.append(static_cast<std::size_t>(indent * depth), ' ');
  }

  static void quote(std::string& out, const std::string& s) {
    out += '"';
    for (const char c : s) {
      if (c == '"' || c == '\\') out += '\\';
      out += c;
    }
    out += '"';
  }

  void write(std::string& out, int indent, int depth) const {
    char buffer[64];
    switch (kind_) {
      case kind::null: out += "null"; return;
      case kind::boolean: out += integer_ ? "true" : "false"; return;
      case kind::integer:
        std::snprintf(buffer, sizeof(buffer), "%lld", integer_);
        out += buffer;
        return;
      case kind::number:
        if (!std::isfinite(number_)) {
          out += "null";
        } else {
          std::snprintf(buffer, sizeof(buffer), "%.17g", number_);
          out += buffer;
        }
        return;
      case kind::string: quote(out, string_); return;
      case kind::array:
      case kind::object: {
        const bool object = kind_ == kind::object;
        out += object ? '{' : '[';
        for (std::size_t k = 0; k < items_.size(); ++k) {
          if (k > 0) out += ',';
          newline(out, indent, depth + 1);
          if (object) {
            quote(out, keys_[k]);
            out += indent >= 0 ? ": " : ":";
          }
          items_[k].write(out, indent, depth + 1);
        }
        if (!items_.empty()) newline(out, indent, depth);
        out += object ? '}' : ']';
        return;
      }
    }
  }

  kind kind_ = kind::null;
  long long integer_ = 0;
  double number_ = 0.0;
  std::string string_;
  std::vector<std::string> keys_;
  std::vector<json> items_;
};

}  // namespace nlohmann
