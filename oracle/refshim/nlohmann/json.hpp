/* Minimal stand-in for nlohmann::json so that the reference pdmpk code
 * compiles as a test oracle: values assigned into a json object are kept
 * as text and dump() writes them as one JSON object (statistics only). */
#pragma once
#include <map>
#include <sstream>
#include <string>
#include <vector>
namespace nlohmann {
class json {
 public:
  json() = default;
  template <typename T>
  json(const T &v) { set(v); }
  json &operator[](const std::string &k) { return kids_[k]; }
  template <typename T>
  json &operator=(const T &v) { set(v); return *this; }
  void push_back(const json &v) { items_.push_back(v.dump()); text_.clear(); }
  std::string dump() const {
    if (!kids_.empty()) {
      std::string s = "{";
      bool first = true;
      for (const auto &kv : kids_) {
        s += (first ? "\"" : ",\"") + kv.first + "\":" + kv.second.dump();
        first = false;
      }
      return s + "}";
    }
    if (!items_.empty()) {
      std::string s = "[";
      for (size_t i = 0; i < items_.size(); i++) s += (i ? "," : "") + items_[i];
      return s + "]";
    }
    return text_.empty() ? "null" : text_;
  }
 private:
  void set(const json &j) { *this = j; }
  void set(const std::string &v) { text_ = "\"" + v + "\""; }
  void set(const char *v) { text_ = std::string("\"") + v + "\""; }
  template <typename K, typename V>
  void set(const std::map<K, V> &m) {
    std::ostringstream o;
    o << "{";
    bool first = true;
    for (const auto &kv : m) { o << (first ? "" : ",") << "\"" << kv.first << "\":" << kv.second; first = false; }
    o << "}";
    text_ = o.str();
  }
  template <typename T>
  void set(const std::vector<T> &v) {
    std::ostringstream o;
    o << "[";
    for (size_t i = 0; i < v.size(); i++) o << (i ? "," : "") << v[i];
    o << "]";
    text_ = o.str();
  }
  template <typename T>
  void set(const T &v) { std::ostringstream o; o << v; text_ = o.str(); }
  std::map<std::string, json> kids_;
  std::vector<std::string> items_;
  std::string text_;
};
}  // namespace nlohmann
