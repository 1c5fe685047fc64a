// yaml_subset.h - reader for the YAML subset that Broombridge files use: block
// mappings and sequences (including "- - x" nesting and sequences at their key's
// indentation), flow mappings and sequences that may continue over several lines,
// plain / single-quoted / double-quoted scalars and # comments. Header-only, host.
#ifndef QPE_YAML_SUBSET_H_
#define QPE_YAML_SUBSET_H_

#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace qpe_yaml {

struct Value {
  enum Kind { Null, Scalar, Seq, Map } kind = Null;
  std::string scalar;
  std::vector<std::shared_ptr<const Value>> seq;
  std::vector<std::pair<std::string, std::shared_ptr<const Value>>> map;

  const Value* get(const std::string& k) const {
    if (kind != Map) return nullptr;
    for (const auto& kv : map)
      if (kv.first == k) return kv.second.get();
    return nullptr;
  }
  const Value* at(size_t i) const { return (kind == Seq && i < seq.size()) ? seq[i].get() : nullptr; }
};
using VP = std::shared_ptr<Value>;

namespace detail {

struct Line {
  int indent;
  std::string text;
};

inline std::string strip_comment(const std::string& s) {
  char q = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (q) {
      if (c == q) q = 0;
    } else if (c == '\'' || c == '"') {
      q = c;
    } else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) {
      return s.substr(0, i);
    }
  }
  return s;
}

inline std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r");
  return s.substr(a, b - a + 1);
}

inline VP scalar(const std::string& raw) {
  auto v = std::make_shared<Value>();
  std::string s = trim(raw);
  if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
    s = s.substr(1, s.size() - 2);
  v->kind = Value::Scalar;
  v->scalar = s;
  return v;
}

// Flow collections: [a, b] and {k: v}.
struct Flow {
  const std::string& s;
  size_t i = 0;
  explicit Flow(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
  }
  std::string token(const char* stops) {
    ws();
    if (i < s.size() && (s[i] == '"' || s[i] == '\'')) {
      char q = s[i++];
      size_t a = i;
      while (i < s.size() && s[i] != q) ++i;
      std::string out = s.substr(a, i - a);
      if (i < s.size()) ++i;
      return out;
    }
    size_t a = i;
    while (i < s.size() && !std::strchr(stops, s[i])) ++i;
    return trim(s.substr(a, i - a));
  }
  VP value() {
    ws();
    if (i < s.size() && s[i] == '[') {
      ++i;
      auto v = std::make_shared<Value>();
      v->kind = Value::Seq;
      ws();
      if (i < s.size() && s[i] == ']') { ++i; return v; }
      while (i < s.size()) {
        v->seq.push_back(value());
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == ']') { ++i; break; }
        throw std::runtime_error("yaml: bad flow sequence");
      }
      return v;
    }
    if (i < s.size() && s[i] == '{') {
      ++i;
      auto v = std::make_shared<Value>();
      v->kind = Value::Map;
      ws();
      if (i < s.size() && s[i] == '}') { ++i; return v; }
      while (i < s.size()) {
        std::string k = token(":,}");
        if (i < s.size() && s[i] == ':') ++i;
        v->map.emplace_back(k, value());
        ws();
        if (i < s.size() && s[i] == ',') { ++i; continue; }
        if (i < s.size() && s[i] == '}') { ++i; break; }
        throw std::runtime_error("yaml: bad flow mapping");
      }
      return v;
    }
    auto v = std::make_shared<Value>();
    v->kind = Value::Scalar;
    v->scalar = token(",]}");
    return v;
  }
};

// Position of the key/value colon: the first ':' outside quotes followed by a
// space or the end of the line.
inline size_t key_colon(const std::string& t) {
  char q = 0;
  for (size_t i = 0; i < t.size(); ++i) {
    char c = t[i];
    if (q) {
      if (c == q) q = 0;
    } else if (c == '\'' || c == '"') {
      q = c;
    } else if (c == '[' || c == '{') {
      return std::string::npos;
    } else if (c == ':' && (i + 1 == t.size() || t[i + 1] == ' ')) {
      return i;
    }
  }
  return std::string::npos;
}

inline bool is_dash(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && t[1] == ' '); }

struct Parser {
  std::vector<Line> L;
  size_t i = 0;

  // Inline value text on line i; flow collections may continue on later lines.
  VP inline_value(std::string text) {
    text = trim(text);
    if (!text.empty() && (text[0] == '[' || text[0] == '{')) {
      auto balanced = [](const std::string& t) {
        int depth = 0;
        char q = 0;
        for (char c : t) {
          if (q) { if (c == q) q = 0; continue; }
          if (c == '\'' || c == '"') q = c;
          else if (c == '[' || c == '{') ++depth;
          else if (c == ']' || c == '}') --depth;
        }
        return depth <= 0;
      };
      while (!balanced(text) && i + 1 < L.size()) {
        ++i;
        text += " " + L[i].text;
      }
      ++i;
      Flow f(text);
      return f.value();
    }
    ++i;
    return scalar(text);
  }

  VP node(int indent) {
    if (i >= L.size()) return std::make_shared<Value>();
    if (is_dash(L[i].text)) return seq(L[i].indent);
    return mapping(L[i].indent);
  }

  VP seq(int ind) {
    auto v = std::make_shared<Value>();
    v->kind = Value::Seq;
    while (i < L.size() && L[i].indent == ind && is_dash(L[i].text)) {
      std::string rest = L[i].text.size() > 1 ? L[i].text.substr(2) : "";
      size_t lead = rest.find_first_not_of(' ');
      if (lead == std::string::npos) {
        ++i;
        if (i < L.size() && L[i].indent > ind) v->seq.push_back(node(L[i].indent));
        else v->seq.push_back(std::make_shared<Value>());
        continue;
      }
      rest = rest.substr(lead);
      const int sub = ind + 2 + (int)lead;
      if (is_dash(rest) || key_colon(rest) != std::string::npos) {
        L[i].indent = sub;  // the item's content starts a block at its own column
        L[i].text = rest;
        v->seq.push_back(node(sub));
      } else {
        v->seq.push_back(inline_value(rest));
      }
    }
    return v;
  }

  VP mapping(int ind) {
    auto v = std::make_shared<Value>();
    v->kind = Value::Map;
    while (i < L.size() && L[i].indent == ind && !is_dash(L[i].text)) {
      const std::string& t = L[i].text;
      size_t c = key_colon(t);
      if (c == std::string::npos) throw std::runtime_error("yaml: expected 'key: value' in: " + t);
      std::string key = trim(t.substr(0, c));
      if (key.size() >= 2 && (key.front() == '"' || key.front() == '\'')) key = key.substr(1, key.size() - 2);
      std::string val = trim(t.substr(c + 1));
      if (!val.empty()) {
        v->map.emplace_back(key, inline_value(val));
      } else {
        ++i;
        if (i < L.size() && (L[i].indent > ind || (L[i].indent == ind && is_dash(L[i].text))))
          v->map.emplace_back(key, node(L[i].indent));
        else
          v->map.emplace_back(key, std::make_shared<Value>());
      }
    }
    return v;
  }
};

}  // namespace detail

inline std::shared_ptr<const Value> parse(const std::string& text) {
  detail::Parser p;
  std::istringstream is(text);
  std::string raw;
  while (std::getline(is, raw)) {
    std::string s = detail::strip_comment(raw);
    std::string t = detail::trim(s);
    if (t.empty() || t == "---" || t == "...") continue;
    int ind = 0;
    while ((size_t)ind < s.size() && s[ind] == ' ') ++ind;
    p.L.push_back(detail::Line{ind, t});
  }
  if (p.L.empty()) return std::make_shared<Value>();
  return p.node(p.L[0].indent);
}

inline std::shared_ptr<const Value> load_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("yaml: cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str());
}

}  // namespace qpe_yaml

#endif  // QPE_YAML_SUBSET_H_
