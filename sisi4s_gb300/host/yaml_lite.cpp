// YAML-subset reader (see yaml_lite.hpp).
#include "yaml_lite.hpp"

#include <cerrno>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace yl {

namespace {

struct Line {
  int indent;
  std::string text;
  int lineno;
};

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r");
  return s.substr(a, b - a + 1);
}

// strip a comment: '#' at line start or after whitespace, outside quotes
std::string strip_comment(const std::string &s) {
  char q = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (q) {
      if (c == q) q = 0;
      continue;
    }
    if (c == '"' || c == '\'') q = c;
    else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t'))
      return s.substr(0, i);
  }
  return s;
}

class Parser {
 public:
  explicit Parser(const std::string &text) {
    std::istringstream in(text);
    std::string raw;
    int no = 0;
    while (std::getline(in, raw)) {
      ++no;
      std::string s = strip_comment(raw);
      if (trim(s).empty()) continue;
      if (trim(s) == "---" || trim(s) == "...") continue;
      int ind = 0;
      while (ind < (int)s.size() && s[ind] == ' ') ++ind;
      std::string t = trim(s);
      // "- rest" expands to a "-" marker line and "rest" two columns deeper
      while (t.size() >= 1 && t[0] == '-' && (t.size() == 1 || t[1] == ' ')) {
        lines_.push_back({ind, "-", no});
        if (t.size() == 1) { t.clear(); break; }
        size_t k = 1;
        while (k < t.size() && t[k] == ' ') ++k;
        ind += (int)k;
        t = t.substr(k);
      }
      if (!t.empty()) lines_.push_back({ind, t, no});
    }
  }

  NodeP document() {
    if (lines_.empty()) return std::make_shared<Node>();
    size_t i = 0;
    NodeP n = block(i, lines_[0].indent);
    if (i != lines_.size())
      throw ParseError("unexpected content at line " + std::to_string(lines_[i].lineno));
    return n;
  }

 private:
  std::vector<Line> lines_;
  std::map<std::string, NodeP> anchors_;

  [[noreturn]] void fail(const Line &l, const std::string &m) {
    throw ParseError("line " + std::to_string(l.lineno) + ": " + m);
  }

  // position of the mapping colon (": " or trailing ":") outside quotes/brackets
  static size_t key_colon(const std::string &t) {
    char q = 0;
    int depth = 0;
    for (size_t i = 0; i < t.size(); ++i) {
      const char c = t[i];
      if (q) {
        if (c == q) q = 0;
        continue;
      }
      if (c == '"' || c == '\'') {
        if (i == 0) q = c;
        continue;
      }
      if (c == '{' || c == '[') ++depth;
      else if (c == '}' || c == ']') --depth;
      else if (c == ':' && depth == 0 && (i + 1 == t.size() || t[i + 1] == ' '))
        return i;
    }
    return std::string::npos;
  }

  NodeP block(size_t &i, int indent) {
    const Line &l = lines_[i];
    if (l.text == "-") return sequence(i, indent);
    if (l.text[0] != '{' && l.text[0] != '[' && key_colon(l.text) != std::string::npos)
      return mapping(i, indent);
    ++i;
    return inline_value(l.text, l);
  }

  NodeP sequence(size_t &i, int indent) {
    auto n = std::make_shared<Node>();
    n->kind = Node::Seq;
    while (i < lines_.size() && lines_[i].indent == indent && lines_[i].text == "-") {
      const Line &dash = lines_[i];
      ++i;
      if (i < lines_.size() && lines_[i].indent > indent) {
        n->seq.push_back(block(i, lines_[i].indent));
      } else {
        n->seq.push_back(std::make_shared<Node>());
      }
      (void)dash;
    }
    return n;
  }

  NodeP mapping(size_t &i, int indent) {
    auto n = std::make_shared<Node>();
    n->kind = Node::Map;
    while (i < lines_.size() && lines_[i].indent == indent && lines_[i].text != "-") {
      const Line &l = lines_[i];
      const size_t c = key_colon(l.text);
      if (c == std::string::npos) fail(l, "expected 'key: value'");
      std::string key = unquote(trim(l.text.substr(0, c)));
      std::string val = trim(l.text.substr(c + 1));
      ++i;
      NodeP child;
      std::string anchor;
      if (!val.empty() && val[0] == '&') {
        size_t sp = val.find(' ');
        anchor = val.substr(1, sp == std::string::npos ? std::string::npos : sp - 1);
        val = sp == std::string::npos ? "" : trim(val.substr(sp));
      }
      if (!val.empty()) {
        child = inline_value(val, l);
      } else if (i < lines_.size() && lines_[i].indent > indent) {
        child = block(i, lines_[i].indent);
      } else if (i < lines_.size() && lines_[i].indent == indent && lines_[i].text == "-") {
        child = sequence(i, indent);  // "key:\n- a" at the key's indentation
      } else {
        child = std::make_shared<Node>();
      }
      if (!anchor.empty()) anchors_[anchor] = child;
      n->map.emplace_back(key, child);
    }
    return n;
  }

  static std::string unquote(const std::string &s) {
    if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') ||
                          (s.front() == '\'' && s.back() == '\'')))
      return s.substr(1, s.size() - 2);
    return s;
  }

  // split a flow collection body at top-level commas
  static std::vector<std::string> split_flow(const std::string &body) {
    std::vector<std::string> out;
    std::string cur;
    char q = 0;
    int depth = 0;
    for (char c : body) {
      if (q) {
        cur += c;
        if (c == q) q = 0;
        continue;
      }
      if (c == '"' || c == '\'') q = c;
      if (c == '{' || c == '[') ++depth;
      if (c == '}' || c == ']') --depth;
      if (c == ',' && depth == 0) {
        out.push_back(trim(cur));
        cur.clear();
        continue;
      }
      cur += c;
    }
    if (!trim(cur).empty()) out.push_back(trim(cur));
    return out;
  }

  NodeP inline_value(std::string v, const Line &l) {
    v = trim(v);
    if (!v.empty() && v[0] == '&') {
      size_t sp = v.find(' ');
      std::string name = v.substr(1, sp == std::string::npos ? std::string::npos : sp - 1);
      NodeP n = sp == std::string::npos ? std::make_shared<Node>()
                                        : inline_value(v.substr(sp), l);
      anchors_[name] = n;
      return n;
    }
    if (!v.empty() && v[0] == '*') {
      auto it = anchors_.find(v.substr(1));
      if (it == anchors_.end()) fail(l, "unknown alias " + v);
      return it->second;
    }
    auto n = std::make_shared<Node>();
    if (!v.empty() && v[0] == '{') {
      if (v.back() != '}') fail(l, "unterminated flow mapping");
      n->kind = Node::Map;
      for (const auto &item : split_flow(v.substr(1, v.size() - 2))) {
        const size_t c = key_colon(item);
        if (c == std::string::npos) fail(l, "expected 'key: value' in flow mapping");
        const std::string val = trim(item.substr(c + 1));
        n->map.emplace_back(unquote(trim(item.substr(0, c))),
                            val.empty() ? std::make_shared<Node>() : inline_value(val, l));
      }
      return n;
    }
    if (!v.empty() && v[0] == '[') {
      if (v.back() != ']') fail(l, "unterminated flow sequence");
      n->kind = Node::Seq;
      for (const auto &item : split_flow(v.substr(1, v.size() - 2)))
        n->seq.push_back(inline_value(item, l));
      return n;
    }
    if (v == "~" || v == "null") return n;
    n->kind = Node::Scalar;
    if (v.size() >= 2 && (v[0] == '"' || v[0] == '\'')) {
      if (v.back() != v[0]) fail(l, "unterminated quoted scalar");
      n->quoted = true;
      n->scalar = v.substr(1, v.size() - 2);
    } else {
      n->scalar = v;
    }
    return n;
  }
};

}  // namespace

NodeP Node::get(const std::string &key) const {
  for (const auto &kv : map)
    if (kv.first == key) return kv.second;
  return nullptr;
}

std::string Node::str() const {
  if (kind != Scalar) throw ParseError("expected a scalar");
  return scalar;
}

bool scalar_is_int(const std::string &s, long long *v) {
  if (s.empty()) return false;
  size_t i = (s[0] == '-' || s[0] == '+') ? 1 : 0;
  if (i == s.size()) return false;
  for (size_t k = i; k < s.size(); ++k)
    if (s[k] < '0' || s[k] > '9') return false;
  errno = 0;
  const long long x = std::strtoll(s.c_str(), nullptr, 10);
  if (errno) return false;
  if (v) *v = x;
  return true;
}

bool scalar_is_double(const std::string &s, double *v) {
  if (s.empty()) return false;
  char *end = nullptr;
  errno = 0;
  const double x = std::strtod(s.c_str(), &end);
  if (errno || end != s.c_str() + s.size()) return false;
  if (v) *v = x;
  return true;
}

double Node::as_double() const {
  double v;
  if (!scalar_is_double(str(), &v)) throw ParseError("not a number: " + scalar);
  return v;
}

long long Node::as_int() const {
  long long v;
  if (!scalar_is_int(str(), &v)) throw ParseError("not an integer: " + scalar);
  return v;
}

bool Node::as_bool() const {
  const std::string s = str();
  if (s == "true" || s == "True" || s == "yes" || s == "1") return true;
  if (s == "false" || s == "False" || s == "no" || s == "0") return false;
  throw ParseError("not a boolean: " + s);
}

NodeP parse(const std::string &text) { return Parser(text).document(); }

NodeP parse_file(const std::string &path) {
  std::ifstream f(path);
  if (!f) throw ParseError("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str());
}

}  // namespace yl
