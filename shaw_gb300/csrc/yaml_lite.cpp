// yaml_lite.cpp -- see yaml_lite.h.
#include "yaml_lite.h"

#include <cctype>
#include <cerrno>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace shaw {
namespace yaml {

namespace {

struct Line {
  int indent;
  std::string text;  // content without indentation and comment, right-trimmed
  int lineno;
};

std::string rtrim(const std::string& s) {
  size_t e = s.size();
  while (e > 0 && std::isspace((unsigned char)s[e - 1])) --e;
  return s.substr(0, e);
}

std::string trim(const std::string& s) {
  size_t b = 0;
  while (b < s.size() && std::isspace((unsigned char)s[b])) ++b;
  return rtrim(s.substr(b));
}

// Remove a trailing comment: '#' at the start or preceded by whitespace, outside quotes.
std::string strip_comment(const std::string& s) {
  char quote = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (quote) {
      if (c == quote) quote = 0;
      continue;
    }
    if (c == '\'' || c == '"') quote = c;
    else if (c == '#' && (i == 0 || std::isspace((unsigned char)s[i - 1]))) return s.substr(0, i);
  }
  return s;
}

std::string unquote(const std::string& s) {
  if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
    return s.substr(1, s.size() - 2);
  return s;
}

[[noreturn]] void syntax(int lineno, const std::string& msg) {
  throw std::runtime_error("yaml: line " + std::to_string(lineno) + ": " + msg);
}

// Position of the mapping ':' (followed by space or end), outside quotes/brackets.
size_t find_colon(const std::string& s) {
  char quote = 0;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (quote) {
      if (c == quote) quote = 0;
      continue;
    }
    if (c == '\'' || c == '"') quote = c;
    else if (c == '[' || c == '{') ++depth;
    else if (c == ']' || c == '}') --depth;
    else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t')) return i;
  }
  return std::string::npos;
}

class FlowParser {
 public:
  FlowParser(const std::string& s, int lineno) : s_(s), i_(0), lineno_(lineno) {}
  Node parse_value() {
    skip();
    if (i_ >= s_.size()) syntax(lineno_, "unexpected end of flow value");
    if (s_[i_] == '{') return parse_map();
    if (s_[i_] == '[') return parse_seq();
    return parse_scalar();
  }
  void expect_end() {
    skip();
    if (i_ != s_.size()) syntax(lineno_, "trailing characters after flow value: '" + s_.substr(i_) + "'");
  }

 private:
  void skip() {
    while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
  }
  Node parse_scalar() {
    skip();
    size_t b = i_;
    char quote = 0;
    while (i_ < s_.size()) {
      const char c = s_[i_];
      if (quote) {
        if (c == quote) quote = 0;
      } else if (c == '\'' || c == '"') {
        quote = c;
      } else if (c == ',' || c == ']' || c == '}') {
        break;
      } else if (c == ':' && (i_ + 1 == s_.size() || s_[i_ + 1] == ' ')) {
        break;
      }
      ++i_;
    }
    Node n;
    const std::string t = trim(s_.substr(b, i_ - b));
    if (t.empty() || t == "~" || t == "null") {
      n.kind = Node::Null;
    } else {
      n.kind = Node::Scalar;
      n.scalar = unquote(t);
    }
    return n;
  }
  Node parse_seq() {
    Node n;
    n.kind = Node::Seq;
    ++i_;  // '['
    skip();
    if (i_ < s_.size() && s_[i_] == ']') {
      ++i_;
      return n;
    }
    while (true) {
      n.seq.push_back(parse_value());
      skip();
      if (i_ >= s_.size()) syntax(lineno_, "unterminated flow sequence");
      if (s_[i_] == ',') {
        ++i_;
        continue;
      }
      if (s_[i_] == ']') {
        ++i_;
        break;
      }
      syntax(lineno_, "expected ',' or ']' in flow sequence");
    }
    return n;
  }
  Node parse_map() {
    Node n;
    n.kind = Node::Map;
    ++i_;  // '{'
    skip();
    if (i_ < s_.size() && s_[i_] == '}') {
      ++i_;
      return n;
    }
    while (true) {
      Node k = parse_scalar();
      skip();
      if (i_ >= s_.size() || s_[i_] != ':') syntax(lineno_, "expected ':' in flow mapping");
      ++i_;
      Node v;
      skip();
      if (i_ < s_.size() && (s_[i_] == ',' || s_[i_] == '}')) v.kind = Node::Null;
      else v = parse_value();
      n.map.emplace_back(k.scalar, v);
      skip();
      if (i_ >= s_.size()) syntax(lineno_, "unterminated flow mapping");
      if (s_[i_] == ',') {
        ++i_;
        continue;
      }
      if (s_[i_] == '}') {
        ++i_;
        break;
      }
      syntax(lineno_, "expected ',' or '}' in flow mapping");
    }
    return n;
  }
  const std::string& s_;
  size_t i_;
  int lineno_;
};

bool balanced(const std::string& s) {
  int depth = 0;
  char quote = 0;
  for (char c : s) {
    if (quote) {
      if (c == quote) quote = 0;
      continue;
    }
    if (c == '\'' || c == '"') quote = c;
    else if (c == '[' || c == '{') ++depth;
    else if (c == ']' || c == '}') --depth;
  }
  return depth <= 0;
}

class BlockParser {
 public:
  explicit BlockParser(std::vector<Line> lines) : L_(std::move(lines)), pos_(0) {}
  Node parse_document() {
    if (L_.empty()) return Node();
    Node n = parse_block(L_[0].indent);
    if (pos_ != L_.size()) syntax(L_[pos_].lineno, "unexpected indentation");
    return n;
  }

 private:
  // A flow value may continue on following lines until its brackets balance.
  std::string gather_flow(std::string text) {
    while (!balanced(text) && pos_ < L_.size()) {
      text += " " + L_[pos_].text;
      ++pos_;
    }
    return text;
  }
  Node scalar_or_flow(const std::string& text, int lineno) {
    FlowParser fp(text, lineno);
    Node n = fp.parse_value();
    fp.expect_end();
    return n;
  }
  Node parse_block(int indent) {
    const Line& first = L_[pos_];
    if (first.text.rfind("- ", 0) == 0 || first.text == "-") return parse_seq(indent);
    return parse_map(indent);
  }
  Node parse_seq(int indent) {
    Node n;
    n.kind = Node::Seq;
    while (pos_ < L_.size() && L_[pos_].indent == indent &&
           (L_[pos_].text.rfind("- ", 0) == 0 || L_[pos_].text == "-")) {
      const Line ln = L_[pos_++];
      const std::string rest = trim(ln.text.substr(1));
      if (rest.empty()) {
        if (pos_ < L_.size() && L_[pos_].indent > indent) n.seq.push_back(parse_block(L_[pos_].indent));
        else n.seq.push_back(Node());
      } else if (find_colon(rest) != std::string::npos && rest[0] != '{' && rest[0] != '[') {
        syntax(ln.lineno, "mappings inside block sequences are not supported");
      } else {
        n.seq.push_back(scalar_or_flow(gather_flow(rest), ln.lineno));
      }
    }
    return n;
  }
  Node parse_map(int indent) {
    Node n;
    n.kind = Node::Map;
    while (pos_ < L_.size() && L_[pos_].indent == indent) {
      const Line ln = L_[pos_++];
      if (ln.text.rfind("- ", 0) == 0) syntax(ln.lineno, "sequence item where a mapping key was expected");
      const size_t c = find_colon(ln.text);
      if (c == std::string::npos) syntax(ln.lineno, "expected 'key: value'");
      const std::string key = unquote(trim(ln.text.substr(0, c)));
      const std::string rest = trim(ln.text.substr(c + 1));
      Node v;
      if (rest.empty()) {
        if (pos_ < L_.size() && L_[pos_].indent > indent) {
          v = parse_block(L_[pos_].indent);
        } else if (pos_ < L_.size() && L_[pos_].indent == indent &&
                   (L_[pos_].text.rfind("- ", 0) == 0 || L_[pos_].text == "-")) {
          v = parse_seq(indent);  // block sequence at the key's own indent
        }
      } else {
        v = scalar_or_flow(gather_flow(rest), ln.lineno);
      }
      // duplicate keys: the last one wins
      bool replaced = false;
      for (auto& kv : n.map)
        if (kv.first == key) {
          kv.second = v;
          replaced = true;
        }
      if (!replaced) n.map.emplace_back(key, v);
    }
    if (pos_ < L_.size() && L_[pos_].indent > indent) syntax(L_[pos_].lineno, "unexpected indentation");
    return n;
  }
  std::vector<Line> L_;
  size_t pos_;
};

}  // namespace

const Node* Node::get(const std::string& key) const {
  if (kind != Map) return nullptr;
  for (const auto& kv : map)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

std::string Node::as_string() const {
  if (kind != Scalar) throw std::runtime_error("yaml: expected a scalar");
  return scalar;
}

double Node::as_double() const {
  const std::string s = trim(as_string());
  if (s.empty()) throw std::runtime_error("yaml: empty number");
  errno = 0;
  char* end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0' || errno == ERANGE)
    throw std::runtime_error("yaml: bad conversion of '" + s + "' to a number");
  return v;
}

bool Node::as_bool() const {
  const std::string s = trim(as_string());
  static const char* T[] = {"true", "True", "TRUE", "yes", "Yes", "YES", "on", "On", "ON", "y", "Y"};
  static const char* F[] = {"false", "False", "FALSE", "no", "No", "NO", "off", "Off", "OFF", "n", "N"};
  for (const char* t : T)
    if (s == t) return true;
  for (const char* f : F)
    if (s == f) return false;
  throw std::runtime_error("yaml: bad conversion of '" + s + "' to bool");
}

long long Node::as_int() const {
  const std::string s = trim(as_string());
  errno = 0;
  char* end = nullptr;
  const long long v = std::strtoll(s.c_str(), &end, 10);
  if (s.empty() || end == s.c_str() || *end != '\0' || errno == ERANGE)
    throw std::runtime_error("yaml: bad conversion of '" + s + "' to an integer");
  return v;
}

unsigned long long Node::as_size() const {
  const long long v = as_int();
  if (v < 0) throw std::runtime_error("yaml: negative value where a size is expected");
  return (unsigned long long)v;
}

std::vector<double> Node::as_double_vector() const {
  if (kind != Seq) throw std::runtime_error("yaml: expected a sequence");
  std::vector<double> out;
  for (const auto& n : seq) out.push_back(n.as_double());
  return out;
}

Node parse_string(const std::string& text) {
  std::vector<Line> lines;
  std::istringstream in(text);
  std::string raw;
  int lineno = 0;
  while (std::getline(in, raw)) {
    ++lineno;
    for (char& c : raw)
      if (c == '\t') c = ' ';
    const std::string t = rtrim(strip_comment(raw));
    size_t ind = 0;
    while (ind < t.size() && t[ind] == ' ') ++ind;
    if (ind == t.size()) continue;
    if (t.substr(ind) == "---" || t.substr(ind) == "...") continue;
    lines.push_back({(int)ind, t.substr(ind), lineno});
  }
  BlockParser p(std::move(lines));
  return p.parse_document();
}

Node parse_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("bad file: " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_string(ss.str());
}

}  // namespace yaml
}  // namespace shaw
