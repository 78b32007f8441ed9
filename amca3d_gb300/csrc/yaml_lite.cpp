// yaml_lite.cpp — see yaml_lite.h.
#include "yaml_lite.h"

#include <cctype>
#include <sstream>

namespace amca {
namespace yaml {

const Node *Node::find(const std::string &key) const {
  if (kind_ != Map) return nullptr;
  for (const auto &e : entries_)
    if (e.first == key) return e.second.get();
  return nullptr;
}

const Node &Node::at(size_t i) const {
  if (kind_ != Seq || i >= items_.size())
    throw ParseError("line " + std::to_string(line_) + ": sequence index " + std::to_string(i) + " out of range");
  return *items_[i];
}

namespace {

std::string scalar_of(const Node &n) {
  if (n.kind() == Node::Scalar) return n.text();
  if (n.kind() == Node::Null) return "~";
  throw ParseError("line " + std::to_string(n.line()) + ": expected a scalar");
}

// yaml-cpp 0.3.0 Convert<numeric>: stream with basefield unset, whole text consumed.
template <typename T>
bool convert_number(const std::string &s, T &v) {
  std::stringstream in(s);
  in.unsetf(std::ios::dec);
  if ((in >> v) && (in >> std::ws).eof()) return true;
  return false;
}

}  // namespace

double Node::as_double() const {
  const std::string s = scalar_of(*this);
  double v;
  if (convert_number(s, v)) return v;
  if (s == ".inf" || s == ".Inf" || s == ".INF" || s == "+.inf" || s == "+.Inf" || s == "+.INF") return 1.0 / 0.0;
  if (s == "-.inf" || s == "-.Inf" || s == "-.INF") return -1.0 / 0.0;
  if (s == ".nan" || s == ".NaN" || s == ".NAN") return 0.0 / 0.0;
  throw ParseError("line " + std::to_string(line_) + ": '" + s + "' is not a number");
}

int Node::as_int() const {
  const std::string s = scalar_of(*this);
  int v;
  if (convert_number(s, v)) return v;
  throw ParseError("line " + std::to_string(line_) + ": '" + s + "' is not an integer");
}

bool Node::as_bool() const {
  const std::string s = scalar_of(*this);
  bool lower = true, upper = true, capital = !s.empty() && std::isupper((unsigned char)s[0]);
  for (size_t i = 0; i < s.size(); ++i) {
    const unsigned char c = (unsigned char)s[i];
    if (std::isupper(c)) lower = false;
    if (std::islower(c)) upper = false;
    if (i > 0 && std::isupper(c)) capital = false;
  }
  if (lower || upper || capital) {
    std::string l(s);
    for (auto &c : l) c = (char)std::tolower((unsigned char)c);
    if (l == "y" || l == "yes" || l == "true" || l == "on") return true;
    if (l == "n" || l == "no" || l == "false" || l == "off") return false;
  }
  throw ParseError("line " + std::to_string(line_) + ": '" + s + "' is not a boolean");
}

std::string Node::as_string() const { return scalar_of(*this); }

namespace {

struct Line {
  int col;
  int no;
  std::string body;
};

bool space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

std::string strip(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && space(s[a])) ++a;
  while (b > a && space(s[b - 1])) --b;
  return s.substr(a, b - a);
}

std::string unquote(const std::string &s) {
  if (s.size() >= 2 && (s.front() == '"' || s.front() == '\'') && s.back() == s.front()) return s.substr(1, s.size() - 2);
  return s;
}

// Remove a comment: '#' at the start or after whitespace, outside quotes.
std::string drop_comment(const std::string &s) {
  char quote = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (quote) {
      if (c == quote) quote = 0;
    } else if (c == '"' || c == '\'') {
      quote = c;
    } else if (c == '#' && (i == 0 || space(s[i - 1]))) {
      return s.substr(0, i);
    }
  }
  return s;
}

// Index of the ':' that ends a mapping key (followed by blank or end of
// line, outside quotes and brackets); npos when the line is not "key: ...".
size_t key_end(const std::string &s) {
  char quote = 0;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (quote) {
      if (c == quote) quote = 0;
    } else if (c == '"' || c == '\'') {
      quote = c;
    } else if (c == '[' || c == '{') {
      ++depth;
    } else if (c == ']' || c == '}') {
      --depth;
    } else if (c == ':' && depth == 0 && (i + 1 == s.size() || space(s[i + 1]))) {
      return i;
    }
  }
  return std::string::npos;
}

bool dash_item(const std::string &s) { return s == "-" || (s.size() >= 2 && s[0] == '-' && space(s[1])); }

class Reader {
 public:
  explicit Reader(std::vector<Line> lines) : L_(std::move(lines)) {}

  std::unique_ptr<Node> document() {
    if (L_.empty()) return Node::make(Node::Null, 0);
    auto n = block(L_[0].col);
    if (at_ < L_.size())
      throw ParseError("line " + std::to_string(L_[at_].no) + ": unexpected indentation");
    return n;
  }

 private:
  std::vector<Line> L_;
  size_t at_ = 0;

  std::unique_ptr<Node> block(int col) {
    const Line &ln = L_[at_];
    if (dash_item(ln.body)) return sequence(col);
    if (key_end(ln.body) != std::string::npos) return mapping(col);
    ++at_;
    return inline_value(ln.body, ln.no);
  }

  std::unique_ptr<Node> sequence(int col) {
    auto seq = Node::make(Node::Seq, L_[at_].no);
    while (at_ < L_.size() && L_[at_].col == col && dash_item(L_[at_].body)) {
      Line &ln = L_[at_];
      const std::string rest = ln.body.substr(1);
      size_t off = 0;
      while (off < rest.size() && space(rest[off])) ++off;
      if (off >= rest.size()) {  // "-" alone: the item is the block below
        ++at_;
        if (at_ < L_.size() && L_[at_].col > col) seq->add_item(block(L_[at_].col));
        else seq->add_item(Node::make(Node::Null, ln.no));
      } else {  // "- content": content opens a block one column past the dash
        ln.col = col + 1 + (int)off;
        ln.body = rest.substr(off);
        seq->add_item(block(ln.col));
      }
    }
    return seq;
  }

  std::unique_ptr<Node> mapping(int col) {
    auto map = Node::make(Node::Map, L_[at_].no);
    while (at_ < L_.size() && L_[at_].col == col && !dash_item(L_[at_].body)) {
      const Line ln = L_[at_];
      const size_t c = key_end(ln.body);
      if (c == std::string::npos) throw ParseError("line " + std::to_string(ln.no) + ": expected 'key: value'");
      const std::string key = unquote(strip(ln.body.substr(0, c)));
      const std::string val = strip(ln.body.substr(c + 1));
      ++at_;
      std::unique_ptr<Node> v;
      if (!val.empty()) v = inline_value(val, ln.no);
      else if (at_ < L_.size() && L_[at_].col > col) v = block(L_[at_].col);
      else if (at_ < L_.size() && L_[at_].col == col && dash_item(L_[at_].body)) v = sequence(col);
      else v = Node::make(Node::Null, ln.no);
      map->add_entry(key, std::move(v));
    }
    return map;
  }

  std::unique_ptr<Node> inline_value(const std::string &v, int no) {
    if (!v.empty() && (v[0] == '[' || v[0] == '{')) {
      size_t i = 0;
      auto n = flow(v, i, no);
      while (i < v.size() && space(v[i])) ++i;
      if (i != v.size()) throw ParseError("line " + std::to_string(no) + ": text after a flow collection");
      return n;
    }
    if (v == "~" || v == "null") return Node::make(Node::Null, no);
    auto n = Node::make(Node::Scalar, no);
    n->set_text(unquote(v));
    return n;
  }

  std::unique_ptr<Node> flow(const std::string &s, size_t &i, int no) {
    while (i < s.size() && space(s[i])) ++i;
    if (i >= s.size()) throw ParseError("line " + std::to_string(no) + ": unterminated flow collection");
    if (s[i] == '[' || s[i] == '{') {
      const bool is_map = s[i] == '{';
      const char close = is_map ? '}' : ']';
      auto n = Node::make(is_map ? Node::Map : Node::Seq, no);
      ++i;
      for (;;) {
        while (i < s.size() && space(s[i])) ++i;
        if (i >= s.size()) throw ParseError("line " + std::to_string(no) + ": unterminated flow collection");
        if (s[i] == close) {
          ++i;
          return n;
        }
        if (is_map) {
          const size_t b = i;
          while (i < s.size() && s[i] != ':') ++i;
          if (i >= s.size()) throw ParseError("line " + std::to_string(no) + ": flow map entry without ':'");
          const std::string key = unquote(strip(s.substr(b, i - b)));
          ++i;
          n->add_entry(key, flow(s, i, no));
        } else {
          n->add_item(flow(s, i, no));
        }
        while (i < s.size() && space(s[i])) ++i;
        if (i < s.size() && s[i] == ',') ++i;
      }
    }
    const size_t b = i;
    char quote = 0;
    for (; i < s.size(); ++i) {
      const char c = s[i];
      if (quote) {
        if (c == quote) quote = 0;
      } else if (c == '"' || c == '\'') {
        quote = c;
      } else if (c == ',' || c == ']' || c == '}') {
        break;
      }
    }
    const std::string t = strip(s.substr(b, i - b));
    if (t.empty() || t == "~" || t == "null") return Node::make(Node::Null, no);
    auto n = Node::make(Node::Scalar, no);
    n->set_text(unquote(t));
    return n;
  }
};

}  // namespace

std::unique_ptr<Node> parse(const std::string &text) {
  std::vector<Line> lines;
  std::istringstream in(text);
  std::string raw;
  int no = 0;
  while (std::getline(in, raw)) {
    ++no;
    std::string s = drop_comment(raw);
    while (!s.empty() && space(s.back())) s.pop_back();
    size_t col = 0;
    while (col < s.size() && s[col] == ' ') ++col;
    if (col == s.size()) continue;
    if (s[col] == '\t') throw ParseError("line " + std::to_string(no) + ": tab used for indentation");
    const std::string body = s.substr(col);
    if (body == "---" || body == "...") continue;
    lines.push_back(Line{(int)col, no, body});
  }
  return Reader(std::move(lines)).document();
}

}  // namespace yaml
}  // namespace amca
