// yaml_lite.h — the YAML subset of AMCA3D input decks.
//
// The reference reads decks with yaml-cpp 0.3.0 (CA/src/Cafe.cpp:111-121,
// CA/include/CafeParsing.h:97-142). This reader accepts what those decks use:
// block mappings and sequences by indentation ("- key: value" items included),
// flow sequences / maps, plain and quoted scalars, '#' comments.
// Scalars convert with yaml-cpp 0.3.0's rules: numbers through an istream
// whose basefield is unset, which must consume the whole text ("10e6" reads
// as 1e7); booleans y/yes/true/on and n/no/false/off (lower, UPPER or
// Capitalised).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace amca {
namespace yaml {

struct ParseError : std::runtime_error {
  explicit ParseError(const std::string &m) : std::runtime_error(m) {}
};

class Node {
 public:
  enum Kind { Null, Scalar, Seq, Map };

  Kind kind() const { return kind_; }
  int line() const { return line_; }
  bool is_map() const { return kind_ == Map; }
  bool is_seq() const { return kind_ == Seq; }
  bool is_scalar() const { return kind_ == Scalar; }
  size_t size() const { return kind_ == Seq ? items_.size() : (kind_ == Map ? entries_.size() : 0); }

  const Node *find(const std::string &key) const;  // map lookup, nullptr if absent
  const Node &at(size_t i) const;                   // sequence item
  const std::vector<std::pair<std::string, std::unique_ptr<Node>>> &entries() const { return entries_; }
  const std::string &text() const { return text_; }

  // yaml-cpp 0.3 conversions; throw ParseError when the scalar does not convert.
  double as_double() const;
  int as_int() const;
  bool as_bool() const;
  std::string as_string() const;

  // building
  static std::unique_ptr<Node> make(Kind k, int line) {
    std::unique_ptr<Node> n(new Node);
    n->kind_ = k;
    n->line_ = line;
    return n;
  }
  void set_text(const std::string &t) { text_ = t; }
  Node *add_item(std::unique_ptr<Node> n) {
    items_.push_back(std::move(n));
    return items_.back().get();
  }
  Node *add_entry(const std::string &k, std::unique_ptr<Node> n) {
    entries_.emplace_back(k, std::move(n));
    return entries_.back().second.get();
  }

 private:
  Kind kind_ = Null;
  int line_ = 0;
  std::string text_;
  std::vector<std::unique_ptr<Node>> items_;
  std::vector<std::pair<std::string, std::unique_ptr<Node>>> entries_;
};

// Parse one document. Throws ParseError with the line number on bad input.
std::unique_ptr<Node> parse(const std::string &text);

}  // namespace yaml
}  // namespace amca
