/*
 * Minimal stand-in for the yaml-cpp 0.3.0 API, used ONLY to compile the
 * unmodified AMCA3D reference sources as a CPU oracle (test infrastructure).
 *
 * Covered: block mappings and sequences by indentation, flow sequences and
 * maps ([a, b], {k: v}), plain / single- / double-quoted scalars, comments.
 * Scalar extraction follows yaml-cpp 0.3.0's Convert(): numbers are read with
 * a std::stringstream whose basefield is unset (so "10e6" reads as 1e7 and
 * integers accept 0x / leading-0 octal) and must consume the whole scalar;
 * booleans accept y/yes/true/on and n/no/false/off in lower, UPPER or
 * Capitalised case.
 */
#ifndef AMCA_ORACLE_SHIM_YAML_H
#define AMCA_ORACLE_SHIM_YAML_H

#include <cmath> /* the real yaml-cpp/Boost headers pull <cmath> in transitively; the reference relies on it */
#include <istream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace YAML {

struct Mark {
  int pos, line, column;
  Mark() : pos(0), line(0), column(0) {}
};

namespace NodeType {
enum value { Null, Scalar, Sequence, Map };
}

class Exception : public std::runtime_error {
 public:
  Mark mark;
  Exception(const Mark &m, const std::string &msg) : std::runtime_error(msg), mark(m) {}
};
class ParserException : public Exception {
 public:
  ParserException(const Mark &m, const std::string &msg) : Exception(m, msg) {}
};
class RepresentationException : public Exception {
 public:
  RepresentationException(const Mark &m, const std::string &msg) : Exception(m, msg) {}
};
class InvalidScalar : public RepresentationException {
 public:
  explicit InvalidScalar(const Mark &m) : RepresentationException(m, "invalid scalar") {}
};
class KeyNotFound : public RepresentationException {
 public:
  KeyNotFound(const Mark &m, const std::string &key) : RepresentationException(m, "key not found: " + key) {}
};
class BadDereference : public Exception {
 public:
  BadDereference() : Exception(Mark(), "bad dereference") {}
};

class Node;

class Iterator {
 public:
  Iterator() : owner_(0), idx_(0) {}
  Iterator(const Node *owner, size_t idx) : owner_(owner), idx_(idx) {}
  const Node &first() const;
  const Node &second() const;
  const Node &operator*() const;
  const Node *operator->() const { return &**this; }
  Iterator &operator++() {
    ++idx_;
    return *this;
  }
  Iterator operator++(int) {
    Iterator t = *this;
    ++idx_;
    return t;
  }
  bool operator==(const Iterator &o) const { return owner_ == o.owner_ && idx_ == o.idx_; }
  bool operator!=(const Iterator &o) const { return !(*this == o); }

 private:
  const Node *owner_;
  size_t idx_;
};

class Node {
 public:
  Node() : type_(NodeType::Null) {}
  ~Node() { clear(); }

  NodeType::value Type() const { return type_; }
  const Mark &GetMark() const { return mark_; }
  size_t size() const { return type_ == NodeType::Sequence ? seq_.size() : (type_ == NodeType::Map ? keys_.size() : 0); }

  Iterator begin() const { return Iterator(this, 0); }
  Iterator end() const { return Iterator(this, size()); }

  const Node *FindValue(const std::string &key) const;
  const Node *FindValue(const char *key) const { return FindValue(std::string(key)); }

  const Node &operator[](size_t i) const;
  const Node &operator[](int i) const { return (*this)[(size_t)i]; }
  const Node &operator[](unsigned i) const { return (*this)[(size_t)i]; }
  const Node &operator[](const std::string &key) const;
  const Node &operator[](const char *key) const { return (*this)[std::string(key)]; }

  bool GetScalar(std::string &s) const {
    if (type_ == NodeType::Scalar) {
      s = scalar_;
      return true;
    }
    if (type_ == NodeType::Null) {
      s = "~";
      return true;
    }
    return false;
  }

  /* building (used by Parser) */
  void clear();
  void set_scalar(const std::string &s, const Mark &m) {
    clear();
    type_ = NodeType::Scalar;
    scalar_ = s;
    mark_ = m;
  }
  void set_null(const Mark &m) {
    clear();
    type_ = NodeType::Null;
    mark_ = m;
  }
  void make_seq(const Mark &m) {
    clear();
    type_ = NodeType::Sequence;
    mark_ = m;
  }
  void make_map(const Mark &m) {
    clear();
    type_ = NodeType::Map;
    mark_ = m;
  }
  Node *push_seq() {
    seq_.push_back(new Node);
    return seq_.back();
  }
  Node *push_map(const std::string &key, const Mark &km) {
    keys_.push_back(new Node);
    keys_.back()->set_scalar(key, km);
    seq_.push_back(new Node);
    return seq_.back();
  }
  void swap_content(Node &o);

 private:
  friend class Iterator;
  Node(const Node &);
  Node &operator=(const Node &);
  NodeType::value type_;
  std::string scalar_;
  std::vector<Node *> seq_;  /* sequence items, or map values */
  std::vector<Node *> keys_; /* map keys (scalars) */
  Mark mark_;
};

inline const Node &Iterator::first() const { return *owner_->keys_.at(idx_); }
inline const Node &Iterator::second() const { return *owner_->seq_.at(idx_); }
inline const Node &Iterator::operator*() const { return *owner_->seq_.at(idx_); }

bool Convert(const std::string &input, bool &output);
inline bool Convert(const std::string &input, std::string &output) {
  output = input;
  return true;
}

template <typename T>
inline bool Convert(const std::string &input, T &output) {
  std::stringstream stream(input);
  stream.unsetf(std::ios::dec);
  if ((stream >> output) && (stream >> std::ws).eof()) return true;
  if (std::numeric_limits<T>::has_infinity) {
    if (input == ".inf" || input == ".Inf" || input == ".INF" || input == "+.inf" || input == "+.Inf" ||
        input == "+.INF") {
      output = std::numeric_limits<T>::infinity();
      return true;
    }
    if (input == "-.inf" || input == "-.Inf" || input == "-.INF") {
      output = -std::numeric_limits<T>::infinity();
      return true;
    }
  }
  if (std::numeric_limits<T>::has_quiet_NaN && (input == ".nan" || input == ".NaN" || input == ".NAN")) {
    output = std::numeric_limits<T>::quiet_NaN();
    return true;
  }
  return false;
}

template <typename T>
inline void operator>>(const Node &node, T &value) {
  std::string s;
  if (!node.GetScalar(s) || !Convert(s, value)) throw InvalidScalar(node.GetMark());
}

class Parser {
 public:
  Parser() : done_(false) {}
  explicit Parser(std::istream &in);
  bool GetNextDocument(Node &doc);
  operator bool() const { return !done_; }

 private:
  std::string text_;
  bool done_;
};

/* Emitter: only used by the reference to format error messages. */
enum EMITTER_MANIP { BeginSeq, EndSeq, BeginMap, EndMap, Key, Value };
class Emitter {
 public:
  Emitter &operator<<(EMITTER_MANIP m);
  Emitter &operator<<(const std::string &s);
  Emitter &operator<<(const char *s) { return *this << std::string(s); }
  const char *c_str() const { return out_.c_str(); }
  unsigned size() const { return (unsigned)out_.size(); }

 private:
  std::string out_;
};

}  // namespace YAML

#endif
