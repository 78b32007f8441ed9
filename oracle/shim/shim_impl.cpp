/*
 * Implementation of the single-rank MPI, yaml-cpp 0.3 subset and Boost
 * subset shims that let the unmodified AMCA3D sources build as a CPU oracle.
 * Test infrastructure only: nothing in the product links this file.
 */
#include <errno.h>
#include <limits.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>

#include <cctype>
#include <cstdio>
#include <deque>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "boost/filesystem.hpp"
#include "boost/program_options.hpp"
#include "mpi.h"
#include "yaml-cpp/yaml.h"

/* ======================================================================
   glibc srand() hook: "seed s" == srand(procID*10000 + s). With np=1 the
   reference calls srand(0), so AMCA_SEED (default 0) is added on top.
   Linked with -Wl,--wrap=srand.
   ====================================================================== */
extern "C" void __real_srand(unsigned int seed);
extern "C" void __wrap_srand(unsigned int seed) {
  const char *env = getenv("AMCA_SEED");
  unsigned int add = env ? (unsigned int)strtoul(env, 0, 10) : 0u;
  __real_srand(seed + add);
}

/* ======================================================================
   MPI (one rank)
   ====================================================================== */
struct amca_shim_dtype {
  /* byte segments (offset, length) of one element, plus its extent */
  std::vector<std::pair<long, long> > segs;
  long extent;
  long size;
};

static amca_shim_dtype g_int = {std::vector<std::pair<long, long> >(1, std::make_pair(0L, 4L)), 4, 4};
static amca_shim_dtype g_dbl = {std::vector<std::pair<long, long> >(1, std::make_pair(0L, 8L)), 8, 8};
static amca_shim_dtype g_chr = {std::vector<std::pair<long, long> >(1, std::make_pair(0L, 1L)), 1, 1};
MPI_Datatype amca_shim_MPI_INTEGER = &g_int;
MPI_Datatype amca_shim_MPI_DOUBLE = &g_dbl;
MPI_Datatype amca_shim_MPI_CHAR = &g_chr;

static void pack(const void *buf, int count, MPI_Datatype dt, std::vector<char> &out) {
  const char *b = (const char *)buf;
  for (int c = 0; c < count; ++c)
    for (size_t s = 0; s < dt->segs.size(); ++s)
      out.insert(out.end(), b + c * dt->extent + dt->segs[s].first,
                 b + c * dt->extent + dt->segs[s].first + dt->segs[s].second);
}
static void unpack(const std::vector<char> &in, void *buf, int count, MPI_Datatype dt) {
  char *b = (char *)buf;
  size_t pos = 0;
  for (int c = 0; c < count; ++c)
    for (size_t s = 0; s < dt->segs.size(); ++s) {
      long n = dt->segs[s].second;
      if (pos + n > in.size()) {
        fprintf(stderr, "mpi shim: receive buffer larger than message\n");
        abort();
      }
      memcpy(b + c * dt->extent + dt->segs[s].first, &in[pos], n);
      pos += n;
    }
}
static void copy_typed(const void *src, int scount, MPI_Datatype sdt, void *dst, int rcount, MPI_Datatype rdt) {
  if (src == MPI_IN_PLACE || src == dst) return;
  std::vector<char> tmp;
  pack(src, scount, sdt, tmp);
  (void)rcount;
  /* receive only as many elements as were sent */
  long relems = rdt->size ? (long)tmp.size() / rdt->size : 0;
  unpack(tmp, dst, (int)relems, rdt);
}

static std::deque<std::vector<char> > g_self_msgs;

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
double MPI_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, 0);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm, int code) {
  exit(code);
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype dt, MPI_Op, MPI_Comm) {
  copy_typed(s, count, dt, r, count, dt);
  return MPI_SUCCESS;
}
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype dt, MPI_Op, int, MPI_Comm) {
  copy_typed(s, count, dt, r, count, dt);
  return MPI_SUCCESS;
}
int MPI_Allgather(const void *s, int sc, MPI_Datatype sdt, void *r, int rc, MPI_Datatype rdt, MPI_Comm) {
  copy_typed(s, sc, sdt, r, rc, rdt);
  return MPI_SUCCESS;
}
int MPI_Allgatherv(const void *s, int sc, MPI_Datatype sdt, void *r, const int *rcounts, const int *displs,
                   MPI_Datatype rdt, MPI_Comm) {
  if (sc > 0) copy_typed(s, sc, sdt, (char *)r + (long)displs[0] * rdt->extent, rcounts[0], rdt);
  return MPI_SUCCESS;
}
int MPI_Gather(const void *s, int sc, MPI_Datatype sdt, void *r, int rc, MPI_Datatype rdt, int, MPI_Comm) {
  copy_typed(s, sc, sdt, r, rc, rdt);
  return MPI_SUCCESS;
}
int MPI_Gatherv(const void *s, int sc, MPI_Datatype sdt, void *r, const int *rcounts, const int *displs,
                MPI_Datatype rdt, int, MPI_Comm) {
  if (sc > 0) copy_typed(s, sc, sdt, (char *)r + (long)displs[0] * rdt->extent, rcounts[0], rdt);
  return MPI_SUCCESS;
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Sendrecv(const void *sb, int sc, MPI_Datatype sdt, int dest, int, void *rb, int rc, MPI_Datatype rdt,
                 int source, int, MPI_Comm, MPI_Status *) {
  if (dest == 0) {
    std::vector<char> m;
    pack(sb, sc, sdt, m);
    g_self_msgs.push_back(m);
  }
  if (source == 0) {
    if (g_self_msgs.empty()) {
      fprintf(stderr, "mpi shim: Sendrecv from self without a message\n");
      abort();
    }
    std::vector<char> m = g_self_msgs.front();
    g_self_msgs.pop_front();
    unpack(m, rb, rc, rdt);
  }
  return MPI_SUCCESS;
}
int MPI_Isend(const void *buf, int count, MPI_Datatype dt, int dest, int, MPI_Comm, MPI_Request *req) {
  if (dest == 0) {
    std::vector<char> m;
    pack(buf, count, dt, m);
    g_self_msgs.push_back(m);
  }
  if (req) *req = 0;
  return MPI_SUCCESS;
}
int MPI_Send(const void *buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm c) {
  MPI_Request r;
  return MPI_Isend(buf, count, dt, dest, tag, c, &r);
}
int MPI_Recv(void *buf, int count, MPI_Datatype dt, int source, int, MPI_Comm, MPI_Status *) {
  if (source == MPI_PROC_NULL) return MPI_SUCCESS;
  if (g_self_msgs.empty()) {
    fprintf(stderr, "mpi shim: Recv from self without a pending message\n");
    abort();
  }
  std::vector<char> m = g_self_msgs.front();
  g_self_msgs.pop_front();
  unpack(m, buf, count, dt);
  return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }

int MPI_Dims_create(int, int ndims, int *dims) {
  for (int i = 0; i < ndims; ++i)
    if (dims[i] == 0) dims[i] = 1;
  return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm, int, const int *, const int *, int, MPI_Comm *cart) {
  *cart = 1;
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm, int maxdims, int *dims, int *periods, int *coords) {
  for (int i = 0; i < maxdims; ++i) {
    dims[i] = 1;
    periods[i] = 0;
    coords[i] = 0;
  }
  return MPI_SUCCESS;
}
int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) {
  *src = MPI_PROC_NULL;
  *dst = MPI_PROC_NULL;
  return MPI_SUCCESS;
}

static MPI_Datatype make_type(MPI_Datatype old, int count, const int *blocklens, const int *displs_elems) {
  amca_shim_dtype *t = new amca_shim_dtype;
  t->size = 0;
  long maxend = 0;
  for (int b = 0; b < count; ++b)
    for (int e = 0; e < blocklens[b]; ++e) {
      long base = ((long)displs_elems[b] + e) * old->extent;
      for (size_t s = 0; s < old->segs.size(); ++s) {
        t->segs.push_back(std::make_pair(base + old->segs[s].first, old->segs[s].second));
        t->size += old->segs[s].second;
      }
      if (base + old->extent > maxend) maxend = base + old->extent;
    }
  t->extent = maxend;
  return t;
}
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out) {
  int bl = count, d = 0;
  *out = make_type(old, 1, &bl, &d);
  return MPI_SUCCESS;
}
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old, MPI_Datatype *out) {
  std::vector<int> bl(count, blocklen), d(count);
  for (int i = 0; i < count; ++i) d[i] = i * stride;
  *out = make_type(old, count, count ? &bl[0] : 0, count ? &d[0] : 0);
  return MPI_SUCCESS;
}
int MPI_Type_indexed(int count, const int *blocklens, const int *displs, MPI_Datatype old, MPI_Datatype *out) {
  *out = make_type(old, count, blocklens, displs);
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype *dt) {
  if (*dt != &g_int && *dt != &g_dbl && *dt != &g_chr) delete *dt;
  *dt = 0;
  return MPI_SUCCESS;
}

/* ======================================================================
   Boost subset
   ====================================================================== */
namespace boost {
namespace filesystem {
path current_path() {
  char buf[PATH_MAX];
  if (!getcwd(buf, sizeof buf)) return path(".");
  return path(std::string(buf));
}
path system_complete(const path &p) {
  if (!p.string().empty() && p.string()[0] == '/') return p;
  if (p.string().empty()) return current_path();
  return path(current_path().string() + "/" + p.string());
}
bool create_directory(const path &p) { return mkdir(p.c_str(), 0755) == 0; }
}  // namespace filesystem

namespace program_options {
static void split_name(const char *name, std::string &lng, std::string &shrt) {
  std::string n(name);
  size_t c = n.find(',');
  lng = n.substr(0, c);
  shrt = c == std::string::npos ? "" : n.substr(c + 1);
}
options_init &options_init::operator()(const char *name, const char *help) {
  option_entry e;
  split_name(name, e.long_name, e.short_name);
  e.help = help;
  e.sem = 0;
  d_->entries.push_back(e);
  return *this;
}
options_init &options_init::operator()(const char *name, value_semantic *sem, const char *help) {
  option_entry e;
  split_name(name, e.long_name, e.short_name);
  e.help = help;
  e.sem = sem;
  d_->entries.push_back(e);
  return *this;
}
parsed_options parse_command_line(int argc, char **argv, const options_description &desc) {
  parsed_options p;
  p.desc = &desc;
  for (int i = 1; i < argc; ++i) {
    std::string a(argv[i]);
    const option_entry *hit = 0;
    for (size_t k = 0; k < desc.entries.size(); ++k) {
      const option_entry &e = desc.entries[k];
      if (a == "--" + e.long_name || (!e.short_name.empty() && a == "-" + e.short_name)) hit = &e;
    }
    if (!hit) throw std::runtime_error("unrecognised option " + a);
    std::string v;
    if (hit->sem) {
      if (i + 1 >= argc) throw std::runtime_error("missing value for " + a);
      v = argv[++i];
    }
    p.values[hit->long_name] = v;
  }
  return p;
}
void store(const parsed_options &p, variables_map &vm) {
  for (size_t k = 0; k < p.desc->entries.size(); ++k) {
    const option_entry &e = p.desc->entries[k];
    std::map<std::string, std::string>::const_iterator it = p.values.find(e.long_name);
    if (it != p.values.end()) {
      vm.present_[e.long_name] = it->second;
      if (e.sem) vm.pending_.push_back(std::make_pair(e.sem, it->second));
    } else if (e.sem && e.sem->has_default) {
      vm.present_[e.long_name] = e.sem->default_str;
      vm.pending_.push_back(std::make_pair(e.sem, e.sem->default_str));
    }
  }
}
void notify(variables_map &vm) {
  for (size_t k = 0; k < vm.pending_.size(); ++k) *vm.pending_[k].first->target = vm.pending_[k].second;
}
}  // namespace program_options
}  // namespace boost

/* ======================================================================
   YAML subset
   ====================================================================== */
namespace YAML {

void Node::clear() {
  for (size_t i = 0; i < seq_.size(); ++i) delete seq_[i];
  for (size_t i = 0; i < keys_.size(); ++i) delete keys_[i];
  seq_.clear();
  keys_.clear();
  scalar_.clear();
  type_ = NodeType::Null;
}
void Node::swap_content(Node &o) {
  std::swap(type_, o.type_);
  scalar_.swap(o.scalar_);
  seq_.swap(o.seq_);
  keys_.swap(o.keys_);
  std::swap(mark_, o.mark_);
}
const Node *Node::FindValue(const std::string &key) const {
  if (type_ != NodeType::Map) return 0;
  for (size_t i = 0; i < keys_.size(); ++i)
    if (keys_[i]->scalar_ == key) return seq_[i];
  return 0;
}
const Node &Node::operator[](size_t i) const {
  if (type_ != NodeType::Sequence || i >= seq_.size()) throw BadDereference();
  return *seq_[i];
}
const Node &Node::operator[](const std::string &key) const {
  const Node *v = FindValue(key);
  if (!v) throw KeyNotFound(mark_, key);
  return *v;
}

bool Convert(const std::string &in, bool &out) {
  static const char *t[] = {"y", "yes", "true", "on"};
  static const char *f[] = {"n", "no", "false", "off"};
  /* yaml-cpp 0.3 accepts all-lower, all-upper or first-letter-capitalised */
  std::string lower(in);
  for (size_t i = 0; i < lower.size(); ++i) lower[i] = (char)tolower((unsigned char)lower[i]);
  bool ok_case = true;
  if (!in.empty()) {
    bool all_lower = true, all_upper = true, cap = isupper((unsigned char)in[0]) != 0;
    for (size_t i = 0; i < in.size(); ++i) {
      if (isupper((unsigned char)in[i])) all_lower = false;
      if (islower((unsigned char)in[i])) all_upper = false;
      if (i > 0 && isupper((unsigned char)in[i])) cap = false;
    }
    ok_case = all_lower || all_upper || cap;
  }
  if (!ok_case) return false;
  for (int i = 0; i < 4; ++i)
    if (lower == t[i]) {
      out = true;
      return true;
    }
  for (int i = 0; i < 4; ++i)
    if (lower == f[i]) {
      out = false;
      return true;
    }
  return false;
}

namespace {
struct Line {
  int indent;
  std::string text;
  int lineno;
};

std::string rtrim(const std::string &s) {
  size_t e = s.find_last_not_of(" \t\r");
  return e == std::string::npos ? std::string() : s.substr(0, e + 1);
}
std::string trim(const std::string &s) {
  size_t b = s.find_first_not_of(" \t\r");
  if (b == std::string::npos) return std::string();
  return rtrim(s.substr(b));
}
/* strip a '#' comment that is not inside quotes */
std::string strip_comment(const std::string &s) {
  char q = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (q) {
      if (c == q) q = 0;
      continue;
    }
    if (c == '"' || c == '\'') {
      q = c;
      continue;
    }
    if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
  }
  return s;
}
std::string unquote(const std::string &s) {
  if (s.size() >= 2 && ((s[0] == '"' && s[s.size() - 1] == '"') || (s[0] == '\'' && s[s.size() - 1] == '\'')))
    return s.substr(1, s.size() - 2);
  return s;
}
/* position of the "key:" separator (colon followed by space or end), or npos */
size_t key_colon(const std::string &s) {
  char q = 0;
  int depth = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    char c = s[i];
    if (q) {
      if (c == q) q = 0;
      continue;
    }
    if (c == '"' || c == '\'') q = c;
    else if (c == '[' || c == '{') ++depth;
    else if (c == ']' || c == '}') --depth;
    else if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t'))
      return i;
  }
  return std::string::npos;
}
bool is_seq_item(const std::string &t) { return t == "-" || (t.size() > 1 && t[0] == '-' && (t[1] == ' ' || t[1] == '\t')); }

class BlockParser {
 public:
  explicit BlockParser(std::vector<Line> &lines) : L(lines), pos(0) {}
  void parse_document(Node &out) {
    if (L.empty()) {
      out.set_null(Mark());
      return;
    }
    parse_block(out, L[0].indent);
  }

 private:
  std::vector<Line> &L;
  size_t pos;

  Mark mark_of(const Line &l) const {
    Mark m;
    m.line = l.lineno;
    m.column = l.indent;
    return m;
  }

  void parse_flow(const std::string &s, size_t &i, Node &out, const Mark &m) {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
    if (i < s.size() && s[i] == '[') {
      out.make_seq(m);
      ++i;
      while (true) {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
        if (i >= s.size()) throw ParserException(m, "unterminated flow sequence");
        if (s[i] == ']') {
          ++i;
          return;
        }
        Node *item = out.push_seq();
        parse_flow(s, i, *item, m);
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
        if (i < s.size() && s[i] == ',') ++i;
      }
    } else if (i < s.size() && s[i] == '{') {
      out.make_map(m);
      ++i;
      while (true) {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
        if (i >= s.size()) throw ParserException(m, "unterminated flow map");
        if (s[i] == '}') {
          ++i;
          return;
        }
        size_t b = i;
        while (i < s.size() && s[i] != ':') ++i;
        std::string key = unquote(trim(s.substr(b, i - b)));
        ++i;
        Node *v = out.push_map(key, m);
        parse_flow(s, i, *v, m);
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
        if (i < s.size() && s[i] == ',') ++i;
      }
    } else {
      size_t b = i;
      char q = 0;
      while (i < s.size()) {
        char c = s[i];
        if (q) {
          if (c == q) q = 0;
        } else if (c == '"' || c == '\'') {
          q = c;
        } else if (c == ',' || c == ']' || c == '}') {
          break;
        }
        ++i;
      }
      std::string v = trim(s.substr(b, i - b));
      if (v.empty() || v == "~" || v == "null") out.set_null(m);
      else out.set_scalar(unquote(v), m);
    }
  }

  void parse_inline_value(const std::string &v, Node &out, const Mark &m) {
    if (!v.empty() && (v[0] == '[' || v[0] == '{')) {
      size_t i = 0;
      parse_flow(v, i, out, m);
    } else if (v == "~" || v == "null") {
      out.set_null(m);
    } else {
      out.set_scalar(unquote(v), m);
    }
  }

  void parse_block(Node &out, int indent) {
    const Line &first = L[pos];
    if (is_seq_item(first.text)) parse_seq(out, indent);
    else if (key_colon(first.text) != std::string::npos) parse_map(out, indent);
    else {
      parse_inline_value(first.text, out, mark_of(first));
      ++pos;
    }
  }

  void parse_seq(Node &out, int indent) {
    out.make_seq(mark_of(L[pos]));
    while (pos < L.size() && L[pos].indent == indent && is_seq_item(L[pos].text)) {
      Line &ln = L[pos];
      Node *item = out.push_seq();
      std::string rest = ln.text.size() > 1 ? ln.text.substr(1) : std::string();
      size_t off = rest.find_first_not_of(" \t");
      if (off == std::string::npos) {
        ++pos;
        if (pos < L.size() && L[pos].indent > indent) parse_block(*item, L[pos].indent);
        else item->set_null(mark_of(ln));
      } else {
        /* the item's content starts a block at the column after "- " */
        ln.indent = indent + 1 + (int)off;
        ln.text = rest.substr(off);
        parse_block(*item, ln.indent);
      }
    }
  }

  void parse_map(Node &out, int indent) {
    out.make_map(mark_of(L[pos]));
    while (pos < L.size() && L[pos].indent == indent && !is_seq_item(L[pos].text)) {
      const Line &ln = L[pos];
      size_t c = key_colon(ln.text);
      if (c == std::string::npos) throw ParserException(mark_of(ln), "expected a mapping key: " + ln.text);
      std::string key = unquote(trim(ln.text.substr(0, c)));
      std::string val = trim(ln.text.substr(c + 1));
      Mark km = mark_of(ln);
      Node *v = out.push_map(key, km);
      ++pos;
      if (!val.empty()) {
        parse_inline_value(val, *v, km);
      } else if (pos < L.size() && L[pos].indent > indent) {
        parse_block(*v, L[pos].indent);
      } else if (pos < L.size() && L[pos].indent == indent && is_seq_item(L[pos].text)) {
        parse_seq(*v, indent);
      } else {
        v->set_null(km);
      }
    }
  }
};
}  // namespace

Parser::Parser(std::istream &in) : done_(false) {
  std::stringstream ss;
  ss << in.rdbuf();
  text_ = ss.str();
}

bool Parser::GetNextDocument(Node &doc) {
  if (done_) return false;
  done_ = true;
  std::vector<Line> lines;
  std::istringstream in(text_);
  std::string raw;
  int no = 0;
  while (std::getline(in, raw)) {
    ++no;
    std::string s = rtrim(strip_comment(raw));
    if (trim(s).empty()) continue;
    if (trim(s) == "---" || trim(s) == "...") continue;
    size_t ind = s.find_first_not_of(' ');
    Line l;
    l.indent = (int)ind;
    l.text = s.substr(ind);
    l.lineno = no;
    lines.push_back(l);
  }
  Node tmp;
  BlockParser(lines).parse_document(tmp);
  doc.swap_content(tmp);
  return true;
}

Emitter &Emitter::operator<<(EMITTER_MANIP m) {
  switch (m) {
    case BeginSeq: out_ += "["; break;
    case EndSeq: out_ += "]"; break;
    case BeginMap: out_ += "{"; break;
    case EndMap: out_ += "}"; break;
    case Key: out_ += " "; break;
    case Value: out_ += ": "; break;
  }
  return *this;
}
Emitter &Emitter::operator<<(const std::string &s) {
  out_ += s;
  out_ += " ";
  return *this;
}

}  // namespace YAML
