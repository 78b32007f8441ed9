/*
 * Minimal stand-in for the parts of boost::filesystem that the AMCA3D
 * reference calls (path, current_path, system_complete, create_directory).
 * Oracle build only; POSIX semantics.
 */
#ifndef AMCA_ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#define AMCA_ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#include <ostream>
#include <string>

namespace boost {
namespace filesystem {
class path {
 public:
  path() {}
  path(const std::string &s) : s_(s) {}
  path(const char *s) : s_(s) {}
  const std::string &string() const { return s_; }
  const char *c_str() const { return s_.c_str(); }

 private:
  std::string s_;
};
inline std::ostream &operator<<(std::ostream &os, const path &p) { return os << '"' << p.string() << '"'; }
path current_path();
path system_complete(const path &p);
bool create_directory(const path &p);
}  // namespace filesystem
}  // namespace boost
#endif
