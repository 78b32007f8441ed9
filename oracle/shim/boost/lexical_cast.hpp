/* Minimal boost::lexical_cast stand-in (oracle build only). */
#ifndef AMCA_ORACLE_SHIM_BOOST_LEXICAL_CAST_HPP
#define AMCA_ORACLE_SHIM_BOOST_LEXICAL_CAST_HPP
#include <sstream>
#include <stdexcept>
namespace boost {
struct bad_lexical_cast : std::runtime_error {
  bad_lexical_cast() : std::runtime_error("bad lexical cast") {}
};
template <typename T, typename S>
T lexical_cast(const S &s) {
  std::stringstream ss;
  ss << s;
  T t;
  if (!(ss >> t)) throw bad_lexical_cast();
  return t;
}
}  // namespace boost
#endif
