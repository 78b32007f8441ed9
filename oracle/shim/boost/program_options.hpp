/*
 * Minimal stand-in for boost::program_options as used by the AMCA3D
 * reference main(): "name,s" options with optional std::string values and
 * default values, store/parse_command_line/notify, variables_map::count.
 * Oracle build only.
 */
#ifndef AMCA_ORACLE_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#define AMCA_ORACLE_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#include <map>
#include <ostream>
#include <string>
#include <vector>

namespace boost {
namespace program_options {

class value_semantic {
 public:
  std::string *target;
  bool has_default;
  std::string default_str;
  value_semantic(std::string *t) : target(t), has_default(false) {}
  value_semantic *default_value(const std::string &v) {
    has_default = true;
    default_str = v;
    return this;
  }
};
template <typename T>
value_semantic *value(T *t) {
  return new value_semantic(t);
}

struct option_entry {
  std::string long_name, short_name, help;
  value_semantic *sem;
};

class options_description;
class options_init {
 public:
  explicit options_init(options_description *d) : d_(d) {}
  options_init &operator()(const char *name, const char *help);
  options_init &operator()(const char *name, value_semantic *sem, const char *help);

 private:
  options_description *d_;
};

class options_description {
 public:
  explicit options_description(const std::string &caption) : caption(caption) {}
  options_init add_options() { return options_init(this); }
  std::string caption;
  std::vector<option_entry> entries;
};
inline std::ostream &operator<<(std::ostream &os, const options_description &d) {
  os << d.caption << ":\n";
  for (size_t i = 0; i < d.entries.size(); ++i)
    os << "  --" << d.entries[i].long_name << " (-" << d.entries[i].short_name << ")  " << d.entries[i].help << "\n";
  return os;
}

struct parsed_options {
  const options_description *desc;
  std::map<std::string, std::string> values; /* long name -> value ("" for flags) */
};
parsed_options parse_command_line(int argc, char **argv, const options_description &desc);

class variables_map {
 public:
  size_t count(const std::string &name) const { return present_.count(name); }
  std::map<std::string, std::string> present_;
  std::vector<std::pair<value_semantic *, std::string> > pending_;
};
void store(const parsed_options &p, variables_map &vm);
void notify(variables_map &vm);

}  // namespace program_options
}  // namespace boost
#endif
