// Oracle test infrastructure: a small short-option parser with the shape of
// boost::program_options as the SOUFFLE driver (md.cpp option table) uses it:
//   desc.add_options()("name,X", value<T>(&v)->default_value(d), "help")...
//   store(parse_command_line(argc, argv, desc), vm); notify(vm); vm.count(..)
// Accepts "-X value", "-Xvalue" and "--name value".  Options not given take
// their default.  Bool values accept true/false/1/0/yes/no/on/off.
#ifndef ORACLE_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#define ORACLE_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#include <cstdlib>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace boost {
namespace program_options {

class value_semantic {
 public:
  virtual ~value_semantic() {}
  virtual void apply_default() = 0;
  virtual void parse(const std::string& s) = 0;
};

template <class T>
inline void oracle_shim_parse_into(const std::string& s, T* out) {
  std::istringstream in(s);
  in >> *out;
  if (in.fail()) {
    std::cerr << "bad option value: " << s << std::endl;
    std::exit(2);
  }
}

template <>
inline void oracle_shim_parse_into<bool>(const std::string& s, bool* out) {
  if (s == "1" || s == "true" || s == "yes" || s == "on")
    *out = true;
  else if (s == "0" || s == "false" || s == "no" || s == "off")
    *out = false;
  else {
    std::cerr << "bad bool option value: " << s << std::endl;
    std::exit(2);
  }
}

template <class T>
class typed_value : public value_semantic {
 public:
  explicit typed_value(T* p) : ptr_(p), has_default_(false) {}
  typed_value* default_value(const T& v) {
    def_ = v;
    has_default_ = true;
    return this;
  }
  void apply_default() override {
    if (has_default_ && ptr_) *ptr_ = def_;
  }
  void parse(const std::string& s) override {
    if (ptr_) oracle_shim_parse_into<T>(s, ptr_);
  }

 private:
  T* ptr_;
  T def_;
  bool has_default_;
};

template <class T>
typed_value<T>* value(T* p) {
  return new typed_value<T>(p);
}

struct oracle_shim_option {
  std::string long_name;
  char short_name;
  std::shared_ptr<value_semantic> sem;  // null for flags such as --help
  std::string help;
};

class options_description;

class options_description_easy_init {
 public:
  explicit options_description_easy_init(options_description* d) : d_(d) {}
  options_description_easy_init& operator()(const char* name, const char* help);
  options_description_easy_init& operator()(const char* name, value_semantic* s,
                                            const char* help);

 private:
  options_description* d_;
};

class options_description {
 public:
  explicit options_description(const std::string& caption = "") : caption_(caption) {}
  options_description_easy_init add_options() { return options_description_easy_init(this); }
  void add(const char* name, value_semantic* s, const char* help) {
    oracle_shim_option o;
    std::string n(name);
    size_t comma = n.find(',');
    o.long_name = n.substr(0, comma);
    o.short_name = (comma == std::string::npos) ? 0 : n[comma + 1];
    o.sem.reset(s);
    o.help = help ? help : "";
    opts_.push_back(o);
  }
  const std::vector<oracle_shim_option>& options() const { return opts_; }
  const std::string& caption() const { return caption_; }

 private:
  std::string caption_;
  std::vector<oracle_shim_option> opts_;
};

inline options_description_easy_init& options_description_easy_init::operator()(
    const char* name, const char* help) {
  d_->add(name, nullptr, help);
  return *this;
}
inline options_description_easy_init& options_description_easy_init::operator()(
    const char* name, value_semantic* s, const char* help) {
  d_->add(name, s, help);
  return *this;
}

inline std::ostream& operator<<(std::ostream& os, const options_description& d) {
  os << d.caption() << "\n";
  for (const auto& o : d.options())
    os << "  -" << (o.short_name ? o.short_name : ' ') << " [" << o.long_name << "] " << o.help
       << "\n";
  return os;
}

struct parsed_options {
  const options_description* desc;
  std::vector<std::pair<int, std::string> > given;  // option index, raw value
};

class variables_map {
 public:
  size_t count(const std::string& name) const { return seen_.count(name); }
  std::map<std::string, int> seen_;
};

inline parsed_options parse_command_line(int argc, char** argv, const options_description& d) {
  parsed_options p;
  p.desc = &d;
  const auto& opts = d.options();
  for (int a = 1; a < argc; ++a) {
    std::string tok(argv[a]);
    int idx = -1;
    std::string val;
    bool inline_val = false;
    if (tok.size() > 2 && tok[0] == '-' && tok[1] == '-') {
      std::string nm = tok.substr(2);
      for (size_t k = 0; k < opts.size(); ++k)
        if (opts[k].long_name == nm) idx = (int)k;
    } else if (tok.size() >= 2 && tok[0] == '-') {
      for (size_t k = 0; k < opts.size(); ++k)
        if (opts[k].short_name == tok[1]) idx = (int)k;
      if (tok.size() > 2) {
        val = tok.substr(2);
        inline_val = true;
      }
    }
    if (idx < 0) {
      std::cerr << "unrecognised option: " << tok << std::endl;
      std::exit(2);
    }
    if (opts[idx].sem && !inline_val) {
      if (a + 1 >= argc) {
        std::cerr << "option needs a value: " << tok << std::endl;
        std::exit(2);
      }
      val = argv[++a];
    }
    p.given.push_back(std::make_pair(idx, val));
  }
  return p;
}

inline void store(const parsed_options& p, variables_map& vm) {
  const auto& opts = p.desc->options();
  for (const auto& o : opts)
    if (o.sem) o.sem->apply_default();
  for (const auto& g : p.given) {
    const auto& o = opts[g.first];
    if (o.sem) o.sem->parse(g.second);
    vm.seen_[o.long_name] = 1;
  }
}

inline void notify(variables_map&) {}

}  // namespace program_options
}  // namespace boost

#endif
