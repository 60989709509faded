// Oracle test infrastructure: boost::filesystem mapped onto std::filesystem,
// plus boost::lexical_cast<double>, the only other Boost utility the SOUFFLE
// sources call (functions.cpp restart-file sniffing).
#ifndef ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#define ORACLE_SHIM_BOOST_FILESYSTEM_HPP
#include <filesystem>
#include <sstream>
#include <stdexcept>
#include <string>

namespace boost {
namespace filesystem = std::filesystem;

class bad_lexical_cast : public std::bad_cast {};

template <class T>
T lexical_cast(const std::string& s) {
  std::istringstream in(s);
  T v;
  in >> v;
  if (in.fail()) throw bad_lexical_cast();
  char extra;
  if (in >> extra) throw bad_lexical_cast();
  return v;
}
}  // namespace boost

#endif
