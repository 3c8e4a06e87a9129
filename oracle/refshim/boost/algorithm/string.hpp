/* Stand-ins for the boost string algorithms the reference's SGF code uses. */
#ifndef ORACLE_BOOST_ALGO_STRING_SHIM
#define ORACLE_BOOST_ALGO_STRING_SHIM
#include <string>
namespace boost { namespace algorithm {
inline bool find_first(const std::string &s, const std::string &p) { return s.find(p) != std::string::npos; }
inline bool starts_with(const std::string &s, const std::string &p) { return s.compare(0, p.size(), p) == 0; }
} }
#endif
