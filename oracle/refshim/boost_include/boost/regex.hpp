/* Stand-in for the part of Boost.Regex that na_calc.cpp uses (regex,
 * smatch, regex_search): std::regex (ECMAScript; na_calc's patterns are
 * plain file-name prefixes).  See filesystem.hpp beside it. */
#ifndef NR_REF_BOOST_REGEX_HPP
#define NR_REF_BOOST_REGEX_HPP
#include <regex>
namespace boost {
using std::regex;
using std::regex_search;
using std::smatch;
}  // namespace boost
#endif
